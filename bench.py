#!/usr/bin/env python3
"""Benchmark: edge-samples validated per second on one GB300.

Workload (default): the 4-arm composite configuration -- four Pandas at the
corners of a 1.0 m square facing the centre, 65536 edges of 28 DOF with
|dq| <= 1.5 rad, 32 samples per edge, a 51-box bin-picking scene, checks of
arm-vs-environment and every arm-vs-arm pair with the reference's verdict
semantics.  Seeded synthetic inputs (no dataset exists for this path).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

A step validates the whole batch once.  `value` is device-timed throughput
with inputs resident in HBM (L2 flushed before every step); `e2e` is the same
metric through the host-buffer C ABI call with page-locked host buffers (the
kernels read the edges from host memory and write the verdicts there, inside
the timed region).  Per-kernel device times for `roofline` come from a second
pass of the same steps with the library's per-launch event timing on.  Under
torchrun
each rank validates its own copy of the batch (independent edges, no
collective); value = all ranks' samples / slowest rank's time.
The reference arm runs the reference's own CUDA edge check
(fkcc_single_buffer<Panda_four>, compiled from the reference sources into
oracle/_ref) on the same inputs, or the CPU restatement when that build is
absent.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "edge-samples validated/s"
UNIT = "edge-samples/s"
L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["mine", "reference"], default="mine")
    ap.add_argument("--workload", choices=["config1", "config2", "config3", "config3s", "config4", "config5",
                                           "planner4", "planner5"],
                    default="config2")
    ap.add_argument("--problems", type=int, default=50, help="planner4/5: reference problems solved")
    ap.add_argument("--planner", choices=["drrt", "compact"], default="drrt",
                    help="config5: the client planner of the served stream")
    ap.add_argument("--streams", type=int, default=0, help="config5: the service's wave slots (0: the planner's default)")
    ap.add_argument("--clients", type=int, default=0, help="config5: client threads (0: the planner's default)")
    ap.add_argument("--fused-edges", type=int, default=0,
                    help="config5: wave groups of at most this many edges run fused (0: the service default, -1: never)")
    ap.add_argument("--rate", type=float, default=200.0, help="config5: query arrivals per second (Poisson)")
    ap.add_argument("--duration", type=float, default=60.0, help="config5: seconds of arrivals")
    ap.add_argument("--isolated", type=int, default=100, help="config5: queries also solved alone, for comparison")
    ap.add_argument("--instances", type=int, default=512, help="config4: planning instances in the batch")
    ap.add_argument("--edges", type=int, default=0,
                    help="config1/2/3: edges (0 = the workload's size); small cases for profiler captures")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle parity counts (CPU leg)")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the secondary device-timed lines of configs 1, 3 and the shortcut set")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, gpu_index: int, util: bool = False):
        self.gpu = gpu_index
        self.util = util  # also report the median GPU utilisation (long runs)
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.lower().startswith("active")})
        util = [float(r[9]) for r in self.rows if len(r) > 9 and r[9].replace(".", "").isdigit()]
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
               "reasons": reasons, "samples": len(self.rows)}
        if self.util:
            out["gpu_util_pct_median"] = statistics.median(util) if util else None
        return out


def host_cpu_times() -> tuple[int, int] | None:
    """(busy, total) jiffies of all host cores from /proc/stat, or None."""
    try:
        with open("/proc/stat") as f:
            v = [int(x) for x in f.readline().split()[1:]]
    except (OSError, ValueError):
        return None
    idle = v[3] + (v[4] if len(v) > 4 else 0)
    return sum(v) - idle, sum(v)


def dist_setup(backend: str = "nccl"):
    """Rank, world size and local GPU from the launcher's environment; one
    process per GPU.  backend "gloo" (CPU, tests) skips the device binding."""
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if backend == "nccl":
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        if backend == "nccl":
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    """The slowest rank's time (every rank gets it)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: int, steps: int, seconds: list, world: int) -> float:
    """Whole-job units/s of independent replicas: every rank's units over the
    slowest rank's time (weak scaling, no data exchange)."""
    t = max_over_ranks(sum(seconds), world)
    return world * units_per_rank * steps / t


def load_workload(pkg, name, edges: int = 0):
    W = pkg.workloads
    if edges and name in ("config1", "config2", "config3"):
        return {"config1": W.config1, "config2": W.config2, "config3": W.config3}[name](n_edges=edges)
    return {"config1": W.config1, "config2": W.config2, "config3": W.config3,
            "config3s": W.config3_shortcuts}[name]()


def workload_config(wl, extra):
    sc = wl.scene
    n_obst = int(len(sc.spheres) + len(sc.capsules) + len(sc.z_capsules) + len(sc.cuboids) + len(sc.z_cuboids))
    cfg = {"workload": wl.name, "edges": int(len(wl.q0)), "granularity": wl.granularity,
           "arms": int(len(wl.bases)) if wl.arm < 0 else 1, "dof": int(wl.q0.shape[1]), "obstacles": n_obst,
           "checks": "env+self" if wl.flags & 3 == 3 else ("self" if wl.flags & 2 else "env"),
           "semantics": "reference verdicts (thread split included)", "l2": "flushed (256 MiB write) before every step"}
    if wl.rule:
        cfg.update({"rule": {1: "connect", 2: "bspline", 3: "shortcut"}[wl.rule], "range": wl.range_,
                    "samples": "segments up to the first colliding one x granularity"})
    cfg.update(extra)
    return cfg


def cpu_baseline(orc, wl, n_edges: int):
    """The CPU restatement on all host threads over the first n_edges edges,
    plus a one-thread figure over an eighth of them (about 15-40 s of CPU
    work in all on the workloads here)."""
    threads = orc.max_threads()
    sub0, sub1 = wl.q0[:n_edges], wl.q1[:n_edges]
    orc.validate(wl.scene, wl.bases, sub0[:64], sub1[:64], wl.granularity, wl.flags, wl.arm, threads=threads)
    t = time.perf_counter()
    orc.validate(wl.scene, wl.bases, sub0, sub1, wl.granularity, wl.flags, wl.arm, threads=threads)
    dt = time.perf_counter() - t
    n1 = max(1, n_edges // 8)
    t = time.perf_counter()
    orc.validate(wl.scene, wl.bases, sub0[:n1], sub1[:n1], wl.granularity, wl.flags, wl.arm, threads=1)
    dt1 = time.perf_counter() - t
    return {"value": n_edges * wl.granularity / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "value_1core": n1 * wl.granularity / dt1,
            "sample": f"first {n_edges} of the {len(wl.q0)} edges, oracle/edge_oracle.c (FP32 restatement of the "
                      f"reference check), OpenMP over edges, {dt:.2f} s wall; value_1core: first {n1} edges on "
                      f"one thread, {dt1:.2f} s"}


def fp32_peak(pkg, torch) -> float:
    """Measured FP32 FMA issue rate of this GPU in TFLOP/s (best of 3)."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, iters = sms * 8, 4000
    scratch = torch.zeros(blocks, device="cuda")
    pkg.mrpop.fp32_peak_probe(blocks, 200, scratch)
    best = 0.0
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fl = pkg.mrpop.fp32_peak_probe(blocks, iters, scratch)
        e.record()
        torch.cuda.synchronize()
        best = max(best, fl / (s.elapsed_time(e) * 1e-3) / 1e12)
    return best


KERNEL_NAMES = {"fused": "validate_kernel", "broad": "broad_kernel", "narrow": "narrow_kernel"}


def committed_profile(kernel: str, workload: str) -> dict:
    """Per-launch figures of one kernel from the committed ncu summary
    (profiles/<kernel>_<workload>.json): DRAM bytes and executed FP32 flops."""
    p = ROOT / "profiles" / f"{kernel}_{workload}.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return {}
    return {}


def step_traffic(kt: dict, workload: str, algorithmic_bytes: int, steps: int) -> dict:
    """DRAM bytes of one step (every kernel of the step, from the committed
    per-launch captures) against the step's algorithmic bytes (endpoints read,
    verdicts written)."""
    per = {}
    for kind, (launches, _) in kt.items():
        if not launches:
            continue
        b = committed_profile(KERNEL_NAMES[kind], workload).get("dram_bytes_per_launch")
        if b is None:
            return {"bytes": None, "algorithmic_bytes": algorithmic_bytes,
                    "basis": f"no committed capture of {KERNEL_NAMES[kind]} on {workload}"}
        per[KERNEL_NAMES[kind]] = b * launches / steps
    total = sum(per.values())
    return {"bytes": total, "per_kernel": per, "algorithmic_bytes": algorithmic_bytes,
            "ratio": total / algorithmic_bytes,
            "basis": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch under application replay with "
                     "--cache-control none (profiles/<kernel>_<workload>.json); the broad kernel's writes include "
                     "the write-back of the L2-flush buffer's dirty lines that its own lines evict"}


def roofline(kt: dict, flops: dict, peak: float, workload: str, arms: int, spl: int, steps: int,
             sm_mhz: float | None = None) -> dict:
    """Roofline of the kernel with the largest share of device time.
    kt: {kind: (launches, total ms)} from the library's event timing over
    `steps` steps; flops: algorithmic flops per step of each kind (a kind may
    launch more than once per step: segment rounds); sm_mhz: the median SM
    clock sampled over the timed region.

    The kernels are bound by instruction issue (FP32 is about a third of what
    they issue; the rest is integer, shared-memory, vote and branch work, and
    culling skips most of the algorithmic flops), so `frac` is the dominant
    kernel's warp-instruction rate against 4 schedulers x SMs x the sampled
    clock.  The FP32 view -- executed FP32 flops against the measured FP32
    FMA peak, and the algorithmic (unculled) flop rate, which can exceed that
    peak because culling skips work -- is kept under `fp32`."""
    import torch
    ran = {k: v for k, v in kt.items() if v[0] > 0}
    total_ms = sum(v[1] for v in ran.values())
    dom = max(ran, key=lambda k: ran[k][1])
    launches, ms = ran[dom]
    launch_s = ms / launches / 1e3
    algorithmic = flops[dom] / (ms / steps / 1e3) / 1e12
    prof = committed_profile(KERNEL_NAMES[dom], workload)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = sm_mhz
    if not mhz and (ROOT / "MEASURED_PEAKS.json").exists():
        mhz = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("sm_max_mhz")
    out = {"bound": "issue", "kernel": f"{KERNEL_NAMES[dom]}<{arms},{spl}>", "achieved": None, "peak": None,
           "unit": "warp instructions/s", "frac": None, "traffic": prof.get("dram_bytes_per_launch"),
           "launch_ms": launch_s * 1e3, "launches_per_step": launches / steps, "share": ms / total_ms}
    if prof.get("warp_instructions") and mhz:
        # every SM has four schedulers that issue at most one warp instruction per clock
        rate = prof["warp_instructions"] / launch_s
        cap = 4 * sms * mhz * 1e6
        out.update({"achieved": rate, "peak": cap, "frac": rate / cap,
                    "peak_source": f"4 schedulers x {sms} SMs x {mhz:.0f} MHz (median SM clock sampled in the "
                                   f"timed region)",
                    "achieved_basis": "warp instructions of one launch (ncu smsp__inst_executed.sum, committed "
                                      f"profile profiles/{KERNEL_NAMES[dom]}_{workload}.json) / the kernel's "
                                      "CUDA-event launch time in this run"})
    else:
        out["frac_note"] = f"no committed ncu instruction count for {KERNEL_NAMES[dom]} on {workload}"
    fp32 = {"peak_tflops": peak,
            "peak_source": "measured: FP32 FMA loop (mrpop_fp32_peak_probe) timed in this run; "
                           "MEASURED_PEAKS.json has no FP32 figure",
            "algorithmic_rate_tflops": algorithmic,
            "algorithmic_basis": f"{flops[dom]:.4g} algorithmic flops per step (FMA=2, unculled per-test costs) / "
                                 f"the kernel's CUDA-event time per step; not a fraction of anything: culling "
                                 f"skips most of this work"}
    if prof.get("executed_fp32_flops_per_launch"):
        ex = prof["executed_fp32_flops_per_launch"] / launch_s / 1e12
        fp32["executed"] = {"achieved_tflops": ex, "frac": ex / peak,
                            "basis": "FP32 flops the kernel executed (ncu: 2*ffma + fadd + fmul thread "
                                     "instructions, committed profile) / live launch time"}
    out["fp32"] = fp32
    if out["traffic"]:
        hbm = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs") \
            if (ROOT / "MEASURED_PEAKS.json").exists() else None
        bw = out["traffic"] / launch_s / 1e9
        out["hbm_check"] = {"achieved_gbs": bw, "peak_gbs": hbm, "frac": bw / hbm if hbm else None,
                            "basis": "ncu DRAM bytes of one launch / live launch time, against the measured copy "
                                     "bandwidth (MEASURED_PEAKS.json): HBM is not the bound"}
    out["kernels"] = {KERNEL_NAMES[k]: {"launches": v[0], "avg_ms": v[1] / v[0], "share": v[1] / total_ms,
                                        "algorithmic_tflops": flops[k] / (v[1] / steps / 1e3) / 1e12}
                      for k, v in ran.items()}
    return out


def parity_counts(orc, pkg, torch, wl, valid: np.ndarray, first: np.ndarray, band: float = 1e-5) -> dict:
    """Verdicts of the timed run against the oracle over the whole workload,
    with the near-contact samples counted: a sample is ambiguous when a
    deciding minimum signed distance (FP64) lies within `band` of zero, and a
    verdict may differ only on an edge holding such a sample.  Edges that
    differ from the host-trig oracle without being ambiguous are checked again
    with the device's __sinf/__cosf values replayed into the oracle."""
    t = time.perf_counter()
    o = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_,
                     band=band, threads=orc.max_threads(), count_ambiguous=True)
    amb = o["ambiguous"].astype(bool)
    diff = (valid != o["valid"]) | (first != o["first_hit"])
    idx = np.nonzero(diff & ~amb)[0]
    replay = 0
    if len(idx):
        def dev_trig(x):
            c, s = pkg.debug_trig(torch.from_numpy(x).cuda())
            torch.cuda.synchronize()
            return c.cpu().numpy(), s.cpu().numpy()
        r = orc.validate_with_trig(wl.scene, wl.bases, wl.q0[idx], wl.q1[idx], wl.granularity, wl.flags, wl.arm,
                                   wl.rule, wl.range_, dev_trig)
        replay = int(((valid[idx] != r["valid"]) | (first[idx] != r["first_hit"])).sum())
    return {"against": "oracle/edge_oracle.c: FP32 restatement of the reference's edge check (host sinf/cosf; "
                       "the device uses __sinf/__cosf), FP64 distances for the ambiguity band",
            "edges": int(len(valid)), "edges_differ": int(diff.sum()),
            "edges_differ_unambiguous": int(len(idx)), "edges_differ_after_device_trig_replay": replay,
            "ambiguous_edges": int(amb.sum()), "ambiguous_samples": int(o["amb_samples"].sum()), "band_m": band,
            "invalid_edges": int((valid == 0).sum()), "oracle_s": round(time.perf_counter() - t, 1)}


def timed_steps(step, steps: int, warmup: int, torch, flush) -> float:
    """Seconds per step: CUDA events around each step, L2 flushed before each."""
    for _ in range(warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for s_, e_ in ev:
        flush.zero_()
        s_.record()
        step()
        e_.record()
    torch.cuda.synchronize()
    return sum(s_.elapsed_time(e_) for s_, e_ in ev) / 1e3 / steps


def segment_counts(orc, wl) -> np.ndarray:
    L = orc.lib()
    return np.array([L.oracle_segment_count(a.ctypes.data, b.ctypes.data, a.shape[0], wl.rule, float(wl.range_))
                     for a, b in zip(wl.q0, wl.q1)], np.int64)


def other_workloads_mine(pkg, torch, steps: int = 5, warmup: int = 3) -> dict:
    """Secondary lines: configs 1 and 3 and the config-3 shortcut set, device-timed
    (CUDA events, L2 flushed before every step), through mrpop_validate_*."""
    out = {}
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for name in ("config1", "config3", "config3s"):
        wl = load_workload(pkg, name)
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        q0, q1 = torch.from_numpy(wl.q0).cuda(), torch.from_numpy(wl.q1).cuda()
        n = len(wl.q0)
        v = torch.empty(n, dtype=torch.uint8, device="cuda")
        f = torch.empty(n, dtype=torch.int32, device="cuda")
        ns = torch.empty(n, dtype=torch.int32, device="cuda") if wl.rule else None

        def step():
            pkg.validate(scene, rb, q0, q1, wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_, valid=v,
                         first_hit=f, n_seg=ns)

        dt = timed_steps(step, steps, warmup, torch, flush)
        samples = n * wl.granularity
        if wl.rule:
            # segments up to the first colliding one (the reference's loop stops there) x g
            vv, ff = v.cpu().numpy(), f.cpu().numpy().astype(np.int64)
            nn = ns.cpu().numpy().astype(np.int64)
            segs = np.where(vv == 1, np.maximum(nn, 0), np.where(ff > 0, (ff - 1) // wl.granularity + 1, 0))
            samples = int(segs.sum()) * wl.granularity
        out[wl.name] = {"value": samples / dt, "unit": UNIT, "ms_per_step": dt * 1e3, "edges": n,
                        "granularity": wl.granularity, "steps": steps, "warmup": warmup}
    return out


def other_workloads_reference(pkg, torch, orc, R, flush, steps: int = 3, warmup: int = 1) -> dict:
    """The same secondary lines on the reference's own edge check (harness
    launches of 8 blocks per SM, one edge per block at a time)."""
    out = {}
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for name in ("config1", "config3", "config3s"):
        wl = load_workload(pkg, name)
        kind = R.KIND_SINGLE if wl.arm >= 0 else R.KIND_COMPOSITE
        arms = len(wl.bases)
        if kind == R.KIND_COMPOSITE:
            R.set_bases(arms, wl.bases)
        env = R.make_env(wl.scene)
        q0, q1 = torch.from_numpy(wl.q0).cuda(), torch.from_numpy(wl.q1).cuda()
        n = len(wl.q0)
        res = (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"))

        def step():
            R.validate(env, q0, q1, wl.granularity, kind, wl.rule, wl.range_, arms if kind == R.KIND_COMPOSITE else 1,
                       max(wl.arm, 0), blocks=sms * 8, out=res)

        dt = timed_steps(step, steps, warmup, torch, flush)
        samples = n * wl.granularity
        if wl.rule:
            v, sf = res[0].cpu().numpy(), res[1].cpu().numpy().astype(np.int64)
            samples = int(np.where(v == 1, np.maximum(segment_counts(orc, wl), 0), sf + 1).sum()) * wl.granularity
        out[wl.name] = {"value": samples / dt, "unit": UNIT, "ms_per_step": dt * 1e3, "edges": n,
                        "granularity": wl.granularity, "steps": steps, "warmup": warmup}
    return out


def run_batch(args, world, rank, local, pkg, torch):
    """Config 4: an uneven batch of planning instances (1-5 arms, lognormal
    edge counts, g in {16, 32, 64}, config-1/2 scenes) through one captured
    CUDA graph of the batch kernels (mrpop_batch_*), tuned launch shapes."""
    W = pkg.workloads
    insts = W.config4_instances(n_instances=args.instances, seed=rank)
    sizes = [wl.q0.size for wl in insts]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    n_edges = np.array([len(wl.q0) for wl in insts])
    eoffs = np.concatenate([[0], np.cumsum(n_edges)])
    # one flat buffer per input and output; instances are views into them
    h0 = torch.empty(int(offs[-1]), dtype=torch.float32).pin_memory()
    h1 = torch.empty(int(offs[-1]), dtype=torch.float32).pin_memory()
    for i, wl in enumerate(insts):
        h0[offs[i]:offs[i + 1]] = torch.from_numpy(wl.q0.ravel())
        h1[offs[i]:offs[i + 1]] = torch.from_numpy(wl.q1.ravel())
    d0, d1 = h0.cuda(), h1.cuda()
    dv = torch.empty(int(eoffs[-1]), dtype=torch.uint8, device="cuda")
    df = torch.empty(int(eoffs[-1]), dtype=torch.int32, device="cuda")
    hv = torch.empty(int(eoffs[-1]), dtype=torch.uint8).pin_memory()
    hf = torch.empty(int(eoffs[-1]), dtype=torch.int32).pin_memory()
    items = []
    for i, wl in enumerate(insts):
        dof = wl.q0.shape[1]
        q0 = d0[offs[i]:offs[i + 1]].view(-1, dof)
        q1 = d1[offs[i]:offs[i + 1]].view(-1, dof)
        items.append((pkg.Scene(wl.scene), pkg.RobotSet(len(wl.bases), wl.bases), q0, q1, wl.granularity, wl.flags,
                      wl.arm, dv[eoffs[i]:eoffs[i + 1]], df[eoffs[i]:eoffs[i + 1]]))
    samples = int(sum(len(wl.q0) * wl.granularity for wl in insts))
    batch = pkg.Batch(items)
    batch.run()
    batch.tune()
    batch.capture()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        flush.zero_()
        batch.launch()
    torch.cuda.synchronize()
    ref_v = dv.clone()
    # per-instance plain calls on the same buffers: the results must be equal
    for it in items:
        pkg.validate(*it[:7], valid=it[7], first_hit=it[8])
    torch.cuda.synchronize()
    assert torch.equal(ref_v, dv), "batch and per-instance results differ"
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    pkg.kernel_times()
    barrier(world)
    torch.cuda.synchronize()
    for s_, e_ in ev:
        flush.zero_()
        s_.record(stream)
        batch.launch()
        e_.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    t_total = max_over_ranks(sum(s_.elapsed_time(e_) for s_, e_ in ev) / 1e3, world)
    value = world * samples * args.steps / t_total
    # the same work as one plain call per instance (no graph, no batching)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(max(1, args.steps // 2)):
        for it in items:
            pkg.validate(*it[:7], valid=it[7], first_hit=it[8])
    torch.cuda.synchronize()
    loop_value = samples * max(1, args.steps // 2) / (time.perf_counter() - t)
    # end to end: host inputs in, verdicts out, every step.  Staged: copies to
    # and from the device buffers around the graph.  In place: a second batch
    # whose items are views of the page-locked host buffers, which its kernels
    # read and write over NVLink-C2C.
    barrier(world)
    t = time.perf_counter()
    for _ in range(args.steps):
        d0.copy_(h0, non_blocking=True)
        d1.copy_(h1, non_blocking=True)
        batch.launch()
        hv.copy_(dv, non_blocking=True)
        hf.copy_(df, non_blocking=True)
        torch.cuda.synchronize()
    dt_staged = max_over_ranks(time.perf_counter() - t, world)
    host_items = []
    for i, it in enumerate(items):
        dof = insts[i].q0.shape[1]
        host_items.append(it[:2] + (h0[offs[i]:offs[i + 1]].view(-1, dof), h1[offs[i]:offs[i + 1]].view(-1, dof))
                          + it[4:7] + (hv[eoffs[i]:eoffs[i + 1]], hf[eoffs[i]:eoffs[i + 1]]))
    hbatch = pkg.Batch(host_items)
    hbatch.tune()
    hbatch.capture()
    hbatch.launch()
    torch.cuda.synchronize()
    assert torch.equal(hv, ref_v.cpu()) and torch.equal(hf, df.cpu()), "in-place host batch and device batch differ"
    barrier(world)
    t = time.perf_counter()
    for _ in range(args.steps):
        hbatch.launch()
        torch.cuda.synchronize()
    dt = max_over_ranks(time.perf_counter() - t, world)
    groups = batch.info()
    arms_hist = np.bincount([len(wl.bases) if wl.arm < 0 else 1 for wl in insts], minlength=6)[1:].tolist()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators)",
        "config": {"workload": f"config4_uneven_batch_{len(insts)}_instances", "instances": len(insts),
                   "edges": int(eoffs[-1]), "samples": samples, "arms_histogram_1_to_5": arms_hist,
                   "granularities": sorted({wl.granularity for wl in insts}),
                   "kernel_groups": batch.shapes(),
                   "launch": "one CUDA graph of the batch kernels (tuned chunk size, warps per CTA and grid)",
                   "per_instance_plain_calls_value": loop_value,
                   "l2": "flushed (256 MiB write) before every step",
                   "parallelism": f"replica x{world}, independent batches"},
        "gpu_launches": 2 * len(groups) * args.steps,
        "clocks": clk,
        "e2e": {"value": world * samples * args.steps / dt, "unit": UNIT,
                "h2d_bytes_per_step": int(h0.numel() * 4 * 2), "d2h_bytes_per_step": int(hv.numel() * 5),
                "path": "mrpop_batch_launch of a batch whose items are page-locked host buffers (endpoints read, "
                        "verdicts written in place over NVLink-C2C), synchronised per step",
                "staged_value": world * samples * args.steps / dt_staged,
                "staged_path": "pinned host buffers -> device copies, mrpop_batch_launch, verdicts -> host copies"},
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_serving(args, world, rank, local, pkg, torch):
    """Served planning stream: Poisson arrivals at --rate for --duration
    seconds, each query a planning run (2-5 Pandas, a fresh seeded scene from
    the single-arm or bin-picking generator, collision-free start and goal) whose
    validation steps go through one validation service (mrpop_server_*), so the
    steps of concurrent queries share waves of batch launches.  The first
    --isolated queries are also solved alone on the same service, one at a
    time, for the latency comparison and the same-result check."""
    P, S = pkg.planner, pkg.serving
    flags = pkg.CHECK_ENV | pkg.CHECK_SELF

    def collision_free(scene_arrays, bases, q):
        scene = pkg.Scene(scene_arrays)
        rb = pkg.RobotSet(len(bases), bases)
        d = torch.from_numpy(np.ascontiguousarray(q)).cuda()
        v, _ = pkg.validate(scene, rb, d, d, 1, flags)
        torch.cuda.synchronize()
        return v.cpu().numpy().astype(bool)

    n = max(1, int(round(args.rate * args.duration)))
    t0 = time.perf_counter()
    queries = P.make_queries(n, seed=rank, collision_free=collision_free)
    gen_s = time.perf_counter() - t0
    if args.planner == "drrt":
        settings = S.served_drrt_settings()
        planner_desc = ("the reference's dRRT / AO-x (mrpop_session_drrt): per-arm roadmaps, direction oracle, "
                        "PHS sampling, first pass + 5 optimising passes, B-spline and shortcut simplification")
        settings_desc = pkg.drrt.settings_dict(settings)
    else:
        settings = P.PlanSettings()
        planner_desc = "batched bidirectional RRT with connect checks and shortcut passes (this library's compact planner)"
        settings_desc = settings.__dict__
    streams = args.streams or (S.SERVED_DRRT_STREAMS if args.planner == "drrt" else 4)
    clients = args.clients or (S.SERVED_DRRT_CLIENTS if args.planner == "drrt" else 256)
    server = pkg.Server(budget_bytes=2 << 30, streams=streams, fused_edges=args.fused_edges)
    S.isolated(server, queries[:min(3, n)], settings)  # warm-up (first-use set-up of the library)
    m = min(args.isolated, n)
    alone = S.isolated(server, queries[:m], settings)
    before = server.stats()
    barrier(world)
    clocks = ClockSampler(local, util=True)
    clocks.start()
    cpu0 = host_cpu_times()
    t0 = time.perf_counter()
    served = S.stream(server, queries, args.rate, settings, seed=rank, clients=clients)
    wall = time.perf_counter() - t0
    cpu1 = host_cpu_times()
    clk = clocks.stop()
    after = server.stats()
    cpu_busy = (cpu1[0] - cpu0[0]) / max(1, cpu1[1] - cpu0[1]) if cpu0 and cpu1 else None
    wall = max_over_ranks(wall, world)
    same = sum(S.same_result(a.result, b.result) for a, b in zip(alone, served[:m]))
    sv, iso = S.summary(served), S.summary(alone)
    samples = sv["edges"] * int(settings.granularity)  # samples per segment; segmented steps check more
    server.close()
    if rank != 0:
        return
    out = {"metric": "served p99 plan latency", "value": sv["p99_ms"], "unit": "ms", "n_gpus": world,
           "steps": n, "warmup": 3, "ms_per_step": sv["mean_ms"], "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded scenes, start/goal rejection-sampled collision-free)",
           "config": {"workload": "config5_served_planning", "rate_qps": args.rate, "duration_s": args.duration,
                      "queries": n, "arms": "2-5 (uniform)", "scenes": "single-arm or bin-picking generator",
                      "planner": planner_desc,
                      "settings": settings_desc, "service": f"mrpop_server: 2 GiB budget, {streams} streams, {clients} client threads",
                      "query_generation_s": round(gen_s, 2)},
           "latency": {"served_p50_ms": sv["p50_ms"], "served_p99_ms": sv["p99_ms"],
                       "isolated_p50_ms": iso["p50_ms"], "isolated_p99_ms": iso["p99_ms"],
                       "isolated_queries": m,
                       "p99_ratio": sv["p99_ms"] / iso["p99_ms"] if iso["p99_ms"] else None},
           "solve_rate": {"served": sv["solve_rate"], "isolated": iso["solve_rate"],
                          "served_same_queries": S.summary(served[:m])["solve_rate"]},
           "mean_cost": {"served": sv["mean_cost"], "isolated": iso["mean_cost"]},
           "same_result_alone_and_mixed": f"{same}/{m}",
           "phase_mean_ms": {"served": sv["phase_mean_ms"], "isolated": iso["phase_mean_ms"]},
           "throughput": {"queries_per_s": n / wall, "steps": sv["steps"], "edges": sv["edges"],
                          "edge_samples_per_s_lower_bound": samples / wall,
                          "waves": after["waves"] - before["waves"],
                          "steps_per_wave": (after["steps"] - before["steps"]) / max(1, after["waves"] - before["waves"]),
                          "max_wave_steps": after["max_wave_steps"],
                          "max_waves_in_flight": after["max_waves_in_flight"],
                          "admission_waits": after["admission_waits"],
                          "step_queue_mean_us": (after["queue_ns"] - before["queue_ns"]) / 1e3 /
                          max(1, after["steps"] - before["steps"]),
                          "step_flight_mean_us": (after["flight_ns"] - before["flight_ns"]) / 1e3 /
                          max(1, after["steps"] - before["steps"]),
                          "wave_device_mean_us": (after["device_ns"] - before["device_ns"]) / 1e3 /
                          max(1, after["waves"] - before["waves"])},
           "gpu_launches": after["kernel_launches"] - before["kernel_launches"],
           "host_cpu_busy": {"fraction": cpu_busy, "cores": os.cpu_count()},
           "clocks": clk,
           "e2e": {"value": sv["p99_ms"], "unit": "ms", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                   "path": "host wall clock from each query's arrival to its plan; endpoints and verdicts in "
                           "page-locked host buffers read and written in place by the kernels"}}
    print(json.dumps(out), flush=True)


def planner_summary(rows: list[dict]) -> dict:
    """Solve rate, costs and latencies of a list of per-problem results."""
    solved = [r for r in rows if r["solved"]]
    k = np.array([r["kernel_ns"] for r in rows if "kernel_ns" in r], np.float64) / 1e6
    w = np.array([r["wall_ns"] for r in rows if "wall_ns" in r], np.float64) / 1e6
    c = np.array([r["cost"] for r in solved], np.float64)
    return {"problems": len(rows), "solved": len(solved), "solve_rate": len(solved) / max(1, len(rows)),
            "cost_median": float(np.median(c)) if len(c) else None,
            "cost_mean": float(c.mean()) if len(c) else None,
            "kernel_ms_p50": float(np.percentile(k, 50)) if len(k) else None,
            "kernel_ms_p99": float(np.percentile(k, 99)) if len(k) else None,
            "wall_ms_p50": float(np.percentile(w, 50)) if len(w) else None,
            "wall_ms_p99": float(np.percentile(w, 99)) if len(w) else None}


def planner_line(args, impl: str, rows: list[dict], extra: dict) -> dict:
    sm = planner_summary(rows)
    arms = 4 if args.workload == "planner4" else 5
    out = {"metric": "dRRT/AO-x solve latency p50 (kernel_ns, the reference's timer)", "value": sm["kernel_ms_p50"],
           "unit": "ms", "n_gpus": 1, "steps": len(rows), "warmup": 1, "ms_per_step": sm["kernel_ms_p50"],
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "the reference's benchmark problems (scripts/panda_{four,five}_problems.json, converted fixture)",
           "config": {"workload": f"planner_{arms}panda_{len(rows)}_problems",
                      "settings": "evaluate_mr: 300 attempts per iteration, g=64, range 2.0, 3 AO-x passes, "
                                  "8 roadmap blocks per arm"},
           "planner": sm, "e2e": {"value": sm["wall_ms_p50"], "unit": "ms", "h2d_bytes_per_step": None,
                                  "d2h_bytes_per_step": None,
                                  "path": "host wall clock of one whole solve call per problem"}}
    if impl == "reference":
        out["impl"] = "reference"
    out["config"].update(extra)
    return out


def run_planner(args, pkg, torch):
    """The reference's planner rebuilt on the batched validator (dRRT::solve,
    mrpop_drrt_solve) over the reference's benchmark problems."""
    arms = 4 if args.workload == "planner4" else 5
    z = np.load(ROOT / "tests" / "golden" / "problems.npz")
    n = min(args.problems, int(z[f"n{arms}"]))
    st = pkg.drrt.evaluate_settings()
    rb = pkg.RobotSet(arms)  # the reference's compiled-in bases, as its driver places the arms
    # warm-up: first-use set-up of the library and the device
    pkg.drrt.solve(pkg.Scene(pkg.SceneArrays(cuboids=z[f"a{arms}_p0_boxes"])), rb, z[f"a{arms}_p0_start"],
                   z[f"a{arms}_p0_goal"], pkg.drrt.evaluate_settings(rrtc_iter=1))
    clocks = ClockSampler(0)
    clocks.start()
    rows = []
    for p in range(n):
        scene = pkg.Scene(pkg.SceneArrays(cuboids=z[f"a{arms}_p{p}_boxes"]))
        t0 = time.perf_counter_ns()
        r = pkg.drrt.solve(scene, rb, z[f"a{arms}_p{p}_start"], z[f"a{arms}_p{p}_goal"], st)
        wall = time.perf_counter_ns() - t0
        rows.append({"problem": p, "solved": r.solved, "cost": r.cost, "kernel_ns": r.stats["kernel_ns"],
                     "wall_ns": wall, "iterations": r.stats["iterations"], "edges": r.stats["edges_validated"],
                     "validate_ns": r.stats["validate_ns"], "nn_ns": r.stats["nn_ns"],
                     "roadmap_ns": r.stats["roadmap_ns"], "oracle_ns": r.stats["oracle_ns"],
                     "validate_calls": r.stats["validate_calls"], "check_ns": r.stats["check_ns"],
                     "check_calls": r.stats["check_calls"]})
    clk = clocks.stop()
    edges = sum(r["edges"] for r in rows)
    out = planner_line(args, "mine", rows, {"validated_edges": edges,
                                            "validate_share_of_kernel_ns": sum(r["validate_ns"] for r in rows) /
                                            max(1, sum(r["kernel_ns"] for r in rows)),
                                            "nn_share_of_kernel_ns": sum(r["nn_ns"] for r in rows) /
                                            max(1, sum(r["kernel_ns"] for r in rows)),
                                            "phase_mean_ms": {k: round(float(np.mean([r[k + "_ns"] for r in rows])) / 1e6, 2)
                                                              for k in ("kernel", "validate", "nn", "roadmap", "oracle")},
                                            "validate_calls_mean": float(np.mean([r["validate_calls"] for r in rows])),
                                            "check_ms_mean": {k: round(float(np.mean([r["check_ns"][k] for r in rows])) / 1e6, 2)
                                                              for k in pkg.drrt.CHECK_KINDS},
                                            "check_calls_mean": {k: float(np.mean([r["check_calls"][k] for r in rows]))
                                                                 for k in pkg.drrt.CHECK_KINDS}})
    out["clocks"] = clk
    out["gpu_launches"] = None
    out["per_problem"] = [{k: r[k] for k in ("problem", "solved", "cost", "kernel_ns")} for r in rows]
    print(json.dumps(out), flush=True)


def run_reference_planner(args, torch):
    """The reference's own planner kernels (oracle/ref_planner.py) on the same problems."""
    import subprocess as sp
    import tempfile
    arms = 4 if args.workload == "planner4" else 5
    with tempfile.TemporaryDirectory() as d:
        out_path = Path(d) / "ref.jsonl"
        sp.run([sys.executable, "-m", "oracle.ref_planner_eval", str(arms), str(out_path), "--first",
                str(args.problems)], cwd=str(ROOT), check=False, stdout=sp.DEVNULL)
        rows = [json.loads(l) for l in open(out_path)] if out_path.exists() else []
    line = planner_line(args, "reference", rows, {
        "harness": "the reference's pop_planner.cu / path_processing.cu / path_simplification.cu compiled "
                   "unmodified for sm_103a; its host loop restated with bounds (oracle/ref_planner.py)"})
    line["per_problem"] = [{k: r.get(k) for k in ("problem", "solved", "cost", "kernel_ns", "stopped")} for r in rows]
    line["gpu_launches"] = None
    print(json.dumps(line), flush=True)


def run_mine(args, world, rank, local):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    lib = pkg.build.lib_path()
    if not lib.exists():
        pkg.build.build()
    pkg.library()
    if args.workload == "config5":
        return run_serving(args, world, rank, local, pkg, torch)
    if args.workload == "config4":
        return run_batch(args, world, rank, local, pkg, torch)
    if args.workload in ("planner4", "planner5"):
        return run_planner(args, pkg, torch) if rank == 0 else None
    wl = load_workload(pkg, args.workload, args.edges)
    scene = pkg.Scene(wl.scene)
    robots = pkg.RobotSet(len(wl.bases), wl.bases)
    q0 = torch.from_numpy(wl.q0).cuda()
    q1 = torch.from_numpy(wl.q1).cuda()
    n = len(wl.q0)
    samples = n * wl.granularity
    valid = torch.empty(n, dtype=torch.uint8, device="cuda")
    first = torch.empty(n, dtype=torch.int32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    nseg = torch.empty(n, dtype=torch.int32, device="cuda") if wl.rule else None

    def step():
        pkg.validate(scene, robots, q0, q1, wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_, valid=valid,
                     first_hit=first, n_seg=nseg)

    if wl.rule:
        # segmented rule: the samples a validation checks are the segments up
        # to the first colliding one (the reference's loop stops there) x g
        step()
        torch.cuda.synchronize()
        v, f, ns = valid.cpu().numpy(), first.cpu().numpy().astype(np.int64), nseg.cpu().numpy().astype(np.int64)
        segs = np.where(v == 1, np.maximum(ns, 0), np.where(f > 0, (f - 1) // wl.granularity + 1, 0))
        samples = int(segs.sum()) * wl.granularity
    flops_launch = float(pkg.count_flops(scene, robots, q0, q1, wl.granularity, wl.flags, wl.arm, wl.rule,
                                         wl.range_).sum().item())
    broad_launch = pkg.broad_flops_per_sample(scene, robots, wl.flags, wl.arm) * samples
    flops = {"fused": flops_launch, "broad": broad_launch, "narrow": flops_launch - broad_launch}
    if wl.rule:  # the tail kernel does both phases of the few edges with more segments than the rounds
        flops["fused"] = 0.0
    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    for s, e in ev:
        flush.zero_()
        s.record(stream)
        step()
        e.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in ev]
    # per-kernel device times for the roofline: the same steps again with the
    # library's event pairs around every launch (kept out of the timed region,
    # whose host-side cost they would add to short steps)
    pkg.kernel_times()
    pkg.kernel_timing(True)
    for _ in ev:
        flush.zero_()
        step()
    torch.cuda.synchronize()
    pkg.kernel_timing(False)
    kt = pkg.kernel_times()
    t_total = max_over_ranks(sum(step_ms) / 1e3, world)
    value = replica_throughput(samples, args.steps, [t_total], 1) * world
    assert scene.status() == 0, "device status word set during the bench"

    peak = fp32_peak(pkg, torch)
    arms = int(len(wl.bases)) if wl.arm < 0 else 1
    spl = 2 if wl.granularity > 32 else 1
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators)",
        "config": workload_config(wl, {"parallelism": f"replica x{world}, independent edge batches"}),
        "gpu_launches": sum(v[0] for v in kt.values()),
        "roofline": roofline(kt, flops, peak, args.workload, arms, spl, args.steps, (clk or {}).get("sm_mhz")),
        "clocks": clk,
    }
    out["roofline"]["step_traffic"] = step_traffic(kt, args.workload, wl.q0.nbytes + wl.q1.nbytes + n * 5, args.steps)
    if not args.no_e2e:
        ws = pkg.Workspace()
        hq0 = torch.from_numpy(wl.q0).pin_memory()
        hq1 = torch.from_numpy(wl.q1).pin_memory()
        hv = torch.empty(n, dtype=torch.uint8).pin_memory()
        hf = torch.empty(n, dtype=torch.int32).pin_memory()
        a0, a1, av, af = hq0.numpy(), hq1.numpy(), hv.numpy(), hf.numpy()
        for _ in range(2):
            ws.validate(scene, robots, a0, a1, wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_, valid=av,
                        first_hit=af)
        barrier(world)
        t = time.perf_counter()
        for _ in range(args.steps):
            ws.validate(scene, robots, a0, a1, wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_, valid=av,
                        first_hit=af)
        dt = max_over_ranks(time.perf_counter() - t, world)
        out["e2e"] = {"value": world * samples * args.steps / dt, "unit": UNIT,
                      "h2d_bytes_per_step": int(a0.nbytes + a1.nbytes), "d2h_bytes_per_step": int(av.nbytes + af.nbytes),
                      "path": "mrpop_validate_edges_host with pinned host buffers, which the kernels read "
                              "(endpoints) and write (verdicts) in place over NVLink-C2C; sync inside"}
        assert np.array_equal(av, valid.cpu().numpy())
    if rank == 0 and world == 1 and not args.no_others and args.workload == "config2" and not args.edges:
        out["other_workloads"] = other_workloads_mine(pkg, torch)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as orc
        out["cpu_baseline"] = cpu_baseline(orc, wl, min(n, 65536))
        if not args.no_parity:
            # outside the timed region: the last timed step's verdicts against the oracle
            out["parity"] = parity_counts(orc, pkg, torch, wl, valid.cpu().numpy(), first.cpu().numpy())
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_reference_batch(args, pkg, torch, ref_runner, out):
    """Config 4 on the reference's kernels: one harness launch per instance
    (the reference validates one planning instance at a time), over the 4- and
    5-arm instances -- its composite kernels exist for those arm counts only,
    and its single-arm form uses its own fixed bases."""
    W = pkg.workloads
    insts = [wl for wl in W.config4_instances(n_instances=args.instances, seed=0)
             if len(wl.bases) in (4, 5) and wl.arm < 0]
    R = ref_runner.RefHarness()
    runs = []
    for wl in insts:
        runs.append((wl, R.make_env(wl.scene), torch.from_numpy(wl.q0).cuda(), torch.from_numpy(wl.q1).cuda()))
    samples = sum(len(wl.q0) * wl.granularity for wl, *_ in runs)
    sms = torch.cuda.get_device_properties(0).multi_processor_count

    def step():
        for wl, env, q0, q1 in runs:
            R.set_bases(len(wl.bases), wl.bases)
            R.validate(env, q0, q1, wl.granularity, R.KIND_COMPOSITE, 0, 0.0, len(wl.bases), 0, blocks=sms * 8)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    value = samples * args.steps / dt
    out.update({"value": value, "ms_per_step": dt / args.steps * 1e3, "gpu_launches": len(runs) * args.steps,
                "config": {"workload": f"config4_uneven_batch_{args.instances}_instances",
                           "subset": f"{len(runs)} instances with 4 or 5 arms", "samples": samples,
                           "launch": f"one reference harness launch per instance, {sms * 8} blocks"},
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": None, "kind": "reference",
                                 "sample": "the reference's own CUDA edge check per instance on this GB300"}})
    out["e2e"] = {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(out), flush=True)


def run_reference(args, world, rank, local):
    if rank != 0:
        return
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from oracle import oracle as orc
    from oracle import ref_runner
    if args.workload in ("planner4", "planner5"):
        from oracle import ref_planner
        if not ref_planner.available():
            print(json.dumps({"impl": "reference", "metric": "dRRT/AO-x solve latency p50", "unit": "ms",
                              "higher_is_better": False,
                              "unavailable": "reference planner cubin not built (oracle/_ref)"}), flush=True)
            return
        return run_reference_planner(args, torch)
    if args.workload == "config5":
        print(json.dumps({"impl": "reference", "metric": "served p99 plan latency", "unit": "ms",
                          "higher_is_better": False,
                          "unavailable": "the reference serves no concurrent queries (one dRRT::solve per process), "
                                         "and its planner executables do not build here (CMake FetchContent of "
                                         "nlohmann_json needs the network; Eigen is absent)"}), flush=True)
        return
    if args.workload == "config4":
        out = {"metric": METRIC, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded generators)", "impl": "reference"}
        if not ref_runner.available():
            out["unavailable"] = "reference harness not built (oracle/_ref)"
            print(json.dumps(out), flush=True)
            return
        return run_reference_batch(args, pkg, torch, ref_runner, out)
    wl = load_workload(pkg, args.workload)
    n = len(wl.q0)
    samples = n * wl.granularity
    out = {"metric": METRIC, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded generators)", "impl": "reference"}
    if ref_runner.available() and args.workload in ("config1", "config2", "config3", "config3s"):
        R = ref_runner.RefHarness()
        kind = R.KIND_SINGLE if wl.arm >= 0 else R.KIND_COMPOSITE
        arms = len(wl.bases)
        if kind == R.KIND_COMPOSITE:
            R.set_bases(arms, wl.bases)
        env = R.make_env(wl.scene)
        q0 = torch.from_numpy(wl.q0).cuda()
        q1 = torch.from_numpy(wl.q1).cuda()
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        blocks = sms * 8
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
        res = (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"))

        def step():
            R.validate(env, q0, q1, wl.granularity, kind, wl.rule, wl.range_, arms if kind == R.KIND_COMPOSITE else 1,
                       max(wl.arm, 0), blocks=blocks, out=res)

        if wl.rule:
            # segmented rule: segments up to the first failing one, x g
            step()
            torch.cuda.synchronize()
            v, sf = res[0].cpu().numpy(), res[1].cpu().numpy().astype(np.int64)
            L = orc.lib()
            ns = np.array([L.oracle_segment_count(a.ctypes.data, b.ctypes.data, a.shape[0], wl.rule, float(wl.range_))
                           for a, b in zip(wl.q0, wl.q1)], np.int64)
            samples = int(np.where(v == 1, np.maximum(ns, 0), sf + 1).sum()) * wl.granularity

        for _ in range(args.warmup):
            flush.zero_()
            step()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        clocks = ClockSampler(local)
        clocks.start()
        torch.cuda.synchronize()
        for s, e in ev:
            flush.zero_()
            s.record()
            step()
            e.record()
        torch.cuda.synchronize()
        clk = clocks.stop()
        t = sum(s.elapsed_time(e) for s, e in ev) / 1e3
        value = samples * args.steps / t
        out.update({"value": value, "ms_per_step": t / args.steps * 1e3, "clocks": clk, "gpu_launches": args.steps,
                    "config": workload_config(wl, {"parallelism": "single GPU", "launch": f"{blocks} blocks x "
                                                                                         f"{4 * wl.granularity} threads, one edge per block at a time"}),
                    "cpu_baseline": {"value": value, "unit": UNIT, "cores": None, "kind": "reference",
                                     "sample": "the reference's own CUDA edge check (fkcc_single_buffer*, "
                                               "utils.cuh:447-686) compiled from its sources for sm_103a and run "
                                               "on this GB300 over the full workload"}})
        if args.workload == "config2" and not args.no_others:
            out["other_workloads"] = other_workloads_reference(pkg, torch, orc, R, flush)
    else:
        threads = orc.max_threads()
        m = min(n, 4096)
        orc.validate(wl.scene, wl.bases, wl.q0[:64], wl.q1[:64], wl.granularity, wl.flags, wl.arm, threads=threads)
        times = []
        for _ in range(max(1, min(args.steps, 3))):
            t = time.perf_counter()
            orc.validate(wl.scene, wl.bases, wl.q0[:m], wl.q1[:m], wl.granularity, wl.flags, wl.arm, threads=threads)
            times.append(time.perf_counter() - t)
        value = m * wl.granularity / (sum(times) / len(times))
        out.update({"value": value, "ms_per_step": None, "gpu_launches": 0,
                    "config": workload_config(wl, {"parallelism": f"{threads} host threads"}),
                    "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                                     "sample": f"reference build absent: CPU restatement over the first {m} edges"}})
    out["e2e"] = {"value": out["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup()
    try:
        if args.impl == "reference":
            run_reference(args, world, rank, local)
        else:
            run_mine(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            if dist.is_initialized():
                dist.destroy_process_group()


if __name__ == "__main__":
    main()
