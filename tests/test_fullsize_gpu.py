"""Full-size parity on the benchmarked workloads.

The 4-arm workload (65,536 edges x 32 samples), the 5-arm workload (262,144
edges x 64 samples) and the 5-arm shortcut set (1,024 paths x 64 pairs, the
shortcut segmentation with range 2.0) are validated whole by this library and
by the reference's own edge check (fkcc_single_buffer<Panda_four/five>,
src/planning/utils.cuh:447-534, through oracle/ref_harness.cu).  Every edge
whose verdict (or failing segment) differs must be ambiguous: one of its
checked samples has a deciding minimum signed distance within 1e-5 m of zero
in FP64 (the oracle's truth).  Against the oracle (host sinf/cosf), the few
edges that differ without being ambiguous are checked again with the device's
__sinf/__cosf values replayed, which must then agree bit for bit.  The counts
of differing edges, ambiguous edges and ambiguous samples are printed and,
when MRPOP_PARITY_OUT names a file, written there as JSON lines.
"""
import json
import os
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BAND = 1e-5  # metres: verdicts may differ only where a deciding distance is this close to zero


@pytest.fixture(scope="module")
def ref(cuda):
    from oracle import ref_runner
    if not ref_runner.available():
        pytest.skip("reference harness cubin not built (reference sources absent when built)")
    return ref_runner.RefHarness()


def _report(row):
    print("PARITY", json.dumps(row))
    out = os.environ.get("MRPOP_PARITY_OUT")
    if out:
        with open(out, "a") as f:
            f.write(json.dumps(row) + "\n")


@pytest.mark.parametrize("name", ["config2", "config3", "config3s"])
def test_full_workload_vs_reference(cuda, pkg, orc, ref, name):
    W = pkg.workloads
    wl = {"config2": W.config2, "config3": W.config3, "config3s": W.config3_shortcuts}[name]()
    arms = len(wl.bases)
    n, g = len(wl.q0), wl.granularity
    ref.set_bases(arms, wl.bases)
    scene = pkg.Scene(wl.scene)
    rb = pkg.RobotSet(arms, wl.bases)
    d0 = cuda.from_numpy(wl.q0).cuda()
    d1 = cuda.from_numpy(wl.q1).cuda()
    valid, first = pkg.validate(scene, rb, d0, d1, g, wl.flags, wl.arm, wl.rule, wl.range_)[:2]
    env = ref.make_env(wl.scene)
    rv, rs = ref.validate(env, d0, d1, g, ref.KIND_COMPOSITE, wl.rule, wl.range_, arms, 0,
                          blocks=cuda.cuda.get_device_properties(0).multi_processor_count * 8)
    cuda.cuda.synchronize()
    valid, first = valid.cpu().numpy(), first.cpu().numpy()
    rv, rs = rv.cpu().numpy(), rs.cpu().numpy()
    assert scene.status() == 0
    # the reference reports the failing segment; this library the first colliding sample
    seg = np.where(first > 0, (first - 1) // g, -1)
    diff_ref = (valid != rv) | (seg != rs)

    t = time.perf_counter()
    o = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, g, wl.flags, wl.arm, wl.rule, wl.range_, band=BAND,
                     threads=orc.max_threads(), count_ambiguous=True)
    oracle_s = time.perf_counter() - t
    amb = o["ambiguous"].astype(bool)
    diff_oracle = (valid != o["valid"]) | (first != o["first_hit"])
    # edges that differ from the host-trig oracle without being ambiguous: the
    # oracle again with the device's trig values replayed
    idx = np.nonzero(diff_oracle & ~amb)[0]
    replay_differ = 0
    if len(idx):
        def dev_trig(x):
            c, s = pkg.debug_trig(cuda.from_numpy(x).cuda())
            cuda.cuda.synchronize()
            return c.cpu().numpy(), s.cpu().numpy()
        r = orc.validate_with_trig(wl.scene, wl.bases, wl.q0[idx], wl.q1[idx], g, wl.flags, wl.arm, wl.rule,
                                   wl.range_, dev_trig)
        replay_differ = int(((valid[idx] != r["valid"]) | (first[idx] != r["first_hit"])).sum())
    row = {"workload": wl.name, "edges": n, "granularity": g, "invalid_edges": int((valid == 0).sum()),
           "edges_differ_vs_reference": int(diff_ref.sum()),
           "edges_differ_vs_reference_unambiguous": int((diff_ref & ~amb).sum()),
           "edges_differ_vs_oracle": int(diff_oracle.sum()),
           "edges_differ_vs_oracle_unambiguous": int((diff_oracle & ~amb).sum()),
           "edges_differ_vs_oracle_after_device_trig_replay": replay_differ,
           "ambiguous_edges": int(amb.sum()), "ambiguous_samples": int(o["amb_samples"].sum()),
           "band_m": BAND, "oracle_s": round(oracle_s, 1),
           "oracle_trig": "host sinf/cosf (the device uses __sinf/__cosf)"}
    _report(row)
    assert row["edges_differ_vs_reference_unambiguous"] == 0, row
    assert row["edges_differ_vs_oracle_after_device_trig_replay"] == 0, row
