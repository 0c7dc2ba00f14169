"""Capture golden vectors from the reference's own edge-check device code.

Runs on a CUDA machine where oracle/_ref/ref_harness.cubin exists (built from
the reference sources by oracle/build.py).  For a set of small seeded cases it
records the inputs, the reference's verdicts (valid + failing segment) and,
for FK, the reference's sphere centres, plus the device's __cosf/__sinf values
of every joint angle the cases use (the hardware approximation the reference
calls; the CPU oracle replays them through its trig table).  Output:
tests/golden/ref_golden.npz (or the path given as argument 1).

  python tests/golden/make_ref_golden.py [out.npz]
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))


def main(out_path=None):
    import torch

    import __graft_entry__ as ge
    pkg = ge.load_package()
    W = pkg.workloads
    from oracle import oracle as orc
    from oracle import ref_runner
    R = ref_runner.RefHarness()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    out = {}
    samples_all = []

    def add_case(name, scene, bases, q0, q1, g, kind, rule, range_, num_robot, robot_id, flags, arm):
        if kind != R.KIND_SINGLE and num_robot in (4, 5):
            R.set_bases(num_robot, bases)
        env = R.make_env(scene)
        v, sf = R.validate(env, dev(q0), dev(q1), g, kind, rule, range_, num_robot, robot_id)
        torch.cuda.synchronize()
        out[f"{name}_q0"], out[f"{name}_q1"] = q0, q1
        out[f"{name}_bases"] = np.asarray(bases, np.float32)
        for k, a in scene.__dict__.items():
            if len(a):
                out[f"{name}_scene_{k}"] = a
        out[f"{name}_meta"] = np.array([g, flags, arm, rule, range_], np.float64)
        out[f"{name}_valid"] = v.cpu().numpy().astype(np.uint8)
        out[f"{name}_segfail"] = sf.cpu().numpy().astype(np.int32)
        samples_all.append(orc.edge_samples(q0, q1, g, rule, range_).ravel())

    rng = np.random.default_rng(2024)
    sc1 = W.scene_config1(0)
    q0, q1 = W.random_edges(rng, 96, 1, 1.0)
    add_case("single", sc1, np.eye(4, dtype=np.float32)[None], q0, q1, 32, R.KIND_SINGLE, 0, 0.0, 1, 0,
             pkg.CHECK_ENV | pkg.CHECK_SELF, 0)
    sc2, b2 = W.scene_config2(0), W.bases_config2()
    q0, q1 = W.random_edges(rng, 48, 4, 1.5)
    add_case("quad", sc2, b2, q0, q1, 32, R.KIND_COMPOSITE, 0, 0.0, 4, 0, pkg.CHECK_ENV | pkg.CHECK_SELF, -1)
    q0, q1 = W.random_edges(rng, 48, 4, 1.5)
    add_case("quad_extend", sc2, b2, q0, q1, 32, R.KIND_EXTEND, 0, 0.0, 4, 0, pkg.CHECK_SELF, -1)
    sc3, b3 = W.scene_config3(0), W.bases_config3()
    q0, q1 = W.random_edges(rng, 16, 5, 1.5)
    add_case("five", sc3, b3, q0, q1, 64, R.KIND_COMPOSITE, 0, 0.0, 5, 0, pkg.CHECK_ENV | pkg.CHECK_SELF, -1)
    q0, q1 = W.random_edges(rng, 16, 4, 3.0)
    add_case("quad_connect", sc2, b2, q0, q1, 16, R.KIND_COMPOSITE, 1, 0.5, 4, 0, pkg.CHECK_ENV | pkg.CHECK_SELF, -1)
    q0, q1 = W.random_edges(rng, 16, 5, 4.0)
    add_case("five_shortcut", sc3, b3, q0, q1, 16, R.KIND_COMPOSITE, 3, 2.0, 5, 0, pkg.CHECK_ENV | pkg.CHECK_SELF,
             -1)
    q0, q1 = W.random_edges(rng, 16, 4, 3.0)
    add_case("quad_bspline", sc2, b2, q0, q1, 16, R.KIND_COMPOSITE, 2, 1.0, 4, 0, pkg.CHECK_ENV | pkg.CHECK_SELF, -1)

    # FK: reference sphere centres for single-arm and composite layouts
    qf = W.random_configs(rng, 64, 1)
    for det in (0, 1):
        out[f"fk1_d{det}"] = R.fk(dev(qf), 0, 1, 0, bool(det)).cpu().numpy()
    out["fk1_q"] = qf
    R.set_bases(4, b2)
    qf4 = W.random_configs(rng, 32, 4)
    for det in (0, 1):
        out[f"fk4_d{det}"] = R.fk(dev(qf4), 4, detailed=bool(det)).cpu().numpy()
    out["fk4_q"] = qf4
    out["fk4_bases"] = b2
    samples_all += [qf.ravel(), qf4.ravel()]

    x = np.unique(np.concatenate(samples_all).astype(np.float32).view(np.uint32)).view(np.float32)
    c, s = pkg.debug_trig(dev(x))
    torch.cuda.synchronize()
    out["trig_x"], out["trig_cos"], out["trig_sin"] = x, c.cpu().numpy(), s.cpu().numpy()
    out["cases"] = np.array(["single", "quad", "quad_extend", "five", "quad_connect", "five_shortcut",
                             "quad_bspline"])
    path = Path(out_path) if out_path else HERE / "ref_golden.npz"
    np.savez_compressed(path, **out)
    print("wrote", path, "trig values:", len(x), "valid rates:",
          {k: float(out[f"{k}_valid"].mean()) for k in out["cases"]})


if __name__ == "__main__":
    main(*sys.argv[1:])
