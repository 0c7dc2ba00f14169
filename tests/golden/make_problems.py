"""Convert the reference benchmark's problem files into a compact fixture.

Reads scripts/panda_four_problems.json and scripts/panda_five_problems.json
from the reference source tree (argument 1, default /root/reference) and
writes tests/golden/problems.npz: per problem the obstacle boxes as packed
cuboid records (built like the reference's problem_dict_to_env,
scripts/evaluate_mr.cu:14-79: every "box" entry becomes a cuboid from centre,
Euler XYZ angles and half extents; the files hold no spheres or cylinders),
the start and goal configurations, and the arm bases from base_positions /
base_orientation_wxyz.  Run here, where the reference sources exist.
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))


def quat_to_base(pos, wxyz):
    w, x, y, z = wxyz
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    t = np.eye(4)
    t[:3, :3] = r
    t[:3, 3] = pos
    return t.astype(np.float32)


def main(ref_root="/root/reference"):
    import __graft_entry__ as ge
    W = ge.load_package().workloads
    out = {}
    for arms, name in ((4, "panda_four"), (5, "panda_five")):
        probs = json.loads((Path(ref_root) / "scripts" / f"{name}_problems.json").read_text())
        probs = [p for p in probs if p["valid"]]
        out[f"n{arms}"] = np.array(len(probs))
        p0 = probs[0]
        out[f"a{arms}_bases"] = np.stack([quat_to_base(p, q) for p, q in
                                          zip(p0["base_positions"], p0["base_orientation_wxyz"])])
        for i, p in enumerate(probs):
            assert not p["sphere"] and not p["cylinder"]
            out[f"a{arms}_p{i}_boxes"] = np.stack([W.box(b["position"], b["orientation_euler_xyz"],
                                                         b["half_extents"]) for b in p["box"]])
            out[f"a{arms}_p{i}_start"] = np.asarray(p["start"], np.float32)
            out[f"a{arms}_p{i}_goal"] = np.asarray(p["goals"][0], np.float32)
    np.savez_compressed(HERE / "problems.npz", **out)
    print("wrote", HERE / "problems.npz")


if __name__ == "__main__":
    main(*sys.argv[1:])
