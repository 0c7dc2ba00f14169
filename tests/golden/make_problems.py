"""Convert the reference benchmark's problem files into a compact fixture.

Reads scripts/panda_four_problems.json and scripts/panda_five_problems.json
from the reference source tree (argument 1, or $MRPOP_REF_ROOT) with the
package's problem loader (mrpop_gb300.problems, which follows the reference's
problem_dict_to_env, scripts/evaluate_mr.cu:14-79) and writes
tests/golden/problems.npz: per valid problem the obstacle boxes as packed
cuboid records built in float32 as the reference's Eigen factory builds them
(the files hold no spheres or cylinders), the boxes' JSON parameters, the
start and first goal configurations, and the arm bases from base_positions /
base_orientation_wxyz.  Run where the reference sources exist.
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))


def main(ref_root):
    import __graft_entry__ as ge
    P = ge.load_package().problems
    out = {}
    for arms, name in ((4, "panda_four"), (5, "panda_five")):
        probs = P.load_problems(Path(ref_root) / "scripts" / f"{name}_problems.json")
        out[f"n{arms}"] = np.array(len(probs))
        out[f"a{arms}_bases"] = probs[0].bases
        for i, p in enumerate(probs):
            assert len(p.scene.spheres) == 0 and len(p.scene.capsules) == 0
            out[f"a{arms}_p{i}_boxes"] = p.scene.cuboids
            # the JSON box parameters (position, Euler XYZ, half extents), so that
            # both constructions can be compared without the source files
            out[f"a{arms}_p{i}_box_params"] = np.array(
                [[*b["position"], *b["orientation_euler_xyz"], *b["half_extents"]] for b in p.raw["box"]],
                np.float64).reshape(-1, 9)
            out[f"a{arms}_p{i}_start"] = p.start
            out[f"a{arms}_p{i}_goal"] = p.goals[0]
    np.savez_compressed(HERE / "problems.npz", **out)
    print("wrote", HERE / "problems.npz")


if __name__ == "__main__":
    import os
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MRPOP_REF_ROOT")
    if not root:
        sys.exit("usage: make_problems.py <reference-root>  (or set MRPOP_REF_ROOT)")
    main(root)
