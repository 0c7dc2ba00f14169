"""Convert the reference benchmark's problem files into a compact fixture.

Reads scripts/panda_four_problems.json and scripts/panda_five_problems.json
from the reference source tree (argument 1, default /root/reference) with the
package's problem loader (mrpop_gb300.problems, which follows the reference's
problem_dict_to_env, scripts/evaluate_mr.cu:14-79) and writes
tests/golden/problems.npz: per valid problem the obstacle boxes as packed
cuboid records (the files hold no spheres or cylinders), the start and first
goal configurations, and the arm bases from base_positions /
base_orientation_wxyz.  Run where the reference sources exist.
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))


def main(ref_root="/root/reference"):
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
            out[f"a{arms}_p{i}_start"] = p.start
            out[f"a{arms}_p{i}_goal"] = p.goals[0]
    np.savez_compressed(HERE / "problems.npz", **out)
    print("wrote", HERE / "problems.npz")


if __name__ == "__main__":
    main(*sys.argv[1:])
