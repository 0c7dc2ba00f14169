"""The reference's own planner on its benchmark problems: solve rate, cost and
time per problem (MEASUREMENT INFRASTRUCTURE; see oracle/ref_planner.py).

    python -m oracle.ref_planner_eval <arms 4|5> <out.jsonl> [--first N] [--timeout S]

Runs every valid problem of the converted fixture (tests/golden/problems.npz,
the reference's scripts/panda_{four,five}_problems.json) through
RefPlanner.solve with the reference driver's settings
(scripts/evaluate_mr.cu:162-166) and the arms on the reference's compiled-in
bases, as its driver's solve(..., arms, 8) call places them.  Problems run in
child processes, several per child; a child that passes the time limit is
stopped, its problem is recorded as timed out, and the next child resumes
after it.  One JSON line per problem.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
FIX = ROOT / "tests" / "golden" / "problems.npz"


def child(arms: int, first: int, last: int, out: str) -> None:
    import numpy as np
    sys.path.insert(0, str(ROOT))
    from oracle.ref_planner import RefPlanner, evaluate_settings
    import __graft_entry__ as ge
    pkg = ge.load_package()
    z = np.load(FIX)
    rp = RefPlanner()
    st = evaluate_settings()
    for p in range(first, last):
        sc = pkg.SceneArrays(cuboids=z[f"a{arms}_p{p}_boxes"])
        r = rp.solve(sc, z[f"a{arms}_p{p}_start"], z[f"a{arms}_p{p}_goal"][None], st, arms, 8)
        row = {"arms": arms, "problem": p, "solved": bool(r["solved"]), "cost": r["cost"],
               "path_length": r["path_length"], "iters": r["iters"], "kernel_ns": r["kernel_ns"],
               "wall_ns": r["wall_ns"], "launches": r["launches"], "roadmap_rounds": r["roadmap_rounds"],
               "roadmap_sizes": r["roadmap_sizes"], "seed_costs": r["seed_costs"], "stopped": r["stopped"],
               "start_tree_size": r.get("start_tree_size"), "goal_tree_size": r.get("goal_tree_size")}
        with open(out, "a") as f:
            f.write(json.dumps(row) + "\n")
        print(json.dumps(row), flush=True)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("arms", type=int, choices=[4, 5])
    ap.add_argument("out")
    ap.add_argument("--first", type=int, default=None, help="only the first N problems")
    ap.add_argument("--timeout", type=float, default=600.0, help="seconds per child")
    ap.add_argument("--per-child", type=int, default=10)
    ap.add_argument("--child", nargs=2, type=int, default=None, help=argparse.SUPPRESS)
    a = ap.parse_args(argv)
    if a.child:
        child(a.arms, a.child[0], a.child[1], a.out)
        return 0
    import numpy as np
    n = int(np.load(FIX)[f"n{a.arms}"])
    if a.first:
        n = min(n, a.first)
    done = set()
    if os.path.exists(a.out):
        done = {json.loads(l)["problem"] for l in open(a.out) if l.strip()}
    p = 0
    while p < n:
        if p in done:
            p += 1
            continue
        last = min(n, p + a.per_child)
        cmd = [sys.executable, "-m", "oracle.ref_planner_eval", str(a.arms), a.out, "--child", str(p), str(last)]
        t0 = time.time()
        try:
            subprocess.run(cmd, cwd=str(ROOT), timeout=a.timeout, check=False)
        except subprocess.TimeoutExpired:
            pass
        done = {json.loads(l)["problem"] for l in open(a.out) if l.strip()} if os.path.exists(a.out) else set()
        while p < last and p in done:
            p += 1
        if p < last:  # the child stopped (time limit or error) inside problem p
            with open(a.out, "a") as f:
                f.write(json.dumps({"arms": a.arms, "problem": p, "solved": False, "stopped": "child ended",
                                    "seconds": round(time.time() - t0, 1)}) + "\n")
            done.add(p)
            p += 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
