"""Pin the planner's results on the GB300 for a CPU test.

Input: the CSV that the problem-set driver wrote on a GB300,
    python -c "import sys, __graft_entry__ as g; m = g.load_package(); m.library(); \
               sys.exit(m.evaluate.main(['panda_four', 'gb300', '--max-iters', '150']))"
(test_output/panda_four_gb300.csv).  Output: tests/golden/planner_gb300_panda_four.json,
the columns solved, cost, path_length, start_tree_size, goal_tree_size and iters of the
chosen problems (indices into the reference's valid 4-arm problems, in file order).
tests/test_evaluate_cpu.py plans the same problems on the CPU with the oracle as the
validator and expects the same rows: the plans depend on every verdict, so equal rows
mean the oracle and the GPU kernels agreed on each one.
"""
import csv
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
PROBLEMS = [0, 1, 5]  # problems that solve within a few dozen iterations (seconds on the CPU)


def main(csv_path="test_output/panda_four_gb300.csv"):
    rows = list(csv.reader(open(csv_path), skipinitialspace=True))
    head, body = rows[0], rows[1:]
    keep = ["solved", "cost", "path_length", "start_tree_size", "goal_tree_size", "iters"]
    out = {"max_iters": 150, "arms": 4,
           "rows": {str(i): {k: body[i][head.index(k)] for k in keep} for i in PROBLEMS}}
    (HERE / "planner_gb300_panda_four.json").write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", HERE / "planner_gb300_panda_four.json")


if __name__ == "__main__":
    main(*sys.argv[1:])
