"""The benchmark driver over the reference's problem sets (evaluate.py): the
converted fixture gives the reference's problems, and rows are written in the
column layout of the reference's evaluate_mr CSV (evaluate_mr.cu:81-109)."""
import csv
import io
from pathlib import Path

import numpy as np

FIXTURE = Path(__file__).resolve().parent / "golden" / "problems.npz"


def test_fixture_queries(pkg):
    E = pkg.evaluate
    for arms in (4, 5):
        qs = E.fixture_queries(FIXTURE, arms)
        assert len(qs) == 50
        assert all(q.start.shape == (7 * arms,) and q.goal.shape == (7 * arms,) for q in qs)
        assert qs[0].bases.shape == (arms, 4, 4) and len(qs[0].scene.cuboids) > 0


def test_csv_layout_and_oracle_plan(pkg, orc):
    E, P = pkg.evaluate, pkg.planner
    q = E.fixture_queries(FIXTURE, 4)[0]
    flags = pkg.CHECK_ENV | pkg.CHECK_SELF
    settings = P.PlanSettings(batch=32, max_iters=6, shortcut_passes=2, shortcut_pairs=8)

    def validate(q0, q1, g, rule, range_):
        r = orc.validate(q.scene, q.bases, q0, q1, g, flags, -1, rule, range_)
        return r["valid"], r["first_hit"]

    res = P.plan(q, validate, settings)
    row = E.Row(res.solved, res.cost, res.path, res.start_tree, res.goal_tree, res.iterations, 12345,
                res.validate_ns)
    text = E.CSV_HEADER + E.csv_row(row, settings)
    rec = list(csv.reader(io.StringIO(text), skipinitialspace=True))
    assert rec[0] == E.CSV_HEADER.strip().split(",")
    assert len(rec[1]) == len(rec[0]) == 19
    assert rec[1][0] == str(int(res.solved)) and int(rec[1][2]) == len(res.path)
    assert int(rec[1][3]) == res.start_tree >= 1 and int(rec[1][4]) == res.goal_tree >= 1
    assert rec[1][9] == "32" and rec[1][10] == "32"
    cfgs = [c for c in rec[1][18].split("\\n") if c]
    assert len(cfgs) == len(res.path)
    if res.solved:
        back = np.array([[float(v) for v in c.split()] for c in cfgs], np.float32)
        assert back.shape == res.path.shape
        assert np.allclose(back, res.path, atol=1e-5 * (1 + np.abs(res.path)).max())


def test_queries_from_a_problem_file(pkg):
    """A problem dict in the reference's file format becomes a query with its
    scene, start, first goal and arm bases."""
    import json
    E = pkg.evaluate
    prob = {"name": "bins", "valid": True, "source_index": 7,
            "start": [0.0] * 28, "goals": [[0.1] * 28, [0.2] * 28],
            "box": [{"position": [0.5, 0.0, 0.3], "orientation_euler_xyz": [0.0, 0.0, 0.3],
                     "half_extents": [0.1, 0.2, 0.05]}],
            "base_positions": [[0.5, 0.5, 0.0], [-0.5, 0.5, 0.0], [-0.5, -0.5, 0.0], [0.5, -0.5, 0.0]],
            "base_orientation_wxyz": [[1.0, 0.0, 0.0, 0.0]] * 4}
    probs = pkg.problems.load_problems(json.dumps([prob, dict(prob, valid=False)]))
    qs = E.problem_queries(probs, 4)
    assert len(qs) == 1
    q = qs[0]
    assert q.qid == 7 and q.arms == 4 and len(q.scene.cuboids) == 1
    assert np.allclose(q.goal, 0.1) and q.bases.shape == (4, 4, 4)
    assert np.allclose(q.bases[1][:3, 3], [-0.5, 0.5, 0.0])


def test_oracle_driven_plans_match_the_gb300_rows(pkg, orc):
    """The planner with the oracle as its validator reproduces the rows that the
    problem-set driver wrote on a GB300 (tests/golden/make_planner_golden.py):
    every verdict along these plans agreed between the oracle and the kernels."""
    import json
    E, P = pkg.evaluate, pkg.planner
    gold = json.loads((FIXTURE.parent / "planner_gb300_panda_four.json").read_text())
    queries = E.fixture_queries(FIXTURE, gold["arms"])
    settings = P.PlanSettings(max_iters=gold["max_iters"])
    flags = pkg.CHECK_ENV | pkg.CHECK_SELF
    for idx, want in gold["rows"].items():
        q = queries[int(idx)]

        def validate(q0, q1, g, rule, range_, q=q):
            r = orc.validate(q.scene, q.bases, q0, q1, g, flags, -1, rule, range_)
            return r["valid"], r["first_hit"]

        r = P.plan(q, validate, settings)
        row = E.Row(r.solved, r.cost, r.path, r.start_tree, r.goal_tree, r.iterations, 0, 0)
        got = next(csv.reader(io.StringIO(E.csv_row(row, settings)), skipinitialspace=True))
        assert got[:6] == [want[k] for k in ("solved", "cost", "path_length", "start_tree_size",
                                             "goal_tree_size", "iters")], idx
