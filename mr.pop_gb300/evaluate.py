"""Benchmark driver over the reference's problem sets, with CSV output in the
format of the reference's `evaluate_mr` (scripts/evaluate_mr.cu:81-109).

For every valid problem (scripts/<robot>_problems.json through
`problems.load_problems`, or the converted fixture tests/golden/problems.npz)
the library's planner runs through a session of the validation service, and
one CSV row is written with the reference's columns:

  solved,cost,path_length,start_tree_size,goal_tree_size,iters,wall_ns,
  kernel_ns,copy_ns,num_new_configs,granularity,range,balance,tree_ratio,
  dynamic_domain,dd_alpha,dd_radius,dd_min_radius,configs_str

Columns of the reference's pop_settings (pop_settings.hh:3-32) that this
planner has no use for (balance, tree_ratio, dynamic_domain, dd_*) carry that
struct's defaults.  kernel_ns is the time the planner waited for the service
(all of its validation steps); copy_ns is 0, since the kernels read and write
the session's page-locked buffers in place.  configs_str lists the path's
configurations, each value followed by a space and each configuration by a
literal backslash-n, as print_cfg_to_ss does (Planners.hh:43-48).
"""
from __future__ import annotations

import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import mrpop as M
from .planner import PlanSettings, Query, result_from_c

CSV_HEADER = ("solved,cost,path_length,start_tree_size,goal_tree_size,iters,wall_ns,kernel_ns,copy_ns,"
              "num_new_configs,granularity,range,balance,tree_ratio,dynamic_domain,dd_alpha,dd_radius,"
              "dd_min_radius,configs_str\n")

# pop_settings defaults of the columns the planner does not use (pop_settings.hh:11-17)
POP_DEFAULTS = {"balance": 2, "tree_ratio": 1.0, "dynamic_domain": 0, "dd_alpha": 0.0001, "dd_radius": 4.0,
                "dd_min_radius": 1.0}


def _g(x: float) -> str:
    """A float as std::ostream prints it by default (6 significant digits)."""
    return f"{float(x):g}"


@dataclass
class Row:
    solved: bool
    cost: float
    path: np.ndarray
    start_tree: int
    goal_tree: int
    iters: int
    wall_ns: int
    kernel_ns: int


def csv_row(r: Row, settings: PlanSettings) -> str:
    cfgs = "".join("".join(_g(v) + " " for v in q) + "\\n" for q in r.path)
    f = [str(int(r.solved)), _g(r.cost if r.solved else 0.0), str(len(r.path)), str(r.start_tree),
         str(r.goal_tree), str(r.iters), str(r.wall_ns), str(r.kernel_ns), "0", str(settings.batch),
         str(settings.granularity), _g(settings.range), str(POP_DEFAULTS["balance"]),
         _g(POP_DEFAULTS["tree_ratio"]), str(POP_DEFAULTS["dynamic_domain"]), _g(POP_DEFAULTS["dd_alpha"]),
         _g(POP_DEFAULTS["dd_radius"]), _g(POP_DEFAULTS["dd_min_radius"])]
    return ", ".join(f) + ", \"" + cfgs + "\"\n"


def fixture_queries(npz_path, arms: int) -> list[Query]:
    """The reference's valid problems of one robot from the converted fixture."""
    d = np.load(npz_path)
    bases = d[f"a{arms}_bases"]
    out = []
    for i in range(int(d[f"n{arms}"])):
        scene = M.SceneArrays(cuboids=d[f"a{arms}_p{i}_boxes"])
        out.append(Query(i, arms, scene, bases, d[f"a{arms}_p{i}_start"], d[f"a{arms}_p{i}_goal"], 1000 + i))
    return out


def problem_queries(problems, arms: int) -> list[Query]:
    """Queries from `problems.load_problems` output (first goal of each)."""
    out = []
    for i, p in enumerate(problems):
        bases = p.bases if p.bases is not None else None
        out.append(Query(p.index, arms, p.scene, bases, p.start, p.goals[0], 1000 + i))
    return out


def run(server: M.Server, queries: list[Query], settings: PlanSettings, out_csv: str | Path | None = None,
        flags: int = M.CHECK_ENV | M.CHECK_SELF) -> list[Row]:
    """Plan every query in turn through one session each; write the CSV."""
    rows = []
    for q in queries:
        t0 = time.perf_counter_ns()
        scene = M.Scene(q.scene, lib=server.lib)
        robots = M.RobotSet(q.arms, q.bases, lib=server.lib)
        sess = server.session(q.arms, max(settings.batch, settings.shortcut_pairs), settings.granularity)
        try:
            res, path = sess.plan(scene, robots, q.start, q.goal, settings.c(q.seed), flags)
        finally:
            sess.close()
        r = result_from_c(q.qid, res, path)
        rows.append(Row(r.solved, r.cost, r.path, r.start_tree, r.goal_tree, r.iterations,
                        time.perf_counter_ns() - t0, r.validate_ns))
    if out_csv is not None:
        write_csv(rows, settings, out_csv)
    return rows


def write_csv(rows: list[Row], settings: PlanSettings, out_csv) -> None:
    with open(out_csv, "w") as f:
        f.write(CSV_HEADER)
        for r in rows:
            f.write(csv_row(r, settings))


def main(argv=None) -> int:
    """evaluate <robot_name> <run_name> [problems.json]: like the reference's
    `evaluate_mr <robot_name> <run_name>` (evaluate_mr.cu:155-186), writing
    test_output/<robot_name>_<run_name>.csv.  Without a problems file the
    converted fixture of the reference's problem sets is used."""
    import argparse
    import sys
    ap = argparse.ArgumentParser(prog="evaluate")
    ap.add_argument("robot_name", choices=["panda_four", "panda_five"])
    ap.add_argument("run_name")
    ap.add_argument("problems", nargs="?", default=None)
    ap.add_argument("--max-iters", type=int, default=PlanSettings.max_iters)
    a = ap.parse_args(argv)
    arms = 4 if a.robot_name == "panda_four" else 5
    if a.problems:
        from .problems import load_problems
        queries = problem_queries(load_problems(a.problems), arms)
    else:
        queries = fixture_queries(Path(__file__).resolve().parents[1] / "tests" / "golden" / "problems.npz", arms)
    settings = PlanSettings(max_iters=a.max_iters)
    Path("test_output").mkdir(exist_ok=True)
    out = Path("test_output") / f"{a.robot_name}_{a.run_name}.csv"
    server = M.Server(budget_bytes=256 << 20, streams=2)
    rows = run(server, queries, settings, out)
    server.close()
    failed = sum(not r.solved for r in rows)
    print(f"Total failed: {failed} / {len(rows)}", file=sys.stdout)
    print(f"wrote {out}")
    return 0
