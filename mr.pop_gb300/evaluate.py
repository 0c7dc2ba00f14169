"""Benchmark driver over the reference's problem sets, with CSV output in the
format of the reference's `evaluate_mr` (scripts/evaluate_mr.cu:81-109).

For every valid problem (scripts/<robot>_problems.json through
`problems.load_problems`, or the converted fixture tests/golden/problems.npz)
one planner runs and one CSV row is written with the reference's columns:
  - `--planner drrt` (default): the reference's planner, dRRT / AO-x
    (mrpop_drrt_solve, `drrt.py`) with the driver's settings
    (scripts/evaluate_mr.cu:162-166: 300 attempts per iteration, granularity
    64, range 2.0, three passes) and the arms on the reference's compiled-in
    bases (solve(..., 4, 8) / solve(..., 5, 8), :133-136);
  - `--planner compact`: this library's compact planner through a session of
    the validation service.
Columns:

  solved,cost,path_length,start_tree_size,goal_tree_size,iters,wall_ns,
  kernel_ns,copy_ns,num_new_configs,granularity,range,balance,tree_ratio,
  dynamic_domain,dd_alpha,dd_radius,dd_min_radius,configs_str

For the dRRT planner the settings columns are its settings and kernel_ns is
the reference's (from the first pass's start to the end).  For the compact
planner the columns of pop_settings (pop_settings.hh:3-32) it has no use for
(balance, tree_ratio, dynamic_domain, dd_*) carry that struct's defaults and
kernel_ns is the time it waited for the service.  copy_ns is 0: nothing is
staged (page-locked buffers are read and written in place).  configs_str lists the path's
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


def settings_columns(settings) -> dict:
    """The settings columns of a row: a PlanSettings (compact planner) or an
    mrpop_drrt_settings (dRRT)."""
    if isinstance(settings, PlanSettings):
        return dict(POP_DEFAULTS, num_new_configs=settings.batch, granularity=settings.granularity,
                    range=settings.range)
    return {k: getattr(settings, k) for k in ("num_new_configs", "granularity", "range", "balance", "tree_ratio",
                                               "dynamic_domain", "dd_alpha", "dd_radius", "dd_min_radius")}


def csv_row(r: Row, settings) -> str:
    c = settings_columns(settings)
    cfgs = "".join("".join(_g(v) + " " for v in q) + "\\n" for q in r.path)
    f = [str(int(r.solved)), _g(r.cost if r.solved else 0.0), str(len(r.path)), str(r.start_tree),
         str(r.goal_tree), str(r.iters), str(r.wall_ns), str(r.kernel_ns), "0", str(c["num_new_configs"]),
         str(c["granularity"]), _g(c["range"]), str(int(c["balance"])), _g(c["tree_ratio"]),
         str(int(c["dynamic_domain"])), _g(c["dd_alpha"]), _g(c["dd_radius"]), _g(c["dd_min_radius"])]
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


def run_drrt(queries: list[Query], st, out_csv: str | Path | None = None, native_bases: bool = True) -> list[Row]:
    """dRRT / AO-x on every query in turn (one mrpop_drrt_solve each); write the CSV.
    native_bases: the arms on the reference's compiled-in layout (as its
    driver's solve(..., arms, 8) call places them), else the problem's bases."""
    from . import drrt
    rows = []
    for q in queries:
        t0 = time.perf_counter_ns()
        scene = M.Scene(q.scene)
        robots = M.RobotSet(q.arms, None if native_bases else q.bases)
        r = drrt.solve(scene, robots, q.start, q.goal, st)
        rows.append(Row(r.solved, r.cost, r.path, r.stats["start_tree_size"], r.stats["goal_tree_size"], r.iters,
                        time.perf_counter_ns() - t0, r.stats["kernel_ns"]))
    if out_csv is not None:
        write_csv(rows, st, out_csv)
    return rows


def write_csv(rows: list[Row], settings, out_csv) -> None:
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
    ap.add_argument("--planner", choices=["drrt", "compact"], default="drrt")
    ap.add_argument("--max-iters", type=int, default=None, help="iterations per launch (pass)")
    a = ap.parse_args(argv)
    arms = 4 if a.robot_name == "panda_four" else 5
    if a.problems:
        from .problems import load_problems
        queries = problem_queries(load_problems(a.problems), arms)
    else:
        queries = fixture_queries(Path(__file__).resolve().parents[1] / "tests" / "golden" / "problems.npz", arms)
    Path("test_output").mkdir(exist_ok=True)
    out = Path("test_output") / f"{a.robot_name}_{a.run_name}.csv"
    if a.planner == "drrt":
        from . import drrt
        st = drrt.evaluate_settings(**({"max_iters": a.max_iters} if a.max_iters else {}))
        rows = run_drrt(queries, st, out)
    else:
        settings = PlanSettings(max_iters=a.max_iters or PlanSettings.max_iters)
        server = M.Server(budget_bytes=256 << 20, streams=2)
        rows = run(server, queries, settings, out)
        server.close()
    failed = sum(not r.solved for r in rows)
    print(f"Total failed: {failed} / {len(rows)}", file=sys.stdout)
    print(f"wrote {out}")
    return 0
