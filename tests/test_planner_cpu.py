"""The library's planner (mrpop_plan) on the CPU, with the oracle as its
validator: deterministic, plans from start to goal, shortcut passes never
lengthen a path, and every waypoint of a returned path is collision-free."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def oracle_queries(pkg, orc):
    flags = pkg.CHECK_ENV | pkg.CHECK_SELF

    def cf(scene, bases, q):
        return orc.validate(scene, bases, q, q, 1, flags)["valid"].astype(bool)

    return pkg.planner.make_queries(4, seed=2, collision_free=cf, arms_range=(2, 3))


def _validator(orc, q, flags, log=None):
    def validate(q0, q1, g, rule, range_):
        if log is not None:
            log.append((len(q0), g, rule, range_))
        r = orc.validate(q.scene, q.bases, q0, q1, g, flags, -1, rule, range_)
        return r["valid"], r["first_hit"]
    return validate


def test_queries_are_collision_free_at_both_ends(pkg, orc, oracle_queries):
    flags = pkg.CHECK_ENV | pkg.CHECK_SELF
    for q in oracle_queries:
        ends = np.stack([q.start, q.goal])
        assert orc.validate(q.scene, q.bases, ends, ends, 1, flags)["valid"].all()
        assert 2 <= q.arms <= 3 and q.start.shape == (7 * q.arms,)


def test_plan_is_deterministic_and_connects_start_to_goal(pkg, orc, oracle_queries, lib_path):
    P = pkg.planner
    flags = pkg.CHECK_ENV | pkg.CHECK_SELF
    settings = P.PlanSettings(max_iters=20, batch=32)
    solved = 0
    for q in oracle_queries:
        log = []
        a = P.plan(q, _validator(orc, q, flags, log), settings)
        b = P.plan(q, _validator(orc, q, flags), settings)
        assert pkg.serving.same_result(a, b)
        assert a.steps == len(log) and a.edges == sum(n for n, _, _, _ in log)
        # the step pattern: plain extends of `batch` edges, connect and shortcut checks
        assert all(g == settings.granularity for _, g, _, _ in log)
        assert log[0] == (settings.batch, settings.granularity, P.RULE_PLAIN, 0.0)
        assert {r for _, _, r, _ in log} <= {P.RULE_PLAIN, P.RULE_CONNECT, P.RULE_SHORTCUT}
        if not a.solved:
            continue
        solved += 1
        assert np.array_equal(a.path[0], q.start) and np.array_equal(a.path[-1], q.goal)
        assert abs(a.cost - P.path_cost(a.path)) < 1e-9
        # every waypoint passes the single-configuration check (each is the
        # start, the goal or the last sample of an accepted extend edge; the
        # reference's verdict rules can leave a sample of an edge without a
        # detailed check, which these problems do not meet; a waypoint within
        # 1e-5 m of contact may round either way)
        r = orc.validate(q.scene, q.bases, a.path, a.path, 1, flags, band=1e-5)
        assert (r["valid"].astype(bool) | r["ambiguous"].astype(bool)).all()
    assert solved >= 1


def test_shortcut_never_lengthens(pkg, orc, oracle_queries):
    P = pkg.planner
    flags = pkg.CHECK_ENV | pkg.CHECK_SELF
    for q in oracle_queries[:2]:
        raw = P.plan(q, _validator(orc, q, flags), P.PlanSettings(max_iters=20, batch=32, shortcut_passes=0))
        cut = P.plan(q, _validator(orc, q, flags), P.PlanSettings(max_iters=20, batch=32, shortcut_passes=5))
        if raw.solved:
            assert cut.solved and cut.cost <= raw.cost + 1e-9 and len(cut.path) <= len(raw.path)


def test_validator_error_aborts_the_plan(pkg, oracle_queries):
    q = oracle_queries[0]

    def broken(q0, q1, g, rule, range_):
        raise RuntimeError("validator down")

    with pytest.raises(RuntimeError, match="validator down"):
        pkg.planner.plan(q, broken)


def test_bad_settings_rejected(pkg, oracle_queries):
    P = pkg.planner
    q = oracle_queries[0]

    def never(q0, q1, g, rule, range_):
        raise AssertionError("no step may run")

    for bad in (P.PlanSettings(batch=0), P.PlanSettings(granularity=65), P.PlanSettings(step=0.0),
                P.PlanSettings(range=-1.0), P.PlanSettings(shortcut_pairs=0)):
        with pytest.raises(pkg.MrpopError) as ei:
            P.plan(q, never, bad)
        assert ei.value.status == 1 and "settings" in str(ei.value)


def test_zero_iterations_returns_unsolved(pkg, oracle_queries):
    P = pkg.planner
    q = oracle_queries[0]
    r = P.plan(q, lambda *a: (_ for _ in ()).throw(AssertionError("no step")), P.PlanSettings(max_iters=0))
    assert not r.solved and r.steps == 0 and r.start_tree == 1 and r.goal_tree == 1 and len(r.path) == 0


def test_served_summary_and_comparison(pkg):
    P, S = pkg.planner, pkg.serving
    path = np.zeros((3, 14), np.float32)
    a = P.PlanResult(0, True, path, 1.0, 2, 5, 100, 7)
    b = P.PlanResult(0, True, path.copy(), 1.0, 2, 5, 100, 7)
    c = P.PlanResult(0, True, path + 1, 1.0, 2, 5, 100, 7)
    d = P.PlanResult(0, True, path.copy(), 1.0, 2, 5, 100, 8)
    assert S.same_result(a, b) and not S.same_result(a, c) and not S.same_result(a, d)
    served = [S.Served(a, 0.0, 0.0, 0.010), S.Served(P.PlanResult(1, False, path[:0], float("inf"), 60, 120, 9000, 1),
                                                     1.0, 1.0, 1.050)]
    s = S.summary(served)
    assert s["queries"] == 2 and s["solve_rate"] == 0.5 and s["mean_cost"] == 1.0
    assert abs(s["p50_ms"] - 30.0) < 1e-9 and s["steps"] == 125 and s["edges"] == 9100
