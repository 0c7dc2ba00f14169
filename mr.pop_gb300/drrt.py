"""The reference's planner -- dRRT over per-arm roadmaps under the AO-x
meta-algorithm (dRRT::solve, src/planning/Planners.hh:57-64 and
pop_planner.cu:739-1030) -- rebuilt on the batched validator: Python side of
mrpop_drrt_solve / mrpop_drrt_solve_with (include/mrpop.h).

`settings()` starts from the reference's pop_settings defaults
(pop_settings.hh:3-32); `evaluate_settings()` applies the overrides of the
reference's benchmark driver (scripts/evaluate_mr.cu:162-166: 300 new
configurations per iteration, granularity 64, range 2.0, three AO-x passes).
A solve returns the reported path in the reference's order, from the goal to
the start, and every improving solution (PlannerResult::seed_paths).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import mrpop as M


@dataclass
class Solution:
    pass_index: int
    cost: float
    path: np.ndarray       # [n][dof], goal -> start, simplified when path_simplify
    raw_path: np.ndarray   # the pass's path before simplification


@dataclass
class Result:
    solved: bool
    cost: float
    iters: int
    path: np.ndarray
    solutions: list = field(default_factory=list)
    stats: dict = field(default_factory=dict)


def settings(**overrides) -> M.DrrtSettingsC:
    lib = M.library()
    s = M.DrrtSettingsC()
    M._check(lib, lib.mrpop_drrt_settings_default(C.byref(s)))
    for k, v in overrides.items():
        if not hasattr(s, k):
            raise AttributeError(f"mrpop_drrt_settings has no field {k!r}")
        setattr(s, k, v)
    return s


def evaluate_settings(**overrides) -> M.DrrtSettingsC:
    """The reference benchmark driver's settings (scripts/evaluate_mr.cu:162-166)."""
    base = dict(num_new_configs=300, granularity=64, range=2.0, rrtc_iter=3)
    base.update(overrides)
    return settings(**base)


def settings_dict(s: M.DrrtSettingsC) -> dict:
    return {name: getattr(s, name) for name, _ in s._fields_}


CHECK_KINDS = ("roadmap", "extend", "connect", "bspline", "shortcut")


def _stats(r: M.DrrtResultC, arms: int) -> dict:
    arrays = ("roadmap_nodes", "roadmap_edges", "check_ns", "check_calls")
    out = {name: getattr(r, name) for name, _ in r._fields_ if name not in arrays}
    out["roadmap_nodes"] = list(r.roadmap_nodes)[:arms]
    out["roadmap_edges"] = list(r.roadmap_edges)[:arms]
    # validate time and calls by kind of check
    for key in ("check_ns", "check_calls"):
        out[key] = dict(zip(CHECK_KINDS, list(getattr(r, key))))
    return out


def _collector(dof: int, sols: list):
    def cb(_ctx, pass_index, cost, path, n, raw, n_raw):
        p = np.ctypeslib.as_array(C.cast(path, C.POINTER(C.c_float)), shape=(n * dof,)).reshape(n, dof).copy() \
            if n else np.zeros((0, dof), np.float32)
        rp = np.ctypeslib.as_array(C.cast(raw, C.POINTER(C.c_float)), shape=(n_raw * dof,)).reshape(n_raw, dof).copy() \
            if n_raw else np.zeros((0, dof), np.float32)
        sols.append(Solution(int(pass_index), float(cost), p, rp))
    return M.SOLUTION_FN(cb)


def _finish(r: M.DrrtResultC, sols: list, dof: int, arms: int) -> Result:
    path = sols[-1].path if sols else np.zeros((0, dof), np.float32)
    return Result(bool(r.solved), float(r.cost), int(r.iters), path, sols, _stats(r, arms))


def solve(scene: M.Scene, robots: M.RobotSet, start, goals, st: M.DrrtSettingsC | None = None) -> Result:
    """dRRT::solve on this library's kernels (current CUDA device)."""
    lib = scene.lib
    arms = robots.n_arms
    dof = 7 * arms
    st = st or settings()
    start = np.ascontiguousarray(np.asarray(start, np.float32).reshape(dof))
    goals = np.ascontiguousarray(np.asarray(goals, np.float32).reshape(-1, dof))
    sols: list = []
    cb = _collector(dof, sols)
    r = M.DrrtResultC()
    M._check(lib, lib.mrpop_drrt_solve(scene.handle, robots.handle, start.ctypes.data, goals.ctypes.data, len(goals),
                                       C.byref(st), None, 0, cb, None, C.byref(r)))
    return _finish(r, sols, dof, arms)


def solve_session(session: M.Session, scene: M.Scene, robots: M.RobotSet, start, goals,
                  st: M.DrrtSettingsC | None = None) -> Result:
    """dRRT::solve with every check served by a session of the validation
    service (mrpop_session_drrt; one call, the GIL released throughout)."""
    lib = scene.lib
    arms = robots.n_arms
    dof = 7 * arms
    st = st or settings()
    start = np.ascontiguousarray(np.asarray(start, np.float32).reshape(dof))
    goals = np.ascontiguousarray(np.asarray(goals, np.float32).reshape(-1, dof))
    sols: list = []
    cb = _collector(dof, sols)
    r = M.DrrtResultC()
    M._check(lib, lib.mrpop_session_drrt(session.handle, scene.handle, robots.handle, start.ctypes.data,
                                         goals.ctypes.data, len(goals), C.byref(st), None, 0, cb, None, C.byref(r)))
    return _finish(r, sols, dof, arms)


def solve_with(arms: int, validate, start, goals, st: M.DrrtSettingsC | None = None, lib=None) -> Result:
    """The same planner with any validator and nearest-neighbour searches on
    the host: validate(q0, q1, g, rule, range, flags, arm) -> (valid u8 [n],
    first_hit i32 [n]) for host arrays q0/q1 [n][dof]."""
    lib = lib or M.library()
    dof = 7 * arms
    st = st or settings()
    start = np.ascontiguousarray(np.asarray(start, np.float32).reshape(dof))
    goals = np.ascontiguousarray(np.asarray(goals, np.float32).reshape(-1, dof))
    err: list = []

    def check(_ctx, q0p, q1p, n, g, rule, range_, flags, arm, validp, firstp):
        try:
            d = 7 if arm >= 0 else dof
            q0 = np.ctypeslib.as_array(C.cast(q0p, C.POINTER(C.c_float)), shape=(n * d,)).reshape(n, d)
            q1 = np.ctypeslib.as_array(C.cast(q1p, C.POINTER(C.c_float)), shape=(n * d,)).reshape(n, d)
            v, f = validate(q0.copy(), q1.copy(), int(g), int(rule), float(range_), int(flags), int(arm))
            C.memmove(validp, np.ascontiguousarray(v, np.uint8).ctypes.data, n)
            C.memmove(firstp, np.ascontiguousarray(f, np.int32).ctypes.data, 4 * n)
            return 0
        except Exception as e:  # reported after the call returns
            err.append(e)
            return 1

    fn = M.CHECK_FN(check)
    sols: list = []
    cb = _collector(dof, sols)
    r = M.DrrtResultC()
    rc = lib.mrpop_drrt_solve_with(arms, fn, None, start.ctypes.data, goals.ctypes.data, len(goals), C.byref(st),
                                   None, 0, cb, None, C.byref(r))
    if err:
        raise err[0]
    M._check(lib, rc)
    return _finish(r, sols, dof, arms)


def release_pool(lib=None) -> int:
    """Frees the idle pooled device resources of past solves (mrpop_drrt_release_pool);
    returns how many sets were freed."""
    return int((lib or M.library()).mrpop_drrt_release_pool())


def path_cost(path: np.ndarray) -> float:
    """Sum of composite Euclidean segment lengths, in float32 as the reference sums them."""
    c = np.float32(0.0)
    for a, b in zip(path[:-1], path[1:]):
        d = (a - b).astype(np.float32)
        c = np.float32(c + np.sqrt(np.float32(np.dot(d, d))))
    return float(c)
