"""Served-planning queries and the host binding of the library's planner.

The planner itself is C++ in the library (`mrpop_plan`, csrc/planner.cu): a
batched bidirectional RRT with connect checks and shortcut passes, the step
pattern of the reference's planner (whose dRRT/AO-x, Planners.hh:57-64, is not
rebuilt).  `plan()` runs it with a Python validator (the oracle in the CPU
tests); `Session.plan` runs it with every step validated by the service.

`make_queries` draws the served-planning queries: 2-5 Pandas facing the centre of a
fresh seeded scene from the single-arm or bin-picking generator, start and goal
rejection-sampled collision-free.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import mrpop as M
from .workloads import SceneArrays, bases_facing_centre, random_configs, scene_config1, scene_config2

RULE_PLAIN, RULE_CONNECT, RULE_SHORTCUT = 0, 1, 3


@dataclass
class Query:
    qid: int
    arms: int
    scene: SceneArrays
    bases: np.ndarray
    start: np.ndarray
    goal: np.ndarray
    seed: int


@dataclass
class PlanSettings:
    """mrpop_plan_settings (defaults of the served workload)."""
    batch: int = 64
    max_iters: int = 60
    granularity: int = 32
    shortcut_passes: int = 5
    shortcut_pairs: int = 32
    step: float = 1.0
    range: float = 1.0

    def c(self, seed: int) -> M.PlanSettingsC:
        return M.PlanSettingsC(self.batch, self.max_iters, self.granularity, self.shortcut_passes,
                               self.shortcut_pairs, self.step, self.range, seed)


@dataclass
class PlanResult:
    qid: int
    solved: bool
    path: np.ndarray
    cost: float
    iterations: int
    steps: int
    edges: int
    verdict_digest: int
    start_tree: int = 0
    goal_tree: int = 0
    validate_ns: int = 0
    phases_ns: dict | None = None  # planner phases (dRRT: wall, validate, nn, roadmap, oracle)


def result_from_c(qid: int, r: M.PlanResultC, path: np.ndarray) -> PlanResult:
    return PlanResult(qid, bool(r.solved), path, float(r.cost) if r.solved else math.inf, int(r.iterations),
                      int(r.steps), int(r.edges), int(r.digest), int(r.start_tree), int(r.goal_tree),
                      int(r.validate_ns))


def path_cost(path: np.ndarray) -> float:
    if len(path) < 2:
        return 0.0
    return float(np.linalg.norm(np.diff(path.astype(np.float64), axis=0), axis=1).sum())


def plan(query: Query, validate, settings: PlanSettings | None = None, lib=None,
         max_waypoints: int = 4096) -> PlanResult:
    """The library's planner with a Python validator:
    validate(q0, q1, granularity, rule, range_) -> (valid u8[n], first_hit i32[n])."""
    s = settings or PlanSettings()
    lib = lib or M.library()
    dof = 7 * query.arms
    err: list = []

    def cb(_ctx, q0p, q1p, n, g, rule, range_, validp, firstp):
        try:
            q0 = np.ctypeslib.as_array(C.cast(q0p, C.POINTER(C.c_float)), shape=(n, dof)).copy()
            q1 = np.ctypeslib.as_array(C.cast(q1p, C.POINTER(C.c_float)), shape=(n, dof)).copy()
            v, f = validate(q0, q1, g, rule, range_)
            np.ctypeslib.as_array(C.cast(validp, C.POINTER(C.c_uint8)), shape=(n,))[:] = v
            np.ctypeslib.as_array(C.cast(firstp, C.POINTER(C.c_int32)), shape=(n,))[:] = f
            return 0
        except Exception as e:  # noqa: BLE001 -- reported after the call
            err.append(e)
            return 1

    fn = M.VALIDATE_FN(cb)
    start = np.ascontiguousarray(query.start, np.float32)
    goal = np.ascontiguousarray(query.goal, np.float32)
    path = np.empty((max_waypoints, dof), np.float32)
    res = M.PlanResultC()
    st = lib.mrpop_plan(query.arms, start.ctypes.data, goal.ctypes.data, C.byref(s.c(query.seed)), fn, None,
                        path.ctypes.data, max_waypoints, C.byref(res))
    if err:
        raise err[0]
    M._check(lib, st)
    return result_from_c(query.qid, res, path[:min(res.waypoints, max_waypoints)].copy())


def make_queries(n: int, seed: int, collision_free, arms_range=(2, 5)) -> list[Query]:
    """Seeded served-planning queries.
    collision_free(scene, bases, q) -> bool array over the candidate rows."""
    rng = np.random.default_rng(5000 + seed)
    out = []
    for qid in range(n):
        arms = int(rng.integers(arms_range[0], arms_range[1] + 1))
        bases = bases_facing_centre(arms, 0.71)
        picked = []
        while len(picked) < 2:
            # a scene whose boxes enclose an arm's base leaves no free
            # configuration: after 1024 candidates without two free ones,
            # the scene is drawn again
            sc_seed = int(rng.integers(0, 1 << 30))
            scene = scene_config1(sc_seed) if rng.random() < 0.5 else scene_config2(sc_seed)
            picked = []
            for _ in range(4):
                cand = random_configs(rng, 256, arms)
                ok = collision_free(scene, bases, cand)
                picked.extend(cand[np.nonzero(ok)[0][:2 - len(picked)]])
                if len(picked) == 2:
                    break
        out.append(Query(qid, arms, scene, bases, picked[0], picked[1], int(rng.integers(0, 1 << 62))))
    return out
