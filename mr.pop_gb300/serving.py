"""Served planning stream: queries arrive as a Poisson process, each runs a
planner on a client thread with its own session of the validation service
(`mrpop_server_*`), and all sessions' steps are co-batched on the GPU by the
service's worker.  The planner is the reference's dRRT / AO-x
(mrpop_session_drrt, `drrt.py`) when the settings are mrpop_drrt_settings, or
the library's compact planner (mrpop_session_plan) for PlanSettings; either
runs as one library call per query with the GIL released.

A query's latency runs from its arrival to its result, and includes waiting
for admission (device-memory budget) and for a client thread, creating its
scene and robot set on the device, and every validation step.
"""
from __future__ import annotations

import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

from . import mrpop as M
from .planner import PlanResult, PlanSettings, Query, result_from_c


@dataclass
class Served:
    result: PlanResult
    arrival: float
    start: float
    finish: float

    @property
    def latency_ms(self) -> float:
        return 1e3 * (self.finish - self.arrival)


DRRT_STEP_EDGES = 8192  # a dRRT session's step size: larger checks are cut into steps of this many edges


# The service shape for dRRT clients: wave slots (CUDA streams) and client
# threads.  Each dRRT query issues a short device call per tree search, so a
# few clients per slot keep the GPU fed without the host's cores spinning.
SERVED_DRRT_STREAMS = 8
SERVED_DRRT_CLIENTS = 16


def served_drrt_settings(**overrides):
    """dRRT / AO-x settings of the served stream: the first pass plus five
    optimising passes (rrtc_iter 6), as the served workload asks, each pass
    capped at 12 iterations of 64 attempts and the roadmaps grown by 4 blocks
    per arm for at most 8 rounds -- a budget scaled down from the reference's
    100k iterations per pass so that 200 queries/s fit on one GPU and the
    host's cores.  Each query's host work runs on its own client thread
    (host_threads 1), which sleeps while its device work runs (blocking_wait):
    the concurrency comes from the queries."""
    from . import drrt
    base = dict(num_new_configs=64, granularity=32, range=1.5, rrtc_iter=6, max_iters=12, block_per_robot=4,
                max_launches=8, host_threads=1, blocking_wait=1)
    return drrt.settings(**base)


def drrt_result(qid: int, r) -> PlanResult:
    """A dRRT result in the fields the stream's summary and comparison read
    (the digest folds the solve's counters: equal solves have equal digests)."""
    s = r.stats
    digest = hash((s["iterations"], s["validate_calls"], s["edges_validated"], tuple(s["roadmap_edges"]),
                   s["start_tree_size"], s["goal_tree_size"]))
    return PlanResult(qid, r.solved, r.path, r.cost if r.solved else float("inf"), int(s["iterations"]),
                      int(s["validate_calls"]), int(s["edges_validated"]), digest, int(s["start_tree_size"]),
                      int(s["goal_tree_size"]), int(s["validate_ns"]),
                      {k: int(s[k + "_ns"]) for k in ("wall", "validate", "nn", "roadmap", "oracle")})


def run_query(server: M.Server, q: Query, settings, flags: int = M.CHECK_ENV | M.CHECK_SELF,
              timeout_ms: int = -1, keep: list | None = None) -> PlanResult:
    """One query through a session of `server`: scene and robot set created on
    the device for the query's lifetime, every step validated by the service.
    keep: a list that takes the scene and robot set instead of freeing them
    here (freeing device memory waits for the work in flight on the device, so
    a stream frees them after its last query)."""
    scene = M.Scene(q.scene, lib=server.lib)
    robots = M.RobotSet(q.arms, q.bases, lib=server.lib)
    if keep is not None:
        keep.append((scene, robots))
    if isinstance(settings, M.DrrtSettingsC):
        from . import drrt
        st = M.DrrtSettingsC.from_buffer_copy(settings)
        st.seed = q.seed
        sess = server.session(q.arms, DRRT_STEP_EDGES, settings.granularity, timeout_ms)
        try:
            return drrt_result(q.qid, drrt.solve_session(sess, scene, robots, q.start, q.goal, st))
        finally:
            sess.close()
    max_edges = max(settings.batch, settings.shortcut_pairs)
    sess = server.session(q.arms, max_edges, settings.granularity, timeout_ms)
    try:
        res, path = sess.plan(scene, robots, q.start, q.goal, settings.c(q.seed), flags)
        return result_from_c(q.qid, res, path)
    finally:
        sess.close()


def isolated(server: M.Server, queries: list[Query], settings) -> list[Served]:
    """Each query alone: one after another, nothing else on the service."""
    out, keep = [], []
    for q in queries:
        t0 = time.perf_counter()
        r = run_query(server, q, settings, keep=keep)
        out.append(Served(r, t0, t0, time.perf_counter()))
    del keep
    return out


def stream(server: M.Server, queries: list[Query], rate: float, settings, seed: int = 0,
           clients: int = 256) -> list[Served]:
    """Poisson arrivals at `rate` queries/s; each query starts on a free client
    thread (a query that finds none waits, and that wait counts as latency)."""
    rng = np.random.default_rng(9000 + seed)
    gaps = rng.exponential(1.0 / rate, size=len(queries))
    out: list[Served | None] = [None] * len(queries)
    lock = threading.Lock()
    keep: list = []

    def work(i: int, arrival: float):
        t0 = time.perf_counter()
        r = run_query(server, queries[i], settings, keep=keep)
        with lock:
            out[i] = Served(r, arrival, t0, time.perf_counter())

    with ThreadPoolExecutor(max_workers=clients) as ex:
        t_next = time.perf_counter()
        futs = []
        for i in range(len(queries)):
            t_next += gaps[i]
            delay = t_next - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(ex.submit(work, i, t_next))
        for f in futs:
            f.result()
    del keep
    return out  # type: ignore[return-value]


def summary(served: list[Served]) -> dict:
    lat = np.array([s.latency_ms for s in served])
    solved = [s for s in served if s.result.solved]
    return {
        "queries": len(served),
        "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
        "mean_ms": float(lat.mean()) if len(lat) else None,
        "solve_rate": len(solved) / max(1, len(served)),
        "mean_cost": float(np.mean([s.result.cost for s in solved])) if solved else None,
        "steps": int(sum(s.result.steps for s in served)),
        "edges": int(sum(s.result.edges for s in served)),
        "phase_mean_ms": phase_means(served),
    }


def phase_means(served: list[Served]) -> dict | None:
    """Mean milliseconds per query in each planner phase (dRRT clients):
    validation (queueing and device time of the checks), nearest-neighbour
    searches, roadmap pair searches, the direction oracle, and the rest of the
    host work ("other" = wall minus those)."""
    ph = [s.result.phases_ns for s in served if s.result.phases_ns]
    if not ph:
        return None
    out = {k: float(np.mean([p[k] for p in ph])) / 1e6 for k in ("wall", "validate", "nn", "roadmap", "oracle")}
    out["other"] = out["wall"] - out["validate"] - out["nn"] - out["roadmap"] - out["oracle"]
    return {k: round(v, 3) for k, v in out.items()}


def same_result(a: PlanResult, b: PlanResult) -> bool:
    """Identical plans: same verdict stream, solve flag and waypoints."""
    return (a.solved == b.solved and a.verdict_digest == b.verdict_digest and a.steps == b.steps
            and a.path.shape == b.path.shape and bool(np.array_equal(a.path, b.path)))
