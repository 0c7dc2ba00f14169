"""The validation service (mrpop_server_* / mrpop_session_*): steps co-batched
from many sessions give the verdicts of the same calls made alone; admission
waits for room in the device-memory budget; a served planning query gives the
same plan alone and in a mix of concurrent queries."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _direct(pkg, cuda, scene, rb, q0, q1, g, flags, arm, rule, range_):
    d0, d1 = cuda.from_numpy(q0).cuda(), cuda.from_numpy(q1).cuda()
    out = pkg.validate(scene, rb, d0, d1, g, flags, arm, rule, range_)
    cuda.cuda.synchronize()
    return out[0].cpu().numpy(), out[1].cpu().numpy()


@pytest.mark.parametrize("fused_edges", [-1, 0, 1 << 40], ids=["split", "default", "fused"])
def test_steps_equal_direct_calls(cuda, pkg, fused_edges):
    """Waves run each group split (broad + narrow kernels), fused (one kernel
    per group) or by the default size rule: every form gives the direct calls'
    verdicts."""
    W = pkg.workloads
    insts = W.config4_instances(n_instances=16, seed=3, scale=0.05)
    rules = [(pkg.RULE_PLAIN, 0.0), (pkg.RULE_CONNECT, 0.6), (pkg.RULE_BSPLINE, 0.5), (pkg.RULE_SHORTCUT, 0.7)]
    server = pkg.Server(budget_bytes=512 << 20, streams=3, fused_edges=fused_edges)
    jobs, arms = [], []
    for k, wl in enumerate(insts):
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        arm = -1
        q0, q1 = wl.q0, wl.q1
        if k % 5 == 2:  # single-arm step on a composite session
            arm = len(wl.bases) - 1
            q0 = np.ascontiguousarray(q0[:, 7 * arm:7 * arm + 7])
            q1 = np.ascontiguousarray(q1[:, 7 * arm:7 * arm + 7])
        rule, rg = rules[k % 4]
        jobs.append((scene, rb, q0, q1, wl.granularity, wl.flags, arm, rule, rg))
        arms.append(len(wl.bases))
    expect = [_direct(pkg, cuda, *j) for j in jobs]
    got = [None] * len(jobs)
    errors = []

    def client(i):
        try:
            scene, rb, q0, q1, g, flags, arm, rule, rg = jobs[i]
            sess = server.session(arms[i], max(1, len(q0)), 64)
            res = []
            for rep in range(3):  # three steps per session: the whole set, a prefix, the whole set
                n = len(q0) if rep != 1 else max(0, len(q0) // 3)
                v, f = sess.validate(scene, rb, q0[:n], q1[:n], g, flags, arm, rule, rg)
                res.append((n, v, f))
            sess.close()
            got[i] = res
        except Exception as e:  # noqa: BLE001
            errors.append((i, e))

    th = [threading.Thread(target=client, args=(i,)) for i in range(len(jobs))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for i, res in enumerate(got):
        ev, ef = expect[i]
        for n, v, f in res:
            assert np.array_equal(v, ev[:n]), i
            assert np.array_equal(f, ef[:n]), i
    st = server.stats()
    assert st["steps"] == sum(1 for r in got for n, _, _ in r if n > 0)
    assert st["bytes_in_use"] == 0
    server.close()


def test_multi_item_submissions_equal_direct_calls(cuda, pkg):
    """mrpop_session_submit_many: a session's several steps (composite and
    single-arm, plain and segmented, different granularities) submitted
    together, from concurrent sessions, give the direct calls' verdicts."""
    W = pkg.workloads
    insts = W.config4_instances(n_instances=8, seed=5, scale=0.04)
    rules = [(pkg.RULE_PLAIN, 0.0), (pkg.RULE_CONNECT, 0.6), (pkg.RULE_SHORTCUT, 0.7)]
    server = pkg.Server(budget_bytes=512 << 20, streams=2)
    jobs = []
    for k, wl in enumerate(insts):
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        A = len(wl.bases)
        checks = []
        for m in range(min(4, A + 1)):
            arm = -1 if m == 0 else m - 1
            q0, q1 = wl.q0, wl.q1
            if arm >= 0:
                q0 = np.ascontiguousarray(q0[:, 7 * arm:7 * arm + 7])
                q1 = np.ascontiguousarray(q1[:, 7 * arm:7 * arm + 7])
            n = max(1, len(q0) // (m + 1))
            rule, rg = rules[(k + m) % 3]
            checks.append((q0[:n], q1[:n], [16, 32, 64][(k + m) % 3], wl.flags, arm, rule, rg))
        jobs.append((scene, rb, A, checks))
    expect = [[_direct(pkg, cuda, scene, rb, *c) for c in checks] for scene, rb, _, checks in jobs]
    got, errors = [None] * len(jobs), []

    def client(i):
        try:
            scene, rb, A, checks = jobs[i]
            sess = server.session(A, sum(len(c[0]) for c in checks), 64)
            got[i] = sess.validate_many(scene, rb, checks)
            sess.close()
        except Exception as e:  # noqa: BLE001
            errors.append((i, e))

    th = [threading.Thread(target=client, args=(i,)) for i in range(len(jobs))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for i in range(len(jobs)):
        for (v, f), (ev, ef) in zip(got[i], expect[i]):
            assert np.array_equal(v, ev), i
            assert np.array_equal(f, ef), i
    st = server.stats()
    assert st["steps"] == sum(len(j[3]) for j in jobs) and st["bytes_in_use"] == 0
    server.close()


def test_admission_waits_for_budget(cuda, pkg):
    W = pkg.workloads
    wl = W.config2(n_edges=256, seed=1)
    probe = pkg.Server(budget_bytes=64 << 20, streams=1)
    s = probe.session(4, 256, 32)
    footprint = probe.stats()["bytes_in_use"]
    s.close()
    probe.close()
    assert footprint > 0

    server = pkg.Server(budget_bytes=footprint, streams=2)
    first = server.session(4, 256, 32)
    with pytest.raises(pkg.MrpopError) as ei:
        server.session(4, 256, 32, timeout_ms=0)
    assert ei.value.status == 4  # MRPOP_ERR_OUT_OF_MEMORY
    admitted = []

    def late():
        admitted.append(server.session(4, 256, 32, timeout_ms=20000))

    t = threading.Thread(target=late)
    t.start()
    t.join(0.3)
    assert not admitted  # still waiting for room
    scene = pkg.Scene(wl.scene)
    rb = pkg.RobotSet(4, wl.bases)
    v1, f1 = first.validate(scene, rb, wl.q0, wl.q1, 32)
    first.close()
    t.join(20)
    assert admitted
    v2, f2 = admitted[0].validate(scene, rb, wl.q0, wl.q1, 32)
    assert np.array_equal(v1, v2) and np.array_equal(f1, f2)
    ev, ef = _direct(pkg, cuda, scene, rb, wl.q0, wl.q1, 32, wl.flags, -1, pkg.RULE_PLAIN, 0.0)
    assert np.array_equal(v1, ev) and np.array_equal(f1, ef)
    with pytest.raises(pkg.MrpopError):  # larger than the session was opened for
        admitted[0].validate(scene, rb, np.concatenate([wl.q0, wl.q0]), np.concatenate([wl.q1, wl.q1]), 32)
    admitted[0].close()
    st = server.stats()
    assert st["admission_waits"] >= 1 and st["admission_timeouts"] >= 1 and st["bytes_in_use"] == 0
    server.close()


def _collision_free(pkg, cuda):
    def cf(scene_arrays, bases, q):
        scene = pkg.Scene(scene_arrays)
        rb = pkg.RobotSet(len(bases), bases)
        d = cuda.from_numpy(np.ascontiguousarray(q)).cuda()
        v, _ = pkg.validate(scene, rb, d, d, 1, pkg.CHECK_ENV | pkg.CHECK_SELF)
        cuda.cuda.synchronize()
        return v.cpu().numpy().astype(bool)
    return cf


def test_served_plans_equal_isolated_plans(cuda, pkg):
    P, S = pkg.planner, pkg.serving
    queries = P.make_queries(10, seed=11, collision_free=_collision_free(pkg, cuda))
    settings = P.PlanSettings(max_iters=30)
    server = pkg.Server(budget_bytes=256 << 20, streams=4)
    alone = S.isolated(server, queries, settings)
    assert server.stats()["max_wave_steps"] == 1
    server.close()
    # one launch slot: steps that arrive while a wave runs wait and share the next one
    shared = pkg.Server(budget_bytes=256 << 20, streams=1)
    mixed = S.stream(shared, queries, rate=1e5, settings=settings, seed=1, clients=16)
    for a, m in zip(alone, mixed):
        assert S.same_result(a.result, m.result), a.result.qid
    assert any(a.result.solved for a in alone)
    st = shared.stats()
    assert st["max_wave_steps"] >= 2  # steps of different queries shared waves
    assert st["bytes_in_use"] == 0
    shared.close()


def test_served_drrt_solves_equal_isolated_solves(cuda, pkg):
    """The reference's planner (dRRT / AO-x) served: each query's checks become
    session steps co-batched with the other queries' steps.  Every query's
    result -- path, cost, counters -- is the same alone and in the mix, and
    equal to a solve on direct library calls."""
    P, S = pkg.planner, pkg.serving
    queries = P.make_queries(6, seed=21, collision_free=_collision_free(pkg, cuda))
    st = pkg.drrt.settings(num_new_configs=48, granularity=16, range=1.5, rrtc_iter=2, max_iters=30,
                           block_per_robot=2, max_launches=4)
    server = pkg.Server(budget_bytes=512 << 20, streams=4)
    alone = S.isolated(server, queries, st)
    server.close()
    shared = pkg.Server(budget_bytes=512 << 20, streams=1)
    mixed = S.stream(shared, queries, rate=1e5, settings=st, seed=2, clients=6)
    for a, m in zip(alone, mixed):
        assert S.same_result(a.result, m.result), a.result.qid
    assert shared.stats()["max_wave_steps"] >= 2
    shared.close()
    # the same solve on direct calls (mrpop_drrt_solve): same path and cost
    q = queries[0]
    s0 = pkg.drrt.settings(**{k: getattr(st, k) for k, _ in st._fields_})
    s0.seed = q.seed
    direct = pkg.drrt.solve(pkg.Scene(q.scene), pkg.RobotSet(q.arms, q.bases), q.start, q.goal, s0)
    assert direct.solved == alone[0].result.solved and np.array_equal(direct.path, alone[0].result.path)
