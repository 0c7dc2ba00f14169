"""GPU parity tests: the CUDA validator (through the C ABI) against the oracle
and against the reference's own device code (oracle/_ref harness)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BAND = 1e-5  # metres: minimum signed distances within this band may legitimately flip


def _trig_table(cuda, pkg, orc, values):
    """Device __cosf/__sinf values for every input the oracle will need."""
    x = cuda.from_numpy(np.ascontiguousarray(values, np.float32).ravel()).cuda()
    c, s = pkg.debug_trig(x)
    cuda.cuda.synchronize()
    return orc.TrigTable(x.cpu().numpy(), c.cpu().numpy(), s.cpu().numpy())


def _edge_trig(cuda, pkg, orc, q0, q1, g, rule=0, range_=0.0):
    samples = orc.edge_samples(q0, q1, g, rule, range_)
    return _trig_table(cuda, pkg, orc, samples)


def _run(cuda, pkg, scene, robots, wl, flags=None, arm=None, rule=None, range_=None, g=None):
    q0 = cuda.from_numpy(wl.q0).cuda()
    q1 = cuda.from_numpy(wl.q1).cuda()
    out = pkg.validate(scene, robots, q0, q1, g or wl.granularity, wl.flags if flags is None else flags,
                       wl.arm if arm is None else arm, wl.rule if rule is None else rule,
                       wl.range_ if range_ is None else range_)
    cuda.cuda.synchronize()
    return [o.cpu().numpy() for o in out]


def _workloads(pkg):
    W = pkg.workloads
    return {
        "c1": W.config1(n_edges=1024, seed=1),
        "c2": W.config2(n_edges=384, seed=2),
        "c3": W.config3(n_edges=96, seed=3),
        "c3s": W.config3_shortcuts(n_paths=8, pairs=8, seed=4),
    }


@pytest.fixture(autouse=True, params=["small-calls-fused", "all-split"])
def launch_form(request, pkg):
    """Every test runs twice: with the default launch form (calls of at most
    2048 edges as one fused launch) and with every call split into the broad
    and narrow kernels (mrpop_set_fused_edges(-1))."""
    lib = pkg.library()
    prev = lib.mrpop_set_fused_edges(0 if request.param == "small-calls-fused" else -1)
    yield request.param
    lib.mrpop_set_fused_edges(prev)


@pytest.fixture(scope="module")
def wls(pkg):
    return _workloads(pkg)


# ---------------------------------------------------------------- FK ------
def test_fk_spheres_within_1e5_of_fp64(cuda, pkg, orc):
    W = pkg.workloads
    rng = np.random.default_rng(0)
    q = W.random_configs(rng, 4096, 1)
    for bases in (np.eye(4, dtype=np.float32)[None], W.bases_config2(), W.bases_config3()):
        rb = pkg.RobotSet(len(bases), bases)
        for arm in range(len(bases)):
            for det in (False, True):
                got = pkg.fk_spheres(rb, arm, cuda.from_numpy(q).cuda(), det).cpu().numpy()
                ref = orc.fk_spheres(bases[arm], q, det, fp64=True)
                assert np.abs(got - ref).max() < 1e-5


def test_fk_spheres_bitexact_vs_oracle_mirror(cuda, pkg, orc):
    W = pkg.workloads
    rng = np.random.default_rng(1)
    q = W.random_configs(rng, 4096, 1)
    trig = _trig_table(cuda, pkg, orc, q)
    bases = W.bases_config2()
    rb = pkg.RobotSet(4, bases)
    for det in (False, True):
        got = pkg.fk_spheres(rb, 1, cuda.from_numpy(q).cuda(), det).cpu().numpy()
        ref = orc.fk_spheres(bases[1], q, det, fp64=False, trig=trig).astype(np.float32)
        assert np.array_equal(got, ref), np.abs(got - ref).max()


# ------------------------------------------------------ validator vs oracle
@pytest.mark.parametrize("name", ["c1", "c2", "c3", "c3s"])
@pytest.mark.parametrize("exact", [False, True])
def test_validate_bitexact_vs_oracle(cuda, pkg, orc, wls, name, exact):
    wl = wls[name]
    scene = pkg.Scene(wl.scene)
    rb = pkg.RobotSet(len(wl.bases), wl.bases)
    flags = wl.flags | (pkg.MODE_EXACT if exact else 0)
    got = _run(cuda, pkg, scene, rb, wl, flags=flags)
    trig = _edge_trig(cuda, pkg, orc, wl.q0, wl.q1, wl.granularity, wl.rule, wl.range_)
    ref = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, flags, wl.arm, wl.rule, wl.range_,
                       trig=trig)
    assert scene.status() == 0
    assert np.array_equal(got[0], ref["valid"])
    assert np.array_equal(got[1], ref["first_hit"])
    if len(got) > 2:
        assert np.array_equal(got[2], ref["n_seg"])


def test_validate_vs_oracle_fp64_trig_outside_band(cuda, pkg, orc, wls):
    """Against the oracle with exact sin/cos: any difference must be an ambiguous edge."""
    for name in ("c1", "c2", "c3"):
        wl = wls[name]
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        got = _run(cuda, pkg, scene, rb, wl)
        ref = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, wl.flags, wl.arm, band=BAND)
        diff = (got[0] != ref["valid"]) | (got[1] != ref["first_hit"])
        assert not (diff & (ref["ambiguous"] == 0)).any()


@pytest.mark.parametrize("g", [1, 2, 16, 31, 32, 33, 48, 64])
def test_granularities(cuda, pkg, orc, g):
    W = pkg.workloads
    wl = W.config2(n_edges=96, seed=10 + g)
    scene = pkg.Scene(wl.scene)
    rb = pkg.RobotSet(4, wl.bases)
    for flags in (wl.flags, pkg.CHECK_SELF, pkg.CHECK_ENV | pkg.MODE_EXACT):
        got = _run(cuda, pkg, scene, rb, wl, flags=flags, g=g)
        trig = _edge_trig(cuda, pkg, orc, wl.q0, wl.q1, g)
        ref = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, g, flags, trig=trig)
        assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])


@pytest.mark.parametrize("arms", [1, 2, 3, 4, 5])
def test_every_arm_count_and_single_arm_forms(cuda, pkg, orc, arms):
    W = pkg.workloads
    rng = np.random.default_rng(100 + arms)
    bases = W.bases_facing_centre(arms, 0.71)
    q0, q1 = W.random_edges(rng, 128, arms, 1.5)
    scene_arrays = W.scene_config2(arms)
    scene = pkg.Scene(scene_arrays)
    rb = pkg.RobotSet(arms, bases)
    g = 32
    trig = _edge_trig(cuda, pkg, orc, q0, q1, g)
    for flags in (pkg.CHECK_ENV | pkg.CHECK_SELF, pkg.CHECK_SELF):
        wl = W.Workload("t", scene_arrays, bases, q0, q1, g, flags)
        got = _run(cuda, pkg, scene, rb, wl)
        ref = orc.validate(scene_arrays, bases, q0, q1, g, flags, trig=trig)
        assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])
    # single-arm (roadmap) form on each arm's base
    for a in range(arms):
        qa0, qa1 = np.ascontiguousarray(q0[:, 7 * a:7 * a + 7]), np.ascontiguousarray(q1[:, 7 * a:7 * a + 7])
        wl = W.Workload("t", scene_arrays, bases, qa0, qa1, g, pkg.CHECK_ENV | pkg.CHECK_SELF, arm=a)
        got = _run(cuda, pkg, scene, rb, wl)
        ref = orc.validate(scene_arrays, bases, qa0, qa1, g, wl.flags, arm=a, trig=trig)
        assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])


@pytest.mark.parametrize("arms,g", [(1, 64), (2, 48), (2, 64)])
def test_one_and_two_arms_above_32_samples(cuda, pkg, orc, arms, g):
    """Small calls of 1 and 2 arms above 32 samples per segment run two warps
    per edge in the fused form (pair_kernel): composite and single-arm forms,
    plain and connect rules."""
    W = pkg.workloads
    rng = np.random.default_rng(200 + 10 * arms + g)
    bases = W.bases_facing_centre(arms, 0.71)
    q0, q1 = W.random_edges(rng, 128, arms, 1.5)
    scene_arrays = W.scene_config2(arms)
    scene = pkg.Scene(scene_arrays)
    rb = pkg.RobotSet(arms, bases)
    for rule, rg in ((0, 0.0), (1, 0.6)):
        trig = _edge_trig(cuda, pkg, orc, q0, q1, g, rule, rg)
        for flags in (pkg.CHECK_ENV | pkg.CHECK_SELF, pkg.CHECK_SELF):
            wl = W.Workload("t", scene_arrays, bases, q0, q1, g, flags, rule=rule, range_=rg)
            got = _run(cuda, pkg, scene, rb, wl)
            ref = orc.validate(scene_arrays, bases, q0, q1, g, flags, -1, rule, rg, trig=trig)
            assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])
        for a in range(arms):
            qa0, qa1 = np.ascontiguousarray(q0[:, 7 * a:7 * a + 7]), np.ascontiguousarray(q1[:, 7 * a:7 * a + 7])
            ta = _edge_trig(cuda, pkg, orc, qa0, qa1, g, rule, rg)
            wl = W.Workload("t", scene_arrays, bases, qa0, qa1, g, pkg.CHECK_ENV | pkg.CHECK_SELF, arm=a, rule=rule,
                            range_=rg)
            got = _run(cuda, pkg, scene, rb, wl)
            ref = orc.validate(scene_arrays, bases, qa0, qa1, g, wl.flags, a, rule, rg, trig=ta)
            assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])
    assert scene.status() == 0


def test_all_obstacle_classes(cuda, pkg, orc):
    """Spheres, capsules, z-capsules, boxes and z-boxes in one scene; cylinders ignored."""
    W = pkg.workloads
    rng = np.random.default_rng(7)
    lo, hi = np.array([-0.9, -0.9, 0.0]), np.array([0.9, 0.9, 1.2])
    sc = pkg.SceneArrays(
        spheres=np.stack([np.array([*rng.uniform(lo, hi), rng.uniform(0.03, 0.15)], np.float32) for _ in range(6)]),
        capsules=np.stack([W.capsule(rng.uniform(lo, hi), rng.uniform(-1, 1, 3), rng.uniform(0.02, 0.08),
                                     rng.uniform(0.1, 0.5)) for _ in range(6)]),
        z_capsules=np.stack([W.capsule(rng.uniform(lo, hi), (0, 0, 0), rng.uniform(0.02, 0.08), rng.uniform(0.1, 0.5))
                             for _ in range(6)]),
        cylinders=np.stack([W.capsule((0, 0, 0.5), (0, 0, 0), 0.5, 0.5)]),
        cuboids=np.stack([W.box(rng.uniform(lo, hi), rng.uniform(-1, 1, 3), rng.uniform(0.03, 0.2, 3))
                          for _ in range(6)]),
        z_cuboids=np.stack([W.box(rng.uniform(lo, hi), (0, 0, rng.uniform(-3, 3)), rng.uniform(0.03, 0.2, 3))
                            for _ in range(6)]))
    bases = W.bases_config2()
    q0, q1 = W.random_edges(rng, 256, 4, 1.5)
    scene = pkg.Scene(sc)
    rb = pkg.RobotSet(4, bases)
    wl = W.Workload("t", sc, bases, q0, q1, 32, pkg.CHECK_ENV | pkg.CHECK_SELF)
    got = _run(cuda, pkg, scene, rb, wl)
    trig = _edge_trig(cuda, pkg, orc, q0, q1, 32)
    ref = orc.validate(sc, bases, q0, q1, 32, wl.flags, trig=trig)
    assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])


@pytest.mark.parametrize("rule", [1, 2, 3])
def test_segment_rules(cuda, pkg, orc, rule):
    W = pkg.workloads
    rng = np.random.default_rng(30 + rule)
    bases = W.bases_config2()
    q0, q1 = W.random_edges(rng, 96, 4, 6.0)
    sc = W.scene_config2(1)
    scene = pkg.Scene(sc)
    rb = pkg.RobotSet(4, bases)
    for rng_ in (0.5, 2.0):
        wl = W.Workload("t", sc, bases, q0, q1, 16, pkg.CHECK_ENV | pkg.CHECK_SELF, rule=rule, range_=rng_)
        got = _run(cuda, pkg, scene, rb, wl)
        trig = _edge_trig(cuda, pkg, orc, q0, q1, 16, rule, rng_)
        ref = orc.validate(sc, bases, q0, q1, 16, wl.flags, rule=rule, range_=rng_, trig=trig)
        assert np.array_equal(got[2], ref["n_seg"])
        assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])


def test_empty_inputs_and_scene(cuda, pkg):
    W = pkg.workloads
    scene = pkg.Scene(pkg.SceneArrays())
    rb = pkg.RobotSet(4, W.bases_config2())
    z = cuda.zeros((0, 28), dtype=cuda.float32, device="cuda")
    v, f = pkg.validate(scene, rb, z, z, 32)
    assert v.numel() == 0
    # empty scene: env flag alone can never fire
    rng = np.random.default_rng(3)
    q0, q1 = W.random_edges(rng, 64, 4, 1.0)
    wl = W.Workload("t", pkg.SceneArrays(), W.bases_config2(), q0, q1, 32, pkg.CHECK_ENV)
    got = _run(cuda, pkg, scene, rb, wl)
    assert got[0].all() and (got[1] == -1).all()


def test_flop_tally_matches_oracle(cuda, pkg, orc, wls):
    for name in ("c1", "c2", "c3s"):
        wl = wls[name]
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        fl = pkg.count_flops(scene, rb, cuda.from_numpy(wl.q0).cuda(), cuda.from_numpy(wl.q1).cuda(),
                             wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_).cpu().numpy()
        trig = _edge_trig(cuda, pkg, orc, wl.q0, wl.q1, wl.granularity, wl.rule, wl.range_)
        ref = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_,
                           trig=trig)
        assert abs(fl.sum() - ref["flops"]) <= 1e-9 * ref["flops"]


def test_host_buffer_path_equals_device_path(cuda, pkg, wls):
    wl = wls["c2"]
    scene = pkg.Scene(wl.scene)
    rb = pkg.RobotSet(4, wl.bases)
    dev = _run(cuda, pkg, scene, rb, wl)
    ws = pkg.Workspace()
    v, f = ws.validate(scene, rb, wl.q0, wl.q1, wl.granularity, wl.flags)
    assert np.array_equal(v, dev[0]) and np.array_equal(f, dev[1])


def test_host_buffer_path_large_batches(cuda, pkg):
    """Full-size batches through the host-buffer path give the device-path
    results, plain and segmented, on a reused workspace."""
    W = pkg.workloads
    for wl in (W.config2(n_edges=70001, seed=41), W.config3_shortcuts(n_paths=1100, pairs=64, seed=42)):
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        dev = _run(cuda, pkg, scene, rb, wl)
        ws = pkg.Workspace()
        for _ in range(2):  # the workspace's buffers are reused
            v, f = ws.validate(scene, rb, wl.q0, wl.q1, wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_)
            assert np.array_equal(v, dev[0]) and np.array_equal(f, dev[1])


def test_host_buffer_path_pinned_in_place(cuda, pkg):
    """Page-locked host buffers are used in place (the kernels read the
    endpoints and write the verdicts in host memory): same results as the
    device path, plain and segmented, and with only some buffers pinned (those
    calls take the copying path)."""
    W = pkg.workloads
    for wl in (W.config2(n_edges=9001, seed=43), W.config3_shortcuts(n_paths=200, pairs=64, seed=44)):
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        dev = _run(cuda, pkg, scene, rb, wl)
        n = len(wl.q0)
        pinned = [cuda.from_numpy(wl.q0).pin_memory(), cuda.from_numpy(wl.q1).pin_memory(),
                  cuda.full((n,), 7, dtype=cuda.uint8).pin_memory(), cuda.full((n,), -9, dtype=cuda.int32).pin_memory()]
        a0, a1, av, af = (t.numpy() for t in pinned)
        ws = pkg.Workspace()
        for outs in ((av, af), (None, None)):
            v, f = ws.validate(scene, rb, a0, a1, wl.granularity, wl.flags, wl.arm, wl.rule, wl.range_,
                               valid=outs[0], first_hit=outs[1])
            assert np.array_equal(v, dev[0]) and np.array_equal(f, dev[1])
        assert np.array_equal(av, dev[0]) and np.array_equal(af, dev[1])


def test_full_size_properties(cuda, pkg, orc):
    """Config 2 at its full size (65536 edges x 32): repeatability, batch-order and
    chunking invariance, and oracle agreement on a random subset."""
    W = pkg.workloads
    wl = W.config2()
    scene = pkg.Scene(wl.scene)
    rb = pkg.RobotSet(4, wl.bases)
    a = _run(cuda, pkg, scene, rb, wl)
    b = _run(cuda, pkg, scene, rb, wl)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    perm = np.random.default_rng(0).permutation(len(wl.q0))
    wp = W.Workload("p", wl.scene, wl.bases, wl.q0[perm], wl.q1[perm], 32, wl.flags)
    c = _run(cuda, pkg, scene, rb, wp)
    assert np.array_equal(c[0], a[0][perm]) and np.array_equal(c[1], a[1][perm])
    half = len(wl.q0) // 2
    wh = W.Workload("h", wl.scene, wl.bases, wl.q0[half:], wl.q1[half:], 32, wl.flags)
    d = _run(cuda, pkg, scene, rb, wh)
    assert np.array_equal(d[0], a[0][half:])
    sub = np.random.default_rng(1).choice(len(wl.q0), 512, replace=False)
    trig = _edge_trig(cuda, pkg, orc, wl.q0[sub], wl.q1[sub], 32)
    ref = orc.validate(wl.scene, wl.bases, wl.q0[sub], wl.q1[sub], 32, wl.flags, trig=trig)
    assert np.array_equal(a[0][sub], ref["valid"]) and np.array_equal(a[1][sub], ref["first_hit"])
    assert scene.status() == 0


def test_forearm_hand_rows_near_contact(cuda, pkg, orc):
    """Edges whose joint-6/7 values cross the cells where the forearm-hand rows
    can fire (the table leaves those cells unmarked): verdicts still match the
    oracle, composite and single-arm readings, REF and EXACT modes."""
    W = pkg.workloads
    T = pkg.mrpop.row5_table()
    rng = np.random.default_rng(77)
    bad = np.argwhere(~T)
    n = 256
    bases = W.bases_config2()
    q0, q1 = W.random_edges(rng, n, 4, 0.6)
    for a in range(4):
        pick = bad[rng.integers(0, len(bad), n)]
        q6 = -0.0873 + (pick[:, 0] + rng.uniform(0, 1, n)) * (3.8223 + 0.0873) / 256
        q7 = -2.9671 + (pick[:, 1] + rng.uniform(0, 1, n)) * (2 * 2.9671) / 384
        q0[:, 7 * a + 5], q0[:, 7 * a + 6] = q6, q7
        q1[:, 7 * a + 5] = np.clip(q6 + rng.uniform(-0.1, 0.1, n), -0.0873, 3.8223)
        q1[:, 7 * a + 6] = np.clip(q7 + rng.uniform(-0.1, 0.1, n), -2.9671, 2.9671)
    q0, q1 = q0.astype(np.float32), q1.astype(np.float32)
    sc = W.scene_config2(4)
    scene = pkg.Scene(sc)
    rb = pkg.RobotSet(4, bases)
    trig = _edge_trig(cuda, pkg, orc, q0, q1, 32)
    fired = 0
    for flags in (pkg.CHECK_SELF, pkg.CHECK_SELF | pkg.MODE_EXACT, pkg.CHECK_ENV | pkg.CHECK_SELF):
        wl = W.Workload("t", sc, bases, q0, q1, 32, flags)
        got = _run(cuda, pkg, scene, rb, wl)
        ref = orc.validate(sc, bases, q0, q1, 32, flags, trig=trig)
        assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])
        fired += int((ref["valid"] == 0).sum())
        for a in range(4):
            qa0, qa1 = np.ascontiguousarray(q0[:, 7 * a:7 * a + 7]), np.ascontiguousarray(q1[:, 7 * a:7 * a + 7])
            wl = W.Workload("t", sc, bases, qa0, qa1, 32, flags, arm=a)
            got = _run(cuda, pkg, scene, rb, wl)
            ref = orc.validate(sc, bases, qa0, qa1, 32, flags, arm=a, trig=trig)
            assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"])
    assert fired > 0


def test_concurrent_host_threads(cuda, pkg):
    """Several host threads validating at once, each on its own stream with its
    own scene size (different shared-memory sizes), give the sequential results."""
    import threading
    W = pkg.workloads
    jobs = []
    for k, wl in enumerate([W.config1(n_edges=512, seed=21), W.config2(n_edges=512, seed=22),
                            W.config3(n_edges=256, seed=23), W.config2(n_edges=300, seed=24)]):
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        q0, q1 = cuda.from_numpy(wl.q0).cuda(), cuda.from_numpy(wl.q1).cuda()
        ref = pkg.validate(scene, rb, q0, q1, wl.granularity, wl.flags, wl.arm)
        cuda.cuda.synchronize()
        jobs.append((scene, rb, q0, q1, wl, [r.cpu().numpy() for r in ref]))
    errors = []

    def work(job):
        scene, rb, q0, q1, wl, ref = job
        s = cuda.cuda.Stream()
        try:
            for _ in range(20):
                with cuda.cuda.stream(s):
                    v, f = pkg.validate(scene, rb, q0, q1, wl.granularity, wl.flags, wl.arm, stream=s)
                s.synchronize()
                if not (np.array_equal(v.cpu().numpy(), ref[0]) and np.array_equal(f.cpu().numpy(), ref[1])):
                    errors.append(wl.name)
                    return
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(j,)) for j in jobs]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors


@pytest.mark.parametrize("seed", [11, 12])
def test_many_seeds_every_rule_and_mode(cuda, pkg, orc, seed):
    """Bit-exact verdicts against the oracle fed the device's sin/cos on larger
    seeded batches: 4 arms with every segmentation rule, 1 and 5 arms, the
    shortcut workload; reference and exact modes."""
    W = pkg.workloads
    cases = [(W.config2(n_edges=2048, seed=seed), [(pkg.RULE_PLAIN, 0.0), (pkg.RULE_CONNECT, 0.3),
                                                  (pkg.RULE_BSPLINE, 0.5), (pkg.RULE_SHORTCUT, 0.4)]),
             (W.config1(n_edges=4096, seed=seed), [(pkg.RULE_PLAIN, 0.0)]),
             (W.config3(n_edges=512, seed=seed), [(pkg.RULE_PLAIN, 0.0)]),
             (W.config3_shortcuts(n_paths=32, pairs=16, seed=seed), [(pkg.RULE_SHORTCUT, 2.0)])]
    for wl, rules in cases:
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        for rule, range_ in rules:
            trig = _edge_trig(cuda, pkg, orc, wl.q0, wl.q1, wl.granularity, rule, range_)
            for exact in (False, True):
                flags = wl.flags | (pkg.MODE_EXACT if exact else 0)
                got = _run(cuda, pkg, scene, rb, wl, flags=flags, rule=rule, range_=range_)
                ref = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, flags, wl.arm, rule, range_,
                                   trig=trig)
                assert np.array_equal(got[0], ref["valid"]) and np.array_equal(got[1], ref["first_hit"]), (rule, exact)
                if len(got) > 2:
                    assert np.array_equal(got[2], ref["n_seg"])
        assert scene.status() == 0
