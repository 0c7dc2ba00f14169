"""GPU parity against the reference's own edge-check device code.

The reference routines run through oracle/ref_harness.cu (compiled from the
reference sources into oracle/_ref/ref_harness.cubin where they are present);
these tests skip where that cubin is absent."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BAND = 1e-5


@pytest.fixture(scope="module")
def ref(cuda):
    from oracle import ref_runner
    if not ref_runner.available():
        pytest.skip("reference harness cubin not built (reference sources absent when built)")
    return ref_runner.RefHarness()


def _dev(cuda, a):
    return cuda.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def test_fk_bitexact_vs_reference(cuda, pkg, ref):
    W = pkg.workloads
    rng = np.random.default_rng(5)
    q1 = W.random_configs(rng, 1000, 1)
    rb1 = pkg.RobotSet(1)
    for det in (False, True):
        mine = pkg.fk_spheres(rb1, 0, _dev(cuda, q1), det).cpu().numpy()
        theirs = ref.fk(_dev(cuda, q1), 0, num_robot=1, robot_id=0, detailed=det).cpu().numpy()[:, 0]
        assert np.array_equal(mine, theirs), np.abs(mine - theirs).max()
    for arms in (4, 5):
        rb = pkg.RobotSet(arms)  # the reference's compiled-in layout
        q = W.random_configs(rng, 500, arms)
        for det in (False, True):
            theirs = ref.fk(_dev(cuda, q), arms, detailed=det).cpu().numpy()
            for a in range(arms):
                mine = pkg.fk_spheres(rb, a, _dev(cuda, q[:, 7 * a:7 * a + 7]), det).cpu().numpy()
                assert np.array_equal(mine, theirs[:, a]), (arms, a, np.abs(mine - theirs[:, a]).max())


def _compare(cuda, pkg, orc, ref, scene_arrays, bases, q0, q1, g, flags, arm, rule, range_, kind, num_robot,
             robot_id, set_bases=True):
    if set_bases and num_robot in (4, 5):
        ref.set_bases(num_robot, bases if len(bases) == num_robot else pkg.workloads.bases_config2())
    scene = pkg.Scene(scene_arrays)
    rb = pkg.RobotSet(len(bases), bases)
    d0, d1 = _dev(cuda, q0), _dev(cuda, q1)
    out = pkg.validate(scene, rb, d0, d1, g, flags, arm, rule, range_)
    env = ref.make_env(scene_arrays)
    rv, rs = ref.validate(env, d0, d1, g, kind, rule, range_, num_robot, robot_id)
    cuda.cuda.synchronize()
    valid = out[0].cpu().numpy()
    first = out[1].cpu().numpy()
    rv, rs = rv.cpu().numpy(), rs.cpu().numpy()
    # the reference reports the failing segment; ours the first colliding sample
    seg = np.where(first > 0, (first - 1) // g, -1)
    diff = (valid != rv) | (seg != rs)
    if diff.any():
        amb = orc.validate(scene_arrays, bases, q0, q1, g, flags, arm, rule, range_, band=BAND)["ambiguous"]
        assert not (diff & (amb == 0)).any(), f"{int(diff.sum())} edges differ, {int((diff & (amb == 0)).sum())} unambiguous"
    return int(diff.sum()), len(valid)


def test_single_arm_roadmap_form(cuda, pkg, orc, ref):
    W = pkg.workloads
    wl = W.config1(n_edges=4096, seed=0)
    n_diff, n = _compare(cuda, pkg, orc, ref, wl.scene, wl.bases, wl.q0, wl.q1, 32, wl.flags, 0, 0, 0.0,
                         ref.KIND_SINGLE, 1, 0)
    assert n_diff == 0


def test_single_arm_on_quad_base(cuda, pkg, orc, ref):
    W = pkg.workloads
    rng = np.random.default_rng(8)
    q0, q1 = W.random_edges(rng, 2048, 1, 1.0)
    sc = W.scene_config2(3)
    bases = W.bases_config2()
    for robot_id in (0, 2):
        _compare(cuda, pkg, orc, ref, sc, bases, q0, q1, 32, pkg.CHECK_ENV | pkg.CHECK_SELF, robot_id, 0, 0.0,
                 ref.KIND_SINGLE, 4, robot_id)


@pytest.mark.parametrize("arms", [4, 5])
def test_composite_env_self(cuda, pkg, orc, ref, arms):
    W = pkg.workloads
    wl = W.config2(n_edges=4096, seed=1) if arms == 4 else W.config3(n_edges=1024, seed=1)
    _compare(cuda, pkg, orc, ref, wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, wl.flags, -1, 0, 0.0,
             ref.KIND_COMPOSITE, arms, 0)


@pytest.mark.parametrize("arms", [4, 5])
def test_composite_native_layout(cuda, pkg, orc, ref, arms):
    """The reference's compiled-in base tables, no overwrite (the benchmark layouts)."""
    W = pkg.workloads
    from oracle import ref_runner  # noqa: F401
    rng = np.random.default_rng(40 + arms)
    from pathlib import Path
    z = np.load(Path(__file__).parent / "golden" / "problems.npz")
    bases = z[f"a{arms}_bases"]
    ref.set_bases(arms, np.stack([np.asarray(b, np.float32) for b in bases]))
    q0, q1 = W.random_edges(rng, 1024, arms, 1.5)
    sc = pkg.SceneArrays(cuboids=z[f"a{arms}_p0_boxes"])
    _compare(cuda, pkg, orc, ref, sc, bases, q0, q1, 32, pkg.CHECK_ENV | pkg.CHECK_SELF, -1, 0, 0.0,
             ref.KIND_COMPOSITE, arms, 0, set_bases=False)


@pytest.mark.parametrize("arms", [4, 5])
def test_extend_self_only(cuda, pkg, orc, ref, arms):
    W = pkg.workloads
    wl = W.config2(n_edges=2048, seed=5) if arms == 4 else W.config3(n_edges=512, seed=5)
    _compare(cuda, pkg, orc, ref, wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, pkg.CHECK_SELF, -1, 0, 0.0,
             ref.KIND_EXTEND, arms, 0)


@pytest.mark.parametrize("rule", [1, 2, 3])
def test_segment_forms(cuda, pkg, orc, ref, rule):
    W = pkg.workloads
    rng = np.random.default_rng(60 + rule)
    bases = W.bases_config2()
    q0, q1 = W.random_edges(rng, 512, 4, 5.0)
    sc = W.scene_config2(6)
    _compare(cuda, pkg, orc, ref, sc, bases, q0, q1, 32, pkg.CHECK_ENV | pkg.CHECK_SELF, -1, rule, 2.0,
             ref.KIND_COMPOSITE, 4, 0)


def test_problem_fixtures_under_reference(cuda, pkg, ref):
    """The 100 benchmark start/goal configurations pass the reference's own check and ours."""
    from pathlib import Path
    z = np.load(Path(__file__).parent / "golden" / "problems.npz")
    for arms in (4, 5):
        bases = z[f"a{arms}_bases"]
        ref.set_bases(arms, bases)
        rb = pkg.RobotSet(arms, bases)
        for p in range(int(z[f"n{arms}"])):
            sc = pkg.SceneArrays(cuboids=z[f"a{arms}_p{p}_boxes"])
            q = np.stack([z[f"a{arms}_p{p}_start"], z[f"a{arms}_p{p}_goal"]]).astype(np.float32)
            d = _dev(cuda, q)
            scene = pkg.Scene(sc)
            v, f = pkg.validate(scene, rb, d, d, 16)
            env = ref.make_env(sc)
            rv, rs = ref.validate(env, d, d, 16, ref.KIND_COMPOSITE, 0, 0.0, arms, 0)
            cuda.cuda.synchronize()
            assert v.cpu().numpy().all() and rv.cpu().numpy().all(), (arms, p)
