"""The reference's planner (dRRT / AO-x, dRRT::solve) on the GPU validator.

A solve through the library's kernels (mrpop_drrt_solve: batched edge checks
on the GPU, nearest-neighbour searches as a kernel over device copies of the
trees) must equal, waypoint for waypoint, the same solve driven by the oracle
(mrpop_drrt_solve_with: the oracle as the validator with the device's
__sinf/__cosf values replayed, searches on the host): the planner's host logic
is shared, the verdicts are bit-identical, and the searches round alike."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIX_NAME = "problems.npz"


def _fixture():
    from pathlib import Path
    return np.load(Path(__file__).parent / "golden" / FIX_NAME)


def _replay_validator(cuda, pkg, orc, scene, bases):
    def validate(q0, q1, g, rule, range_, flags, arm):
        samples = orc.edge_samples(q0, q1, g, rule, range_)
        x = cuda.from_numpy(np.ascontiguousarray(samples, np.float32).ravel()).cuda()
        c, s = pkg.debug_trig(x)
        cuda.cuda.synchronize()
        trig = orc.TrigTable(x.cpu().numpy(), c.cpu().numpy(), s.cpu().numpy())
        o = orc.validate(scene, bases, q0, q1, g, flags, arm, rule, range_, trig=trig, threads=orc.max_threads())
        return o["valid"], o["first_hit"]
    return validate


@pytest.mark.parametrize("arms,prob", [(4, 0), (5, 2)])
def test_gpu_solve_equals_oracle_driven_solve(cuda, pkg, orc, arms, prob):
    z = _fixture()
    bases = z[f"a{arms}_bases"]
    sc = pkg.SceneArrays(cuboids=z[f"a{arms}_p{prob}_boxes"])
    start, goal = z[f"a{arms}_p{prob}_start"], z[f"a{arms}_p{prob}_goal"]
    st = pkg.drrt.settings(num_new_configs=48, granularity=16, range=2.0, rrtc_iter=2, max_iters=40,
                           block_per_robot=2, max_launches=6)
    scene = pkg.Scene(sc)
    rb = pkg.RobotSet(arms, bases)
    gpu = pkg.drrt.solve(scene, rb, start, goal, st)
    cpu = pkg.drrt.solve_with(arms, _replay_validator(cuda, pkg, orc, sc, bases), start, goal, st)
    assert scene.status() == 0
    assert gpu.solved == cpu.solved and gpu.cost == cpu.cost and gpu.iters == cpu.iters
    assert np.array_equal(gpu.path, cpu.path)
    assert [s.cost for s in gpu.solutions] == [s.cost for s in cpu.solutions]
    for k in ("iterations", "validate_calls", "edges_validated", "roadmap_nodes", "roadmap_edges",
              "start_tree_size", "goal_tree_size", "launches"):
        assert gpu.stats[k] == cpu.stats[k], k


def test_reference_problems_with_the_drivers_settings(cuda, pkg):
    """The benchmark driver's settings (300 attempts per iteration, g = 64,
    range 2.0, three AO-x passes) on reference problems: solutions run from
    the goal to the start and improve from pass to pass."""
    z = _fixture()
    st = pkg.drrt.evaluate_settings()
    for arms, prob in ((4, 1), (5, 3)):
        bases = z[f"a{arms}_bases"]
        scene = pkg.Scene(pkg.SceneArrays(cuboids=z[f"a{arms}_p{prob}_boxes"]))
        rb = pkg.RobotSet(arms, bases)
        start, goal = z[f"a{arms}_p{prob}_start"], z[f"a{arms}_p{prob}_goal"]
        r = pkg.drrt.solve(scene, rb, start, goal, st)
        assert scene.status() == 0
        if r.solved:
            assert np.array_equal(r.path[0], goal) and np.array_equal(r.path[-1], start)
            costs = [s.cost for s in r.solutions]
            assert costs == sorted(costs, reverse=True)
        print(f"drrt arms={arms} problem={prob} solved={r.solved} cost={r.cost:.4f} "
              f"wall_ms={r.stats['wall_ns'] / 1e6:.1f} iterations={r.stats['iterations']} "
              f"validate_calls={r.stats['validate_calls']} edges={r.stats['edges_validated']}")


def test_blocking_wait_and_host_threads_do_not_change_the_solve(cuda, pkg):
    """blocking_wait (sleep on a blocking-sync event instead of spinning) and
    host_threads change only how the host waits and splits its work."""
    z = _fixture()
    bases = z["a4_bases"]
    scene = pkg.Scene(pkg.SceneArrays(cuboids=z["a4_p1_boxes"]))
    rb = pkg.RobotSet(4, bases)
    start, goal = z["a4_p1_start"], z["a4_p1_goal"]
    kw = dict(num_new_configs=64, granularity=32, range=1.5, rrtc_iter=3, max_iters=12, block_per_robot=4,
              max_launches=8)
    a = pkg.drrt.solve(scene, rb, start, goal, pkg.drrt.settings(**kw))
    b = pkg.drrt.solve(scene, rb, start, goal, pkg.drrt.settings(**kw, blocking_wait=1, host_threads=1))
    assert scene.status() == 0
    assert a.solved == b.solved and a.cost == b.cost and np.array_equal(a.path, b.path)
    for k in ("iterations", "validate_calls", "edges_validated", "roadmap_nodes", "roadmap_edges",
              "start_tree_size", "goal_tree_size"):
        assert a.stats[k] == b.stats[k], k


def test_pooled_device_resources_are_reused_and_released(cuda, pkg):
    """Solves take their device resources from a pool and give them back:
    back-to-back solves leave one idle set, releasing frees it, and a solve
    after the release (on fresh resources) gives the same result."""
    z = _fixture()
    scene = pkg.Scene(pkg.SceneArrays(cuboids=z["a4_p0_boxes"]))
    rb = pkg.RobotSet(4, z["a4_bases"])
    st = pkg.drrt.settings(num_new_configs=48, granularity=16, range=2.0, rrtc_iter=2, max_iters=20,
                           block_per_robot=2, max_launches=4)
    pkg.drrt.release_pool(scene.lib)
    a = pkg.drrt.solve(scene, rb, z["a4_p0_start"], z["a4_p0_goal"], st)
    b = pkg.drrt.solve(scene, rb, z["a4_p0_start"], z["a4_p0_goal"], st)
    assert pkg.drrt.release_pool(scene.lib) == 1
    assert pkg.drrt.release_pool(scene.lib) == 0
    c = pkg.drrt.solve(scene, rb, z["a4_p0_start"], z["a4_p0_goal"], st)
    assert scene.status() == 0
    for r in (b, c):
        assert r.solved == a.solved and r.cost == a.cost and np.array_equal(r.path, a.path)
