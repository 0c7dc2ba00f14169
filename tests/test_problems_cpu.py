"""The problem-file loader (mrpop_gb300.problems) on hand-made problem dicts in
the reference's JSON schema, and against the committed benchmark fixture."""
import json

import numpy as np


def _problem(name, valid=True):
    return {
        "name": name, "valid": valid, "source_index": 7,
        "sphere": [{"name": "s0", "position": [0.1, 0.2, 0.3], "radius": 0.05}],
        "cylinder": [{"name": "c0", "position": [0.4, 0.0, 0.2], "orientation_euler_xyz": [0.1, 0.2, 0.3],
                      "radius": 0.04, "length": 0.3}],
        "box": [{"name": "b0", "position": [0.0, 0.5, 0.1], "orientation_euler_xyz": [0.0, 0.0, 0.7],
                 "half_extents": [0.1, 0.2, 0.05]}],
        "start": [0.0] * 28, "goals": [[0.1] * 28, [0.2] * 28],
        "base_positions": [[0.5, 0.5, 0.0]] * 4, "base_orientation_wxyz": [[1.0, 0.0, 0.0, 0.0]] * 4,
    }


def test_loader_maps_every_shape(pkg):
    P = pkg.problems
    W = pkg.workloads
    probs = P.load_problems(json.dumps([_problem("table"), _problem("box"), _problem("shelf", valid=False)]))
    assert [p.name for p in probs] == ["table", "box"]
    t, b = probs
    assert t.index == 7 and t.start.shape == (28,) and t.goals.shape == (2, 28)
    assert np.allclose(t.scene.spheres, [[0.1, 0.2, 0.3, 0.05]])
    assert np.array_equal(t.scene.capsules[0], W.capsule_f32([0.4, 0.0, 0.2], [0.1, 0.2, 0.3], 0.04, 0.3))
    assert np.array_equal(t.scene.cuboids[0], W.box_f32([0.0, 0.5, 0.1], [0.0, 0.0, 0.7], [0.1, 0.2, 0.05]))
    # the float64 construction agrees to 1e-6
    t64 = P.load_problems(json.dumps([_problem("table")]))[0]
    assert np.abs(P.problem_scene(_problem("table"), "f64").cuboids - t64.scene.cuboids).max() < 1e-6
    # problems named "box" turn cylinders into boxes of half extents (r, r, r/2), ahead of the boxes
    assert len(b.scene.capsules) == 0 and len(b.scene.cuboids) == 2
    assert np.allclose(b.scene.cuboids[0][12:], [0.04, 0.04, 0.02])
    assert b.bases.shape == (4, 4, 4) and np.allclose(b.bases[0][:3, 3], [0.5, 0.5, 0.0])
    assert len(P.load_problems([_problem("x", valid=False)], include_invalid=True)) == 1


def test_capsule_record_is_a_segment(pkg):
    c = pkg.workloads.capsule([0.0, 0.0, 0.5], [0.0, 0.0, 0.0], 0.05, 0.4)
    assert np.allclose(c[:3], [0, 0, 0.7]) and np.allclose(c[3:6], [0, 0, -0.4])
    assert np.isclose(c[7], 1.0 / 0.16, rtol=1e-6)


def test_fixture_bases_are_rigid(pkg):
    from pathlib import Path
    d = np.load(Path(__file__).parent / "golden" / "problems.npz")
    for arms in (4, 5):
        b = d[f"a{arms}_bases"].astype(np.float64)
        for t in b:
            assert np.allclose(t[:3, :3] @ t[:3, :3].T, np.eye(3), atol=1e-6)


def test_float32_factory_matches_float64_on_every_fixture_problem(pkg):
    """The boxes of the reference's 100 benchmark problems, built in float32 as
    its Eigen factory does (AngleAxisf products, factory.hh:26-41), agree with
    the float64 construction to 1e-6, and the fixture holds the float32 ones."""
    from pathlib import Path
    W = pkg.workloads
    d = np.load(Path(__file__).parent / "golden" / "problems.npz")
    worst = 0.0
    for arms in (4, 5):
        for i in range(int(d[f"n{arms}"])):
            params = d[f"a{arms}_p{i}_box_params"]
            boxes = d[f"a{arms}_p{i}_boxes"]
            assert len(params) == len(boxes)
            for prm, rec in zip(params, boxes):
                f32 = W.box_f32(prm[0:3], prm[3:6], prm[6:9])
                f64 = W.box(prm[0:3], prm[3:6], prm[6:9])
                assert np.array_equal(f32, rec)
                worst = max(worst, float(np.abs(f32.astype(np.float64) - f64).max()))
    assert worst < 1e-6


def test_float32_factory_on_general_rotations(pkg):
    """Arbitrary Euler angles (the fixture's are mostly plain yaws): boxes and
    capsules from the float32 path stay within 1e-6 of the float64 path."""
    W = pkg.workloads
    rng = np.random.default_rng(3)
    for _ in range(500):
        c, e = rng.uniform(-1, 1, 3), rng.uniform(-3.2, 3.2, 3)
        h = rng.uniform(0.01, 0.3, 3)
        assert np.abs(W.box_f32(c, e, h).astype(np.float64) - W.box(c, e, h)).max() < 1e-6
        a, b = W.capsule_f32(c, e, 0.05, 0.4), W.capsule(c, e, 0.05, 0.4)
        assert np.abs(a[:7].astype(np.float64) - b[:7]).max() < 1e-6
        assert abs(a[7] / b[7] - 1) < 1e-5
