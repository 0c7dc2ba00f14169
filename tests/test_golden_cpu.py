"""The oracle pinned against the reference itself (no GPU needed here).

tests/golden/ref_golden.npz holds small seeded cases run through the
reference's own fkcc_single_buffer* device code on a GB300 (made by
tests/golden/make_ref_golden.py): inputs, the reference's verdicts and failing
segment, the reference's sphere centres, and the device sin/cos values of
every joint angle used.  The oracle, replaying those sin/cos values, must
reproduce every verdict and every sphere centre bit for bit."""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).parent / "golden" / "ref_golden.npz"


@pytest.fixture(scope="module")
def gold():
    if not GOLDEN.exists():
        pytest.skip("golden vectors not captured")
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def trig(gold, orc):
    return orc.TrigTable(gold["trig_x"], gold["trig_cos"], gold["trig_sin"])


def _scene(pkg, gold, name):
    kw = {}
    for k in ("spheres", "capsules", "z_capsules", "cylinders", "cuboids", "z_cuboids"):
        key = f"{name}_scene_{k}"
        if key in gold:
            kw[k] = gold[key]
    return pkg.SceneArrays(**kw)


@pytest.mark.parametrize("name", ["single", "quad", "quad_extend", "five", "quad_connect", "five_shortcut",
                                  "quad_bspline"])
def test_oracle_reproduces_reference_verdicts(pkg, orc, gold, trig, name):
    g, flags, arm, rule, rng = gold[f"{name}_meta"]
    g, flags, arm, rule = int(g), int(flags), int(arm), int(rule)
    r = orc.validate(_scene(pkg, gold, name), gold[f"{name}_bases"], gold[f"{name}_q0"], gold[f"{name}_q1"], g,
                     flags, arm, rule, float(rng), trig=trig)
    assert np.array_equal(r["valid"], gold[f"{name}_valid"])
    seg = np.where(r["first_hit"] > 0, (r["first_hit"] - 1) // g, -1)
    assert np.array_equal(seg, gold[f"{name}_segfail"])


def test_oracle_reproduces_reference_sphere_centres(orc, gold, trig):
    for det in (0, 1):
        ref = gold[f"fk1_d{det}"][:, 0]
        got = orc.fk_spheres(np.eye(4), gold["fk1_q"], det, fp64=False, trig=trig).astype(np.float32)
        assert np.array_equal(got, ref)
        ref4 = gold[f"fk4_d{det}"]
        for a in range(4):
            got = orc.fk_spheres(gold["fk4_bases"][a], gold["fk4_q"][:, 7 * a:7 * a + 7], det, fp64=False,
                                 trig=trig).astype(np.float32)
            assert np.array_equal(got, ref4[:, a])


def test_other_pair_order_does_not_reproduce(orc, gold, trig):
    """The pin is sharp: fusing the other product of each two-product sum
    (pair_order=1) changes sphere centres."""
    got = orc.fk_spheres(np.eye(4), gold["fk1_q"], 1, fp64=False, pair_order=1, trig=trig).astype(np.float32)
    assert not np.array_equal(got, gold["fk1_d1"][:, 0])
