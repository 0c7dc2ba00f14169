"""The forearm-hand rows table (panda_model.cuh, built by the library's host
code) against the oracle: for configurations in cells the table marks apart,
no detailed row between the joint-5 spheres and the hand may fire, under
either reading of the rows (sphere index, or the composite robots' position
of sphere r with the radius of first(r), panda_four.cuh:388-413)."""
import numpy as np

LO6, HI6, LO7, HI7 = -0.0873, 3.8223, -2.9671, 2.9671


def _cells(T, q6, q7):
    n6, n7 = T.shape
    f6 = (np.float32(q6) - np.float32(LO6)) * np.float32(n6 / (np.float32(HI6) - np.float32(LO6)))
    f7 = (np.float32(q7) - np.float32(LO7)) * np.float32(n7 / (np.float32(HI7) - np.float32(LO7)))
    ok = (f6 >= 0) & (f6 < n6) & (f7 >= 0) & (f7 < n7)
    apart = np.zeros(len(q6), bool)
    apart[ok] = T[f6[ok].astype(int), f7[ok].astype(int)]
    return apart


def _row_hits(P, det_r):
    """Per sample: does any forearm-hand row fire (FP32 test as in utils.cuh:100-107)?"""
    P = P.astype(np.float32)
    hit = np.zeros(len(P), bool)
    for s in range(17, 29):
        for rad_s in {det_r[s], det_r[s + 4] if s + 4 <= 28 else det_r[s]}:
            d = P[:, s, None, :] - P[:, 32:59, :]
            sq = (d * d).sum(-1, dtype=np.float32)
            rs = np.float32(rad_s) + det_r[32:59].astype(np.float32)
            hit |= (sq - rs * rs < 0).any(1)
    return hit


def test_table_never_marks_a_firing_row(pkg, lib_path, orc):
    lib = pkg.library(path=lib_path)
    T = pkg.mrpop.row5_table(lib)
    assert T.shape == (256, 384) and 0.85 < T.mean() < 0.99
    W = pkg.workloads
    rng = np.random.default_rng(0)
    det_r = orc.det_spheres()[:, 3]
    n = 60000
    q = W.random_configs(rng, n, 1)
    # half the samples near the unsafe cells, where the rows can fire
    bad = np.argwhere(~T)
    pick = bad[rng.integers(0, len(bad), n // 2)]
    q[: n // 2, 5] = LO6 + (pick[:, 0] + rng.uniform(0, 1, n // 2)) * (HI6 - LO6) / 256
    q[: n // 2, 6] = LO7 + (pick[:, 1] + rng.uniform(0, 1, n // 2)) * (HI7 - LO7) / 384
    q = q.astype(np.float32)
    apart = _cells(T, q[:, 5], q[:, 6])
    base = W.bases_config2()[1]
    P32 = orc.fk_spheres(base, q, True, fp64=False)
    hits = _row_hits(P32, det_r)
    assert hits.sum() > 100          # the rows do fire near the unmarked cells
    assert not (hits & apart).any()  # and never in a marked one
    # FP64 distances in marked cells clear the table's margin
    P64 = orc.fk_spheres(base, q[apart][:5000], True, fp64=True)
    gap = np.inf
    for s in range(17, 29):
        rad = max(det_r[s], det_r[s + 4]) if s + 4 <= 28 else det_r[s]
        d = np.linalg.norm(P64[:, s, None, :] - P64[:, 32:59, :], axis=2) - rad - det_r[32:59]
        gap = min(gap, d.min())
    assert gap > 2e-4
