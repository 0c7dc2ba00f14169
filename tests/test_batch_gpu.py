"""Batched validation of many planning instances (mrpop_batch_*): results equal
the per-instance plain calls bit for bit, through a plain run, after the
launch-shape tuner, and through the captured CUDA graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(pkg, cuda, n, scale, seed):
    W = pkg.workloads
    insts = W.config4_instances(n_instances=n, seed=seed, scale=scale)
    items = []
    keep = []
    for k, wl in enumerate(insts):
        scene = pkg.Scene(wl.scene)
        rb = pkg.RobotSet(len(wl.bases), wl.bases)
        q0 = cuda.from_numpy(wl.q0).cuda()
        q1 = cuda.from_numpy(wl.q1).cuda()
        arm = -1
        if k % 7 == 3:  # a single-arm (roadmap) item on one arm's base
            arm = len(wl.bases) - 1
            q0 = q0[:, 7 * arm:7 * arm + 7].contiguous()
            q1 = q1[:, 7 * arm:7 * arm + 7].contiguous()
        flags = wl.flags if k % 5 else (pkg.CHECK_SELF | pkg.MODE_EXACT)
        items.append((scene, rb, q0, q1, wl.granularity, flags, arm))
        keep.append(wl)
    # an empty item in the middle
    items.insert(5, (items[0][0], items[0][1], items[0][2][:0], items[0][3][:0], 32, pkg.CHECK_SELF, -1))
    return items


def _reference(pkg, cuda, items):
    out = []
    for scene, rb, q0, q1, g, flags, arm in items:
        v, f = pkg.validate(scene, rb, q0, q1, g, flags, arm)
        out.append((v.cpu().numpy(), f.cpu().numpy()))
    cuda.cuda.synchronize()
    return out


def _check(batch, ref):
    for i, (v, f) in enumerate(ref):
        assert np.array_equal(batch.valid[i].cpu().numpy(), v), i
        assert np.array_equal(batch.first_hit[i].cpu().numpy(), f), i


def test_batch_equals_per_instance_calls(cuda, pkg):
    items = _instances(pkg, cuda, 48, 0.1, seed=1)
    ref = _reference(pkg, cuda, items)
    b = pkg.Batch(items)
    groups = b.info()
    assert len(groups) >= 5 and all(1 <= a <= 5 and s in (1, 2) and seg == 0 for a, s, seg, _, _ in groups)
    b.run()
    cuda.cuda.synchronize()
    _check(b, ref)
    # rerun on cleared outputs after tuning, then through the captured graph
    for v, f in zip(b.valid, b.first_hit):
        v.fill_(7)
        f.fill_(-9)
    b.tune()
    b.run()
    cuda.cuda.synchronize()
    _check(b, ref)
    for v, f in zip(b.valid, b.first_hit):
        v.fill_(7)
        f.fill_(-9)
    b.capture()
    b.launch()
    b.launch()
    cuda.cuda.synchronize()
    _check(b, ref)
    for it in items:
        assert it[0].status() == 0


def test_batch_every_launch_shape_gives_the_same_results(cuda, pkg):
    """Every chunk size and warps-per-CTA choice the tuner searches, and a
    small grid, leave the verdicts unchanged (plain and segmented groups)."""
    items = _instances(pkg, cuda, 24, 0.06, seed=7)
    seg_items = []
    for k, (scene, rb, q0, q1, g, flags, arm) in enumerate(items[:10]):
        if len(q0) and arm < 0:
            seg_items.append((scene, rb, q0, q1, g, pkg.CHECK_ENV | pkg.CHECK_SELF, -1, None, None,
                              pkg.RULE_SHORTCUT, 0.8))
    ref = _reference(pkg, cuda, items)
    sref = []
    for scene, rb, q0, q1, g, flags, arm, _, _, rule, rg in seg_items:
        v, f = pkg.validate(scene, rb, q0, q1, g, flags, arm, rule, rg)[:2]
        sref.append((v.cpu().numpy(), f.cpu().numpy()))
    b = pkg.Batch(items)
    sb = pkg.Batch(seg_items)
    for batch, expect in ((b, ref), (sb, sref)):
        n_groups = len(batch.shapes())
        for chunk in (24, 48, 96, 192):
            for w in (2, 3, 4, 6):
                for gi in range(n_groups):
                    batch.set_shape(gi, chunk, (w, w, w), (0, 0, 0))
                for v, f in zip(batch.valid, batch.first_hit):
                    v.fill_(7)
                    f.fill_(-9)
                batch.run()
                cuda.cuda.synchronize()
                _check(batch, expect)
                sh = batch.shapes()
                assert all(s["chunk_edges"] == chunk and s["broad_warps"] == w and s["narrow_warps"] == w for s in sh)
        for gi in range(n_groups):  # a grid smaller than the SM count
            batch.set_shape(gi, 48, (3, 4, 6), (7, 5, 3))
        batch.run()
        cuda.cuda.synchronize()
        _check(batch, expect)
        batch.tune()
        for v, f in zip(batch.valid, batch.first_hit):
            v.fill_(7)
            f.fill_(-9)
        batch.capture()
        batch.launch()
        cuda.cuda.synchronize()
        _check(batch, expect)
        for s in batch.shapes():
            assert s["chunk_edges"] in (24, 48, 96, 192) and s["broad_warps"] in (2, 3, 4, 6)
            assert s["narrow_warps"] in (2, 3, 4, 6) and s["broad_grid"] >= 1


def test_batch_refilled_inputs(cuda, pkg):
    """A captured batch reads its input buffers at execution time."""
    items = _instances(pkg, cuda, 12, 0.05, seed=2)
    b = pkg.Batch(items)
    b.capture()
    W = pkg.workloads
    rng = np.random.default_rng(9)
    for scene, rb, q0, q1, g, flags, arm in items:
        if q0.shape[0] == 0:
            continue
        arms = q0.shape[1] // 7
        a0, a1 = W.random_edges(rng, q0.shape[0], arms, 1.5)
        q0.copy_(cuda.from_numpy(a0))
        q1.copy_(cuda.from_numpy(a1))
    b.launch()
    cuda.cuda.synchronize()
    _check(b, _reference(pkg, cuda, items))


def test_batch_rejects_bad_items(cuda, pkg):
    items = _instances(pkg, cuda, 4, 0.02, seed=3)
    scene, rb, q0, q1, g, flags, arm = items[1]
    bad = list(items)
    bad[1] = (scene, rb, q0, q1, 65, flags, arm)
    with pytest.raises(pkg.MrpopError, match="item 1"):
        pkg.Batch(bad)


def test_batch_chunk_boundaries(cuda, pkg):
    """One group (4 arms, g = 32) whose instances end just before, at and just
    after the 96-edge chunks, with the scene changing between neighbours, so
    that CTAs restage scenes between chunks of different instances."""
    W = pkg.workloads
    rng = np.random.default_rng(11)
    bases = W.bases_facing_centre(4, 0.71)
    rb = pkg.RobotSet(4, bases)
    scenes = [pkg.Scene(W.scene_config1(3)), pkg.Scene(W.scene_config2(4))]
    items = []
    for k, n in enumerate([1, 95, 96, 97, 191, 192, 193, 2, 288, 1]):
        a0, a1 = W.random_edges(rng, n, 4, 1.5)
        items.append((scenes[k % 2], rb, cuda.from_numpy(a0).cuda(), cuda.from_numpy(a1).cuda(), 32,
                      pkg.CHECK_ENV | pkg.CHECK_SELF, -1))
    ref = _reference(pkg, cuda, items)
    b = pkg.Batch(items)
    assert len(b.info()) == 1
    for _ in range(2):  # a second run starts from re-zeroed chunk counters
        for v, f in zip(b.valid, b.first_hit):
            v.fill_(7)
            f.fill_(-9)
        b.run()
        cuda.cuda.synchronize()
        _check(b, ref)
    for s in scenes:
        assert s.status() == 0


def test_batch_items_in_page_locked_host_memory(cuda, pkg):
    """Items whose endpoints and outputs are page-locked host buffers are read
    and written in place by the batch kernels: same verdicts as device items."""
    items = _instances(pkg, cuda, 16, 0.05, seed=5)
    ref = _reference(pkg, cuda, items)
    host = []
    for scene, rb, q0, q1, g, flags, arm in items:
        n = q0.shape[0]
        host.append((scene, rb, q0.cpu().pin_memory(), q1.cpu().pin_memory(), g, flags, arm,
                     cuda.full((n,), 7, dtype=cuda.uint8).pin_memory(),
                     cuda.full((n,), -9, dtype=cuda.int32).pin_memory()))
    b = pkg.Batch(host)
    b.capture()
    b.launch()
    cuda.cuda.synchronize()
    _check(b, ref)


def test_batch_segmented_items(cuda, pkg):
    """Connect, B-spline and shortcut items (with plain ones) in one batch:
    segment rounds and the fused tail per group give the per-item
    mrpop_validate_segments results bit for bit, through a plain run, after
    tuning and through the captured graph, on a rerun of cleared outputs."""
    W = pkg.workloads
    rng = np.random.default_rng(21)
    items = []
    for k in range(12):
        arms = 1 + k % 5
        g = (16, 32, 64)[k % 3]
        rule = (pkg.RULE_PLAIN, pkg.RULE_CONNECT, pkg.RULE_BSPLINE, pkg.RULE_SHORTCUT)[k % 4]
        # long edges, so that many take more segments than the split rounds
        n = int(rng.integers(40, 400))
        a0, a1 = W.random_edges(rng, n, arms, 3.0)
        sc = pkg.Scene(W.scene_config1(k) if k % 2 else W.scene_config2(k))
        rb = pkg.RobotSet(arms, W.bases_facing_centre(arms, 0.71))
        rng_ = 0.0 if rule == pkg.RULE_PLAIN else float((0.25, 0.5, 1.0)[k % 3])
        items.append((sc, rb, cuda.from_numpy(a0).cuda(), cuda.from_numpy(a1).cuda(), g,
                      pkg.CHECK_ENV | pkg.CHECK_SELF, -1, None, None, rule, rng_))
    ref = []
    for sc, rb, q0, q1, g, flags, arm, _, _, rule, rng_ in items:
        out = pkg.validate(sc, rb, q0, q1, g, flags, arm, rule, rng_)
        ref.append((out[0].cpu().numpy(), out[1].cpu().numpy()))
    cuda.cuda.synchronize()
    b = pkg.Batch(items)
    assert any(seg for _, _, seg, _, _ in b.info())
    b.run()
    cuda.cuda.synchronize()
    _check(b, ref)
    for step in ("tune", "capture"):
        for v, f in zip(b.valid, b.first_hit):
            v.fill_(7)
            f.fill_(-9)
        if step == "tune":
            b.tune()
            b.run()
        else:
            b.capture()
            b.launch()
        cuda.cuda.synchronize()
        _check(b, ref)
    for it in items:
        assert it[0].status() == 0
