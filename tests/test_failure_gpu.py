"""Failure detection on the device, without a fault: every wait of the kernels
on a bulk copy into shared memory is bounded in time.  mrpop_debug_wait_timeout
runs that wait out on purpose (an mbarrier whose bytes no copy delivers, with a
20 ms limit in place of the kernels' 1 s): the wait gives up, sets the status
bit the scene status reports, and returns; the context stays usable."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT_NS = 20_000_000


def test_bounded_copy_wait_gives_up_reports_and_returns(cuda, pkg, orc):
    lib = pkg.library()
    status, elapsed = C.c_uint32(0), C.c_int64(0)
    assert lib.mrpop_debug_wait_timeout(LIMIT_NS, C.byref(status), C.byref(elapsed)) == 0
    assert status.value == 1
    # the first wait runs out, the second (for a copy that may still be writing) too
    assert 2 * LIMIT_NS <= elapsed.value < 2 * LIMIT_NS + 500_000_000
    # the context is still usable: a validation afterwards equals the oracle
    # (the device's trig values replayed) and leaves the scene's status clear
    wl = pkg.workloads.config1(n_edges=256, seed=5)
    scene = pkg.Scene(wl.scene)
    rb = pkg.RobotSet(len(wl.bases), wl.bases)
    d0, d1 = cuda.from_numpy(wl.q0).cuda(), cuda.from_numpy(wl.q1).cuda()
    v, f = pkg.validate(scene, rb, d0, d1, wl.granularity, wl.flags, wl.arm)
    cuda.cuda.synchronize()
    samples = orc.edge_samples(wl.q0, wl.q1, wl.granularity, 0, 0.0)
    x = cuda.from_numpy(np.ascontiguousarray(samples, np.float32).ravel()).cuda()
    c, s = pkg.debug_trig(x)
    cuda.cuda.synchronize()
    trig = orc.TrigTable(x.cpu().numpy(), c.cpu().numpy(), s.cpu().numpy())
    ref = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, wl.flags, wl.arm, 0, 0.0, trig=trig)
    assert scene.status() == 0
    assert np.array_equal(v.cpu().numpy(), ref["valid"]) and np.array_equal(f.cpu().numpy(), ref["first_hit"])


def test_bad_limits_are_refused(pkg):
    lib = pkg.library()
    status, elapsed = C.c_uint32(0), C.c_int64(0)
    assert lib.mrpop_debug_wait_timeout(0, C.byref(status), C.byref(elapsed)) != 0
    assert lib.mrpop_debug_wait_timeout(3_000_000_000, C.byref(status), C.byref(elapsed)) != 0
