"""mrpop_validate_edges_noalloc: the single-segment validator for callers that
must not allocate device memory while they run (a server that reserves its
device-memory budget up front, a loop that may not enter the allocator).  It
runs the same kernels as mrpop_validate_edges with its scratch in a fixed array
of the library, so its verdicts must equal that entry point's exactly -- on
consecutive calls too, since every call reuses the same array.  The file sorts
last so a stop-at-first-failure run has done everything else first."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(cuda, lib, fn, scene, robots, q0, q1, g, flags, arm):
    n = q0.shape[0]
    valid = cuda.full((n,), 7, dtype=cuda.uint8, device="cuda")
    first = cuda.full((n,), -7, dtype=cuda.int32, device="cuda")
    st = fn(scene.handle, robots.handle, q0.data_ptr(), q1.data_ptr(), n, g, flags, arm, valid.data_ptr(),
            first.data_ptr(), C.c_void_p(cuda.cuda.current_stream().cuda_stream))
    assert st == 0, lib.mrpop_last_error()
    cuda.cuda.synchronize()
    return valid.cpu().numpy(), first.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(cuda, pkg):
    lib = pkg.library()
    W = pkg.workloads
    cases = [W.config2(n_edges=4096, seed=11), W.config1(n_edges=2048, seed=12),
             W.config3(n_edges=1024, seed=13), W.config2(n_edges=pkg.mrpop.NOALLOC_MAX_EDGES, seed=14),
             # the layout that fills the array exactly: 5 arms at granularity 64
             W.config3(n_edges=pkg.mrpop.NOALLOC_MAX_EDGES, seed=15)]
    for wl in cases:
        scene = pkg.Scene(wl.scene)
        robots = pkg.RobotSet(len(wl.bases), wl.bases)
        q0 = cuda.from_numpy(wl.q0).cuda()
        q1 = cuda.from_numpy(wl.q1).cuda()
        ref = _call(cuda, lib, lib.mrpop_validate_edges, scene, robots, q0, q1, wl.granularity, wl.flags, wl.arm)
        for _ in range(2):  # the shared array keeps the previous call's contents
            got = _call(cuda, lib, lib.mrpop_validate_edges_noalloc, scene, robots, q0, q1, wl.granularity,
                        wl.flags, wl.arm)
            assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
        assert scene.status() == 0


def test_noalloc_rejects_batches_above_its_limit(cuda, pkg):
    lib = pkg.library()
    W = pkg.workloads
    n = pkg.mrpop.NOALLOC_MAX_EDGES + 1
    rng = np.random.default_rng(1)
    q0, q1 = W.random_edges(rng, n, 4, 1.0)
    scene = pkg.Scene(W.scene_config2(0))
    robots = pkg.RobotSet(4, W.bases_config2())
    d0, d1 = cuda.from_numpy(q0).cuda(), cuda.from_numpy(q1).cuda()
    valid = cuda.empty(n, dtype=cuda.uint8, device="cuda")
    first = cuda.empty(n, dtype=cuda.int32, device="cuda")
    st = lib.mrpop_validate_edges_noalloc(scene.handle, robots.handle, d0.data_ptr(), d1.data_ptr(), n, 32, 3, -1,
                                          valid.data_ptr(), first.data_ptr(), None)
    assert st == 1 and b"MRPOP_NOALLOC_MAX_EDGES" in lib.mrpop_last_error()


def test_noalloc_takes_no_device_memory_after_warm_up(cuda, pkg):
    """After the warm-up call (first use of the array and of the kernel variant
    on this device), repeated calls leave the device's free memory unchanged."""
    lib = pkg.library()
    W = pkg.workloads
    wl = W.config3(n_edges=4096, seed=16)
    scene = pkg.Scene(wl.scene)
    robots = pkg.RobotSet(len(wl.bases), wl.bases)
    q0 = cuda.from_numpy(wl.q0).cuda()
    q1 = cuda.from_numpy(wl.q1).cuda()
    n = q0.shape[0]
    valid = cuda.empty(n, dtype=cuda.uint8, device="cuda")
    first = cuda.empty(n, dtype=cuda.int32, device="cuda")
    st = C.c_void_p(cuda.cuda.current_stream().cuda_stream)

    def call():
        rc = lib.mrpop_validate_edges_noalloc(scene.handle, robots.handle, q0.data_ptr(), q1.data_ptr(), n,
                                              wl.granularity, wl.flags, wl.arm, valid.data_ptr(), first.data_ptr(),
                                              st)
        assert rc == 0, lib.mrpop_last_error()

    call()
    cuda.cuda.synchronize()
    free0, _ = cuda.cuda.mem_get_info()
    for _ in range(5):
        call()
    cuda.cuda.synchronize()
    free1, _ = cuda.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
