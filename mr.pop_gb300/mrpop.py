"""Python host binding of the C ABI (include/mrpop.h) over ctypes.

Device buffers are torch CUDA tensors (PyTorch is used for device memory and
streams only); host-buffer calls take numpy arrays.  Every call goes through
the compiled library: there is no Python or CPU fallback, and a missing
library raises at load time.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import build as _build

CHECK_ENV = 0x1
CHECK_SELF = 0x2
MODE_EXACT = 0x10
RULE_PLAIN, RULE_CONNECT, RULE_BSPLINE, RULE_SHORTCUT = 0, 1, 2, 3
MAX_ARMS = 5
MAX_GRANULARITY = 64

STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "CUDA", 3: "UNSUPPORTED", 4: "OUT_OF_MEMORY", 5: "DEVICE_TIMEOUT"}

EXPORTED = [
    "mrpop_scene_create", "mrpop_scene_destroy", "mrpop_scene_status", "mrpop_robotset_create",
    "mrpop_robotset_destroy", "mrpop_validate_edges", "mrpop_validate_segments", "mrpop_workspace_create",
    "mrpop_workspace_destroy", "mrpop_validate_edges_host", "mrpop_fk_spheres", "mrpop_count_flops",
    "mrpop_debug_trig", "mrpop_fp32_peak_probe", "mrpop_last_error", "mrpop_version",
    "mrpop_validate_edges_noalloc", "mrpop_broad_flops_per_sample", "mrpop_kernel_timing", "mrpop_kernel_times",
    "mrpop_debug_row5_table", "mrpop_batch_create", "mrpop_batch_run", "mrpop_batch_tune", "mrpop_batch_capture",
    "mrpop_batch_launch", "mrpop_batch_info", "mrpop_batch_destroy", "mrpop_server_create", "mrpop_server_destroy",
    "mrpop_server_get_stats", "mrpop_session_open", "mrpop_session_submit", "mrpop_session_wait",
    "mrpop_session_close", "mrpop_session_host_buffers", "mrpop_plan", "mrpop_session_plan",
    "mrpop_drrt_settings_default", "mrpop_drrt_solve", "mrpop_drrt_solve_with", "mrpop_session_drrt",
    "mrpop_batch_shapes", "mrpop_batch_set_shape", "mrpop_drrt_release_pool", "mrpop_session_submit_many",
    "mrpop_set_fused_edges", "mrpop_debug_wait_timeout",
]
KERNEL_KINDS = ("fused", "broad", "narrow")
NOALLOC_MAX_EDGES = 16384


class MrpopError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mrpop {STATUS.get(status, status)}: {msg}")
        self.status = status


class SceneDesc(C.Structure):
    _fields_ = [
        ("spheres", C.c_void_p), ("num_spheres", C.c_uint32),
        ("capsules", C.c_void_p), ("num_capsules", C.c_uint32),
        ("z_capsules", C.c_void_p), ("num_z_capsules", C.c_uint32),
        ("cylinders", C.c_void_p), ("num_cylinders", C.c_uint32),
        ("cuboids", C.c_void_p), ("num_cuboids", C.c_uint32),
        ("z_cuboids", C.c_void_p), ("num_z_cuboids", C.c_uint32),
    ]


class BatchItem(C.Structure):
    _fields_ = [
        ("scene", C.c_void_p), ("robots", C.c_void_p), ("q0", C.c_void_p), ("q1", C.c_void_p),
        ("n_edges", C.c_int64), ("granularity", C.c_int32), ("flags", C.c_uint32), ("arm", C.c_int32),
        ("valid", C.c_void_p), ("first_hit", C.c_void_p), ("rule", C.c_int32), ("range", C.c_float),
    ]


class ServerConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_int64), ("streams", C.c_int32), ("max_wave_steps", C.c_int32),
                ("max_wave_chunks", C.c_int64), ("host_bytes", C.c_int64), ("fused_edges", C.c_int64)]


class PlanSettingsC(C.Structure):
    _fields_ = [("batch", C.c_int32), ("max_iters", C.c_int32), ("granularity", C.c_int32),
                ("shortcut_passes", C.c_int32), ("shortcut_pairs", C.c_int32), ("step", C.c_float),
                ("range", C.c_float), ("seed", C.c_uint64)]


class PlanResultC(C.Structure):
    _fields_ = [("solved", C.c_int32), ("iterations", C.c_int32), ("steps", C.c_int32), ("edges", C.c_int64),
                ("waypoints", C.c_int64), ("cost", C.c_double), ("digest", C.c_uint64), ("start_tree", C.c_int64),
                ("goal_tree", C.c_int64), ("validate_ns", C.c_int64)]


VALIDATE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_float,
                          C.c_void_p, C.c_void_p)


class DrrtSettingsC(C.Structure):
    """mrpop_drrt_settings: the reference's pop_settings fields in order, then this library's additions."""
    _fields_ = [("max_samples", C.c_int32), ("max_iters", C.c_int32), ("optimize_iters", C.c_int32),
                ("num_new_configs", C.c_int32), ("granularity", C.c_int32), ("range", C.c_float),
                ("balance", C.c_int32), ("tree_ratio", C.c_float), ("dynamic_domain", C.c_int32),
                ("dd_alpha", C.c_float), ("dd_radius", C.c_float), ("dd_min_radius", C.c_float),
                ("roadmap_reassign", C.c_int32), ("rrtc_iter", C.c_int32), ("resample_iter", C.c_int32),
                ("cost_bound_resample", C.c_int32), ("path_simplify", C.c_int32), ("phs", C.c_int32),
                ("simplify_round", C.c_int32), ("bspline_step", C.c_int32), ("bspline_min_change", C.c_float),
                ("perturb_step", C.c_int32), ("perturb_empty_step", C.c_int32), ("block_per_robot", C.c_int32),
                ("max_launches", C.c_int32), ("seed", C.c_uint64), ("host_threads", C.c_int32),
                ("blocking_wait", C.c_int32)]


class DrrtResultC(C.Structure):
    _fields_ = [("solved", C.c_int32), ("iters", C.c_int32), ("cost", C.c_float), ("passes", C.c_int32),
                ("solutions", C.c_int32), ("launches", C.c_int32), ("start_tree_size", C.c_int64),
                ("goal_tree_size", C.c_int64), ("path_length", C.c_int64), ("roadmap_nodes", C.c_int64 * 5),
                ("roadmap_edges", C.c_int64 * 5), ("validate_calls", C.c_int64), ("edges_validated", C.c_int64),
                ("iterations", C.c_int64), ("wall_ns", C.c_int64), ("kernel_ns", C.c_int64),
                ("validate_ns", C.c_int64), ("nn_ns", C.c_int64), ("oracle_ns", C.c_int64),
                ("roadmap_ns", C.c_int64), ("check_ns", C.c_int64 * 5), ("check_calls", C.c_int64 * 5)]


CHECK_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_float,
                       C.c_uint32, C.c_int, C.c_void_p, C.c_void_p)
SOLUTION_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int32, C.c_float, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64)


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "budget_bytes", "bytes_in_use", "peak_bytes_in_use", "sessions", "admission_waits", "admission_timeouts",
        "waves", "steps", "max_wave_steps", "max_waves_in_flight", "kernel_launches", "queue_ns", "flight_ns",
        "device_ns")]


_LIBS: dict[str, C.CDLL] = {}


def library(variant: str = "", path: str | Path | None = None) -> C.CDLL:
    """Load (not build) the compiled library; raises if it is missing."""
    p = Path(path) if path else _build.lib_path(variant)
    key = str(p)
    if key in _LIBS:
        return _LIBS[key]
    if not p.exists():
        raise FileNotFoundError(f"mrpop CUDA library not built: {p} (run __graft_entry__.build())")
    lib = C.CDLL(str(p))
    vp, i64, i32, u32, f32 = C.c_void_p, C.c_int64, C.c_int, C.c_uint32, C.c_float
    sig = {
        "mrpop_scene_create": [C.POINTER(SceneDesc), C.POINTER(vp)],
        "mrpop_scene_destroy": [vp],
        "mrpop_scene_status": [vp, C.POINTER(C.c_uint32)],
        "mrpop_robotset_create": [i32, vp, C.POINTER(vp)],
        "mrpop_robotset_destroy": [vp],
        "mrpop_validate_edges": [vp, vp, vp, vp, i64, i32, u32, i32, vp, vp, vp],
        "mrpop_validate_segments": [vp, vp, vp, vp, i64, i32, i32, f32, u32, i32, vp, vp, vp, vp],
        "mrpop_workspace_create": [C.POINTER(vp)],
        "mrpop_workspace_destroy": [vp],
        "mrpop_validate_edges_host": [vp, vp, vp, vp, vp, i64, i32, u32, i32, i32, f32, vp, vp],
        "mrpop_fk_spheres": [vp, i32, vp, i64, i32, vp, vp],
        "mrpop_count_flops": [vp, vp, vp, vp, i64, i32, i32, f32, u32, i32, vp, vp],
        "mrpop_debug_trig": [vp, i64, vp, vp, vp],
        "mrpop_fp32_peak_probe": [i32, i32, vp, C.POINTER(C.c_double), vp],
        "mrpop_validate_edges_noalloc": [vp, vp, vp, vp, i64, i32, u32, i32, vp, vp, vp],
        "mrpop_broad_flops_per_sample": [vp, vp, u32, i32, C.POINTER(C.c_double)],
        "mrpop_kernel_timing": [i32],
        "mrpop_kernel_times": [C.POINTER(C.c_int64), C.POINTER(C.c_double)],
        "mrpop_debug_row5_table": [vp, i64, C.POINTER(C.c_int), C.POINTER(C.c_int)],
        "mrpop_batch_create": [C.POINTER(BatchItem), i64, C.POINTER(vp)],
        "mrpop_batch_run": [vp, vp],
        "mrpop_batch_tune": [vp, vp],
        "mrpop_batch_capture": [vp],
        "mrpop_batch_launch": [vp, vp],
        "mrpop_batch_info": [vp, C.POINTER(C.c_int64), vp, i64],
        "mrpop_batch_destroy": [vp],
        "mrpop_batch_shapes": [vp, C.POINTER(C.c_int64), vp, i64],
        "mrpop_batch_set_shape": [vp, i64, i32, vp, vp],
        "mrpop_server_create": [C.POINTER(ServerConfig), C.POINTER(vp)],
        "mrpop_server_destroy": [vp],
        "mrpop_server_get_stats": [vp, C.POINTER(ServerStats)],
        "mrpop_session_open": [vp, i32, i64, i32, i64, C.POINTER(vp)],
        "mrpop_session_submit": [vp, C.POINTER(BatchItem)],
        "mrpop_session_submit_many": [vp, C.POINTER(BatchItem), i32],
        "mrpop_debug_wait_timeout": [i64, C.POINTER(C.c_uint32), C.POINTER(C.c_int64)],
        "mrpop_session_wait": [vp, i64],
        "mrpop_session_close": [vp],
        "mrpop_session_host_buffers": [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)],
        "mrpop_plan": [i32, vp, vp, C.POINTER(PlanSettingsC), VALIDATE_FN, vp, vp, i64, C.POINTER(PlanResultC)],
        "mrpop_session_plan": [vp, vp, vp, u32, vp, vp, C.POINTER(PlanSettingsC), vp, i64, C.POINTER(PlanResultC)],
        "mrpop_drrt_settings_default": [C.POINTER(DrrtSettingsC)],
        "mrpop_drrt_solve": [vp, vp, vp, vp, i32, C.POINTER(DrrtSettingsC), vp, i64, SOLUTION_FN, vp,
                             C.POINTER(DrrtResultC)],
        "mrpop_drrt_solve_with": [i32, CHECK_FN, vp, vp, vp, i32, C.POINTER(DrrtSettingsC), vp, i64, SOLUTION_FN, vp,
                                  C.POINTER(DrrtResultC)],
        "mrpop_session_drrt": [vp, vp, vp, vp, vp, i32, C.POINTER(DrrtSettingsC), vp, i64, SOLUTION_FN, vp,
                               C.POINTER(DrrtResultC)],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.mrpop_set_fused_edges.argtypes = [C.c_int64]
    lib.mrpop_set_fused_edges.restype = C.c_int64
    lib.mrpop_drrt_release_pool.argtypes = []
    lib.mrpop_drrt_release_pool.restype = C.c_int64
    lib.mrpop_last_error.restype = C.c_char_p
    lib.mrpop_last_error.argtypes = []
    lib.mrpop_version.restype = C.c_char_p
    lib.mrpop_version.argtypes = []
    _LIBS[key] = lib
    return lib


def _check(lib: C.CDLL, status: int) -> None:
    if status != 0:
        raise MrpopError(status, lib.mrpop_last_error().decode())


def _f32(a, cols: int) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, cols))
    return a


@dataclass
class SceneArrays:
    """Obstacles as packed float32 records (field order of include/mrpop.h)."""
    spheres: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.float32))
    capsules: np.ndarray = field(default_factory=lambda: np.zeros((0, 8), np.float32))
    z_capsules: np.ndarray = field(default_factory=lambda: np.zeros((0, 8), np.float32))
    cylinders: np.ndarray = field(default_factory=lambda: np.zeros((0, 8), np.float32))
    cuboids: np.ndarray = field(default_factory=lambda: np.zeros((0, 15), np.float32))
    z_cuboids: np.ndarray = field(default_factory=lambda: np.zeros((0, 15), np.float32))

    def __post_init__(self):
        self.spheres = _f32(self.spheres, 4)
        self.capsules = _f32(self.capsules, 8)
        self.z_capsules = _f32(self.z_capsules, 8)
        self.cylinders = _f32(self.cylinders, 8)
        self.cuboids = _f32(self.cuboids, 15)
        self.z_cuboids = _f32(self.z_cuboids, 15)

    def counts(self) -> dict:
        return {k: len(getattr(self, k)) for k in
                ("spheres", "capsules", "z_capsules", "cylinders", "cuboids", "z_cuboids")}


def _ptr(a: np.ndarray):
    return a.ctypes.data if a.size else None


class Scene:
    """Device-resident scene (mrpop_scene)."""

    def __init__(self, arrays: SceneArrays, lib: C.CDLL | None = None):
        self.lib = lib or library()
        self.arrays = arrays
        d = SceneDesc(_ptr(arrays.spheres), len(arrays.spheres), _ptr(arrays.capsules), len(arrays.capsules),
                      _ptr(arrays.z_capsules), len(arrays.z_capsules), _ptr(arrays.cylinders),
                      len(arrays.cylinders), _ptr(arrays.cuboids), len(arrays.cuboids),
                      _ptr(arrays.z_cuboids), len(arrays.z_cuboids))
        h = C.c_void_p()
        _check(self.lib, self.lib.mrpop_scene_create(C.byref(d), C.byref(h)))
        self.handle = h

    def status(self) -> int:
        v = C.c_uint32()
        _check(self.lib, self.lib.mrpop_scene_status(self.handle, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mrpop_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RobotSet:
    """Arm bases (mrpop_robotset); base: (n, 4, 4) row-major or None (built-in)."""

    def __init__(self, n_arms: int, base: np.ndarray | None = None, lib: C.CDLL | None = None):
        self.lib = lib or library()
        self.n_arms = n_arms
        self.base = None if base is None else np.ascontiguousarray(np.asarray(base, np.float32).reshape(n_arms, 16))
        h = C.c_void_p()
        _check(self.lib, self.lib.mrpop_robotset_create(n_arms, None if self.base is None else self.base.ctypes.data,
                                                         C.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mrpop_robotset_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream_ptr(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


def validate(scene: Scene, robots: RobotSet, q0, q1, granularity: int, flags: int = CHECK_ENV | CHECK_SELF,
             arm: int = -1, rule: int = RULE_PLAIN, range_: float = 0.0, valid=None, first_hit=None,
             n_seg=None, stream=None):
    """Validate edges held in CUDA tensors q0/q1 [n, dof]; returns (valid u8, first_hit i32[, n_seg])."""
    import torch
    lib = scene.lib
    n = q0.shape[0]
    dev = q0.device
    assert q0.is_cuda and q1.is_cuda and q0.dtype == torch.float32 and q0.is_contiguous() and q1.is_contiguous()
    if valid is None:
        valid = torch.empty(n, dtype=torch.uint8, device=dev)
    if first_hit is None:
        first_hit = torch.empty(n, dtype=torch.int32, device=dev)
    st = _stream_ptr(stream)
    if rule == RULE_PLAIN and n_seg is None:
        _check(lib, lib.mrpop_validate_edges(scene.handle, robots.handle, q0.data_ptr(), q1.data_ptr(), n,
                                             granularity, flags, arm, valid.data_ptr(), first_hit.data_ptr(), st))
        return valid, first_hit
    if n_seg is None:
        n_seg = torch.empty(n, dtype=torch.int32, device=dev)
    _check(lib, lib.mrpop_validate_segments(scene.handle, robots.handle, q0.data_ptr(), q1.data_ptr(), n,
                                            granularity, rule, float(range_), flags, arm, valid.data_ptr(),
                                            first_hit.data_ptr(), n_seg.data_ptr(), st))
    return valid, first_hit, n_seg


def count_flops(scene: Scene, robots: RobotSet, q0, q1, granularity: int, flags: int = CHECK_ENV | CHECK_SELF,
                arm: int = -1, rule: int = RULE_PLAIN, range_: float = 0.0, stream=None):
    import torch
    out = torch.empty(q0.shape[0], dtype=torch.float64, device=q0.device)
    _check(scene.lib, scene.lib.mrpop_count_flops(scene.handle, robots.handle, q0.data_ptr(), q1.data_ptr(),
                                                  q0.shape[0], granularity, rule, float(range_), flags, arm,
                                                  out.data_ptr(), _stream_ptr(stream)))
    return out


def fk_spheres(robots: RobotSet, arm: int, q, detailed: bool, stream=None):
    import torch
    n = q.shape[0]
    ns = 59 if detailed else 11
    out = torch.empty((n, ns, 3), dtype=torch.float32, device=q.device)
    _check(robots.lib, robots.lib.mrpop_fk_spheres(robots.handle, arm, q.data_ptr(), n, int(detailed),
                                                   out.data_ptr(), _stream_ptr(stream)))
    return out


def debug_trig(x, lib: C.CDLL | None = None, stream=None):
    import torch
    lib = lib or library()
    c = torch.empty_like(x)
    s = torch.empty_like(x)
    _check(lib, lib.mrpop_debug_trig(x.data_ptr(), x.numel(), c.data_ptr(), s.data_ptr(), _stream_ptr(stream)))
    return c, s


def fp32_peak_probe(blocks: int, iters: int, scratch, stream=None, lib: C.CDLL | None = None) -> float:
    """Launch the FMA loop; returns its flop count (time it with CUDA events)."""
    lib = lib or library()
    f = C.c_double()
    _check(lib, lib.mrpop_fp32_peak_probe(blocks, iters, scratch.data_ptr(), C.byref(f), _stream_ptr(stream)))
    return f.value


def broad_flops_per_sample(scene: Scene, robots: RobotSet, flags: int = CHECK_ENV | CHECK_SELF,
                           arm: int = -1) -> float:
    """Algorithmic (unculled) broad-phase flops of one sample, FMA = 2."""
    f = C.c_double()
    _check(scene.lib, scene.lib.mrpop_broad_flops_per_sample(scene.handle, robots.handle, flags, arm, C.byref(f)))
    return f.value


def row5_table(lib: C.CDLL | None = None) -> np.ndarray:
    """The forearm-hand rows table as a bool array [n6, n7] (True: rows apart)."""
    lib = lib or library()
    words = np.zeros(1 << 14, np.uint32)
    n6, n7 = C.c_int(), C.c_int()
    _check(lib, lib.mrpop_debug_row5_table(words.ctypes.data, len(words), C.byref(n6), C.byref(n7)))
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[: n6.value * n7.value]
    return bits.reshape(n6.value, n7.value).astype(bool)


def kernel_timing(enable: bool, lib: C.CDLL | None = None) -> None:
    """Turn the library's per-kernel CUDA-event timing on or off."""
    lib = lib or library()
    _check(lib, lib.mrpop_kernel_timing(1 if enable else 0))


def kernel_times(lib: C.CDLL | None = None) -> dict:
    """{kind: (launches, total ms)} recorded since the previous read."""
    lib = lib or library()
    n = (C.c_int64 * 3)()
    ms = (C.c_double * 3)()
    _check(lib, lib.mrpop_kernel_times(n, ms))
    return {k: (int(n[i]), float(ms[i])) for i, k in enumerate(KERNEL_KINDS)}


class Batch:
    """Many independent validate calls in one launch per kernel variant
    (mrpop_batch_*).  items: (scene, robots, q0, q1, granularity, flags, arm)
    with q0/q1 CUDA (or page-locked host) tensors; outputs are allocated here
    (self.valid[i], self.first_hit[i]) unless given as items[i][7:9] (either
    may be None); items[i][9:11] = (rule, range) for a segmented item."""

    def __init__(self, items, lib: C.CDLL | None = None):
        import torch
        self.lib = lib or library()
        self.items = list(items)
        self.valid, self.first_hit = [], []
        arr = (BatchItem * max(1, len(self.items)))()
        for i, it in enumerate(self.items):
            scene, robots, q0, q1, g, flags, arm = it[:7]
            n = q0.shape[0]
            v = it[7] if len(it) > 7 and it[7] is not None else torch.empty(n, dtype=torch.uint8, device=q0.device)
            f = it[8] if len(it) > 8 and it[8] is not None else torch.empty(n, dtype=torch.int32, device=q0.device)
            rule, range_ = (int(it[9]), float(it[10])) if len(it) > 10 else (RULE_PLAIN, 0.0)
            self.valid.append(v)
            self.first_hit.append(f)
            arr[i] = BatchItem(scene.handle, robots.handle, q0.data_ptr() if n else None,
                               q1.data_ptr() if n else None, n, g, flags, arm, v.data_ptr() if n else None,
                               f.data_ptr() if n else None, rule, range_)
        h = C.c_void_p()
        _check(self.lib, self.lib.mrpop_batch_create(arr, len(self.items), C.byref(h)))
        self.handle = h

    def run(self, stream=None):
        _check(self.lib, self.lib.mrpop_batch_run(self.handle, _stream_ptr(stream)))

    def tune(self, stream=None):
        _check(self.lib, self.lib.mrpop_batch_tune(self.handle, _stream_ptr(stream)))

    def capture(self):
        _check(self.lib, self.lib.mrpop_batch_capture(self.handle))

    def launch(self, stream=None):
        _check(self.lib, self.lib.mrpop_batch_launch(self.handle, _stream_ptr(stream)))

    def info(self) -> list[tuple[int, int, int, int, int]]:
        """Per group: (arms, samples per lane, segmented, broad grid, narrow grid)."""
        n = C.c_int64()
        grids = np.zeros(5 * 32, np.int32)
        _check(self.lib, self.lib.mrpop_batch_info(self.handle, C.byref(n), grids.ctypes.data, 32))
        return [tuple(int(x) for x in grids[5 * i:5 * i + 5]) for i in range(min(n.value, 32))]

    SHAPE_KEYS = ("arms", "samples_per_lane", "segmented", "chunk_edges", "chunks", "broad_warps", "broad_grid",
                  "narrow_warps", "narrow_grid", "fused_warps", "fused_grid")

    def shapes(self) -> list[dict]:
        """Per group: the launch shape (mrpop_batch_shapes)."""
        n = C.c_int64()
        out = np.zeros(12 * 32, np.int32)
        _check(self.lib, self.lib.mrpop_batch_shapes(self.handle, C.byref(n), out.ctypes.data, 32))
        return [dict(zip(self.SHAPE_KEYS, (int(x) for x in out[12 * i:12 * i + 11]))) for i in range(min(n.value, 32))]

    def set_shape(self, group: int, chunk_edges: int = 0, warps=(0, 0, 0), grids=(0, 0, 0)):
        w = np.asarray(warps, np.int32)
        g = np.asarray(grids, np.int32)
        _check(self.lib, self.lib.mrpop_batch_set_shape(self.handle, group, chunk_edges, w.ctypes.data,
                                                        g.ctypes.data))

    def __del__(self):
        if getattr(self, "handle", None):
            self.lib.mrpop_batch_destroy(self.handle)
            self.handle = None


class Workspace:
    """Host-buffer path (mrpop_validate_edges_host)."""

    def __init__(self, lib: C.CDLL | None = None):
        self.lib = lib or library()
        h = C.c_void_p()
        _check(self.lib, self.lib.mrpop_workspace_create(C.byref(h)))
        self.handle = h

    def validate(self, scene: Scene, robots: RobotSet, q0: np.ndarray, q1: np.ndarray, granularity: int,
                 flags: int = CHECK_ENV | CHECK_SELF, arm: int = -1, rule: int = RULE_PLAIN, range_: float = 0.0,
                 valid: np.ndarray | None = None, first_hit: np.ndarray | None = None):
        n = q0.shape[0]
        assert q0.dtype == np.float32 and q0.flags.c_contiguous and q1.flags.c_contiguous
        if valid is None:
            valid = np.empty(n, np.uint8)
        if first_hit is None:
            first_hit = np.empty(n, np.int32)
        _check(self.lib, self.lib.mrpop_validate_edges_host(self.handle, scene.handle, robots.handle, q0.ctypes.data,
                                                            q1.ctypes.data, n, granularity, flags, arm, rule,
                                                            float(range_), valid.ctypes.data,
                                                            first_hit.ctypes.data))
        return valid, first_hit

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mrpop_workspace_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching validation service (mrpop_server_*): sessions are
    admitted against a fixed device-memory budget and their steps co-batched."""

    def __init__(self, budget_bytes: int = 1 << 30, streams: int = 4, max_wave_steps: int = 1024,
                 max_wave_chunks: int = 16384, host_bytes: int = 256 << 20, fused_edges: int = 0,
                 lib: C.CDLL | None = None):
        self.lib = lib or library()
        cfg = ServerConfig(budget_bytes, streams, max_wave_steps, max_wave_chunks, host_bytes, fused_edges)
        h = C.c_void_p()
        _check(self.lib, self.lib.mrpop_server_create(C.byref(cfg), C.byref(h)))
        self.handle = h

    def stats(self) -> dict:
        st = ServerStats()
        _check(self.lib, self.lib.mrpop_server_get_stats(self.handle, C.byref(st)))
        return {n: int(getattr(st, n)) for n, _ in ServerStats._fields_}

    def session(self, arms: int, max_edges: int, max_granularity: int, timeout_ms: int = -1) -> "Session":
        return Session(self, arms, max_edges, max_granularity, timeout_ms)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mrpop_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Session:
    """One admitted query: the session's page-locked endpoint and verdict
    buffers of max_edges edges (from the server's host arena, read and written
    in place by the kernels), one step at a time."""

    def __init__(self, server: Server, arms: int, max_edges: int, max_granularity: int, timeout_ms: int = -1):
        self.server, self.lib = server, server.lib
        self.arms, self.max_edges = arms, max_edges
        h = C.c_void_p()
        _check(self.lib, self.lib.mrpop_session_open(server.handle, arms, max_edges, max_granularity, timeout_ms,
                                                     C.byref(h)))
        self.handle = h
        p = [C.c_void_p() for _ in range(4)]
        _check(self.lib, self.lib.mrpop_session_host_buffers(h, *[C.byref(x) for x in p]))
        dof = 7 * arms
        self._ptrs = [x.value for x in p]
        self.q0 = np.ctypeslib.as_array(C.cast(p[0], C.POINTER(C.c_float)), shape=(max_edges, dof))
        self.q1 = np.ctypeslib.as_array(C.cast(p[1], C.POINTER(C.c_float)), shape=(max_edges, dof))
        self.valid = np.ctypeslib.as_array(C.cast(p[2], C.POINTER(C.c_uint8)), shape=(max_edges,))
        self.first_hit = np.ctypeslib.as_array(C.cast(p[3], C.POINTER(C.c_int32)), shape=(max_edges,))

    def submit(self, scene: Scene, robots: RobotSet, q0: np.ndarray, q1: np.ndarray, granularity: int,
               flags: int = CHECK_ENV | CHECK_SELF, arm: int = -1, rule: int = RULE_PLAIN, range_: float = 0.0):
        n = q0.shape[0]
        self._n = n
        if n:
            # the step's rows [n][dof] packed at the start of the buffers (a
            # single-arm step on a composite session has 7-float rows)
            dof = q0.shape[1]
            if n > self.max_edges or dof > self.q0.shape[1]:
                raise MrpopError(1, f"session step of {n} edges x {dof} exceeds the session's "
                                    f"{self.max_edges} x {self.q0.shape[1]}")
            self.q0.reshape(-1)[:n * dof] = np.asarray(q0, np.float32).reshape(-1)
            self.q1.reshape(-1)[:n * dof] = np.asarray(q1, np.float32).reshape(-1)
        q0p, q1p, vp_, fp = self._ptrs if n else (None, None, None, None)
        item = BatchItem(scene.handle, robots.handle, q0p, q1p, n, granularity, flags, arm, vp_, fp, rule,
                         float(range_))
        _check(self.lib, self.lib.mrpop_session_submit(self.handle, C.byref(item)))

    def wait(self, timeout_ms: int = -1):
        _check(self.lib, self.lib.mrpop_session_wait(self.handle, timeout_ms))
        n = self._n
        return self.valid[:n].copy(), self.first_hit[:n].copy()

    def validate(self, scene, robots, q0, q1, granularity, flags=CHECK_ENV | CHECK_SELF, arm=-1, rule=RULE_PLAIN,
                 range_=0.0):
        self.submit(scene, robots, q0, q1, granularity, flags, arm, rule, range_)
        return self.wait()

    def validate_many(self, scene: Scene, robots: RobotSet, checks: list[tuple]):
        """Several steps submitted together (mrpop_session_submit_many), packed
        one after another in the session's buffers; checks: (q0, q1,
        granularity, flags, arm, rule, range_) tuples.  Returns a (valid,
        first_hit) pair per check."""
        items, spans = (BatchItem * max(1, len(checks)))(), []
        q_at = e_at = 0
        fq0, fq1 = self.q0.reshape(-1), self.q1.reshape(-1)
        for k, (q0, q1, g, flags, arm, rule, rg) in enumerate(checks):
            n, dof = q0.shape
            if e_at + n > self.max_edges or q_at + n * dof > fq0.size:
                raise MrpopError(1, "session steps exceed the session's buffers")
            fq0[q_at:q_at + n * dof] = np.asarray(q0, np.float32).reshape(-1)
            fq1[q_at:q_at + n * dof] = np.asarray(q1, np.float32).reshape(-1)
            items[k] = BatchItem(scene.handle, robots.handle, self._ptrs[0] + 4 * q_at, self._ptrs[1] + 4 * q_at, n, g,
                                 flags, arm, self._ptrs[2] + e_at, self._ptrs[3] + 4 * e_at, rule, float(rg))
            spans.append((e_at, n))
            q_at += n * dof
            e_at += n
        _check(self.lib, self.lib.mrpop_session_submit_many(self.handle, items, len(checks)))
        _check(self.lib, self.lib.mrpop_session_wait(self.handle, -1))
        return [(self.valid[a:a + n].copy(), self.first_hit[a:a + n].copy()) for a, n in spans]

    def plan(self, scene: Scene, robots: RobotSet, start: np.ndarray, goal: np.ndarray, settings: PlanSettingsC,
             flags: int = CHECK_ENV | CHECK_SELF, max_waypoints: int = 4096):
        """The library's planner with every step validated by this session
        (mrpop_session_plan; one call, the GIL released throughout).
        Returns (PlanResultC, path [waypoints, dof])."""
        dof = 7 * self.arms
        start = np.ascontiguousarray(start, np.float32)
        goal = np.ascontiguousarray(goal, np.float32)
        path = np.empty((max_waypoints, dof), np.float32)
        res = PlanResultC()
        _check(self.lib, self.lib.mrpop_session_plan(self.handle, scene.handle, robots.handle, flags,
                                                     start.ctypes.data, goal.ctypes.data, C.byref(settings),
                                                     path.ctypes.data, max_waypoints, C.byref(res)))
        return res, path[:min(res.waypoints, max_waypoints)].copy()

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mrpop_session_close(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
