"""ctypes binding of the CPU oracle (oracle/edge_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker; nothing in the product imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

RULE_PLAIN, RULE_CONNECT, RULE_BSPLINE, RULE_SHORTCUT = 0, 1, 2, 3


class _Scene(C.Structure):
    _fields_ = [("spheres", C.c_void_p), ("n_spheres", C.c_int32), ("capsules", C.c_void_p),
                ("n_capsules", C.c_int32), ("zcapsules", C.c_void_p), ("n_zcapsules", C.c_int32),
                ("cuboids", C.c_void_p), ("n_cuboids", C.c_int32), ("zcuboids", C.c_void_p),
                ("n_zcuboids", C.c_int32)]


class _Robots(C.Structure):
    _fields_ = [("n_arms", C.c_int32), ("base", C.c_float * 80)]


class _Trig(C.Structure):
    _fields_ = [("keys", C.c_void_p), ("cosv", C.c_void_p), ("sinv", C.c_void_p), ("n", C.c_int64)]


_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        p = _build.build_oracle()
        L = C.CDLL(str(p))
        vp = C.c_void_p
        L.oracle_validate.argtypes = [C.POINTER(_Scene), C.POINTER(_Robots), vp, vp, C.c_int64, C.c_int, C.c_int,
                                      C.c_int, C.c_int, C.c_float, C.c_int, C.c_double, C.POINTER(_Trig), C.c_int,
                                      vp, vp, vp, C.POINTER(C.c_double), vp, vp]
        L.oracle_validate.restype = C.c_int
        L.oracle_fk_spheres.argtypes = [vp, vp, C.c_int64, C.c_int, C.c_int, C.c_int, C.POINTER(_Trig), vp]
        L.oracle_fk_spheres.restype = C.c_int
        L.oracle_edge_samples.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_float, vp, C.c_int64]
        L.oracle_edge_samples.restype = C.c_int64
        L.oracle_segment_count.argtypes = [vp, vp, C.c_int, C.c_int, C.c_float]
        L.oracle_segment_count.restype = C.c_int
        L.oracle_max_threads.restype = C.c_int
        L.oracle_det_spheres.argtypes = [vp]
        L.oracle_det_spheres.restype = C.c_int
        L.oracle_env_hit.argtypes = [C.POINTER(_Scene), C.c_float, C.c_float, C.c_float, C.c_float, C.c_int]
        L.oracle_env_hit.restype = C.c_int
        L.oracle_env_sd.argtypes = [C.POINTER(_Scene), C.c_double, C.c_double, C.c_double, C.c_double]
        L.oracle_env_sd.restype = C.c_double
        _LIB = L
    return _LIB


def _arr(a, cols):
    a = np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, cols))
    return a


class TrigTable:
    """Sorted table of (float bits -> cos, sin) values, e.g. device __cosf/__sinf."""

    def __init__(self, x: np.ndarray, cosv: np.ndarray, sinv: np.ndarray):
        x = np.ascontiguousarray(x, np.float32).ravel()
        keys = x.view(np.uint32)
        order = np.argsort(keys, kind="stable")
        keys = keys[order]
        uniq = np.ones(len(keys), bool)
        uniq[1:] = keys[1:] != keys[:-1]
        self.keys = np.ascontiguousarray(keys[uniq])
        self.cosv = np.ascontiguousarray(np.asarray(cosv, np.float32).ravel()[order][uniq])
        self.sinv = np.ascontiguousarray(np.asarray(sinv, np.float32).ravel()[order][uniq])
        self._c = _Trig(self.keys.ctypes.data, self.cosv.ctypes.data, self.sinv.ctypes.data, len(self.keys))


def _scene_struct(scene):
    keep = [_arr(scene.spheres, 4), _arr(scene.capsules, 8), _arr(scene.z_capsules, 8), _arr(scene.cuboids, 15),
            _arr(scene.z_cuboids, 15)]
    p = [k.ctypes.data if k.size else None for k in keep]
    s = _Scene(p[0], len(keep[0]), p[1], len(keep[1]), p[2], len(keep[2]), p[3], len(keep[3]), p[4], len(keep[4]))
    return s, keep


def _robots_struct(bases: np.ndarray):
    bases = np.asarray(bases, np.float32).reshape(-1, 16)
    r = _Robots()
    r.n_arms = len(bases)
    flat = np.zeros(80, np.float32)
    flat[:bases.size] = bases.ravel()
    r.base[:] = flat.tolist()
    return r


def validate(scene, bases, q0, q1, g, flags, arm=-1, rule=RULE_PLAIN, range_=0.0, pair_order=0, band=0.0,
             trig: TrigTable | None = None, threads=0, count_ambiguous=False):
    """Oracle verdicts: dict(valid u8, first_hit i32, ambiguous u8, flops float, n_seg i32).

    With band > 0 an edge is ambiguous when one of its checked samples has a
    deciding minimum signed distance (FP64) within band metres of zero;
    count_ambiguous=True also returns amb_samples i32, the number of such
    samples per edge (every checked sample is then examined)."""
    L = lib()
    q0 = np.ascontiguousarray(q0, np.float32)
    q1 = np.ascontiguousarray(q1, np.float32)
    n = q0.shape[0]
    sc, keep = _scene_struct(scene)
    rb = _robots_struct(bases)
    valid = np.zeros(n, np.uint8)
    first = np.zeros(n, np.int32)
    amb = np.zeros(n, np.uint8)
    nseg = np.zeros(n, np.int32)
    fl = C.c_double(0.0)
    ams = np.zeros(n, np.int32) if count_ambiguous else None
    rc = L.oracle_validate(C.byref(sc), C.byref(rb), q0.ctypes.data, q1.ctypes.data, n, g, flags, arm, rule,
                           float(range_), pair_order, float(band), C.byref(trig._c) if trig else None, threads,
                           valid.ctypes.data, first.ctypes.data, amb.ctypes.data, C.byref(fl), nseg.ctypes.data,
                           ams.ctypes.data if ams is not None else None)
    if rc == 1:
        raise ValueError("oracle_validate: bad arguments")
    if rc == 2:
        raise KeyError("oracle_validate: a sine/cosine input was missing from the trig table")
    out = {"valid": valid, "first_hit": first, "ambiguous": amb, "flops": fl.value, "n_seg": nseg}
    if ams is not None:
        out["amb_samples"] = ams
    return out


def validate_with_trig(scene, bases, q0, q1, g, flags, arm, rule, range_, trig_fn, threads=0):
    """validate() with the sine/cosine values of every sample taken from
    trig_fn(x) -> (cos, sin) (e.g. the device's __cosf/__sinf), which makes the
    restatement bit-exact against device code."""
    samples = edge_samples(q0, q1, g, rule, range_)
    x = np.ascontiguousarray(samples, np.float32).ravel()
    c, s = trig_fn(x)
    return validate(scene, bases, q0, q1, g, flags, arm, rule, range_, trig=TrigTable(x, c, s), threads=threads)


def fk_spheres(base, q, detailed, fp64=False, pair_order=0, trig: TrigTable | None = None) -> np.ndarray:
    L = lib()
    base = np.ascontiguousarray(np.asarray(base, np.float32).reshape(16))
    q = np.ascontiguousarray(q, np.float32).reshape(-1, 7)
    ns = 59 if detailed else 11
    out = np.zeros((len(q), ns, 3), np.float64)
    rc = L.oracle_fk_spheres(base.ctypes.data, q.ctypes.data, len(q), int(detailed), int(fp64), pair_order,
                             C.byref(trig._c) if trig else None, out.ctypes.data)
    if rc == 2:
        raise KeyError("oracle_fk_spheres: a sine/cosine input was missing from the trig table")
    return out


def edge_samples(q0, q1, g, rule=RULE_PLAIN, range_=0.0) -> np.ndarray:
    """All interpolated sample configurations of the edges (n_samples, dof)."""
    L = lib()
    q0 = np.ascontiguousarray(q0, np.float32)
    q1 = np.ascontiguousarray(q1, np.float32)
    dim = q0.shape[1]
    chunks = []
    for a, b in zip(q0, q1):
        n = L.oracle_segment_count(a.ctypes.data, b.ctypes.data, dim, rule, float(range_))
        m = max(n, 0) * g * dim
        out = np.zeros(max(m, 1), np.float32)
        L.oracle_edge_samples(a.ctypes.data, b.ctypes.data, dim, g, rule, float(range_), out.ctypes.data, m)
        chunks.append(out[:m].reshape(-1, dim))
    return np.concatenate(chunks) if chunks else np.zeros((0, dim), np.float32)


def env_hit(scene, x, y, z, r, pair_order=0) -> bool:
    """FP32 verdict of one sphere against the scene (reference scene loop)."""
    sc, keep = _scene_struct(scene)
    return bool(lib().oracle_env_hit(C.byref(sc), float(x), float(y), float(z), float(r), pair_order))


def env_sd(scene, x, y, z, r) -> float:
    """FP64 signed distance of one sphere to the closest obstacle."""
    sc, keep = _scene_struct(scene)
    return float(lib().oracle_env_sd(C.byref(sc), float(x), float(y), float(z), float(r)))


def det_spheres() -> np.ndarray:
    """The detailed sphere table (59, 4): local centre and radius."""
    out = np.zeros((59, 4), np.float32)
    lib().oracle_det_spheres(out.ctypes.data)
    return out


def max_threads() -> int:
    return lib().oracle_max_threads()
