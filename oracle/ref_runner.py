"""Loader for the reference-harness cubin (oracle/_ref/ref_harness.cubin).

TEST INFRASTRUCTURE ONLY.  Runs the reference's own edge-check device code on
the current CUDA device through the driver API (ctypes on libcuda), with
torch tensors for device memory.  The cubin is built from the reference
sources by oracle/build.py where they are present; where it is absent every
entry point raises FileNotFoundError and callers skip.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_CU = None


def _cuda():
    global _CU
    if _CU is None:
        for name in ("libcuda.so.1", "libcuda.so"):
            try:
                _CU = C.CDLL(name)
                break
            except OSError:
                continue
        if _CU is None:
            raise OSError("libcuda not found")
    return _CU


def _ck(rc, what):
    if rc != 0:
        s = C.c_char_p()
        _cuda().cuGetErrorString(rc, C.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value.decode() if s.value else '?'})")


def available() -> bool:
    return _build.ref_cubin().exists()


class RefHarness:
    """The reference's fkcc_single_buffer* routines wrapped as batch kernels."""

    KIND_COMPOSITE, KIND_EXTEND, KIND_SINGLE = 0, 1, 2

    def __init__(self, cubin: Path | None = None):
        import torch
        p = Path(cubin) if cubin else _build.ref_cubin()
        if not p.exists():
            raise FileNotFoundError(f"reference harness not built: {p}")
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        cu = _cuda()
        self.mod = C.c_void_p()
        _ck(cu.cuModuleLoad(C.byref(self.mod), str(p).encode()), "cuModuleLoad")
        self.fn = {}
        for name in ("ref_sizes", "ref_env_build", "ref_validate", "ref_fk"):
            f = C.c_void_p()
            _ck(cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()), f"cuModuleGetFunction {name}")
            self.fn[name] = f
        self.torch = torch
        sz = torch.zeros(4, dtype=torch.int32, device="cuda")
        self._launch("ref_sizes", 1, 1, [C.c_void_p(sz.data_ptr())])
        torch.cuda.synchronize()
        self.sizes = sz.cpu().numpy().tolist()  # Environment, Sphere, Capsule, Cuboid
        self._scratch = None

    def _launch(self, name, grid, block, args, stream=None):
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        st = C.c_void_p(stream.cuda_stream if stream is not None else self.torch.cuda.current_stream().cuda_stream)
        _ck(_cuda().cuLaunchKernel(self.fn[name], grid, 1, 1, block, 1, 1, 0, st, arr, None), f"launch {name}")

    def set_symbol(self, name: str, values: np.ndarray):
        """Overwrite a __constant__ table of the module (e.g. a base layout)."""
        dptr, nbytes = C.c_uint64(), C.c_size_t()
        _ck(_cuda().cuModuleGetGlobal_v2(C.byref(dptr), C.byref(nbytes), self.mod, name.encode()),
            f"cuModuleGetGlobal {name}")
        v = np.ascontiguousarray(values, np.float32)
        if v.nbytes > nbytes.value:
            raise ValueError(f"{name}: {v.nbytes} bytes > {nbytes.value}")
        self.torch.cuda.synchronize()
        _ck(_cuda().cuMemcpyHtoD_v2(dptr, v.ctypes.data, C.c_size_t(v.nbytes)), f"cuMemcpyHtoD {name}")

    # mangled names of the reference's base tables
    SYM_BASE4 = "_ZN4ppln9collision27robot_base_transform_4pandaE"
    SYM_BASE5 = "_ZN4ppln9collision27robot_base_transform_5pandaE"
    SYM_QUAD = "_ZN4ppln9collision26quad_franka_base_transformE"
    SYM_FIVE = "_ZN4ppln9collision26five_franka_base_transformE"

    def set_bases(self, n_arms: int, bases: np.ndarray):
        """Point the composite robot of `n_arms` (4 or 5) and the single-arm
        table of the same size at `bases` (n_arms x 4 x 4 row-major)."""
        b = np.asarray(bases, np.float32).reshape(n_arms, 16)
        if n_arms == 4:
            self.set_symbol(self.SYM_BASE4, b)
            self.set_symbol(self.SYM_QUAD, b)
        elif n_arms == 5:
            self.set_symbol(self.SYM_BASE5, b)
            self.set_symbol(self.SYM_FIVE, b)
        else:
            raise ValueError("the reference has compiled-in layouts for 4 and 5 arms only")

    def make_env(self, scene):
        """Build a device Environment<float> from SceneArrays; returns an owner dict."""
        torch = self.torch
        env_sz, sph_sz, cap_sz, cub_sz = self.sizes

        def dev(a, cols):
            a = np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, cols))
            return torch.from_numpy(a).cuda() if a.size else torch.zeros(1, device="cuda")

        src = [dev(scene.spheres, 4), dev(scene.capsules, 8), dev(scene.z_capsules, 8), dev(scene.cuboids, 15),
               dev(scene.z_cuboids, 15)]
        counts = [len(scene.spheres), len(scene.capsules), len(scene.z_capsules), len(scene.cuboids),
                  len(scene.z_cuboids)]
        sizes = [sph_sz, cap_sz, cap_sz, cub_sz, cub_sz]
        dst = [torch.zeros(max(1, n) * s, dtype=torch.uint8, device="cuda") for n, s in zip(counts, sizes)]
        env = torch.zeros(env_sz, dtype=torch.uint8, device="cuda")
        args = [C.c_void_p(env.data_ptr())]
        for s, n in zip(src, counts):
            args += [C.c_void_p(s.data_ptr()), C.c_int(n)]
        args += [C.c_void_p(d.data_ptr()) for d in dst]
        self._launch("ref_env_build", 1, 1, args)
        torch.cuda.synchronize()
        return {"env": env, "keep": src + dst}

    def scratch(self, blocks: int):
        torch = self.torch
        if self._scratch is None or self._scratch[0] < blocks:
            self._scratch = (blocks, torch.zeros(blocks * 57344, dtype=torch.float32, device="cuda"),
                             torch.zeros(blocks * 8000, dtype=torch.int32, device="cuda"))
        return self._scratch[1], self._scratch[2]

    def validate(self, env, q0, q1, g, kind, rule=0, range_=0.0, num_robot=4, robot_id=0, blocks=None,
                 stream=None, out=None):
        """q0/q1: CUDA float32 tensors [n, dof].  Returns (valid i32, seg_fail i32) tensors."""
        torch = self.torch
        n = q0.shape[0]
        if blocks is None:
            blocks = min(n, 152 * 4)
        sp, lc = self.scratch(blocks)
        if out is None:
            out = (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"))
        args = [C.c_void_p(env["env"].data_ptr()), C.c_void_p(q0.data_ptr()), C.c_void_p(q1.data_ptr()), C.c_int(n),
                C.c_int(g), C.c_int(kind), C.c_int(rule), C.c_float(range_), C.c_int(num_robot),
                C.c_int(robot_id), C.c_void_p(sp.data_ptr()), C.c_void_p(lc.data_ptr()),
                C.c_void_p(out[0].data_ptr()), C.c_void_p(out[1].data_ptr())]
        self._launch("ref_validate", blocks, 4 * g, args, stream)
        return out

    def fk(self, q, kind, num_robot=1, robot_id=0, detailed=False):
        """Sphere centres: kind 0 single arm (q [n,7]); 4/5 composite (q [n,28|35])."""
        torch = self.torch
        n = q.shape[0]
        blocks = (n + 63) // 64
        sp, _ = self.scratch(blocks)
        ns = 59 if detailed else 11
        arms = 1 if kind == 0 else kind
        out = torch.empty((n, arms, ns, 3), dtype=torch.float32, device="cuda")
        args = [C.c_void_p(q.data_ptr()), C.c_int(n), C.c_int(kind), C.c_int(num_robot), C.c_int(robot_id),
                C.c_int(int(detailed)), C.c_void_p(sp.data_ptr()), C.c_void_p(out.data_ptr())]
        self._launch("ref_fk", blocks, 256, args)
        return out
