"""The reference's own planner kernels, run on the current CUDA device.

TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the product never loads it.

oracle/_ref/ref_planner.cubin is the reference's src/planning/pop_planner.cu,
path_processing.cu and path_simplification.cu compiled unmodified for sm_103a
(relocatable) and device-linked into one module (oracle/build.py).  Its
kernels -- build_roadmap<Panda>, rrtc<Panda_four|Panda_five>,
multiBlock_simplify<...>, init_xorwow, init_rng -- run here exactly as
compiled; the host side of dRRT::solve (pop_planner.cu:739-1030) cannot run
here (its host code is built for another machine), so `RefPlanner.solve`
restates it through the CUDA driver API: the same allocations, pointer
tables, symbol copies, launch shapes and pass loop, with three bounds the
reference does not have, so that no launch can overrun its fixed arrays:

  - the roadmaps are seeded on the host with what the first build_roadmap
    launch writes (start and goal rows, sizes, component ids, edge bits,
    roadmap_interior.cuh:67-83) and roadmap_launch_cnt is set, so every
    launch runs one round of 230 samples per block and returns; the host
    relaunches it until every arm's start and goal are connected (the first
    launch of the reference loops inside the kernel instead, and later
    launches also grow the arms that are connected -- here that happens in
    the first pass too), stopping before a roadmap could pass
    MAX_ROADMAP_SIZE (roadmap_interior.cuh:21, whose overflow would write
    past the roadmap arrays);
  - the first pass repeats build_roadmap + rrtc while unsolved as the
    reference's do/while does (pop_planner.cu:958-984), at most
    `max_launches` times and only while the trees have room for another
    launch (max_iters x 2 nodes per block; the reference writes past them);
  - the simplification kernel runs only once a path exists (with none it
    would read simplify_path_cost[-1]).
Each solve loads the module afresh (its __device__ state starts as the
reference's does after cudaDeviceReset, pop_planner.cu:1028).
"""
from __future__ import annotations

import ctypes as C
import time
from pathlib import Path

import numpy as np

from . import build as _build
from .ref_runner import RefHarness, _ck, _cuda

UNWRITTEN = -9999.0  # UNWRITTEN_VAL (pop_planner_state.cuh:10)
MAX_ROADMAP = 100000  # MAX_ROADMAP_SIZE (roadmap_interior.cuh:21)
ROADMAP_ITER = 230  # ROADMAP_BUILD_ITER (roadmap_interior.cuh:20)
CURAND_STATE_BYTES = 64  # >= sizeof(curandStateXORWOW_t)


class PopSettings(C.Structure):
    """pop_settings (src/planning/pop_settings.hh:3-32), byte for byte."""
    _fields_ = [("max_samples", C.c_int32), ("max_iters", C.c_int32), ("optimize_iters", C.c_int32),
                ("num_new_configs", C.c_int32), ("granularity", C.c_int32), ("range", C.c_float),
                ("balance", C.c_int32), ("tree_ratio", C.c_float), ("dynamic_domain", C.c_bool),
                ("dd_alpha", C.c_float), ("dd_radius", C.c_float), ("dd_min_radius", C.c_float),
                ("roadmap_reassign", C.c_bool), ("rrtc_iter", C.c_int32), ("resample_iter", C.c_int32),
                ("cost_bound_resample", C.c_bool), ("path_simplify", C.c_bool), ("phs", C.c_bool),
                ("simplify_round", C.c_int32), ("bspline_step", C.c_int32), ("bspline_min_change", C.c_float),
                ("perturb_step", C.c_int32), ("perturb_empty_step", C.c_int32)]


def pop_settings(**kw) -> PopSettings:
    """The struct's defaults, then the overrides."""
    s = PopSettings(max_samples=1000000, max_iters=1000, optimize_iters=400000, num_new_configs=256,
                    granularity=16, range=0.5, balance=2, tree_ratio=1.0, dynamic_domain=False, dd_alpha=0.0001,
                    dd_radius=4.0, dd_min_radius=1.0, roadmap_reassign=False, rrtc_iter=1, resample_iter=5,
                    cost_bound_resample=False, path_simplify=True, phs=True, simplify_round=1, bspline_step=3,
                    bspline_min_change=0.01, perturb_step=3, perturb_empty_step=2)
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def evaluate_settings(**kw) -> PopSettings:
    """The reference benchmark driver's settings (scripts/evaluate_mr.cu:162-166)."""
    base = dict(num_new_configs=300, granularity=64, range=2.0, rrtc_iter=3)
    base.update(kw)
    return pop_settings(**base)


def available() -> bool:
    return _build.ref_planner_cubin().exists() and _build.ref_cubin().exists()


def _sym(*names: str) -> str:
    """Itanium mangling of a namespace-scope variable dRRT::name."""
    return "_ZN" + "".join(f"{len(n)}{n}" for n in names) + "E"


class RefPlanner:
    """dRRT::solve of the reference, its kernels from the cubin."""

    def __init__(self, cubin: Path | None = None):
        import torch
        self.torch = torch
        p = Path(cubin) if cubin else _build.ref_planner_cubin()
        if not p.exists():
            raise FileNotFoundError(f"reference planner not built: {p}")
        self.path = p
        self.env_builder = RefHarness()  # builds device Environment<float> with the reference's own layout
        self.cu = _cuda()
        self.mod = None

    # -- module ---------------------------------------------------------------
    def _load(self):
        cu = self.cu
        if self.mod is not None:
            _ck(cu.cuModuleUnload(self.mod), "cuModuleUnload")
        self.mod = C.c_void_p()
        _ck(cu.cuModuleLoad(C.byref(self.mod), str(self.path).encode()), "cuModuleLoad ref_planner")
        n = C.c_uint()
        _ck(cu.cuModuleGetFunctionCount(C.byref(n), self.mod), "cuModuleGetFunctionCount")
        fns = (C.c_void_p * n.value)()
        _ck(cu.cuModuleEnumerateFunctions(fns, n, self.mod), "cuModuleEnumerateFunctions")
        self.fn = {}
        for f in fns:
            name = C.c_char_p()
            _ck(cu.cuFuncGetName(C.byref(name), C.c_void_p(f)), "cuFuncGetName")
            self.fn[name.value.decode()] = C.c_void_p(f)

    def _kernel(self, *parts: str) -> C.c_void_p:
        hits = [k for k in self.fn if all(p in k for p in parts)]
        if len(hits) != 1:
            raise KeyError(f"kernel {parts}: {hits}")
        return self.fn[hits[0]]

    def _global(self, name: str):
        dptr, nbytes = C.c_uint64(), C.c_size_t()
        _ck(self.cu.cuModuleGetGlobal_v2(C.byref(dptr), C.byref(nbytes), self.mod, _sym("dRRT", name).encode()),
            f"cuModuleGetGlobal {name}")
        return dptr.value, nbytes.value

    def _put(self, name: str, data: bytes | np.ndarray):
        dptr, nb = self._global(name)
        b = data.tobytes() if isinstance(data, np.ndarray) else bytes(data)
        assert len(b) <= nb, (name, len(b), nb)
        _ck(self.cu.cuMemcpyHtoD_v2(C.c_uint64(dptr), b, C.c_size_t(len(b))), f"HtoD {name}")

    def _get(self, name: str, dtype, count: int) -> np.ndarray:
        dptr, nb = self._global(name)
        out = np.zeros(count, dtype)
        assert out.nbytes <= nb
        _ck(self.cu.cuMemcpyDtoH_v2(out.ctypes.data, C.c_uint64(dptr), C.c_size_t(out.nbytes)), f"DtoH {name}")
        return out

    def _launch(self, f, grid, block, args, cooperative=False):
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        st = C.c_void_p(0)
        if cooperative:
            _ck(self.cu.cuLaunchCooperativeKernel(f, grid, 1, 1, block, 1, 1, 0, st, arr), "cooperative launch")
        else:
            _ck(self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, st, arr, None), "launch")

    def _sync(self):
        _ck(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    # -- one solve ---------------------------------------------------------------
    def solve(self, scene, start, goals, settings: PopSettings, num_robots: int, block_per_robot: int = 8,
              bases: np.ndarray | None = None, max_launches: int = 10) -> dict:
        """One dRRT::solve(start, goals, env, settings, num_robots, block_per_robot).
        bases: overwrite the compiled-in base table of num_robots arms (None:
        the reference's own layout)."""
        torch = self.torch
        t_wall = time.perf_counter_ns()
        self._load()
        robot = {4: "Panda_four", 5: "Panda_five"}[num_robots]
        k_init = self._kernel("init_xorwow")
        k_rng = self._kernel("init_rng")
        k_road = self._kernel("13build_roadmapIN4ppln6robots5PandaE")
        k_rrtc = self._kernel(f"4rrtcIN4ppln6robots{len(robot)}{robot}E")
        k_simp = self._kernel(f"19multiBlock_simplifyIN4ppln6robots{len(robot)}{robot}E")
        if bases is not None:
            self._put_bases(num_robots, bases)
        S = settings
        dim = 7 * num_robots
        g = int(S.granularity)
        goals = np.ascontiguousarray(np.asarray(goals, np.float32).reshape(-1, dim))
        start = np.ascontiguousarray(np.asarray(start, np.float32).reshape(dim))
        ng = len(goals)
        dev = "cuda"
        keep = []

        def ptr(t):
            return t.data_ptr()

        def ptr_table(ptrs):
            t = torch.from_numpy(np.asarray(ptrs, np.uint64).view(np.int64)).to(dev)
            keep.append(t)
            return t

        states = torch.zeros(S.num_new_configs * dim * CURAND_STATE_BYTES, dtype=torch.uint8, device=dev)
        rng_states = torch.zeros(S.num_new_configs * dim * CURAND_STATE_BYTES, dtype=torch.uint8, device=dev)
        self._launch(k_init, S.num_new_configs, dim, [C.c_void_p(ptr(states)), C.c_ulonglong(1234)])
        self._launch(k_rng, 5, 64, [C.c_void_p(ptr(rng_states)), C.c_ulong(1), C.c_int(S.num_new_configs * dim)])
        self._put("d_settings", bytes(S))
        d_start = torch.from_numpy(start).to(dev)
        d_goals = torch.from_numpy(goals.ravel()).to(dev)
        nodes = [torch.empty(S.max_samples * dim, dtype=torch.float32, device=dev) for _ in range(2)]
        parents = [torch.zeros(S.max_samples, dtype=torch.int32, device=dev) for _ in range(2)]
        radii = [torch.zeros(S.max_samples, dtype=torch.float32, device=dev) for _ in range(2)]
        cost = [torch.zeros(S.max_samples, dtype=torch.float32, device=dev) for _ in range(2)]
        d_nodes, d_parents = ptr_table([ptr(t) for t in nodes]), ptr_table([ptr(t) for t in parents])
        d_radii, d_cost = ptr_table([ptr(t) for t in radii]), ptr_table([ptr(t) for t in cost])
        sphere = torch.zeros(300 * 100000, dtype=torch.float32, device=dev)
        d_sphere = ptr_table([ptr(sphere) + 4 * 100000 * i for i in range(300)])
        roadmaps = torch.full((8, 700000), UNWRITTEN, dtype=torch.float32, device=dev)
        d_roadmaps = ptr_table([ptr(roadmaps) + 4 * 700000 * i for i in range(8)])
        comp = torch.zeros((8, MAX_ROADMAP), dtype=torch.int32, device=dev)
        d_comp = ptr_table([ptr(comp) + 4 * MAX_ROADMAP * i for i in range(8)])
        D1, D2 = 100000, 3200
        edges = torch.zeros((8, D1, D2), dtype=torch.int32, device=dev)  # 10.24 GB, as the reference
        mids = [ptr_table([ptr(edges) + 4 * (D1 * D2 * i + D2 * j) for j in range(D1)]) for i in range(8)]
        d_edges = ptr_table([ptr(m) for m in mids])
        env = self.env_builder.make_env(scene)
        keep.append(env)
        env_ptr = env["env"].data_ptr()
        radii[0][0] = float(np.finfo(np.float32).max)
        radii[1][:ng] = float(np.finfo(np.float32).max)
        parents[1][:ng] = torch.arange(ng, dtype=torch.int32, device=dev)
        nra = [torch.zeros(8 * S.max_samples, dtype=torch.int32, device=dev) for _ in range(2)]
        nra_mid = [ptr_table([ptr(t) + 4 * S.max_samples * j for j in range(8)]) for t in nra]
        d_nra = ptr_table([ptr(m) for m in nra_mid])
        # what the first build_roadmap launch writes (roadmap_interior.cuh:67-83)
        for r in range(num_robots):
            roadmaps[r, 0:7] = d_start[7 * r:7 * r + 7]
            for t in range(ng):
                roadmaps[r, 7 * (1 + t):7 * (2 + t)] = d_goals[t * dim + 7 * r:t * dim + 7 * r + 7]
            comp[r, 0] = 0
            comp[r, 1:1 + ng] = 1
            edges[r, 0, 0] = 1
            for i in range(ng):
                edges[r, i + 1, (i + 1) >> 5] |= 1 << ((i + 1) & 31)
        self._put("roadmap_size", np.array([ng + 1 if r < num_robots else 0 for r in range(8)], np.int32))
        self._put("roadmap_launch_cnt", np.array([1], np.int32))
        torch.cuda.synchronize()

        road_args = [C.c_void_p(env_ptr), C.c_void_p(ptr(d_start)), C.c_void_p(ptr(d_goals)), C.c_void_p(ptr(d_sphere)),
                     C.c_void_p(ptr(d_roadmaps)), C.c_void_p(ptr(d_comp)), C.c_void_p(ptr(d_edges)), C.c_int(ng),
                     C.c_void_p(ptr(states)), C.c_int(block_per_robot), C.c_int(num_robots), C.c_int(g)]
        rrtc_args = [C.c_void_p(ptr(d_nodes)), C.c_void_p(ptr(d_parents)), C.c_void_p(ptr(d_cost)),
                     C.c_void_p(ptr(d_nra)), C.c_void_p(ptr(d_sphere)), C.c_void_p(ptr(d_roadmaps)),
                     C.c_void_p(ptr(d_edges)), C.c_void_p(ptr(d_radii)), C.c_void_p(ptr(states)),
                     C.c_void_p(ptr(rng_states)), C.c_void_p(env_ptr)]
        simp_args = [C.c_int(16), C.c_int(4 * g), C.c_void_p(env_ptr), C.c_void_p(ptr(d_sphere))]
        road_grid, road_block = num_robots * block_per_robot, 4 * g

        def roadmap_sizes():
            return self._get("roadmap_size", np.int32, 8)[:num_robots]

        def build_round():
            self._launch(k_road, road_grid, road_block, road_args, cooperative=True)
            self._sync()

        room = MAX_ROADMAP - block_per_robot * ROADMAP_ITER * 2
        res = {"solved": False, "cost": 0.0, "path": np.zeros((0, dim), np.float32), "iters": 0,
               "seed_costs": [], "launches": 0, "roadmap_rounds": 0, "passes": 0, "stopped": None}
        init_sol = False
        t_kernel = time.perf_counter_ns()
        for pass_i in range(S.rrtc_iter):
            res["passes"] += 1
            for t in range(2):
                nodes[t].fill_(UNWRITTEN)
            self._put("atomic_free_index", np.array([1, ng], np.int32))
            self._put("nodes_size", np.array([1, ng], np.int32))
            self._put("completed_nodes", np.array([1, ng], np.int32))
            nodes[0][:dim] = d_start
            nodes[1][:ng * dim] = d_goals
            optimize = 1 if pass_i else 0
            self._put("optimize", np.array([optimize], np.int32))
            torch.cuda.synchronize()
            solved = 0
            first_launch = True
            while True:
                # build_roadmap: one round; in the first pass's first launch,
                # rounds until every arm's start and goal are connected
                while True:
                    if int(roadmap_sizes().max()) >= room:
                        res["stopped"] = "roadmap size"
                        break
                    build_round()
                    res["roadmap_rounds"] += 1
                    if not (first_launch and pass_i == 0):
                        break
                    conn = self._get("start_goal_connected", np.uint8, 8)[:num_robots]
                    if conn.all() or res["roadmap_rounds"] >= 50:
                        break
                first_launch = False
                self._launch(k_rrtc, S.num_new_configs, 4 * g, rrtc_args)
                self._sync()
                solved = int(self._get("solved", np.int32, 1)[0])
                if not optimize:
                    res["launches"] += 1
                if solved > 0 or optimize:
                    break
                free = self._get("atomic_free_index", np.int32, 2)
                if res["launches"] >= max_launches:
                    res["stopped"] = "launch bound"
                    break
                if int(free.max()) + 2 * S.num_new_configs * S.max_iters >= S.max_samples:
                    res["stopped"] = "tree capacity"
                    break
            have_path = int(self._get("path_size", np.int32, 2).sum()) > 0
            if S.path_simplify and have_path:
                self._launch(k_simp, 16, 4 * g, simp_args, cooperative=True)
                self._sync()
            h_cost = float(self._get("cost", np.float32, 1)[0])
            if solved > 0 and (not init_sol or res["cost"] > h_cost):
                init_sol = True
                ps = self._get("path_size", np.int32, 2)
                n_total = int(ps.sum())
                po = self._get("path_out", np.float32, n_total * dim).reshape(n_total, dim)
                po = po[po[:, 0] != UNWRITTEN]
                free = self._get("atomic_free_index", np.int32, 2)
                res.update(solved=True, cost=h_cost, path=po, iters=int(self._get("solved_iters", np.int32, 1)[0]),
                           start_tree_size=int(free[0]), goal_tree_size=int(free[1]))
                res["seed_costs"].append(h_cost)
        res["kernel_ns"] = time.perf_counter_ns() - t_kernel
        res["roadmap_sizes"] = roadmap_sizes().tolist()
        res["path_length"] = int(len(res["path"]))
        del keep, edges, mids, nodes, roadmaps, sphere
        torch.cuda.synchronize()
        res["wall_ns"] = time.perf_counter_ns() - t_wall
        return res

    def _put_bases(self, n_arms: int, bases: np.ndarray):
        b = np.ascontiguousarray(np.asarray(bases, np.float32).reshape(n_arms, 16))
        names = {4: ("_ZN4ppln9collision27robot_base_transform_4pandaE",
                     "_ZN4ppln9collision26quad_franka_base_transformE"),
                 5: ("_ZN4ppln9collision27robot_base_transform_5pandaE",
                     "_ZN4ppln9collision26five_franka_base_transformE")}[n_arms]
        for nm in names:
            dptr, nbytes = C.c_uint64(), C.c_size_t()
            if self.cu.cuModuleGetGlobal_v2(C.byref(dptr), C.byref(nbytes), self.mod, nm.encode()) != 0:
                continue
            assert b.nbytes <= nbytes.value
            _ck(self.cu.cuMemcpyHtoD_v2(dptr, b.ctypes.data, C.c_size_t(b.nbytes)), f"HtoD {nm}")
