"""The reference's planner (dRRT over per-arm roadmaps under AO-x) on the
batched validator, on the CPU: the settings and result layout, the C++
drop-in compiled against the reference's own headers, and solves driven by
the oracle as the validator (mrpop_drrt_solve_with: the planner's host logic
with nearest-neighbour searches on the host)."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
FIX = Path(__file__).parent / "golden" / "problems.npz"


def _ref_root():
    r = os.environ.get("MRPOP_REF_ROOT") or str(ROOT.parent / "reference")
    return Path(r) if (Path(r) / "src" / "planning" / "Planners.hh").exists() else None


def test_settings_defaults_are_pop_settings(pkg, lib_path):
    pkg.library(path=lib_path)
    s = pkg.drrt.settings_dict(pkg.drrt.settings())
    # src/planning/pop_settings.hh:3-32
    ref = dict(max_samples=1000000, max_iters=1000, optimize_iters=400000, num_new_configs=256, granularity=16,
               range=0.5, balance=2, tree_ratio=1.0, dynamic_domain=0, dd_alpha=0.0001, dd_radius=4.0,
               dd_min_radius=1.0, roadmap_reassign=0, rrtc_iter=1, resample_iter=5, cost_bound_resample=0,
               path_simplify=1, phs=1, simplify_round=1, bspline_step=3, bspline_min_change=0.01, perturb_step=3,
               perturb_empty_step=2)
    for k, v in ref.items():
        assert s[k] == pytest.approx(v), k
    # the driver's overrides (scripts/evaluate_mr.cu:162-166)
    e = pkg.drrt.settings_dict(pkg.drrt.evaluate_settings())
    assert (e["num_new_configs"], e["granularity"], e["range"], e["rrtc_iter"]) == (300, 64, 2.0, 3)
    assert (e["block_per_robot"], e["seed"]) == (8, 1234)


def test_bad_settings_are_refused(pkg, lib_path):
    pkg.library(path=lib_path)
    z = np.load(FIX)
    with pytest.raises(pkg.MrpopError):
        pkg.drrt.solve_with(4, lambda *a: None, z["a4_p0_start"], z["a4_p0_goal"], pkg.drrt.settings(granularity=0))
    with pytest.raises(pkg.MrpopError):
        pkg.drrt.solve_with(4, lambda *a: None, z["a4_p0_start"], z["a4_p0_goal"], pkg.drrt.settings(range=0.0))


def _oracle_validator(orc, scene, bases, calls=None):
    def validate(q0, q1, g, rule, range_, flags, arm):
        if calls is not None:
            calls.append((len(q0), g, rule, flags, arm))
        o = orc.validate(scene, bases, q0, q1, g, flags, arm, rule, range_, threads=orc.max_threads())
        return o["valid"], o["first_hit"]
    return validate


def _small(pkg, **kw):
    base = dict(num_new_configs=32, granularity=8, range=2.0, rrtc_iter=2, max_iters=40, max_launches=6)
    base.update(kw)
    return pkg.drrt.settings(**base)


def test_oracle_driven_solve_follows_the_reference_structure(pkg, lib_path, orc):
    """A 4-arm reference problem: the call pattern, the path's orientation and
    the bookkeeping of improving solutions."""
    pkg.library(path=lib_path)
    z = np.load(FIX)
    bases = z["a4_bases"]
    sc = pkg.SceneArrays(cuboids=z["a4_p0_boxes"])
    start, goal = z["a4_p0_start"], z["a4_p0_goal"]
    calls = []
    r = pkg.drrt.solve_with(4, _oracle_validator(orc, sc, bases, calls), start, goal, _small(pkg))
    assert r.solved and r.stats["passes"] == 2
    # reported path: goal -> start (record_connected_path order), every waypoint within the limits
    assert np.array_equal(r.path[0], goal) and np.array_equal(r.path[-1], start)
    lo, hi = np.tile(pkg.workloads.PANDA_LO, 4), np.tile(pkg.workloads.PANDA_HI, 4)
    assert ((r.path >= lo - 1e-5) & (r.path <= hi + 1e-5)).all()
    # improving solutions only, each reported with its cost; the last is the result
    costs = [s.cost for s in r.solutions]
    assert costs == sorted(costs, reverse=True) and costs[-1] == pytest.approx(r.cost)
    assert r.stats["path_length"] == len(r.path)
    # the check forms: roadmap nodes (one arm, g = 1) and edges (one arm, g), extend
    # (self only), connect, and the simplification's B-spline and shortcut rules
    kinds = {(g == 1, rule, flags, arm >= 0) for _, g, rule, flags, arm in calls}
    assert (True, 0, 3, True) in kinds and (False, 0, 3, True) in kinds
    assert (False, 0, 2, False) in kinds and (False, 1, 3, False) in kinds
    assert (False, 3, 3, False) in kinds
    assert r.stats["validate_calls"] == len(calls)
    assert all(n > 0 for n in r.stats["roadmap_nodes"]) and all(e > 0 for e in r.stats["roadmap_edges"])
    # calls by kind: roadmap (single-arm), extend (composite plain), connect, B-spline, shortcut
    by_kind = r.stats["check_calls"]
    assert sum(by_kind.values()) == len(calls)
    assert by_kind["roadmap"] == sum(1 for _, _, _, _, arm in calls if arm >= 0)
    assert by_kind["extend"] == sum(1 for _, _, rule, _, arm in calls if arm < 0 and rule == 0)
    assert by_kind["connect"] == sum(1 for _, _, rule, _, arm in calls if arm < 0 and rule == 1)
    assert all(r.stats["check_ns"][k] >= 0 for k in by_kind)


def test_oracle_driven_solve_is_deterministic(pkg, lib_path, orc):
    pkg.library(path=lib_path)
    z = np.load(FIX)
    bases = z["a5_bases"]
    sc = pkg.SceneArrays(cuboids=z["a5_p1_boxes"])
    st = _small(pkg, rrtc_iter=1, num_new_configs=24)
    a = pkg.drrt.solve_with(5, _oracle_validator(orc, sc, bases), z["a5_p1_start"], z["a5_p1_goal"], st)
    b = pkg.drrt.solve_with(5, _oracle_validator(orc, sc, bases), z["a5_p1_start"], z["a5_p1_goal"], st)
    assert a.solved == b.solved and a.cost == b.cost and np.array_equal(a.path, b.path)
    for k in ("iterations", "validate_calls", "edges_validated", "roadmap_nodes", "roadmap_edges"):
        assert a.stats[k] == b.stats[k], k
    c = pkg.drrt.solve_with(5, _oracle_validator(orc, sc, bases), z["a5_p1_start"], z["a5_p1_goal"],
                            _small(pkg, rrtc_iter=1, num_new_configs=24, seed=99))
    assert c.stats["roadmap_edges"] != a.stats["roadmap_edges"]  # another seed, other roadmaps


def test_dropin_builds_against_the_reference_headers(pkg, lib_path, tmp_path):
    """mr.pop_gb300/dropin/pop_planner_gb300.cu compiled with the reference's
    real Planners.hh / Robots.hh / pop_settings.hh / environment.hh, linked with
    a driver that calls dRRT::solve as the reference's benchmark driver does.
    Without a GPU the call reports the CUDA error and returns unsolved, as the
    reference's prints its errors and returns."""
    ref = _ref_root()
    if ref is None:
        pytest.skip("reference source tree not present (MRPOP_REF_ROOT)")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    inc = [f"-I{ref}", f"-I{ref / 'src' / 'planning'}", f"-I{ROOT / 'include'}"]
    arch = ["-gencode", "arch=compute_103a,code=sm_103a"]
    pp, drv, exe = tmp_path / "pp.o", tmp_path / "drv.o", tmp_path / "drv"
    subprocess.run([nvcc, "-std=c++17", *arch, "-w", *inc, "-c", str(ROOT / "mr.pop_gb300/dropin/pop_planner_gb300.cu"),
                    "-o", str(pp)], check=True)
    subprocess.run([nvcc, "-std=c++17", *arch, "-w", *inc, "-c", str(ROOT / "tests/dropin/drive_solve.cu"), "-o",
                    str(drv)], check=True)
    libdir = Path(lib_path).parent
    subprocess.run([nvcc, *arch, str(drv), str(pp), f"-L{libdir}", "-lmrpop_gb300", f"-Xlinker", f"-rpath={libdir}",
                    "-o", str(exe)], check=True)
    syms = subprocess.run(["nm", "-C", str(pp)], capture_output=True, text=True, check=True).stdout
    for robot, dim in (("Panda_four", 28), ("Panda_five", 35)):
        assert f"PlannerResult<ppln::robots::{robot}> dRRT::solve<ppln::robots::{robot}>" in syms
    z = np.load(FIX)
    prob = tmp_path / "p.txt"
    b = z["a4_p0_boxes"]
    with open(prob, "w") as f:
        f.write(f"4 {len(b)}\n")
        for r in b:
            f.write(" ".join(repr(float(x)) for x in r) + "\n")
        f.write(" ".join(repr(float(x)) for x in z["a4_p0_start"]) + "\n")
        f.write(" ".join(repr(float(x)) for x in z["a4_p0_goal"]) + "\n")
    out = subprocess.run([str(exe), str(prob)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    line = [l for l in out.stdout.splitlines() if l.startswith("result ")]
    assert line, out.stdout + out.stderr
    if "cuda" not in (out.stderr or "").lower() and "CUDA" not in out.stderr:
        # a GPU was present: the solve ran
        assert "solved=" in line[0]
    else:
        assert "solved=0" in line[0]


def test_reference_settings_struct_layout(tmp_path):
    """oracle/ref_planner.PopSettings (written into the reference module's
    __constant__ d_settings) has the byte layout of the reference's pop_settings."""
    ref = _ref_root()
    if ref is None:
        pytest.skip("reference source tree not present (MRPOP_REF_ROOT)")
    import ctypes as C
    from oracle.ref_planner import PopSettings
    src = tmp_path / "layout.cu"
    fields = [f for f, _ in PopSettings._fields_]
    body = "".join(f'std::printf("{f} %zu %zu\\n", offsetof(pop_settings, {f}), sizeof(((pop_settings*)0)->{f}));'
                   for f in fields)
    src.write_text('#include <cstdio>\n#include <cstddef>\n#include "src/planning/pop_settings.hh"\n'
                   'int main() {' + body + 'std::printf("sizeof %zu 0\\n", sizeof(pop_settings)); }\n')
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    exe = tmp_path / "layout"
    subprocess.run([nvcc, "-std=c++17", f"-I{ref}", str(src), "-o", str(exe)], check=True)
    got = {l.split()[0]: (int(l.split()[1]), int(l.split()[2]))
           for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()}
    assert got.pop("sizeof")[0] == C.sizeof(PopSettings)
    for f in fields:
        assert got[f] == (getattr(PopSettings, f).offset, getattr(PopSettings, f).size), f
