"""Build recipe for the CPU oracle (test infrastructure only).

  oracle/_build/libedge_oracle.so  the C restatement (gcc, OpenMP, no FP contraction)
  oracle/_ref/ref_planner.cubin    the reference's planner kernels: its
                                   pop_planner.cu, path_processing.cu and
                                   path_simplification.cu compiled unmodified
                                   and device-linked (same source tree)
  oracle/_ref/ref_harness.cubin    the reference's own device code wrapped by
                                   oracle/ref_harness.cu, compiled from the
                                   reference source tree named by the caller
                                   (argument, or the MRPOP_REF_ROOT environment
                                   variable); skipped when none is given

  python oracle/build.py [reference-root]
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def ref_root(arg: str | os.PathLike | None = None) -> Path | None:
    """The reference source tree: the argument, else $MRPOP_REF_ROOT, else None."""
    r = arg if arg is not None else os.environ.get("MRPOP_REF_ROOT")
    return Path(r) if r else None


def oracle_lib() -> Path:
    return HERE / "_build" / "libedge_oracle.so"


def ref_cubin() -> Path:
    return HERE / "_ref" / "ref_harness.cubin"


def ref_planner_cubin() -> Path:
    return HERE / "_ref" / "ref_planner.cubin"


def build_oracle(verbose: bool = False) -> Path:
    out = oracle_lib()
    out.parent.mkdir(parents=True, exist_ok=True)
    src = HERE / "edge_oracle.c"
    if out.exists() and out.stat().st_mtime > src.stat().st_mtime:
        return out
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           str(src), "-o", str(out), "-lm"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return out


def build_ref_harness(verbose: bool = False, root: str | os.PathLike | None = None) -> Path | None:
    """Compile the reference's edge-check device code into a cubin (needs the sources)."""
    REF_ROOT = ref_root(root)
    if REF_ROOT is None or not (REF_ROOT / "src" / "planning" / "utils.cuh").exists():
        return None
    out = ref_cubin()
    out.parent.mkdir(parents=True, exist_ok=True)
    src = HERE / "ref_harness.cu"
    if out.exists() and out.stat().st_mtime > src.stat().st_mtime:
        return out
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    # the reference's own flags (CMakeLists.txt:5-9): -lineinfo, default FP settings
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-std=c++17", "-w",
           f"-I{REF_ROOT}", f"-I{REF_ROOT / 'src' / 'planning'}", str(src), "-o", str(out)]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return out


def build_ref_planner(verbose: bool = False, root: str | os.PathLike | None = None) -> Path | None:
    """Compile the reference's planner sources (pop_planner.cu, path_processing.cu,
    path_simplification.cu) unmodified into relocatable cubins and device-link
    them into one module (oracle/ref_planner.py runs it)."""
    REF_ROOT = ref_root(root)
    if REF_ROOT is None or not (REF_ROOT / "src" / "planning" / "pop_planner.cu").exists():
        return None
    out = ref_planner_cubin()
    out.parent.mkdir(parents=True, exist_ok=True)
    if out.exists():
        return out
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    nvcc, nvlink = os.path.join(cuda, "bin", "nvcc"), os.path.join(cuda, "bin", "nvlink")
    parts = []
    for name in ("pop_planner", "path_processing", "path_simplification"):
        obj = out.parent / f"ref_{name}.rdc.cubin"
        # the reference's own flags (CMakeLists.txt:5-9): separable compilation, -lineinfo
        cmd = [nvcc, "-cubin", "-rdc=true", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-std=c++17",
               "-w", f"-I{REF_ROOT}", f"-I{REF_ROOT / 'src' / 'planning'}",
               str(REF_ROOT / "src" / "planning" / f"{name}.cu"), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        parts.append(str(obj))
    cmd = [nvlink, "-arch=sm_103a", *parts, "-o", str(out)]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref_harness(verbose=True, root=sys.argv[1] if len(sys.argv) > 1 else None))
    print(build_ref_planner(verbose=True, root=sys.argv[1] if len(sys.argv) > 1 else None))
