"""Build recipe for the CPU oracle (test infrastructure only).

  oracle/_build/libedge_oracle.so  the C restatement (gcc, OpenMP, no FP contraction)
  oracle/_ref/ref_harness.cubin    the reference's own device code wrapped by
                                   oracle/ref_harness.cu, compiled from the
                                   reference sources when they are present
                                   (`REF_ROOT`, default /root/reference)
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_ROOT = Path(os.environ.get("REF_ROOT", "/root/reference"))


def oracle_lib() -> Path:
    return HERE / "_build" / "libedge_oracle.so"


def ref_cubin() -> Path:
    return HERE / "_ref" / "ref_harness.cubin"


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


def build_ref_harness(verbose: bool = False) -> Path | None:
    """Compile the reference's edge-check device code into a cubin (needs the sources)."""
    if not (REF_ROOT / "src" / "planning" / "utils.cuh").exists():
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


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref_harness(verbose=True))
