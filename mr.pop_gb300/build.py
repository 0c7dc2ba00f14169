"""Build recipe for the CUDA library (sm_103a only).

Compiles each translation unit under csrc/ with nvcc in parallel and links
`_build/libmrpop_gb300.so`.  Sources are rebuilt when newer than their object.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
SOURCES = ["api.cu", "batch.cu", "server.cu", "planner.cu", "drrt.cu", "peak_probe.cu", "no_alloc.cu"] + \
    [f"validate_a{a}.cu" for a in range(1, 6)]
# the planners' host arithmetic is written with explicit fmaf where the
# reference's compiler fuses; no other contraction, so x86 and Arm hosts agree;
# their per-attempt host work runs on OpenMP threads
SOURCE_FLAGS = {"drrt.cu": ["-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp"]}
LINK_FLAGS = ["-Xcompiler", "-fopenmp"]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def lib_path(variant: str = "") -> Path:
    return PKG / "_build" / (variant or "default") / "libmrpop_gb300.so"


def build(variant: str = "", defines: tuple[str, ...] = (), verbose: bool = False, jobs: int = 0) -> Path:
    """Compile and link the library; returns the .so path.

    variant/defines select an alternative build (e.g. a different
    MRPOP_PAIR_ORDER) into its own directory.
    """
    out_dir = lib_path(variant).parent
    out_dir.mkdir(parents=True, exist_ok=True)
    deps = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [INCLUDE / "mrpop.h"]
    dep_mtime = max(p.stat().st_mtime for p in deps)
    nvcc = _nvcc()
    dflags = [f"-D{d}" for d in defines]

    def compile_one(src: str) -> Path:
        obj = out_dir / (Path(src).stem + ".o")
        s = CSRC / src
        if obj.exists() and obj.stat().st_mtime > max(s.stat().st_mtime, dep_mtime):
            return obj
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *SOURCE_FLAGS.get(src, []), *dflags, f"-I{INCLUDE}", "-c", str(s), "-o",
               str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    n = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=n) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    lib = lib_path(variant)
    if not lib.exists() or lib.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart", *LINK_FLAGS]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    variant = sys.argv[1] if len(sys.argv) > 1 else ""
    defs = tuple(sys.argv[2:])
    print(build(variant, defs, verbose=True))
