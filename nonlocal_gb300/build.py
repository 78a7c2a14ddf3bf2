"""Builds the CUDA library nonlocal_gb300/lib/libnlgpu.so for sm_103a.

Each translation unit of csrc/ is compiled by nvcc in parallel
(-gencode arch=compute_103a,code=sm_103a), then linked into one shared
library exporting the C ABI of include/nlgpu.h.  The mesh and neighbour-search
units are compiled without fused multiply-add contraction so their
coordinates and distances round exactly as the reference's host code.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libnlgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = ["util.cu", "mesh.cu", "neighbours.cu", "boundary.cu", "pattern.cu", "assemble.cu", "solver.cu",
         "onedim.cu", "sweep.cu", "jacobi.cu", "mixed.cu", "flux.cu", "renumber.cu", "su2.cu", "nonlinear.cu",
         "bicgstab.cu", "elastic.cu", "coarse.cu", "iltbuild.cu",
         "batch.cu", "tc_gemm.cu",
         "mpnn.cu", "noalloc.cu", "api.cu"]
HEADERS = ["common.cuh", "ff.cuh", "influence.cuh"]
NO_FMA = {"mesh.cu", "neighbours.cu"}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(unit: str) -> list[str]:
    f = ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
         "--expt-relaxed-constexpr", "-Xptxas", "-O3"] + ARCH
    if unit in NO_FMA:
        f.append("--fmad=false")
    return f


def _deps() -> list[str]:
    return ([os.path.join(SRC, u) for u in UNITS + HEADERS] +
            [os.path.join(HERE, "..", "include", "nlgpu.h")])


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    cc = nvcc()

    def compile_unit(unit: str) -> str:
        obj = os.path.join(OUT, "obj", unit.replace(".cu", ".o"))
        cmd = [cc, "-c", os.path.join(SRC, unit), "-o", obj] + _flags(unit)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    # the CUDA runtime is linked statically: the library needs no libcudart at run time
    cmd = [cc, "-shared", "-cudart", "static", "-o", tmp] + objs + ARCH
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
