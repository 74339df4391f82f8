"""Build libphase_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared
library next to this file.  Host code is compiled with -ffp-contract=off so
mesh geometry rounds exactly as the reference's x86 build (no fused
multiply-add); device kernels that must match the reference bit for bit use
explicitly rounded intrinsics.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libphase_gb300.so")
SOURCES = ["host.cpp", "capi.cu", "solver.cu", "kernels.cu", "ilu.cu", "dd.cu", "batch.cu", "coarse.cu",
           "mpnn.cu", "noalloc.cu", "krylov.cu", "gcib.cu", "lu_host.cpp", "lu.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required")


def _flags(verbose_ptxas: bool):
    f = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler",
                "-fPIC,-ffp-contract=off,-O2", "-Xcudafe",
                "--diag_suppress=177"]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "phase_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not _needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = _flags(verbose_ptxas)

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        cmd = [cc, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    objs = [o for o, _ in results]
    if verbose_ptxas:
        for _, err in results:
            sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)
