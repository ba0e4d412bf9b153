"""Build recipe of libsnkpt.so (nvcc, sm_103a, in-tree).

Each .cu translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a``; the shading/ReSTIR units use
``--fmad=false`` so their binary32 arithmetic is evaluated exactly as written
(no multiply-add contraction), and host code uses ``-ffp-contract=off`` for the
same reason.  The shared library links the CUDA runtime statically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
REPO = os.path.dirname(ROOT)
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libsnkpt.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", os.path.join(REPO, "include")]
# translation units and whether they need exact (uncontracted) float arithmetic
UNITS = {
    "api.cu": True,
    "bvh_build.cu": False,
    "trace_kernels.cu": False,
    "pt_kernels.cu": True,
    "restir.cu": True,
    "noalloc.cu": False,
    "mlp_cache.cu": False,
    "taa.cu": True,
    "meshdata.cpp": False,
    "particles.cu": True,
    "scene_tables.cu": True,
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _sources():
    return [os.path.join(CSRC, u) for u in UNITS]


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(REPO, "include", "snk_pt.h")]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(x) > t for x in [src] + _headers())


def compile_unit(name: str, exact: bool, extra=()) -> str:
    src = os.path.join(CSRC, name)
    obj = os.path.join(BUILD, name + ".o")
    if _stale(obj, src):
        cmd = [nvcc(), *ARCH, *COMMON, *(["--fmad=false"] if exact else []), *extra, "-c", src, "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda kv: compile_unit(*kv), UNITS.items()))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
