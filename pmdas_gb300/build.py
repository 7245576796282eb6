"""In-tree build of libpmdas_gb300.so for sm_103a (GB300).

Each translation unit is compiled with the flags its arithmetic needs:

* ``kdgrid_fast.cu`` — ``--use_fast_math``, the reference's flags
  (SDK/CMakeLists.txt:163-180), so results match the reference's kernels;
* ``kdgrid_ieee.cu``, ``integrand.cu`` and ``order.cu`` — strict IEEE binary32 (no FMA
  contraction, IEEE division and square root, subnormals kept), so results
  match a CPU restatement bit for bit;
* host code — ``-ffp-contract=off`` so scene generation gives the same floats
  on x86-64 and aarch64 hosts.

Usage: ``python -m pmdas_gb300.build`` or ``pmdas_gb300.build.build()``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libpmdas_gb300.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "-I", CSRC, "-I", os.path.join(ROOT, "include")]
IEEE = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
FAST = ["--use_fast_math"]

UNITS = [
    ("kdgrid_fast.cu", FAST),
    ("kdgrid_ieee.cu", IEEE),
    ("integrand.cu", IEEE),
    ("capi.cu", []),
    ("noalloc.cu", FAST),
    ("order.cu", IEEE),
    ("mlp.cu", []),
]
CXX_UNITS = ["env.cpp", "image_io.cpp"]
HEADERS = ["grid_types.h", "ieee_math.h", "integrand.h", "kdgrid_kernels.cuh", "batch_kernels.cuh", "scene.h", "order.h", "mlp.h", "leaf_raw.h", "ld_hint.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpmdas_gb300")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}):\n{' '.join(cmd)}\n{r.stdout}")
    if verbose and r.stdout.strip():
        print(r.stdout, flush=True)
    return r.stdout


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every translation unit (in parallel) and link the shared library."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "mdas.h"), __file__]
    dep_time = _newest(deps)
    nv = nvcc()
    jobs = []
    objs = []
    for src, flags in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        extra = ["-Xptxas", "-v"] if ptxas_info else []
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(dep_time, os.path.getmtime(s)):
            jobs.append([nv] + ARCH + NVCC_COMMON + flags + extra + ["-c", s, "-o", o])
    for src in CXX_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(dep_time, os.path.getmtime(s)):
            jobs.append([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off",
                         "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(lambda c: _run(c, verbose), jobs))
        if ptxas_info:
            for o in outs:
                print(o)
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        _run([nv] + ARCH + ["-shared", "-o", LIB] + objs, verbose)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
