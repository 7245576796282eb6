"""Build recipe for the test oracle (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles the CPU restatement ``oracle/mdas_oracle.cpp``
  into ``oracle/_build/liboracle.so`` (g++, -ffp-contract=off, OpenMP).
* ``prepare_ref_sources()`` — only where the reference checkout exists
  (``$MDAS_REFERENCE_ROOT``, else a checkout named ``reference`` beside this
  repository) — copies the reference's MDAS sources and the headers
  they include into ``oracle/_ref/src`` and applies four mechanical edits
  that CUDA 13 needs (texture references were removed in CUDA 12; the
  reference also relies on an MSVC leniency for a missing ``typename``):

    1. ``texture<float4, 1> t_nodes;``  ->  ``__device__ const float4* t_nodes;``
    2. ``tex1Dfetch(t_nodes, i)``       ->  ``__ldg(t_nodes + i)``
    3. ``KDGrid<Point>::Node* nodes,`` ->  ``typename KDGrid<Point>::Node* nodes,``
    4. ``cudaBindTexture(0, &t_nodes, nodes.Data(), ...)`` -> ``cudaMemcpyToSymbol``
       of the node pointer.

  ``optix_types.h`` is replaced by a stub holding the one constant the sampler
  uses (OPTIX_ACCEL_BUFFER_BYTE_ALIGNMENT = 128).  Everything lands in the
  git-ignored ``oracle/_ref``; no reference source is committed.
* ``build_ref()`` compiles ``oracle/ref_harness.cu`` against those sources with
  the reference's flags (``--use_fast_math -lineinfo``, arch raised to sm_103a)
  into ``oracle/_ref/libmdas_ref.so``.  It runs wherever ``oracle/_ref/src``
  exists, so the prepared sources can be compiled on a machine without the
  reference checkout.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
ORACLE_LIB = os.path.join(BUILD, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SRC = os.path.join(REF_DIR, "src")
REF_LIB = os.path.join(REF_DIR, "libmdas_ref.so")
# the reference checkout: $MDAS_REFERENCE_ROOT, else ../reference relative to the repository
REFERENCE = os.environ.get("MDAS_REFERENCE_ROOT") or os.path.normpath(os.path.join(ROOT, os.pardir, "reference"))

# (path in the reference checkout, path under oracle/_ref/src)
REF_FILES = [
    ("SDK/lib/mdas/kdgrid.cu", "mdas/kdgrid.cu"),
    ("SDK/lib/mdas/kdgrid.h", "mdas/kdgrid.h"),
    ("SDK/lib/mdas/aabb.h", "mdas/aabb.h"),
    ("SDK/lib/mdas/point.h", "mdas/point.h"),
    ("SDK/lib/mdas/buffer.h", "mdas/buffer.h"),
    ("SDK/sutil/vec_math.h", "sutil/vec_math.h"),
    ("SDK/sutil/Preprocessor.h", "sutil/Preprocessor.h"),
    ("SDK/cuda/helpers.h", "cuda/helpers.h"),
    ("SDK/cuda/random.h", "cuda/random.h"),
]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}")
    return r.stdout


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "mdas_oracle.cpp")
    deps = [src, os.path.join(ROOT, "pmdas_gb300", "csrc", "ieee_math.h"),
            os.path.join(ROOT, "pmdas_gb300", "csrc", "integrand.h")]
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < max(map(os.path.getmtime, deps)):
        _run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
              "-fopenmp", src, "-o", ORACLE_LIB])
    return ORACLE_LIB


def _patch_kdgrid(text: str) -> str:
    text = text.replace("\r\n", "\n")
    text, n1 = re.subn(r"texture<float4,\s*1>\s*t_nodes;", "__device__ const float4* t_nodes;", text)
    text, n2 = re.subn(r"tex1Dfetch\(t_nodes,\s*nodeIndex\)", "__ldg(t_nodes + nodeIndex)", text)
    text, n3 = re.subn(r"(?<!typename )KDGrid<Point>::Node\* nodes,", "typename KDGrid<Point>::Node* nodes,", text)
    text, n4 = re.subn(
        r"CUDA_CHECK\(cudaBindTexture\(0, &t_nodes, nodes\.Data\(\), &desc, sizeof\(KDGrid::Node\) \* numberOfNodes\)\);",
        "{ const float4* nodesPtr_ = (const float4*)nodes.Data(); "
        "CUDA_CHECK(cudaMemcpyToSymbol(t_nodes, &nodesPtr_, sizeof(nodesPtr_))); }",
        text)
    if (n1, n2 >= 3, n3 >= 2, n4) != (1, True, True, 2):
        raise RuntimeError(f"unexpected reference source: edits applied {n1}, {n2}, {n3}, {n4}")
    return text


def prepare_ref_sources() -> bool:
    """Copy + patch the reference's sampler sources into oracle/_ref/src.  False if absent."""
    if not os.path.isdir(os.path.join(REFERENCE, "SDK", "lib", "mdas")):
        return False
    for rel, dst in REF_FILES:
        s = os.path.join(REFERENCE, rel)
        d = os.path.join(REF_SRC, dst)
        os.makedirs(os.path.dirname(d), exist_ok=True)
        with open(s, "r", encoding="utf-8", errors="replace") as f:
            text = f.read()
        if dst == "mdas/kdgrid.cu":
            text = _patch_kdgrid(text)
        with open(d, "w") as f:
            f.write(text)
    with open(os.path.join(REF_SRC, "optix_types.h"), "w") as f:
        f.write("#pragma once\n#define OPTIX_ACCEL_BUFFER_BYTE_ALIGNMENT 128ull\n")
    return True


def build_ref(force: bool = False) -> str | None:
    """Compile the reference harness; None when the prepared sources are absent."""
    kd = os.path.join(REF_SRC, "mdas", "kdgrid.cu")
    if not os.path.exists(kd):
        return None
    harness = os.path.join(HERE, "ref_harness.cu")
    deps = [harness] + [os.path.join(REF_SRC, d) for _, d in REF_FILES]
    if force or not os.path.exists(REF_LIB) or os.path.getmtime(REF_LIB) < max(map(os.path.getmtime, deps)):
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        _run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "--use_fast_math", "-lineinfo", "-O3",
              "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-w",
              "-I", REF_SRC, "-I", os.path.join(REF_SRC, "mdas"), harness, "-o", REF_LIB])
    return REF_LIB


def build_all(force: bool = False):
    build_oracle(force)
    prepare_ref_sources()
    return build_ref(force)


if __name__ == "__main__":
    print(build_oracle("--force" in sys.argv))
    print(prepare_ref_sources())
    print(build_ref("--force" in sys.argv))
