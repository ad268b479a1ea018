"""Builds the engine's shared library in-tree: klampt_gb300/_lib/libkgpu.so.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked with
nvcc into one shared library exporting the C ABI of include/kgpu.h.  Host code
that touches FP64 geometry is compiled with ``-ffp-contract=off`` so that the
canonical arithmetic of include/kgpu_exact.h is never fused.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libkgpu.so")

CU_SOURCES = ["kgpu_api.cu", "kgpu_collide.cu", "kgpu_plain.cu", "kgpu_dist.cu", "kgpu_noalloc.cu", "kgpu_ray.cu", "kgpu_ik.cu",
              "kgpu_lbvh.cu", "kgpu_geom.cu"]
CPP_SOURCES = ["bvh.cpp"]
HEADERS = ["kgpu_internal.h", "kgpu_device.cuh", "kgpu_dist32.cuh"]
INCLUDE_HEADERS = ["kgpu.h", "kgpu_exact.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest_input() -> float:
    paths = [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES + HEADERS]
    paths += [os.path.join(ROOT, "include", f) for f in INCLUDE_HEADERS]
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def needs_build() -> bool:
    return not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest_input()


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    """Compiles and links libkgpu.so if any input is newer; returns its path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    common += list(extra_flags or [])
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(OBJ_DIR, src + ".o")
        jobs.append([nv, *ARCH, *common, "-Xptxas", "-warn-spills" if not verbose else "-v", "-c",
                     os.path.join(CSRC, src), "-o", obj])
    for src in CPP_SOURCES:
        obj = os.path.join(OBJ_DIR, src + ".o")
        jobs.append([nv, *common, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        results = list(ex.map(run, jobs))
    for cmd, r in results:
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    objs = [os.path.join(OBJ_DIR, s + ".o") for s in CU_SOURCES + CPP_SOURCES]
    tmp = LIB + ".tmp"
    link = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: " + " ".join(link) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
