"""Builds the in-tree shared library getfem_gb300/libgfgpu.so for sm_103a.

Host C++ sources are compiled with g++, CUDA sources with nvcc
(-gencode arch=compute_103a,code=sm_103a), all in parallel, then linked
with nvcc -shared.  No cmake, no torch extension machinery.
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
LIB = os.path.join(HERE, "libgfgpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

HOST_SOURCES = ["host/refelem.cc", "gfgpu_host.cc"]
CUDA_SOURCES = ["gfgpu_api.cu", "k_simplex.cu", "k_simplex_ten.cu", "k_assemble.cu",
                "k_probe.cu", "k_noalloc.cu", "k_hex.cu", "k_gauss.cu", "k_affine_hex.cu",
                "k_solve.cu", "k_dofs.cu"]
# per-file nvcc flags: the Gauss-point kernels round like the reference's
# sequence of products and sums (no implicit contraction; explicit fma only)
CUDA_FLAGS = {"k_hex.cu": ["-fmad=false"], "k_gauss.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(obj: str, srcs: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = []
    for root, _, files in os.walk(CSRC):
        headers += [os.path.join(root, f) for f in files if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "gfgpu.h"))
    jobs = []
    objs = []
    for s in HOST_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace("/", "_") + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-ffp-contract=off", "-c", src,
                         "-o", obj])
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace("/", "_") + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off"] + CUDA_FLAGS.get(s, []) +
                        ["-Xptxas", "-v" if verbose else "-O3", "-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if jobs or not os.path.exists(LIB):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
