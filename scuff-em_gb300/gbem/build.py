"""Build the CUDA library libgbem.so in-tree (sm_103a only).

Each translation unit is compiled in parallel; host geometry code is compiled
with FMA contraction off so its rounding matches the reference's.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, "csrc")
REPO = os.path.dirname(PKG)
OUT = os.path.join(HERE, "libgbem.so")
BUILD = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(REPO, "include")]
CUDA_UNITS = ["assemble.cu", "lu.cu", "gemm_tc.cu", "capi.cu", "fippi_cache.cu", "sptrf.cu"]
CXX_UNITS = ["geometry.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for u in CUDA_UNITS:
        jobs.append([nvcc] + ARCH + NVFLAGS + ["-c", os.path.join(CSRC, u), "-o", os.path.join(BUILD, u + ".o")])
    for u in CXX_UNITS:
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + os.path.join(REPO, "include"),
                     "-I/usr/local/cuda/include", "-c", os.path.join(CSRC, u), "-o", os.path.join(BUILD, u + ".o")])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            if lg.strip():
                print(lg)
    objs = [os.path.join(BUILD, u + ".o") for u in CUDA_UNITS + CXX_UNITS]
    tmp = OUT + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True))
