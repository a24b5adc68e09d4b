"""Builds libukgpu.so (the C-ABI library with the CUDA smoothers) in-tree.

nvcc compiles every translation unit for sm_103a only, in parallel, and links
them into ultimate_kalman_gb300/libukgpu.so.  Run directly or through
``__graft_entry__.build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libukgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["oddeven.cu", "associative.cu", "builder.cu", "filter.cu", "profiling.cu", "host_api.cpp", "matrix_ops.c"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found")


def _compile(src, verbose):
    out = os.path.join(BUILD, os.path.basename(src) + ".o")
    inc = ["-I", os.path.join(REPO, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        # --split-compile=0: nvcc optimizes the translation unit's kernels in parallel on every core
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--split-compile=0", "-Xcompiler", "-fPIC", *inc,
               "-c", src, "-o", out]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    elif src.endswith(".cpp"):
        cmd = [nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-fPIC", *inc, "-c", src, "-o", out]
    else:
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-Wall", *inc, "-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{r.stdout}\n{r.stderr}")
    return out, r.stderr


def build(verbose=False, force=False):
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    # every header of the library and of include/ is a dependency of every object
    deps = srcs + sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                         glob.glob(os.path.join(REPO, "include", "*.h")))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    objs = [o for o, _ in results]
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking libukgpu.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
