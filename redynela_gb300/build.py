"""Build libdnlgpu.so (sm_103a) in-tree with nvcc: one object per .cu file, compiled in parallel.

    python -m redynela_gb300.build [--force]
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libdnlgpu.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code: no contraction of a*b+c into fused multiply-adds (GCC's default on aarch64), so the
# host-side constants (material moduli, integration parameters) round as the reference's x86
# build and identically in every translation unit.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "-I" + INCLUDE, "--expt-relaxed-constexpr"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + \
        [os.path.join(INCLUDE, "dnl_gpu.h"), os.path.abspath(__file__)]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


# Element kernels: no implicit multiply-add contraction on the device either; the source writes every
# fused multiply-add it wants as fma(), so each instantiation of the shared element code rounds the
# same way whatever the inlining context.
FILE_FLAGS = {"dnl_elem.cu": ["-fmad=false"]}


def _compile(src):
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    cmd = [NVCC] + ARCH + FLAGS + FILE_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA source for sm_103a and link libdnlgpu.so; returns the library path."""
    if not force and not _stale(LIB, _deps()):
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        objs = list(ex.map(_compile, _sources()))
    cmd = [NVCC] + ARCH + ["-shared", "--cudart", "static", "-o", LIB] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
