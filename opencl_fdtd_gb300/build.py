"""
Build the CUDA C-ABI library ``opencl_fdtd_gb300/_lib/libfdtd_gb300.so`` for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked with the static CUDA
runtime; the result stays in the source tree (git-ignored). ``python -m
opencl_fdtd_gb300.build`` rebuilds what is out of date.
"""
from __future__ import annotations

import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libfdtd_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"]

# Translation units and their extra flags. The Yee kernels are compiled without FMA
# contraction so that they keep the reference's rounding; the monitors as well, so that the
# DFT sample the H+S kernel takes in its own launch has the monitor kernel's bits.
UNITS = {
    "yee_kernels.cu": ["--fmad=false"],
    "step_kernel.cu": ["--fmad=false"],
    "hs_fused.cu": ["--fmad=false"],
    "batch.cu": ["--fmad=false"],
    "batch_abi.cu": [],
    "lbc.cu": [],
    "lbc_abi.cu": [],
    "monitors.cu": ["--fmad=false"],
    "noalloc.cu": [],
    "fdtd_abi.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit: str, flags, verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    if _stale(obj, [src, __file__] + _headers()):
        cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, r.stdout, r.stderr))
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, u, f + extra, verbose or ptxas_info) for u, f in UNITS.items()]
        objs = [f.result() for f in futs]
    if _stale(LIB, objs):
        tmp = LIB + ".%d.tmp" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
