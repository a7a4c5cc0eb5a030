"""Compiles libewt.so (the CUDA kernels + C ABI) for sm_103a with nvcc.

Translation units compile in parallel, then one nvcc link produces
``ecl_wavelet_gb300/libewt.so`` in-tree.  Rebuilds only when a source or
header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
OBJ_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libewt.so")
SCHED_LIB = os.path.join(PKG, "libewt_sched.so")  # CUDA-free scheduler core

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
              "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin",
                        "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu"))
                  + glob.glob(os.path.join(CSRC, "*.cpp")))


def headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(INCLUDE, "**", "*.h*"), recursive=True))


def _stale(target, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra) -> str:
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    if _stale(obj, [src] + headers()):
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + list(extra) + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (
                src, " ".join(cmd), r.stderr[-6000:]))
    return obj


def build(verbose: bool = False, extra_flags=()) -> str:
    """Builds libewt.so if stale; returns its path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra_flags), srcs))
    if _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc link failed:\n%s\n%s" % (" ".join(cmd),
                                                            r.stderr[-4000:]))
        os.replace(tmp, LIB)
    build_sched()
    if verbose:
        print("built", LIB)
    return LIB


def build_sched() -> str:
    """Builds libewt_sched.so (the serving scheduler core, no CUDA) with the
    host C++ compiler, so its tests run on hosts without a GPU or nvcc."""
    src = os.path.join(CSRC, "sched_capi.cpp")
    deps = [src, os.path.join(CSRC, "serve_sched.h"), os.path.join(INCLUDE, "ewt_sched.h")]
    if _stale(SCHED_LIB, deps):
        tmp = SCHED_LIB + ".tmp%d" % os.getpid()
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared",
               "-I", INCLUDE, "-I", CSRC, src, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("g++ failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
        os.replace(tmp, SCHED_LIB)
    return SCHED_LIB


if __name__ == "__main__":
    build(verbose=True, extra_flags=sys.argv[1:])
