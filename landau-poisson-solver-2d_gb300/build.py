"""Builds liblp_gb300.so (CUDA kernels for sm_103a + the C ABI) and the C++
drop-in test driver in-tree, under landau-poisson-solver-2d_gb300/_build/.

Usage: python landau-poisson-solver-2d_gb300/build.py [--force]
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "liblp_gb300.so")
DROPIN_TEST = os.path.join(OUT, "dropin_driver")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")


def _cuda_home() -> str:
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(INCLUDE, "lp_gb300.h")]
    for d in (CSRC, HOST):
        if os.path.isdir(d):
            hs += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh"))]
    return hs


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    cu_flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                       "-I", INCLUDE, "-I", CSRC]
    for name in ("lp_kernels.cu", "lp_api.cu", "lp_noalloc.cu", "lp_adjoint.cu", "lp_fftq.cu", "lp_fqf.cu",
                 "lp_pjtc.cu", "lp_corr.cu"):
        src = os.path.join(CSRC, name)
        obj = os.path.join(OUT, name.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([NVCC] + cu_flags + ["-c", src, "-o", obj])
    cxx_flags = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
                 "-I", os.path.join(_cuda_home(), "include")]
    src = os.path.join(CSRC, "lp_tables.cpp")
    obj = os.path.join(OUT, "lp_tables.o")
    objs.append(obj)
    if force or _stale(obj, [src] + hdrs):
        jobs.append([CXX] + cxx_flags + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=6) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
    if force or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-ldl"])
    # C++ drop-in driver (reference routine signatures over the C ABI)
    dsrc = [os.path.join(HOST, "lp_dropin.cpp"), os.path.join(HOST, "dropin_driver.cpp")]
    if all(os.path.exists(s) for s in dsrc) and (force or _stale(DROPIN_TEST, dsrc + [LIB] + hdrs)):
        _run([CXX, "-O2", "-std=c++17", "-ffp-contract=off", "-I", INCLUDE, "-I", HOST] + dsrc +
             ["-o", DROPIN_TEST, "-L" + OUT, "-llp_gb300", "-Wl,-rpath," + OUT])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
