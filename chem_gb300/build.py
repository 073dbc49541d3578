"""Compile the native parts in-tree (no CMake): the CUDA engine libgbjk.so
for sm_103a and the host integral engine libgbints.so.  Both compile in
parallel; a library is rebuilt only when one of its sources is newer."""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIBDIR = os.path.join(PKG, "lib")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build failed: " + " ".join(cmd))
    return r.stdout + r.stderr


def build_gbjk(force=False, verbose=False):
    out = os.path.join(LIBDIR, "libgbjk.so")
    srcs = glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "gbjk*.h"))
    if force or _stale(out, srcs):
        cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
               "-I" + INCLUDE, os.path.join(CSRC, "gbjk.cu"), "-o", out]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        log = _run(cmd)
        if verbose:
            print(log)
    return out


def build_gbints(force=False):
    out = os.path.join(LIBDIR, "libgbints.so")
    d = os.path.join(CSRC, "ints")
    srcs = glob.glob(os.path.join(d, "*.cpp")) + glob.glob(os.path.join(d, "*.hpp")) + \
        [os.path.join(INCLUDE, "gbints.h")]
    if force or _stale(out, srcs):
        _run(["g++", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c++17", "-I" + INCLUDE,
              os.path.join(d, "md_engine.cpp"), os.path.join(d, "gbints.cpp"), "-o", out])
    return out


def build_all(force=False):
    os.makedirs(LIBDIR, exist_ok=True)
    with ThreadPoolExecutor(2) as ex:
        fs = [ex.submit(build_gbjk, force), ex.submit(build_gbints, force)]
        return [f.result() for f in fs]


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
