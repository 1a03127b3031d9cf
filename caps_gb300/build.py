"""Builds libcaps_gb300.so and the randombenchmark / fromfile1 drivers in-tree.

nvcc for sm_103a only (-gencode arch=compute_103a,code=sm_103a), translation
units compiled in parallel.  Outputs (git-ignored):
    caps_gb300/lib/libcaps_gb300.so
    caps_gb300/bin/randombenchmark, caps_gb300/bin/fromfile1
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
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libcaps_gb300.so")

CU_SOURCES = ["engine.cu", "kernels_elementwise.cu", "kernels_dmma.cu", "kernels_split.cu", "kernels_crt.cu",
              "noalloc.cu"]
CPP_SOURCES = ["compat.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    # every translation unit is rebuilt when any shared header changes (the
    # split kernels' tile constants, wait limit and descriptors live in
    # split_common.cuh)
    headers = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h")))
    headers += [os.path.join(ROOT, "include", "caps_gb300.h"), os.path.join(ROOT, "include", "caps_compat.h")]
    nv = nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [nv] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                 "-Xcompiler", "-Wall", "-c", path, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [nv, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-x", "c++", "-c", path, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    # drivers
    inc = os.path.join(cuda_home(), "include")
    libcuda = os.path.join(cuda_home(), "lib64")
    for drv in ("randombenchmark", "fromfile1"):
        src = os.path.join(PKG, "drivers", drv + ".cpp")
        out = os.path.join(BINDIR, drv)
        if force or _stale(out, [src, LIB, os.path.join(ROOT, "include", "caps_compat.h")]):
            _run(["g++", "-O2", "-std=c++17", "-I" + inc, src, "-o", out, "-L" + LIBDIR, "-lcaps_gb300",
                  "-Wl,-rpath,$ORIGIN/../lib", "-L" + libcuda, "-lcudart"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
