"""Builds libagx.so (the CUDA library) in-tree with nvcc for sm_103a.

Translation units are compiled in parallel; the plain FP64 unit is compiled
with --fmad=false so that its arithmetic rounds exactly like the reference's
FP64 path.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libagx.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I" + INCLUDE, "-I" + CSRC]

# (source, extra flags)
UNITS = [
    ("agx_plain.cu", ["--fmad=false"]),
    ("agx_api.cu", ["--fmad=false"]),
    ("agx_mixed.cu", ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]),
    ("agx_noalloc.cu", ["--fmad=false"]),
    ("agx_probe.cu", []),
]

# host C++ units (g++, OpenMP): the native mesh and table builders
HOST_UNITS = [
    ("agx_mesh.cpp", []),
]
HOST_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-I" + INCLUDE, "-I" + CSRC]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libagx")
    return exe


def _sources():
    return [(os.path.join(CSRC, s), f) for s, f in UNITS if os.path.exists(os.path.join(CSRC, s))]


def _deps():
    out = []
    for fn in os.listdir(CSRC):
        if fn.endswith((".cu", ".cuh", ".h", ".cpp")):
            out.append(os.path.join(CSRC, fn))
    for fn in os.listdir(INCLUDE):
        if fn.endswith(".h"):
            out.append(os.path.join(INCLUDE, fn))
    return out


def cxx():
    exe = shutil.which("g++") or shutil.which("c++")
    if not exe:
        raise RuntimeError("g++ not found: a C++17 compiler is required to build libagx")
    return exe


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force=False, verbose=False, ptxas_info=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    exe = nvcc()
    jobs = []
    for src, flags in _sources():
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [exe] + ARCH + COMMON + flags + ["-c", src, "-o", obj]
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        jobs.append((cmd, obj))
    for name, flags in HOST_UNITS:
        src = os.path.join(CSRC, name)
        if not os.path.exists(src):
            continue
        obj = os.path.join(objdir, name + ".o")
        jobs.append(([cxx()] + HOST_FLAGS + flags + ["-c", src, "-o", obj], obj))

    def run(job):
        cmd, obj = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        for lg in logs:
            sys.stderr.write(lg)
    tmp = LIB + ".tmp"
    cmd = [exe] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", tmp] + [o for _, o in jobs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
