"""In-tree build of ``libchimescalc.so`` for GB300 (sm_103a).

CUDA translation units go through nvcc with one ``-gencode
arch=compute_103a,code=sm_103a``; host C++ goes through g++.  Both use
``-ffp-contract=off`` on the host side so that the cell algebra rounds every
product before summing it, as the reference's x86-64 build does.  Objects
land in ``chimes_calculator_gb300/_build/`` and the library next to this file.
Only translation units whose sources (or headers) changed are recompiled.
"""

from __future__ import annotations

import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libchimescalc.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CXX_SOURCES = ["ck_params.cpp", "ck_geom.cpp", "ck_engine.cpp", "ck_capi.cpp", "ck_chimesff.cpp", "ck_server.cpp", "ck_nl.cpp"]
CU_SOURCES = ["ck_lists.cu", "ck_force.cu", "ck_factored.cu", "ck_tensor.cu", "ck_neigh.cu", "ck_direct.cu",
              "ck_noalloc.cu",
              "ck_fingerprint.cu"]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(REPO, "include", "*.h"))


def _stale(obj: str, src: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + list(headers))


def _compile(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stderr


BOUNDS_LIB = os.path.join(HERE, "libchimescalc_bounds.so")


def build(force: bool = False, verbose: bool = False, bounds: bool = False) -> str:
    """Compiles the library if needed and returns its path.  bounds=True
    builds the checked variant libchimescalc_bounds.so instead: the CUDA
    sources compiled with -DCK_BOUNDS (index checks that raise an error flag
    and skip the access), the host objects shared with the normal build."""
    if not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at %s" % NVCC)
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    inc = ["-I" + CSRC, "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(CUDA_HOME, "include")]
    jobs = []
    objs = []
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, s, headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         *inc, "-c", s, "-o", o])
    cu_dir = os.path.join(BUILD, "bounds") if bounds else BUILD
    os.makedirs(cu_dir, exist_ok=True)
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(cu_dir, src + ".o")
        objs.append(o)
        if force or _stale(o, s, headers):
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         *(["-DCK_BOUNDS"] if bounds else []), *inc, "-c", s, "-o", o])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
            for err in ex.map(_compile, jobs):
                if verbose and err.strip():
                    print(err, file=sys.stderr)
    lib = BOUNDS_LIB if bounds else LIB
    if jobs or force or not os.path.exists(lib) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in objs):
        tmp = lib + ".tmp"
        _compile([NVCC, *ARCH, "-shared", "-Xcompiler", "-pthread", "-o", tmp, *objs, "-lpthread", "-ldl", "-lrt"])
        shutil.move(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
