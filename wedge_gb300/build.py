"""Build recipe of the sm_103a engine.

Compiles the CUDA translation units in ``csrc/`` (in parallel, one
``-gencode arch=compute_103a,code=sm_103a``) into ``lib/libwedge_cuda.so`` and
the C host program ``bin/wedge`` (the drop-in for the reference's ``wedge``
command line) that links it.  No cmake, no torch extension machinery: plain
``nvcc`` and ``gcc``, so the same recipe runs on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
OUT_LIB = os.path.join(PKG, "lib")
OUT_BIN = os.path.join(PKG, "bin")
OBJ = os.path.join(PKG, "_build")
LIB_NAME = "libwedge_cuda.so"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]
NVCC_FLAGS += os.environ.get("WEDGE_NVCC_EXTRA", "").split()  # tuning experiments only

CUDA_SOURCES = ["engine.cu", "graph.cu", "sched.cu", "batch.cu"]
HOST_SOURCES = ["main.c", "cmdline.c", "application.c"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def build_lib(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA engine into lib/libwedge_cuda.so and return its path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(OUT_LIB, exist_ok=True)
    hdrs = _headers()
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([NVCC] + ARCH + NVCC_FLAGS + ["-Xptxas", "-v", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(CUDA_SOURCES)) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                sys.stderr.write(r.stderr)
    lib = os.path.join(OUT_LIB, LIB_NAME)
    if force or _stale(lib, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs)
    return lib


def build_cli(force: bool = False) -> str:
    """Compile the C host program bin/wedge against the engine library."""
    os.makedirs(OUT_BIN, exist_ok=True)
    exe = os.path.join(OUT_BIN, "wedge")
    srcs = [os.path.join(HOST, f) for f in HOST_SOURCES]
    lib = os.path.join(OUT_LIB, LIB_NAME)
    deps = srcs + [lib] + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + _headers()
    if force or _stale(exe, deps):
        _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-I" + INCLUDE, "-I" + HOST] + srcs +
             ["-o", exe, "-L" + OUT_LIB, "-lwedge_cuda", "-Wl,-rpath,$ORIGIN/../lib", "-lm"])
    return exe


def build_gen(force: bool = False) -> str:
    """Compile bin/wedge-gen, the writer of the synthetic graphs in the reference's file format."""
    os.makedirs(OUT_BIN, exist_ok=True)
    exe = os.path.join(OUT_BIN, "wedge-gen")
    src = os.path.join(HOST, "gen.c")
    lib = os.path.join(OUT_LIB, LIB_NAME)
    if force or _stale(exe, [src, lib] + _headers()):
        _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-I" + INCLUDE, src, "-o", exe, "-L" + OUT_LIB, "-lwedge_cuda",
              "-Wl,-rpath,$ORIGIN/../lib"])
    return exe


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_lib(force=force, verbose=verbose)
    build_cli(force=force)
    build_gen(force=force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(os.path.join(OUT_LIB, LIB_NAME))
