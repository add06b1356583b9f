"""In-tree build of libmeso_gpu.so (sm_103a) and the oracle's C library.

Usage: python meso-lts_gb300/build.py [--force]

Host C++ is compiled with -ffp-contract=off so the geometry it builds matches
the reference bit for bit on x86-64 and aarch64 alike.  The plain FP64 kernels
are compiled twice: the 2-D ones with multiply-adds contracted (their parity
gates hold at 1e-12 that way and the FP64 pipe bounds them), the 3-D ones with
-fmad=false.  Objects are rebuilt when their source or any header in the tree
is newer.
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
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
ORACLE = os.path.join(ROOT, "oracle")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SRCS = ["host/mesh.cpp", "host/config.cpp", "host/case.cpp", "host/renumber.cpp", "host/output.cpp",
             "host/tiles.cpp", "host/fp32_host.cpp", "capi.cpp", "batch.cpp", "server.cpp", "autotune.cpp"]
# (source, extra nvcc flags, object name)
CUDA_SRCS = [("kernels/plain_fp64.cu", ["-DMESO_PLAIN_DIM=2"], "plain_fp64_2d"),
             ("kernels/plain_fp64.cu", ["-DMESO_PLAIN_DIM=3", "-fmad=false"], "plain_fp64_3d"),
             ("kernels/fp32_step.cu", [], "fp32_step"),
             ("kernels/moments_noalloc.cu", ["-fmad=false"], "moments_noalloc")]

LIB = os.path.join(LIBDIR, "libmeso_gpu.so")
ORACLE_LIB = os.path.join(ORACLE, "lib", "libmeso_oracle.so")


def _newest_header() -> float:
    t = 0.0
    for d in (CSRC, INCLUDE):
        for dp, _, fs in os.walk(d):
            for f in fs:
                if f.endswith((".h", ".cuh", ".hpp")):
                    t = max(t, os.path.getmtime(os.path.join(dp, f)))
    return t


def _stale(src: str, obj: str, hdr_t: float) -> bool:
    if not os.path.exists(obj):
        return True
    ot = os.path.getmtime(obj)
    return os.path.getmtime(src) > ot or hdr_t > ot


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_library(force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    hdr_t = _newest_header()
    nvcc = os.path.join(CUDA, "bin", "nvcc")
    inc = ["-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(CUDA, "include")]
    jobs_list = []
    objs = []
    for s in HOST_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJDIR, s.replace("/", "_") + ".o")
        objs.append(obj)
        if force or _stale(src, obj, hdr_t):
            jobs_list.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                              *inc, "-c", src, "-o", obj])
    for s, extra, name in CUDA_SRCS:
        src = os.path.join(CSRC, s)
        if not os.path.exists(src):
            continue
        obj = os.path.join(OBJDIR, name + ".cu.o")
        objs.append(obj)
        if force or _stale(src, obj, hdr_t):
            jobs_list.append([nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                              "-Xcompiler", "-ffp-contract=off", *extra, *inc, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs_list))
    if jobs_list or not os.path.exists(LIB):
        _run(["g++", "-shared", "-o", LIB, *objs, "-L" + os.path.join(CUDA, "lib64"),
              "-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-lcudart", "-lpthread"])
    return LIB


APP = os.path.join(LIBDIR, "meso_gpu_run")


def build_apps(force: bool = False) -> str:
    """The C++ drop-in driver (apps/meso_gpu_run.cpp over include/meso_solver.hpp)."""
    src = os.path.join(PKG, "apps", "meso_gpu_run.cpp")
    hdr_t = max(os.path.getmtime(os.path.join(INCLUDE, "meso_solver.hpp")),
                os.path.getmtime(os.path.join(INCLUDE, "meso_gpu.h")), os.path.getmtime(LIB))
    if force or _stale(src, APP, hdr_t):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, src, "-o", APP, "-L" + LIBDIR, "-lmeso_gpu",
              "-Wl,-rpath," + LIBDIR])
    return APP


def build_oracle(force: bool = False) -> str:
    src = os.path.join(ORACLE, "meso_oracle.c")
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    hdr_t = max(os.path.getmtime(os.path.join(ORACLE, "meso_oracle.h")),
                os.path.getmtime(os.path.join(INCLUDE, "meso_gpu.h")))
    if force or _stale(src, ORACLE_LIB, hdr_t):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-I" + INCLUDE,
              src, "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def build_reference() -> bool:
    """Builds oracle/_ref/meso_ref (test infrastructure) from a reference checkout named by the
    MESO_REF_SRC environment variable; without it, or without the sources there, does nothing.
    Not part of build_all(): the product build never reaches outside the repository."""
    src = os.environ.get("MESO_REF_SRC")
    if not src or not os.path.isdir(os.path.join(src, "src")) or not shutil.which("g++"):
        return False
    _run(["bash", os.path.join(ORACLE, "build_ref.sh")])
    return True


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_library, force)
        b = ex.submit(build_oracle, force)
        a.result()
        b.result()
    build_apps(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB, ORACLE_LIB)
