"""Build libhmec_gpu.so in-tree with nvcc for sm_103a (GB300).

Each translation unit under csrc/ is compiled in parallel to an object file,
then linked into one shared library.  Host code is portable C++17 (the same
sources build on x86-64 and aarch64 hosts).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.path.dirname(PKG), "csrc")
INC = os.path.join(os.path.dirname(os.path.dirname(PKG)), "include")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libhmec_gpu.so")
UNITS = ["hmec_api.cu", "hmec_graph.cu", "hmec_tune.cu", "k_p2g.cu", "k_iter.cu", "k_solver.cu", "k_advect.cu", "k_p2g_static.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the GPU library cannot be built")
    return cand


def _flags(extra=()):
    # host code: no fused multiply-add (GCC fuses by default on aarch64), so the
    # host-side grid coordinates are the same IEEE values on every host
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "-I", INC, "-I", SRC] + list(extra)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(SRC, "hmec_internal.cuh"), os.path.join(SRC, "hmec_sort.cuh"),
               os.path.join(SRC, "hmec_bits.cuh"), os.path.join(SRC, "hmec_dfexp.cuh"),
               os.path.join(SRC, "hmec_mprop.cuh"), os.path.join(INC, "hmec.h")]
    objs = []
    jobs = []
    for u in UNITS:
        src = os.path.join(SRC, u)
        obj = os.path.join(OUT_DIR, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc()] + _flags(extra_flags) + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, res):
            if verbose or r.returncode != 0:
                print(" ".join(cmd))
                print(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for %s" % cmd[-3])
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".%d.tmp" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stdout + r.stderr)
            raise RuntimeError("link of libhmec_gpu.so failed")
        os.replace(tmp, LIB)
    build_driver(force)
    return LIB


DRIVER_SRC = os.path.join(os.path.dirname(PKG), "driver", "hmec_run.cpp")
DRIVER = os.path.join(OUT_DIR, "hmec_run")


def build_driver(force: bool = False) -> str:
    """The C++ host loop mirroring the reference's main(), linked to the library."""
    deps = [DRIVER_SRC, os.path.join(os.path.dirname(DRIVER_SRC), "checkpoint.hpp"), LIB, os.path.join(INC, "hmec.h")]
    if not force and not _stale(DRIVER, deps):
        return DRIVER
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", INC, DRIVER_SRC, "-o", DRIVER + ".tmp",
           "-L", OUT_DIR, "-lhmec_gpu", "-Wl,-rpath," + OUT_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print(" ".join(cmd))
        print(r.stdout + r.stderr)
        raise RuntimeError("build of hmec_run failed")
    os.replace(DRIVER + ".tmp", DRIVER)
    return DRIVER


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True))
