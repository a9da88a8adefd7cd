"""Builds libpa_gb300.so in-tree with nvcc for sm_103a (no torch, no cmake).

    python -m privacyamplification_gb300.build [--force]

Translation units are compiled in parallel, then linked into one shared library next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpa_gb300.so")
SOURCES = ["pa_kernels.cu", "pa_passes.cu", "pa_lanes.cu", "pa_ntt.cu", "pa_chunk.cu", "pa_engine.cu", "pa_batch.cu",
           "pa_noalloc.cu", "pa_selftest.cu", "pa_dft_tc.cu", "pa_group.cu", "pa_fused.cu"]
HOST_SOURCES = ["pa_sha3.cpp", "pa_config.cpp", "pa_zmtp.cpp", "pa_service.cpp"]  # plain C++, no CUDA
SERVICE_MAIN = "pa_service_main.cpp"
SERVICE = os.path.join(HERE, "pa_service")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall"]
HEADERS = ["pa_device.cuh", "pa_fft.cuh", "pa_tma.cuh", "pa_kernels.cuh", "pa_pass_bodies.cuh", "pa_lanes.cuh", "pa_engine_impl.h",
           os.path.join("..", "..", "include", "pa_gb300.h"), os.path.join("..", "..", "include", "pa_service.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpa_gb300.so")


def cxx() -> str:
    for c in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("g++ not found: a C++17 compiler is required for the host loop")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.normpath(os.path.join(CSRC, h)) for h in HEADERS]
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([cxx(), *CXX_FLAGS, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    main = os.path.join(CSRC, SERVICE_MAIN)
    if force or _stale(SERVICE, [LIB, main] + hdrs):
        cmd = [cxx(), "-O2", "-std=c++17", main, "-o", SERVICE, "-L" + HERE, "-lpa_gb300", "-Wl,-rpath,$ORIGIN",
               "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("pa_service link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
