"""GPU baselines: the reference's plain single-block cuFFT pipeline and its sub-block bank (batched cuFFT
plans over equal sub-blocks), both in cufft_plain.cu, built and bound here.

    python -m baseline.cufft_plain          # build libcufft_plain.so in-tree

Not part of the engine: `bench.py` times it beside the engine on the same inputs and the GPU tests
compare its output bits with the engine's and the oracle's.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cufft_plain.cu")
LIB = os.path.join(HERE, "libcufft_plain.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    from privacyamplification_gb300.build import ARCH, nvcc
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-shared", "-Xcompiler", "-fPIC", "-Xcompiler",
           "-fvisibility=hidden", SRC, "-o", LIB, "-lcufft"]
    subprocess.run(cmd, check=True)
    return LIB


class CufftPlain:
    """One (n, v) pipeline with its own device buffers, cuFFT plans and pinned host slots."""

    def __init__(self, n: int, v: int):
        if not os.path.exists(LIB):
            raise RuntimeError("%s not built: run `python -m baseline.cufft_plain`" % LIB)
        lib = ctypes.CDLL(LIB)
        vp, u32p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)
        lib.cp_create.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(vp)]
        lib.cp_create.restype = ctypes.c_int
        lib.cp_destroy.argtypes = [vp]
        lib.cp_destroy.restype = None
        for name in ("cp_seed_slot", "cp_key_start_slot", "cp_key_rest_slot", "cp_output_slot"):
            getattr(lib, name).argtypes = [vp]
            getattr(lib, name).restype = vp
        lib.cp_process.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.cp_process.restype = ctypes.c_int
        lib.cp_residual.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]
        lib.cp_residual.restype = ctypes.c_int
        lib.cp_step_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        lib.cp_step_ms.restype = None
        lib.cp_load_reference.argtypes = [ctypes.c_char_p, ctypes.c_uint32]
        lib.cp_load_reference.restype = ctypes.c_int
        lib.cp_unload_reference.argtypes = []
        lib.cp_unload_reference.restype = None
        self._lib, self.n, self.v = lib, n, v
        h = vp()
        rc = lib.cp_create(n, v, ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("cp_create(%d, %d) failed: %d" % (n, v, rc))
        self._h = h
        words = n // 32

        def view(ptr, count, dtype):
            return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_uint32)), (count,)).view(dtype)

        self.seed = view(lib.cp_seed_slot(h), words, np.uint32)
        self.key_start = view(lib.cp_key_start_slot(h), words, np.uint32)
        self.key_rest = view(lib.cp_key_rest_slot(h), words + 31, np.uint32)
        self.out = view(lib.cp_output_slot(h), words + 31, np.uint32).view(np.uint8)

    def load(self, seed=None, key_start=None, key_rest=None):
        """Copies inputs into the pinned slots (outside any timed region)."""
        if seed is not None:
            self.seed[:] = np.asarray(seed, np.uint32)[: self.seed.size]
        if key_start is not None:
            ks = np.asarray(key_start, np.uint32)
            self.key_start[:] = 0
            self.key_start[: ks.size] = ks
        if key_rest is not None:
            kr = np.asarray(key_rest, np.uint32)
            self.key_rest[:] = 0
            self.key_rest[: kr.size] = kr

    def use_reference_kernels(self, fatbin: str):
        """From now on (for every pipeline in this process) launch the reference's own kernels, compiled
        from PrivacyAmplification.cu (baseline/ref_cuda.py), with their constants for this n."""
        rc = self._lib.cp_load_reference(fatbin.encode(), self.n)
        if rc != 0:
            raise RuntimeError("cp_load_reference(%s) failed: %d" % (fatbin, rc))

    def use_restated_kernels(self):
        self._lib.cp_unload_reference()

    def process(self, recalc_seed: bool, do_xor: bool = True, do_compress: bool = True) -> float:
        """Runs one block; returns its host wall time in ms."""
        ms = ctypes.c_double()
        rc = self._lib.cp_process(self._h, int(recalc_seed), int(do_xor), int(do_compress), ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError("cp_process failed: %d" % rc)
        return ms.value

    STEPS = ("unpack_seed", "unpack_key", "correction", "r2c_key", "r2c_seed", "zero_dc_product", "c2r", "pack")

    def step_ms(self) -> dict:
        """Host wall ms of each step of the last block (every step ends in a host sync)."""
        ms = (ctypes.c_double * 8)()
        self._lib.cp_step_ms(self._h, ms)
        return {k: ms[i] for i, k in enumerate(self.STEPS)}

    def output(self, nbytes: int) -> np.ndarray:
        return self.out[:nbytes].copy()

    def residual(self, out_bits: int) -> float:
        r = ctypes.c_float()
        rc = self._lib.cp_residual(self._h, out_bits, ctypes.byref(r))
        if rc != 0:
            raise RuntimeError("cp_residual failed: %d" % rc)
        return r.value

    def close(self):
        if self._h:
            self._lib.cp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CufftBank:
    """The sub-block bank (cb_*): B equal sub-blocks of s bits, one batched cuFFT plan per direction, device
    inputs, device-timed."""

    def __init__(self, s: int, v: int, B: int):
        if not os.path.exists(LIB):
            raise RuntimeError("%s not built: run `python -m baseline.cufft_plain`" % LIB)
        lib = ctypes.CDLL(LIB)
        vp, u32p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)
        lib.cb_create.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(vp)]
        lib.cb_create.restype = ctypes.c_int
        lib.cb_destroy.argtypes = [vp]
        lib.cb_destroy.restype = None
        lib.cb_load.argtypes = [vp, u32p, u32p, u32p]
        lib.cb_load.restype = ctypes.c_int
        lib.cb_run.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        lib.cb_run.restype = ctypes.c_int
        lib.cb_output.argtypes = [vp, u32p]
        lib.cb_output.restype = ctypes.c_int
        self._lib, self.s, self.v, self.B = lib, s, v, B
        h = vp()
        rc = lib.cb_create(s, v, B, ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("cb_create(%d, %d, %d) failed: %d" % (s, v, B, rc))
        self._h = h

    @staticmethod
    def _ptr(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, np.uint32)
        return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))

    def load(self, seed=None, key_start=None, key_rest=None):
        """seed, key_start: (B, s/32) words; key_rest: (B, v/32) words (None: keep)."""
        keep = [self._ptr(x) for x in (seed, key_start, key_rest)]
        rc = self._lib.cb_load(self._h, *[k[1] if k else None for k in keep])
        if rc != 0:
            raise RuntimeError("cb_load failed: %d" % rc)

    def run(self, recalc_seed: bool, do_xor: bool = True) -> float:
        """One bank; returns its device time in ms."""
        ms = ctypes.c_float()
        rc = self._lib.cb_run(self._h, int(recalc_seed), int(do_xor), ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError("cb_run failed: %d" % rc)
        return ms.value

    def outputs(self) -> np.ndarray:
        """(B, v/8) output bytes."""
        out = np.empty(self.B * self.v // 32, np.uint32)
        rc = self._lib.cb_output(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        if rc != 0:
            raise RuntimeError("cb_output failed: %d" % rc)
        return out.view(np.uint8).reshape(self.B, self.v // 8)

    def close(self):
        if self._h:
            self._lib.cb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
