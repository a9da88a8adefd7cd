"""GB300 privacy-amplification engine: Python binding of the C ABI in include/pa_gb300.h.

The compute path is libpa_gb300.so (hand-written sm_103a kernels, built in-tree by
``privacyamplification_gb300.build``).  There is no CPU fallback: if the library is missing or cannot
be loaded, every entry point raises.

Typical use (the per-block body of the reference host loop, PrivacyAmplification.cu:1686-2118)::

    eng = Engine(max_sample_size=1 << 27)
    eng.set_seed(seed_words, n, reuse_seed_amount=-1)
    key_start, key_rest = key_split(recv_key, n, v)
    out = eng.process(key_start, key_rest, n, v)          # v/8 bytes, reference byte order
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpa_gb300.so")

PA_OK = 0
PA_ERR_INVALID_ARG = -1
PA_ERR_CUDA = -2
PA_ERR_NO_SEED = -3
PA_ERR_TOO_LARGE = -4
PA_ERR_PRECISION = -5
PA_ERR_BUSY = -6
PA_PENDING = 1
BATCH_GRAPH = 1
BATCH_SERIAL = 2
BATCH_PERSISTENT = 4
BATCH_NO_GROUP = 8
FLAG_XOR_KEY_REST = 1
FLAG_COMPRESS = 2
FLAG_EXACT = 4
DEFAULT_FLAGS = FLAG_XOR_KEY_REST | FLAG_COMPRESS

# Every symbol include/pa_gb300.h declares.
EXPORTS = ("pa_create", "pa_destroy", "pa_set_seed", "pa_process", "pa_set_seed_device", "pa_process_device",
           "pa_sync", "pa_key_split", "pa_output_bytes", "pa_kernels_per_block", "pa_set_timing",
           "pa_stage_times", "pa_error_string", "pa_last_cuda_error", "pa_process_noalloc", "pa_set_pool",
           "pa_seed_cache_add", "pa_seed_cache_clear", "pa_batch_run", "pa_batch_sync", "pa_submit", "pa_poll",
           "pa_set_split", "pa_get_split", "pa_autotune", "pa_pool_reserve", "pa_selftest_wait_timeout",
           "pa_set_lanes", "pa_serve_start", "pa_serve_submit", "pa_serve_poll", "pa_serve_stop", "pa_dft16_stages",
           "pa_set_groups")


class PAError(RuntimeError):
    def __init__(self, code: int, what: str, cuda: int = 0):
        msg = "%s failed: %s (%d)" % (what, error_string(code), code)
        if cuda:
            msg += ", cudaError %d" % cuda
        super().__init__(msg)
        self.code = code
        self.cuda = cuda


class PAConfig(ctypes.Structure):
    _fields_ = [("device_id", ctypes.c_int32), ("max_sample_size", ctypes.c_uint32),
                ("reduction_exp", ctypes.c_uint32), ("pre_mul_reduction_exp", ctypes.c_uint32),
                ("residual_limit", ctypes.c_float)]


class PAStats(ctypes.Structure):
    _fields_ = [("max_residual", ctypes.c_float), ("popcount_key", ctypes.c_uint64),
                ("popcount_seed", ctypes.c_uint64), ("gpu_ms", ctypes.c_float),
                ("seed_uses_left", ctypes.c_int32), ("exact", ctypes.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class PAJob(ctypes.Structure):
    """pa_job: one block of a batch (device pointers) or a served request (host pointers)."""
    _fields_ = [("seed_words", ctypes.c_void_p), ("seed_id", ctypes.c_int32), ("key_start", ctypes.c_void_p),
                ("key_rest", ctypes.c_void_p), ("n", ctypes.c_uint32), ("v", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("out", ctypes.c_void_p)]


_lib = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libpa_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("%s not found: build it with `python -m privacyamplification_gb300.build`" % path)
    lib = ctypes.CDLL(path)
    u32p, u8p, vp = ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint8), ctypes.c_void_p
    eng = ctypes.c_void_p
    sig = {
        "pa_create": ([ctypes.POINTER(PAConfig), ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
        "pa_destroy": ([eng], None),
        "pa_set_seed": ([eng, u32p, ctypes.c_uint32, ctypes.c_int32], ctypes.c_int),
        "pa_process": ([eng, u32p, u32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, u8p,
                        ctypes.POINTER(PAStats)], ctypes.c_int),
        "pa_set_seed_device": ([eng, vp, ctypes.c_uint32, ctypes.c_int32, vp], ctypes.c_int),
        "pa_process_device": ([eng, vp, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, vp, vp],
                              ctypes.c_int),
        "pa_sync": ([eng, ctypes.POINTER(PAStats)], ctypes.c_int),
        "pa_key_split": ([u32p, ctypes.c_uint32, ctypes.c_uint32, u32p, u32p], ctypes.c_int),
        "pa_output_bytes": ([ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_size_t),
        "pa_kernels_per_block": ([ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
        "pa_set_timing": ([eng, ctypes.c_int], ctypes.c_int),
        "pa_stage_times": ([eng, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                            ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "pa_error_string": ([ctypes.c_int], ctypes.c_char_p),
        "pa_last_cuda_error": ([eng], ctypes.c_int),
        "pa_process_noalloc": ([vp, vp, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, vp, vp], ctypes.c_int),
        "pa_set_pool": ([eng, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
        "pa_seed_cache_add": ([eng, u32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                               ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
        "pa_seed_cache_clear": ([eng], ctypes.c_int),
        "pa_batch_run": ([eng, ctypes.POINTER(PAJob), ctypes.c_uint32, ctypes.c_uint32, vp], ctypes.c_int),
        "pa_batch_sync": ([eng, ctypes.POINTER(PAStats), ctypes.c_uint32], ctypes.c_int),
        "pa_submit": ([eng, ctypes.POINTER(PAJob), ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
        "pa_poll": ([eng, ctypes.c_uint64, ctypes.POINTER(PAStats)], ctypes.c_int),
        "pa_set_split": ([eng, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
        "pa_get_split": ([eng, ctypes.c_uint32], ctypes.c_int),
        "pa_autotune": ([eng, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
        "pa_pool_reserve": ([eng, ctypes.c_uint32, ctypes.c_int32], ctypes.c_int),
        "pa_set_lanes": ([eng, ctypes.c_int32, ctypes.c_uint32], ctypes.c_int),
        "pa_set_groups": ([eng, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
        "pa_serve_start": ([eng, ctypes.c_int32, ctypes.c_uint32, ctypes.c_int32], ctypes.c_int),
        "pa_serve_submit": ([eng, ctypes.POINTER(PAJob), ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
        "pa_serve_poll": ([eng, ctypes.c_uint64, ctypes.POINTER(PAStats)], ctypes.c_int),
        "pa_serve_stop": ([eng], ctypes.c_int),
        "pa_selftest_wait_timeout": ([ctypes.c_int32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
        "pa_dft16_stages": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32,
                             ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def error_string(code: int) -> str:
    return load_library().pa_error_string(code).decode()


def output_bytes(n: int, v: int, flags: int = DEFAULT_FLAGS) -> int:
    return int(load_library().pa_output_bytes(n, v, flags))


def kernels_per_block(n: int, v: int, flags: int = DEFAULT_FLAGS) -> int:
    return int(load_library().pa_kernels_per_block(n, v, flags))


def process_noalloc(d_seed: int, d_key_start: int, d_key_rest: int, n: int, v: int, d_out: int,
                    flags: int = DEFAULT_FLAGS, stream: int = 0):
    """pa_process_noalloc: one block (n <= 2^15) with its own seed, device pointers only, no engine and no
    device allocation; queued on `stream`, returns without synchronising."""
    rc = load_library().pa_process_noalloc(d_seed, d_key_start, d_key_rest or None, n, v, flags, d_out,
                                           stream or None)
    if rc != 0:
        raise PAError(rc, "pa_process_noalloc")


DFT16_FP32, DFT16_TC_SPLIT, DFT16_TC_TF32 = 0, 1, 2


def dft16_stages(d_in: int, d_out: int, butterflies: int, reps: int, method: int, d_err: int,
                 ctas_per_sm: int = 4, stream: int = 0):
    """pa_dft16_stages: `reps` radix-16 DFT stages on device data by FP32 butterflies (DFT16_FP32) or on
    the tensor cores (DFT16_TC_SPLIT, FP32-level accuracy; DFT16_TC_TF32, one TF32 product); queued on
    `stream`, not synchronised."""
    rc = load_library().pa_dft16_stages(d_in, d_out, butterflies, reps, method, ctas_per_sm, d_err, stream or None)
    if rc != 0:
        raise PAError(rc, "pa_dft16_stages")


def selftest_wait_timeout(device_id: int = 0, rounds: int = 4096) -> int:
    """Runs a bounded device wait that is never satisfied; returns the device error word (1 = expired)."""
    st = ctypes.c_int32()
    rc = load_library().pa_selftest_wait_timeout(device_id, rounds, ctypes.byref(st))
    if rc != 0:
        raise PAError(rc, "pa_selftest_wait_timeout")
    return st.value


def _u32(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a


def _p32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def key_split(recv_key, n: int, v: int):
    """key2StartRest (PrivacyAmplification.cu:861-892) through the C ABI.
    Returns (key_start[n/32], key_rest[v/32])."""
    rk = _u32(recv_key)
    if rk.size < n // 32 + 1:
        raise ValueError("recv_key needs n/32+1 words")
    ks = np.zeros(n // 32, np.uint32)
    kr = np.zeros(v // 32, np.uint32)
    rc = load_library().pa_key_split(_p32(rk), n, v, _p32(ks), _p32(kr))
    if rc:
        raise PAError(rc, "pa_key_split")
    return ks, kr


class Engine:
    """One GPU's privacy-amplification engine (pa_create / pa_destroy)."""

    def __init__(self, max_sample_size: int, device_id: int = 0, residual_limit: float = 0.25,
                 reduction_exp: int = 11, pre_mul_reduction_exp: int = 5):
        self._lib = load_library()
        cfg = PAConfig(device_id, max_sample_size, reduction_exp, pre_mul_reduction_exp, residual_limit)
        h = ctypes.c_void_p()
        rc = self._lib.pa_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc:
            raise PAError(rc, "pa_create")
        self._h = h
        self.max_sample_size = max_sample_size
        self.last_stats = PAStats()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pa_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, what):
        if rc:
            raise PAError(rc, what, self._lib.pa_last_cuda_error(self._h))

    def set_seed(self, seed_words, n: int, reuse_seed_amount: int = -1):
        s = _u32(seed_words)
        if s.size < n // 32:
            raise ValueError("seed needs n/32 words")
        self._check(self._lib.pa_set_seed(self._h, _p32(s), n, reuse_seed_amount), "pa_set_seed")

    def process(self, key_start, key_rest, n: int, v: int, flags: int = DEFAULT_FLAGS,
                check: bool = True, out: np.ndarray = None) -> np.ndarray:
        ks = _u32(key_start)
        if ks.size < (n - v) // 32 + 1:
            raise ValueError("key_start needs h/32+1 words")
        kr = _u32(key_rest) if key_rest is not None else None
        if flags & FLAG_XOR_KEY_REST and (kr is None or kr.size < v // 32):
            raise ValueError("key_rest needs v/32 words")
        nb = output_bytes(n, v, flags)
        if out is None:
            out = np.zeros(nb, np.uint8)
        elif out.dtype != np.uint8 or out.size < nb or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous uint8 array of %d bytes" % nb)
        rc = self._lib.pa_process(self._h, _p32(ks), _p32(kr) if kr is not None else None, n, v, flags,
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), ctypes.byref(self.last_stats))
        if check or rc != PA_ERR_PRECISION:
            self._check(rc, "pa_process")
        return out

    # ---- device-resident forms (pointers are integers, e.g. torch.Tensor.data_ptr()) -------------
    def set_seed_device(self, d_seed: int, n: int, reuse_seed_amount: int = -1, stream: int = 0):
        self._check(self._lib.pa_set_seed_device(self._h, d_seed, n, reuse_seed_amount, stream or None),
                    "pa_set_seed_device")

    def process_device(self, d_key_start: int, d_key_rest: int, n: int, v: int, d_out: int,
                       flags: int = DEFAULT_FLAGS, stream: int = 0):
        self._check(self._lib.pa_process_device(self._h, d_key_start, d_key_rest or None, n, v, flags, d_out,
                                                stream or None), "pa_process_device")

    def set_timing(self, enable: bool = True):
        self._check(self._lib.pa_set_timing(self._h, int(enable)), "pa_set_timing")

    def stage_times(self):
        """Mean device ms per kernel over the blocks recorded since the last call, and the block count."""
        ms = (ctypes.c_float * 8)()
        ns, nb = ctypes.c_int(), ctypes.c_int()
        self._check(self._lib.pa_stage_times(self._h, ms, 8, ctypes.byref(ns), ctypes.byref(nb)), "pa_stage_times")
        return [ms[i] for i in range(ns.value)], nb.value

    # ---- batched and served blocks (slot pool) ------------------------------------------------------
    def set_pool(self, hbm_budget_bytes: int = 0, max_slots: int = 0, batch_slots: int = 0):
        self._check(self._lib.pa_set_pool(self._h, hbm_budget_bytes, max_slots, batch_slots), "pa_set_pool")

    def pool_reserve(self, max_np: int, count: int) -> int:
        """Creates idle slots for cyclic length <= max_np up front; returns how many such slots exist."""
        rc = self._lib.pa_pool_reserve(self._h, max_np, count)
        if rc < 0:
            self._check(rc, "pa_pool_reserve")
        return rc

    def set_groups(self, min_blocks: int = 0, log_bits: int = 0):
        """Grouped launches of equal jobs: at least min_blocks per group (0 = 4), up to 2^log_bits bits of
        cyclic length per group (0 = 24)."""
        self._check(self._lib.pa_set_groups(self._h, min_blocks, log_bits), "pa_set_groups")

    def set_lanes(self, ctas_per_lane: int = 0, max_np: int = 0) -> int:
        """Persistent lanes (PA_BATCH_PERSISTENT): CTAs per lane and the largest cyclic length they hold;
        returns the number of lanes allocated (0 until the first persistent batch when max_np is 0)."""
        rc = self._lib.pa_set_lanes(self._h, ctas_per_lane, max_np)
        if rc < 0:
            self._check(rc, "pa_set_lanes")
        return rc

    # ---- device-resident serving loop -----------------------------------------------------------------
    def serve_start(self, ctas_per_lane: int = 0, max_np: int = 1 << 27, ring_slots: int = 0) -> int:
        """Starts the serving loop on the device; returns the number of lanes."""
        rc = self._lib.pa_serve_start(self._h, ctas_per_lane, max_np, ring_slots)
        if rc < 0:
            self._check(rc, "pa_serve_start")
        return rc

    def serve_submit(self, job: PAJob):
        """Publishes a request (host buffers pinned); returns its ticket, or None when the ring is full."""
        t = ctypes.c_uint64()
        rc = self._lib.pa_serve_submit(self._h, ctypes.byref(job), ctypes.byref(t))
        if rc == PA_ERR_BUSY:
            return None
        self._check(rc, "pa_serve_submit")
        return t.value

    def serve_poll(self, ticket: int):
        """None while the request runs, then its PAStats (job.out holds the result)."""
        st = PAStats()
        rc = self._lib.pa_serve_poll(self._h, ticket, ctypes.byref(st))
        if rc == PA_PENDING:
            return None
        self._check(rc, "pa_serve_poll")
        return st

    def serve_stop(self):
        self._check(self._lib.pa_serve_stop(self._h), "pa_serve_stop")

    def seed_cache_add(self, seed_words, n: int, v: int, flags: int = DEFAULT_FLAGS) -> int:
        s = _u32(seed_words)
        if s.size < n // 32:
            raise ValueError("seed needs n/32 words")
        sid = ctypes.c_int32()
        self._check(self._lib.pa_seed_cache_add(self._h, _p32(s), n, v, flags, ctypes.byref(sid)),
                    "pa_seed_cache_add")
        return sid.value

    def seed_cache_clear(self):
        self._check(self._lib.pa_seed_cache_clear(self._h), "pa_seed_cache_clear")

    def batch_run(self, jobs, batch_flags: int = 0, stream: int = 0):
        """jobs: a sequence of PAJob with device pointers (integers)."""
        arr = (PAJob * max(1, len(jobs)))(*jobs)
        self._check(self._lib.pa_batch_run(self._h, arr, len(jobs), batch_flags, stream or None), "pa_batch_run")

    def batch_sync(self, count: int):
        st = (PAStats * max(1, count))()
        self._check(self._lib.pa_batch_sync(self._h, st, count), "pa_batch_sync")
        return [st[i] for i in range(count)]

    def submit(self, job: PAJob):
        """Returns a ticket, or None when no slot / HBM is free now (PA_ERR_BUSY)."""
        t = ctypes.c_uint64()
        rc = self._lib.pa_submit(self._h, ctypes.byref(job), ctypes.byref(t))
        if rc == PA_ERR_BUSY:
            return None
        self._check(rc, "pa_submit")
        return t.value

    def poll(self, ticket: int):
        """None while the block runs; its PAStats once its output is in the job's host buffer."""
        st = PAStats()
        rc = self._lib.pa_poll(self._h, ticket, ctypes.byref(st))
        if rc == PA_PENDING:
            return None
        self._check(rc, "pa_poll")
        return st

    def set_split(self, log_n: int, log_n2: int):
        self._check(self._lib.pa_set_split(self._h, log_n, log_n2), "pa_set_split")

    def get_split(self, log_n: int) -> int:
        return int(self._lib.pa_get_split(self._h, log_n))

    def autotune(self, min_n: int, max_n: int):
        """Times every split of each size class in [min_n, max_n]; returns {log_n: (log_n2, best ms)}."""
        ms = (ctypes.c_float * 32)()
        self._check(self._lib.pa_autotune(self._h, min_n, max_n, ms), "pa_autotune")
        return {i: (self.get_split(i), ms[i]) for i in range(32) if ms[i] > 0}

    def sync(self, check: bool = True) -> PAStats:
        rc = self._lib.pa_sync(self._h, ctypes.byref(self.last_stats))
        if check or rc != PA_ERR_PRECISION:
            self._check(rc, "pa_sync")
        return self.last_stats
