"""CPU oracle for the privacy-amplification hot path (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import this module.  It is the
checker, never the thing measured or shipped: the product library has no CPU fallback.

Three restatements of the same arithmetic (paths relative to the nicoboss/PrivacyAmplification tree):

* ``direct``   -- C, bit-packed rows (AND + parity), ``oracle/pa_oracle.c``
* ``ntt``      -- C, exact integer cyclic convolution modulo 2^64-2^32+1, ``oracle/pa_oracle.c``
  (``NttSeed`` keeps a seed's transform for many keys)
* ``numpy_reference`` -- pure numpy, small n only; follows the same reference lines:
  bit order ``PrivacyAmplification.cu:223-257,584-593``; key split ``PrivacyAmplification.cu:861-892``;
  convolution ``PrivacyAmplification.cu:1898-1979``; rounding/XOR/packing
  ``PrivacyAmplification.cu:740-813`` with ``AMPOUT_REVERSE_ENDIAN`` (``PrivacyAmplification.h:38``).

The restatement is pinned by the SHA3-256 known-answer vectors of
``examples/LargeBlocksizeExample/Matrix.h`` (committed as fixtures under tests/golden/).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import threading

import numpy as np

FLAG_XOR_KEY_REST = 1
FLAG_COMPRESS = 2

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpa_oracle.so")
_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile the C oracle with its Makefile (gcc, OpenMP).  Returns the library path."""
    src = os.path.join(_HERE, "pa_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(_LIB_PATH)
            u32p = ctypes.POINTER(ctypes.c_uint32)
            u8p = ctypes.POINTER(ctypes.c_uint8)
            lib.pa_oracle_key_split.argtypes = [u32p, ctypes.c_uint32, ctypes.c_uint32, u32p, u32p]
            lib.pa_oracle_key_split.restype = None
            lib.pa_oracle_direct.argtypes = [u32p, u32p, u32p, ctypes.c_uint32, ctypes.c_uint32,
                                             ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, u8p,
                                             ctypes.c_int]
            lib.pa_oracle_direct.restype = ctypes.c_int
            lib.pa_oracle_ntt.argtypes = [u32p, u32p, u32p, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_uint32, u8p, ctypes.c_int]
            lib.pa_oracle_ntt.restype = ctypes.c_int
            lib.pa_oracle_conv_exact.argtypes = [u32p, u32p, ctypes.c_uint32, ctypes.c_uint32,
                                                 ctypes.c_uint64, ctypes.POINTER(ctypes.c_int64),
                                                 ctypes.c_int]
            lib.pa_oracle_conv_exact.restype = ctypes.c_int
            lib.pa_oracle_ntt_seed_prepare.argtypes = [u32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
            lib.pa_oracle_ntt_seed_prepare.restype = ctypes.c_void_p
            lib.pa_oracle_ntt_seed_free.argtypes = [ctypes.c_void_p]
            lib.pa_oracle_ntt_seed_free.restype = None
            lib.pa_oracle_ntt_with_seed.argtypes = [ctypes.c_void_p, u32p, u32p, ctypes.c_uint32, u8p,
                                                    ctypes.c_int]
            lib.pa_oracle_ntt_with_seed.restype = ctypes.c_int
            lib.pa_oracle_popcount.argtypes = [u32p, ctypes.c_uint64]
            lib.pa_oracle_popcount.restype = ctypes.c_uint64
            lib.pa_oracle_direct_prepare.argtypes = [u32p, u32p, ctypes.c_uint32, ctypes.c_uint32]
            lib.pa_oracle_direct_prepare.restype = ctypes.c_void_p
            lib.pa_oracle_direct_rows.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, u8p,
                                                  ctypes.c_int]
            lib.pa_oracle_direct_rows.restype = None
            lib.pa_oracle_direct_free.argtypes = [ctypes.c_void_p]
            lib.pa_oracle_direct_free.restype = None
            _lib = lib
    return _lib


def _p32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def _p8(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def out_bits(n: int, v: int, flags: int) -> int:
    """Output length in bits (PrivacyAmplification.cu:1197): v when compressing, else n/2."""
    return v if flags & FLAG_COMPRESS else n // 2


def key_split(recv_key: np.ndarray, n: int, v: int):
    """key2StartRest (PrivacyAmplification.cu:861-892).  recv_key: n/32+1 uint32 words.
    Returns (key_start[n/32], key_rest[v/32])."""
    recv_key = np.ascontiguousarray(recv_key, dtype=np.uint32)
    assert recv_key.size >= n // 32 + 1
    ks = np.zeros(n // 32, dtype=np.uint32)
    kr = np.zeros(max(v // 32, 1), dtype=np.uint32)
    _load().pa_oracle_key_split(_p32(recv_key), n, v, _p32(ks), _p32(kr))
    return ks, kr[: v // 32]


def direct(seed, key_start, key_rest, n, v, flags=FLAG_XOR_KEY_REST | FLAG_COMPRESS,
           rows=None, threads=0) -> np.ndarray:
    """Direct bit-packed GF(2) Toeplitz product.  rows=(i0, i1) computes only those output bits
    (the rest of the returned byte array is zero)."""
    seed = np.ascontiguousarray(seed, dtype=np.uint32)
    key_start = np.ascontiguousarray(key_start, dtype=np.uint32)
    kr = np.ascontiguousarray(key_rest if key_rest is not None else np.zeros(1, np.uint32), dtype=np.uint32)
    ob = out_bits(n, v, flags)
    out = np.zeros(ob // 8, dtype=np.uint8)
    i0, i1 = rows if rows is not None else (0, ob)
    rc = _load().pa_oracle_direct(_p32(seed), _p32(key_start), _p32(kr), n, v, flags, i0, i1, _p8(out),
                                  threads)
    if rc:
        raise ValueError("oracle rejected sizes n=%d v=%d" % (n, v))
    return out


def ntt(seed, key_start, key_rest, n, v, flags=FLAG_XOR_KEY_REST | FLAG_COMPRESS, threads=0) -> np.ndarray:
    """Exact NTT convolution, full block."""
    seed = np.ascontiguousarray(seed, dtype=np.uint32)
    key_start = np.ascontiguousarray(key_start, dtype=np.uint32)
    kr = np.ascontiguousarray(key_rest if key_rest is not None else np.zeros(1, np.uint32), dtype=np.uint32)
    out = np.zeros(out_bits(n, v, flags) // 8, dtype=np.uint8)
    rc = _load().pa_oracle_ntt(_p32(seed), _p32(key_start), _p32(kr), n, v, flags, _p8(out), threads)
    if rc:
        raise ValueError("oracle rejected sizes n=%d v=%d" % (n, v))
    return out


class NttSeed:
    """A seed's exact transform for blocks of size (n, v), kept for many keys (the static-seed case:
    each block then costs one forward and one inverse transform)."""

    def __init__(self, seed, n, v, threads=0):
        self._seed = np.ascontiguousarray(seed, dtype=np.uint32)
        self.n, self.v = n, v
        self._ctx = _load().pa_oracle_ntt_seed_prepare(_p32(self._seed), n, v, threads)
        if not self._ctx:
            raise ValueError("oracle rejected sizes n=%d v=%d" % (n, v))

    def block(self, key_start, key_rest, flags=FLAG_XOR_KEY_REST | FLAG_COMPRESS, threads=0) -> np.ndarray:
        key_start = np.ascontiguousarray(key_start, dtype=np.uint32)
        kr = np.ascontiguousarray(key_rest if key_rest is not None else np.zeros(1, np.uint32), dtype=np.uint32)
        out = np.zeros(out_bits(self.n, self.v, flags) // 8, dtype=np.uint8)
        if _load().pa_oracle_ntt_with_seed(self._ctx, _p32(key_start), _p32(kr), flags, _p8(out), threads):
            raise ValueError("oracle failed")
        return out

    def close(self):
        if self._ctx:
            _load().pa_oracle_ntt_seed_free(self._ctx)
            self._ctx = None

    def __del__(self):
        self.close()


def conv_exact(seed, key_start, n, v, count, threads=0) -> np.ndarray:
    """Exact integer values c[i] = sum_j key_start[j]*seed[(i-j) mod n], i < count."""
    seed = np.ascontiguousarray(seed, dtype=np.uint32)
    key_start = np.ascontiguousarray(key_start, dtype=np.uint32)
    out = np.zeros(count, dtype=np.int64)
    rc = _load().pa_oracle_conv_exact(_p32(seed), _p32(key_start), n, v, count,
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), threads)
    if rc:
        raise ValueError("oracle rejected sizes")
    return out


class DirectBlock:
    """The direct method split into its per-block setup and its per-row work (for timing the CPU
    baseline: a CPU implementation pays the setup once per block and the row work v times)."""

    def __init__(self, seed, key_start, n, v):
        self._seed = np.ascontiguousarray(seed, dtype=np.uint32)
        self._ks = np.ascontiguousarray(key_start, dtype=np.uint32)
        self.n, self.v = n, v
        self._ctx = _load().pa_oracle_direct_prepare(_p32(self._seed), _p32(self._ks), n, v)
        if not self._ctx:
            raise ValueError("oracle rejected sizes")

    def rows(self, i0, i1, threads=0) -> np.ndarray:
        par = np.zeros(i1 - i0, np.uint8)
        _load().pa_oracle_direct_rows(self._ctx, i0, i1, _p8(par), threads)
        return par

    def close(self):
        if self._ctx:
            _load().pa_oracle_direct_free(self._ctx)
            self._ctx = None

    def __del__(self):
        self.close()


def popcount(words, bits) -> int:
    words = np.ascontiguousarray(words, dtype=np.uint32)
    return int(_load().pa_oracle_popcount(_p32(words), bits))


# ----------------------------------------------------------------------------- pure numpy, small n

def bits_msb(words: np.ndarray, count: int) -> np.ndarray:
    """Bit i = (word[i/32] >> (31 - i%32)) & 1  (PrivacyAmplification.cu:584-593)."""
    w = np.ascontiguousarray(words, dtype=np.uint32)
    b = np.unpackbits(w.byteswap().view(np.uint8))  # big-endian bytes, MSB first
    return b[:count].astype(np.int64)


def pack_output(par: np.ndarray, key_rest, v: int, flags: int) -> np.ndarray:
    """Bit i -> byte i/8, bit 7-i%8; XOR key_rest bit i for i < v when FLAG_XOR_KEY_REST."""
    par = (np.asarray(par) & 1).astype(np.uint8)
    if flags & FLAG_XOR_KEY_REST:
        kr = bits_msb(key_rest, v).astype(np.uint8)
        par = par.copy()
        m = min(v, par.size)
        par[:m] ^= kr[:m]
    return np.packbits(par)


def numpy_reference(seed, key_start, key_rest, n, v, flags=FLAG_XOR_KEY_REST | FLAG_COMPRESS):
    """O(n*h) restatement for tiny n (tests only)."""
    h = n - v
    s = bits_msb(seed, n)
    k = bits_msb(key_start, h + 1)
    ob = out_bits(n, v, flags)
    idx = (np.arange(ob)[:, None] - np.arange(h + 1)[None, :]) % n
    par = (s[idx] * k[None, :]).sum(axis=1) & 1
    return pack_output(par, key_rest, v, flags)


def sha3_256(data) -> str:
    return hashlib.sha3_256(bytes(np.ascontiguousarray(data).view(np.uint8))).hexdigest().upper()


def random_block(n: int, v: int, rng_seed: int = 0x5EED):
    """Seeded i.i.d. Bernoulli(0.5) seed and key words (the synthetic inputs of every benchmark
    configuration).  Returns (seed[n/32], recv_key[n/32+1])."""
    rng = np.random.Generator(np.random.PCG64(rng_seed))
    seed = rng.integers(0, 2 ** 32, size=n // 32, dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2 ** 32, size=n // 32 + 1, dtype=np.uint64).astype(np.uint32)
    return seed, key
