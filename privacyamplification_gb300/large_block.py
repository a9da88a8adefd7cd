"""Large-block decomposition: one privacy-amplification block of any size as many smaller engine blocks.

The reference shows the technique in examples/LargeBlocksizeExample/main.cpp (GetLocalSeed :104-107,
GetLocalKey :111-118, XorWithRow :120-124, the diagonal schedule :313-515).  Stated generally: the
block's result bit i (i < out_bits) is

    out[i] = XOR_{j=0..h} key_start[j] AND T[i - j],   T[m] = seed[m mod n]   (m in [-h, out_bits)),

a linear Toeplitz product.  Cut rows i into chunks of `side` and key positions j into chunks of `side`
(the last one zero-padded); chunk (a, b) contributes, for i' < side,

    sum_{j' < side} key_start[b*side + j'] * T[(a - b)*side + i' - j'],

which is exactly one engine block of n' = 2*side, v' = h' = side (no XOR, no compression) with
key_start' = the key chunk followed by a zero bit, and seed' = T[d*side, d*side + side) followed by
T[d*side - side, d*side) for d = a - b.  Chunks on one diagonal d share seed', so each diagonal sets its
seed once with reuse_seed_amount = its chunk count and the engine keeps the seed spectrum.  The chunk
results are XORed into row a; key_rest is XORed at the end.

Uses: blocks larger than one engine call allows (n > 2^30), or keeping very large blocks on the FP32
path in chunks of n' = 2^27 instead of the exact path.
"""
from __future__ import annotations

import numpy as np

from . import FLAG_COMPRESS, FLAG_XOR_KEY_REST


def _bits_to_bytes_msb(words: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(words, dtype=np.uint32).astype(">u4").view(np.uint8)


def plan(n: int, v: int, flags: int, side: int):
    """Chunk grid: (rows of chunks A, key columns of chunks B, out_bits)."""
    h = n - v
    ob = v if flags & FLAG_COMPRESS else n // 2
    return -(-ob // side), -(-(h + 1) // side), ob


def hash_large_block(engine, seed_words, key_start, key_rest, n: int, v: int,
                     flags: int = FLAG_XOR_KEY_REST | FLAG_COMPRESS, side: int = 1 << 26) -> np.ndarray:
    """pa_process semantics for (n, v, flags), computed as side x side chunks on `engine`.

    seed_words: n/32 words; key_start: at least h/32+1 words (bits past h are ignored); key_rest: v/32
    words when FLAG_XOR_KEY_REST.  side: power of two, 512 <= side, 2*side <= engine.max_sample_size.
    Returns pa_output_bytes(n, v, flags) bytes."""
    if side < 512 or side & (side - 1) or n % 32 or v % 32 or not 0 < v < n:
        raise ValueError("side must be a power of two >= 512; n, v multiples of 32 with 0 < v < n")
    if 2 * side > engine.max_sample_size:
        raise ValueError("2*side exceeds the engine's max_sample_size")
    h = n - v
    seed = np.ascontiguousarray(seed_words, dtype=np.uint32)[: n // 32]
    A, B, ob = plan(n, v, flags, side)
    sw = side // 32
    # key_start masked to bits 0..h and zero-padded to B*side bits
    ks = np.zeros(B * sw, dtype=np.uint32)
    src = np.ascontiguousarray(key_start, dtype=np.uint32)[: h // 32 + 1]
    ks[: src.size] = src
    ks[h // 32] &= np.uint32((0xFFFFFFFF << (31 - h % 32)) & 0xFFFFFFFF)
    ks[h // 32 + 1:] = 0
    nw = n // 32

    def T(start_bit, count_bits):  # T[m] = seed[m mod n]; start and count multiples of 32
        idx = (np.arange(start_bit // 32, (start_bit + count_bits) // 32) % nw)
        return seed[idx]

    acc = np.zeros(A * side // 8, dtype=np.uint8)
    key_chunk = np.zeros(2 * sw, dtype=np.uint32)  # chunk bits, then zeros (h' = side: bit `side` is 0)
    for d in range(-(B - 1), A):
        chunks = [(a, a - d) for a in range(max(0, d), min(A, B + d))]
        if not chunks:
            continue
        local = np.concatenate([T(d * side, side), T(d * side - side, side)])
        engine.set_seed(local, 2 * side, len(chunks))
        for a, b in chunks:
            key_chunk[:sw] = ks[b * sw: (b + 1) * sw]
            out = engine.process(key_chunk, None, 2 * side, side, 0)
            acc[a * side // 8: (a + 1) * side // 8] ^= out
    res = acc[: ob // 8].copy()
    if flags & FLAG_XOR_KEY_REST:
        kr = _bits_to_bytes_msb(np.ascontiguousarray(key_rest, dtype=np.uint32)[: v // 32])
        m = min(v, ob) // 8
        res[:m] ^= kr[:m]
    return res
