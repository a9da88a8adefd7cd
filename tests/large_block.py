"""Large-block decomposition known-answer test (restatement of examples/LargeBlocksizeExample/main.cpp).

A (v x (h+1)) Toeplitz product with n = 2^14, v = 6144, h = 10240 is cut into 1024 x 1025 Toeplitz
chunks.  Each chunk is one privacy-amplification call with n = 2^11, v = h = 1024,
do_xor_key_rest = false, do_compress = false (main.cpp:44-60).  Per chunk:

* seed  = seed words [r+32, r+64) followed by [r, r+32)           (GetLocalSeed, main.cpp:104-107)
* key_start = 0 followed by key bits keyNr*1024 .. keyNr*1024+1023  (GetLocalKey, main.cpp:111-118)
* the 1024-bit result is XORed into accumulator row ``row``        (XorWithRow, main.cpp:120-124)

The schedule (seedProvider/keyProvider/receiveAmpOut, main.cpp:313-515) walks the chunk columns
right to left, then the remaining rows.  After all 60 chunks the accumulator is XORed with
key_rest = key bits h .. h+v-1 (main.cpp:505-512).

``compute(pa)`` runs the whole schedule through a callable ``pa(seed_words, key_start_words) ->
bytes`` (128 output bytes) and returns every SHA3-256 the example asserts, in order.
"""
import hashlib

import numpy as np

N_BIG, V_BIG, H_BIG = 1 << 14, 6144, 10240
N_CHUNK = 1 << 11
SIDE = 1024  # chunk_side
SIDE_W = SIDE // 32
V_CHUNKS, H_CHUNKS = V_BIG // SIDE, H_BIG // SIDE  # 6, 10


def words_from_bits(bits):
    """binTo4byteLittleEndian (main.cpp:220-230): 32 bits per word, first bit in the MSB."""
    return np.packbits(np.asarray(bits, dtype=np.uint8)).view(">u4").astype(np.uint32)


def schedule():
    """Yields (r, keyNr, row, first_of_column) in the example's order (main.cpp:313-429)."""
    r = 0
    for col in range(H_CHUNKS - 1, -1, -1):
        row = 0
        for key_nr in range(col, col + min(H_CHUNKS - col, V_CHUNKS)):
            yield r, key_nr, row, key_nr == col
            row += 1
        r += SIDE_W
    for row_nr in range(1, V_CHUNKS):
        row = row_nr
        for key_nr in range(0, min(H_BIG // SIDE_W, V_CHUNKS - row_nr)):
            yield r, key_nr, row, False
            row += 1
        r += SIDE_W


def chunk_inputs(seed_words, key_words, r, key_nr):
    local_seed = np.concatenate([seed_words[r + SIDE_W: r + 2 * SIDE_W], seed_words[r: r + SIDE_W]])
    off = key_words[key_nr * SIDE_W: key_nr * SIDE_W + SIDE_W].astype(np.uint64)
    ks = np.zeros(SIDE_W + 1, dtype=np.uint64)
    ks[0] = off[0] >> 1
    ks[1:SIDE_W] = ((off[:-1] & 1) << 31) | (off[1:] >> 1)
    ks[SIDE_W] = (off[SIDE_W - 1] & 1) << 31
    key_start = np.zeros(N_CHUNK // 32, dtype=np.uint32)
    key_start[: SIDE_W + 1] = ks.astype(np.uint32)
    return local_seed.astype(np.uint32), key_start


def compute(pa, key_bits, seed_bits):
    """Returns dict with lists 'chunk' (60), 'intermediate' (70) and 'pre', 'key_rest', 'result'."""
    sha = lambda b: hashlib.sha3_256(bytes(b)).digest()
    seed_words = words_from_bits(seed_bits)
    key_words = words_from_bits(key_bits)
    acc = np.zeros(V_CHUNKS * SIDE // 8, dtype=np.uint8)
    out = {"chunk": [], "intermediate": []}
    for r, key_nr, row, first in schedule():
        if first:
            out["intermediate"].append(sha(acc))
        s, k = chunk_inputs(seed_words, key_words, r, key_nr)
        amp = np.asarray(pa(s, k), dtype=np.uint8)
        assert amp.size == SIDE // 8
        out["chunk"].append(sha(amp))
        acc[row * (SIDE // 8): (row + 1) * (SIDE // 8)] ^= amp
        out["intermediate"].append(sha(acc))
    out["pre"] = sha(acc)
    key_bytes = key_words.astype("<u4").view(np.uint8)
    key_rest = key_bytes[H_BIG // 8: H_BIG // 8 + V_BIG // 8]
    out["key_rest"] = sha(key_rest)
    res = acc.copy().reshape(-1, 4)
    res ^= key_rest.reshape(-1, 4)[:, ::-1]
    out["result"] = sha(res.reshape(-1))
    return out


def composite_inputs(key_bits, seed_bits):
    """The same n = 2^14 product as ONE block in the reference's own format.

    Summing the chunk products gives composite[i] = sum_{J<h} K[J] * S[h-1+i-J] (i < v), a linear
    Toeplitz product over seed bits 0 .. n-2.  The reference computes
    out[i] = sum_{j<=h} key_start[j] * seed[(i-j) mod n]; with recv_key = a zero bit followed by K
    (key_start[j] = K[j-1], key_rest = K bits h .. h+v-1, as key2StartRest builds them) and the seed
    rotated left by h bits (seed[m] = S[(m+h) mod n]) the two agree bit for bit."""
    seed_words = np.roll(words_from_bits(seed_bits), -(H_BIG // 32))
    kb = np.concatenate([[0], np.asarray(key_bits, dtype=np.uint8), np.zeros(31, dtype=np.uint8)])
    recv_key = words_from_bits(kb[: N_BIG + 32])
    return seed_words, recv_key
