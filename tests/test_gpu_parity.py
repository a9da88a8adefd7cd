"""GPU parity: the sm_103a engine, called through the C ABI, against the CPU oracle.

Bar: bit-exact output bytes (integer/bit work).  Sizes where the oracle runs in seconds are compared
in full; the full-size n=2^27 block is checked through GF(2) linearity, sampled rows and the XOR
structure.
"""
import hashlib

import numpy as np
import pytest

import large_block as LB
import privacyamplification_gb300 as pa
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS


def run_block(eng, n, v, rng_seed, flags=DEFAULT, reuse=0):
    seed, recv = O.random_block(n, v, rng_seed)
    ks, kr = O.key_split(recv, n, v)
    eng.set_seed(seed, n, reuse)
    out = eng.process(ks, kr, n, v, flags)
    return seed, ks, kr, out


def test_large_block_kat_through_engine(gpu_engine, golden):
    """The reference's 60-chunk known-answer test (n=2^11, no XOR, no compression)."""
    kb, sb = np.unpackbits(golden["key_bits"]), np.unpackbits(golden["seed_bits"])

    def pa_call(s, k):
        gpu_engine.set_seed(s, 2048, 0)
        return gpu_engine.process(k, None, 2048, 1024, 0)

    res = LB.compute(pa_call, kb, sb)
    assert [bytes(h) for h in golden["chunk_hash"]] == res["chunk"]
    assert [bytes(h) for h in golden["intermediate_hash"]] == res["intermediate"]
    assert bytes(golden["result_hash"]) == res["result"]


def test_large_block_composite_through_engine(gpu_engine, golden):
    """The same product as one n=2^14 block with key split and key_rest XOR: final SHA3 of the example."""
    kb, sb = np.unpackbits(golden["key_bits"]), np.unpackbits(golden["seed_bits"])
    seed, recv = LB.composite_inputs(kb, sb)
    ks, kr = pa.key_split(recv, LB.N_BIG, LB.V_BIG)
    gpu_engine.set_seed(seed, LB.N_BIG, -1)
    out = gpu_engine.process(ks, kr, LB.N_BIG, LB.V_BIG, DEFAULT)
    assert hashlib.sha3_256(bytes(out)).digest() == bytes(golden["result_hash"])
    pre = gpu_engine.process(ks, kr, LB.N_BIG, LB.V_BIG, pa.FLAG_COMPRESS)
    assert hashlib.sha3_256(bytes(pre)).digest() == bytes(golden["pre_hash"])


@pytest.mark.parametrize("logn", list(range(10, 21)))
def test_pow2_sizes_vs_oracle(gpu_engine, logn):
    n = 1 << logn
    v = n // 4 + n // 8
    seed, ks, kr, out = run_block(gpu_engine, n, v, 1000 + logn)
    ref = O.direct(seed, ks, kr, n, v, DEFAULT) if logn <= 16 else O.ntt(seed, ks, kr, n, v, DEFAULT)
    assert np.array_equal(out, ref)
    assert gpu_engine.last_stats.max_residual < 0.1


@pytest.mark.parametrize("logn", [22, 24])
def test_large_pow2_vs_ntt(gpu_engine, logn):
    n = 1 << logn
    v = n // 4 + n // 8
    seed, ks, kr, out = run_block(gpu_engine, n, v, 77 + logn)
    assert np.array_equal(out, O.ntt(seed, ks, kr, n, v, DEFAULT))


# n = 2^22 runs rows of 2^14 (last inverse stage radix 32 over 512 butterflies, columns of 2^7): pass C
# rounds only the last-stage outputs r < 32 * KEEP8 / 8 that can hold samples below out_bits, with
# KEEP8 = 2, 3, 4 or 8.  These v sit on and just past each boundary (live outputs r = ceil(v / 2^17)).
@pytest.mark.parametrize("v,flags,split", [
    (1 << 20, DEFAULT, 0), ((1 << 20) + 32, DEFAULT, 0), (3 << 19, DEFAULT, 0), ((3 << 19) + 32, DEFAULT, 0),
    ((1 << 21) - 32, pa.FLAG_COMPRESS, 0), (3 << 19, 0, 0), ((1 << 21) + 32, DEFAULT, 0), (32, DEFAULT, 0),
    ((3 << 19) + 32, DEFAULT, 12), ((1 << 20) + 32, DEFAULT, 13)])
def test_pass_c_output_share_variants(gpu_engine, v, flags, split):
    n = 1 << 22
    if split:
        gpu_engine.set_split(21, split)
    try:
        seed, ks, kr, out = run_block(gpu_engine, n, v, v + flags, flags)
    finally:
        if split:
            gpu_engine.set_split(21, 14)
    assert np.array_equal(out, O.ntt(seed, ks, kr, n, v, flags))


# n = 2^24 (rows 2^14, columns 2^9): key bit rows and the final transpose run in their tiled forms
# (256 x 256 blocks through shared memory).  Output ratios and flags change which plane words and
# key_rest words the finish reads.
@pytest.mark.parametrize("v,flags", [
    ((1 << 22) + (1 << 21), DEFAULT), ((1 << 22) + 32, pa.FLAG_COMPRESS), ((1 << 23) - 4096, 0),
    ((1 << 21) + 96, pa.FLAG_XOR_KEY_REST)])
def test_tiled_transposes_vs_ntt(gpu_engine, v, flags):
    n = 1 << 24
    seed, ks, kr, out = run_block(gpu_engine, n, v, 0x71E + v + flags, flags)
    assert np.array_equal(out, O.ntt(seed, ks, kr, n, v, flags))


@pytest.mark.parametrize("n,v,flags", [
    (1 << 16, 24576, 0), (1 << 16, 24576, pa.FLAG_COMPRESS), (1 << 16, 24576, pa.FLAG_XOR_KEY_REST),
    (1 << 16, 61440, DEFAULT), (1 << 16, 32, DEFAULT), (1 << 16, 65504, DEFAULT), (1 << 16, 32768, 0),
    (1 << 12, 4064, DEFAULT), (1 << 12, 32, 0)])
def test_flags_and_ratios(gpu_engine, n, v, flags):
    seed, ks, kr, out = run_block(gpu_engine, n, v, n + v + flags, flags)
    assert np.array_equal(out, O.direct(seed, ks, kr, n, v, flags))


@pytest.mark.parametrize("n,v,flags", [
    (1056, 416, DEFAULT), (3072, 1152, DEFAULT), (40960, 15360, DEFAULT), (40960, 15360, 0),
    (99328, 9984, DEFAULT), (1 << 18 | 1024, 98304, DEFAULT), (700416, 630272, DEFAULT)])
def test_non_pow2_sizes(gpu_engine, n, v, flags):
    seed, ks, kr, out = run_block(gpu_engine, n, v, n ^ v, flags)
    ref = O.direct(seed, ks, kr, n, v, flags) if n <= 1 << 17 else O.ntt(seed, ks, kr, n, v, flags)
    assert np.array_equal(out, ref)


def test_config1_static_seed_16_blocks(gpu_engine):
    """n=2^16, h=40960, v=24576, static seed, 16 consecutive blocks, bit-exact vs the direct oracle."""
    n, v = 1 << 16, 24576
    seed, _ = O.random_block(n, v, 0x5EED)
    gpu_engine.set_seed(seed, n, -1)
    for b in range(16):
        _, recv = O.random_block(n, v, 0x5EED + 1 + b)
        ks, kr = O.key_split(recv, n, v)
        out = gpu_engine.process(ks, kr, n, v, DEFAULT)
        assert np.array_equal(out, O.direct(seed, ks, kr, n, v, DEFAULT)), b


def test_reuse_seed_amount_semantics(gpu_engine):
    """0: one block, k>0: k blocks, -1: unlimited (PrivacyAmplification.cu:1786, 2099-2101)."""
    n, v = 4096, 1536
    seed, recv = O.random_block(n, v, 9)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, 0)
    gpu_engine.process(ks, kr, n, v)
    with pytest.raises(pa.PAError) as ei:
        gpu_engine.process(ks, kr, n, v)
    assert ei.value.code == pa.PA_ERR_NO_SEED
    gpu_engine.set_seed(seed, n, 3)
    for _ in range(3):
        gpu_engine.process(ks, kr, n, v)
    with pytest.raises(pa.PAError):
        gpu_engine.process(ks, kr, n, v)
    gpu_engine.set_seed(seed, n, -1)
    for _ in range(5):
        gpu_engine.process(ks, kr, n, v)
    assert gpu_engine.last_stats.seed_uses_left == -1


def test_rejects_bad_sizes(gpu_engine):
    seed, recv = O.random_block(4096, 1536, 1)
    gpu_engine.set_seed(seed, 4096, -1)
    ks, kr = O.key_split(recv, 4096, 1536)
    # buffers large enough for any (n, v) below, so that the C ABI's own checks decide
    ks_big = np.concatenate([ks, np.zeros(8, np.uint32)])
    kr_big = np.concatenate([kr, np.zeros(4096 // 32, np.uint32)])
    for n, v in [(4096, 0), (4096, 4096), (4096, 100), (4000, 1536), (512, 256), (4096, 4064 + 64)]:
        with pytest.raises(pa.PAError) as ei:
            gpu_engine.process(ks_big, kr_big, n, v)
        assert ei.value.code == pa.PA_ERR_INVALID_ARG, (n, v)
    with pytest.raises(pa.PAError) as ei:
        gpu_engine.set_seed(np.zeros((1 << 28) // 32, np.uint32), 1 << 28, -1)
    assert ei.value.code in (pa.PA_ERR_TOO_LARGE, pa.PA_ERR_INVALID_ARG)
    # the engine still works after rejected calls
    gpu_engine.set_seed(seed, 4096, -1)
    assert np.array_equal(gpu_engine.process(ks, kr, 4096, 1536), O.direct(seed, ks, kr, 4096, 1536))


def test_popcounts_reported(gpu_engine):
    n, v = 1 << 20, (1 << 20) // 4 + (1 << 20) // 8
    seed, ks, kr, out = run_block(gpu_engine, n, v, 4)
    st = gpu_engine.last_stats
    assert st.popcount_seed == O.popcount(seed, n)
    assert st.popcount_key == O.popcount(ks, n - v + 1)


def test_full_size_2p27_properties(gpu_engine):
    """n=2^27, v=50331648: sampled rows vs the direct oracle, GF(2) linearity in the key, and the XOR."""
    n, v = 1 << 27, 50331648
    h = n - v
    seed, recv1 = O.random_block(n, v, 2027)
    _, recv2 = O.random_block(n, v, 2028)
    ks1, kr1 = O.key_split(recv1, n, v)
    ks2, _ = O.key_split(recv2, n, v)
    gpu_engine.set_seed(seed, n, -1)
    o1 = gpu_engine.process(ks1, kr1, n, v, pa.FLAG_COMPRESS)
    assert gpu_engine.last_stats.max_residual < 0.1
    o2 = gpu_engine.process(ks2, kr1, n, v, pa.FLAG_COMPRESS)
    o12 = gpu_engine.process(ks1 ^ ks2, kr1, n, v, pa.FLAG_COMPRESS)
    assert np.array_equal(o12, o1 ^ o2)
    ox = gpu_engine.process(ks1, kr1, n, v, DEFAULT)
    kr_bytes = kr1.astype(">u4").view(np.uint8)
    assert np.array_equal(ox, o1 ^ kr_bytes)
    rng = np.random.default_rng(5)
    for r0 in [0, v - 64] + list(rng.integers(0, v // 64, 6) * 64):
        ref = O.direct(seed, ks1, kr1, n, v, pa.FLAG_COMPRESS, rows=(int(r0), int(r0) + 64))
        assert np.array_equal(o1[r0 // 8: r0 // 8 + 8], ref[r0 // 8: r0 // 8 + 8]), r0
    assert h == 83886080


@pytest.mark.parametrize("n,v", [(2118656, 1371520), (4635648, 3624576), (9630720, 4456320), (17133568, 11170816)])
def test_padded_nonpow2_stays_within_fp32_budget(gpu_engine, n, v):
    """Non-power-of-two blocks whose padded cyclic length leaves a region no output reads (n + h < Np):
    the FP32 path keeps its usual residual there, so no exact recompute is needed."""
    seed, recv = O.random_block(n, v, n ^ v)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, -1)
    out = gpu_engine.process(ks, kr, n, v)
    st = gpu_engine.last_stats
    assert st.exact == 0 and st.max_residual < 0.1, st.max_residual
    if n <= 1 << 23:
        assert np.array_equal(out, O.ntt(seed, ks, kr, n, v))
    else:
        blk = O.DirectBlock(seed, ks, n, v)
        krb = O.bits_msb(kr, v).astype(np.uint8)
        for r0 in (0, v // 2 // 64 * 64, v - 64):
            assert np.array_equal(np.unpackbits(out[r0 // 8: r0 // 8 + 8]), blk.rows(r0, r0 + 64) ^ krb[r0: r0 + 64])
        blk.close()
