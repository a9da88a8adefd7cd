"""The CPU oracle pinned against the reference's own known-answer vectors (no GPU needed).

Golden data: examples/LargeBlocksizeExample/Matrix.h (tests/golden/large_block_kat.npz, made by
tests/golden/make_golden.py).  The 60 chunk hashes exercise n=2^11, v=h=1024, no XOR, no compression;
the composite hashes exercise a full n=2^14, v=6144 block with the key split and the key_rest XOR.
"""
import hashlib

import numpy as np
import pytest

import large_block as LB
from oracle import oracle as O

NOXOR_UNCOMPRESSED = 0
DEFAULT = O.FLAG_XOR_KEY_REST | O.FLAG_COMPRESS


def _bits(golden):
    return np.unpackbits(golden["key_bits"]), np.unpackbits(golden["seed_bits"])


def _check_schedule(res, golden):
    assert [bytes(h) for h in golden["chunk_hash"]] == res["chunk"]
    assert [bytes(h) for h in golden["intermediate_hash"]] == res["intermediate"]
    assert bytes(golden["pre_hash"]) == res["pre"]
    assert bytes(golden["key_rest_hash"]) == res["key_rest"]
    assert bytes(golden["result_hash"]) == res["result"]


@pytest.mark.parametrize("method", ["direct", "ntt", "numpy"])
def test_large_block_kat_chunks(golden, method):
    fn = {
        "direct": lambda s, k: O.direct(s, k, None, 2048, 1024, NOXOR_UNCOMPRESSED),
        "ntt": lambda s, k: O.ntt(s, k, None, 2048, 1024, NOXOR_UNCOMPRESSED),
        "numpy": lambda s, k: O.numpy_reference(s, k, None, 2048, 1024, NOXOR_UNCOMPRESSED),
    }[method]
    kb, sb = _bits(golden)
    _check_schedule(LB.compute(fn, kb, sb), golden)


@pytest.mark.parametrize("method", ["direct", "ntt"])
def test_large_block_kat_composite(golden, method):
    kb, sb = _bits(golden)
    seed, recv_key = LB.composite_inputs(kb, sb)
    ks, kr = O.key_split(recv_key, LB.N_BIG, LB.V_BIG)
    f = O.direct if method == "direct" else O.ntt
    pre = f(seed, ks, kr, LB.N_BIG, LB.V_BIG, O.FLAG_COMPRESS)
    assert hashlib.sha3_256(bytes(pre)).digest() == bytes(golden["pre_hash"])
    out = f(seed, ks, kr, LB.N_BIG, LB.V_BIG, DEFAULT)
    assert hashlib.sha3_256(bytes(out)).digest() == bytes(golden["result_hash"])


def test_key_split_matches_reference_definition():
    """key2StartRest: key_start = bits 0..h, key_rest = bits h+1..h+v (PrivacyAmplification.cu:861-892)."""
    n, v = 4096, 1536
    _, recv = O.random_block(n, v, 11)
    ks, kr = O.key_split(recv, n, v)
    bits = O.bits_msb(recv, n + 32)
    h = n - v
    assert np.array_equal(O.bits_msb(ks, n)[: h + 1], bits[: h + 1])
    assert not O.bits_msb(ks, n)[h + 1:].any()
    assert np.array_equal(O.bits_msb(kr, v), bits[h + 1: h + 1 + v])


@pytest.mark.parametrize("n,v,flags", [
    (1024, 384, DEFAULT), (2048, 1024, NOXOR_UNCOMPRESSED), (1024, 512, O.FLAG_COMPRESS),
    (1056, 416, DEFAULT), (1024, 992, DEFAULT), (1024, 32, DEFAULT), (3072, 1152, O.FLAG_XOR_KEY_REST)])
def test_three_restatements_agree(n, v, flags):
    seed, recv = O.random_block(n, v, n + v)
    ks, kr = O.key_split(recv, n, v)
    a = O.direct(seed, ks, kr, n, v, flags)
    b = O.ntt(seed, ks, kr, n, v, flags)
    c = O.numpy_reference(seed, ks, kr, n, v, flags)
    assert np.array_equal(a, b) and np.array_equal(a, c)


@pytest.mark.parametrize("n,v", [(1 << 16, 24576), (1 << 18, 98304), (40960, 12288)])
def test_direct_vs_ntt_medium(n, v):
    seed, recv = O.random_block(n, v, 7)
    ks, kr = O.key_split(recv, n, v)
    assert np.array_equal(O.direct(seed, ks, kr, n, v), O.ntt(seed, ks, kr, n, v))


def test_direct_row_subset():
    n, v = 1 << 16, 24576
    seed, recv = O.random_block(n, v, 3)
    ks, kr = O.key_split(recv, n, v)
    full = O.direct(seed, ks, kr, n, v)
    part = O.direct(seed, ks, kr, n, v, rows=(4096, 8192))
    assert np.array_equal(full[512:1024], part[512:1024])
    assert not part[:512].any() and not part[1024:].any()


def test_conv_exact_values():
    n, v = 2048, 768
    seed, recv = O.random_block(n, v, 5)
    ks, _ = O.key_split(recv, n, v)
    c = O.conv_exact(seed, ks, n, v, n)
    s = O.bits_msb(seed, n)
    k = O.bits_msb(ks, n - v + 1)
    ref = np.array([sum(int(k[j]) * int(s[(i - j) % n]) for j in range(n - v + 1)) for i in range(0, n, 97)])
    assert np.array_equal(c[::97], ref)


def test_popcount():
    w = np.array([0xFFFFFFFF, 0x80000001, 0xF0000000], np.uint32)
    assert O.popcount(w, 96) == 32 + 2 + 4
    assert O.popcount(w, 34) == 33


def test_workload_generator_matches_oracle_generator():
    """The bench draws its inputs from the package's generator; the GPU tests rebuild them with the
    oracle's: both must give the same words."""
    from privacyamplification_gb300 import workloads as W
    for n, v, sd in ((1 << 12, 1536, 7), (1 << 16, 24576, 0x5EED)):
        a, b = W.random_block(n, v, sd), O.random_block(n, v, sd)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_sub_block_bank_layout(pa_lib):
    """Sub-blocks of a bank: B = bank / s blocks with v = 3s/8, each key split by key2StartRest of its own
    received key (bits past h of key_start are zero)."""
    from privacyamplification_gb300 import workloads as W
    s, v, seeds, ks, kr = W.sub_block_bank(12, bank_bits=6 << 12, rng_seed=3)
    assert (s, v) == (4096, 1536) and seeds.shape == (6, 128) and ks.shape == (6, 128) and kr.shape == (6, 48)
    h = s - v
    for i in range(6):
        seed, recv = O.random_block(s, v, 3 + i)
        assert np.array_equal(seeds[i], seed)
        k0, k1 = O.key_split(recv, s, v)
        assert np.array_equal(ks[i], k0) and np.array_equal(kr[i], k1)
        assert not ks[i][h // 32 + 1:].any()
