"""Exact integer path (NTT mod 3*2^30+1) and the FP32 precision guard, through the C ABI.

Precision-stress configuration: blocks whose FP32 rounding budget is exceeded (a seed with a long run of
ones and an all-ones key) must still be bit-exact -- pa_process detects them by their residual and
recomputes them exactly.  Blocks beyond 2^27 bits (n = 2^29 with a fresh seed per block) run on the FP32
path as 2^27-bit chunk blocks under the same guard, with the exact path as the fallback.
"""
import numpy as np
import pytest

import privacyamplification_gb300 as pa
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS


def std_sizes(n):
    return n, n // 4 + n // 8


@pytest.mark.parametrize("n,v,flags", [
    (1 << 10, 384, DEFAULT), (1 << 14, 6144, 0), (1 << 16, 24576, DEFAULT), (1 << 18, 98304, pa.FLAG_COMPRESS),
    (1 << 20, 393216, DEFAULT), (40960, 15360, DEFAULT), (99328, 9984, 0)])
def test_exact_flag_matches_oracle(gpu_engine, n, v, flags):
    seed, recv = O.random_block(n, v, 31 * n + v)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, -1)
    out = gpu_engine.process(ks, kr, n, v, flags | pa.FLAG_EXACT)
    assert gpu_engine.last_stats.exact == 1
    ref = O.direct(seed, ks, kr, n, v, flags) if n <= 1 << 17 else O.ntt(seed, ks, kr, n, v, flags)
    assert np.array_equal(out, ref)
    assert np.array_equal(gpu_engine.process(ks, kr, n, v, flags), ref)  # FP32 path agrees
    assert gpu_engine.last_stats.exact == 0


def run_structured(n, v):
    """Seed: first n/2 bits one; key: all ones -- the FP32-breaking block."""
    seed = np.zeros(n // 32, np.uint32)
    seed[: n // 64] = 0xFFFFFFFF
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    return seed, recv


@pytest.mark.parametrize("logn", [22, 24])
def test_guard_falls_back_to_exact(gpu_engine, logn):
    n, v = std_sizes(1 << logn)
    seed, recv = run_structured(n, v)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, -1)
    out = gpu_engine.process(ks, kr, n, v)
    st = gpu_engine.last_stats
    assert st.max_residual > 0.25, "the FP32 path was expected to exceed its budget on this block"
    assert st.exact == 1
    assert np.array_equal(out, O.ntt(seed, ks, kr, n, v))


def test_all_ones_block_is_benign(gpu_engine):
    """All-ones key and seed: the seed spectrum is pure DC, which the path drops, so FP32 stays exact."""
    n, v = std_sizes(1 << 22)
    seed = np.full(n // 32, 0xFFFFFFFF, np.uint32)
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, -1)
    out = gpu_engine.process(ks, kr, n, v)
    assert gpu_engine.last_stats.exact == 0
    assert np.array_equal(out, O.ntt(seed, ks, kr, n, v))


def test_adversarial_2p27_sampled_rows(gpu_engine):
    n, v = 1 << 27, 50331648
    seed, recv = run_structured(n, v)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, -1)
    out = gpu_engine.process(ks, kr, n, v)
    assert gpu_engine.last_stats.exact == 1
    blk = O.DirectBlock(seed, ks, n, v)
    krb = O.bits_msb(kr, v).astype(np.uint8)
    for r0 in (0, 64 * 12345, v // 2, v - 64):
        ref = blk.rows(r0, r0 + 64) ^ krb[r0: r0 + 64]
        assert np.array_equal(np.unpackbits(out[r0 // 8: r0 // 8 + 8]), ref), r0


@pytest.fixture(scope="module")
def big_engine(pa_lib):
    eng = pa.Engine(max_sample_size=1 << 29)
    yield eng
    eng.close()


def test_config3_2p29_dynamic_seed(big_engine):
    """n = 2^29, h = n/2+n/8, v = n/4+n/8, a fresh seed per block (FP32 path in 2^27-bit chunk blocks):
    sampled rows against the direct oracle, GF(2) linearity in the key for a fixed seed, and the
    key_rest XOR."""
    n, v = std_sizes(1 << 29)
    rng = np.random.default_rng(29)
    outs = []
    for blk_no in range(2):
        seed, recv = O.random_block(n, v, 2900 + blk_no)
        ks, kr = O.key_split(recv, n, v)
        big_engine.set_seed(seed, n, 0)
        out = big_engine.process(ks, kr, n, v)
        assert big_engine.last_stats.exact == 2 and big_engine.last_stats.max_residual < 0.1
        blk = O.DirectBlock(seed, ks, n, v)
        krb = O.bits_msb(kr, v).astype(np.uint8)
        for r0 in [0, v - 64] + [int(x) * 64 for x in rng.integers(0, v // 64, 3)]:
            ref = blk.rows(r0, r0 + 64) ^ krb[r0: r0 + 64]
            assert np.array_equal(np.unpackbits(out[r0 // 8: r0 // 8 + 8]), ref), (blk_no, r0)
        outs.append((seed, ks, kr, out))
    seed, ks1, kr1, _ = outs[1]
    _, ks2, _, _ = outs[0]
    big_engine.set_seed(seed, n, -1)
    o1 = big_engine.process(ks1, kr1, n, v, pa.FLAG_COMPRESS)
    o2 = big_engine.process(ks2, kr1, n, v, pa.FLAG_COMPRESS)
    o12 = big_engine.process(ks1 ^ ks2, kr1, n, v, pa.FLAG_COMPRESS)
    assert np.array_equal(o12, o1 ^ o2)
    ox = big_engine.process(ks1, kr1, n, v, DEFAULT)
    assert np.array_equal(ox, o1 ^ kr1.astype(">u4").view(np.uint8))


@pytest.mark.parametrize("n,v,flags", [(1 << 28, (1 << 26) + (1 << 25), DEFAULT),
                                       ((1 << 28) + (1 << 20), 100663296, pa.FLAG_COMPRESS),
                                       ((1 << 28) - 1024, 33554432, pa.FLAG_XOR_KEY_REST),
                                       (1 << 28, 1 << 27, DEFAULT),
                                       ((1 << 28) + (1 << 20), (1 << 27) + (1 << 20), pa.FLAG_COMPRESS)])
def test_chunked_fp32_equals_exact_path(big_engine, n, v, flags):
    """Blocks beyond 2^27 bits: the FP32 chunk path reproduces the exact path bit for bit (whole
    output), powers of two and not, with and without compression / XOR.  The last two have h = 2^27,
    a multiple of the chunk side: their one tap past the last full key column rides in that column."""
    seed, recv = O.random_block(n, v, n % 1000 + flags)
    ks, kr = pa.key_split(recv, n, v)
    big_engine.set_seed(seed, n, -1)
    out = big_engine.process(ks, kr, n, v, flags)
    assert big_engine.last_stats.exact == 2 and big_engine.last_stats.max_residual < 0.1
    ref = big_engine.process(ks, kr, n, v, flags | pa.FLAG_EXACT)
    assert big_engine.last_stats.exact == 1
    assert np.array_equal(out, ref)


def test_chunked_guard_falls_back_to_exact(big_engine):
    """Run-structured block at n = 2^28: the chunk residuals exceed the budget and the block is
    recomputed on the exact path."""
    n, v = std_sizes(1 << 28)
    seed, recv = run_structured(n, v)
    ks, kr = pa.key_split(recv, n, v)
    big_engine.set_seed(seed, n, -1)
    out = big_engine.process(ks, kr, n, v)
    st = big_engine.last_stats
    assert st.max_residual > 0.25 and st.exact == 1
    blk = O.DirectBlock(seed, ks, n, v)
    krb = O.bits_msb(kr, v).astype(np.uint8)
    for r0 in (0, v // 2 // 64 * 64, v - 64):
        assert np.array_equal(np.unpackbits(out[r0 // 8: r0 // 8 + 8]), blk.rows(r0, r0 + 64) ^ krb[r0: r0 + 64])
    blk.close()


def test_maximum_size_2p30(pa_lib):
    """The largest block the engine accepts, n = 2^30 (66 chunk blocks): sampled rows against the
    direct oracle, and the key_rest XOR; n = 2^30 + 1024 is refused."""
    n, v = std_sizes(1 << 30)
    rng = np.random.default_rng(30)
    seed = rng.integers(0, 1 << 32, n // 32, dtype=np.uint64).astype(np.uint32)
    recv = rng.integers(0, 1 << 32, n // 32 + 1, dtype=np.uint64).astype(np.uint32)
    ks, kr = pa.key_split(recv, n, v)
    with pa.Engine(max_sample_size=n) as eng:
        eng.set_seed(seed, n, -1)
        out = eng.process(ks, kr, n, v)
        assert eng.last_stats.exact == 2 and eng.last_stats.max_residual < 0.1
        plain = eng.process(ks, kr, n, v, pa.FLAG_COMPRESS)
        assert np.array_equal(out, plain ^ kr.astype(">u4").view(np.uint8))
        with pytest.raises(pa.PAError):
            eng.set_seed(np.zeros((n + 1024) // 32, np.uint32), n + 1024, -1)
    blk = O.DirectBlock(seed, ks, n, v)
    krb = O.bits_msb(kr, v).astype(np.uint8)
    for r0 in (0, 64 * 1234567, v - 64):
        assert np.array_equal(np.unpackbits(out[r0 // 8: r0 // 8 + 8]), blk.rows(r0, r0 + 64) ^ krb[r0: r0 + 64]), r0
    blk.close()


def structured_families(n, v):
    """Inputs that concentrate the convolution's spectrum: runs of ones of several lengths, all ones,
    periodic bit patterns and a single set bit, each with an all-ones and a random key."""
    rng = np.random.default_rng(n + v)
    words = n // 32
    fams = {}
    for frac in (2, 4, 8, 16):
        s = np.zeros(words, np.uint32)
        s[: words // frac] = 0xFFFFFFFF
        fams["run_1/%d" % frac] = s
    fams["ones"] = np.full(words, 0xFFFFFFFF, np.uint32)
    fams["alt"] = np.full(words, 0xAAAAAAAA, np.uint32)
    fams["bytes"] = np.full(words, 0xFF00FF00, np.uint32)
    one = np.zeros(words, np.uint32)
    one[0] = 0x80000000
    fams["single"] = one
    keys = {"ones": np.full(words + 1, 0xFFFFFFFF, np.uint32),
            "random": rng.integers(0, 1 << 32, words + 1, dtype=np.uint64).astype(np.uint32)}
    return fams, keys


@pytest.mark.parametrize("logn", [10, 12, 14, 15])
def test_single_cta_blocks_stay_within_fp32_budget(gpu_engine, logn):
    """Blocks up to n = 2^15 run in one CTA (the path pa_process_noalloc uses, which has no guard): over
    structured inputs that concentrate the spectrum, the FP32 residual stays below half the 0.25 guard and
    every output is exact."""
    n = 1 << logn
    v = n // 4 + n // 8
    fams, keys = structured_families(n, v)
    worst = 0.0
    for fname, seed in fams.items():
        for kname, recv in keys.items():
            ks, kr = O.key_split(recv, n, v)
            gpu_engine.set_seed(seed, n, -1)
            out = gpu_engine.process(ks, kr, n, v)
            st = gpu_engine.last_stats
            assert st.exact == 0, (fname, kname, st.max_residual)
            worst = max(worst, st.max_residual)
            assert np.array_equal(out, O.direct(seed, ks, kr, n, v)), (fname, kname)
    print("n=2^%d worst residual %.4f" % (logn, worst))
    assert worst < 0.125, worst
