"""GPU: a seed that serves one block only is transformed inside that block's column pass.

With reuse_seed_amount 0 or 1 and columns of 2^10 .. 2^12 (n >= 2^21), the seed's row pass writes where
its spectrum would go and one column pass transforms each seed tile, parks its spectrum tile in L2 and
runs the key tile against it.  The spectrum values are the same arithmetic as the cached-spectrum path,
so the output, the residual and both popcounts must equal that path's exactly, and the output the
exact CPU oracle's.
"""
import numpy as np
import pytest

import privacyamplification_gb300 as pa
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS


def one_use_and_cached(eng, seed, ks, kr, n, v, flags):
    eng.set_seed(seed, n, 1)
    fused = eng.process(ks, kr, n, v, flags)
    sf = eng.last_stats
    eng.set_seed(seed, n, -1)
    cached = eng.process(ks, kr, n, v, flags)
    sc = eng.last_stats
    return fused, sf, cached, sc


@pytest.mark.parametrize("n,v,flags", [
    (1 << 21, (1 << 19) + (1 << 18), DEFAULT),                    # columns of 2^10
    (1 << 22, (1 << 20) + (1 << 19), DEFAULT),                    # columns of 2^11
    (1 << 23, 1 << 21, pa.FLAG_COMPRESS),                         # columns of 2^12
    (3 << 20, 1 << 20, pa.FLAG_XOR_KEY_REST),                     # placed seed, cyclic length 2^22
    ((1 << 24) + (1 << 20), 5 << 20, DEFAULT),                    # placed seed, cyclic length 2^25
    (1 << 24, 1 << 22, 0),
])
def test_one_use_seed_equals_cached_and_oracle(gpu_engine, n, v, flags):
    seed, recv = O.random_block(n, v, 7000 + n % 997 + flags)
    ks, kr = pa.key_split(recv, n, v)
    fused, sf, cached, sc = one_use_and_cached(gpu_engine, seed, ks, kr, n, v, flags)
    assert np.array_equal(fused, cached)
    assert sf.exact == 0 and sc.exact == 0
    assert sf.max_residual == sc.max_residual and sf.max_residual < 0.1
    assert (sf.popcount_key, sf.popcount_seed) == (sc.popcount_key, sc.popcount_seed)
    assert sf.popcount_seed > 0 and sf.popcount_key > 0
    ref = O.ntt(seed, ks, kr, n, v, flags)
    assert np.array_equal(fused, ref)


def test_one_use_seed_full_size(gpu_engine):
    """n = 2^27 (columns of 2^12, rows of 2^14): fused and cached paths agree bit for bit."""
    n, v = 1 << 27, (1 << 25) + (1 << 24)
    seed, recv = O.random_block(n, v, 2727)
    ks, kr = pa.key_split(recv, n, v)
    fused, sf, cached, sc = one_use_and_cached(gpu_engine, seed, ks, kr, n, v, DEFAULT)
    assert np.array_equal(fused, cached)
    assert sf.max_residual == sc.max_residual and sf.max_residual < 0.1
    assert (sf.popcount_key, sf.popcount_seed) == (sc.popcount_key, sc.popcount_seed)


def test_one_use_seed_guard_fallback(gpu_engine):
    """A run-structured one-use block exceeds the FP32 budget in the fused pass as in the cached one and
    is recomputed exactly."""
    n, v = 1 << 22, (1 << 20) + (1 << 19)
    seed = np.zeros(n // 32, np.uint32)
    seed[: n // 64] = 0xFFFFFFFF
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    ks, kr = pa.key_split(recv, n, v)
    fused, sf, cached, sc = one_use_and_cached(gpu_engine, seed, ks, kr, n, v, DEFAULT)
    assert sf.max_residual == sc.max_residual and sf.max_residual > 0.25
    assert sf.exact == 1 and sc.exact == 1
    assert np.array_equal(fused, cached)
    assert np.array_equal(fused, O.ntt(seed, ks, kr, n, v, DEFAULT))


def test_seed_sequence_switches_paths(gpu_engine):
    """A seed for two blocks (cached spectrum), then one-use seeds (fused), then a static seed: every
    block against the oracle, so no path reads a spectrum another one left behind."""
    n, v = 1 << 22, (1 << 20) + (1 << 19)
    rng = np.random.default_rng(4242)
    words = lambda k: rng.integers(0, 1 << 32, k, dtype=np.uint64).astype(np.uint32)
    plan = [2, None, 1, 0, -1, None, None]  # reuse per new seed; None: another block, same seed
    seed = None
    for step, reuse in enumerate(plan):
        if reuse is not None:
            seed = words(n // 32)
            gpu_engine.set_seed(seed, n, reuse)
        recv = words(n // 32 + 1)
        ks, kr = pa.key_split(recv, n, v)
        out = gpu_engine.process(ks, kr, n, v, DEFAULT)
        assert gpu_engine.last_stats.exact == 0
        assert np.array_equal(out, O.ntt(seed, ks, kr, n, v, DEFAULT)), step
