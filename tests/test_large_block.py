"""Large-block decomposition (privacyamplification_gb300/large_block.py).

CPU: the chunk arithmetic against whole-block oracle results, driven by a stand-in engine whose blocks
are computed by the oracle; and the reference's LargeBlocksizeExample known answer (Matrix.h: pre-XOR
and final SHA3-256 of the n = 2^14 composite) through the general module with 1024-bit chunks.
GPU: the real engine, against single blocks, including n = 2^28 against the exact path."""
import hashlib

import numpy as np
import pytest

import privacyamplification_gb300 as pa
from privacyamplification_gb300 import large_block as L
import large_block as LB
from oracle import oracle as O

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS


class OracleEngine:
    """set_seed / process with pa_process semantics, computed by the oracle (test stand-in only)."""

    def __init__(self, max_sample_size):
        self.max_sample_size = max_sample_size
        self.calls = self.seeds = 0

    def set_seed(self, seed, n, reuse):
        self.seed, self.left = np.array(seed, dtype=np.uint32), reuse
        self.seeds += 1

    def process(self, ks, kr, n, v, flags):
        assert self.left != 0
        self.left -= 1
        self.calls += 1
        return O.direct(self.seed, ks, kr, n, v, flags)


@pytest.mark.parametrize("n,v,flags,side", [
    (8192, 3072, DEFAULT, 512), (8192, 3072, 0, 1024), (12288, 5120, pa.FLAG_COMPRESS, 512),
    (10240, 1024, DEFAULT, 2048), (9984, 3968, pa.FLAG_XOR_KEY_REST, 512)])
def test_decomposition_matches_whole_block(pa_lib, n, v, flags, side):
    seed, recv = O.random_block(n, v, n + v + flags)
    ks, kr = O.key_split(recv, n, v)
    ks_dirty = ks.copy()
    ks_dirty[(n - v) // 32 + 1:] = 0xDEADBEEF  # bits past h must be ignored
    eng = OracleEngine(2 * side)
    got = L.hash_large_block(eng, seed, ks_dirty, kr, n, v, flags, side=side)
    assert np.array_equal(got, O.direct(seed, ks, kr, n, v, flags))
    A, B, _ = L.plan(n, v, flags, side)
    assert eng.calls == A * B and eng.seeds == A + B - 1  # one seed spectrum per chunk diagonal


def test_reference_kat_through_decomposition(pa_lib, golden):
    kb, sb = np.unpackbits(golden["key_bits"]), np.unpackbits(golden["seed_bits"])
    seed, recv = LB.composite_inputs(kb, sb)
    ks, kr = O.key_split(recv, LB.N_BIG, LB.V_BIG)
    eng = OracleEngine(2048)
    pre = L.hash_large_block(eng, seed, ks, kr, LB.N_BIG, LB.V_BIG, pa.FLAG_COMPRESS, side=1024)
    assert hashlib.sha3_256(bytes(pre)).digest() == bytes(golden["pre_hash"])
    out = L.hash_large_block(eng, seed, ks, kr, LB.N_BIG, LB.V_BIG, DEFAULT, side=1024)
    assert hashlib.sha3_256(bytes(out)).digest() == bytes(golden["result_hash"])


@pytest.mark.gpu
def test_decomposition_on_gpu_matches_single_block(gpu_engine, golden):
    kb, sb = np.unpackbits(golden["key_bits"]), np.unpackbits(golden["seed_bits"])
    seed, recv = LB.composite_inputs(kb, sb)
    ks, kr = O.key_split(recv, LB.N_BIG, LB.V_BIG)
    out = L.hash_large_block(gpu_engine, seed, ks, kr, LB.N_BIG, LB.V_BIG, DEFAULT, side=1024)
    assert hashlib.sha3_256(bytes(out)).digest() == bytes(golden["result_hash"])
    for n, v, side in [(1 << 20, 393216, 1 << 14), (1 << 20, 393216, 1 << 18), (99328, 9984, 4096)]:
        seed, recv = O.random_block(n, v, 3 * n + side)
        ks, kr = O.key_split(recv, n, v)
        gpu_engine.set_seed(seed, n, -1)
        want = gpu_engine.process(ks, kr, n, v)
        assert np.array_equal(L.hash_large_block(gpu_engine, seed, ks, kr, n, v, side=side), want), (n, side)


@pytest.mark.gpu
def test_decomposition_2p28_fp32_chunks_equal_exact_block(pa_lib):
    """n = 2^28 is beyond one FP32 pass: the Python decomposition with 2^27-bit chunk blocks and the
    engine's own chunked block both reproduce the exact path."""
    n = 1 << 28
    v = n // 4 + n // 8
    rng = np.random.default_rng(28)
    seed = rng.integers(0, 1 << 32, n // 32, dtype=np.uint64).astype(np.uint32)
    recv = rng.integers(0, 1 << 32, n // 32 + 1, dtype=np.uint64).astype(np.uint32)
    ks, kr = pa.key_split(recv, n, v)
    with pa.Engine(max_sample_size=n) as eng:
        eng.set_seed(seed, n, -1)
        want = eng.process(ks, kr, n, v, DEFAULT | pa.FLAG_EXACT)
        assert eng.last_stats.exact == 1
        chunked = eng.process(ks, kr, n, v)
        assert eng.last_stats.exact == 2
        got = L.hash_large_block(eng, seed, ks, kr, n, v, side=1 << 26)
    assert np.array_equal(got, want) and np.array_equal(chunked, want)
