"""The engine against the reference's plain cuFFT pipeline (baseline/cufft_plain.cu) on the same inputs,
with the pipeline's restated kernels and with the reference's own kernels (compiled from
PrivacyAmplification.cu into baseline/_ref_cuda/ by baseline/ref_cuda.py).

Both must equal the oracle where the oracle finishes quickly; at n = 2^27 the engine's output must be
SHA3-equal to the cuFFT pipeline's on identical inputs (the reference's own 2^27 golden files are not
available, so this is the stand-in for its SHA3 check).
"""
import numpy as np
import pytest

import privacyamplification_gb300 as pa
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS


@pytest.fixture(scope="module")
def plain_lib():
    from baseline import cufft_plain
    cufft_plain.build()
    return cufft_plain


def flags_of(do_xor, do_compress):
    return (pa.FLAG_XOR_KEY_REST if do_xor else 0) | (pa.FLAG_COMPRESS if do_compress else 0)


@pytest.mark.parametrize("logn,do_xor,do_compress", [(16, True, True), (16, False, False), (18, False, True),
                                                      (20, True, True)])
def test_plain_matches_oracle_and_engine(plain_lib, gpu_engine, logn, do_xor, do_compress):
    n = 1 << logn
    v = n // 4 + n // 8
    flags = flags_of(do_xor, do_compress)
    cp = plain_lib.CufftPlain(n, v)
    seed, _ = O.random_block(n, v, 500 + logn)
    try:
        for blk in range(3):  # static seed: computed on the first block, reused after
            _, recv = O.random_block(n, v, 900 + 7 * logn + blk)
            ks, kr = O.key_split(recv, n, v)
            cp.load(seed=seed if blk == 0 else None, key_start=ks, key_rest=kr)
            cp.process(recalc_seed=(blk == 0), do_xor=do_xor, do_compress=do_compress)
            ob = pa.output_bytes(n, v, flags)
            got = cp.output(ob)
            gpu_engine.set_seed(seed, n, -1)
            mine = gpu_engine.process(ks, kr, n, v, flags)
            assert np.array_equal(got, mine), blk
            if n <= 1 << 16:
                assert np.array_equal(got, O.direct(seed, ks, kr, n, v, flags)), blk
            else:
                assert np.array_equal(got, O.ntt(seed, ks, kr, n, v, flags)), blk
    finally:
        cp.close()


def test_2p27_sha3_equal_to_plain_cufft(plain_lib, gpu_engine):
    """Config-2 size: engine bits SHA3-equal to the cuFFT pipeline's on the same inputs, static seed,
    two consecutive key blocks, plus both residuals well inside the rounding budget."""
    n, v = 1 << 27, 50331648
    seed, recv = O.random_block(n, v, 0x5EED)
    cp = plain_lib.CufftPlain(n, v)
    try:
        gpu_engine.set_seed(seed, n, -1)
        cp.load(seed=seed)
        for blk in range(2):
            if blk:
                _, recv = O.random_block(n, v, 0x5EED + blk)
            ks, kr = O.key_split(recv, n, v)
            cp.load(key_start=ks, key_rest=kr)
            cp.process(recalc_seed=(blk == 0))
            got = cp.output(v // 8)
            mine = gpu_engine.process(ks, kr, n, v, DEFAULT)
            assert O.sha3_256(got.tobytes()) == O.sha3_256(mine.tobytes()), blk
            assert cp.residual(v) < 0.25
            assert gpu_engine.last_stats.max_residual < 0.25
    finally:
        cp.close()


@pytest.fixture(scope="module")
def ref_kernels(plain_lib):
    from baseline import ref_cuda
    fb = ref_cuda.fatbin()
    if fb is None:
        pytest.skip("the reference's kernels were not compiled (its source tree was absent at build time)")
    return fb


@pytest.mark.parametrize("logn,do_xor,do_compress", [(16, True, True), (17, False, False), (20, False, True)])
def test_reference_kernels_match_engine_and_oracle(plain_lib, ref_kernels, gpu_engine, logn, do_xor, do_compress):
    """The reference's own binInt2float / correction / DC zero / product / ToBinaryArray[NoXOR] kernels with
    cuFFT give the engine's bits and the oracle's, static seed over three blocks."""
    n = 1 << logn
    v = n // 4 + n // 8
    flags = flags_of(do_xor, do_compress)
    cp = plain_lib.CufftPlain(n, v)
    cp.use_reference_kernels(ref_kernels)
    seed, _ = O.random_block(n, v, 700 + logn)
    try:
        for blk in range(3):
            _, recv = O.random_block(n, v, 1900 + 7 * logn + blk)
            ks, kr = O.key_split(recv, n, v)
            cp.load(seed=seed if blk == 0 else None, key_start=ks, key_rest=kr)
            cp.process(recalc_seed=(blk == 0), do_xor=do_xor, do_compress=do_compress)
            got = cp.output(pa.output_bytes(n, v, flags))
            gpu_engine.set_seed(seed, n, -1)
            assert np.array_equal(got, gpu_engine.process(ks, kr, n, v, flags)), blk
            assert np.array_equal(got, O.ntt(seed, ks, kr, n, v, flags)), blk
    finally:
        cp.use_restated_kernels()
        cp.close()


def test_2p27_sha3_equal_to_reference_kernels(plain_lib, ref_kernels, gpu_engine):
    """The bench's n = 2^27 inputs: the engine's output SHA3-equal to the reference's own kernels + cuFFT."""
    n, v = 1 << 27, 50331648
    seed, _ = O.random_block(n, v, 0x5EED)
    cp = plain_lib.CufftPlain(n, v)
    cp.use_reference_kernels(ref_kernels)
    try:
        gpu_engine.set_seed(seed, n, -1)
        cp.load(seed=seed)
        for blk in range(2):
            _, recv = O.random_block(n, v, 0x5EED + 1 + blk)
            ks, kr = O.key_split(recv, n, v)
            cp.load(key_start=ks, key_rest=kr)
            cp.process(recalc_seed=(blk == 0))
            got = cp.output(v // 8)
            mine = gpu_engine.process(ks, kr, n, v, DEFAULT)
            assert O.sha3_256(got.tobytes()) == O.sha3_256(mine.tobytes()), blk
    finally:
        cp.use_restated_kernels()
        cp.close()


@pytest.mark.parametrize("log_s,B", [(16, 8), (20, 2)])
def test_sub_block_bank_matches_oracle_and_engine(plain_lib, log_s, B):
    """The sub-block bank (B equal blocks on batched cuFFT plans) and the engine's batch of the same blocks
    (static: one cached spectrum per block; dynamic: each block's own seed) against the oracle, block by
    block, and against each other."""
    from privacyamplification_gb300 import workloads as W
    s, v, seeds, ks, kr = W.sub_block_bank(log_s, bank_bits=B << log_s, rng_seed=0x5B + log_s)
    want = [(O.direct if s <= 1 << 16 else O.ntt)(seeds[i], ks[i], kr[i], s, v, DEFAULT) for i in range(B)]
    bank = plain_lib.CufftBank(s, v, B)
    try:
        bank.load(seeds, ks, kr)
        for recalc in (False, False, True):  # static: computed once, then reused; then recomputed
            bank.run(recalc_seed=recalc)
            got = bank.outputs()
            for i in range(B):
                assert np.array_equal(got[i], want[i]), (recalc, i)
    finally:
        bank.close()
    with pa.Engine(max_sample_size=s) as eng:
        for static in (True, False):
            db = W.DeviceBank(eng, s, v, seeds, ks, kr, static)
            for rep in range(2):
                stats = db.run(pa.BATCH_GRAPH)
                assert all(x.exact == 0 for x in stats)
                mine = db.outputs()
                for i in range(B):
                    assert np.array_equal(mine[i], want[i]), (static, rep, i)
            del db
