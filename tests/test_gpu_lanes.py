"""The persistent lane launch (PA_BATCH_PERSISTENT) through the C ABI, against the exact CPU oracle.

A batch runs as one persistent kernel whose lanes of CTAs take the blocks longest first; every block's
output is compared in full with the oracle: uneven mixes (static and own seeds, all flag combinations,
sizes below the lanes' smallest cyclic length of 2^20), the config-4 distribution as a captured and
replayed graph, several lane widths, the headline 2^27 block, and a block that trips the FP32 guard.
"""
import numpy as np
import pytest

import privacyamplification_gb300 as pa
from privacyamplification_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS
PERSIST = pa.BATCH_PERSISTENT


@pytest.fixture(scope="module")
def torch_cuda(pa_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a CUDA device")
    return torch


def oracle_outputs(mix, blocks):
    return [O.ntt(mix.seed_words(b), mix.key_start(b), mix.key_rest(b), b.n, b.v, b.flags) for b in blocks]


def check(mix, blocks, want, flags, reps=1):
    for rep in range(reps):
        mix.d_out.fill_(0xC3)
        stats = mix.run(flags)
        got = mix.outputs()
        for i, b in enumerate(blocks):
            assert np.array_equal(got[i], want[i]), (flags, rep, i, b)
        assert all(s.exact == 0 and s.max_residual < 0.25 for s in stats)
    return stats


def test_small_mix_all_flags(torch_cuda):
    """Blocks of 2^12 .. 2^21 bits (most placed in the lanes' smallest cyclic length 2^20), static and own
    seeds, all four flag combinations, powers of two and not."""
    blocks = W.uneven_mix(count=24, lo=12, hi=21, rng_seed=0x1A9E)
    blocks[3].flags = 0
    blocks[5].flags = pa.FLAG_COMPRESS
    blocks[7].flags = pa.FLAG_XOR_KEY_REST
    blocks.append(W.Block(n=1 << 16, v=24576, static=True))
    blocks.append(W.Block(n=1 << 20, v=1 << 18, static=True, flags=0))
    with pa.Engine(max_sample_size=1 << 22) as eng:
        mix = W.DeviceMix(eng, blocks)
        want = oracle_outputs(mix, blocks)
        check(mix, blocks, want, PERSIST, reps=2)
        check(mix, blocks, want, 0)  # the per-pass form on the same engine agrees


def test_config4_draw_persistent_graph(torch_cuda):
    """The config-4 distribution (n log-uniform in [2^18, 2^25]) as one persistent launch, then as its
    captured graph (capture, replay)."""
    blocks = W.uneven_mix(count=48, lo=18, hi=25, rng_seed=0xC0F4)
    with pa.Engine(max_sample_size=1 << 25) as eng:
        mix = W.DeviceMix(eng, blocks)
        want = oracle_outputs(mix, blocks)
        check(mix, blocks, want, PERSIST)
        check(mix, blocks, want, PERSIST | pa.BATCH_GRAPH, reps=2)


@pytest.mark.parametrize("ctas", [1, 2, 8, 38])
def test_lane_widths(torch_cuda, ctas):
    blocks = W.uneven_mix(count=10, lo=16, hi=23, rng_seed=0x1A4E + ctas)
    with pa.Engine(max_sample_size=1 << 23) as eng:
        lanes = eng.set_lanes(ctas, 1 << 23)
        assert lanes >= 1
        mix = W.DeviceMix(eng, blocks)
        want = oracle_outputs(mix, blocks)
        check(mix, blocks, want, PERSIST)


def test_headline_block_on_lanes(torch_cuda):
    """n = 2^27 with the bench's inputs, two keys, on lanes of 38 CTAs (four lanes)."""
    n, v = 1 << 27, 50331648
    seed, _ = O.random_block(n, v, 0x5EED)
    keys = []
    for i in range(2):
        _, recv = O.random_block(n, v, 0x5EED + 1 + i)
        keys.append(O.key_split(recv, n, v))
    ref = O.NttSeed(seed, n, v)
    want = [ref.block(ks, kr, DEFAULT) for ks, kr in keys]
    ref.close()
    dev = torch_cuda.device("cuda")
    t = lambda a: torch_cuda.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)
    with pa.Engine(max_sample_size=n) as eng:
        assert eng.set_lanes(38, n) >= 1
        sid = eng.seed_cache_add(seed, n, v)
        d_keys = [(t(ks), t(kr)) for ks, kr in keys]
        outs = [torch_cuda.full((v // 8,), 0x3C, dtype=torch_cuda.uint8, device=dev) for _ in range(2)]
        jobs = [pa.PAJob(None, sid, d_keys[i][0].data_ptr(), d_keys[i][1].data_ptr(), n, v, DEFAULT,
                         outs[i].data_ptr()) for i in range(2)]
        eng.batch_run(jobs, PERSIST)
        stats = eng.batch_sync(2)
        assert all(s.exact == 0 and s.max_residual < 0.1 for s in stats), [s.as_dict() for s in stats]
        for i in range(2):
            assert np.array_equal(outs[i].cpu().numpy(), want[i]), i
        # the same key with its own seed (seed stages on the lane)
        d_seed = t(seed)
        jobs[1] = pa.PAJob(d_seed.data_ptr(), -1, d_keys[1][0].data_ptr(), d_keys[1][1].data_ptr(), n, v, DEFAULT,
                           outs[1].data_ptr())
        outs[1].fill_(0)
        torch_cuda.cuda.synchronize()
        eng.batch_run(jobs, PERSIST)
        eng.batch_sync(2)
        assert np.array_equal(outs[1].cpu().numpy(), want[1])


def test_guard_recomputes_exactly_on_lanes(torch_cuda):
    """A run-structured block (FP32 budget exceeded) among ordinary ones: recomputed exactly at sync."""
    n, v = 1 << 22, (1 << 20) + (1 << 19)
    seed = np.zeros(n // 32, np.uint32)
    seed[: n // 64] = 0xFFFFFFFF
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    ks, kr = O.key_split(recv, n, v)
    dev = torch_cuda.device("cuda")
    t = lambda a: torch_cuda.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)
    d_seed, d_ks, d_kr = t(seed), t(ks), t(kr)
    seed2, recv2 = O.random_block(n, v, 77)
    ks2, kr2 = O.key_split(recv2, n, v)
    d_seed2, d_ks2, d_kr2 = t(seed2), t(ks2), t(kr2)
    outs = [torch_cuda.zeros(v // 8, dtype=torch_cuda.uint8, device=dev) for _ in range(2)]
    with pa.Engine(max_sample_size=n) as eng:
        jobs = [pa.PAJob(d_seed.data_ptr(), -1, d_ks.data_ptr(), d_kr.data_ptr(), n, v, DEFAULT, outs[0].data_ptr()),
                pa.PAJob(d_seed2.data_ptr(), -1, d_ks2.data_ptr(), d_kr2.data_ptr(), n, v, DEFAULT,
                         outs[1].data_ptr())]
        eng.batch_run(jobs, PERSIST)
        st = eng.batch_sync(2)
    assert st[0].max_residual > 0.25 and st[0].exact == 1
    assert st[1].exact == 0
    assert np.array_equal(outs[0].cpu().numpy(), O.ntt(seed, ks, kr, n, v))
    assert np.array_equal(outs[1].cpu().numpy(), O.ntt(seed2, ks2, kr2, n, v))
