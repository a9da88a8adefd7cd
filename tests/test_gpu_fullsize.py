"""Whole-output parity at the configuration sizes, against the exact CPU oracle (an NTT modulo
2^64 - 2^32 + 1 on all host cores; its values are exact integers, so the parity of every output is known).

Every output byte of each block is compared -- no sampled rows:

* the bench workload, n = 2^27 (h = 83,886,080, v = 50,331,648) with the bench's own inputs (seed from
  PCG64 0x5EED, keys from 0x5EED + 1 ..), static seed, XOR + compression: one block at a time through
  pa_process, and two blocks in flight through the slot pool with the cached spectrum (pa_batch_run);
* the run-structured 2^27 block (first n/2 seed bits one, all-ones key): the FP32 guard trips and the
  exact path recomputes the block;
* the all-ones 2^27 block, whose every convolution value is h + 1 (checked in closed form);
* one n = 2^29 block with its own seed (the FP32 path in 2^27-bit chunk blocks);
* a config-4 draw: 32 blocks, n log-uniform in [2^18, 2^25], v/n uniform in [0.1, 0.9], half with a
  cached static seed, half with their own, as one CUDA graph (pa_batch_run with PA_BATCH_GRAPH), captured
  and then replayed;
* a config-5 draw: 16 served requests, n log-uniform in [2^20, 2^27], v/n uniform in [0.2, 0.8], arriving
  faster than they complete (pa_submit / pa_poll), so they overlap on the device.

Oracle wall time on 16 host cores is a few seconds per 2^27 block and about 20 s for the 2^29 block.
"""
import numpy as np
import pytest

import privacyamplification_gb300 as pa
from privacyamplification_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS
N27, V27 = 1 << 27, 50331648


@pytest.fixture(scope="module")
def torch_cuda(pa_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a CUDA device")
    return torch


@pytest.fixture(scope="module")
def bench_inputs(pa_lib):
    """The bench's seed and its first two keys, with the oracle's output for each (seed transform once)."""
    seed, _ = O.random_block(N27, V27, 0x5EED)
    keys = []
    for i in range(2):
        _, recv = O.random_block(N27, V27, 0x5EED + 1 + i)
        keys.append(O.key_split(recv, N27, V27))
    ref = O.NttSeed(seed, N27, V27)
    try:
        want = [ref.block(ks, kr, DEFAULT) for ks, kr in keys]
    finally:
        ref.close()
    return seed, keys, want


def test_bench_block_whole_output(gpu_engine, bench_inputs):
    seed, keys, want = bench_inputs
    gpu_engine.set_seed(seed, N27, -1)
    for (ks, kr), w in zip(keys, want):
        out = gpu_engine.process(ks, kr, N27, V27, DEFAULT)
        st = gpu_engine.last_stats
        assert st.exact == 0 and st.max_residual < 0.1, st.as_dict()
        assert out.size == V27 // 8
        bad = np.flatnonzero(out != w)
        assert bad.size == 0, "%d of %d bytes differ, first at %s" % (bad.size, out.size, bad[:8])


def test_bench_blocks_in_flight_whole_output(torch_cuda, bench_inputs):
    """The bench's headline form: two blocks in flight on two slots of the pool, spectrum cached once."""
    seed, keys, want = bench_inputs
    dev = torch_cuda.device("cuda")
    t = lambda a: torch_cuda.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)
    with pa.Engine(max_sample_size=N27) as eng:
        sid = eng.seed_cache_add(seed, N27, V27)
        eng.set_pool(0, 16, 2)
        d_keys = [(t(ks), t(kr)) for ks, kr in keys]
        outs = [torch_cuda.full((V27 // 8,), 0xA5, dtype=torch_cuda.uint8, device=dev) for _ in range(4)]
        jobs = [pa.PAJob(None, sid, d_keys[i % 2][0].data_ptr(), d_keys[i % 2][1].data_ptr(), N27, V27, DEFAULT,
                         outs[i].data_ptr()) for i in range(4)]
        eng.batch_run(jobs)
        stats = eng.batch_sync(len(jobs))
        assert all(s.exact == 0 and s.max_residual < 0.1 for s in stats)
        for i in range(4):
            assert np.array_equal(outs[i].cpu().numpy(), want[i % 2]), i


def test_run_structured_2p27_whole_output(gpu_engine):
    """The FP32-breaking block at the headline size: guard fallback to the exact path, every bit checked."""
    n, v = N27, V27
    seed = np.zeros(n // 32, np.uint32)
    seed[: n // 64] = 0xFFFFFFFF
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, -1)
    out = gpu_engine.process(ks, kr, n, v, DEFAULT)
    st = gpu_engine.last_stats
    assert st.max_residual > 0.25 and st.exact == 1, st.as_dict()
    assert np.array_equal(out, O.ntt(seed, ks, kr, n, v, DEFAULT))


def test_all_ones_2p27_closed_form(gpu_engine):
    """All-ones key and seed: every convolution value is h + 1, so output bit i is (h + 1) mod 2 XOR
    key_rest bit i; the FP32 path holds it (the seed spectrum is pure DC, which the path drops)."""
    n, v = N27, V27
    h = n - v
    seed = np.full(n // 32, 0xFFFFFFFF, np.uint32)
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, -1)
    out = gpu_engine.process(ks, kr, n, v, DEFAULT)
    assert gpu_engine.last_stats.exact == 0
    par = np.full(v, (h + 1) & 1, np.uint8)
    assert np.array_equal(out, O.pack_output(par, kr, v, DEFAULT))
    plain = gpu_engine.process(ks, kr, n, v, 0)  # no XOR, n/2 output bits
    assert np.array_equal(plain, O.pack_output(np.full(n // 2, (h + 1) & 1, np.uint8), None, v, 0))


def test_config3_2p29_whole_output(pa_lib):
    """n = 2^29 with its own seed: the FP32 path as 2^27-bit chunk blocks, whole output against the oracle."""
    n = 1 << 29
    v = n // 4 + n // 8
    seed, recv = O.random_block(n, v, 2929)
    ks, kr = O.key_split(recv, n, v)
    with pa.Engine(max_sample_size=n) as eng:
        eng.set_seed(seed, n, 0)
        out = eng.process(ks, kr, n, v, DEFAULT)
        st = eng.last_stats
    assert st.exact == 2 and st.max_residual < 0.1, st.as_dict()
    assert np.array_equal(out, O.ntt(seed, ks, kr, n, v, DEFAULT))


def test_config4_draw_graph_whole_output(torch_cuda):
    """32 blocks of the config-4 distribution as one captured and replayed CUDA graph."""
    blocks = W.uneven_mix(count=32, lo=18, hi=25, rng_seed=0xC0F4)
    assert min(b.n for b in blocks) >= 1 << 18 and max(b.n for b in blocks) <= 1 << 25
    with pa.Engine(max_sample_size=1 << 25) as eng:
        mix = W.DeviceMix(eng, blocks)
        want = [O.ntt(mix.seed_words(b), mix.key_start(b), mix.key_rest(b), b.n, b.v, b.flags) for b in blocks]
        for rep in range(2):  # capture, then replay
            mix.d_out.fill_(0x5A)
            stats = mix.run(pa.BATCH_GRAPH)
            got = mix.outputs()
            for i, b in enumerate(blocks):
                assert np.array_equal(got[i], want[i]), (rep, i, b)
            assert all(s.exact == 0 for s in stats)


def test_config5_draw_served_whole_output(torch_cuda):
    """16 requests of the config-5 distribution arriving at 2000/s, served with overlap on the device."""
    reqs = W.poisson_requests(rate=2000, count=16, lo=20, hi=27, rng_seed=0x5E7E)
    assert min(r.n for r in reqs) >= 1 << 20 and max(r.n for r in reqs) <= 1 << 27
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    with pa.Engine(max_sample_size=1 << 27) as eng:
        eng.set_pool(max_slots=4)
        res = W.serve(eng, reqs, banks, out_slots=6, keep=lambda r: True)
    assert len(res.outputs) == len(reqs)
    for r in reqs:
        want = O.ntt(banks.seed_words(r), banks.key_start(r), banks.key_rest(r), r.n, r.v, r.flags)
        assert np.array_equal(res.outputs[r.rid], want), r
