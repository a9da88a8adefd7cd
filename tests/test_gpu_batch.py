"""Slot pool through the C ABI: every three-pass split, batched uneven mixes (serial, concurrent, CUDA
graph) and the served form (pa_submit / pa_poll) -- each block bit-exact with the same block alone."""
import numpy as np
import pytest

import privacyamplification_gb300 as pa
from privacyamplification_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS


@pytest.fixture(scope="module")
def torch_cuda(pa_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a CUDA device")
    return torch


@pytest.fixture()
def engine(pa_lib):
    eng = pa.Engine(max_sample_size=1 << 25)
    yield eng
    eng.close()


@pytest.mark.parametrize("log_n", [15, 17, 19, 21, 22, 24])
def test_every_split_matches_oracle(engine, log_n):
    n = 1 << (log_n + 1)
    v = n // 4 + n // 8
    seed, recv = O.random_block(n, v, 77 + log_n)
    ks, kr = O.key_split(recv, n, v)
    ref = O.ntt(seed, ks, kr, n, v)
    lo, hi = max(10, log_n - 12), min(14, log_n - 5)
    for l2 in range(lo, hi + 1):
        engine.set_split(log_n, l2)
        assert engine.get_split(log_n) == l2
        engine.set_seed(seed, n, -1)
        assert np.array_equal(engine.process(ks, kr, n, v), ref), l2


def test_split_rejects_out_of_range(engine):
    with pytest.raises(pa.PAError):
        engine.set_split(20, 15)
    with pytest.raises(pa.PAError):
        engine.set_split(20, 7)


def alone(engine, seed, ks, kr, n, v, flags):
    engine.set_seed(seed, n, -1)
    return engine.process(ks, kr, n, v, flags)


def small_mix():
    blocks = W.uneven_mix(count=24, lo=12, hi=20, rng_seed=0xBEE)
    blocks[3].flags = 0                      # no XOR, no compression (n/16 output bytes)
    blocks[5].flags = pa.FLAG_COMPRESS       # compression without XOR
    return blocks


def test_batch_modes_match_alone(torch_cuda, engine):
    blocks = small_mix()
    mix = W.DeviceMix(engine, blocks)
    want = [alone(engine, mix.seed_words(b), mix.key_start(b), mix.key_rest(b), b.n, b.v, b.flags) for b in blocks]
    for i, b in enumerate(blocks[:6]):
        if b.n <= 1 << 16:
            assert np.array_equal(want[i], O.direct(mix.seed_words(b), mix.key_start(b), mix.key_rest(b), b.n, b.v,
                                                    b.flags)), i
    for mode in (pa.BATCH_SERIAL, 0, pa.BATCH_GRAPH, pa.BATCH_GRAPH):  # graph twice: capture, then replay
        mix.d_out.zero_()
        stats = mix.run(mode)
        got = mix.outputs()
        for i in range(len(blocks)):
            assert np.array_equal(got[i], want[i]), (mode, i, blocks[i])
        assert all(s.max_residual < 0.25 and s.exact == 0 for s in stats)


def test_batch_after_autotune(torch_cuda, engine):
    tuned = engine.autotune(1 << 16, 1 << 21)
    assert set(tuned) == set(range(15, 21))
    for ln, (l2, ms) in tuned.items():
        assert max(10, ln - 12) <= l2 <= min(14, ln - 5) and ms > 0
    blocks = small_mix()
    mix = W.DeviceMix(engine, blocks)  # spectra cached with the tuned splits
    want = [alone(engine, mix.seed_words(b), mix.key_start(b), mix.key_rest(b), b.n, b.v, b.flags) for b in blocks]
    mix.run(pa.BATCH_GRAPH)
    assert all(np.array_equal(g, w) for g, w in zip(mix.outputs(), want))


def test_batch_guard_recomputes_exactly(torch_cuda, engine):
    """A run-structured block (FP32 budget exceeded at n = 2^22) inside a batch comes back exact."""
    n, v = 1 << 22, (1 << 20) + (1 << 19)
    seed = np.zeros(n // 32, np.uint32)
    seed[: n // 64] = 0xFFFFFFFF
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    ks, kr = O.key_split(recv, n, v)
    dev = torch_cuda.device("cuda")
    t = lambda a: torch_cuda.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)
    d_seed, d_ks, d_kr = t(seed), t(ks), t(kr)
    d_out = torch_cuda.zeros(v // 8, dtype=torch_cuda.uint8, device=dev)
    job = pa.PAJob(d_seed.data_ptr(), -1, d_ks.data_ptr(), d_kr.data_ptr(), n, v, DEFAULT, d_out.data_ptr())
    engine.batch_run([job])
    st = engine.batch_sync(1)[0]
    assert st.max_residual > 0.25 and st.exact == 1
    assert np.array_equal(d_out.cpu().numpy(), O.ntt(seed, ks, kr, n, v))


def test_served_requests_match_alone(torch_cuda, engine):
    """Poisson arrivals faster than the GPU drains them: blocks overlap, queue and are admitted as slots
    free up; every result equals the same request alone."""
    reqs = W.poisson_requests(rate=4000, count=48, lo=14, hi=20, rng_seed=11)
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    engine.set_pool(max_slots=4)
    res = W.serve(engine, reqs, banks, out_slots=6, keep=lambda r: True)
    assert len(res.latency_ms) == len(reqs) and res.exact == 0
    for r in reqs:
        want = alone(engine, banks.seed_words(r), banks.key_start(r), banks.key_rest(r), r.n, r.v, r.flags)
        assert np.array_equal(res.outputs[r.rid], want), r


def test_served_static_seeds_and_busy(torch_cuda, engine):
    """Static (cached) seeds per power-of-two size; a budget of one slot forces PA_ERR_BUSY admission."""
    reqs = W.poisson_requests(rate=2000, count=16, lo=14, hi=18, static=True, rng_seed=12)
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    seed_ids = {}
    for r in reqs:
        if W.seed_key(r.n, r.v, r.flags) not in seed_ids:
            seed_ids[W.seed_key(r.n, r.v, r.flags)] = engine.seed_cache_add(banks.seed_words(r), r.n, r.v, r.flags)
    engine.set_pool(max_slots=1)
    res = W.serve(engine, reqs, banks, out_slots=4, keep=lambda r: True, seed_ids=seed_ids)
    assert len(res.latency_ms) == len(reqs)
    for r in reqs:
        want = alone(engine, banks.seed_words(r), banks.key_start(r), banks.key_rest(r), r.n, r.v, r.flags)
        assert np.array_equal(res.outputs[r.rid], want), r


def test_served_admission_evicts_idle_slots_within_budget(torch_cuda, engine):
    """A 30 MB budget holds one 2^21-bit slot (26.5 MB) but not it and a 2^20-bit one: growing blocks
    make the pool free idle slots first; a block that can never fit is refused with PA_ERR_TOO_LARGE."""
    engine.set_pool(hbm_budget_bytes=30 << 20, max_slots=4)
    sizes = [1 << 19, 1 << 20, 1 << 21, 1 << 19, 1 << 21]
    reqs = []
    for i, n in enumerate(sizes):
        v = n // 4 + n // 8
        reqs.append(W.Request(rid=i, arrival=0.0, n=n, v=v, static=False, seed_word0=64 * i, key_word0=128 * i))
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    res = W.serve(engine, reqs, banks, out_slots=1, keep=lambda r: True)  # one at a time
    for r in reqs:
        want = alone(engine, banks.seed_words(r), banks.key_start(r), banks.key_rest(r), r.n, r.v, r.flags)
        assert np.array_equal(res.outputs[r.rid], want), r
    big = W.Request(rid=9, arrival=0.0, n=1 << 22, v=(1 << 20) + (1 << 19), static=False, seed_word0=0, key_word0=0)
    banks2 = W.HostBanks(big.n // 32 + 64)
    out = np.zeros(big.v // 8, np.uint8)
    job = pa.PAJob(banks2.seed_words(big).ctypes.data, -1, banks2.key_start(big).ctypes.data,
                   banks2.key_rest(big).ctypes.data, big.n, big.v, DEFAULT, out.ctypes.data)
    with pytest.raises(pa.PAError) as ei:
        engine.submit(job)
    assert ei.value.code == pa.PA_ERR_TOO_LARGE


def test_pool_reserve_then_serve(torch_cuda, engine):
    """Reserved slots exist before any request: a budget for two 2^20-bit slots gives two; requests
    served afterwards still equal the same request alone."""
    per_slot = int(12.625 * (1 << 20)) + 8192
    engine.set_pool(hbm_budget_bytes=2 * per_slot + 4096, max_slots=8)
    assert engine.pool_reserve(1 << 20, 5) == 2
    assert engine.pool_reserve(1 << 20, 1) == 2  # already there
    with pytest.raises(pa.PAError):
        engine.pool_reserve(3 << 18, 1)  # not a power of two
    reqs = W.poisson_requests(rate=3000, count=12, lo=14, hi=20, rng_seed=21)
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    res = W.serve(engine, reqs, banks, out_slots=3, keep=lambda r: True)
    for r in reqs:
        want = alone(engine, banks.seed_words(r), banks.key_start(r), banks.key_rest(r), r.n, r.v, r.flags)
        assert np.array_equal(res.outputs[r.rid], want), r


def test_pool_refuses_blocks_beyond_one_fp32_pass(torch_cuda, engine):
    """Batches and served blocks run single-pass FP32 blocks (n <= 2^27); larger ones (pa_process's
    chunked path) are refused before any work is queued."""
    n, v = 1 << 28, (1 << 26) + (1 << 25)
    d = torch_cuda.zeros(16, dtype=torch_cuda.int32, device="cuda")
    p = d.data_ptr()
    job = pa.PAJob(p, -1, p, p, n, v, DEFAULT, p)
    with pytest.raises(pa.PAError) as ei:
        engine.batch_run([job])
    assert ei.value.code == pa.PA_ERR_TOO_LARGE
    host = np.zeros(4, np.uint32)
    hjob = pa.PAJob(host.ctypes.data, -1, host.ctypes.data, host.ctypes.data, n, v, DEFAULT, host.ctypes.data)
    with pytest.raises(pa.PAError) as ei:
        engine.submit(hjob)
    assert ei.value.code == pa.PA_ERR_TOO_LARGE


def test_two_slots_concurrently_many_times(torch_cuda, engine):
    """Two blocks of different sizes -- a power of two with a cached static seed, and a padded size with
    its own seed -- run concurrently on two slots, 200 times over (streams, then graph replays), and each
    result is compared with the oracle every time.  Slots share no mutable device state: each has its
    own working set, error word and tensor maps; per-job counters and residual words are per job; the
    cached spectrum is only read."""
    dev = torch_cuda.device("cuda")
    t = lambda a: torch_cuda.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)
    na, va = 1 << 22, 3 << 19
    nb, vb = 3 * (1 << 20) + 5 * 1024, 1234 * 128
    seed_a, recv_a = O.random_block(na, va, 0xA11)
    seed_b, recv_b = O.random_block(nb, vb, 0xB22)
    ks_a, kr_a = O.key_split(recv_a, na, va)
    ks_b, kr_b = O.key_split(recv_b, nb, vb)
    want_a = O.ntt(seed_a, ks_a, kr_a, na, va, DEFAULT)
    want_b = O.ntt(seed_b, ks_b, kr_b, nb, vb, pa.FLAG_COMPRESS)
    sid = engine.seed_cache_add(seed_a, na, va)
    engine.set_pool(0, 16, 2)
    d = [t(x) for x in (ks_a, kr_a, seed_b, ks_b, kr_b)]
    out_a = torch_cuda.zeros(va // 8, dtype=torch_cuda.uint8, device=dev)
    out_b = torch_cuda.zeros(vb // 8, dtype=torch_cuda.uint8, device=dev)
    jobs = [pa.PAJob(None, sid, d[0].data_ptr(), d[1].data_ptr(), na, va, DEFAULT, out_a.data_ptr()),
            pa.PAJob(d[2].data_ptr(), -1, d[3].data_ptr(), d[4].data_ptr(), nb, vb, pa.FLAG_COMPRESS,
                     out_b.data_ptr())]
    for it in range(200):
        out_a.fill_(it & 0xFF)
        out_b.fill_(~it & 0xFF)
        torch_cuda.cuda.synchronize()  # the fills run on torch's stream, the batch on the engine's
        engine.batch_run(jobs, pa.BATCH_GRAPH if it >= 150 else 0)
        st = engine.batch_sync(2)
        assert st[0].exact == 0 and st[1].exact == 0
        assert np.array_equal(out_a.cpu().numpy(), want_a), it
        assert np.array_equal(out_b.cpu().numpy(), want_b), it
