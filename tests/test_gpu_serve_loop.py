"""The device-resident serving loop (pa_serve_start / pa_serve_submit / pa_serve_poll / pa_serve_stop)
through the C ABI: requests published to a ring in pinned host memory are taken by lanes of a persistent
kernel, which read the inputs from host memory and write the outputs there.  Every result is compared in
full with the exact CPU oracle, for requests that overlap on the device."""
import time

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


def oracle_of(banks, r):
    return O.ntt(banks.seed_words(r), banks.key_start(r), banks.key_rest(r), r.n, r.v, r.flags)


def test_overlapping_requests_match_oracle(torch_cuda):
    """Poisson arrivals faster than the loop drains them (own seed per request, all flag sets)."""
    reqs = W.poisson_requests(rate=5000, count=40, lo=12, hi=22, rng_seed=0x5E1)
    reqs[2].flags = 0
    reqs[4].flags = pa.FLAG_COMPRESS
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    with pa.Engine(max_sample_size=1 << 22) as eng:
        lanes = eng.serve_start(ctas_per_lane=19, max_np=1 << 22, ring_slots=16)
        assert lanes >= 2
        res = W.serve_device(eng, reqs, banks, out_slots=12, keep=lambda r: True)
        eng.serve_stop()
    assert len(res.outputs) == len(reqs) and res.exact == 0
    for r in reqs:
        assert np.array_equal(res.outputs[r.rid], oracle_of(banks, r)), r


def test_requests_queued_behind_busy_lanes(torch_cuda):
    """Every request arrives at once and two lanes serve 24 of them, so a lane takes its next request
    while its other CTAs still finish the previous one: each completion is published for its own request."""
    reqs = W.poisson_requests(rate=1e7, count=24, lo=16, hi=23, rng_seed=0x5E3)
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    with pa.Engine(max_sample_size=1 << 23) as eng:
        assert eng.serve_start(ctas_per_lane=76, max_np=1 << 23, ring_slots=32) == 2
        res = W.serve_device(eng, reqs, banks, out_slots=24, keep=lambda r: True, stall_s=30.0)
        eng.serve_stop()
    for r in reqs:
        assert np.array_equal(res.outputs[r.rid], oracle_of(banks, r)), r


def test_static_seeds_served(torch_cuda):
    """Static seeds (spectra cached before the loop starts), powers of two from 2^16 to 2^22."""
    reqs = W.poisson_requests(rate=3000, count=20, lo=16, hi=22, static=True, rng_seed=0x5E2)
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    with pa.Engine(max_sample_size=1 << 22) as eng:
        seed_ids = {}
        for r in reqs:
            k = W.seed_key(r.n, r.v, r.flags)
            if k not in seed_ids:
                seed_ids[k] = eng.seed_cache_add(banks.seed_words(r), r.n, r.v, r.flags)
        eng.serve_start(ctas_per_lane=38, max_np=1 << 22)
        res = W.serve_device(eng, reqs, banks, keep=lambda r: True, seed_ids=seed_ids)
        eng.serve_stop()
    for r in reqs:
        assert np.array_equal(res.outputs[r.rid], oracle_of(banks, r)), r


def test_idle_loop_restarts_and_ring_full(torch_cuda):
    """The loop ends by itself when idle and the next submit starts it again; a full ring says busy;
    pageable host buffers are refused."""
    n, v = 1 << 20, 393216
    torch = torch_cuda
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).pin_memory().numpy().view(np.uint32)
    blocks = []
    for k in range(3):
        seed, recv = O.random_block(n, v, 900 + k)
        ks, kr = O.key_split(recv, n, v)
        out = torch.zeros(v // 8, dtype=torch.uint8).pin_memory().numpy()
        blocks.append((pin(seed), pin(ks), pin(kr), out, O.ntt(seed, ks, kr, n, v)))
    job = lambda b: pa.PAJob(b[0].ctypes.data, -1, b[1].ctypes.data, b[2].ctypes.data, n, v, DEFAULT, b[3].ctypes.data)
    with pa.Engine(max_sample_size=n) as eng:
        eng.serve_start(ctas_per_lane=38, max_np=n, ring_slots=2)
        t0 = eng.serve_submit(job(blocks[0]))
        t1 = eng.serve_submit(job(blocks[1]))
        assert eng.serve_submit(job(blocks[2])) is None  # both ring slots hold uncollected requests
        for t, b in ((t0, blocks[0]), (t1, blocks[1])):
            deadline = time.time() + 30
            while eng.serve_poll(t) is None:
                assert time.time() < deadline
            assert np.array_equal(b[3], b[4])
        time.sleep(3.5)  # longer than the loop's two idle seconds: it has ended
        t2 = eng.serve_submit(job(blocks[2]))
        deadline = time.time() + 30
        while eng.serve_poll(t2) is None:
            assert time.time() < deadline
        assert np.array_equal(blocks[2][3], blocks[2][4])
        seed, recv = O.random_block(n, v, 5)
        ks, kr = O.key_split(recv, n, v)
        out = np.zeros(v // 8, np.uint8)
        with pytest.raises(pa.PAError) as ei:  # pageable memory: the device cannot read it directly
            eng.serve_submit(pa.PAJob(seed.ctypes.data, -1, ks.ctypes.data, kr.ctypes.data, n, v, DEFAULT,
                                      out.ctypes.data))
        assert ei.value.code == pa.PA_ERR_INVALID_ARG
        eng.serve_stop()


def test_guard_recomputes_served_block(torch_cuda):
    n, v = 1 << 22, (1 << 20) + (1 << 19)
    torch = torch_cuda
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).pin_memory().numpy().view(np.uint32)
    seed = np.zeros(n // 32, np.uint32)
    seed[: n // 64] = 0xFFFFFFFF
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    ks, kr = O.key_split(recv, n, v)
    ps, pk, pr = pin(seed), pin(ks), pin(kr)
    out = torch.zeros(v // 8, dtype=torch.uint8).pin_memory().numpy()
    with pa.Engine(max_sample_size=n) as eng:
        eng.serve_start(ctas_per_lane=38, max_np=n)
        t = eng.serve_submit(pa.PAJob(ps.ctypes.data, -1, pk.ctypes.data, pr.ctypes.data, n, v, DEFAULT,
                                      out.ctypes.data))
        deadline = time.time() + 30
        st = eng.serve_poll(t)
        while st is None:
            assert time.time() < deadline
            st = eng.serve_poll(t)
        eng.serve_stop()
    assert st.max_residual > 0.25 and st.exact == 1
    assert np.array_equal(out, O.ntt(seed, ks, kr, n, v))


def test_config5_draw_device_loop(torch_cuda):
    """16 requests of the config-5 distribution (n log-uniform in [2^20, 2^27]) at 2000/s through the
    device-resident loop, whole outputs against the oracle."""
    reqs = W.poisson_requests(rate=2000, count=16, lo=20, hi=27, rng_seed=0x5E7E)
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
    banks = W.HostBanks(words)
    with pa.Engine(max_sample_size=1 << 27) as eng:
        eng.serve_start(ctas_per_lane=38, max_np=1 << 27)
        res = W.serve_device(eng, reqs, banks, out_slots=8, keep=lambda r: True, stall_s=60.0)
        eng.serve_stop()
    for r in reqs:
        assert np.array_equal(res.outputs[r.rid], oracle_of(banks, r)), r
