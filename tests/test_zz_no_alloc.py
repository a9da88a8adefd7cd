"""pa_process_noalloc (one block, n <= 2^15, scratch in a static device array) against pa_process.

Collected last on purpose (file name), so that it runs both after every other GPU test in one session
and alone in a fresh process (`pytest tests/test_zz_no_alloc.py -m gpu`).  Device buffers are
allocated here by the test; the entry point itself allocates nothing.
"""
import numpy as np
import pytest

import privacyamplification_gb300 as pa
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEFAULT = pa.FLAG_XOR_KEY_REST | pa.FLAG_COMPRESS


@pytest.fixture(scope="module")
def torch_cuda(pa_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a CUDA device")
    return torch


def dev_u32(torch, a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return torch.from_numpy(a.view(np.int32).copy()).cuda()


def run_noalloc(torch, seed, ks, kr, n, v, flags, stream=None):
    """Queues one block; returns the device output tensor (caller synchronises)."""
    d_seed, d_ks, d_kr = dev_u32(torch, seed), dev_u32(torch, ks), dev_u32(torch, kr)
    ob = pa.output_bytes(n, v, flags)
    d_out = torch.zeros((ob + 3) // 4 * 4, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    s = stream.cuda_stream if stream is not None else 0
    pa.process_noalloc(d_seed.data_ptr(), d_ks.data_ptr(), d_kr.data_ptr(), n, v, d_out.data_ptr(), flags, s)
    return d_out, ob, (d_seed, d_ks, d_kr)


def engine_result(eng, seed, ks, kr, n, v, flags):
    eng.set_seed(seed, n, -1)
    return eng.process(ks, kr, n, v, flags)


@pytest.fixture(scope="module")
def small_engine(pa_lib):
    eng = pa.Engine(max_sample_size=1 << 15)
    yield eng
    eng.close()


@pytest.mark.parametrize("n,v,flags", [
    (1 << 15, 12288, DEFAULT), (1 << 14, 6144, 0), (1 << 10, 384, DEFAULT), (1 << 15, 4096, pa.FLAG_COMPRESS),
    (20480, 7680, DEFAULT), (1056, 480, 0), (1 << 10, 32, DEFAULT), (1 << 10, 992, pa.FLAG_COMPRESS)])
def test_two_calls_in_a_row_match_pa_process(torch_cuda, small_engine, n, v, flags):
    """Two different blocks queued back to back on one stream: each equals pa_process on the same inputs
    (so nothing of the first call leaks into the second through the shared scratch)."""
    blocks = []
    for k in range(2):
        seed, recv = O.random_block(n, v, 7000 + 13 * n + v + k)
        ks, kr = O.key_split(recv, n, v)
        blocks.append((seed, ks, kr))
    stream = torch_cuda.cuda.Stream()
    outs = [run_noalloc(torch_cuda, *b, n, v, flags, stream) for b in blocks]
    stream.synchronize()
    for (seed, ks, kr), (d_out, ob, _) in zip(blocks, outs):
        got = d_out.cpu().numpy()[:ob]
        want = engine_result(small_engine, seed, ks, kr, n, v, flags)
        assert np.array_equal(got, want)
        if n <= 1 << 14:
            assert np.array_equal(got, O.direct(seed, ks, kr, n, v, flags))


def test_default_stream_and_repeat(torch_cuda, small_engine):
    n, v = 1 << 15, 12288
    seed, recv = O.random_block(n, v, 4242)
    ks, kr = O.key_split(recv, n, v)
    want = engine_result(small_engine, seed, ks, kr, n, v, DEFAULT)
    for _ in range(2):
        d_out, ob, _bufs = run_noalloc(torch_cuda, seed, ks, kr, n, v, DEFAULT)
        torch_cuda.cuda.synchronize()
        assert np.array_equal(d_out.cpu().numpy()[:ob], want)


def test_structured_block_within_fp32_budget(torch_cuda, small_engine):
    """Long run of seed ones, all-ones key: at n = 2^15 the FP32 path stays exact (engine sees no
    fallback), and the no-allocation result equals it."""
    n, v = 1 << 15, 12288
    seed = np.zeros(n // 32, np.uint32)
    seed[: n // 64] = 0xFFFFFFFF
    recv = np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32)
    ks, kr = O.key_split(recv, n, v)
    want = engine_result(small_engine, seed, ks, kr, n, v, DEFAULT)
    assert small_engine.last_stats.exact == 0
    d_out, ob, _bufs = run_noalloc(torch_cuda, seed, ks, kr, n, v, DEFAULT)
    torch_cuda.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy()[:ob], want)
    assert np.array_equal(want, O.direct(seed, ks, kr, n, v, DEFAULT))


def test_rejects_beyond_limit(torch_cuda):
    buf = torch_cuda.zeros(1 << 14, dtype=torch_cuda.int32, device="cuda")
    p = buf.data_ptr()
    with pytest.raises(pa.PAError) as ei:
        pa.process_noalloc(p, p, p, 1 << 16, 24576, p, DEFAULT)
    assert ei.value.code == -4  # PA_ERR_TOO_LARGE
    with pytest.raises(pa.PAError) as ei:
        pa.process_noalloc(p, p, p, 1 << 15, 12288, p, DEFAULT | pa.FLAG_EXACT)
    assert ei.value.code == -1
    with pytest.raises(pa.PAError) as ei:  # padded cyclic length 2^16 for this non-power-of-two n
        pa.process_noalloc(p, p, p, 30720, 1024, p, 0)
    assert ei.value.code == -4
