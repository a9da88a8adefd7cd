"""The radix-16 DFT stage on the tensor cores (tcgen05.mma kind::tf32) and on the FP32 butterflies,
through the C ABI, against numpy's FFT in double precision.

One stage: each group of 16 complex values against np.fft.fft.  64 stages: F^4 = 256 I and the kernels
scale by 1/256 after every fourth stage, so the output must return the input; the relative error shows
how each method's rounding accumulates over as many stages as several passes apply.
"""
import numpy as np
import pytest

import privacyamplification_gb300 as pa

pytestmark = pytest.mark.gpu

# relative RMS error bounds: FP32 and the three-product TF32 split hold FP32-level accuracy, one TF32
# product about 2^-11 per stage
ONE_STAGE = {pa.DFT16_FP32: 1e-6, pa.DFT16_TC_SPLIT: 2e-6, pa.DFT16_TC_TF32: 2e-3}
MANY_STAGES = {pa.DFT16_FP32: 2e-5, pa.DFT16_TC_SPLIT: 4e-5, pa.DFT16_TC_TF32: 5e-2}


@pytest.fixture(scope="module")
def torch_cuda(pa_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a CUDA device")
    return torch


def run(torch, x, butterflies, reps, method, cps=2):
    dev = torch.device("cuda")
    d_in = torch.from_numpy(x.astype(np.float32)).to(dev)
    d_out = torch.full_like(d_in, float("nan"))
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    pa.dft16_stages(d_in.data_ptr(), d_out.data_ptr(), butterflies, reps, method, err.data_ptr(), cps,
                    torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return d_out.cpu().numpy()


@pytest.mark.parametrize("method", [pa.DFT16_FP32, pa.DFT16_TC_SPLIT, pa.DFT16_TC_TF32])
def test_one_stage_against_numpy(torch_cuda, method):
    rng = np.random.default_rng(16)
    b = 128 * 37  # more tiles than CTAs of a small grid, and a partial last wave
    x = rng.uniform(-1, 1, b * 32)
    got = run(torch_cuda, x, b, 1, method, cps=1).astype(np.float64).view(np.complex128).reshape(b, 16)
    want = np.fft.fft(x.astype(np.float32).astype(np.float64).view(np.complex128).reshape(b, 16), axis=1)
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel < ONE_STAGE[method], rel


@pytest.mark.parametrize("method", [pa.DFT16_FP32, pa.DFT16_TC_SPLIT, pa.DFT16_TC_TF32])
def test_64_stages_return_the_input(torch_cuda, method):
    rng = np.random.default_rng(64)
    b = 128 * 152 * 2
    x = rng.uniform(-1, 1, b * 32).astype(np.float32)
    got = run(torch_cuda, x, b, 64, method)
    rel = np.linalg.norm(got.astype(np.float64) - x) / np.linalg.norm(x.astype(np.float64))
    assert rel < MANY_STAGES[method], rel


def test_structured_inputs(torch_cuda):
    """Unit impulses and 0/1 bit patterns (the passes' inputs): the split tensor product stays at FP32
    accuracy on them too."""
    b = 128
    x = np.zeros((b, 32), np.float64)
    for r in range(b):
        if r < 32:
            x[r, r] = 1.0
        else:
            x[r] = (np.arange(32) * (r + 3) % 7 < 3)
    x = x.reshape(-1)
    want = np.fft.fft(x.view(np.complex128).reshape(b, 16), axis=1)
    for m in (pa.DFT16_FP32, pa.DFT16_TC_SPLIT):
        got = run(torch_cuda, x, b, 1, m, cps=1).astype(np.float64).view(np.complex128).reshape(b, 16)
        assert np.max(np.abs(got - want)) < 1e-5, m
