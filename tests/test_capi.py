"""The C ABI library loads and exports what include/pa_gb300.h declares; host-only entry points.

No test here launches a kernel: these run on machines without a GPU.
"""
import os
import re

import numpy as np
import pytest

import privacyamplification_gb300 as pa
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pa_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pa_[a-z0-9_]+)\s*\(", text)))


def test_header_matches_binding_list():
    assert declared_functions() == sorted(pa.EXPORTS)


def test_library_exports_every_declared_symbol(pa_lib):
    for name in declared_functions():
        assert hasattr(pa_lib, name), name


def test_output_bytes():
    assert pa.output_bytes(1 << 27, 50331648, pa.DEFAULT_FLAGS) == 50331648 // 8
    assert pa.output_bytes(2048, 1024, 0) == 2048 // 16
    assert pa.output_bytes(2048, 1024, pa.FLAG_XOR_KEY_REST) == 2048 // 16


def test_kernels_per_block():
    assert pa.kernels_per_block(2048, 1024, 0) == 1
    assert pa.kernels_per_block(1 << 27, 50331648) == 5  # bit rows, passes A, B, C, finish
    assert pa.kernels_per_block(1000, 96) == 0  # rejected size


def test_key_split_matches_oracle(pa_lib):
    for n, v in [(1024, 384), (1 << 16, 24576), (4096, 4064), (4096, 32)]:
        _, recv = O.random_block(n, v, n ^ v)
        a = pa.key_split(recv, n, v)
        b = O.key_split(recv, n, v)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_key_split_rejects_bad_sizes(pa_lib):
    recv = np.zeros(1 << 10, np.uint32)
    for n, v in [(1024, 0), (1024, 1024), (1000, 96), (1024, 100)]:
        try:
            pa.key_split(recv, n, v)
        except pa.PAError as e:
            assert e.code == pa.PA_ERR_INVALID_ARG
        else:
            raise AssertionError("accepted n=%d v=%d" % (n, v))


def test_error_strings(pa_lib):
    assert pa.error_string(pa.PA_OK) == "ok"
    assert "seed" in pa.error_string(pa.PA_ERR_NO_SEED)


def test_cufft_baseline_builds_and_exports():
    """The cuFFT pipeline baseline (timed beside the engine) builds for sm_103a and exports its entry points."""
    import ctypes
    from baseline import cufft_plain
    lib = ctypes.CDLL(cufft_plain.build())
    for name in ("cp_create", "cp_destroy", "cp_seed_slot", "cp_key_start_slot", "cp_key_rest_slot",
                 "cp_output_slot", "cp_process", "cp_residual"):
        assert hasattr(lib, name), name


def test_dft16_stages_rejects_bad_arguments(pa_lib):
    """Argument checks of the tensor-core stage measurement come before any CUDA call."""
    import privacyamplification_gb300 as pa
    bad = [(0, 0, 128, 1, pa.DFT16_FP32, 16), (16, 16, 100, 1, pa.DFT16_FP32, 16), (16, 16, 128, 0, 0, 16),
           (16, 16, 128, 1, 3, 16), (16, 16, 128, 1, pa.DFT16_TC_SPLIT, 16, 5), (8, 16, 128, 1, 0, 16),
           (16, 16, 128, 1, pa.DFT16_FP32, 16, 17)]
    for a in bad:
        with pytest.raises(pa.PAError) as e:
            pa.dft16_stages(*a)
        assert e.value.code == -1, a
