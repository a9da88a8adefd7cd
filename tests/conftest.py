import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpa_gb300.so")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = np.load(os.path.join(ROOT, "tests", "golden", "large_block_kat.npz"))
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def pa_lib():
    """Builds (if stale) and loads the product library."""
    from privacyamplification_gb300 import build, load_library
    build.build()
    return load_library()


@pytest.fixture(scope="session")
def gpu_engine(pa_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a CUDA device")
    from privacyamplification_gb300 import Engine
    eng = Engine(max_sample_size=1 << 27)
    yield eng
    eng.close()
