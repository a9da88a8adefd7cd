"""Failure detection without a GPU fault: a bounded device wait that is never satisfied (a barrier that
nothing arrives on) ends with an error status the host reads, and the context stays usable -- the
path every TMA wait of the three-pass kernels takes if its copy never completes."""
import numpy as np
import pytest

import privacyamplification_gb300 as pa
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_expired_wait_is_reported_and_context_survives(gpu_engine):
    assert pa.selftest_wait_timeout(0, rounds=4096) == 1
    assert pa.selftest_wait_timeout(0, rounds=1) == 1
    with pytest.raises(pa.PAError):
        pa.selftest_wait_timeout(0, rounds=0)
    # the same process and context go on hashing correctly
    n, v = 1 << 18, 98304
    seed, recv = O.random_block(n, v, 404)
    ks, kr = O.key_split(recv, n, v)
    gpu_engine.set_seed(seed, n, -1)
    assert np.array_equal(gpu_engine.process(ks, kr, n, v), O.ntt(seed, ks, kr, n, v))
