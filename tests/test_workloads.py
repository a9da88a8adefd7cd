"""CPU: the synthetic workloads have the shapes the configurations name.

Config 4: 512 blocks, n log-uniform in [2^18, 2^25], v/n uniform in [0.1, 0.9] (v + h = n), half with a
static seed.  Config 5: Poisson arrivals at a given rate, n log-uniform in [2^20, 2^27], v/n uniform in
[0.2, 0.8]; the static-seed variant rounds n to a power of two.  Every n and v is a multiple of 32, the
granularity the engine takes.
"""
import numpy as np

from privacyamplification_gb300 import workloads as W


def check_sizes(pairs, lo, hi, r0, r1):
    ns = np.array([n for n, _ in pairs], np.float64)
    vs = np.array([v for _, v in pairs], np.float64)
    assert all(n % 32 == 0 and v % 32 == 0 and 0 < v < n for n, v in pairs)
    logn = np.log2(ns)
    assert logn.min() >= lo - 0.01 and logn.max() <= hi + 0.01
    ratio = vs / ns
    assert ratio.min() >= r0 - 0.01 and ratio.max() <= r1 + 0.01
    # uniform in log2 n and in the ratio: means and spreads near those of the uniform laws
    assert abs(logn.mean() - (lo + hi) / 2) < 0.25 * (hi - lo) / np.sqrt(len(pairs)) * 4
    assert abs(logn.std() - (hi - lo) / np.sqrt(12)) < 0.1 * (hi - lo)
    assert abs(ratio.mean() - (r0 + r1) / 2) < 0.05
    assert abs(ratio.std() - (r1 - r0) / np.sqrt(12)) < 0.05


def test_config4_mix_shape():
    blocks = W.uneven_mix()
    assert len(blocks) == 512
    check_sizes([(b.n, b.v) for b in blocks], 18, 25, 0.1, 0.9)
    assert sum(b.static for b in blocks) == 256
    again = W.uneven_mix()
    assert [(b.n, b.v, b.static, b.seed_word0, b.key_word0) for b in blocks] == \
           [(b.n, b.v, b.static, b.seed_word0, b.key_word0) for b in again]


def test_config5_requests_shape():
    rate, count = 2000.0, 2000
    reqs = W.poisson_requests(rate, count)
    assert len(reqs) == count
    check_sizes([(r.n, r.v) for r in reqs], 20, 27, 0.2, 0.8)
    gaps = np.diff([0.0] + [r.arrival for r in reqs])
    assert (gaps > 0).all()
    assert abs(gaps.mean() * rate - 1.0) < 0.1            # exponential gaps of mean 1 / rate
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.1      # coefficient of variation 1
    static = W.poisson_requests(rate, 256, static=True)
    assert all(r.n & (r.n - 1) == 0 and 1 << 20 <= r.n <= 1 << 27 for r in static)
    assert all(r.v % 32 == 0 and 0 < r.v < r.n for r in static)
