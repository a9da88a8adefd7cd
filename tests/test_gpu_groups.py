"""Grouped launches (pa_group.cu): equal blocks of a batch run as one launch per pass.  Every block's
output is compared in full with the exact CPU oracle, and with the same batch launched block by block
(PA_BATCH_NO_GROUP): static and own seeds, single-CTA sizes (n <= 2^15) and three-pass ones, all flag
combinations, padded (non-power-of-two) geometries,
groups cut at 2^24 and 2^27 bits with a remainder, groups beside single blocks, graph capture and replay,
and a block that trips the FP32 guard inside a group.
"""
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


def oracle_block(seed, ks, kr, n, v, flags):
    return (O.direct if n <= 1 << 16 else O.ntt)(seed, ks, kr, n, v, flags)


class Blocks:
    """Equal blocks (n, v, flags) with their own seeds and keys, on the device, as pa_batch_run jobs."""

    def __init__(self, torch, eng, n, v, count, flags=DEFAULT, static=True, rng_seed=1):
        self.n, self.v, self.count, self.flags = n, v, count, flags
        dev = torch.device("cuda")
        self.seeds, self.ks, self.kr = [], [], []
        for i in range(count):
            sd, recv = W.random_block(n, v, rng_seed * 1000 + i)
            k0, k1 = O.key_split(recv, n, v)
            self.seeds.append(sd)
            self.ks.append(k0)
            self.kr.append(k1)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)
        self.d_seed = [t(x) for x in self.seeds]
        self.d_ks = [t(x) for x in self.ks]
        self.d_kr = [t(x) for x in self.kr]
        self.ob = pa.output_bytes(n, v, flags)
        stride = (self.ob + 255) // 256 * 256
        self.d_out = torch.zeros(count * stride, dtype=torch.uint8, device=dev)
        self.stride = stride
        sids = [eng.seed_cache_add(self.seeds[i], n, v, flags) for i in range(count)] if static else None
        torch.cuda.synchronize()
        self.jobs = [pa.PAJob(None if static else self.d_seed[i].data_ptr(), sids[i] if static else -1,
                              self.d_ks[i].data_ptr(), self.d_kr[i].data_ptr(), n, v, flags,
                              self.d_out.data_ptr() + i * stride) for i in range(count)]

    def outputs(self):
        host = self.d_out.cpu().numpy()
        return [host[i * self.stride: i * self.stride + self.ob].copy() for i in range(self.count)]

    def want(self, i):
        return oracle_block(self.seeds[i], self.ks[i], self.kr[i], self.n, self.v, self.flags)


def run(eng, jobs, flags):
    eng.batch_run(jobs, flags)
    return eng.batch_sync(len(jobs))


@pytest.mark.parametrize("log_n,count,static", [(18, 12, True), (18, 12, False), (20, 6, True), (16, 8, False),
                                               (12, 20, True), (15, 9, False), (10, 6, False)])
def test_group_matches_oracle_and_single_launches(torch_cuda, log_n, count, static):
    n = 1 << log_n
    v = n // 4 + n // 8
    with pa.Engine(max_sample_size=n) as eng:
        bl = Blocks(torch_cuda, eng, n, v, count, static=static, rng_seed=log_n)
        want = [bl.want(i) for i in range(count)]
        for flags in (0, pa.BATCH_GRAPH, pa.BATCH_GRAPH, pa.BATCH_NO_GROUP):  # run, capture, replay, alone
            bl.d_out.fill_(0xA5)
            st = run(eng, bl.jobs, flags)
            got = bl.outputs()
            for i in range(count):
                assert np.array_equal(got[i], want[i]), (flags, i)
            assert all(s.exact == 0 and s.max_residual < 0.1 for s in st)
            assert all(s.popcount_key == int(np.unpackbits(bl.ks[i].view(np.uint8)).sum()) for i, s in enumerate(st))


@pytest.mark.parametrize("flags", [0, pa.FLAG_COMPRESS, pa.FLAG_XOR_KEY_REST])
def test_group_flag_variants(torch_cuda, flags):
    n, v = 1 << 17, 40960
    with pa.Engine(max_sample_size=n) as eng:
        bl = Blocks(torch_cuda, eng, n, v, 5, flags=flags, static=False, rng_seed=7 + flags)
        st = run(eng, bl.jobs, 0)
        got = bl.outputs()
        for i in range(5):
            assert np.array_equal(got[i], bl.want(i)), i
        assert all(s.exact == 0 for s in st)


def test_group_padded_single_cta_geometry(torch_cuda):
    """n = 3 * 2^10 (padded, one CTA per block): a group of single-CTA blocks, static and own seeds."""
    n, v = 3 << 10, 1152
    with pa.Engine(max_sample_size=1 << 13) as eng:
        for static in (True, False):
            bl = Blocks(torch_cuda, eng, n, v, 7, static=static, rng_seed=41)
            for flags in (0, pa.BATCH_GRAPH):
                bl.d_out.fill_(0x11)
                run(eng, bl.jobs, flags)
                got = bl.outputs()
                for i in range(7):
                    assert np.array_equal(got[i], bl.want(i)), (static, flags, i)


def test_group_padded_geometry(torch_cuda):
    """n = 3 * 2^16 (not a power of two): the padded seed placement inside a group, static and own seeds."""
    n, v = 3 << 16, 3 << 14
    with pa.Engine(max_sample_size=1 << 18) as eng:
        for static in (True, False):
            bl = Blocks(torch_cuda, eng, n, v, 6, static=static, rng_seed=33)
            run(eng, bl.jobs, pa.BATCH_GRAPH)
            got = bl.outputs()
            for i in range(6):
                assert np.array_equal(got[i], bl.want(i)), (static, i)


@pytest.mark.parametrize("log_bits", [0, 27])
def test_groups_cut_with_a_remainder_beside_single_blocks(torch_cuda, log_bits):
    """130 blocks of 2^20 (default groups of 2^24 bits: 8 groups of 16 and one of 2; groups of 2^27 bits:
    128 and 2) plus three blocks of another size (alone: fewer than four) in one batch; against the same
    batch launched block by block, and the oracle on a sample."""
    n, v = 1 << 20, (1 << 18) + (1 << 17)
    with pa.Engine(max_sample_size=1 << 20) as eng:
        eng.set_groups(0, log_bits)
        big = Blocks(torch_cuda, eng, n, v, 130, static=True, rng_seed=5)
        odd = Blocks(torch_cuda, eng, 1 << 19, 1 << 17, 3, static=False, rng_seed=6)
        jobs = big.jobs + odd.jobs
        run(eng, jobs, pa.BATCH_GRAPH)
        g_big, g_odd = big.outputs(), odd.outputs()
        big.d_out.fill_(0)
        odd.d_out.fill_(0)
        run(eng, jobs, pa.BATCH_NO_GROUP)
        a_big, a_odd = big.outputs(), odd.outputs()
        for i in range(130):
            assert np.array_equal(g_big[i], a_big[i]), i
        for i in range(3):
            assert np.array_equal(g_odd[i], a_odd[i]), i
            assert np.array_equal(g_odd[i], odd.want(i)), i
        for i in (0, 1, 127, 128, 129):
            assert np.array_equal(g_big[i], big.want(i)), i


def test_guard_inside_a_group(torch_cuda):
    """A run-structured block among ordinary ones of the same geometry: the group's residual word for it
    trips the guard and pa_batch_sync recomputes it exactly; the others are unaffected."""
    n, v = 1 << 22, (1 << 20) + (1 << 19)
    with pa.Engine(max_sample_size=n) as eng:
        eng.set_groups(4, 24)  # four blocks of 2^22 bits to a group
        bl = Blocks(torch_cuda, eng, n, v, 4, static=False, rng_seed=9)
        seed = np.zeros(n // 32, np.uint32)
        seed[: n // 64] = 0xFFFFFFFF
        ks, kr = O.key_split(np.full(n // 32 + 1, 0xFFFFFFFF, np.uint32), n, v)
        bl.seeds[2], bl.ks[2], bl.kr[2] = seed, ks, kr
        bl.d_seed[2].copy_(torch_cuda.from_numpy(seed.view(np.int32)))
        bl.d_ks[2].copy_(torch_cuda.from_numpy(ks.view(np.int32)))
        bl.d_kr[2].copy_(torch_cuda.from_numpy(kr.view(np.int32)))
        torch_cuda.cuda.synchronize()
        st = run(eng, bl.jobs, 0)
        assert st[2].exact == 1 and st[2].max_residual > 0.25
        assert all(st[i].exact == 0 for i in (0, 1, 3))
        got = bl.outputs()
        for i in range(4):
            assert np.array_equal(got[i], bl.want(i)), i


def test_set_groups_arguments(pa_lib):
    with pa.Engine(max_sample_size=1 << 16) as eng:
        for a in ((1, 0), (-1, 0), (0, 16), (0, 31), (0, -2)):
            with pytest.raises(pa.PAError):
                eng.set_groups(*a)
        eng.set_groups(2, 17)
        eng.set_groups(0, 0)


def test_group_buffers_give_way_to_the_budget(torch_cuda):
    """After a grouped batch, a tight HBM budget: adding a cached seed frees the group working sets
    first; the next batch regroups if they fit again, or runs block by block, with the same outputs."""
    n = 1 << 18
    v = n // 4 + n // 8
    with pa.Engine(max_sample_size=1 << 20) as eng:
        bl = Blocks(torch_cuda, eng, n, v, 16, static=True, rng_seed=77)
        want = [bl.want(i) for i in range(16)]
        run(eng, bl.jobs, pa.BATCH_GRAPH)
        eng.set_pool(64 << 20, 16, 8)  # below what the slots, spectra and group working set hold now
        seed, _ = W.random_block(1 << 20, 1 << 18, 78)
        eng.seed_cache_add(seed, 1 << 20, 1 << 18)
        for flags in (0, pa.BATCH_GRAPH):
            bl.d_out.fill_(0)
            st = run(eng, bl.jobs, flags)
            got = bl.outputs()
            for i in range(16):
                assert np.array_equal(got[i], want[i]), (flags, i)
            assert all(s.exact == 0 for s in st)
