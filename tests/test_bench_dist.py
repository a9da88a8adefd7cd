"""bench.py's multi-GPU (replica) host logic on CPU: two `gloo` ranks, as torchrun launches them.

Blocks are independent, so N GPUs run N replicas with no collective on the data path; the only
cross-rank steps are the barrier and the max over ranks of each timed region.  This checks that
reduction, the whole-job value, and that only rank 0 of the reference arm does work."""
import argparse
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_setup() == (world, rank, rank)
        times = bench.max_over_ranks([1.0 + rank, 10.0 - rank], dist, "cpu")
        value = bench.job_value(world, 8, bench.N_BITS, times[0])
        dist.barrier()
        args = argparse.Namespace(steps=1, warmup=3, gpus=world)
        ref_rc = bench.run_reference(args) if rank != 0 else None  # non-zero ranks return at once
        out[rank] = (times, value, ref_rc)
    finally:
        dist.destroy_process_group()


def test_two_rank_max_and_job_value():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(world, _port(), out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    import sys
    sys.path.insert(0, ROOT)
    import bench
    for rank in range(world):
        times, value, ref_rc = res[rank]
        assert times == [2.0, 10.0]  # max over ranks, element-wise
        assert value == pytest.approx(world * 8 * bench.N_BITS / 2.0 / 1e9)
    assert res[1][2] == 0
