"""Replicas on several ranks (``bench.py --gpus N`` under torchrun): every
rank evaluates its own copy of the workload, the ranks meet at barriers, and
the reported time is the slowest rank's.  Checked with two ``gloo`` ranks on
the CPU (no GPU)."""

import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_env()
        assert (w, r, local) == (world, rank, rank)
        dist.barrier()
        slowest = bench.max_over_ranks(10.0 * (rank + 1))   # rank times 10 ms, 20 ms
        out[rank] = (slowest, bench.replica_rate(1000, w, slowest))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    world, port = 2, _free_port()
    # the shared dict's server process is spawned too (no fork of a
    # multi-threaded test process)
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (20.0, 2 * 1000 / 0.020)


def test_one_process_is_its_own_slowest_rank():
    sys.path.insert(0, ROOT)
    import bench

    assert not dist.is_initialized()
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.replica_rate(10, 1, 5.0) == pytest.approx(2000.0)
