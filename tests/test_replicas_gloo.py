"""Replica bookkeeping over two CPU ranks (gloo): max time, summed units."""

import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from matfree_gb300 import replicas


def _worker(rank, world_size, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world_size), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        r, w, lr = replicas.world()
        assert (r, w, lr) == (rank, world_size, rank)
        replicas.barrier(w)
        # rank 0 processed 3 solves in 2 s, rank 1 processed 3 solves in 4 s
        secs = 2.0 if rank == 0 else 4.0
        tput = replicas.aggregate_throughput(3.0, secs, w)
        slowest = replicas.max_over_ranks(secs, w)
        out[rank] = (tput, slowest)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_replica_throughput_is_total_units_over_slowest_rank():
    port = 29500 + (os.getpid() % 1000)
    manager = mp.get_context("spawn").Manager()  # no fork of this multi-threaded process
    out = manager.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for rank in (0, 1):
        tput, slowest = out[rank]
        assert slowest == 4.0
        assert tput == pytest.approx(6.0 / 4.0)


def test_single_process_defaults():
    assert replicas.max_over_ranks(1.5, 1) == 1.5
    assert replicas.aggregate_throughput(10.0, 2.0, 1) == 5.0
