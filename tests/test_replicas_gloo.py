"""bench.py's replica aggregation across ranks (two gloo ranks on CPU)."""

import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # Rank r "took" 100 * (r + 1) ms for 4 solves.
    value, elapsed = bench.replica_aggregate(100.0 * (rank + 1), 4.0, dist, torch.device("cpu"))
    out[rank] = (value, elapsed)
    dist.destroy_process_group()


def test_two_rank_replica_throughput():
    world = 2
    port = 29500 + os.getpid() % 1000
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for rank in range(world):
        value, elapsed = out[rank]
        assert elapsed == pytest.approx(200.0)
        assert value == pytest.approx(8.0 / 0.2)


def test_single_rank_throughput():
    import bench

    value, elapsed = bench.replica_aggregate(250.0, 4.0, None, torch.device("cpu"))
    assert elapsed == 250.0 and value == pytest.approx(16.0)
