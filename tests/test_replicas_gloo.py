"""The multi-GPU path of bench.py (one replica per rank, timings max-reduced and counts sum-reduced over the
ranks) on CPU: two gloo ranks on 127.0.0.1."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r: a replica that took (10 + r) ms device time and placed 1000 * (r + 1) spheres
    times, counts = bench.aggregate([10.0 + rank, 20.0 - rank, 5.0], [1000.0 * (rank + 1), 7.0], dist, "cpu")
    out[rank] = (times, counts)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    world = 2
    port = 29500 + (os.getpid() % 1000)
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        times, counts = res[rank]
        assert times == [11.0, 20.0, 5.0]  # max over ranks
        assert counts == [3000.0, 14.0]  # sum over ranks


def test_replica_seeds_are_distinct_per_rank():
    # each rank samples an independent instance: seed = workload seed + rank (bench.py main)
    sys.path.insert(0, ROOT)
    import bench
    dim, L, r, seed0, _ = bench.WORKLOADS["config2"]
    assert len({seed0 + rank for rank in range(8)}) == 8
