"""The multi-GPU paths of bench.py on CPU, as two gloo ranks on 127.0.0.1: replicas (one instance per rank,
timings max-reduced and counts sum-reduced over the ranks) and the batched form's instance shards (the
instance list split over the ranks with no exchange, each rank running its own shard)."""
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


# a CPU stand-in for the batched form: small independent instances, each run to maximality by the oracle
SMALL = [(2, [0.5 + 0.05 * i, 0.6], 0.03, 100 + i) for i in range(8)] + \
        [(3, [0.3 + 0.02 * i] * 3, 0.05, 200 + i) for i in range(6)]


def _oracle_count(inst):
    from oracle import oracle as O
    dim, sup, r, seed = inst
    o = O.Oracle(dim, [0.0] * dim, sup, [(r, 1.0, 0)])
    o.proceed(seed % 2**32)
    return len(o.spheres()[1])


def _shard_rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    from rsa_mpi_gb300.sampler import partition_instances
    dist.init_process_group("gloo", rank=rank, world_size=world)
    full = bench.config4_instances()
    mine = partition_instances(full, world)[rank]
    shards = [None] * world
    dist.all_gather_object(shards, mine)
    small = partition_instances(SMALL, world)[rank]
    n = sum(_oracle_count(SMALL[i]) for i in small)
    times, counts = bench.aggregate([float(len(small))], [float(n)], dist, "cpu")
    out[rank] = (shards, counts[0], times[0])
    dist.barrier()
    dist.destroy_process_group()


def test_batch_shards_two_gloo_ranks():
    """Each rank computes the same split with no exchange; the shards are disjoint and cover the 4,096
    instances of the batched workload; and the sum-reduced counts of the ranks' shards, each instance run to
    maximality by the oracle, equal the one-rank total."""
    world = 2
    port = 29500 + ((os.getpid() + 500) % 1000)
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_shard_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    shards = res[0][0]
    assert res[1][0] == shards
    assert set(shards[0]).isdisjoint(shards[1])
    assert sorted(shards[0] + shards[1]) == list(range(4096))
    total = sum(_oracle_count(x) for x in SMALL)
    assert res[0][1] == res[1][1] == float(total)


def test_batch_shards_are_balanced():
    sys.path.insert(0, ROOT)
    import bench
    from rsa_mpi_gb300.sampler import expected_spheres, partition_instances
    full = bench.config4_instances()
    for world in (1, 2, 4, 8):
        parts = partition_instances(full, world)
        assert sorted(i for p in parts for i in p) == list(range(len(full)))
        loads = [sum(expected_spheres(full[i]) for i in p) for p in parts]
        assert max(loads) / (sum(loads) / world) < 1.02, loads
