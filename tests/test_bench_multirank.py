"""The multi-GPU host logic of bench.py on CPU: two gloo ranks (world size 2).

Each rank steps its own replicas (weak scaling, no data-path collective); the only collective
is the MAX reduction of the timed region.  Uneven sweeps are split by sites.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = bench.rank_members(rank, world, 3)
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
        results[rank] = (mine, slowest)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_partition_and_reduce():
    with mp.Manager() as manager:
        results = manager.dict()
        mp.spawn(_rank_main, args=(2, _free_port(), results), nprocs=2, join=True)
        got = dict(results)
    assert got[0][0] == [0, 1, 2] and got[1][0] == [3, 4, 5]
    assert got[0][1] == got[1][1] == 15.0


def test_replica_seeds_and_pumps_differ_between_ranks():
    import bench

    a = bench.workload(2, first=0)
    b = bench.workload(2, first=2)
    both = bench.workload(4, first=0)
    assert a["seeds"] == [42, 43] and b["seeds"] == [44, 45]
    assert np.allclose(np.concatenate([a["sigmas"], b["sigmas"]]), both["sigmas"])
    assert not np.array_equal(a["psi"], b["psi"])


def test_uneven_members_are_balanced_by_sites():
    import bench

    sites = [128 ** 2, 256 ** 2, 512 ** 2] * 10
    parts = bench.partition_by_sites(sites, 4)
    assert sorted(m for p in parts for m in p) == list(range(len(sites)))
    loads = [sum(sites[m] for m in p) for p in parts]
    assert max(loads) - min(loads) <= 512 ** 2
