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


def test_reference_arm_line_on_cpu():
    """``--impl reference`` on CPU: one JSON line with the same metric, unit and config keys as
    the GPU arm, a cpu_baseline describing the run and an e2e entry without host copies."""
    import json
    import subprocess
    import sys

    from tests.conftest import ROOT

    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--grid", "64",
                          "--members", "2", "--steps", "2", "--warmup", "3"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"].startswith("RK4 site-updates/s")
    assert line["unit"] == "site-updates/s" and line["higher_is_better"] is True
    assert line["warmup"] == 3 and line["steps"] == 2 and line["same_steps"] is True
    assert line["value"] > 0
    assert line["config"]["grid"] == [64, 64] and line["config"]["members"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "site-updates/s",
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
