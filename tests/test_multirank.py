"""Multi-rank host logic on CPU ranks (gloo, world size 2): the instance
partition of the batched workload and the max-over-ranks timing of the bench.
The GPU path itself needs one GPU per rank; instances never couple, so ranks
exchange nothing but the final timing."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from pyshocks_gb300.batched import partition_instances

        sizes, _ = bench.workload_params(bench.SEED)
        mine = partition_instances(sizes, world)[rank]
        # every rank computes the same partition independently
        gathered = [None] * world
        dist.all_gather_object(gathered, mine.tolist())
        # max over ranks of a per-rank time, as the bench reports it
        t = torch.tensor([float(rank + 1)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        out[rank] = (gathered, float(t.item()), int(np.sum(sizes[mine])))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_partition_and_timing_over_two_gloo_ranks():
    import bench

    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True,
                           start_method="spawn")
        res = dict(out)
    sizes, _ = bench.workload_params(bench.SEED)
    parts = res[0][0]
    assert parts == res[1][0]  # identical on both ranks
    allidx = sorted(i for p in parts for i in p)
    assert allidx == list(range(sizes.size))  # disjoint, complete cover
    loads = [res[r][2] for r in range(world)]
    assert abs(loads[0] - loads[1]) <= max(sizes)  # LPT bound
    assert res[0][1] == res[1][1] == 2.0  # max over ranks


def test_partition_balances_uneven_sizes():
    from pyshocks_gb300.batched import partition_instances

    rng = np.random.default_rng(0)
    sizes = rng.choice([4096, 8192, 16384, 32768, 65536], size=1024)
    for world in (2, 4, 8):
        parts = partition_instances(sizes, world)
        loads = np.array([sizes[p].sum() for p in parts])
        assert sorted(np.concatenate(parts).tolist()) == list(range(1024))
        assert loads.max() - loads.min() <= sizes.max()
