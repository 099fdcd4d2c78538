"""Replica sharding across ranks, run as two gloo processes on the CPU: every
item is processed by exactly one rank, the ranks agree on the assignment
without communicating, and the step time is the maximum over ranks."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from fastgeodis_gb300.replicas import partition, transform_cost


def test_partition_balances_and_covers():
    costs = [transform_cost((h, w), 2) for h, w in [(2048, 2048), (128, 128), (1024, 512), (512, 512), (2048, 128)]]
    parts = partition(costs, 2)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) <= max(costs) + min(loads)  # LPT bound
    assert partition(costs, 1) == [list(range(len(costs)))]
    with pytest.raises(ValueError):
        partition(costs, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = [transform_cost(s, 2) for s in sizes]
    mine = partition(costs, world)[rank]
    # every rank derives the same assignment: gather and compare
    got = [None] * world
    dist.all_gather_object(got, mine)
    # "time" of this rank's share, reduced with MAX as bench.py does
    t = torch.tensor([sum(costs[i] for i in mine)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, got, float(t.item())))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_and_cover():
    sizes = [(2048, 2048), (128, 2048), (512, 512), (64, 64, 64), (256, 1024), (1000, 600), (300, 300)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res.sort()
    assert res[0][1] == res[1][1]  # identical assignment on both ranks
    parts = res[0][1]
    assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
    costs = [transform_cost(s, 2) for s in sizes]
    assert res[0][2] == res[1][2] == max(sum(costs[i] for i in p) for p in parts)
