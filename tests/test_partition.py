"""Specimen sharding across ranks (host logic, CPU): a world-size-2 gloo group checks that the
ranks' shares partition the specimens, balance the particle counts, and that the totals the
bench reduces over ranks equal the whole job's."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from sudodem_gb300.partition import partition_scenes, rank_share


def test_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    sizes = np.exp(rng.uniform(np.log(300), np.log(8000), size=512)).astype(int).tolist()
    for ws in (1, 2, 3, 4, 8):
        parts = partition_scenes(sizes, ws)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(512))
        loads = [sum(sizes[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)   # greedy LPT bound


def _worker(rank, ws, port, sizes, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    mine = rank_share(sizes, rank, ws)
    n = torch.tensor([sum(sizes[i] for i in mine)], dtype=torch.int64)
    dist.all_reduce(n)
    gathered = [None] * ws
    dist.all_gather_object(gathered, mine)
    t = torch.tensor([1.0 + rank], dtype=torch.float64)   # per-rank time: the bench takes the max
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        q.put((int(n.item()), gathered, float(t.item())))
    dist.destroy_process_group()


def test_two_rank_gloo_shares_partition_the_job():
    rng = np.random.default_rng(1)
    sizes = np.exp(rng.uniform(np.log(300), np.log(8000), size=64)).astype(int).tolist()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    total, gathered, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert total == sum(sizes)
    assert sorted(i for g in gathered for i in g) == list(range(64))
    assert not set(gathered[0]) & set(gathered[1])
    assert tmax == 2.0
