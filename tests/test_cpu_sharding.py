"""Sharding simulations over ranks: LPT partition properties, and two gloo ranks on CPU
that agree on a disjoint, complete partition without exchanging it and reduce their
timings to the maximum."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from tfg import configs
from tfg.sharding import lpt_partition, max_over_ranks, shard


def test_lpt_partition_complete_and_balanced():
    ns, _ = configs.ensemble_sizes(512, seed=3)
    work = ns * 1000
    for k in (1, 2, 3, 8):
        parts = lpt_partition(work, k)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(work)))
        loads = [work[p].sum() for p in parts]
        # LPT bound: max load <= (4/3 - 1/(3k)) * optimum <= that times the mean
        assert max(loads) <= (4 / 3) * np.mean(loads) + work.max()


def test_ensemble_indices_reproduce_members():
    full = configs.ensemble(count=6, nmax=2000, seed=5)
    sub = configs.ensemble(count=6, nmax=2000, seed=5, indices=[4, 1])
    assert np.array_equal(sub[0].x, full[4].x) and np.array_equal(sub[1].x, full[1].x)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ns, _ = configs.ensemble_sizes(64, seed=9)
    mine = shard(ns * 100, rank, world)
    got = [None] * world
    dist.all_gather_object(got, mine)
    t = max_over_ranks(1.0 + rank, dist)
    q.put((rank, mine, got, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_shards():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, mine, got, t in res:
        assert got[rank] == mine
        assert t == 2.0
        assert not set(got[0]) & set(got[1])
        assert sorted(got[0] + got[1]) == list(range(64))
