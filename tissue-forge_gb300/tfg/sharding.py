"""Sharding independent simulations over ranks (one GPU per rank, no data-path exchange).

Simulations of an ensemble or a request stream are independent units, so N GPUs run
disjoint subsets of them and never communicate while stepping.  The subsets come from a
longest-processing-time bin-pack on each simulation's work (particles x steps): sort by
work, largest first, each to the currently lightest rank (ties to the lowest rank).  Every
rank computes the same partition from the same inputs, so no exchange is needed to agree
on it; the only collective is the max of the ranks' timings at the end of a benchmark.
"""
import numpy as np


def lpt_partition(work, nranks):
    """Indices of `work` for each of `nranks` ranks (LPT greedy, deterministic)."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    work = np.asarray(work, np.float64)
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    load = [0.0] * nranks
    parts = [[] for _ in range(nranks)]
    for i in order:
        r = min(range(nranks), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += work[i]
    return [sorted(p) for p in parts]


def shard(work, rank, nranks):
    return lpt_partition(work, nranks)[rank]


def max_over_ranks(value, dist=None, device=None):
    """The largest `value` over all ranks (the slowest rank's time); identity without a
    process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
