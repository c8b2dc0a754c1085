"""Data-parallel history sharding over ranks (one process per GPU).

Histories are independent and the Philox keying makes every history's result
independent of where it runs, so N GPUs split a job into N disjoint,
contiguous history ranges and never talk during transport.  The one exchange
is at the end: per-bin (sum, sum of squares) of every rank, merged in rank
order so the merged result does not depend on arrival order.
"""
from __future__ import annotations

import numpy as np


def shard_range(n_total: int, world: int, rank: int, first: int = 0):
    """(first, n) of rank's contiguous share of [first, first + n_total)."""
    base, extra = divmod(n_total, world)
    start = first + rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def merge_in_rank_order(parts):
    """parts: list over ranks of (sum, sumsq) arrays -> merged (sum, sumsq),
    added in rank order."""
    s = np.zeros_like(np.asarray(parts[0][0], np.float64))
    q = np.zeros_like(s)
    for ps, pq in parts:
        s = s + np.asarray(ps, np.float64)
        q = q + np.asarray(pq, np.float64)
    return s, q


def gather_sums(sum_, sumsq, dist, group=None, device="cpu"):
    """Gather every rank's (sum, sumsq) on all ranks (torch.distributed, any
    backend; device "cuda" for NCCL, whose collectives take device tensors)
    and merge them in rank order."""
    import torch
    t = torch.from_numpy(np.concatenate([np.asarray(sum_, np.float64),
                                         np.asarray(sumsq, np.float64)])).to(device)
    world = dist.get_world_size(group)
    outs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(outs, t, group=group)
    n = len(sum_)
    return merge_in_rank_order([(o[:n].cpu().numpy(), o[n:].cpu().numpy()) for o in outs])


def statistics(sum_, sumsq, n_histories):
    """Mean and standard error per bin (Estimator.cpp:347-367, one cycle)."""
    N = float(n_histories)
    m = np.asarray(sum_) / N
    var = (np.asarray(sumsq) / N - m * m) / (N - 1.0)
    return m, np.sqrt(var)
