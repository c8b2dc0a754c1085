"""Data-parallel history sharding over ranks (one process per GPU).

Histories are independent and the Philox keying makes every history's result
independent of where it runs, so N GPUs split a job into N disjoint,
contiguous history ranges and never talk during transport.  The one exchange
is at the end: per-bin (sum, sum of squares) of every rank, merged in rank
order so the merged result does not depend on arrival order.

FP64 runs also keep those sums exactly (include/mcgpu.h, mc_exact_sums_read:
integers in units of 2^-1074 as EXACT_LIMBS signed 64-bit limbs).  Exact
sums of disjoint ranges added limb by limb and rounded once equal, bit for
bit, the rounded exact sums of one run over all the histories
(merge_exact, gather_exact, round_exact).
"""
from __future__ import annotations

import math

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


EXACT_LIMBS = 68   # MC_EXACT_LIMBS
_DIGIT = 1 << 32


def exact_int(value: float) -> int:
    """A finite double as an exact integer number of 2^-1074 units."""
    import fractions
    q = fractions.Fraction(value) * (1 << 1074)
    assert q.denominator == 1
    return int(q)


def limbs_of_int(M: int) -> np.ndarray:
    """The normalised limbs of M (units of 2^-1074): limbs 0..K-2 the base
    2^32 digits, the last one the signed rest (Python's floor shift)."""
    out = np.zeros(EXACT_LIMBS, np.int64)
    for j in range(EXACT_LIMBS - 1):
        out[j] = (M >> (32 * j)) & (_DIGIT - 1)
    out[-1] = M >> (32 * (EXACT_LIMBS - 1))
    return out


def int_of_limbs(limbs) -> int:
    return sum(int(v) << (32 * j) for j, v in enumerate(np.asarray(limbs, np.int64)))


def exact_limbs_from_values(rows) -> np.ndarray:
    """Exact sums of per-history rows [n, bins] (sum of the values and of
    their FP64 squares), shaped [bins, 2, EXACT_LIMBS]: what the library
    keeps for the same histories."""
    rows = np.asarray(rows, np.float64)
    nb = rows.shape[1] if rows.ndim == 2 else 0
    out = np.zeros((nb, 2, EXACT_LIMBS), np.int64)
    for b in range(nb):
        col = rows[:, b]
        nz = col[col != 0.0]
        out[b, 0] = limbs_of_int(sum(exact_int(float(v)) for v in nz))
        sq = [float(v) * float(v) for v in nz]
        out[b, 1] = limbs_of_int(sum(exact_int(x) for x in sq if math.isfinite(x)))
    return out


def merge_exact(parts) -> np.ndarray:
    """Limb-wise sum of exact sums (any order), normalised."""
    parts = [np.asarray(p, np.int64) for p in parts]
    out = np.zeros_like(parts[0])
    flat_in = [p.reshape(-1, EXACT_LIMBS) for p in parts]
    flat_out = out.reshape(-1, EXACT_LIMBS)
    for i in range(flat_out.shape[0]):
        flat_out[i] = limbs_of_int(sum(int_of_limbs(f[i]) for f in flat_in))
    return out


def round_exact(limbs) -> np.ndarray:
    """Nearest doubles (ties to even) of exact values: Python's integer
    true division rounds correctly."""
    a = np.asarray(limbs, np.int64)
    flat = a.reshape(-1, EXACT_LIMBS)
    return np.array([int_of_limbs(r) / (1 << 1074) for r in flat], np.float64).reshape(a.shape[:-1])


def gather_exact(limbs, dist, group=None, device="cpu"):
    """Gather every rank's exact sums ([bins, 2, EXACT_LIMBS] int64) and
    merge them: the same limbs on every rank, whatever the arrival order."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(limbs, np.int64)).to(device)
    world = dist.get_world_size(group)
    outs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(outs, t, group=group)
    return merge_exact([o.cpu().numpy() for o in outs])
