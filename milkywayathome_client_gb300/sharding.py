"""Sharded evaluation across ranks: the reference's slicing and composition.

The reference's distributed evaluator (cpu/astronomy_worker.c:67-143,
cpu/mpi_astronomy.c) gives each rank a contiguous slice of the linearised
(mu, nu, r) cell index of every integral area (split_astronomy_parameters,
cpu/parameters.c:502-522) and of the catalogue (split_star_points,
cpu/star_points.c:105-131); ranks evaluate their slices, the integrals are
summed (integral_compose), every rank evaluates its stars' likelihood with the
summed integrals, and the likelihood sums are added (likelihood_compose:
prob_sum / (N - bad_jacobians) - 3).

Here the cross-rank sums are gathered and added in rank order with a
compensated (TwoSum) accumulation, so the composed result is the same
whatever reduction tree the collective library uses.  The collective is
torch.distributed (gloo on CPU, nccl on GPUs); every run of this build has one
GPU, so multi-GPU evaluation is replicas only and these functions are tested
with CPU ranks.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np


def slice_bounds(total: int, rank: int, nranks: int):
    """[first, last) of rank's slice of `total` units: the reference's
    (int)(total * (rank / nranks)) formula (cpu/parameters.c:511-512,
    cpu/star_points.c:113-114)."""
    if nranks < 1 or not 0 <= rank < nranks:
        raise ValueError("rank must be in [0, nranks)")
    first = int(float(total) * (float(rank) / float(nranks)))
    last = int(float(total) * ((float(rank) + 1.0) / float(nranks)))
    return first, last


def compensated_sum(rows: np.ndarray) -> np.ndarray:
    """Column sums of rows [R][n] added in row order with TwoSum."""
    rows = np.asarray(rows, dtype=np.float64)
    s = np.zeros(rows.shape[1:], dtype=np.float64)
    c = np.zeros_like(s)
    for r in rows:
        t = s + r
        bp = t - s
        c += (s - (t - bp)) + (r - bp)
        s = t
    return s + c


def allreduce_sum(values, group=None) -> np.ndarray:
    """Sum a float64 vector over all ranks: all-gather, then a compensated sum
    in rank order (identical on every rank, independent of the collective's
    own reduction order).  Without an initialised process group it is the
    identity."""
    import torch
    import torch.distributed as dist
    v = np.ascontiguousarray(values, dtype=np.float64)
    if not (dist.is_available() and dist.is_initialized()):
        return v.copy()
    world = dist.get_world_size(group)
    t = torch.from_numpy(v.copy())
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    return compensated_sum(np.stack([p.numpy() for p in parts]))


def integral_compose(rank_integrals: Sequence[Sequence[float]]) -> np.ndarray:
    """integral_compose (cpu/astronomy_worker.c:67-92): the (1 + S) integrals
    of each rank's slice, already cut-subtracted, summed over ranks."""
    return compensated_sum(np.asarray(rank_integrals, dtype=np.float64))


def likelihood_compose(rank_results: Sequence[Sequence[float]], total_stars: int) -> float:
    """likelihood_compose (cpu/astronomy_worker.c:121-143): rank_results[r] =
    (prob_sum, bad_jacobians) of rank r's stars; returns
    sum prob_sum / (N - sum bad_jacobians) - 3."""
    s = compensated_sum(np.asarray(rank_results, dtype=np.float64).reshape(-1, 2))
    return float(s[0] / (float(total_stars) - s[1]) - 3.0)
