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


def evaluate_sharded(params_path: str, stars_path: str, theta, precision: int = 0, group=None, device: int = 0):
    """One evaluation sharded over the ranks of the process group, as the
    reference's distributed client runs it (cpu/astronomy_worker.c,
    cpu/mpi_astronomy.c), on this rank's GPU through the library:

      1. this rank's cells of every area (split_astronomy_parameters) are
         integrated (mwsep_ctx_integrals, integral_f);
      2. the ranks' cut-subtracted integrals are summed (integral_compose,
         allreduce_sum);
      3. this rank's stars (split_star_points) are evaluated against the sum
         (mwsep_ctx_likelihood, likelihood_f);
      4. the ranks' (prob_sum, bad_jacobians) are summed and composed
         (likelihood_compose).

    The only exchanges are the two host-side sums.  Without an initialised
    process group it is one rank's whole evaluation.  Returns
    (integrals [1 + S], log-likelihood)."""
    import torch.distributed as dist
    from .separation import AstronomyParameters, Context, StarPoints
    world = dist.get_world_size(group) if dist.is_available() and dist.is_initialized() else 1
    rank = dist.get_rank(group) if world > 1 else 0
    ap = AstronomyParameters.read(params_path)
    sp = StarPoints.read(stars_path)
    total_stars = sp.number_stars
    if world > 1:
        ap.split(rank, world)
        sp.split(rank, world)
    with Context(device) as ctx:
        ctx.set_problem(ap)
        mine = ctx.integrals(theta, precision)
        integrals = allreduce_sum(mine.integrals, group)
        lk = np.zeros(2)
        if sp.number_stars > 0:
            ctx.set_stars(sp)
            r = ctx.likelihood(theta, integrals, precision)
            lk[0] = r.prob_sum
    lk = allreduce_sum(lk, group)
    return integrals, likelihood_compose([lk], total_stars)
