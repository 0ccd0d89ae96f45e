"""Partitioning of the polychromatic / many-source work across ranks.

The units of the hot path (wavelengths, sources, requests) are independent;
the only exchange is a sum of the partial images (and gradients). Each rank
owns a contiguous block of units, computes its partial image with the fused
plan, and the partials are summed with one all-reduce (NCCL between GPUs,
gloo on the host). With one GPU per box this runs as independent replicas;
the block assignment and the reduction are exercised on host ranks in the
tests.
"""

from __future__ import annotations

import torch

__all__ = ["shard_range", "shard_units", "reduce_partial"]


def shard_range(n_units: int, world: int, rank: int):
    """Contiguous [lo, hi) block of ``n_units`` for ``rank`` (sizes differ by at most one)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(int(n_units), world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def shard_units(values, world: int, rank: int):
    lo, hi = shard_range(len(values), world, rank)
    return values[lo:hi]


def reduce_partial(t: torch.Tensor, group=None) -> torch.Tensor:
    """Sum a rank's partial image (or gradient) over the group, in place."""
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM, group=group)
    return t
