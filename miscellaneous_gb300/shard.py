"""Host-side sharding of one 2D NFFT across ranks (one process per GPU).

The points are the unit that shards:
  * type 2 (forward): every rank holds the full N1 x N2 coefficients, gathers
    at its own slice of the points; outputs stay sharded -- no exchange.
  * type 1 (adjoint / spreading): every rank spreads, transforms and crops its
    own slice (all linear), then ONE all-reduce (sum) of the N1 x N2 result --
    four times smaller than reducing the sigma^2-oversampled grid.
Independent transforms (batches) shard whole, with no exchange.

The local transform is passed in as a callable, so the same logic drives the
GPU plans (NCCL process group) and the CPU tests (gloo process group).
"""
from __future__ import annotations

from typing import Callable

import torch
import torch.distributed as dist


def shard_bounds(M: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous slice [start, end) of M points owned by `rank`; sizes differ by at most one."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(M, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def sharded_forward(local_type2: Callable[[torch.Tensor], torch.Tensor], F: torch.Tensor) -> torch.Tensor:
    """Forward on this rank's points; the result is this rank's slice (no collective)."""
    return local_type2(F)


def sharded_adjoint(local_type1: Callable[[torch.Tensor], torch.Tensor], f_local: torch.Tensor,
                    group=None) -> torch.Tensor:
    """Adjoint over all ranks' points: local type 1 of this rank's slice, then
    one sum all-reduce of the N1 x N2 coefficients."""
    F = local_type1(f_local)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(F, op=dist.ReduceOp.SUM, group=group)
    return F


def shard_batch(n_transforms: int, rank: int, world: int) -> list[int]:
    """Round-robin assignment of independent transforms to ranks."""
    return list(range(rank, n_transforms, world))
