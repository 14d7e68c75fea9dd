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


class ShardedPlan:
    """One 2D NFFT whose nonuniform points are split over the ranks of a
    process group, one GPU per rank: each rank holds a library plan of the
    full N1 x N2 problem bound to its own points.

    forward(F): every rank gathers its points from the same coefficients
    (outputs stay sharded; no collective).  adjoint(f_local): every rank
    spreads, transforms and crops its points, then one sum all-reduce of
    the N1 x N2 result (NCCL on GPUs) gives every rank the full adjoint.
    """

    def __init__(self, N1: int, N2: int, sigma: float = 2.0, K: int = 6, precision: str = "f32",
                 stream: torch.cuda.Stream | None = None, group=None):
        from .nfft import Plan
        self.plan = Plan(N1, N2, sigma=sigma, K=K, precision=precision, stream=stream)
        self.group = group
        self.world = dist.get_world_size(group) if dist.is_available() and dist.is_initialized() else 1
        self.rank = dist.get_rank(group) if self.world > 1 else 0

    def set_points(self, x1: torch.Tensor, x2: torch.Tensor, units: str = "unit", full: bool = False,
                   sync: bool = True) -> None:
        """Bind this rank's points: x1, x2 are its own slice, or (full=True)
        the whole point set, of which the rank keeps shard_bounds' slice."""
        if full:
            s, e = shard_bounds(x1.numel(), self.rank, self.world)
            x1, x2 = x1[s:e].contiguous(), x2[s:e].contiguous()
        self.plan.set_points(x1, x2, units=units, sync=sync)

    def forward(self, F: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        return sharded_forward(lambda c: self.plan.forward(c, out=out), F)

    def adjoint(self, f_local: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        return sharded_adjoint(lambda v: self.plan.adjoint(v, out=out), f_local, self.group)

    def synchronize(self) -> None:
        self.plan.synchronize()

    def close(self) -> None:
        self.plan.close()
