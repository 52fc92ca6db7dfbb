"""View sharding over ranks: one process per GPU, each holding its own copy of the volumes.

Views are independent (the reference renders them in a serial loop, projector.py:679-685), so a
multi-GPU run shards the view list and needs no collective on the forward data path. The only
exchanges are the benchmark's max-over-ranks timing and, for a sharded adjoint, one sum of the
density gradient (each rank back-projects its own views into a full-size gradient volume).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple


def shard_bounds(n: int, rank: int, world: int) -> Tuple[int, int]:
    """[begin, end) of rank's contiguous share of n items; shares differ by at most one item."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    if n < 0:
        raise ValueError("n must be >= 0")
    q, r = divmod(n, world)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)


def shard(items: Sequence, rank: int, world: int) -> List:
    b, e = shard_bounds(len(items), rank, world)
    return list(items[b:e])


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over the default process group (the value itself without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_gradient_(grad, group=None) -> None:
    """In-place sum of a gradient tensor over `group` (default: the default process group; no-op
    without one). A gloo group sums through host memory: a CUDA tensor is copied there and back."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) <= 1:
        return
    if grad.is_cuda and dist.get_backend(group) == "gloo":
        host = grad.detach().cpu()
        dist.all_reduce(host, op=dist.ReduceOp.SUM, group=group)
        grad.copy_(host)
    else:
        dist.all_reduce(grad, op=dist.ReduceOp.SUM, group=group)
