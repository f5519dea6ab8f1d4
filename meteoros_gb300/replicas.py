"""Host logic of the multi-GPU layout: replicas, no collective on the data path.

Pixels, views and sessions are independent, and the only cross-pixel reads
(reprojection, TXAA) stay inside one view on one GPU, so the work shards by
view or session with each session pinned to one rank (its previous frame
stays resident there).  The one collective is on the measurement path: the
frame time reported for a run is the maximum over ranks.
"""
from __future__ import annotations


def rank_seed(seed: int, rank: int) -> int:
    """Seed of a rank's own workload (each replica renders its own session)."""
    return seed + rank


def shard(n_items: int, rank: int, world: int) -> range:
    """The contiguous block of items (sessions, views) pinned to `rank`:
    blocks differ in size by at most one and together cover 0..n_items-1."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value: float, device=None) -> float:
    """All-reduce MAX of a per-rank scalar (the slowest rank's time)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
