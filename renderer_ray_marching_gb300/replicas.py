"""Host-side logic for running the renderer as independent replicas.

The path has no exchange step: views (and radii queries) are independent
given a replicated cloud, so N processes each own one GPU, render a
disjoint share of the views and never communicate on the data path.  This
mirrors the reference's own multi-GPU form (one process per GPU, shared
work split through per-output lock files, main.cu:172-191).  The only
collective is the benchmark's max-over-ranks of the step time.
"""
from __future__ import annotations


def shard(items, rank: int, world: int):
    """Round-robin share of `items` for `rank` (stable, disjoint, covering)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return items[rank::world]


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank scalar (the slowest rank sets the job time)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
