"""Replica sharding of independent walk entries across ranks (no data-path collective).

Entries, ensembles and walker ranges are independent (the reference shards them
as SLURM array tasks, scripts/fit_data.py:472-504); under torchrun each rank
walks a contiguous block and only the per-entry results travel, once, to rank 0.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple


def shard_range(n: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous [start, stop) block of n items for `rank` of `world` (sizes differ by <= 1)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(int(n), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard(items: Sequence, rank: int, world: int) -> list:
    a, b = shard_range(len(items), rank, world)
    return list(items[a:b])


def max_over_ranks(value: float) -> float:
    """Max of a per-rank float (e.g. elapsed seconds) over the process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_rank0(obj) -> List:
    """Per-rank objects collected on rank 0 in rank order (None elsewhere)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out
