"""Replica sharding across ranks (one process per GPU, no data exchange).

The focal path shards by independent units -- DEM tiles of a batch, bands of
a stack, or whole rasters -- so N GPUs run N replicas with no collective on
the data path.  ``assign`` splits units across ranks (longest-first greedy on
pixel counts, deterministic on every rank); ``max_over_ranks`` reduces timings
with the job's process group (the slowest rank defines the step time).
"""

from __future__ import annotations


def assign(sizes, world_size: int, rank: int) -> list[int]:
    """Indices of the units rank ``rank`` processes, balancing total size."""
    if world_size < 1 or not (0 <= rank < world_size):
        raise ValueError(f"bad rank {rank} for world size {world_size}")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    load = [0] * world_size
    owner = [0] * len(sizes)
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += int(sizes[i])
    return [i for i in range(len(sizes)) if owner[i] == rank]


def max_over_ranks(values, device=None):
    """Element-wise max of ``values`` over the process group (identity if none)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]
