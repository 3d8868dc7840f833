"""Several GPUs: walkers and queries are independent, so N GPUs run N
replicas of the graph, each on work of its own, with no collective on the
data path (the reference is single-node shared memory; there is nothing to
exchange).  Only the measurement is reduced across ranks: the slowest rank's
time and the summed steps.  One process per GPU, launched by torchrun."""
from __future__ import annotations

import os

_GOLDEN = 0x9E3779B97F4A7C15


def rank_env():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(seed: int, rank: int) -> int:
    """Philox key of `rank`'s replica: rank 0 keeps `seed`, the others get
    distinct keys, so replicas draw independent streams."""
    return (seed + rank * _GOLDEN) & 0xFFFFFFFFFFFFFFFF


def shard(total: int, rank: int, world: int):
    """Contiguous [begin, end) block of `total` items for `rank` (sizes differ by at most one)."""
    base, extra = divmod(total, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def reduce_timing(seconds: float, steps: float, world: int, device=None):
    """(max seconds, summed steps) over the ranks of the default process group."""
    if world <= 1:
        return float(seconds), float(steps)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    s = torch.tensor([float(steps)], dtype=torch.float64, device=device)
    dist.all_reduce(s)
    return float(t.item()), float(s.item())
