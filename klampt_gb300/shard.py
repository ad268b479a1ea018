"""Replica sharding of independent work items (configurations, edges,
trajectories) across ranks, one GPU per rank.

The path has no exchange step: every item is independent and the robot and
environment are read-only, so ranks take contiguous ranges of the item list,
compute them with no collective on the data path, and the host gathers the
per-item results at the end (all_gather of each rank's slice).
"""

from __future__ import annotations

from typing import Callable, Tuple

import numpy as np


def shard_range(n: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous [begin, end) of n items for `rank` of `world`; sizes differ
    by at most one and the ranges tile [0, n)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def run_sharded(n: int, compute: Callable[[int, int], np.ndarray], group=None) -> np.ndarray:
    """compute(begin, end) on this rank's range, then gather every rank's
    slice (in rank order) on all ranks.  Without torch.distributed
    initialised this is compute(0, n)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return compute(0, n)
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    b, e = shard_range(n, rank, world)
    mine = compute(b, e)
    parts = [None] * world
    dist.all_gather_object(parts, mine, group=group)
    return np.concatenate(parts)
