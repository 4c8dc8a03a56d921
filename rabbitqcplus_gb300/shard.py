"""Anchor sharding across replicas.

Anchors are independent once the read store and hash tables exist (every
replica holds all of them), so N GPUs split the anchor range with no exchange
on the data path.  Paired-end ranges keep pairs (2i, 2i+1) together.
"""
from __future__ import annotations


def shard_range(num_anchors: int, rank: int, world: int, paired: bool = False) -> tuple[int, int]:
    """[first, first+count) of anchors for `rank` of `world`, contiguous and balanced."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    unit = 2 if paired else 1
    units = num_anchors // unit
    per, extra = divmod(units, world)
    first = rank * per + min(rank, extra)
    count = per + (1 if rank < extra else 0)
    first *= unit
    count *= unit
    if rank == world - 1:
        count = num_anchors - first
    return first, count
