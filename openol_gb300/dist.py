"""Multi-GPU partitioning (host side).

The path has no exchange step that needs a collective: holograms are
independent, propagations in a batch are independent, and a Fresnel/exact
CGH hologram splits by pixel rows.  So N GPUs run replicas or disjoint shards,
one process per GPU, and the only communication is gathering results (when a
caller wants them on one rank) and reducing timings.
"""
from __future__ import annotations

import os


def rank_world():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def shard_items(n_items, rank, world):
    """Contiguous, balanced split of range(n_items): [start, stop) for `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_by_cost(costs, world):
    """Greedy largest-first assignment of items with the given costs to `world`
    ranks (for uneven batches: a 4096^2 field costs 64x a 512^2 one).
    Returns one list of item indices per rank; every item appears once."""
    order = sorted(range(len(costs)), key=lambda i: -costs[i])
    loads = [0.0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: loads[k])
        out[r].append(i)
        loads[r] += costs[i]
    for lst in out:
        lst.sort()
    return out


def hologram_rows(ny, rank, world):
    """Rows [h0, h1) of an ny-row hologram computed by `rank` (CGH shards by rows;
    a shard is the hologram of the points shifted up by h0 pixels)."""
    return shard_items(ny, rank, world)
