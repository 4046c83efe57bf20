"""Multi-GPU policy: replicas only.

A single bundle-adjustment solve does not shard without an exchange in every
PCG iteration, so one process per GPU solves whole problems.  Independent
problems (a batch of local-BA windows, a stream of requests) are split across
ranks by contiguous, balanced ranges; no data-path collective is needed, only
a gather of the per-problem summaries on the host.
"""
from __future__ import annotations

from typing import Callable, Sequence


def shard_range(n_items: int, rank: int, world: int) -> range:
    """Contiguous balanced range of item indices owned by `rank`."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def solve_sharded(items: Sequence, rank: int, world: int, solve_one: Callable, gather=None) -> list:
    """Solves this rank's share with `solve_one(item)`; with `gather` (e.g.
    torch.distributed.all_gather_object) returns every rank's results in item
    order, else only this rank's."""
    mine = [(i, solve_one(items[i])) for i in shard_range(len(items), rank, world)]
    if gather is None:
        return [r for _, r in mine]
    parts = [None] * world
    gather(parts, mine)
    out = [None] * len(items)
    for part in parts:
        for i, r in part:
            if out[i] is not None:
                raise RuntimeError(f"item {i} solved twice")
            out[i] = r
    if any(r is None for r in out):
        raise RuntimeError("an item was not solved")
    return out
