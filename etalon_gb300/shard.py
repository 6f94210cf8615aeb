"""Sharding of independent simulations across GPUs (one process per GPU).

Batched workloads — parameter sweeps, design variants — are independent simulations, so N
GPUs split them with no exchange on the data path: each rank steps its own share as one
batch and only results travel. ``shard`` balances the shares by cell count (largest first
onto the least-loaded rank, ties to the lower rank), which is deterministic, so every rank
computes the same assignment without communicating.
"""

from __future__ import annotations

from collections.abc import Sequence


def assignment(cells: Sequence[int], world: int) -> list[int]:
    """Rank of each simulation, given its cell count."""
    if world < 1:
        raise ValueError("world must be at least 1")
    load = [0] * world
    rank = [0] * len(cells)
    for k in sorted(range(len(cells)), key=lambda q: (-int(cells[q]), q)):
        r = min(range(world), key=lambda q: (load[q], q))
        rank[k] = r
        load[r] += int(cells[k])
    return rank


def shard(items: Sequence, cells: Sequence[int], rank: int, world: int) -> list:
    """The items that rank ``rank`` of ``world`` steps, in their original order."""
    owner = assignment(cells, world)
    return [it for it, r in zip(items, owner) if r == rank]
