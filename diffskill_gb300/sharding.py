"""Scene sharding across ranks (one process per GPU).

Scenes are independent (no shared grid or tools), so the path shards by scene
with no collective on the data path.  ``shard_scenes`` balances the ranks by
total particle count with a greedy longest-processing-time assignment, and
keeps each rank's scenes in their original order.
"""
from __future__ import annotations

from typing import List, Sequence


def shard_scenes(n_per_scene: Sequence[int], world: int, rank: int) -> List[int]:
    """Indices of the scenes rank ``rank`` of ``world`` runs."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of world {world}")
    load = [0] * world
    owner = [0] * len(n_per_scene)
    for i in sorted(range(len(n_per_scene)), key=lambda i: (-int(n_per_scene[i]), i)):
        r = min(range(world), key=lambda r: (load[r], r))
        owner[i] = r
        load[r] += int(n_per_scene[i])
    return [i for i in range(len(n_per_scene)) if owner[i] == rank]
