"""Independent decks across GPUs: one process per GPU, decks assigned round
robin, no data exchange during the solves.

A single deck is never split across GPUs (the reference has one Chunk and no
domain decomposition); several GPUs help only by solving independent decks,
so scaling is weak.  The collectives here are host-side bookkeeping after the
timed work: the maximum time over ranks and the gather of per-deck results.
"""
from __future__ import annotations

from typing import Any, List, Sequence


def deck_shard(n_decks: int, rank: int, world: int) -> List[int]:
    """The deck indices rank `rank` of `world` solves (round robin)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    return list(range(rank, n_decks, world))


def max_over_ranks(value: float, dist=None) -> float:
    """The largest `value` over all ranks (the slowest rank sets the time)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def gather_by_deck(results: Sequence[Any], n_decks: int, dist=None) -> List[Any]:
    """Every rank's per-deck results, merged back into deck order."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return list(results)
    world, rank = dist.get_world_size(), dist.get_rank()
    parts: List[Any] = [None] * world
    dist.all_gather_object(parts, (rank, list(results)))
    merged: List[Any] = [None] * n_decks
    for r, res in parts:
        for k, idx in enumerate(deck_shard(n_decks, r, world)):
            merged[idx] = res[k]
    return merged
