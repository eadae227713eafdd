"""Multi-GPU use of the renderer: replicas and view sharding.

A frame is never split across GPUs: a screen split would need every shadow map
on every GPU. The units that shard with no exchange step are whole frames (each
rank is a replica that renders its own frames) and the views of a batch (each
rank renders a contiguous range of views into its own context). The only
communication is the host-side gather of per-rank results to rank 0, after the
timed region; nothing on the data path is a collective.
"""
from __future__ import annotations


def shard_range(count: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [begin, end) share of `count` units for `rank` of `world`.
    The first `count % world` ranks take one extra unit; every unit is owned by
    exactly one rank, in order, so concatenating the ranks' results in rank
    order gives the single-GPU order."""
    if world < 1 or not 0 <= rank < world or count < 0:
        raise ValueError(f"bad shard request: count={count} rank={rank} world={world}")
    base, extra = divmod(count, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def gather_to_rank0(obj, world: int):
    """Gathers one picklable object per rank on rank 0 (in rank order); other
    ranks get None. With world == 1 returns [obj]."""
    if world == 1:
        return [obj]
    import torch.distributed as dist

    rank = dist.get_rank()
    out = [None] * world if rank == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


def merge_in_rank_order(parts: list[list]) -> list:
    """Concatenates per-rank result lists (each in its shard's order)."""
    merged = []
    for p in parts:
        merged.extend(p)
    return merged
