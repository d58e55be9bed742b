"""Replica-parallel helpers: several GPUs (one process each) beamform disjoint work.

Delay-and-sum has no exchange step: requests, frames and pixel tiles are independent,
and every ``dimension`` mode writes disjoint outputs per pixel
(+mex/source/das_c.cpp:324-353).  Multi-GPU use is therefore replicas: each rank
takes its own share of the requests (or of an ensemble's frames) and nothing is
communicated on the data path; the only collective is the timing reduction.
"""
from __future__ import annotations

from typing import List

import torch


def shard(n_items: int, rank: int, world: int) -> List[int]:
    """Round-robin share of ``n_items`` (requests or frames) for ``rank`` of ``world``."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(range(rank, n_items, world))


def frame_range(n_frames: int, rank: int, world: int):
    """Contiguous block of frames for ``rank`` (ensembles keep frames in one launch)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(n_frames, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank scalar (e.g. a step time) over the process group; the
    value itself without an initialised group."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
