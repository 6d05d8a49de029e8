"""Host-side helpers for running frames on several GPUs as independent
replicas (one process per GPU, no collective on the data path).

Frames are independent units of work, so a batch of frames is partitioned
across ranks; the only cross-rank traffic is the timing reduction.
"""
from __future__ import annotations

from typing import List, Sequence


def frames_for_rank(sizes: Sequence[int], world: int, rank: int) -> List[int]:
    """Longest-processing-time assignment of frames (by particle count) to
    ranks; deterministic, every frame goes to exactly one rank."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    load = [0] * world
    owner = [0] * len(sizes)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += int(sizes[i])
    return [i for i in range(len(sizes)) if owner[i] == rank]


def max_over_ranks(value: float, device=None) -> float:
    """Largest value over all ranks of the default process group (the
    slowest replica bounds the job); the value itself when not distributed."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
