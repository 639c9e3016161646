"""Beam sharding across ranks (one rank per GPU).  Beams are independent searches, so a rank
owns a contiguous slice of them and no data crosses ranks; the only cross-rank steps are the
timing barrier and a max over ranks."""
from __future__ import annotations

from typing import List


def beams_for_rank(nbeams: int, rank: int, world: int) -> List[int]:
    """Contiguous, balanced slice of beam indices owned by `rank` (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(nbeams, world)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Largest value over all ranks (the slowest rank's time); identity without a group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None, device=None) -> float:
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
