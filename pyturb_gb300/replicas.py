"""Multi-GPU replicas: how independent work is split across ranks.

The phase-screen path has no data-path exchange: Monte-Carlo screens are
independent draws and frozen-flow frames are random access in time. So N
GPUs run N replicas, one process per GPU, each on a disjoint share:

- Monte-Carlo: screen indices are split into contiguous ranges and each rank
  draws from its own stream, ``SeedSequence(seed).spawn(world)[rank]``, so
  the union over ranks is a set of independent screens whatever ``world`` is.
- Frames: each rank renders its own time window.

Only timing uses a collective: the slowest rank's time (``max_over_ranks``).
"""

from __future__ import annotations

from typing import Tuple

import numpy as np


def shard(total: int, rank: int, world: int) -> Tuple[int, int]:
    """(start, count) of rank's contiguous share of ``total`` items."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    if total < 0:
        raise ValueError("total must be >= 0")
    base, extra = divmod(int(total), int(world))
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def rank_seed(seed: int, rank: int, world: int) -> int:
    """An integer seed for rank's own noise stream, independent across ranks."""
    child = np.random.SeedSequence(seed).spawn(world)[rank]
    return int(child.generate_state(1, dtype=np.uint64)[0])


def time_window(rank: int, step: int, frames_per_step: int, dt: float,
                stride_frames: int = 1_000_000) -> np.ndarray:
    """Frame times of ``step`` on ``rank``: windows never overlap across ranks
    while ``step * frames_per_step < stride_frames``."""
    if (step + 1) * frames_per_step > stride_frames:
        raise ValueError("time windows of different ranks would overlap")
    t0 = (rank * stride_frames + step * frames_per_step) * dt
    return t0 + dt * np.arange(frames_per_step)


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Largest ``value`` over all ranks of the default process group (or value)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
