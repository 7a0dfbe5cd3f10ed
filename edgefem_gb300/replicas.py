"""Multi-GPU sweeps as independent replicas (one process per GPU).

A frequency sweep is a set of independent (instance, frequency) solves that
share only the read-only mesh: there is no exchange step, so N GPUs take
disjoint contiguous slices of the frequency list, solve them with the
batched engine, and the small S matrices are gathered at the end.  No
collective runs on the data path; `torch.distributed` (NCCL on GPUs, gloo
on CPU) is used only to gather results and to take the slowest rank's time.
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence

import numpy as np


def shard_bounds(n: int, rank: int, world: int) -> tuple:
    """[lo, hi) of rank's contiguous share of n units (sizes differ by <= 1)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(value: float) -> float:
    """Largest value over all ranks (the value itself without a process group)."""
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sharded_sweep(solve: Callable[[np.ndarray], np.ndarray], freqs: Sequence[float]) -> np.ndarray:
    """Solve this rank's slice of `freqs` with `solve(freq_slice) -> S[slice]`
    and return the full S[len(freqs), ...] on every rank, in frequency order."""
    f = np.asarray(freqs, np.float64)
    dist = _dist()
    if dist is None:
        return np.asarray(solve(f))
    rank, world = dist.get_rank(), dist.get_world_size()
    lo, hi = shard_bounds(f.size, rank, world)
    local = np.asarray(solve(f[lo:hi])) if hi > lo else None
    parts: list = [None] * world
    dist.all_gather_object(parts, (lo, local))
    parts = sorted((p for p in parts if p[1] is not None), key=lambda p: p[0])
    return np.concatenate([p[1] for p in parts], axis=0)
