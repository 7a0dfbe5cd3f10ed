"""Multi-GPU sweeps: one process per GPU, frequencies sharded across ranks.

A frequency sweep is a set of independent (instance, frequency) solves that
share only the read-only mesh (src/sweep.cpp:249-329 loops over them one at
a time): there is no exchange step, so N GPUs take disjoint shares of the
frequency list, solve them with the batched engine, and the small S
matrices are gathered at the end.  No collective runs on the data path;
`torch.distributed` (NCCL on GPUs, gloo on CPU) is used only to gather the
results and to take the slowest rank's time.

Shares are interleaved by default (rank r takes frequencies r, r + N, ...),
so every rank gets frequencies from the whole band: the iteration count of
a solve grows with frequency, and contiguous slices would leave the top of
the band to the last rank.
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


def shard_indices(n: int, rank: int, world: int, interleave: bool = True) -> np.ndarray:
    """Indices of rank's share of n units: every world-th from rank
    (interleaved) or the contiguous slice of shard_bounds."""
    lo, hi = shard_bounds(n, rank, world)
    return np.arange(rank, n, world) if interleave else np.arange(lo, hi)


def _dist():
    try:
        import torch.distributed as dist
    except Exception:  # torch absent: no process group can exist
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def world_info() -> tuple:
    """(rank, world size) of the current process group, (0, 1) without one."""
    dist = _dist()
    if dist is None:
        return 0, 1
    return dist.get_rank(), dist.get_world_size()


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


def sharded_sweep(solve: Callable[[np.ndarray], np.ndarray], freqs: Sequence[float],
                  interleave: bool = True) -> np.ndarray:
    """Solve this rank's share of `freqs` with `solve(freq_share) -> S[share]`
    and return the full S[len(freqs), ...] on every rank, in frequency order.
    Without a process group (or with one rank) this is solve(freqs)."""
    f = np.asarray(freqs, np.float64)
    rank, world = world_info()
    if world <= 1:
        return np.asarray(solve(f))
    idx = shard_indices(f.size, rank, world, interleave)
    local = np.asarray(solve(f[idx])) if idx.size else None
    parts: list = [None] * world
    _dist().all_gather_object(parts, (idx, local))
    first = next(p[1] for p in parts if p[1] is not None)
    out = np.empty((f.size,) + first.shape[1:], first.dtype)
    for ids, loc in parts:
        if loc is not None:
            out[ids] = loc
    return out
