"""Replica (one process per GPU) sweep logic on CPU with gloo, world size 2:
shard bounds, gather order, and the max-over-ranks timing the bench uses.
The per-rank solve is a stand-in; the GPU solve it replaces is covered by
the GPU tests."""
import os
import socket

import numpy as np
import pytest

from edgefem_gb300.replicas import shard_bounds


def test_shard_bounds_cover_exactly():
    for n in (0, 1, 5, 64, 101):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from edgefem_gb300.replicas import max_over_ranks, sharded_sweep
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        freqs = np.linspace(8e9, 12e9, 7)
        # stand-in per-frequency 2x2 "S": depends only on the frequency
        solve = lambda f: np.stack([np.array([[fi, 2 * fi], [3 * fi, rank]]) for fi in f]) if len(f) else None
        S = sharded_sweep(solve, freqs)
        t = max_over_ranks(10.0 + rank)
        np.save(os.path.join(out_dir, f"r{rank}.npy"), np.concatenate([S[:, :, :1].ravel(), [t]]))
    finally:
        dist.destroy_process_group()


def test_sharded_sweep_two_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    freqs = np.linspace(8e9, 12e9, 7)
    want = np.stack([[[f], [3 * f]] for f in freqs]).ravel()
    for r in range(2):
        got = np.load(tmp_path / f"r{r}.npy")
        assert np.array_equal(got[:-1], want)  # every rank holds the full sweep in order
        assert got[-1] == 11.0                 # slowest rank's time
