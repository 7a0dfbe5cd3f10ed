"""Sharded sweeps (one process per GPU) on CPU with gloo, world size 2:
shard bounds and indices, gather order, the max-over-ranks timing the bench
uses, and the SDK sweep entry points sharding their frequencies under a
process group.  The per-rank GPU solve is replaced by a stand-in; the GPU
solve itself is covered by the GPU tests."""
import os
import socket

import numpy as np
import pytest

from edgefem_gb300.replicas import shard_bounds, shard_indices


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
    for n in (0, 1, 7, 64):
        for world in (1, 2, 3, 8):
            for inter in (True, False):
                got = np.sort(np.concatenate([shard_indices(n, r, world, inter) for r in range(world)]))
                assert np.array_equal(got, np.arange(n))
    assert np.array_equal(shard_indices(7, 1, 3), [1, 4])


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
        S_c = sharded_sweep(solve, freqs, interleave=False)
        assert np.array_equal(S[:, :, :1], S_c[:, :, :1])
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


def _sdk_worker(rank, world, port, out_dir):
    """Each rank calls the SDK sweep entry points with its GPU solve replaced
    by a stand-in that records which frequencies it was given."""
    import torch.distributed as dist
    import edgefem_gb300 as em
    from edgefem_gb300 import sdk
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seen = {}
    try:
        def fake_driven(mesh, p, bc, ports, f, opts):
            seen["driven"] = np.array(f)
            S = np.stack([np.array([[fi * 1e-9 + 1j * rank]]) for fi in f])
            return S, {"n_converged": len(f), "n_total": len(f)}

        def fake_eigen(instances, f, opts):
            seen["eigen"] = np.array(f)
            S = np.zeros((2, len(f), 2, 2), complex)
            for k, fi in enumerate(f):
                S[:, k] = fi * 1e-9
                S[1, k, 1, 0] = -fi * 1e-9
            return S, {"n_converged": 2 * len(f)}

        sdk._frequency_sweep_batched_local = fake_driven
        sdk._sparams_eigenmode_batched_local = fake_eigen
        freqs = np.linspace(2e9, 3e9, 5)
        sw, st = em.frequency_sweep_batched(None, None, None, [None], freqs)
        driven_seen = seen["driven"]
        S_e, st_e = em.sparams_eigenmode_batched([None, None], freqs)
        sw1, st1 = em.frequency_sweep_batched(None, None, None, [None], freqs, shard=False)
        np.savez(os.path.join(out_dir, f"sdk{rank}.npz"), driven=np.array([S[0, 0] for S in sw.S_matrices]),
                 driven_seen=driven_seen, eigen=S_e, eigen_seen=seen["eigen"], ranks=st["ranks"],
                 unsharded_n=st1["n_total"])
    finally:
        dist.destroy_process_group()


def test_sdk_sweeps_shard_across_two_ranks_gloo(tmp_path):
    """frequency_sweep_batched and sparams_eigenmode_batched under a world-2
    process group: each rank solves the interleaved half of the band and
    returns the whole sweep in frequency order; shard=False solves it all."""
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_sdk_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    freqs = np.linspace(2e9, 3e9, 5)
    for r in range(2):
        d = np.load(tmp_path / f"sdk{r}.npz")
        assert np.array_equal(d["driven_seen"], freqs[r::2])
        assert np.array_equal(d["eigen_seen"], freqs[r::2])
        # every rank holds the full sweep; the stand-in marks the solving rank
        want = freqs * 1e-9 + 1j * (np.arange(5) % 2)
        assert np.allclose(d["driven"], want)
        assert d["eigen"].shape == (2, 5, 2, 2)
        assert np.allclose(d["eigen"][0, :, 0, 0], freqs * 1e-9)
        assert np.allclose(d["eigen"][1, :, 1, 0], -freqs * 1e-9)
        assert int(d["ranks"]) == 2 and int(d["unsharded_n"]) == 5
