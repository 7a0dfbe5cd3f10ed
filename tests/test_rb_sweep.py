"""Reduced-basis initial guesses of the batched engine (BatchOptions.rb_samples):
the sweep solves a few evenly spaced sample frequencies first and starts
every column from the Galerkin solution on their solutions.  S must be that
of the cold solve (same tolerance 1e-8 on the true residual; |dS| <= 1e-6
here, as for every batched result) and of the oracle's direct solve."""
import math

import numpy as np
import pytest

import edgefem_oracle as O
import edgefem_gb300 as em
from edgefem_gb300.mesh import box_tet_mesh

pytestmark = pytest.mark.gpu
A = 0.02286
SLAB = 2.2 * (1 - 0.001j)


def guide(grid=(8, 4, 20), slab=True):
    m = em.waveguide_mesh(*grid, slab=(20e-3, 30e-3) if slab else None)
    M = em.Mesh.from_arrays(m)
    bc = em.build_edge_pec(M, 1)
    mode = em.solve_te10_mode(em.RectWaveguidePort(A, 0.01016), 10e9)
    ports = [em.build_wave_port_2d(M, t, mode, bc.dirichlet_edges, (math.pi / A) ** 2) for t in (2, 3)]
    p = em.MaxwellParams()
    if slab:
        p.set_eps_r_region(101, SLAB)
    return m, em.BatchInstance(M, p, bc, ports)


def sample_indices(F, n):
    return sorted(set(int(math.floor(i * (F - 1) / (n - 1) + 0.5)) for i in range(n)))


def test_rb_eigenmode_sweep_matches_cold_and_oracle(gpu):
    m, inst = guide()
    freqs = np.linspace(8e9, 12e9, 48)
    S0, st0 = gpu.sparams_eigenmode_batched([inst], freqs, em.BatchOptions(rb_samples=0))
    S1, st1 = gpu.sparams_eigenmode_batched([inst], freqs, em.BatchOptions(rb_samples=16))
    assert st0["rb_samples"] == 0
    assert st1["rb_samples"] == 16 and 16 <= st1["rb_basis"] <= 32
    assert st1["n_converged"] == st1["n_total"] == 96 and st1["max_residual"] <= 1e-8
    assert st1["rb_done_at_guess"] > 0
    assert np.abs(S1 - S0).max() <= 1e-6
    # a frequency that is not a sample, against the oracle's direct solve
    k = next(i for i in range(48) if i not in sample_indices(48, 16))
    prob = O.make_problem(m)
    f = freqs[k]
    eps = O.tet_eps(prob, 2 * math.pi * f, eps_regions={101: SLAB})
    Sr = O.calculate_sparams_eigenmode(prob, 2 * math.pi * f, O.waveguide_ports(prob, A, f), eps)
    assert np.abs(S1[0, k] - Sr).max() <= 1e-6


def test_rb_fewer_iterations_than_cold(gpu):
    """With 16 sample frequencies the guesses do the work of the other
    columns: their iterations (the sample columns report those of their
    sample solve) are a small fraction of the cold solve's."""
    _, inst = guide()
    freqs = np.linspace(8e9, 12e9, 48)
    s0 = gpu.BatchSolver([inst], freqs, em.BatchOptions(rb_samples=0))
    s0.solve()
    _, it0, _ = s0.rhs_stats()
    s1 = gpu.BatchSolver([inst], freqs, em.BatchOptions(rb_samples=16))
    s1.solve()
    st1, it1, r1 = s1.rhs_stats()
    samples = sample_indices(48, 16)
    rest = [i for i in range(48) if i not in samples]
    assert (st1 == 1).all() and (r1 <= 1e-8).all()
    assert it1[0, rest].sum() <= 0.25 * it0[0, rest].sum()
    assert (it1[0, samples] >= it0[0, samples] * 0.8).all()  # samples solved to a tenth of the tolerance


def test_rb_driven_lumped_ports_abc_debye(gpu):
    """Driven ports (w w^T / Z0 blocks), the jk0 absorbing wall and a Debye
    medium enter the Galerkin system through the port-face terms."""
    m = box_tet_mesh(6, 6, 6, 0.02, 0.02, 0.02)
    M = em.Mesh.from_arrays(m)
    bc = em.BC()
    ports = [gpu.build_lumped_port(M, t, 50.0, (1.0, 0.0, 0.0)) for t in (2, 3)]
    p = em.MaxwellParams()
    p.use_abc = True
    p.abc_surface_tags = {1}
    for tag in set(int(v) for v in m.tet_phys):
        p.set_debye_region(tag, 4.488, 4.312, 1.0 / (2 * math.pi * 3e9))
    freqs = np.linspace(2.5e9, 4e9, 40)
    cold, st0 = gpu.frequency_sweep_batched(M, p, bc, ports, freqs, em.BatchOptions(formulation=1, rb_samples=0))
    warm, st1 = gpu.frequency_sweep_batched(M, p, bc, ports, freqs, em.BatchOptions(formulation=1, rb_samples=8))
    assert st1["rb_samples"] == 8 and st1["n_converged"] == st1["n_total"] == 80
    assert np.abs(np.array(warm.S_matrices) - np.array(cold.S_matrices)).max() <= 1e-6


def test_rb_uneven_instances_and_repeated_samples(gpu):
    """Two meshes in one batch (a basis each); a sweep of 10 frequencies each
    listed four times, so that 16 samples land on 10 distinct frequencies and
    the repeated sample solutions add nothing to the basis (dropped by the
    Gram-Schmidt test)."""
    _, i1 = guide((8, 4, 20))
    _, i2 = guide((6, 3, 16), slab=False)
    freqs = np.repeat(np.linspace(8.5e9, 11.5e9, 10), 4)
    S0, _ = gpu.sparams_eigenmode_batched([i1, i2], freqs, em.BatchOptions(rb_samples=0))
    S1, st = gpu.sparams_eigenmode_batched([i1, i2], freqs, em.BatchOptions(rb_samples=16))
    assert st["rb_samples"] == 16 and st["rb_basis"] <= 20
    assert st["n_converged"] == st["n_total"]
    assert np.abs(S1 - S0).max() <= 1e-6


def test_rb_off_for_short_sweeps(gpu):
    _, inst = guide()
    freqs = np.linspace(8e9, 12e9, 20)  # fewer than 2 x 16 sample frequencies
    S, st = gpu.sparams_eigenmode_batched([inst], freqs, em.BatchOptions(rb_samples=16))
    assert st["rb_samples"] == 0 and st["n_converged"] == st["n_total"]
    # 40 sample frequencies x 2 ports would exceed 64 basis columns: capped at 32
    _, st = gpu.sparams_eigenmode_batched([inst], np.linspace(8e9, 12e9, 80), em.BatchOptions(rb_samples=40))
    assert st["rb_samples"] == 32 and st["n_converged"] == st["n_total"]


def test_rb_with_reordering_and_split_sweeps(gpu):
    """The sample engine renumbers like the main one (reorder = 1), and a
    sweep longer than one batch (80 frequencies x 2 ports > 128 columns,
    solved as two batches of 64 and 16 frequencies) runs the reduced-basis
    phase per batch where it is long enough."""
    _, inst = guide()
    freqs = np.linspace(8e9, 12e9, 80)
    S0, st0 = gpu.sparams_eigenmode_batched([inst], freqs, em.BatchOptions(rb_samples=0))
    S1, st1 = gpu.sparams_eigenmode_batched([inst], freqs, em.BatchOptions(rb_samples=16, reorder=True))
    assert st1["rb_samples"] == 16  # the 64-frequency batch only
    assert st1["n_converged"] == st1["n_total"] == 160
    assert np.abs(S1 - S0).max() <= 1e-6


def test_rb_with_fp32_mass_precision(gpu):
    """precision = 1 (double-float K, FP32 M): the sample engine runs in the
    same precision and the guesses feed it the same way."""
    _, inst = guide()
    freqs = np.linspace(8e9, 12e9, 40)
    S0, _ = gpu.sparams_eigenmode_batched([inst], freqs, em.BatchOptions(precision=1, rb_samples=0))
    S1, st = gpu.sparams_eigenmode_batched([inst], freqs, em.BatchOptions(precision=1, rb_samples=16))
    assert st["rb_samples"] == 16 and st["n_converged"] == st["n_total"] == 80
    assert np.abs(S1 - S0).max() <= 1e-6
