"""GPU parity: every hot-path entry point through the C-ABI against the
complex128 oracle on the same inputs.

Tolerances: sparsity and edge numbering bit-exact; FP64 assembly values
1e-12 relative; plain FP64 S-parameters |dS| <= 1e-8 at solver tolerance
1e-12; batched S-parameters (double-float, or complex64 with FP64 residual
replacement) |dS| <= 1e-6 at relative residual tolerance 1e-8; adjoint gradients 1e-8 relative to the oracle
adjoint and 1e-5 to central differences (h = 1e-4)."""
import json
import math
import os

import numpy as np
import pytest

import edgefem_oracle as O
from conftest import GOLDEN, published

import edgefem_gb300 as em

pytestmark = pytest.mark.gpu
A = 0.02286
TIGHT = em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=100000)


def setup(m, freq=10e9, eps_regions=None, eps_tet=None):
    M = em.Mesh.from_arrays(m)
    bc = em.build_edge_pec(M, 1)
    mode = em.solve_te10_mode(em.RectWaveguidePort(A, 0.01016), freq)
    ports = [em.build_wave_port_2d(M, t, mode, bc.dirichlet_edges, (math.pi / A) ** 2) for t in (2, 3)]
    p = em.MaxwellParams()
    p.omega = 2 * math.pi * freq
    for k, v in (eps_regions or {}).items():
        p.set_eps_r_region(k, v)
    if eps_tet is not None:
        p.eps_r_tet = eps_tet
    return M, bc, ports, p


def oracle_S(m, freq, eps):
    prob = O.make_problem(m)
    return O.calculate_sparams_eigenmode(prob, 2 * math.pi * freq, O.waveguide_ports(prob, A, freq), eps)


def test_assembly_matches_oracle(gpu, wr90_mesh):
    for m in (wr90_mesh, em.waveguide_mesh(8, 4, 20, slab=(20e-3, 30e-3))):
        prob = O.make_problem(m)
        M, bc, _, p = setup(m, 9e9, eps_regions={101: 2.2 - 0.0022j})
        asm = gpu.assemble_maxwell(M, p, bc, [], -1)
        eps = O.tet_eps(prob, p.omega, eps_regions={101: 2.2 - 0.0022j})
        Ar, br = O.assemble_maxwell(prob, p.omega, eps)
        rp, ci, v = asm.A.csr()
        assert np.array_equal(rp, Ar.indptr) and np.array_equal(ci, Ar.indices)
        assert np.abs(v - Ar.data).max() <= 1e-12 * np.abs(Ar.data).max()
        assert np.array_equal(asm.b, br)


def test_km_split_matches_oracle(gpu):
    m = em.waveguide_mesh(6, 3, 12, slab=(20e-3, 30e-3))
    prob = O.make_problem(m)
    M, bc, _, p = setup(m, eps_regions={101: 3.0 - 0.1j})
    K, Mm = gpu.assemble_maxwell_km(M, p, bc)
    Kr, Mr = O.assemble_km(prob, O.tet_eps(prob, 0.0, eps_regions={101: 3.0 - 0.1j}))
    for Ag, Ar in ((K, Kr), (Mm, Mr)):
        rp, ci, v = Ag.csr()
        assert np.array_equal(ci, Ar.indices)
        assert np.abs(v - Ar.data).max() <= 1e-12 * np.abs(Ar.data).max()


def test_wr90_published_table_on_gpu(gpu, wr90_mesh):
    """The plain GPU path reproduces docs/validation.md:20-29."""
    wg = gpu.RectWaveguideDesign(A, 0.01016, 0.05)
    wg.set_mesh(wr90_mesh)
    wg.solve_options = TIGHT
    prob = O.make_problem(wr90_mesh)
    for row in published()["wr90_7_12ghz"]:
        f = row["freq_ghz"] * 1e9
        S = wg.sparams_at_freq(f)
        Sr = O.calculate_sparams_eigenmode(prob, 2 * math.pi * f, O.waveguide_ports(prob, A, f),
                                           np.ones(wr90_mesh.num_tets, complex))
        assert np.abs(S - Sr).max() <= 1e-8
        assert round(abs(S[0, 0]), 3) == pytest.approx(row["s11_mag"], abs=1e-9)
        assert round(abs(S[1, 0]), 4) == pytest.approx(row["s21_mag"], abs=1e-9)
        assert round(math.degrees(np.angle(S[1, 0])), 1) == pytest.approx(row["s21_phase_deg"], abs=1e-9)


def test_plain_eigenmode_slab_and_bicgstab(gpu):
    m = em.waveguide_mesh(10, 5, 24, slab=(20e-3, 30e-3))
    eps = O.tet_eps(O.make_problem(m), 0.0, eps_regions={101: 2.2 * (1 - 0.001j)})
    Sr = oracle_S(m, 11e9, eps)
    M, bc, ports, p = setup(m, 11e9, eps_regions={101: 2.2 * (1 - 0.001j)})
    S = gpu.calculate_sparams_eigenmode(M, p, bc, ports, TIGHT)
    assert np.abs(S - Sr).max() <= 1e-8
    S2 = gpu.calculate_sparams_eigenmode(M, p, bc, ports, em.SolveOptions(use_bicgstab=True, tolerance=1e-12,
                                                                           max_iterations=100000))
    assert np.abs(S2 - Sr).max() <= 1e-8


def test_solve_linear_matches_direct(gpu, wr90_mesh):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    M, bc, _, p = setup(wr90_mesh, 10e9)
    p.eps_r = 1 - 0.05j
    asm = gpu.assemble_maxwell(M, p, bc, [], -1)
    rp, ci, v = asm.A.csr()
    Ad = sp.csr_matrix((v, ci, rp), shape=(asm.A.n, asm.A.n))
    b = np.random.default_rng(0).normal(size=asm.A.n) + 1j * np.random.default_rng(1).normal(size=asm.A.n)
    b[bc.pec_array()] = 0
    x_ref = spla.spsolve(Ad.tocsc(), b)
    for bicg in (True, False):
        res = gpu.solve_linear(asm.A, b, em.SolveOptions(use_bicgstab=bicg, tolerance=1e-12, max_iterations=100000))
        assert res.converged and res.residual <= 1e-12
        assert np.linalg.norm(res.x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
        assert res.method.startswith("BiCGSTAB" if bicg else "COCG")


def test_solve_linear_preconditioners(gpu):
    """solve_linear's preconditioner choice (reference callers: assemble_maxwell
    then solve_linear, stacked_patch.py:556-559, waveguide.py:499-502): the
    matrix from assemble_maxwell carries its mesh data and gets the
    auxiliary space; the same values as a raw CSR matrix get block-Jacobi;
    use_ilut=False gives Jacobi.  Every form reaches the SuperLU solution,
    and the iteration counts order as aux < block-Jacobi < Jacobi."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    m = em.waveguide_mesh(10, 5, 24, slab=(20e-3, 30e-3))
    M, bc, ports, p = setup(m, 11e9, eps_regions={101: 2.2 * (1 - 0.001j)})
    asm = gpu.assemble_maxwell(M, p, bc, ports, 0)
    rp, ci, v = asm.A.csr()
    Ad = sp.csr_matrix((v, ci, rp), shape=(asm.A.n, asm.A.n))
    x_ref = spla.spsolve(Ad.tocsc(), asm.b)
    raw = em.sdk.SpMatC.from_csr(rp, ci, v, asm.A.n)
    its = {}
    for name, A_, opts in (("aux", asm.A, em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=200000)),
                           ("block", raw, em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=200000)),
                           ("jacobi", raw, em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=200000,
                                                           use_ilut=False)),
                           ("block_bicg", raw, em.SolveOptions(use_bicgstab=True, tolerance=1e-12,
                                                               max_iterations=200000))):
        res = gpu.solve_linear(A_, asm.b, opts)
        assert res.converged, (name, res.error_message)
        assert np.linalg.norm(res.x - x_ref) <= 1e-8 * np.linalg.norm(x_ref), name
        its[name] = res.iters
        want = {"aux": "AuxSpace", "block": "BlockJacobi", "jacobi": "+Jacobi", "block_bicg": "BlockJacobi"}[name]
        assert want in res.method, (name, res.method)
    assert its["aux"] < its["block"] < its["jacobi"], its
    # block-Jacobi on a mesh-attached matrix when asked for explicitly
    res = gpu.solve_linear(asm.A, asm.b, em.SolveOptions(use_bicgstab=False, tolerance=1e-12,
                                                         max_iterations=200000, preconditioner="block_jacobi"))
    # (FP64 atomic reduction order varies run to run: counts agree closely)
    assert res.converged and abs(res.iters - its["block"]) <= 0.05 * its["block"] and "BlockJacobi" in res.method


def test_block_jacobi_ragged_and_singular_blocks(gpu):
    """Block-Jacobi with a last block shorter than 16 rows and a singular
    diagonal block (which falls back to its diagonal): the solve still
    reaches the dense solution."""
    import scipy.sparse as sp
    rng = np.random.default_rng(3)
    n = 53
    A = np.zeros((n, n), complex)
    for i in range(n):
        for j in range(max(0, i - 3), min(n, i + 4)):
            A[i, j] = A[j, i] = 0.3 * (rng.normal() + 1j * rng.normal())
    A += np.diag(4.0 + 0.5j + rng.uniform(0, 1, n))
    A[0, :16] = A[1, :16] = A[:16, 0] = A[:16, 1] = 0.0
    A[0, 0] = A[0, 1] = A[1, 0] = A[1, 1] = 2.0  # rows 0 and 1 equal inside block 0
    A[0, 20] = A[20, 0] = 1.0  # coupling outside the block keeps A regular
    assert abs(np.linalg.det(A)) > 1e-6
    S = sp.csr_matrix(A)
    S.sort_indices()
    b = rng.normal(size=n) + 1j * rng.normal(size=n)
    x_ref = np.linalg.solve(A, b)
    raw = em.sdk.SpMatC.from_csr(S.indptr, S.indices, S.data, n)
    res = gpu.solve_linear(raw, b, em.SolveOptions(use_bicgstab=True, tolerance=1e-12, max_iterations=20000,
                                                   preconditioner="block_jacobi"))
    assert res.converged, res.error_message
    assert np.linalg.norm(res.x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def test_wwh_ports_abc_normalize_sweep(gpu):
    """calculate_sparams / normalize_port_weights / frequency_sweep with
    lumped (w w^H) ports and the jk0 ABC, against the oracle."""
    from edgefem_gb300.mesh import box_tet_mesh
    m = box_tet_mesh(6, 6, 6, 0.02, 0.02, 0.02)
    prob = O.make_problem(m)
    M = em.Mesh.from_arrays(m)
    bc = em.BC()  # no PEC: the two port faces and an absorbing wall
    ports = [gpu.build_lumped_port(M, 2, 50.0, (1.0, 0.0, 0.0)), gpu.build_lumped_port(M, 3, 50.0, (1.0, 0.0, 0.0))]
    oports = [O.build_lumped_port(prob, 2, (1.0, 0.0, 0.0), 50.0), O.build_lumped_port(prob, 3, (1.0, 0.0, 0.0), 50.0)]
    prob.pec = np.zeros(0, np.int64)
    p = em.MaxwellParams()
    p.omega = 2 * math.pi * 3e9
    p.eps_r = 2.0 - 0.05j
    p.use_abc = True
    p.abc_surface_tags = {1}
    eps = np.full(m.num_tets, 2.0 - 0.05j)
    opts = em.SolveOptions(use_bicgstab=True, tolerance=1e-12, max_iterations=200000)
    n_g = gpu.normalize_port_weights(M, p, bc, ports, opts)
    n_o = O.normalize_port_weights(prob, p.omega, eps, oports, use_abc=True, abc_tags=(1,))
    for a, b in zip(n_g, n_o):
        assert np.allclose(a.weights, b.weights, rtol=1e-8, atol=1e-12)
    S = gpu.calculate_sparams(M, p, bc, n_g, opts)
    Sr = O.calculate_sparams(prob, p.omega, eps, n_o, use_abc=True, abc_tags=(1,))
    assert np.abs(S - Sr).max() <= 1e-8
    sw = gpu.frequency_sweep(M, p, bc, n_g, [2.5e9, 3e9], opts)
    assert np.abs(sw.S_matrices[1] - Sr).max() <= 1e-8
    asm = gpu.assemble_maxwell(M, p, bc, n_g, 0)
    Ar, br = O.assemble_maxwell(prob, p.omega, eps, n_o, 0, use_abc=True, abc_tags=(1,))
    rp, ci, v = asm.A.csr()
    assert np.array_equal(ci, Ar.indices)
    assert np.abs(v - Ar.data).max() <= 1e-12 * np.abs(Ar.data).max()
    assert np.abs(asm.b - br).max() <= 1e-12 * np.abs(br).max()


@pytest.mark.parametrize("abc_type", [1, 2, 3, 4])
def test_legacy_port_abc_matches_oracle(gpu, wr90_mesh, abc_type):
    """assemble_maxwell with use_port_abc (src/assemble_maxwell.cpp:274-313):
    every type's diagonal on the wave ports' non-PEC edges, against the oracle."""
    M, bc, ports, p = setup(wr90_mesh, 10e9)
    p.use_port_abc = True
    p.port_abc_type = abc_type
    asm = gpu.assemble_maxwell(M, p, bc, ports, 0)
    prob = O.make_problem(wr90_mesh)
    oports = O.waveguide_ports(prob, A, 10e9)
    for op, gp in zip(oports, ports):  # the w w^H form uses the ports' Z0 and kc
        op.Z0, op.kc = gp.mode.Z0, gp.mode.kc
    Ar, br = O.assemble_maxwell(prob, p.omega, np.ones(wr90_mesh.num_tets, complex), oports, 0,
                                use_port_abc=True, port_abc_type=abc_type)
    rp, ci, v = asm.A.csr()
    assert np.array_equal(ci, Ar.indices)
    assert np.abs(v - Ar.data).max() <= 1e-12 * np.abs(Ar.data).max()
    assert np.abs(asm.b - br).max() <= 1e-12 * np.abs(br).max()


def _lumped_box(gpu, eps=2.0 - 0.05j, debye=None):
    """6x6x6 box, two lumped ports (faces 2, 3), absorbing wall (tag 1), no PEC."""
    from edgefem_gb300.mesh import box_tet_mesh
    m = box_tet_mesh(6, 6, 6, 0.02, 0.02, 0.02)
    M = em.Mesh.from_arrays(m)
    bc = em.BC()
    ports = [gpu.build_lumped_port(M, t, 50.0, (1.0, 0.0, 0.0)) for t in (2, 3)]
    p = em.MaxwellParams()
    p.eps_r = eps
    p.use_abc = True
    p.abc_surface_tags = {1}
    if debye is not None:
        for tag in set(int(v) for v in m.tet_phys):
            p.set_debye_region(tag, *debye)
    return m, M, bc, ports, p


def test_batched_driven_sweep_matches_plain_and_oracle(gpu):
    """frequency_sweep as one batched solve (driven w w^H/Z0 ports + jk0 ABC)
    against the per-frequency plain sweep and the oracle."""
    m, M, bc, ports, p = _lumped_box(gpu)
    freqs = [2.5e9, 3.0e9, 3.5e9, 4.0e9]
    sw, st = gpu.frequency_sweep_batched(M, p, bc, ports, freqs)
    assert st["n_converged"] == st["n_total"] == 8
    plain = gpu.frequency_sweep(M, p, bc, ports, freqs,
                                em.SolveOptions(use_bicgstab=True, tolerance=1e-12, max_iterations=200000))
    prob = O.make_problem(m)
    prob.pec = np.zeros(0, np.int64)
    oports = [O.build_lumped_port(prob, t, (1.0, 0.0, 0.0), 50.0) for t in (2, 3)]
    eps = np.full(m.num_tets, p.eps_r)
    for k, f in enumerate(freqs):
        assert np.abs(sw.S_matrices[k] - plain.S_matrices[k]).max() <= 1e-6
        Sr = O.calculate_sparams(prob, 2 * math.pi * f, eps, oports, use_abc=True, abc_tags=(1,))
        assert np.abs(sw.S_matrices[k] - Sr).max() <= 1e-6


def test_batched_debye_both_formulations(gpu):
    """A Debye dielectric (FR-4-like) through the batched engine: eigenmode
    ports against calculate_sparams_eigenmode, driven ports against
    calculate_sparams, each per frequency on the plain FP64 path."""
    tight = em.SolveOptions(use_bicgstab=True, tolerance=1e-12, max_iterations=200000)
    tau = 1.0 / (2 * math.pi * 10e9)
    m = em.waveguide_mesh(8, 4, 20, slab=(20e-3, 30e-3))
    M, bc, ports, p = setup(m)
    p.set_debye_region(101, 4.488, 4.312, tau)
    freqs = np.array([8.5e9, 10e9, 11.5e9])
    S, st = gpu.sparams_eigenmode_batched([em.BatchInstance(M, p, bc, ports)], freqs)
    assert st["n_converged"] == st["n_total"]
    for k, f in enumerate(freqs):
        p.omega = 2 * math.pi * f
        Sp = gpu.calculate_sparams_eigenmode(M, p, bc, ports, tight)
        assert np.abs(S[0, k] - Sp).max() <= 1e-6
    m2, M2, bc2, ports2, p2 = _lumped_box(gpu, debye=(4.488, 4.312, 1.0 / (2 * math.pi * 3e9)))
    fr = [2.5e9, 3.0e9, 3.5e9]
    sw, st2 = gpu.frequency_sweep_batched(M2, p2, bc2, ports2, fr)
    assert st2["n_converged"] == st2["n_total"]
    for k, f in enumerate(fr):
        p2.omega = 2 * math.pi * f
        Sp = gpu.calculate_sparams(M2, p2, bc2, ports2, tight)
        assert np.abs(sw.S_matrices[k] - Sp).max() <= 1e-6


FR4_DEBYE = (4.488, 4.312, 1.0 / (2 * math.pi * 2.5e9))  # eps_s, eps_inf, tau: 4.4(1 - 0.02j) at 2.5 GHz


def patch_problem(gpu, h_fine=3e-3, h_coarse=10e-3, f_norm=2.5e9):
    """Probe-fed patch on Debye FR-4 with an absorbing box and a 50-ohm lumped
    port normalised once at f_norm (the patch-antenna workload at a coarse
    resolution)."""
    from edgefem_gb300.mesh import patch_antenna_mesh
    m = patch_antenna_mesh(h_fine=h_fine, h_coarse=h_coarse)
    M = em.Mesh.from_arrays(m)
    bc = em.build_edge_pec(M, 1)
    bc.dirichlet_edges |= em.build_edge_pec(M, 10).dirichlet_edges
    ports = [gpu.build_lumped_port(M, 20, 50.0, (0.0, 0.0, 1.0))]
    p = em.MaxwellParams()
    p.set_debye_region(101, *FR4_DEBYE)
    p.use_abc = True
    p.abc_surface_tags = {50}
    p.omega = 2 * math.pi * f_norm
    ports = gpu.normalize_port_weights(M, p, bc, ports,
                                       em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=400000))
    return m, M, bc, ports, p


def test_patch_antenna_sweep_matches_plain_and_oracle(gpu):
    """Batched driven sweep of the coarse patch against the plain per-frequency
    solve and the oracle's direct solve (fixture from
    tests/golden/make_patch_golden.py: same mesh, Debye FR-4, ABC, port)."""
    with open(os.path.join(GOLDEN, "patch_antenna_S.json")) as fh:
        gold = json.load(fh)
    m, M, bc, ports, p = patch_problem(gpu, f_norm=gold["f_norm"], **gold["mesh"])
    freqs = gold["freqs"]
    sw, st = gpu.frequency_sweep_batched(M, p, bc, ports, freqs)
    assert st["n_converged"] == st["n_total"] == len(freqs)
    opts = em.SolveOptions(use_bicgstab=False, tolerance=1e-10, max_iterations=400000)
    for k, f in enumerate(freqs):
        assert np.abs(sw.S_matrices[k][0, 0] - complex(*gold["S11"][k])) <= 1e-6
        p.omega = 2 * math.pi * f
        Sp = gpu.calculate_sparams(M, p, bc, ports, opts)
        assert np.abs(sw.S_matrices[k] - Sp).max() <= 1e-6


@pytest.mark.parametrize("precision", [2, 1, 0])
def test_batched_matches_oracle(gpu, precision):
    """Each Krylov arithmetic of the batched engine (2: double-float K and M,
    1: double-float K, 0: complex64) against the oracle's direct solve."""
    m = em.waveguide_mesh(8, 4, 20, slab=(20e-3, 30e-3))
    epsr = {101: 2.2 * (1 - 0.001j)}
    M, bc, ports, p = setup(m, eps_regions=epsr)
    freqs = np.linspace(8e9, 12e9, 6)
    S, st = gpu.sparams_eigenmode_batched([em.BatchInstance(M, p, bc, ports)], freqs,
                                          em.BatchOptions(precision=precision))
    assert st["n_converged"] == st["n_total"] == 12
    prob = O.make_problem(m)
    eps = O.tet_eps(prob, 0.0, eps_regions=epsr)
    for k, f in enumerate(freqs):
        Sr = O.calculate_sparams_eigenmode(prob, 2 * math.pi * f, O.waveguide_ports(prob, A, f), eps)
        assert np.abs(S[0, k] - Sr).max() <= 1e-6


def test_batched_uneven_instances(gpu):
    """Several meshes of different sizes and per-tet permittivity in one batch."""
    rng = np.random.default_rng(7)
    grids = [(6, 3, 12), (8, 4, 18), (7, 3, 15)]
    insts, refs = [], []
    freqs = np.array([9e9, 10.5e9])
    for g in grids:
        L = 0.03 + 0.01 * g[2] / 12
        m = em.waveguide_mesh(*g, A, 0.01016, L)
        eps = 1 + 3 * rng.uniform(size=m.num_tets) - 0.002j
        M, bc, ports, p = setup(m, eps_tet=eps)
        insts.append(em.BatchInstance(M, p, bc, ports))
        prob = O.make_problem(m)
        refs.append([O.calculate_sparams_eigenmode(prob, 2 * math.pi * f, O.waveguide_ports(prob, A, f), eps)
                     for f in freqs])
    S, st = gpu.sparams_eigenmode_batched(insts, freqs)
    assert st["n_converged"] == st["n_total"]
    for b in range(len(grids)):
        for k in range(freqs.size):
            assert np.abs(S[b, k] - refs[b][k]).max() <= 1e-6


def test_batched_resident_repeatable(gpu):
    m = em.waveguide_mesh(8, 4, 20)
    M, bc, ports, p = setup(m)
    bs = gpu.BatchSolver([em.BatchInstance(M, p, bc, ports)], [9e9, 10e9, 11e9])
    S1, st1 = bs.solve()
    S2, st2 = bs.solve()
    # FP64 atomics sum the dot products in run-dependent order, so repeated
    # solves agree to the solver tolerance, not bit for bit.
    assert st1["n_converged"] == st2["n_converged"] == st1["n_total"]
    assert np.abs(S1 - S2).max() <= 1e-7


def test_adjoint_matches_oracle_and_fd(gpu):
    m = em.waveguide_mesh(6, 3, 10)
    rng = np.random.default_rng(3)
    eps = 1.0 + rng.uniform(0, 1, m.num_tets) + 0j
    M, bc, ports, p = setup(m, 10e9, eps_tet=eps)
    g, S = gpu.sparams_eigenmode_adjoint(M, p, bc, ports, 1, 0, TIGHT)
    prob = O.make_problem(m)
    go, So = O.sparams_eigenmode_adjoint(prob, p.omega, O.waveguide_ports(prob, A, 10e9), eps, 1, 0)
    assert np.abs(S - So).max() <= 1e-8
    assert np.abs(g - go).max() <= 1e-8 * np.abs(go).max()
    h = 1e-4
    for t in rng.choice(m.num_tets, 5, replace=False).tolist() + [O.port_beta_tet(prob, 2)]:
        ep, en = eps.copy(), eps.copy()
        ep[t] += h
        en[t] -= h
        p.eps_r_tet = ep
        Sp = gpu.calculate_sparams_eigenmode(M, p, bc, ports, TIGHT)
        p.eps_r_tet = en
        Sn = gpu.calculate_sparams_eigenmode(M, p, bc, ports, TIGHT)
        fd = (abs(Sp[1, 0]) ** 2 - abs(Sn[1, 0]) ** 2) / (2 * h)
        # relative 1e-5 with an absolute floor of 1e-7 of the largest gradient
        # (the difference quotient's noise, solve error / h, is absolute)
        assert abs(g[t] - fd) <= 1e-5 * max(abs(fd), 1e-2 * np.abs(g).max())


def test_lossy_guide_attenuation(gpu):
    """The reference's lossy-dielectric validation
    (python/tests/test_validation_suite.py:221-268): WR-90, 50 mm, filled with
    eps_r = 2.2 (1 - 0.05j) at 10 GHz; |S21| within 35% of
    exp(-alpha_d L), alpha_d = k0^2 eps_r tan_d / (2 beta).  Checked on the
    plain path and on the batched engine (and the two agree to 1e-6)."""
    m = em.waveguide_mesh(10, 5, 22)  # about 10 cells per guide wavelength, as the reference meshes
    M, bc, ports, p = setup(m, 10e9)
    p.eps_r = complex(2.2, -2.2 * 0.05)
    k0 = 2 * math.pi * 10e9 / 299792458.0
    beta = math.sqrt(2.2 * k0 ** 2 - (math.pi / A) ** 2)
    s21_an = math.exp(-(k0 ** 2 * 2.2 * 0.05 / (2 * beta)) * 50e-3)
    S = gpu.calculate_sparams_eigenmode(M, p, bc, ports, TIGHT)
    Sb, st = gpu.sparams_eigenmode_batched([em.BatchInstance(M, p, bc, ports)], [10e9])
    assert st["n_converged"] == st["n_total"]
    assert np.abs(Sb[0, 0] - S).max() <= 1e-6
    s21 = abs(S[1, 0])
    assert 0.1 < s21 < 1.0
    assert abs(s21 - s21_an) / s21_an < 0.35


def test_failure_semantics(gpu):
    """Evanescent port -> NaN S (the reference returns an uninitialised
    matrix); non-convergence -> NaN column; below cutoff -> ValueError."""
    m = em.waveguide_mesh(6, 3, 10)
    M, bc, ports, p = setup(m, 10e9)
    p.omega = 2 * math.pi * 5e9
    S = gpu.calculate_sparams_eigenmode(M, p, bc, ports, TIGHT)
    assert np.all(np.isnan(S))
    p.omega = 2 * math.pi * 10e9
    S = gpu.calculate_sparams_eigenmode(M, p, bc, ports, em.SolveOptions(use_bicgstab=False, max_iterations=3))
    assert np.all(np.isnan(S))
    wg = gpu.RectWaveguideDesign(A, 0.01016, 0.05)
    with pytest.raises(RuntimeError):
        wg.sparams_at_freq(10e9)
    wg.set_mesh(m)
    with pytest.raises(ValueError):
        wg.sparams_at_freq(6e9)
    Sb, st = gpu.sparams_eigenmode_batched([em.BatchInstance(M, p, bc, ports)], [5e9, 10e9])
    assert np.all(np.isnan(Sb[0, 0])) and np.all(np.isfinite(Sb[0, 1]))


def test_spmv_bulk_kernel_matches_scipy(gpu):
    """The complex64 SpMV that streams the matrix through shared memory with
    bulk asynchronous copies (efgk_spmv32_bulk) against the exact product of
    the complex64-rounded operands, to 1e-5 of sum_j |A_ij x_j| per row: the
    assembled WR-90 operators (many tiles per CTA), a matrix whose entry
    count is not a multiple of 4 (tail read directly), one with a row longer
    than a stage (that tile read directly) and a single-row matrix;
    misaligned arrays are rejected before any launch."""
    import ctypes as C

    import scipy.sparse as sp
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch has no CUDA device")
    from edgefem_gb300 import _lib
    fn = _lib.lib.efgk_spmv32_bulk
    fn.restype = C.c_int
    fn.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 7
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(5)
    mats = []
    for g in ((8, 4, 20), (24, 12, 60)):
        M, bc, _, p = setup(em.waveguide_mesh(*g), 10e9, eps_regions={100: 2.2 * (1 - 0.01j)})
        rp, ci, v = gpu.assemble_maxwell(M, p, bc, [], -1).A.csr()
        mats.append(sp.csr_matrix((v, ci, rp)))
    R = sp.random(3001, 3001, density=0.003, format="csr", random_state=3, dtype=np.float64)
    R = R + sp.eye(3001)
    R.data = R.data * (1 + 0.5j)
    mats.append(R.tocsr())
    L = sp.lil_matrix((5000, 5000), dtype=np.complex128)
    L.setdiag(2.0 + 1j)
    L[10, rng.choice(5000, 4000, replace=False)] = rng.normal(size=4000) + 1j
    mats.append(L.tocsr())
    mats.append(sp.csr_matrix(np.array([[1.0 + 2j]])))
    for A in mats:
        A.sort_indices()
        n = A.shape[0]
        vv = A.data.astype(np.complex64)
        xx = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
        d_rp = torch.from_numpy(A.indptr.astype(np.int32)).to(dev)
        d_ci = torch.from_numpy(A.indices.astype(np.int32)).to(dev)
        d_v = torch.from_numpy(vv.view(np.float32)).to(dev)
        d_x = torch.from_numpy(xx.view(np.float32)).to(dev)
        d_y = torch.full((2 * n,), float("nan"), dtype=torch.float32, device=dev)
        d_st = torch.zeros(1, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        assert fn(n, A.nnz, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_x.data_ptr(), d_y.data_ptr(),
                  d_st.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert int(d_st.item()) == 0
        y = d_y.cpu().numpy().view(np.complex64).astype(np.complex128)
        Ar = sp.csr_matrix((vv.astype(np.complex128), A.indices, A.indptr), shape=(n, n))
        y_ref = Ar @ xx.astype(np.complex128)
        scale = abs(Ar) @ np.abs(xx.astype(np.complex128))
        assert np.all(np.abs(y - y_ref) <= 1e-5 * scale + 1e-30), (n, A.nnz)
    # a value array that does not start on a 16-byte boundary
    rc = fn(n, A.nnz, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr() + 8, d_x.data_ptr(), d_y.data_ptr(),
            d_st.data_ptr(), None)
    assert rc != 0


def test_spmv_kernels_match_scipy(gpu):
    """Plain CSR SpMVs through the kernel C-ABI on caller-owned device
    arrays: the complex128 product against scipy to FP64 rounding, the
    complex64 product (FP32 accumulation) against the exact product of the
    complex64-rounded operands to 1e-5 of sum_j |A_ij x_j| per row."""
    import ctypes as C

    import scipy.sparse as sp
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch has no CUDA device")
    from edgefem_gb300 import _lib
    M, bc, _, p = setup(em.waveguide_mesh(8, 4, 20), 10e9, eps_regions={100: 2.2 * (1 - 0.01j)})
    asm = gpu.assemble_maxwell(M, p, bc, [], -1)
    rp, ci, v = asm.A.csr()
    n = asm.A.n
    rng = np.random.default_rng(11)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    dev = torch.device("cuda:0")

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    d_rp, d_ci = d(rp.astype(np.int32)), d(ci.astype(np.int32))
    args = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    for name, cdt, rdt in (("efgk_spmv64", np.complex128, np.float64), ("efgk_spmv32", np.complex64, np.float32)):
        fn = getattr(_lib.lib, name)
        fn.restype, fn.argtypes = C.c_int, args
        vv, xx = v.astype(cdt), x.astype(cdt)
        d_v, d_x = d(vv.view(rdt)), d(xx.view(rdt))
        d_y = torch.full((2 * n,), float("nan"), dtype=d_v.dtype, device=dev)
        torch.cuda.synchronize()
        assert fn(n, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_x.data_ptr(), d_y.data_ptr(), None) == 0
        torch.cuda.synchronize()
        y = d_y.cpu().numpy().view(cdt).astype(np.complex128)
        Ar = sp.csr_matrix((vv.astype(np.complex128), ci, rp), shape=(n, n))
        y_ref = Ar @ xx.astype(np.complex128)
        scale = abs(Ar) @ np.abs(xx.astype(np.complex128))
        tol = 1e-14 if cdt is np.complex128 else 1e-5
        assert np.all(np.abs(y - y_ref) <= tol * scale + 1e-300), name
        if name == "efgk_spmv32":
            y32 = y
    # sliced-ELLPACK copy: same sums, same order per row as the CSR kernel's
    # terms, so within the same bound; every row written exactly once
    plan, fill, sell = _lib.lib.efgk_sell32_plan, _lib.lib.efgk_sell32_fill, _lib.lib.efgk_spmv32_sell
    plan.restype = fill.restype = sell.restype = C.c_int
    plan.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64), C.c_void_p]
    fill.argtypes = [C.c_int32] + [C.c_void_p] * 8
    sell.argtypes = [C.c_int32] + [C.c_void_p] * 7
    ns = (n + 31) // 32
    d_perm = torch.empty(n, dtype=torch.int32, device=dev)
    d_sp = torch.empty(ns + 1, dtype=torch.int64, device=dev)
    ent = C.c_int64()
    assert plan(n, d_rp.data_ptr(), d_perm.data_ptr(), d_sp.data_ptr(), C.byref(ent), None) == 0
    assert np.array_equal(np.sort(d_perm.cpu().numpy()), np.arange(n))
    lens = np.diff(rp)[d_perm.cpu().numpy()]
    sp_h = d_sp.cpu().numpy()
    assert sp_h[0] == 0 and sp_h[-1] == ent.value and ent.value >= rp[-1]
    for w in range(0, n, 1024):  # decreasing lengths inside every window
        assert np.all(np.diff(lens[w:w + 1024]) <= 0)
    d_sc = torch.empty(ent.value, dtype=torch.int32, device=dev)
    d_sv = torch.empty(2 * ent.value, dtype=torch.float32, device=dev)
    vv, xx = v.astype(np.complex64), x.astype(np.complex64)
    d_v, d_x = d(vv.view(np.float32)), d(xx.view(np.float32))
    d_y = torch.full((2 * n,), float("nan"), dtype=torch.float32, device=dev)
    assert fill(n, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_perm.data_ptr(), d_sp.data_ptr(),
                d_sc.data_ptr(), d_sv.data_ptr(), None) == 0
    assert sell(n, d_perm.data_ptr(), d_sp.data_ptr(), d_sc.data_ptr(), d_sv.data_ptr(), d_x.data_ptr(),
                d_y.data_ptr(), None) == 0
    torch.cuda.synchronize()
    y = d_y.cpu().numpy().view(np.complex64).astype(np.complex128)
    assert np.all(np.isfinite(y))
    assert np.all(np.abs(y - y_ref) <= 1e-5 * scale + 1e-300)
    assert np.abs(y - y32).max() <= 1e-5 * scale.max()


def _shuffled(m, seed):
    """The same mesh with its node order permuted and random, non-contiguous
    node ids, so that index order and id order disagree."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(m.node_ids))
    new_ids = rng.choice(10 ** 9, size=len(m.node_ids), replace=False).astype(np.int64) + 5
    remap = dict(zip(np.asarray(m.node_ids).tolist(), new_ids.tolist()))
    f = np.vectorize(remap.get, otypes=[np.int64])
    from edgefem_gb300.mesh import TetMesh
    return TetMesh(new_ids[perm], np.asarray(m.xyz)[perm], f(m.tets), m.tet_phys,
                   f(m.tris) if len(m.tris) else m.tris, m.tri_phys)


@pytest.mark.parametrize("which", ["wr90", "cube", "grid_shuffled", "slab_40x20x100", "no_tris"])
def test_gpu_edge_numbering_matches_host(gpu, wr90_mesh, cube_mesh, which):
    """build_edges on the GPU (bucketing by smaller node, per-bucket sort,
    scan of first occurrences) against the host numbering, which is
    bit-exact with the oracle: edge list, element edge ids and orientations
    identical."""
    from edgefem_gb300.mesh import TetMesh
    m = {"wr90": lambda: wr90_mesh, "cube": lambda: cube_mesh,
         "grid_shuffled": lambda: _shuffled(em.waveguide_mesh(8, 4, 20), 3),
         "slab_40x20x100": lambda: em.waveguide_mesh(40, 20, 100),
         "no_tris": lambda: TetMesh(cube_mesh.node_ids, cube_mesh.xyz, cube_mesh.tets, cube_mesh.tet_phys,
                                    np.zeros((0, 3), np.int64), np.zeros(0, np.int32))}[which]()
    host = em.Mesh.from_arrays(m).topology()
    timing = {}
    dev = gpu.build_edges_gpu(m, timing)
    for h, d, name in zip(host, dev, ("edges", "tet_edges", "tet_orient", "tri_edges", "tri_orient")):
        assert h.shape == d.shape and np.array_equal(h, d), name
    assert timing["device_ms"] > 0


def test_gpu_validate_mesh_matches_host_and_oracle(gpu, wr90_mesh, cube_mesh):
    """validate_mesh on the GPU: the report equal to the host's to the last
    bit, bad tetrahedra as the oracle flags them (one inverted, one
    degenerate with a zero-length edge and an infinite aspect ratio)."""
    from test_host_abi import _quality_meshes
    for name, m in list(_quality_meshes(wr90_mesh, cube_mesh).items()) + [("slab", em.waveguide_mesh(40, 20, 100))]:
        M = em.Mesh.from_arrays(m)
        host = em.validate_mesh(M)
        timing = {}
        dev = gpu.validate_mesh_gpu(M, timing)
        assert (dev.num_degenerate_tets, dev.num_inverted_tets) == (host.num_degenerate_tets, host.num_inverted_tets)
        assert dev.min_volume == host.min_volume and dev.max_aspect_ratio == host.max_aspect_ratio, name
        flags = O.validate_mesh(m.node_ids, m.xyz, m.tets)[0]
        assert dev.bad_tet_indices.tolist() == np.flatnonzero(flags).tolist(), name
        assert timing["device_ms"] > 0


@pytest.mark.parametrize("debye", [False, True])
def test_driven_adjoint_matches_oracle(gpu, debye):
    """d|S_ji|^2/d eps_r per tet for driven lumped ports with the jk0 ABC
    (the patch configuration's formulation): GPU (forward solves only, the
    adjoint vector a scaled forward solution) against the oracle's adjoint
    solved with A^T, itself checked against central differences; per-tet
    lossy permittivity, or a Debye medium everywhere."""
    from test_oracle_golden import _driven_box
    m, prob, omega, eps, oports = _driven_box()
    M = em.Mesh.from_arrays(m)
    p = em.MaxwellParams()
    p.omega = omega
    p.use_abc = True
    p.abc_surface_tags = {1}
    if debye:
        tau = 1.0 / (2 * math.pi * 2.5e9)
        p.set_debye_region(100, 4.488, 4.312, tau)
        eps = np.full(m.num_tets, O.debye_eps(4.488, 4.312, tau)(omega))
    else:
        p.eps_r_tet = eps
    gports = []
    for t, op in zip((2, 3), oports):
        g = gpu.build_lumped_port(M, t, 50.0, (1.0, 0.0, 0.0))
        assert np.array_equal(np.asarray(g.edges), np.asarray(op.edges))
        gports.append(em.WavePort(g.surface_tag, g.mode, np.asarray(g.edges, np.int32),
                                  np.asarray(op.weights, np.complex128)))
    opts = em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=200000)
    for j, i in ((0, 0), (1, 0)):
        g, S = gpu.sparams_driven_adjoint(M, p, em.BC(), gports, j, i, opts)
        go, So = O.sparams_driven_adjoint(prob, omega, eps, oports, j, i, use_abc=True, abc_tags=(1,))
        assert abs(S[j, i] - So) <= 1e-8
        assert np.abs(g - go).max() <= 1e-7 * np.abs(go).max(), (j, i)
