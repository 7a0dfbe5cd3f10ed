"""The oracle's C iterative solver (oracle/krylov_c.c) and its K/M sweep form
against the oracle's direct solve (no GPU).  These pin the solver that checks
the GPU results at sizes a direct factorisation cannot reach."""
import math

import numpy as np
import pytest
import scipy.sparse.linalg as spla

import edgefem_oracle as O
from conftest import published
from edgefem_gb300.mesh import waveguide_mesh

A_WR90 = 0.02286


@pytest.fixture(scope="module")
def slab_system():
    m = waveguide_mesh(10, 5, 24, A_WR90, 10.16e-3, 50e-3, slab=(20e-3, 30e-3))
    prob = O.make_problem(m)
    f = 11e9
    w = 2 * math.pi * f
    ports = O.waveguide_ports(prob, A_WR90, f)
    eps = O.tet_eps(prob, w, eps_regions={101: 2.2 * (1 - 0.001j)})
    return prob, ports, eps, w


@pytest.mark.parametrize("level", [0, 1, 2])
def test_c_cocg_matches_direct_solve(slab_system, level):
    """Jacobi, + gradient space, + vector-nodal space: the C COCG reaches the
    SuperLU solution to the tolerance's order and follows the NumPy COCG's
    iteration count."""
    prob, ports, eps, w = slab_system
    sys_ = O.eigenmode_system(prob, w, ports, eps)
    A = sys_.A.tocsr()
    b = sys_.B[:, 0]
    x_lu = spla.splu(A.tocsc()).solve(b)
    r = O.cocg_aux_c(prob, A, b, tol=1e-12, level=level, threads=2, tol1=1e-8)
    assert r["converged"] and r["relres"] < 1e-12
    assert np.abs(r["x"] - x_lu).max() <= 1e-9 * np.abs(x_lu).max()
    assert 0 < r["iterations_tol1"] <= r["iterations"]
    prec = None if level == 0 else O.aux_preconditioner(prob, A, vector=level > 1)
    _, it_py, _, _ = O.cocg_jacobi(A, b, tol=1e-12, prec=prec)
    assert abs(r["iterations"] - it_py) <= max(5, 0.05 * it_py)


def test_c_cocg_thread_counts_agree(slab_system):
    prob, ports, eps, w = slab_system
    sys_ = O.eigenmode_system(prob, w, ports, eps)
    r1 = O.cocg_aux_c(prob, sys_.A, sys_.B[:, 1], tol=1e-10, threads=1)
    r3 = O.cocg_aux_c(prob, sys_.A, sys_.B[:, 1], tol=1e-10, threads=3)
    assert np.abs(r1["x"] - r3["x"]).max() <= 1e-8 * np.abs(r1["x"]).max()


def test_eigenmode_sweep_matches_eigenmode_system(slab_system):
    """A(f) from one K/M assembly plus the per-frequency port terms equals
    the per-frequency assembly, and gives the same S."""
    prob, ports, eps, _ = slab_system
    sw = O.EigenmodeSweep(prob, ports, eps)
    for f in (8.2e9, 12e9):
        w = 2 * math.pi * f
        s1 = O.eigenmode_system(prob, w, ports, eps)
        s2 = sw.system(w)
        assert np.array_equal(s1.A.indices, s2.A.indices) and np.array_equal(s1.A.indptr, s2.A.indptr)
        assert np.abs((s1.A - s2.A).data).max() <= 1e-13 * np.abs(s1.A.data).max()
        assert np.abs(s1.B - s2.B).max() <= 1e-13 * np.abs(s1.B).max()
        X1 = spla.splu(s1.A.tocsc()).solve(s1.B)
        X2 = np.column_stack([O.cocg_aux_c(prob, s2.A, s2.B[:, k], tol=1e-12, threads=2)["x"] for k in range(2)])
        assert np.abs(O.sparams_from_solution(s1, X1) - O.sparams_from_solution(s2, X2)).max() < 1e-9


def test_c_cocg_reproduces_published_table(wr90_mesh):
    """The C solver on the reference's rect_waveguide.msh reproduces the
    published 10 GHz row of docs/validation.md:20-29 (the direct solve's pin
    carried over to the iterative solver)."""
    prob = O.make_problem(wr90_mesh)
    row = next(r for r in published()["wr90_7_12ghz"] if r["freq_ghz"] == 10)
    f = 10e9
    sw = O.EigenmodeSweep(prob, O.waveguide_ports(prob, A_WR90, f), np.ones(wr90_mesh.num_tets, complex))
    sys_ = sw.system(2 * math.pi * f)
    X = np.column_stack([O.cocg_aux_c(prob, sys_.A, sys_.B[:, k], tol=1e-12, threads=2)["x"] for k in range(2)])
    S = O.sparams_from_solution(sys_, X)
    assert round(abs(S[0, 0]), 3) == pytest.approx(row["s11_mag"], abs=1e-9)
    assert round(abs(S[1, 0]), 4) == pytest.approx(row["s21_mag"], abs=1e-9)
    assert round(math.degrees(np.angle(S[1, 0])), 1) == pytest.approx(row["s21_phase_deg"], abs=1e-9)


def test_c_matvec(slab_system):
    prob, ports, eps, w = slab_system
    A = O.eigenmode_system(prob, w, ports, eps).A
    x = np.random.default_rng(1).normal(size=A.shape[0]) * (1 + 0.5j)
    assert np.abs(O.csr_matvec_c(A, x, 2) - A @ x).max() <= 1e-12 * np.abs(A @ x).max()


def test_iterative_adjoints_match_direct():
    """The oracle's adjoints with their solves done by the C COCG (the form
    the benchmark uses at sizes SuperLU cannot take) equal the direct-solve
    adjoints: driven lumped ports with the jk0 ABC, and eigenmode ports."""
    from edgefem_gb300.mesh import box_tet_mesh
    m = box_tet_mesh(6, 6, 6, 0.02, 0.02, 0.02)
    prob = O.make_problem(m)
    prob.pec = np.zeros(0, np.int64)
    ports = [O.build_lumped_port(prob, 2, (1.0, 0.0, 0.0), 50.0), O.build_lumped_port(prob, 3, (1.0, 0.0, 0.0), 50.0)]
    w = 2 * math.pi * 3e9
    eps = np.full(m.num_tets, 2.0 - 0.1j)
    g1, S1 = O.sparams_driven_adjoint(prob, w, eps, ports, 1, 0, use_abc=True, abc_tags=(1,))
    g2, S2 = O.sparams_driven_adjoint(prob, w, eps, ports, 1, 0, use_abc=True, abc_tags=(1,), iterative_tol=1e-13,
                                      threads=2)
    assert abs(S1 - S2) < 1e-12 and np.abs(g1 - g2).max() <= 1e-10 * np.abs(g1).max()
    mw = waveguide_mesh(8, 4, 16, A_WR90, 10.16e-3, 40e-3)
    pw = O.make_problem(mw)
    f = 10e9
    ew = np.ones(mw.num_tets, complex) * 1.5
    gd, Sd = O.sparams_eigenmode_adjoint(pw, 2 * math.pi * f, O.waveguide_ports(pw, A_WR90, f), ew, 1, 0)
    gi, Si = O.sparams_eigenmode_adjoint(pw, 2 * math.pi * f, O.waveguide_ports(pw, A_WR90, f), ew, 1, 0,
                                         iterative_tol=1e-13)
    assert np.abs(Sd - Si).max() < 1e-10 and np.abs(gd - gi).max() <= 1e-8 * np.abs(gd).max()
