"""The complex128 oracle against the reference's published numbers and
known-answer tests (no GPU).  These pin the oracle before it is trusted as
the parity reference for the GPU path."""
import math

import numpy as np
import pytest

import edgefem_oracle as O
from conftest import published

A_WR90 = 0.02286
L_WR90 = 0.05


@pytest.fixture(scope="module")
def wr90_prob(wr90_mesh):
    return O.make_problem(wr90_mesh)


def test_wr90_published_table(wr90_prob, wr90_mesh):
    """docs/validation.md:20-29: |S11|, |S21|, phase(S21) on
    examples/rect_waveguide.msh at 7-12 GHz, to the printed digits."""
    eps = np.ones(wr90_mesh.num_tets, complex)
    for row in published()["wr90_7_12ghz"]:
        f = row["freq_ghz"] * 1e9
        S = O.calculate_sparams_eigenmode(wr90_prob, 2 * math.pi * f, O.waveguide_ports(wr90_prob, A_WR90, f), eps)
        assert round(abs(S[0, 0]), 3) == pytest.approx(row["s11_mag"], abs=1e-9)
        assert round(abs(S[1, 0]), 4) == pytest.approx(row["s21_mag"], abs=1e-9)
        assert round(math.degrees(np.angle(S[1, 0])), 1) == pytest.approx(row["s21_phase_deg"], abs=1e-9)
        # reciprocity and symmetry of the two-port
        assert abs(S[0, 1] - S[1, 0]) < 1e-9
        # pass criteria of tests/benchmark_wr90.cpp:91-92
        k0 = 2 * math.pi * f / O.C0
        beta = math.sqrt(k0 * k0 - (math.pi / A_WR90) ** 2)
        expected = (math.degrees(-beta * L_WR90) + 180) % 360 - 180
        err = abs(math.degrees(np.angle(S[1, 0])) - expected)
        err = min(err, 360 - err)
        assert abs(S[0, 0]) < 0.15 and abs(S[1, 0]) > 0.90 and err < 15
        assert abs(S[0, 0]) ** 2 + abs(S[1, 0]) ** 2 <= 1.05


def test_wr90_port_abc_scale_table(wr90_prob, wr90_mesh):
    """docs/validation.md:50-56: |S11|, |S21| versus port_abc_scale at 10 GHz.
    Nine of the ten printed values are reproduced to the printed digit; |S21|
    at alpha = 1.5 comes out 0.92146 against the printed 0.922, one unit in
    the last place, so the check allows one unit."""
    f = 10e9
    eps = np.ones(wr90_mesh.num_tets, complex)
    ports = O.waveguide_ports(wr90_prob, A_WR90, f)
    exact = 0
    for row in published()["port_abc_scale_10ghz"]:
        S = O.calculate_sparams_eigenmode(wr90_prob, 2 * math.pi * f, ports, eps, port_abc_scale=row["alpha"])
        for got, want in ((abs(S[0, 0]), row["s11_mag"]), (abs(S[1, 0]), row["s21_mag"])):
            assert abs(round(got, 3) - want) <= 1e-3 + 1e-12
            exact += abs(round(got, 3) - want) < 1e-12
    assert exact >= 9


def test_triangle_mass_quadrature():
    """tests/test_triangle_mass_matrix.cpp:66-105: closed form equals a 7-point
    degree-5 quadrature of N_e . N_f to 1e-12, symmetric, positive definite."""
    w0 = 9.0 / 40.0
    a1, b1, w1 = 0.059715871789770, 0.470142064105115, 0.132394152788506
    a2, b2, w2 = 0.797426985353087, 0.101286507323456, 0.125939180544827
    pts = [(1 / 3, 1 / 3, 1 / 3, w0), (a1, b1, b1, w1), (b1, a1, b1, w1), (b1, b1, a1, w1),
           (a2, b2, b2, w2), (b2, a2, b2, w2), (b2, b2, a2, w2)]
    for tri in published()["triangle_mass_triangles"]:
        v = np.array(tri, float)
        M = O.triangle_whitney_mass(v[None])[0]
        nrm = np.cross(v[1] - v[0], v[2] - v[0])
        a2x = np.linalg.norm(nrm)
        nh = nrm / a2x
        g = [np.cross(nh, v[2] - v[1]) / a2x, np.cross(nh, v[0] - v[2]) / a2x, np.cross(nh, v[1] - v[0]) / a2x]
        Mq = np.zeros((3, 3))
        for l0, l1, l2, w in pts:
            lam = (l0, l1, l2)
            N = [lam[a] * g[b] - lam[b] * g[a] for a, b in O.TRI_PAIRS]
            for i in range(3):
                for j in range(3):
                    Mq[i, j] += w * (a2x / 2) * N[i] @ N[j]
        assert np.linalg.norm(M - Mq) / np.linalg.norm(Mq) < 1e-12
        assert np.linalg.norm(M - M.T) < 1e-14 * np.linalg.norm(M)
        assert np.linalg.eigvalsh(M).min() > 0


def test_edge_indexing_invariants(cube_mesh):
    """tests/test_edge_indexing.cpp:6-34 on examples/cube_cavity.msh."""
    t = O.build_edges(cube_mesh.tets, cube_mesh.tris)
    assert t.n > 0
    assert np.all(t.edges[:, 0] < t.edges[:, 1])
    for k, (p, q) in enumerate(O.TET_PAIRS):
        a, b = cube_mesh.tets[:, p], cube_mesh.tets[:, q]
        e = t.edges[t.tet_edges[:, k]]
        assert np.array_equal(e[:, 0], np.minimum(a, b)) and np.array_equal(e[:, 1], np.maximum(a, b))
        assert np.array_equal(t.tet_signs[:, k], np.where(a < b, 1, -1))


def test_maxwell_hermitian_and_lossy(cube_mesh):
    """tests/test_maxwell.cpp:8-17 (lossless, omega = 1: A Hermitian) and
    :94-105 (eps_r = 1 - 0.1j: not Hermitian).  At omega = 1 rad/s the loss
    term k0^2 Im(eps) M is ~1e-19 of |A|, below the reference's 1e-9 isApprox
    threshold, so that assertion holds only with assertions compiled out; the
    lossy case is checked here at 1 GHz, where the loss is visible."""
    prob = O.make_problem(cube_mesh)
    A, _ = O.assemble_maxwell(prob, 1.0, np.ones(cube_mesh.num_tets, complex))
    D = A.toarray()
    assert np.allclose(D, D.conj().T, rtol=1e-9, atol=1e-9 * abs(D).max())
    w = 2 * math.pi * 1e9
    A1, _ = O.assemble_maxwell(prob, w, np.ones(cube_mesh.num_tets, complex))
    D1 = A1.toarray()
    assert np.allclose(D1, D1.conj().T, rtol=1e-9, atol=1e-9 * abs(D1).max())
    A2, _ = O.assemble_maxwell(prob, w, np.full(cube_mesh.num_tets, 1 - 0.1j))
    D2 = A2.toarray()
    assert not np.allclose(D2, D2.conj().T, rtol=1e-9, atol=1e-9 * abs(D2).max())
    assert np.allclose(D2, D2.T, rtol=1e-12, atol=1e-12 * abs(D2).max())  # complex symmetric


def test_wave_port_source(cube_mesh):
    """tests/test_maxwell.cpp:19-52: b = 2/sqrt(Z0) at the excited port edge."""
    prob = O.make_problem(cube_mesh)
    e1 = 10 if 10 not in set(prob.pec.tolist()) else int(np.setdiff1d(np.arange(prob.n), prob.pec)[0])
    p1 = O.WavePort(0, np.array([e1]), np.ones(1, complex), Z0=50.0)
    p2 = O.WavePort(0, np.array([20]), np.ones(1, complex), Z0=50.0)
    _, b = O.assemble_maxwell(prob, 1.0, np.ones(cube_mesh.num_tets, complex), [p1, p2], 0)
    assert abs(b[e1] - 2 / math.sqrt(50.0)) < 1e-9


def test_debye_kat():
    """include/edgefem/materials/dispersive.hpp:62-66: eps(0) = eps_s,
    eps(inf) -> eps_inf, eps(1/tau) = (eps_s + eps_inf)/2 - j(eps_s - eps_inf)/2."""
    es, ei, tau = 80.1, 4.9, 9.3e-12
    f = O.debye_eps(es, ei, tau)
    assert abs(f(0.0) - es) < 1e-12
    assert abs(f(1e20) - ei) < 1e-6
    v = f(1 / tau)
    assert abs(v - complex((es + ei) / 2, -(es - ei) / 2)) < 1e-12


def test_adjoint_oracle_fd():
    """The oracle's complex128 adjoint against central differences."""
    from edgefem_gb300.mesh import waveguide_mesh
    m = waveguide_mesh(6, 3, 10)
    prob = O.make_problem(m)
    f = 10e9
    ports = O.waveguide_ports(prob, A_WR90, f)
    rng = np.random.default_rng(3)
    eps = 1.0 + rng.uniform(0, 1, m.num_tets) + 0j
    g, _ = O.sparams_eigenmode_adjoint(prob, 2 * math.pi * f, ports, eps, 1, 0)
    h = 1e-4
    for t in rng.choice(m.num_tets, 4, replace=False).tolist() + [O.port_beta_tet(prob, 2)]:
        ep, em_ = eps.copy(), eps.copy()
        ep[t] += h
        em_[t] -= h
        Sp = O.calculate_sparams_eigenmode(prob, 2 * math.pi * f, ports, ep)
        Sm = O.calculate_sparams_eigenmode(prob, 2 * math.pi * f, ports, em_)
        fd = (abs(Sp[1, 0]) ** 2 - abs(Sm[1, 0]) ** 2) / (2 * h)
        assert abs(g[t] - fd) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(g).max())


def test_adjoint_oracle_iterative_matches_direct():
    """The oracle adjoint with its complex128 COCG solves (used where a direct
    factorisation is too slow) equals the SuperLU one."""
    from edgefem_gb300.mesh import waveguide_mesh
    m = waveguide_mesh(6, 3, 10)
    prob = O.make_problem(m)
    f = 10e9
    ports = O.waveguide_ports(prob, A_WR90, f)
    eps = 1.0 + np.random.default_rng(9).uniform(0, 3, m.num_tets) + 0j
    g, S = O.sparams_eigenmode_adjoint(prob, 2 * math.pi * f, ports, eps, 1, 0)
    gi, Si = O.sparams_eigenmode_adjoint(prob, 2 * math.pi * f, ports, eps, 1, 0, iterative_tol=1e-13)
    assert np.abs(Si - S).max() <= 1e-9
    assert np.abs(gi - g).max() <= 1e-8 * np.abs(g).max()


def _driven_box(seed=1):
    """Two 50-ohm lumped ports on opposite faces of a 20 mm box, jk0 ABC on
    the other walls, heterogeneous lossy permittivity, 3 GHz."""
    from edgefem_gb300.mesh import box_tet_mesh
    m = box_tet_mesh(6, 6, 6, 0.02, 0.02, 0.02)
    prob = O.make_problem(m)
    prob.pec = np.zeros(0, np.int64)
    omega = 2 * math.pi * 3e9
    eps = (1.5 + np.random.default_rng(seed).uniform(0, 2, m.num_tets)) * (1 - 0.02j)
    ports = [O.build_lumped_port(prob, t, (1.0, 0.0, 0.0), 50.0) for t in (2, 3)]
    ports = O.normalize_port_weights(prob, omega, eps, ports, use_abc=True, abc_tags=(1,))
    return m, prob, omega, eps, ports


def test_driven_adjoint_oracle_fd():
    """The oracle's driven-port adjoint (adjoint system solved with A^T as
    it stands) against central differences (h = 1e-4) of |S11|^2 and
    |S21|^2 with lumped ports, the ABC and lossy per-tet permittivity."""
    m, prob, omega, eps, ports = _driven_box()
    rng = np.random.default_rng(4)
    h = 1e-4
    for j, i in ((0, 0), (1, 0)):
        g, _ = O.sparams_driven_adjoint(prob, omega, eps, ports, j, i, use_abc=True, abc_tags=(1,))
        for t in rng.choice(m.num_tets, 3, replace=False).tolist():
            ep, em_ = eps.copy(), eps.copy()
            ep[t] += h
            em_[t] -= h
            fp = abs(O.calculate_sparams(prob, omega, ep, ports, True, (1,))[j, i]) ** 2
            fm = abs(O.calculate_sparams(prob, omega, em_, ports, True, (1,))[j, i]) ** 2
            fd = (fp - fm) / (2 * h)
            assert abs(g[t] - fd) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(g).max()), (j, i, t)


def test_validate_mesh_known_answers(cube_mesh):
    """The known answers of the reference's tests/test_mesh_quality.cpp:
    regular tet volume 1/(6 sqrt 2), the mirrored tet inverted, a coplanar
    tet degenerate (|vol| < 1e-15), cube_cavity.msh valid with max aspect
    ratio in (0, 100), the unit right tet's aspect ratio sqrt 2; for the
    oracle restatement and for the library's validate_mesh."""
    import edgefem_gb300 as em
    from edgefem_gb300.mesh import TetMesh

    def one(pts):
        return TetMesh(np.arange(4, dtype=np.int64), np.asarray(pts, np.float64), np.arange(4, dtype=np.int64)[None],
                       np.zeros(1, np.int32), np.zeros((0, 3), np.int64), np.zeros(0, np.int32))

    s3, s23 = math.sqrt(3.0), math.sqrt(2.0 / 3.0)
    regular = one([[0, 0, 0], [1, 0, 0], [0.5, s3 / 2, 0], [0.5, s3 / 6, s23]])
    mirrored = one([[0, 0, 0], [1, 0, 0], [0.5, s3 / 2, 0], [0.5, s3 / 6, -s23]])
    coplanar = one([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]])
    right = one([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
    cases = {"regular": regular, "mirrored": mirrored, "coplanar": coplanar, "right": right, "cube": cube_mesh}
    for name, m in cases.items():
        flags, nd, ni, vmin, amax = O.validate_mesh(m.node_ids, m.xyz, m.tets)
        q = em.validate_mesh(em.Mesh.from_arrays(m))
        assert (q.num_degenerate_tets, q.num_inverted_tets, q.min_volume, q.max_aspect_ratio) == (nd, ni, vmin, amax)
        if name == "regular":
            assert abs(vmin - 1.0 / (6.0 * math.sqrt(2.0))) < 1e-10 and (nd, ni) == (0, 0)
        elif name == "mirrored":
            assert vmin < 0 and (nd, ni) == (0, 1)
        elif name == "coplanar":
            assert abs(vmin) < 1e-15 and (nd, ni) == (1, 0)
        elif name == "right":
            assert abs(amax - math.sqrt(2.0)) < 1e-10
        else:
            assert (nd, ni) == (0, 0) and vmin > 0 and 0 < amax < 100


def test_abc_diagonal_rule(cube_mesh):
    """tests/test_abc.cpp's scenario (cube_cavity.msh, omega = 2, ABC on vs
    off) with the rule of the reference's source, assemble_maxwell.cpp:244-264:
    the ABC adds j k0 = j omega / c0 to the diagonal of every non-PEC edge of
    the absorbing surface and nothing else.  (test_abc.cpp asserts j omega,
    which its source contradicts; and with the cube's all-PEC boundary its
    scenario damps no edge.  The PEC set is left empty here so that the
    surface has edges to damp.)"""
    prob = O.make_problem(cube_mesh)
    pec_full = prob.pec.copy()
    prob.pec = np.zeros(0, np.int64)
    eps = np.ones(cube_mesh.num_tets, np.complex128)
    A0, _ = O.assemble_maxwell(prob, 2.0, eps)
    A1, _ = O.assemble_maxwell(prob, 2.0, eps, use_abc=True)
    D = (A1 - A0).tocoo()
    boundary = np.unique(prob.topo.tri_edges)
    assert D.nnz > 0 and np.array_equal(D.row, D.col)
    assert np.array_equal(np.sort(D.row), boundary)
    assert np.allclose(D.data, 2.0j / O.C0, rtol=1e-14, atol=0)
    # With the cube's PEC walls (every boundary edge), nothing is damped.
    prob.pec = pec_full
    B0, _ = O.assemble_maxwell(prob, 2.0, eps)
    B1, _ = O.assemble_maxwell(prob, 2.0, eps, use_abc=True)
    assert abs(B1 - B0).max() == 0


def test_wr90_eigenmode_pass_criteria(wr90_prob, wr90_mesh):
    """Pass criteria of tests/test_eigenmode_sparams.cpp on
    examples/rect_waveguide.msh at 10 GHz: |S11| < 0.1, |S21| > 0.95,
    |S11|^2 + |S21|^2 <= 1.01, phase(S21) within 10 degrees of -beta L,
    |S12 - S21| < 0.05."""
    f = 10e9
    eps = np.ones(wr90_mesh.num_tets, complex)
    S = O.calculate_sparams_eigenmode(wr90_prob, 2 * math.pi * f, O.waveguide_ports(wr90_prob, A_WR90, f), eps)
    k0 = 2 * math.pi * f / O.C0
    beta = math.sqrt(k0 * k0 - (math.pi / A_WR90) ** 2)
    expected = (math.degrees(-beta * L_WR90) + 180) % 360 - 180
    err = abs(math.degrees(np.angle(S[1, 0])) - expected)
    err = min(err, 360 - err)
    assert abs(S[0, 0]) < 0.1 and abs(S[1, 0]) > 0.95 and err < 10
    assert abs(S[0, 0]) ** 2 + abs(S[1, 0]) ** 2 <= 1.01
    assert abs(S[0, 1] - S[1, 0]) < 0.05
