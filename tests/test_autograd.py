"""torch.autograd front end of the adjoint sensitivity: the gradient that
backward() delivers equals the library's adjoint and central finite
differences of the forward solve (h = 1e-4, the reference-scale check of
the adjoint workload), on a smooth permittivity field."""
import math

import numpy as np
import pytest

import edgefem_gb300 as em

torch = pytest.importorskip("torch")
from edgefem_gb300.autograd import sparam_power  # noqa: E402

A, B = 22.86e-3, 10.16e-3


def smooth_eps(m, seed=11, n_blobs=8, sigma=4e-3):
    """eps_r(x) = clip(1 + sum_k a_k exp(-|x - c_k|^2 / (2 sigma^2)), 1, 6)
    at tetrahedron centroids, seeded."""
    rng = np.random.default_rng(seed)
    lo, hi = m.xyz.min(axis=0), m.xyz.max(axis=0)
    idx = {int(i): k for k, i in enumerate(m.node_ids)}
    cent = np.array([[m.xyz[idx[int(v)]] for v in t] for t in m.tets]).mean(axis=1)
    eps = np.ones(len(cent))
    for _ in range(n_blobs):
        c = lo + rng.uniform(size=3) * (hi - lo)
        eps += rng.uniform(0, 5) * np.exp(-((cent - c) ** 2).sum(axis=1) / (2 * sigma ** 2))
    return np.clip(eps, 1.0, 6.0)


def problem(m, freq):
    M = em.Mesh.from_arrays(m)
    bc = em.build_edge_pec(M, 1)
    mode = em.solve_te10_mode(em.RectWaveguidePort(A, B), freq)
    ports = [em.build_wave_port_2d(M, t, mode, bc.dirichlet_edges, (math.pi / A) ** 2) for t in (2, 3)]
    p = em.MaxwellParams()
    p.omega = 2 * math.pi * freq
    return M, bc, ports, p


def test_autograd_rejects_wrong_size():
    m = em.waveguide_mesh(4, 2, 6)
    M, bc, ports, p = problem(m, 10e9)
    with pytest.raises(ValueError):
        sparam_power(torch.ones(m.num_tets + 1, dtype=torch.float64), M, p, bc, ports)


@pytest.mark.gpu
def test_autograd_gradient_matches_adjoint_and_fd(gpu):
    m = em.waveguide_mesh(12, 6, 24)
    M, bc, ports, p = problem(m, 10e9)
    eps0 = smooth_eps(m)
    tight = em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=200000)
    x = torch.tensor(eps0, dtype=torch.float64, requires_grad=True)
    y = sparam_power(x, M, p, bc, ports, 1, 0, opts=tight)
    y.backward()
    # Same quantity straight from the library.
    p.eps_r_tet = eps0.astype(np.complex128)
    g_lib, S = gpu.sparams_eigenmode_adjoint(M, p, bc, ports, 1, 0, tight)
    assert abs(y.item() - abs(S[1, 0]) ** 2) <= 1e-12
    assert np.abs(x.grad.numpy() - g_lib).max() <= 1e-9 * np.abs(g_lib).max()
    # Central differences of the forward solve at seeded tetrahedra.
    h = 1e-4
    rng = np.random.default_rng(5)
    for t in rng.choice(m.num_tets, 6, replace=False).tolist():
        ep, en = eps0.copy(), eps0.copy()
        ep[t] += h
        en[t] -= h
        yp = float(sparam_power(torch.tensor(ep), M, p, bc, ports, 1, 0, opts=tight))
        yn = float(sparam_power(torch.tensor(en), M, p, bc, ports, 1, 0, opts=tight))
        fd = (yp - yn) / (2 * h)
        # relative 1e-5, with an absolute floor of 1e-7 of the largest
        # gradient: the difference quotient's noise (solve error / h, about
        # 1e-8 here) does not shrink with the entry
        assert abs(x.grad[t].item() - fd) <= 1e-5 * max(abs(fd), 1e-2 * np.abs(g_lib).max()), t


@pytest.mark.gpu
def test_autograd_driven_gradient_matches_oracle(gpu):
    """driven=True: |S21|^2 of two lumped ports with the ABC as a function of
    the real permittivity per tet (fixed loss), its torch gradient against
    the oracle's driven adjoint (itself checked by central differences)."""
    import math
    import edgefem_oracle as O
    from test_oracle_golden import _driven_box
    m, prob, omega, eps, oports = _driven_box()
    M = em.Mesh.from_arrays(m)
    p = em.MaxwellParams()
    p.omega = omega
    p.use_abc = True
    p.abc_surface_tags = {1}
    gports = [em.WavePort(g.surface_tag, g.mode, np.asarray(g.edges, np.int32), np.asarray(o.weights, np.complex128))
              for g, o in zip([gpu.build_lumped_port(M, t, 50.0, (1.0, 0.0, 0.0)) for t in (2, 3)], oports)]
    tight = em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=200000)
    x = torch.tensor(eps.real, dtype=torch.float64, requires_grad=True)
    y = sparam_power(x, M, p, bc=em.BC(), ports=gports, out_j=1, in_i=0, eps_imag=eps.imag, opts=tight, driven=True)
    y.backward()
    go, So = O.sparams_driven_adjoint(prob, omega, eps, oports, 1, 0, use_abc=True, abc_tags=(1,))
    assert abs(y.item() - abs(So) ** 2) <= 1e-9
    assert np.abs(x.grad.numpy() - go).max() <= 1e-7 * np.abs(go).max()
    assert math.isfinite(y.item())
