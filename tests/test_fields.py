"""Field post-processing: E from an edge solution (evaluate_edge_field,
src/edge_basis.cpp:162-193) at points and tet centroids, and the VTK exports
(src/io/vtk_export.cpp).  The oracle is pinned by the Whitney space's known
answers (constant and rotational fields are reproduced exactly); the GPU
path is compared with the oracle."""
import math
import re

import numpy as np
import pytest

import edgefem_oracle as O

import edgefem_gb300 as em
from edgefem_gb300.mesh import box_tet_mesh, waveguide_mesh


def jittered_box():
    m = box_tet_mesh(4, 3, 5, 0.02, 0.015, 0.025)
    rng = np.random.default_rng(11)
    h = 0.02 / 4
    inner = np.all((m.xyz > 1e-9) & (m.xyz < np.array([0.02, 0.015, 0.025]) - 1e-9), axis=1)
    m.xyz[inner] += rng.uniform(-0.15 * h, 0.15 * h, size=(inner.sum(), 3))
    return m


def interpolant(prob, E0, b):
    """Edge DOFs of E(x) = E0 + b x x: the line integral along each global edge
    (exact at the midpoint, the field being linear)."""
    e = prob.topo.edges
    x0 = prob.xyz[prob.node_lut[e[:, 0]]]
    x1 = prob.xyz[prob.node_lut[e[:, 1]]]
    mid = 0.5 * (x0 + x1)
    return np.einsum("ek,ek->e", E0 + np.cross(b, mid), x1 - x0)


def random_points(prob, rng, n):
    tets = rng.integers(0, prob.tets.shape[0], n)
    lam = rng.dirichlet(np.ones(4), n)
    X = prob.xyz[prob.node_lut[prob.tets[tets]]]
    return tets, np.einsum("qk,qkd->qd", lam, X), lam


def test_oracle_reproduces_whitney_fields():
    """Known answer: constant and rotational fields lie in the lowest-order
    Nedelec space, so their interpolant evaluates back to the field."""
    m = jittered_box()
    prob = O.make_problem(m)
    rng = np.random.default_rng(5)
    E0 = rng.normal(size=3) + 1j * rng.normal(size=3)
    b = rng.normal(size=3) * 40
    x = interpolant(prob, E0.real, b) + 1j * interpolant(prob, E0.imag, np.zeros(3))
    tets, pts, lam = random_points(prob, rng, 200)
    E = O.edge_field(prob, x, tets, pts)
    want = E0 + np.cross(b, pts)
    assert np.abs(E - want).max() <= 1e-12 * np.abs(want).max()
    X = prob.xyz[prob.node_lut[prob.tets[tets]]]
    assert np.allclose(O.barycentric(X, pts), lam, rtol=0, atol=1e-12)


def test_barycentric_host_helper():
    rng = np.random.default_rng(2)
    V = rng.normal(size=(4, 3))
    lam = rng.dirichlet(np.ones(4))
    p = lam @ V
    assert np.allclose(em.compute_barycentric(V, p), lam, rtol=0, atol=1e-12)
    assert np.allclose(em.compute_barycentric(V, p), O.barycentric(V[None], p[None])[0], rtol=0, atol=1e-13)


@pytest.mark.gpu
def test_field_points_and_centroids_match_oracle(gpu):
    m = jittered_box()
    M = em.Mesh.from_arrays(m)
    prob = O.make_problem(m)
    rng = np.random.default_rng(8)
    x = rng.normal(size=prob.n) + 1j * rng.normal(size=prob.n)
    Ec = gpu.evaluate_field(M, x)
    Ro = O.edge_field(prob, x)
    assert Ec.shape == (m.num_tets, 3)
    assert np.abs(Ec - Ro).max() <= 1e-12 * np.abs(Ro).max()
    tets, pts, _ = random_points(prob, rng, 500)
    Ep = gpu.evaluate_field(M, x, tets, pts)
    Rp = O.edge_field(prob, x, tets, pts)
    assert np.abs(Ep - Rp).max() <= 1e-12 * np.abs(Rp).max()
    # Whitney known answer through the GPU path
    E0, b = np.array([1.0, -2.0, 0.5]), np.array([10.0, 0.0, -30.0])
    Ew = gpu.evaluate_field(M, interpolant(prob, E0, b).astype(complex), tets, pts)
    want = E0 + np.cross(b, pts)
    assert np.abs(Ew - want).max() <= 1e-12 * np.abs(want).max()
    with pytest.raises(ValueError, match="entries"):
        gpu.evaluate_field(M, x[:-1])


@pytest.mark.gpu
def test_evaluate_edge_field_single_tet(gpu):
    rng = np.random.default_rng(4)
    for _ in range(5):
        V = rng.normal(size=(4, 3))
        orient = rng.choice([-1, 1], size=6)
        dofs = rng.normal(size=6) + 1j * rng.normal(size=6)
        p = rng.dirichlet(np.ones(4)) @ V
        E = gpu.evaluate_edge_field(V, orient, dofs, p)
        lam = O.barycentric(V[None], p[None])[0]
        g, _ = O.gradients_and_volume(V[None])
        want = sum(orient[i] * dofs[i] * (lam[a] * g[0, b] - lam[b] * g[0, a])
                   for i, (a, b) in enumerate(O.TET_PAIRS))
        assert np.abs(E - want).max() <= 1e-12 * np.abs(want).max()


_NUM = re.compile(r"^-?\d+\.\d+e[+-]\d+$")


def same_text(got: str, want: str, rtol=2e-8):
    """Line by line; numbers printed as %.8e may differ in the last digit
    (the GPU and numpy sum in different orders), everything else is equal."""
    g, w = got.splitlines(), want.splitlines()
    assert len(g) == len(w)
    for a, b in zip(g, w):
        if a == b:
            continue
        ta, tb = a.split(), b.split()
        assert len(ta) == len(tb), (a, b)
        for u, v in zip(ta, tb):
            if u != v:
                assert _NUM.match(u) and _NUM.match(v), (a, b)
                assert abs(float(u) - float(v)) <= rtol * max(abs(float(v)), 1e-300), (a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [dict(), dict(export_real=True, export_imag=True, export_phase=False)])
def test_vtk_exports_match_oracle(gpu, tmp_path, opts):
    m = jittered_box()
    M = em.Mesh.from_arrays(m)
    prob = O.make_problem(m)
    x = np.random.default_rng(1).normal(size=prob.n) * (1 + 0.5j)
    o = em.VTKExportOptions(**opts)
    gpu.export_fields_vtk(M, x, str(tmp_path / "f.vtu"), o)
    same_text((tmp_path / "f.vtu").read_text(),
              O.vtu_text(prob, x, o.export_magnitude, o.export_phase, o.export_real, o.export_imag,
                         o.export_vector))
    gpu.export_fields_vtk_legacy(M, x, str(tmp_path / "f.vtk"), o)
    same_text((tmp_path / "f.vtk").read_text(), O.vtk_legacy_text(prob, x, o.export_magnitude, o.export_vector))


@pytest.mark.gpu
def test_design_export_fields_vtk(gpu, tmp_path):
    """RectWaveguideDesign.export_fields_vtk (waveguide.py:466-509): driven
    solve with port 1 active, one field magnitude per tet written."""
    wg = em.RectWaveguideDesign(a=22.86e-3, b=10.16e-3, length=50e-3)
    wg.set_mesh(waveguide_mesh(8, 4, 20, 22.86e-3, 10.16e-3, 50e-3))
    path = tmp_path / "wg.vtu"
    wg.export_fields_vtk(str(path), 10e9)
    text = path.read_text()
    assert text.startswith('<?xml version="1.0"?>') and 'Name="E_magnitude"' in text
    mags = re.search(r'Name="E_magnitude" format="ascii">\n(.*?)\n\s*</DataArray>', text, re.S).group(1)
    mag = np.array([float(v) for v in mags.split()])
    assert mag.size == wg.mesh.num_tets and mag.max() > 0
