"""StackedPatchDesign (the drop-in for python/edgefem/designs/stacked_patch.py):
host-side behaviour without a GPU, and simulate / frequency_sweep on the GPU
against the committed coarse-patch oracle fixture
(tests/golden/make_patch_golden.py)."""
import json
import math
import os

import numpy as np
import pytest

import edgefem_gb300 as em
from conftest import GOLDEN
from edgefem_gb300 import mesh as M

FR4_DEBYE = (4.488, 4.312, 1.0 / (2 * math.pi * 2.5e9))  # 4.4(1 - 0.02j) at 2.5 GHz


def fixture_design():
    """The fixture's mesh (mesh.py tags) with the reference's tag scheme, in a
    design whose Debye substrate equals the fixture's medium."""
    with open(os.path.join(GOLDEN, "patch_antenna_S.json")) as fh:
        gold = json.load(fh)
    arrays = M.patch_antenna_mesh(**gold["mesh"])
    arrays.tet_phys = np.where(arrays.tet_phys == M.DIELECTRIC_TAG, 110, 150).astype(np.int32)
    arrays.tri_phys = np.where(arrays.tri_phys == M.FEED_TAG, 5, arrays.tri_phys).astype(np.int32)
    d = em.StackedPatchDesign(patches=[{"width": 38e-3, "length": 29e-3, "height": 1.6e-3}],
                              substrates=[{"thickness": 1.6e-3, "eps_r": 4.4, "tan_d": 0.02, "debye": FR4_DEBYE}],
                              cavity_size=35e-3, cavity_depth=5e-3, probe_offset=(0.0, -5e-3),
                              ground_plane_size=100e-3)
    d.set_mesh(arrays)
    d.port_e_direction = (0.0, 0.0, 1.0)
    return d, gold


def test_constructor_and_repr():
    with pytest.raises(ValueError):
        em.StackedPatchDesign([], [{"thickness": 1e-3, "eps_r": 2.0}], 0.03, 0.005)
    with pytest.raises(ValueError):
        em.StackedPatchDesign([{"width": 0.03, "length": 0.025, "height": 1.6e-3}], [], 0.03, 0.005)
    d = em.StackedPatchDesign([{"width": 30e-3, "length": 25e-3, "height": 1.6e-3}],
                              [{"thickness": 1.6e-3, "eps_r": 4.4}], 35e-3, 5e-3)
    s = repr(d)
    assert "StackedPatchDesign" in s and "1 patch" in s  # python/tests/test_stacked_patch.py:180-188
    assert d.ground_plane_size == pytest.approx(90e-3)
    with pytest.raises(RuntimeError):
        d.simulate(2.4e9)
    two = em.StackedPatchDesign([{"width": 30e-3, "length": 25e-3, "height": 1.6e-3},
                                 {"width": 32e-3, "length": 27e-3, "height": 4.8e-3}],
                                [{"thickness": 1.6e-3, "eps_r": 4.4}, {"thickness": 3.2e-3, "eps_r": 1.05}],
                                35e-3, 5e-3)
    assert "2 patches" in repr(two) and "2 substrates" in repr(two)
    with pytest.raises(NotImplementedError):
        two.generate_mesh(density=8)


def test_generated_mesh_uses_reference_tags():
    d = em.StackedPatchDesign([{"width": 30e-3, "length": 25e-3, "height": 1.6e-3}],
                              [{"thickness": 1.6e-3, "eps_r": 4.4, "tan_d": 0.02}], 35e-3, 5e-3,
                              probe_offset=(0.0, -4e-3))
    d.generate_mesh(density=6)
    a = d.mesh.arrays()
    assert set(np.unique(a.tri_phys)) == {1, 5, 10, 50}
    assert set(np.unique(a.tet_phys)) == {110, 150}
    assert em.validate_mesh(d.mesh).is_valid()
    d._setup_simulation(2.4e9)
    pec = set(d._bc.dirichlet_edges)
    for tag in (1, 10):
        assert set(em.build_edge_pec(d.mesh, tag).dirichlet_edges) <= pec
    port = d._ports[0]
    assert port.edges.size > 0 and np.abs(port.weights).max() > 0
    assert port.mode.Z0 == pytest.approx(50.0)


@pytest.mark.gpu
def test_patch_design_sweep_and_simulate_match_oracle(gpu):
    """frequency_sweep(2.2, 2.8 GHz, 3 points) normalises at 2.5 GHz and
    solves on the batched engine: S11 within 1e-6 of the oracle's direct
    solve at each point; Z_in = z0 (1 + S11)/(1 - S11).  simulate(2.5 GHz)
    normalises at the same frequency: the same S11, and its solution vector
    solves the driven system of assemble_maxwell to the solver's tolerance.
    The plain per-frequency sweep agrees with the batched one."""
    d, gold = fixture_design()
    freqs, Z, S11 = d.frequency_sweep(2.2e9, 2.8e9, 3)
    assert np.allclose(freqs, gold["freqs"])
    for k in range(3):
        s_ref = complex(*gold["S11"][k])
        assert abs(S11[k] - s_ref) <= 1e-6
        assert abs(Z[k] - 50.0 * (1 + S11[k]) / (1 - S11[k])) <= 1e-9 * abs(Z[k])
    d.use_batched_sweep = False
    _, _, S11_plain = d.frequency_sweep(2.2e9, 2.8e9, 3)
    assert np.abs(S11_plain - S11).max() <= 1e-6
    S11_5, x = d.simulate(2.5e9)
    assert abs(S11_5 - complex(*gold["S11"][1])) <= 1e-6
    p = d._params(2.5e9)
    ports = em.normalize_port_weights(d.mesh, p, d._bc, d._ports, d._opts())
    asm = em.assemble_maxwell(d.mesh, p, d._bc, ports, 0)
    rp, ci, v = asm.A.csr()
    import scipy.sparse as sp
    A = sp.csr_matrix((v, ci, rp), shape=(asm.A.n, asm.A.n))
    assert np.linalg.norm(A @ x - asm.b) <= 1e-9 * np.linalg.norm(asm.b)
    Zin = d.input_impedance(2.5e9)
    assert np.isfinite(Zin.real) and np.isfinite(Zin.imag)
    assert d.return_loss(2.5e9) == pytest.approx(20 * math.log10(abs(S11_5) + 1e-30), abs=1e-6)
    # near field: E at the centroid of a substrate tet equals the centroid field
    a = d.mesh.arrays()
    t = int(np.flatnonzero(a.tet_phys == 110)[0])
    c = a.xyz[a.node_index()[a.tets[t]]].mean(axis=0)
    E = d.near_field(2.5e9, c[None, :])
    Ec = em.evaluate_field(d.mesh, d._last_solutions[2.5e9])[t]
    assert np.abs(E[0] - Ec).max() <= 1e-9 * max(np.abs(Ec).max(), 1e-30)
