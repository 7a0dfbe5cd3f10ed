"""C-ABI library and host-side logic (no GPU): every symbol the headers
declare is exported, and the host set-up (edge numbering, pattern, PEC set,
port modes, element kernels, mesh I/O) matches the oracle."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

import edgefem_oracle as O
from conftest import ROOT

import edgefem_gb300 as em
from edgefem_gb300 import _lib
from edgefem_gb300.mesh import read_gmsh_v2, waveguide_mesh, write_gmsh_v2


def declared_symbols():
    names = set()
    for h in ("edgefem_gb300.h", "edgefem_gb300_kernels.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(efgk?_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    names = declared_symbols()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_error_path_reports_message():
    with pytest.raises(_lib.EdgefemError, match="Failed to open mesh file"):
        em.load_gmsh("/nonexistent/file.msh")
    assert _lib.lib.efg_abi_version() == 5


@pytest.mark.parametrize("which", ["wr90", "grid"])
def test_topology_pattern_ports_match_oracle(which, wr90_mesh):
    m = wr90_mesh if which == "wr90" else waveguide_mesh(8, 4, 20)
    M = em.Mesh.from_arrays(m)
    prob = O.make_problem(m)
    en, te, to, re_, ro = M.topology()
    assert np.array_equal(en, prob.topo.edges)
    assert np.array_equal(te, prob.topo.tet_edges) and np.array_equal(to, prob.topo.tet_signs)
    assert np.array_equal(re_, prob.topo.tri_edges) and np.array_equal(ro, prob.topo.tri_signs)
    rp, ci, ncol = M.pattern()
    P = O.pattern(prob)
    assert np.array_equal(rp, P.indptr) and np.array_equal(ci, P.indices)
    assert 1 <= ncol <= 64
    bc = em.build_edge_pec(M, 1)
    assert np.array_equal(bc.pec_array(), prob.pec)
    a = 0.02286
    mode = em.solve_te10_mode(em.RectWaveguidePort(a, 0.01016), 10e9)
    ref = O.waveguide_ports(prob, a, 10e9)
    for tag, q in zip((2, 3), ref):
        p = em.build_wave_port_2d(M, tag, mode, bc.dirichlet_edges, (math.pi / a) ** 2)
        assert np.array_equal(p.edges, q.edges)
        assert abs(p.mode.kc - q.kc) <= 1e-12 * q.kc
        assert np.abs(p.weights - q.weights).max() <= 1e-11 * np.abs(q.weights).max()


def test_synthetic_mesh_counts():
    """Sizes of the Kuhn split used by the benchmark configurations."""
    def kuhn_edges(nx, ny, nz):
        axis = nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz
        faces = nx * ny * (nz + 1) + nx * (ny + 1) * nz + (nx + 1) * ny * nz
        return axis + faces + nx * ny * nz

    for grid, T, n, nnz in (((8, 4, 20), 3840, 5328, 77712), ((12, 6, 30), 12960, kuhn_edges(12, 6, 30), None)):
        m = waveguide_mesh(*grid)
        M = em.Mesh.from_arrays(m)
        assert M.num_tets == T and M.num_edges == n
        if nnz:
            assert M.pattern()[1].size == nnz
        q = em.validate_mesh(M)
        assert q.is_valid() and q.num_inverted_tets == 0


def test_element_kernels_match_oracle():
    rng = np.random.default_rng(1)
    X = rng.normal(size=(6, 4, 3))
    Kr, Mr, _ = O.whitney_matrices(X)
    for t in range(X.shape[0]):
        K, Mm = em.sdk.element_matrices(X[t])
        assert np.allclose(K, Kr[t], rtol=1e-12, atol=1e-12 * abs(Kr[t]).max())
        assert np.allclose(Mm, Mr[t], rtol=1e-12, atol=1e-12 * abs(Mr[t]).max())
    V = rng.normal(size=(5, 3, 3))
    Tr = O.triangle_whitney_mass(V)
    for s in range(V.shape[0]):
        assert np.allclose(em.sdk.triangle_mass(V[s]), Tr[s], rtol=1e-12, atol=1e-14)


def test_gmsh_roundtrip(tmp_path):
    m = waveguide_mesh(3, 2, 4)
    path = str(tmp_path / "box.msh")
    write_gmsh_v2(path, m)
    m2 = read_gmsh_v2(path)
    assert np.array_equal(m.tets, m2.tets) and np.array_equal(m.tris, m2.tris)
    assert np.allclose(m.xyz, m2.xyz, rtol=0, atol=0)
    M = em.load_gmsh(path)
    assert (M.num_nodes, M.num_tets, M.num_tris) == (m.num_nodes, m.num_tets, m.num_tris)
    assert np.array_equal(M.arrays().tets, m.tets)


def test_lumped_port_weights_match_oracle():
    from edgefem_gb300.mesh import box_tet_mesh
    m = box_tet_mesh(4, 4, 4, 0.01, 0.01, 0.01)
    M = em.Mesh.from_arrays(m)
    prob = O.make_problem(m)
    p = em.build_lumped_port(M, 2, 50.0, (1.0, 0.0, 0.0))
    q = O.build_lumped_port(prob, 2, (1.0, 0.0, 0.0), 50.0)
    assert np.array_equal(p.edges, q.edges)
    assert np.allclose(p.weights, q.weights, rtol=1e-12, atol=1e-14)
    assert abs(np.linalg.norm(p.weights) - math.sqrt(50.0)) < 1e-12
    with pytest.raises(_lib.EdgefemError, match="no triangles"):
        em.build_lumped_port(M, 77, 50.0, (1.0, 0.0, 0.0))


def test_batched_rejects_bad_inputs_without_gpu():
    """Argument validation happens before any device work."""
    m = waveguide_mesh(2, 1, 2)
    M = em.Mesh.from_arrays(m)
    bc = em.build_edge_pec(M, 1)
    inst = em.BatchInstance(M, em.MaxwellParams(), bc, [])
    with pytest.raises(_lib.EdgefemError, match="at least one port"):
        em.sparams_eigenmode_batched([inst], [10e9])


def test_batched_formulation_checks_without_gpu():
    """Driven-port, ABC and Debye options are validated before device work."""
    m = waveguide_mesh(2, 1, 2)
    M = em.Mesh.from_arrays(m)
    bc = em.build_edge_pec(M, 1)
    mode = em.solve_te10_mode(em.RectWaveguidePort(0.02286, 0.01016), 10e9)
    ports = [em.build_wave_port_2d(M, t, mode, bc.dirichlet_edges, (math.pi / 0.02286) ** 2) for t in (2, 3)]
    p = em.MaxwellParams()
    p.use_abc = True
    with pytest.raises(_lib.EdgefemError, match="driven-port formulation"):
        em.sparams_eigenmode_batched([em.BatchInstance(M, p, bc, ports)], [10e9])
    p = em.MaxwellParams()
    p.set_debye_region(100, 4.5, 4.3, 1e-11)
    with pytest.raises(_lib.EdgefemError, match="double-float"):
        em.sparams_eigenmode_batched([em.BatchInstance(M, p, bc, ports)], [10e9], em.BatchOptions(precision=0))
    with pytest.raises(_lib.EdgefemError, match="formulation must be"):
        em.sparams_eigenmode_batched([em.BatchInstance(M, em.MaxwellParams(), bc, ports)], [10e9],
                                     em.BatchOptions(formulation=5))


def test_patch_antenna_mesh_features():
    """The patch workload's mesh: valid after jitter, patch and feed faces are
    tetrahedron faces (their edges exist), the feed strip spans ground to patch."""
    from edgefem_gb300.mesh import patch_antenna_mesh
    m = patch_antenna_mesh(h_fine=3e-3, h_coarse=10e-3)
    M = em.Mesh.from_arrays(m)
    q = em.validate_mesh(M)
    assert q.num_inverted_tets == 0 and q.num_degenerate_tets == 0
    assert {1, 10, 20, 50} <= set(np.unique(m.tri_phys).tolist())
    lut = m.node_index()
    z_patch = m.xyz[lut[m.tris[m.tri_phys == 10]]][:, :, 2]
    assert np.allclose(z_patch, 1.6e-3)
    zf = m.xyz[lut[m.tris[m.tri_phys == 20]]][:, :, 2]
    assert abs(zf.min()) < 1e-12 and abs(zf.max() - 1.6e-3) < 1e-12
    port = em.build_lumped_port(M, 20, 50.0, (0.0, 0.0, 1.0))
    assert len(port.edges) > 0 and abs(np.linalg.norm(port.weights) - math.sqrt(50.0)) < 1e-9


def test_gpu_edge_builder_checks_without_gpu():
    """Device edge numbering: scratch sizing and argument checks run without
    a GPU; with no device the call fails loudly (no host fallback)."""
    fn = _lib.lib.efgk_build_edges_scratch_bytes
    fn.restype = ctypes.c_int64
    fn.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int32]
    assert fn(-1, 0, 0) == -1
    small, big = fn(10, 4, 20), fn(480000, 16000, 86961)
    assert 0 < small < big and big % 256 == 0
    # bucket keys (8 B), first/flag (4 B each) per occurrence, at least
    assert big >= 16 * (6 * 480000 + 3 * 16000)
    m = waveguide_mesh(2, 1, 2)
    bad = em.mesh.TetMesh(m.node_ids, m.xyz, np.where(m.tets == m.node_ids[0], 10 ** 9, m.tets), m.tet_phys,
                          m.tris, m.tri_phys)
    with pytest.raises(ValueError, match="unknown node id"):
        em.build_edges_gpu(bad)
    n = ctypes.c_int64()
    rc = _lib.lib.efg_build_edges_gpu(0, None, 1, None, 0, None, None, None, None, None, None, ctypes.byref(n), None)
    assert rc == -1 and "null argument" in _lib.lib.efg_last_error().decode()
    if em.device_count() == 0:
        with pytest.raises(_lib.EdgefemError):
            em.build_edges_gpu(m)


def _quality_meshes(wr90_mesh, cube_mesh):
    m = waveguide_mesh(4, 2, 4)
    tets = m.tets.copy()
    tets[3, [0, 1]] = tets[3, [1, 0]]  # inverted
    tets[7, 3] = tets[7, 0]            # degenerate: a repeated node (zero volume, zero-length edge)
    bad = em.mesh.TetMesh(m.node_ids, m.xyz, tets, m.tet_phys, m.tris, m.tri_phys)
    return {"wr90": wr90_mesh, "cube": cube_mesh, "bad": bad}


def test_validate_mesh_matches_oracle(wr90_mesh, cube_mesh):
    """Host validate_mesh against the oracle restatement of
    mesh_quality.cpp:10-83: counts, min volume and max aspect ratio equal
    to the last bit (same operation order, no fused operations)."""
    for name, m in _quality_meshes(wr90_mesh, cube_mesh).items():
        q = em.validate_mesh(em.Mesh.from_arrays(m))
        flags, nd, ni, vmin, amax = O.validate_mesh(m.node_ids, m.xyz, m.tets)
        assert (q.num_degenerate_tets, q.num_inverted_tets) == (nd, ni), name
        assert q.min_volume == vmin and q.max_aspect_ratio == amax, name
        if name == "bad":
            assert (nd, ni) == (1, 1) and np.flatnonzero(flags).tolist() == [3, 7] and math.isinf(amax)


def test_driven_adjoint_rejects_bad_inputs_without_gpu():
    """Port indices and complex port weights are refused before any device
    work (the adjoint relies on A = A^T, which needs real weights)."""
    from edgefem_gb300.mesh import box_tet_mesh
    M = em.Mesh.from_arrays(box_tet_mesh(2, 2, 2, 0.02, 0.02, 0.02))
    port = em.build_lumped_port(M, 2, 50.0, (1.0, 0.0, 0.0))
    p = em.MaxwellParams()
    p.omega = 2 * math.pi * 3e9
    with pytest.raises(_lib.EdgefemError, match="port index out of range"):
        em.sparams_driven_adjoint(M, p, em.BC(), [port], 1, 0)
    cport = em.WavePort(port.surface_tag, port.mode, np.asarray(port.edges, np.int32),
                        np.asarray(port.weights) * (1 + 0.5j))
    with pytest.raises(_lib.EdgefemError, match="port weights must be real"):
        em.sparams_driven_adjoint(M, p, em.BC(), [cport], 0, 0)


def test_lumped_port_reference_checks(cube_mesh):
    """tests/test_lumped_port.cpp's checks on cube_cavity.msh (surface tag 1,
    e = z, 50 ohm): edges found, one weight per edge, Z0 = 50, beta = 0,
    nonzero weights; and the same edges and weights as the oracle."""
    M = em.Mesh.from_arrays(cube_mesh)
    port = em.build_lumped_port(M, 1, 50.0, (0.0, 0.0, 1.0))
    assert len(port.edges) > 0 and len(port.weights) == len(port.edges)
    assert abs(port.mode.Z0 - 50.0) < 1e-10 and port.mode.beta == 0
    assert np.linalg.norm(port.weights) > 1e-10
    prob = O.make_problem(cube_mesh)
    q = O.build_lumped_port(prob, 1, (0.0, 0.0, 1.0), 50.0)
    assert np.array_equal(np.asarray(port.edges), q.edges)
    assert np.allclose(port.weights, q.weights, rtol=1e-12, atol=1e-14)


def test_batch_option_defaults_agree():
    """The SDK's BatchOptions and the C-ABI default (efg_batch_options_default,
    the C++ BatchOptions) hold the same values field by field, including the
    reduced-basis sample count."""
    import ctypes as C
    from edgefem_gb300 import _lib as L
    c = L.BatchOptionsC()
    L.lib.efg_batch_options_default(C.byref(c))
    py = em.BatchOptions().to_c()
    for name, _ in L.BatchOptionsC._fields_:
        assert getattr(c, name) == getattr(py, name), name
    assert c.rb_samples == 16 and c.precision == 2 and c.reorder == 0
