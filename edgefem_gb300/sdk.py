"""Python SDK over the C-ABI, with the names of the reference's `pyedgefem`
module (python/pyedgefem.cpp) for the hot path:

    load_gmsh, build_edge_pec, solve_te10_mode, build_wave_port_2d,
    build_lumped_port, MaxwellParams, SolveOptions, assemble_maxwell,
    solve_linear, calculate_sparams, calculate_sparams_eigenmode,
    normalize_port_weights, assemble_maxwell_km, frequency_sweep,
    check_passivity, validate_mesh

plus the chosen forms `sparams_eigenmode_batched` / `BatchSolver` and
`sparams_eigenmode_adjoint`.  Every solve runs on the GPU.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import sys
from typing import Dict, Iterable, List, Optional, Sequence, Set

import numpy as np

from . import _lib as L
from .mesh import TetMesh

C0 = 299792458.0


# ---------------------------------------------------------------------- mesh

class Mesh:
    """Owning handle on a library mesh (`Mesh` of include/edgefem/mesh.hpp:43-52)
    with its global edge numbering."""

    def __init__(self, handle):
        self._h = handle
        nn, nt, ns, ne = (C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64())
        L.check(L.lib.efg_mesh_sizes(self._h, C.byref(nn), C.byref(nt), C.byref(ns), C.byref(ne)))
        self.num_nodes, self.num_tets, self.num_tris, self.num_edges = nn.value, nt.value, ns.value, ne.value
        self._topo = None
        self._arrays = None

    @classmethod
    def from_arrays(cls, m: TetMesh) -> "Mesh":
        nid = np.ascontiguousarray(m.node_ids, np.int64)
        xyz = np.ascontiguousarray(m.xyz, np.float64)
        tets = np.ascontiguousarray(m.tets, np.int64)
        tp = np.ascontiguousarray(m.tet_phys, np.int32)
        tris = np.ascontiguousarray(m.tris, np.int64)
        sp_ = np.ascontiguousarray(m.tri_phys, np.int32)
        h = C.c_void_p()
        L.check(L.lib.efg_mesh_create(L.ptr(nid, C.c_int64), L.ptr(xyz, C.c_double), nid.size,
                                      L.ptr(tets, C.c_int64), L.ptr(tp, C.c_int32), tets.shape[0],
                                      L.ptr(tris, C.c_int64), L.ptr(sp_, C.c_int32), tris.shape[0],
                                      C.byref(h)), "mesh_create")
        out = cls(h)
        out._arrays = m
        return out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.lib.efg_mesh_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def arrays(self) -> TetMesh:
        if self._arrays is None:
            nid = np.empty(self.num_nodes, np.int64)
            xyz = np.empty((self.num_nodes, 3), np.float64)
            tets = np.empty((self.num_tets, 4), np.int64)
            tp = np.empty(self.num_tets, np.int32)
            tris = np.empty((self.num_tris, 3), np.int64)
            sp_ = np.empty(self.num_tris, np.int32)
            L.check(L.lib.efg_mesh_arrays(self._h, L.ptr(nid, C.c_int64), L.ptr(xyz, C.c_double),
                                          L.ptr(tets, C.c_int64), L.ptr(tp, C.c_int32),
                                          L.ptr(tris, C.c_int64), L.ptr(sp_, C.c_int32)))
            self._arrays = TetMesh(nid, xyz, tets, tp, tris, sp_)
        return self._arrays

    def topology(self):
        """(edges (n,2) node ids, tet_edges (T,6), tet_orient (T,6),
        tri_edges (S,3), tri_orient (S,3))."""
        if self._topo is None:
            en = np.empty((self.num_edges, 2), np.int64)
            te = np.empty((self.num_tets, 6), np.int32)
            to = np.empty((self.num_tets, 6), np.int8)
            re = np.empty((self.num_tris, 3), np.int32)
            ro = np.empty((self.num_tris, 3), np.int8)
            L.check(L.lib.efg_mesh_topology(self._h, L.ptr(en, C.c_int64), L.ptr(te, C.c_int32),
                                            L.ptr(to, C.c_int8), L.ptr(re, C.c_int32), L.ptr(ro, C.c_int8)))
            self._topo = (en, te, to, re, ro)
        return self._topo

    @property
    def edges(self):
        return self.topology()[0]

    def pattern(self):
        """Host CSR pattern (rowptr, colidx) and number of tet colours."""
        nnz = C.c_int64()
        nc = C.c_int32()
        L.check(L.lib.efg_pattern(self._h, None, None, C.byref(nnz), C.byref(nc)))
        rp = np.empty(self.num_edges + 1, np.int32)
        ci = np.empty(nnz.value, np.int32)
        L.check(L.lib.efg_pattern(self._h, L.ptr(rp, C.c_int32), L.ptr(ci, C.c_int32), C.byref(nnz),
                                  C.byref(nc)))
        return rp, ci, nc.value


def load_gmsh(path: str) -> Mesh:
    """load_gmsh_v2 (src/mesh_gmsh.cpp:15-101); raises EdgefemError if unreadable."""
    h = C.c_void_p()
    L.check(L.lib.efg_mesh_load_gmsh_v2(str(path).encode(), C.byref(h)), "load_gmsh")
    return Mesh(h)


def as_mesh(m) -> Mesh:
    return m if isinstance(m, Mesh) else Mesh.from_arrays(m)


@dataclasses.dataclass
class MeshQualityReport:
    num_degenerate_tets: int
    num_inverted_tets: int
    min_volume: float
    max_aspect_ratio: float
    bad_tet_indices: Optional[np.ndarray] = None

    def is_valid(self) -> bool:
        return self.num_degenerate_tets == 0 and self.num_inverted_tets == 0


def build_edges_gpu(m: TetMesh, timing: Optional[dict] = None):
    """Global edge numbering and orientations computed on the GPU
    (build_edges, mesh_gmsh.cpp:104-147): the same tuple as
    Mesh.topology(), i.e. (edges (n,2) node ids, tet_edges (T,6), tet_orient
    (T,6), tri_edges (S,3), tri_orient (S,3)).  `timing`, if given,
    receives the device time of the numbering kernels as "device_ms"."""
    ids = np.ascontiguousarray(m.node_ids, np.int64)
    order = np.argsort(ids, kind="stable")
    sorted_ids = ids[order]

    def dense(conn):
        conn = np.asarray(conn, np.int64)
        pos = np.searchsorted(sorted_ids, conn)
        pos = np.minimum(pos, max(len(ids) - 1, 0))
        if conn.size and (len(ids) == 0 or not np.array_equal(sorted_ids[pos], conn)):
            raise ValueError("build_edges_gpu: element references unknown node id")
        return np.ascontiguousarray(order[pos], np.int32) if conn.size else np.zeros(conn.shape, np.int32)

    tets = dense(m.tets).reshape(-1, 4)
    tris = dense(m.tris).reshape(-1, 3) if len(m.tris) else np.zeros((0, 3), np.int32)
    T, S = tets.shape[0], tris.shape[0]
    cap = max(6 * T + 3 * S, 1)
    en = np.empty((cap, 2), np.int64)
    te = np.empty((T, 6), np.int32)
    to = np.empty((T, 6), np.int8)
    re = np.empty((S, 3), np.int32)
    ro = np.empty((S, 3), np.int8)
    n = C.c_int64()
    ms = C.c_double()
    L.check(L.lib.efg_build_edges_gpu(ids.size, L.ptr(ids, C.c_int64), T, L.ptr(tets, C.c_int32), S,
                                      L.ptr(tris, C.c_int32), L.ptr(en, C.c_int64), L.ptr(te, C.c_int32),
                                      L.ptr(to, C.c_int8), L.ptr(re, C.c_int32), L.ptr(ro, C.c_int8),
                                      C.byref(n), C.byref(ms)), "build_edges_gpu")
    if timing is not None:
        timing["device_ms"] = ms.value
    return en[: n.value].copy(), te, to, re, ro


def validate_mesh(mesh: Mesh) -> MeshQualityReport:
    a, b = C.c_int32(), C.c_int32()
    c, d = C.c_double(), C.c_double()
    L.check(L.lib.efg_validate_mesh(mesh.handle, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
    return MeshQualityReport(a.value, b.value, c.value, d.value)


def validate_mesh_gpu(mesh: Mesh, timing: Optional[dict] = None) -> MeshQualityReport:
    """validate_mesh computed on the GPU (bit-identical report); the report's
    bad_tet_indices holds the degenerate and inverted tetrahedra in order
    (mesh_quality.cpp:71-77).  `timing`, if given, receives "device_ms"."""
    a, b = C.c_int32(), C.c_int32()
    c, d, ms = C.c_double(), C.c_double(), C.c_double()
    flags = np.empty(mesh.num_tets, np.int8)
    L.check(L.lib.efg_validate_mesh_gpu(mesh.handle, C.byref(a), C.byref(b), C.byref(c), C.byref(d),
                                        L.ptr(flags, C.c_int8), C.byref(ms)), "validate_mesh_gpu")
    if timing is not None:
        timing["device_ms"] = ms.value
    r = MeshQualityReport(a.value, b.value, c.value, d.value)
    r.bad_tet_indices = np.flatnonzero(flags).astype(np.int64)
    return r


class BC:
    """include/edgefem/bc.hpp:10-13."""

    def __init__(self, dirichlet_edges: Iterable[int] = ()):
        self.dirichlet_edges: Set[int] = set(int(e) for e in dirichlet_edges)
        self.dirichlet_nodes: Set[int] = set()

    def pec_array(self) -> np.ndarray:
        return np.array(sorted(self.dirichlet_edges), np.int32)

    def merge(self, other: "BC") -> None:
        """Add another BC's PEC edges and nodes (include/edgefem/bc.hpp)."""
        self.dirichlet_edges |= set(other.dirichlet_edges)
        self.dirichlet_nodes |= set(other.dirichlet_nodes)
        self._pec = None


def build_edge_pec(mesh: Mesh, pec_tag: int) -> BC:
    cnt = C.c_int64()
    L.check(L.lib.efg_build_edge_pec(mesh.handle, int(pec_tag), None, 0, C.byref(cnt)))
    out = np.empty(cnt.value, np.int32)
    L.check(L.lib.efg_build_edge_pec(mesh.handle, int(pec_tag), L.ptr(out, C.c_int32), out.size, C.byref(cnt)))
    bc = BC()
    bc.dirichlet_edges = set(out.tolist())
    bc._pec = out
    return bc


def has_surface_tag(mesh: Mesh, tag: int) -> bool:
    """True when a boundary triangle of `mesh` carries physical tag `tag`
    (the pyedgefem helper the design classes use to merge PEC tags)."""
    return bool(np.any(np.asarray(mesh.arrays().tri_phys) == int(tag)))


def merge_bc(*bcs) -> BC:
    """Union of the PEC edge sets (BC::merge of the reference's bindings)."""
    out = BC()
    for b in bcs:
        out.merge(b)
    return out


def _pec_of(bc) -> np.ndarray:
    if bc is None:
        return np.zeros(0, np.int32)
    arr = getattr(bc, "_pec", None)
    if arr is None or arr.size != len(bc.dirichlet_edges):
        arr = np.array(sorted(bc.dirichlet_edges), np.int32)
    return arr


# --------------------------------------------------------------------- ports

@dataclasses.dataclass
class RectWaveguidePort:
    a: float = 0.0
    b: float = 0.0


@dataclasses.dataclass
class PortMode:
    fc: float = 0.0
    kc: float = 0.0
    omega: float = 0.0
    eps: complex = 0j
    mu: complex = 0j
    beta: complex = 0j
    Z0: complex = 0j

    def to_c(self) -> L.PortMode:
        m = L.PortMode()
        m.fc, m.kc, m.omega = self.fc, self.kc, self.omega
        for name in ("eps", "mu", "beta", "Z0"):
            v = complex(getattr(self, name))
            getattr(m, name)[0] = v.real
            getattr(m, name)[1] = v.imag
        return m

    @classmethod
    def from_c(cls, m: L.PortMode) -> "PortMode":
        return cls(m.fc, m.kc, m.omega, complex(m.eps[0], m.eps[1]), complex(m.mu[0], m.mu[1]),
                   complex(m.beta[0], m.beta[1]), complex(m.Z0[0], m.Z0[1]))


@dataclasses.dataclass
class WavePort:
    """include/edgefem/ports/wave_port.hpp:19-24."""
    surface_tag: int
    mode: PortMode
    edges: np.ndarray      # int32
    weights: np.ndarray    # complex128


def solve_te10_mode(port: RectWaveguidePort, freq: float) -> PortMode:
    m = L.PortMode()
    L.check(L.lib.efg_solve_te10_mode(float(port.a), float(port.b), float(freq), C.byref(m)))
    return PortMode.from_c(m)


def build_wave_port_2d(mesh: Mesh, surface_tag: int, mode: PortMode, pec_edges, target_kc_sq: float) -> WavePort:
    pec = np.array(sorted(int(e) for e in pec_edges), np.int32)
    cm = mode.to_c()
    cnt = C.c_int64()
    kc = C.c_double()
    L.check(L.lib.efg_build_wave_port_2d(mesh.handle, int(surface_tag), C.byref(cm), L.ptr(pec, C.c_int32),
                                         pec.size, float(target_kc_sq), None, None, 0, C.byref(cnt),
                                         C.byref(kc)))
    edges = np.empty(cnt.value, np.int32)
    w = np.empty(cnt.value, np.complex128)
    L.check(L.lib.efg_build_wave_port_2d(mesh.handle, int(surface_tag), C.byref(cm), L.ptr(pec, C.c_int32),
                                         pec.size, float(target_kc_sq), L.ptr(edges, C.c_int32),
                                         L.ptr(w.view(np.float64), C.c_double), edges.size, C.byref(cnt),
                                         C.byref(kc)), "build_wave_port_2d")
    m = dataclasses.replace(mode, kc=kc.value)
    return WavePort(int(surface_tag), m, edges, w)


def build_lumped_port(mesh: Mesh, surface_tag: int, z0: float = 50.0, e_direction=(0.0, 0.0, 1.0),
                      weight_mode: int = 0) -> WavePort:
    e = np.asarray(e_direction, np.float64)
    cnt = C.c_int64()
    L.check(L.lib.efg_build_lumped_port(mesh.handle, int(surface_tag), float(z0), L.ptr(e, C.c_double),
                                        int(weight_mode), None, None, 0, C.byref(cnt)), "build_lumped_port")
    edges = np.empty(cnt.value, np.int32)
    w = np.empty(cnt.value, np.complex128)
    L.check(L.lib.efg_build_lumped_port(mesh.handle, int(surface_tag), float(z0), L.ptr(e, C.c_double),
                                        int(weight_mode), L.ptr(edges, C.c_int32),
                                        L.ptr(w.view(np.float64), C.c_double), edges.size, C.byref(cnt)))
    return WavePort(int(surface_tag), PortMode(Z0=complex(z0)), edges, w)


# --------------------------------------------------------------- parameters

class MaxwellParams:
    """include/edgefem/maxwell.hpp:46-143 (without PML).  `eps_r_tet` (one
    complex value per tetrahedron) is an extension that replaces the region
    lookup when set."""

    def __init__(self):
        self.omega = 0.0
        self.eps_r = 1.0 + 0j
        self.mu_r = 1.0 + 0j
        self.eps_r_regions: Dict[int, complex] = {}
        self.mu_r_regions: Dict[int, complex] = {}
        self.eps_models: Dict[int, tuple] = {}   # tag -> (eps_s, eps_inf, tau) Debye
        self.eps_r_tet: Optional[np.ndarray] = None
        self.use_abc = False
        self.abc_surface_tags: Set[int] = set()
        self.port_abc_scale = 1.0
        # legacy port ABC (maxwell.hpp:36-82): 0 None, 1 Beta, 2 BetaNorm,
        # 3 ImpedanceMatch, 4 ModalAdmittance
        self.use_port_abc = False
        self.port_abc_type = 1

    def set_eps_r_region(self, tag: int, eps) -> None:
        self.eps_r_regions[int(tag)] = complex(eps)

    def set_mu_r_region(self, tag: int, mu) -> None:
        self.mu_r_regions[int(tag)] = complex(mu)

    def set_debye_region(self, tag: int, eps_s: float, eps_inf: float, tau: float) -> None:
        if tau <= 0:
            raise ValueError("DebyeMaterial: tau must be positive")
        self.eps_models[int(tag)] = (float(eps_s), float(eps_inf), float(tau))

    def to_c(self, keep: list) -> L.MaxwellParamsC:
        p = L.MaxwellParamsC()
        L.lib.efg_maxwell_params_default(C.byref(p))
        p.omega = float(self.omega)
        p.eps_r[0], p.eps_r[1] = complex(self.eps_r).real, complex(self.eps_r).imag
        p.mu_r[0], p.mu_r[1] = complex(self.mu_r).real, complex(self.mu_r).imag

        def regions(d):
            tags = np.array(list(d.keys()), np.int32)
            vals = np.array([complex(v) for v in d.values()], np.complex128).view(np.float64)
            keep.extend([tags, vals])
            return len(d), L.ptr(tags, C.c_int32), L.ptr(vals, C.c_double)

        p.n_eps_regions, p.eps_region_tags, p.eps_region_vals = regions(self.eps_r_regions)
        p.n_mu_regions, p.mu_region_tags, p.mu_region_vals = regions(self.mu_r_regions)
        if self.eps_models:
            tags = np.array(list(self.eps_models.keys()), np.int32)
            prm = np.array([list(v) for v in self.eps_models.values()], np.float64).ravel()
            keep.extend([tags, prm])
            p.n_debye, p.debye_tags, p.debye_params = len(tags), L.ptr(tags, C.c_int32), L.ptr(prm, C.c_double)
        if self.eps_r_tet is not None:
            et = np.ascontiguousarray(np.asarray(self.eps_r_tet, np.complex128)).view(np.float64)
            keep.append(et)
            p.eps_tet = L.ptr(et, C.c_double)
        p.use_abc = int(bool(self.use_abc))
        if self.abc_surface_tags:
            at = np.array(sorted(self.abc_surface_tags), np.int32)
            keep.append(at)
            p.n_abc_tags, p.abc_tags = at.size, L.ptr(at, C.c_int32)
        p.port_abc_scale = float(self.port_abc_scale)
        p.use_port_abc = int(bool(self.use_port_abc))
        p.port_abc_type = int(self.port_abc_type)
        return p


@dataclasses.dataclass
class SolveOptions:
    """include/edgefem/solver.hpp:16-46 (GPU iterative methods only)."""
    use_bicgstab: bool = True
    use_direct: bool = False
    tolerance: float = 1e-10
    max_iterations: int = 10000
    verbose: bool = False
    # "aux" (Jacobi + nodal gradient + vector-nodal spaces), "gradient"
    # (Jacobi + nodal gradient space), "block_jacobi" (16-row diagonal
    # blocks) or "jacobi".  "aux" and "gradient" need mesh data: the drivers
    # have it, solve_linear has it for matrices from assemble_maxwell and
    # uses "block_jacobi" in their place on other matrices.
    preconditioner: str = "aux"
    # False: Jacobi, as the reference's BiCGSTAB without ILUT
    use_ilut: bool = True

    def to_c(self) -> L.SolveOptionsC:
        o = L.SolveOptionsC()
        o.use_bicgstab, o.use_direct = int(self.use_bicgstab), int(self.use_direct)
        o.tolerance, o.max_iterations, o.verbose = float(self.tolerance), int(self.max_iterations), int(self.verbose)
        levels = {"jacobi": 0, "gradient": 1, "aux": 2, "block_jacobi": 3}
        if self.preconditioner not in levels:
            raise ValueError("preconditioner must be 'aux', 'gradient', 'block_jacobi' or 'jacobi'")
        o.preconditioner = levels[self.preconditioner]
        o.use_ilut = int(bool(self.use_ilut))
        return o


@dataclasses.dataclass
class SolveResult:
    method: str
    iters: int
    residual: float
    converged: bool
    error_message: str
    x: np.ndarray


def _ports_c(ports: Sequence[WavePort], keep: list):
    arr = (L.WavePortC * max(1, len(ports)))()
    for i, pt in enumerate(ports):
        e = np.ascontiguousarray(pt.edges, np.int32)
        w = np.ascontiguousarray(pt.weights, np.complex128)
        keep.extend([e, w])
        arr[i].surface_tag = int(pt.surface_tag)
        arr[i].n_edges = e.size
        arr[i].edges = L.ptr(e, C.c_int32)
        arr[i].weights = L.ptr(w.view(np.float64), C.c_double)
        arr[i].mode = pt.mode.to_c()
    return arr


# ----------------------------------------------------------- sparse matrix

class SpMatC:
    """Complex CSR matrix owned by the library (SpMatC of edgefem.hpp)."""

    def __init__(self, handle):
        self._h = handle
        n, nnz = C.c_int32(), C.c_int64()
        L.check(L.lib.efg_spmat_info(self._h, C.byref(n), C.byref(nnz)))
        self.n, self.nnz = n.value, nnz.value

    @classmethod
    def from_csr(cls, indptr, indices, data, n: int) -> "SpMatC":
        rp = np.ascontiguousarray(indptr, np.int32)
        ci = np.ascontiguousarray(indices, np.int32)
        v = np.ascontiguousarray(data, np.complex128)
        h = C.c_void_p()
        L.check(L.lib.efg_spmat_create(int(n), ci.size, L.ptr(rp, C.c_int32), L.ptr(ci, C.c_int32),
                                       L.ptr(v.view(np.float64), C.c_double), C.byref(h)), "spmat_create")
        return cls(h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.lib.efg_spmat_destroy(h)
            self._h = None

    def csr(self):
        rp = np.empty(self.n + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        v = np.empty(self.nnz, np.complex128)
        L.check(L.lib.efg_spmat_export(self._h, L.ptr(rp, C.c_int32), L.ptr(ci, C.c_int32),
                                       L.ptr(v.view(np.float64), C.c_double)))
        return rp, ci, v

    def nonZeros(self) -> int:
        return self.nnz

    def to_dense(self) -> np.ndarray:
        rp, ci, v = self.csr()
        D = np.zeros((self.n, self.n), np.complex128)
        rows = np.repeat(np.arange(self.n), np.diff(rp))
        np.add.at(D, (rows, ci), v)
        return D

    def coeff(self, r: int, c: int) -> complex:
        rp, ci, v = self.csr()
        seg = ci[rp[r]:rp[r + 1]]
        k = np.searchsorted(seg, c)
        return complex(v[rp[r] + k]) if k < seg.size and seg[k] == c else 0j


@dataclasses.dataclass
class MaxwellAssembly:
    A: SpMatC
    b: np.ndarray


# -------------------------------------------------------------- entry points

def assemble_maxwell(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort] = (),
                     active_port_idx: int = -1) -> MaxwellAssembly:
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    pa = _ports_c(ports, keep)
    h = C.c_void_p()
    b = np.empty(mesh.num_edges, np.complex128)
    L.check(L.lib.efg_assemble_maxwell(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size, pa, len(ports),
                                       int(active_port_idx), C.byref(h), L.ptr(b.view(np.float64), C.c_double)),
            "assemble_maxwell")
    return MaxwellAssembly(SpMatC(h), b)


def solve_linear(A: SpMatC, b: np.ndarray, opts: Optional[SolveOptions] = None) -> SolveResult:
    opts = opts or SolveOptions()
    bb = np.ascontiguousarray(b, np.complex128)
    x = np.empty(A.n, np.complex128)
    oc = opts.to_c()
    rc = L.SolveResultC()
    L.check(L.lib.efg_solve_linear(A._h, L.ptr(bb.view(np.float64), C.c_double), C.byref(oc),
                                   L.ptr(x.view(np.float64), C.c_double), C.byref(rc)), "solve_linear")
    return SolveResult(rc.method.decode(), rc.iters, rc.residual, bool(rc.converged),
                       rc.error_message.decode(), x)


def calculate_sparams(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort],
                      opts: Optional[SolveOptions] = None) -> np.ndarray:
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    pa = _ports_c(ports, keep)
    oc = (opts or SolveOptions()).to_c()
    S = np.empty((len(ports), len(ports)), np.complex128)
    L.check(L.lib.efg_calculate_sparams(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size, pa, len(ports),
                                        C.byref(oc), L.ptr(S.view(np.float64), C.c_double)), "calculate_sparams")
    return S


def normalize_port_weights(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort],
                           opts: Optional[SolveOptions] = None) -> List[WavePort]:
    """Returns a normalised copy of the ports, like the reference's binding
    (pyedgefem.cpp:552-563)."""
    out = [dataclasses.replace(pt, weights=np.array(pt.weights, np.complex128, copy=True)) for pt in ports]
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    pa = _ports_c(out, keep)
    oc = (opts or SolveOptions()).to_c()
    L.check(L.lib.efg_normalize_port_weights(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size, pa,
                                             len(out), C.byref(oc)), "normalize_port_weights")
    # weights were updated in place through the pointers kept alive above
    return out


def calculate_sparams_eigenmode(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort],
                                opts: Optional[SolveOptions] = None, stats: Optional[dict] = None) -> np.ndarray:
    """Plain form: unbatched FP64 COCG on the GPU, one active port at a time.
    `stats`, if given, receives the summed iterations and worst residual."""
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    pa = _ports_c(ports, keep)
    oc = opts.to_c() if opts is not None else None
    S = np.empty((len(ports), len(ports)), np.complex128)
    rc = L.SolveResultC()
    L.check(L.lib.efg_calculate_sparams_eigenmode(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size, pa,
                                                  len(ports), C.byref(oc) if oc is not None else None,
                                                  L.ptr(S.view(np.float64), C.c_double), C.byref(rc)),
            "calculate_sparams_eigenmode")
    if stats is not None:
        stats.update(iters=rc.iters, residual=rc.residual, converged=bool(rc.converged), method=rc.method.decode())
    return S


def assemble_maxwell_km(mesh: Mesh, p: MaxwellParams, bc: BC):
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    hk, hm = C.c_void_p(), C.c_void_p()
    L.check(L.lib.efg_assemble_maxwell_km(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size,
                                          C.byref(hk), C.byref(hm)), "assemble_maxwell_km")
    return SpMatC(hk), SpMatC(hm)


@dataclasses.dataclass
class SweepResult:
    frequencies: np.ndarray
    S_matrices: List[np.ndarray]


def frequency_sweep(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort], frequencies,
                    opts: Optional[SolveOptions] = None) -> SweepResult:
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    pa = _ports_c(ports, keep)
    f = np.ascontiguousarray(frequencies, np.float64)
    oc = (opts or SolveOptions()).to_c()
    S = np.empty((f.size, len(ports), len(ports)), np.complex128)
    L.check(L.lib.efg_frequency_sweep(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size, pa, len(ports),
                                      L.ptr(f, C.c_double), f.size, C.byref(oc),
                                      L.ptr(S.view(np.float64), C.c_double)), "frequency_sweep")
    return SweepResult(f, [S[i] for i in range(f.size)])


def krylov_totals(reset: bool = False) -> dict:
    """Plain-path Krylov totals of this thread (iterations, solves, largest
    residual, device ms) since the last reset."""
    it, so, res, ms = C.c_int64(), C.c_int32(), C.c_double(), C.c_double()
    L.lib.efg_krylov_totals(1 if reset else 0, C.byref(it), C.byref(so), C.byref(res), C.byref(ms))
    return {"iters": it.value, "solves": so.value, "max_residual": res.value, "device_ms": ms.value}


def _frequency_sweep_batched_local(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort], freqs,
                                   opts: Optional["BatchOptions"]):
    """One process's batched driven sweep: (S[F, P, P], stats)."""
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    pa = _ports_c(ports, keep)
    f = np.ascontiguousarray(freqs, np.float64)
    oc = (opts or BatchOptions()).to_c()
    S = np.empty((f.size, len(ports), len(ports)), np.complex128)
    st = L.BatchStatsC()
    L.check(L.lib.efg_frequency_sweep_batched(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size, pa,
                                              len(ports), L.ptr(f, C.c_double), f.size, C.byref(oc),
                                              L.ptr(S.view(np.float64), C.c_double), C.byref(st)),
            "frequency_sweep_batched")
    return S, _stats(st)


def _shard_wanted(shard: Optional[bool]) -> bool:
    if shard is False:
        return False
    from .replicas import world_info
    return world_info()[1] > 1


def frequency_sweep_batched(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort], frequencies,
                            opts: Optional["BatchOptions"] = None, shard: Optional[bool] = None):
    """frequency_sweep (src/sweep.cpp:174-349) as one batched double-float
    solve of all frequencies x active ports.  Returns (SweepResult, stats).

    Under a torch.distributed process group of several ranks (one process
    per GPU) the frequencies are sharded across the ranks (interleaved; each
    rank solves its share on its own GPU) and every rank returns the full
    sweep; stats then describe this rank's share (stats["ranks"] = world
    size).  shard=False keeps the whole sweep on this process."""
    f = np.ascontiguousarray(frequencies, np.float64)
    if not _shard_wanted(shard):
        S, st = _frequency_sweep_batched_local(mesh, p, bc, ports, f, opts)
        return SweepResult(f, [S[i] for i in range(f.size)]), st
    from .replicas import sharded_sweep, world_info
    local_stats: dict = {}

    def solve(fl):
        S_, st_ = _frequency_sweep_batched_local(mesh, p, bc, ports, fl, opts)
        local_stats.update(st_)
        return S_

    S = sharded_sweep(solve, f)
    local_stats["ranks"] = world_info()[1]
    return SweepResult(f, [S[i] for i in range(f.size)]), local_stats


# ------------------------------------------------------ field post-processing

def _pf(a: np.ndarray):
    return a.ctypes.data_as(L.P(L.f64))


def compute_barycentric(vertices, point) -> np.ndarray:
    """compute_barycentric (src/edge_basis.cpp:131-151)."""
    v = np.ascontiguousarray(np.asarray(vertices, np.float64).reshape(4, 3))
    p = np.ascontiguousarray(np.asarray(point, np.float64).reshape(3))
    out = np.empty(4, np.float64)
    L.check(L.lib.efg_compute_barycentric(_pf(v), _pf(p), _pf(out)), "compute_barycentric")
    return out


def evaluate_edge_field(vertices, edge_orient, edge_dofs, point) -> np.ndarray:
    """evaluate_edge_field (src/edge_basis.cpp:162-193): E (3 complex) at a
    point of one tetrahedron from its six edge DOFs (GPU)."""
    v = np.ascontiguousarray(np.asarray(vertices, np.float64).reshape(4, 3))
    o = np.ascontiguousarray(np.asarray(edge_orient, np.int32).reshape(6))
    d = np.ascontiguousarray(np.asarray(edge_dofs, np.complex128).reshape(6))
    p = np.ascontiguousarray(np.asarray(point, np.float64).reshape(3))
    E = np.empty(3, np.complex128)
    L.check(L.lib.efg_evaluate_edge_field(_pf(v), o.ctypes.data_as(L.P(L.i32)), _f64(d), _pf(p), _f64(E)),
            "evaluate_edge_field")
    return E


def evaluate_field(mesh: Mesh, solution, tet_of=None, points=None) -> np.ndarray:
    """E of an edge solution on the GPU: at `points` (point i inside tet
    tet_of[i]) or, with neither given, at every tet centroid.  [n][3] complex."""
    x = np.ascontiguousarray(np.asarray(solution, np.complex128))
    if x.size != mesh.num_edges:
        raise ValueError(f"solution has {x.size} entries, the mesh {mesh.num_edges} edges")
    if tet_of is None and points is None:
        E = np.empty((mesh.num_tets, 3), np.complex128)
        L.check(L.lib.efg_evaluate_field(mesh._h, _f64(x), 0, None, None, _f64(E)), "evaluate_field")
        return E
    to = np.ascontiguousarray(np.asarray(tet_of, np.int32).ravel())
    pts = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1, 3))
    if to.size != pts.shape[0]:
        raise ValueError("tet_of and points differ in length")
    E = np.empty((to.size, 3), np.complex128)
    L.check(L.lib.efg_evaluate_field(mesh._h, _f64(x), to.size, to.ctypes.data_as(L.P(L.i32)), _pf(pts),
                                     _f64(E)), "evaluate_field")
    return E


@dataclasses.dataclass
class VTKExportOptions:
    """include/edgefem/io/vtk_export.hpp:10-26."""
    export_magnitude: bool = True
    export_phase: bool = True
    export_real: bool = False
    export_imag: bool = False
    export_vector: bool = True

    def to_c(self) -> L.VTKOptionsC:
        return L.VTKOptionsC(int(self.export_magnitude), int(self.export_phase), int(self.export_real),
                             int(self.export_imag), int(self.export_vector))


def _export_vtk(mesh: Mesh, solution, filename: str, options, legacy: int):
    x = np.ascontiguousarray(np.asarray(solution, np.complex128))
    if x.size != mesh.num_edges:
        raise ValueError(f"solution has {x.size} entries, the mesh {mesh.num_edges} edges")
    o = (options or VTKExportOptions()).to_c()
    L.check(L.lib.efg_export_fields_vtk(mesh._h, _f64(x), str(filename).encode(), C.byref(o), legacy),
            "export_fields_vtk")


def export_fields_vtk(mesh: Mesh, solution, filename: str, options: Optional[VTKExportOptions] = None) -> None:
    """export_fields_vtk (src/io/vtk_export.cpp:44-200): .vtu with E at the
    tet centroids (evaluated on the GPU)."""
    _export_vtk(mesh, solution, filename, options, 0)


def export_fields_vtk_legacy(mesh: Mesh, solution, filename: str,
                             options: Optional[VTKExportOptions] = None) -> None:
    """export_fields_vtk_legacy (src/io/vtk_export.cpp:202-272): legacy .vtk."""
    _export_vtk(mesh, solution, filename, options, 1)


# ------------------------------------------- network parameters, Touchstone

def _square(S) -> np.ndarray:
    S = np.ascontiguousarray(np.asarray(S, dtype=np.complex128))
    if S.ndim != 2 or S.shape[0] != S.shape[1]:
        raise ValueError("S-matrix must be square")
    return S


def _f64(a: np.ndarray):
    return a.view(np.float64).ctypes.data_as(L.P(L.f64))


@dataclasses.dataclass
class CouplingMatrix:
    """include/edgefem/coupling.hpp:9-17."""
    Z: np.ndarray
    Y: np.ndarray
    S: np.ndarray
    frequency: float
    z0: float
    num_ports: int


def compute_coupling(S, freq: float, z0: float = 50.0) -> CouplingMatrix:
    """compute_coupling (src/coupling.cpp:9-50)."""
    S = _square(S)
    n = S.shape[0]
    Z = np.empty((n, n), np.complex128)
    Y = np.empty((n, n), np.complex128)
    L.check(L.lib.efg_compute_coupling(n, _f64(S), float(freq), float(z0), _f64(Z), _f64(Y)), "compute_coupling")
    return CouplingMatrix(Z, Y, S.copy(), float(freq), float(z0), n)


def mutual_coupling_db(cm: CouplingMatrix) -> np.ndarray:
    """mutual_coupling_db (src/coupling.cpp:52-65)."""
    S = _square(cm.S)
    out = np.empty(S.shape, np.float64)
    L.check(L.lib.efg_mutual_coupling_db(S.shape[0], _f64(S), out.ctypes.data_as(L.P(L.f64))), "mutual_coupling_db")
    return out


def active_reflection(S, excitation) -> np.ndarray:
    """active_reflection (src/coupling.cpp:67-94)."""
    S = _square(S)
    a = np.ascontiguousarray(np.asarray(excitation, dtype=np.complex128).ravel())
    if a.size != S.shape[0]:
        raise ValueError("Excitation vector size must match S-matrix dimension")
    g = np.empty(S.shape[0], np.complex128)
    L.check(L.lib.efg_active_reflection(S.shape[0], _f64(S), _f64(a), _f64(g)), "active_reflection")
    return g


def _predicate(name: str, S, tol: float) -> bool:
    S = np.asarray(S, dtype=np.complex128)
    if S.ndim != 2 or S.shape[0] != S.shape[1]:
        return False
    S = np.ascontiguousarray(S)
    return bool(L.check(getattr(L.lib, name)(S.shape[0], _f64(S), float(tol)), name))


def is_passive(S, tolerance: float = 1e-6) -> bool:
    """is_passive (src/coupling.cpp:96-112): largest singular value <= 1 + tol."""
    return _predicate("efg_is_passive", S, tolerance)


def is_lossless(S, tolerance: float = 1e-6) -> bool:
    """is_lossless (src/coupling.cpp:114-126): S^H S approximately I."""
    return _predicate("efg_is_lossless", S, tolerance)


def is_reciprocal(S, tolerance: float = 1e-6) -> bool:
    """is_reciprocal (src/coupling.cpp:128-136): S approximately S^T."""
    return _predicate("efg_is_reciprocal", S, tolerance)


def check_passivity(S, tolerance: float = 1e-6) -> bool:
    """check_passivity (pyedgefem.cpp:701-730): is_passive, with a warning on
    stderr (largest singular value; 2-port column power sums) when violated."""
    S = np.asarray(S, dtype=np.complex128)
    if S.size == 0 or not np.all(np.isfinite(S)):
        return False
    return _predicate("efg_check_passivity", S, tolerance)


def singular_values(S) -> np.ndarray:
    """Singular values of S, largest first."""
    S = _square(S)
    out = np.empty(S.shape[0], np.float64)
    L.check(L.lib.efg_singular_values(S.shape[0], _f64(S), out.ctypes.data_as(L.P(L.f64))), "singular_values")
    return out


class TouchstoneFormat:
    """include/edgefem/io/touchstone.hpp:12-17."""
    RI = 0
    MA = 1
    DB = 2


@dataclasses.dataclass
class TouchstoneOptions:
    """include/edgefem/io/touchstone.hpp:19-23."""
    format: int = TouchstoneFormat.RI
    z0: float = 50.0


def write_touchstone_nport(path: str, freq, S_matrices, opts: Optional[TouchstoneOptions] = None) -> None:
    """write_touchstone_nport (src/io/touchstone.cpp:64-139); the same checks
    in the same order (empty data, port count, shapes, count mismatch)."""
    opts = opts or TouchstoneOptions()
    f = np.ascontiguousarray(np.asarray(list(freq), dtype=np.float64))
    mats = [np.asarray(S, dtype=np.complex128) for S in S_matrices]
    if f.size == 0 or not mats:
        raise L.EdgefemError("Empty frequency or S-parameter data")
    n = mats[0].shape[0] if mats[0].ndim == 2 else 0
    if not 1 <= n <= 99:
        raise L.EdgefemError(f"Invalid number of ports: {n}")
    for k, S in enumerate(mats):
        if S.shape != (n, n):
            raise L.EdgefemError(f"S-matrix dimension mismatch at frequency {k}")
    if len(mats) != f.size:
        raise L.EdgefemError("Frequency and S-matrix count mismatch")
    arr = np.ascontiguousarray(np.stack(mats))
    L.check(L.lib.efg_write_touchstone_nport(str(path).encode(), f.size, f.ctypes.data_as(L.P(L.f64)), n,
                                             _f64(arr), int(opts.format), float(opts.z0)),
            "write_touchstone_nport")


def write_touchstone(path: str, freq, data) -> None:
    """write_touchstone (src/io/touchstone.cpp:48-60): 2-port legacy form;
    `data` holds per frequency (s11, s21, s12, s22) or a 2x2 matrix."""
    f = np.ascontiguousarray(np.asarray(list(freq), dtype=np.float64))
    rows = []
    for d in data:
        d = np.asarray(d, dtype=np.complex128)
        rows.append([d[0, 0], d[1, 0], d[0, 1], d[1, 1]] if d.shape == (2, 2) else list(d.ravel()[:4]))
    arr = np.ascontiguousarray(np.asarray(rows, np.complex128).reshape(-1, 4))
    if arr.shape[0] < f.size:
        raise L.EdgefemError("Frequency and S-parameter count mismatch")
    L.check(L.lib.efg_write_touchstone(str(path).encode(), f.size, f.ctypes.data_as(L.P(L.f64)),
                                       _f64(arr) if arr.size else None), "write_touchstone")


def touchstone_extension(num_ports: int) -> str:
    """touchstone_extension (src/io/touchstone.cpp:141-149)."""
    buf = C.create_string_buffer(16)
    L.check(L.lib.efg_touchstone_extension(int(num_ports), buf, 16), "touchstone_extension")
    return buf.value.decode()


# ------------------------------------------------------------ chosen forms

@dataclasses.dataclass
class BatchOptions:
    tolerance: float = 1e-8
    max_iterations: int = 40000
    refine_interval: int = 0
    rows_per_block: int = 0
    use_graph: bool = True
    verbose: bool = False
    time_spmm: bool = False
    # 2: double-float K and M (default); 1: double-float K, FP32 M;
    # 0: complex64 vectors restarted at each FP64 residual replacement
    precision: int = 2
    # 0: eigenmode wave ports; 1: driven ports (w w^H / Z0, ABC, Debye)
    formulation: int = 0
    # add the vector-nodal (Pi) auxiliary space to the double-float preconditioner
    vector_aux: bool = True
    # renumber edges and nodes in Z-order inside the engine (gather locality;
    # about 2% faster solves, about 2 s more set-up at 580k edges)
    reorder: bool = False
    # reduced-basis initial guesses: solve rb_samples evenly spaced sample
    # frequencies first and start every column from the Galerkin solution on
    # their solutions (0 = off; capped at 64 / ports; needs at least twice as
    # many frequencies)
    rb_samples: int = 16

    def to_c(self) -> L.BatchOptionsC:
        o = L.BatchOptionsC()
        o.tolerance, o.max_iterations = float(self.tolerance), int(self.max_iterations)
        o.refine_interval, o.rows_per_block = int(self.refine_interval), int(self.rows_per_block)
        o.use_graph, o.verbose, o.time_spmm = int(self.use_graph), int(self.verbose), int(self.time_spmm)
        o.precision = int(self.precision)
        o.formulation = int(self.formulation)
        o.vector_aux = int(bool(self.vector_aux))
        o.reorder = int(bool(self.reorder))
        o.rb_samples = int(self.rb_samples)
        return o


@dataclasses.dataclass
class BatchInstance:
    mesh: Mesh
    params: MaxwellParams
    bc: BC
    ports: Sequence[WavePort]


def _batch_c(instances: Sequence[BatchInstance], keep: list):
    arr = (L.BatchInstanceC * len(instances))()
    for i, inst in enumerate(instances):
        arr[i].mesh = inst.mesh.handle
        arr[i].params = inst.params.to_c(keep)
        pec = _pec_of(inst.bc)
        keep.append(pec)
        arr[i].pec, arr[i].n_pec = L.ptr(pec, C.c_int32), pec.size
        pa = _ports_c(inst.ports, keep)
        keep.append(pa)
        arr[i].ports, arr[i].n_ports = C.cast(pa, C.POINTER(L.WavePortC)), len(inst.ports)
    return arr


def _stats(st: L.BatchStatsC) -> dict:
    return {k: getattr(st, k) for k, _ in L.BatchStatsC._fields_}


def _sparams_eigenmode_batched_local(instances: Sequence[BatchInstance], freqs, opts: Optional[BatchOptions]):
    """One process's batched eigenmode solve: (S[instance, F, P, P], stats)."""
    keep: list = []
    arr = _batch_c(instances, keep)
    f = np.ascontiguousarray(freqs, np.float64)
    P_ = len(instances[0].ports)
    S = np.empty((len(instances), f.size, P_, P_), np.complex128)
    st = L.BatchStatsC()
    oc = (opts or BatchOptions()).to_c()
    L.check(L.lib.efg_sparams_eigenmode_batched(arr, len(instances), L.ptr(f, C.c_double), f.size, C.byref(oc),
                                                L.ptr(S.view(np.float64), C.c_double), C.byref(st)),
            "sparams_eigenmode_batched")
    return S, _stats(st)


def sparams_eigenmode_batched(instances: Sequence[BatchInstance], freqs, opts: Optional[BatchOptions] = None,
                              shard: Optional[bool] = None):
    """S[instance, frequency, P, P] of many meshes x frequencies in one batched
    double-float solve (FP32 pipes, about 48 bits; convergence confirmed on
    an FP64-accurate true residual).  Returns (S, stats).

    Under a torch.distributed process group of several ranks the frequencies
    are sharded across the ranks (interleaved, every instance on every rank)
    and every rank returns the full S; stats describe this rank's share
    (stats["ranks"] = world size).  shard=False keeps the whole solve on
    this process."""
    f = np.ascontiguousarray(freqs, np.float64)
    if not _shard_wanted(shard):
        return _sparams_eigenmode_batched_local(instances, f, opts)
    from .replicas import sharded_sweep, world_info
    local_stats: dict = {}

    def solve(fl):
        S_, st_ = _sparams_eigenmode_batched_local(instances, fl, opts)
        local_stats.update(st_)
        return np.moveaxis(S_, 1, 0)  # frequency first for the gather

    S = np.moveaxis(sharded_sweep(solve, f), 0, 1)
    local_stats["ranks"] = world_info()[1]
    return np.ascontiguousarray(S), local_stats


class BatchSolver:
    """Resident batched solve: set-up once, `solve()` repeatedly."""

    def __init__(self, instances: Sequence[BatchInstance], freqs, opts: Optional[BatchOptions] = None):
        keep: list = []
        arr = _batch_c(instances, keep)
        self.freqs = np.ascontiguousarray(freqs, np.float64)
        self.n_inst = len(instances)
        self.P = len(instances[0].ports)
        self._h = C.c_void_p()
        oc = (opts or BatchOptions()).to_c()
        L.check(L.lib.efg_batch_create(arr, self.n_inst, L.ptr(self.freqs, C.c_double), self.freqs.size,
                                       C.byref(oc), C.byref(self._h)), "batch_create")
        rows, nnz = C.c_int64(), C.c_int64()
        rhs, rpc = C.c_int32(), C.c_int32()
        L.check(L.lib.efg_batch_info(self._h, C.byref(rows), C.byref(nnz), C.byref(rhs), C.byref(rpc)))
        self.rows, self.nnz, self.rhs, self.rows_per_chunk = rows.value, nnz.value, rhs.value, rpc.value

    def solve(self):
        S = np.empty((self.n_inst, self.freqs.size, self.P, self.P), np.complex128)
        st = L.BatchStatsC()
        L.check(L.lib.efg_batch_solve(self._h, L.ptr(S.view(np.float64), C.c_double), C.byref(st)), "batch_solve")
        return S, _stats(st)

    def rhs_stats(self):
        """Per (instance, frequency, active port) status, iterations and
        relative FP64 residual of the last solve (arrays [inst, F, P])."""
        n = self.n_inst * self.rhs
        stt = np.empty(n, np.int32)
        its = np.empty(n, np.int32)
        res = np.empty(n, np.float64)
        L.check(L.lib.efg_batch_rhs_stats(self._h, L.ptr(stt, C.c_int32), L.ptr(its, C.c_int32),
                                          L.ptr(res, C.c_double)))
        k = self.freqs.size * self.P
        shape = (self.n_inst, self.freqs.size, self.P)
        pick = lambda a: a.reshape(self.n_inst, self.rhs)[:, :k].reshape(shape)
        return pick(stt), pick(its), pick(res)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.lib.efg_batch_destroy(h)
            self._h = None


def sparams_eigenmode_adjoint(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort], out_j: int,
                              in_i: int, opts: Optional[SolveOptions] = None):
    """(d|S_ji|^2/d eps_r per tetrahedron, S)."""
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    pa = _ports_c(ports, keep)
    oc = opts.to_c() if opts is not None else None
    g = np.empty(mesh.num_tets, np.float64)
    S = np.empty((len(ports), len(ports)), np.complex128)
    L.check(L.lib.efg_sparams_eigenmode_adjoint(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size, pa,
                                                len(ports), int(out_j), int(in_i),
                                                C.byref(oc) if oc is not None else None, L.ptr(g, C.c_double),
                                                L.ptr(S.view(np.float64), C.c_double)), "sparams_eigenmode_adjoint")
    return g, S


def sparams_driven_adjoint(mesh: Mesh, p: MaxwellParams, bc: BC, ports: Sequence[WavePort], out_j: int,
                           in_i: int, opts: Optional[SolveOptions] = None):
    """(d|S_ji|^2/d eps_r per tetrahedron, S) for the driven ports of
    calculate_sparams (lumped or wave ports with real weights, w w^T / Z0
    port blocks, jk0 ABC, Debye media)."""
    keep: list = []
    pc = p.to_c(keep)
    pec = _pec_of(bc)
    pa = _ports_c(ports, keep)
    oc = opts.to_c() if opts is not None else None
    g = np.empty(mesh.num_tets, np.float64)
    S = np.empty((len(ports), len(ports)), np.complex128)
    L.check(L.lib.efg_sparams_driven_adjoint(mesh.handle, C.byref(pc), L.ptr(pec, C.c_int32), pec.size, pa,
                                             len(ports), int(out_j), int(in_i),
                                             C.byref(oc) if oc is not None else None, L.ptr(g, C.c_double),
                                             L.ptr(S.view(np.float64), C.c_double)), "sparams_driven_adjoint")
    return g, S


def element_matrices(xyz4) -> tuple:
    x = np.ascontiguousarray(xyz4, np.float64).reshape(12)
    K = np.empty(36)
    M = np.empty(36)
    L.check(L.lib.efg_element_matrices(L.ptr(x, C.c_double), L.ptr(K, C.c_double), L.ptr(M, C.c_double)))
    return K.reshape(6, 6), M.reshape(6, 6)


def triangle_mass(xyz3) -> np.ndarray:
    x = np.ascontiguousarray(xyz3, np.float64).reshape(9)
    M = np.empty(9)
    L.check(L.lib.efg_triangle_mass(L.ptr(x, C.c_double), L.ptr(M, C.c_double)))
    return M.reshape(3, 3)


def transfer_counters():
    """(host->device bytes, device->host bytes) copied by the library so far."""
    a, b = C.c_int64(), C.c_int64()
    L.lib.efg_transfer_counters(C.byref(a), C.byref(b))
    return a.value, b.value


def device_count() -> int:
    return int(L.lib.efg_device_count())
