"""CPU complex128 oracle for the EdgeFEM frequency-domain Maxwell path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: tests, the smoke
check and the CPU-baseline leg of the benchmark import it to compute the
answer the GPU path must reproduce.  It is never part of the product path.

It restates, in NumPy/SciPy with complex128 arithmetic and a SuperLU direct
solve, the reference algorithms of jman4162/EdgeFEM:

* global edge numbering and orientation      src/mesh_gmsh.cpp:104-147
* Whitney element matrices                   src/edge_basis.cpp:14-130
* volume assembly, ports, ABC, Dirichlet     src/assemble_maxwell.cpp:46-350
* w w^H port S-parameters, normalisation     src/assemble_maxwell.cpp:352-494
* eigenmode S-parameters                     src/assemble_maxwell.cpp:637-787
* 2D port mode, port surface mass            src/ports/wave_port.cpp:410-585
* analytic TE10 mode                         src/ports/port_eigensolve.cpp:45-65
* PEC edges                                  src/bc.cpp:47-80
* mesh quality report                        src/mesh_quality.cpp:10-83
* lumped port weights                        src/ports/lumped_port.cpp:21-160
* K/M split and frequency sweep              src/sweep.cpp:82-349
* Debye permittivity                         include/edgefem/materials/dispersive.hpp:62-66

Where the reference leaves something unspecified this oracle fixes it the
same way the GPU library does:

* Port-mode eigenvector sign (the reference inherits whatever sign its dense
  eigensolver returns, wave_port.cpp:509-513): the mode field integrated over
  the port face, sum_e w_e * integral(N_e dS), is made to have a positive
  component along the coordinate axis where that integral is largest.
* An evanescent port returns an all-NaN S matrix (the reference returns an
  uninitialised matrix, assemble_maxwell.cpp:687-697).

Per-tetrahedron material arrays (`eps_tet`) extend the reference's
per-region lookup (include/edgefem/maxwell.hpp:109-143); when given they
replace it.

The adjoint (`sparams_eigenmode_adjoint`) has no reference counterpart; it
differentiates the restated eigenmode S-parameters exactly, including the
dependence of the port propagation constant on the permittivity of the one
tetrahedron the reference reads it from (assemble_maxwell.cpp:670-684).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence

import numpy as np
import scipy.linalg
import scipy.sparse as sp
import scipy.sparse.linalg as spla

C0 = 299792458.0
MU0 = 4.0 * math.pi * 1e-7
EPS0 = 1.0 / (MU0 * C0 * C0)
ETA0_PORT = 376.730313668          # port_eigensolve.cpp:15

TET_PAIRS = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))   # mesh_gmsh.cpp:105-108
TRI_PAIRS = ((0, 1), (1, 2), (2, 0))                           # mesh_gmsh.cpp:109-111


# ------------------------------------------------------------------ topology

@dataclasses.dataclass
class Topology:
    edges: np.ndarray        # (n, 2) node ids, n0 < n1
    tet_edges: np.ndarray    # (T, 6) int
    tet_signs: np.ndarray    # (T, 6) +1/-1
    tri_edges: np.ndarray    # (S, 3)
    tri_signs: np.ndarray    # (S, 3)

    @property
    def n(self) -> int:
        return int(self.edges.shape[0])


def build_edges(tets: np.ndarray, tris: np.ndarray) -> Topology:
    """mesh_gmsh.cpp:104-147: number edges by first appearance scanning the
    tetrahedra (local pairs 01,02,03,12,13,23) then the triangles (01,12,20);
    orientation +1 iff the first local node id is the smaller."""
    index: Dict[tuple, int] = {}
    edges: List[tuple] = []
    T = tets.shape[0]
    tet_edges = np.empty((T, 6), np.int64)
    tet_signs = np.empty((T, 6), np.int64)
    tl = tets.tolist()
    for t in range(T):
        c = tl[t]
        for e, (p, q) in enumerate(TET_PAIRS):
            a, b = c[p], c[q]
            key = (a, b) if a < b else (b, a)
            idx = index.get(key)
            if idx is None:
                idx = len(edges)
                index[key] = idx
                edges.append(key)
            tet_edges[t, e] = idx
            tet_signs[t, e] = 1 if a < b else -1
    S = tris.shape[0]
    tri_edges = np.empty((S, 3), np.int64)
    tri_signs = np.empty((S, 3), np.int64)
    rl = tris.tolist()
    for s in range(S):
        c = rl[s]
        for e, (p, q) in enumerate(TRI_PAIRS):
            a, b = c[p], c[q]
            key = (a, b) if a < b else (b, a)
            idx = index.get(key)
            if idx is None:
                idx = len(edges)
                index[key] = idx
                edges.append(key)
            tri_edges[s, e] = idx
            tri_signs[s, e] = 1 if a < b else -1
    return Topology(np.array(edges, np.int64).reshape(-1, 2), tet_edges, tet_signs,
                    tri_edges, tri_signs)


def validate_mesh(node_ids: np.ndarray, xyz: np.ndarray, tets: np.ndarray):
    """mesh_quality.cpp:52-83 with tet_volume (:10-25) and tet_aspect_ratio
    (:27-50): per tet the signed volume (p1-p0).((p2-p0) x (p3-p0))/6 and
    the ratio of its longest to its shortest edge (+inf when the shortest
    is below machine epsilon); flags 1 degenerate (|vol| < 1e-15), 2
    inverted (vol < 0).  Returns (flags, num_degenerate, num_inverted,
    min_volume, max_aspect_ratio); elementwise float64 without fused
    operations, in the reference's order of operations."""
    lut = {int(v): i for i, v in enumerate(np.asarray(node_ids).tolist())}
    idx = np.vectorize(lut.__getitem__, otypes=[np.int64])(np.asarray(tets)) if len(tets) else np.zeros((0, 4), np.int64)
    P = np.asarray(xyz, np.float64)[idx]  # (T, 4, 3)
    u, v, w = P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]
    c0 = v[:, 1] * w[:, 2] - v[:, 2] * w[:, 1]
    c1 = v[:, 0] * w[:, 2] - v[:, 2] * w[:, 0]
    c2 = v[:, 0] * w[:, 1] - v[:, 1] * w[:, 0]
    vol = (u[:, 0] * c0 - u[:, 1] * c1 + u[:, 2] * c2) / 6.0
    L = np.empty((len(idx), 6))
    for k, (a, b) in enumerate(((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))):
        d = P[:, a] - P[:, b]
        L[:, k] = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    emin, emax = L.min(axis=1), L.max(axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        ar = np.where(emin < np.finfo(np.float64).eps, np.inf, emax / np.where(emin > 0, emin, 1.0))
    flags = np.where(np.abs(vol) < 1e-15, 1, np.where(vol < 0, 2, 0)).astype(np.int8)
    min_vol = float(vol.min()) if len(vol) else float(np.finfo(np.float64).max)
    max_ar = float(ar.max()) if len(ar) else 0.0
    return flags, int((flags == 1).sum()), int((flags == 2).sum()), min_vol, max_ar


def build_edge_pec(tri_edges: np.ndarray, tri_phys: np.ndarray, pec_tag: int) -> np.ndarray:
    """bc.cpp:47-80: sorted unique edges of triangles tagged `pec_tag`."""
    return np.unique(tri_edges[tri_phys == pec_tag].ravel())


# ------------------------------------------------------------ element kernels

def gradients_and_volume(X: np.ndarray):
    """edge_basis.cpp:14-26 for a batch X (T,4,3): B=[v0-v3,v1-v3,v2-v3],
    g_i = columns of B^{-T}, g3 = -(g0+g1+g2), V = |det B|/6."""
    B = np.stack([X[:, 0] - X[:, 3], X[:, 1] - X[:, 3], X[:, 2] - X[:, 3]], axis=2)  # columns
    BinvT = np.linalg.inv(B).transpose(0, 2, 1)
    g = np.empty((X.shape[0], 4, 3))
    g[:, 0] = BinvT[:, :, 0]
    g[:, 1] = BinvT[:, :, 1]
    g[:, 2] = BinvT[:, :, 2]
    g[:, 3] = -g[:, 0] - g[:, 1] - g[:, 2]
    V = np.abs(np.linalg.det(B)) / 6.0
    return g, V


def whitney_matrices(X: np.ndarray):
    """edge_basis.cpp:48-87: (T,6,6) curl-curl K_ij = V c_i.c_j with
    c = 2 g_a x g_b, and mass M_ij = sum of four g.g * lambda_int terms
    (lambda_int = V/10 on the diagonal, V/20 off it)."""
    g, V = gradients_and_volume(X)
    T = X.shape[0]
    curls = np.empty((T, 6, 3))
    for i, (a, b) in enumerate(TET_PAIRS):
        curls[:, i] = 2.0 * np.cross(g[:, a], g[:, b])
    K = V[:, None, None] * np.einsum("tik,tjk->tij", curls, curls)
    gg = np.einsum("tak,tbk->tab", g, g)  # (T,4,4)

    def li(p, q):
        return np.where(p == q, 0.1, 0.05)

    M = np.zeros((T, 6, 6))
    for i, (a, b) in enumerate(TET_PAIRS):
        for j, (c, d) in enumerate(TET_PAIRS):
            M[:, i, j] = V * (gg[:, b, d] * li(a, c) - gg[:, b, c] * li(a, d)
                              - gg[:, a, d] * li(b, c) + gg[:, a, c] * li(b, d))
    return K, M, V


def triangle_whitney_mass(v: np.ndarray) -> np.ndarray:
    """edge_basis.cpp:89-130 for a batch v (S,3,3): 3x3 edge mass with local
    edges (0,1),(1,2),(2,0), in-plane gradients g0 = n x (v2-v1)/2A etc.,
    integral(lambda_i lambda_j) = A/6 (i=j), A/12 (i!=j).  Degenerate
    triangles (2A < 1e-30) give zero."""
    normal = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    area2 = np.linalg.norm(normal, axis=1)
    ok = area2 >= 1e-30
    a2 = np.where(ok, area2, 1.0)
    nh = normal / a2[:, None]
    area = a2 / 2.0
    g = np.stack([np.cross(nh, v[:, 2] - v[:, 1]), np.cross(nh, v[:, 0] - v[:, 2]),
                  np.cross(nh, v[:, 1] - v[:, 0])], axis=1) / a2[:, None, None]
    gg = np.einsum("sak,sbk->sab", g, g)
    out = np.zeros((v.shape[0], 3, 3))
    for i, (a, b) in enumerate(TRI_PAIRS):
        for j, (c, d) in enumerate(TRI_PAIRS):
            def lam(p, q):
                return area / 6.0 if p == q else area / 12.0
            out[:, i, j] = (gg[:, b, d] * lam(a, c) - gg[:, b, c] * lam(a, d)
                            - gg[:, a, d] * lam(b, c) + gg[:, a, c] * lam(b, d))
    out[~ok] = 0.0
    return out


def triangle_surface_curls(v: np.ndarray):
    """wave_port.cpp:446-469: in-plane gradients and the constant surface
    curls 2 (g_a x g_b).n for the three local edges, plus areas."""
    normal = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    area2 = np.linalg.norm(normal, axis=1)
    ok = area2 >= 1e-30
    a2 = np.where(ok, area2, 1.0)
    nh = normal / a2[:, None]
    g = np.stack([np.cross(nh, v[:, 2] - v[:, 1]), np.cross(nh, v[:, 0] - v[:, 2]),
                  np.cross(nh, v[:, 1] - v[:, 0])], axis=1) / a2[:, None, None]
    curls = np.stack([2.0 * np.einsum("sk,sk->s", np.cross(g[:, a], g[:, b]), nh)
                      for (a, b) in TRI_PAIRS], axis=1)
    return g, curls, a2 / 2.0, ok


# ------------------------------------------------------------------- problem

@dataclasses.dataclass
class Problem:
    """Mesh arrays plus derived topology, PEC set and per-tet geometry."""
    xyz: np.ndarray
    node_lut: np.ndarray
    tets: np.ndarray
    tet_phys: np.ndarray
    tris: np.ndarray
    tri_phys: np.ndarray
    topo: Topology
    pec: np.ndarray
    Kloc: np.ndarray
    Mloc: np.ndarray
    vol: np.ndarray

    @property
    def n(self) -> int:
        return self.topo.n


def make_problem(mesh, pec_tag: int = 1) -> Problem:
    lut = np.full(int(mesh.node_ids.max()) + 1, -1, np.int64)
    lut[mesh.node_ids] = np.arange(mesh.node_ids.size)
    topo = build_edges(mesh.tets, mesh.tris)
    pec = build_edge_pec(topo.tri_edges, mesh.tri_phys, pec_tag)
    X = mesh.xyz[lut[mesh.tets]]
    K, M, V = whitney_matrices(X)
    return Problem(mesh.xyz, lut, mesh.tets, mesh.tet_phys, mesh.tris, mesh.tri_phys,
                   topo, pec, K, M, V)


def tet_eps(prob: Problem, omega: float, eps_r=1.0, eps_regions: Optional[dict] = None,
            eps_models: Optional[dict] = None, eps_tet: Optional[np.ndarray] = None) -> np.ndarray:
    """maxwell.hpp:109-119: dispersive model > region value > global."""
    if eps_tet is not None:
        return np.asarray(eps_tet, np.complex128)
    out = np.full(prob.tets.shape[0], complex(eps_r), np.complex128)
    for tag, val in (eps_regions or {}).items():
        out[prob.tet_phys == tag] = complex(val)
    for tag, model in (eps_models or {}).items():
        out[prob.tet_phys == tag] = model(omega)
    return out


def debye_eps(eps_s: float, eps_inf: float, tau: float):
    """dispersive.hpp:62-66: eps_inf + (eps_s - eps_inf)/(1 + j omega tau)."""
    def f(omega):
        return eps_inf + (eps_s - eps_inf) / complex(1.0, omega * tau)
    return f


def _scatter(prob: Problem, loc: np.ndarray) -> sp.csr_matrix:
    te, ts = prob.topo.tet_edges, prob.topo.tet_signs
    rows = np.repeat(te, 6, axis=1).ravel()
    cols = np.tile(te, (1, 6)).ravel()
    sgn = (ts[:, :, None] * ts[:, None, :]).reshape(-1)
    n = prob.n
    A = sp.coo_matrix((loc.reshape(-1) * sgn, (rows, cols)), shape=(n, n)).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return A


def pattern(prob: Problem) -> sp.csr_matrix:
    """Sparsity of the assembled matrix: all (gi, gj) pairs of each tet
    (setFromTriplets, assemble_maxwell.cpp:205-207) plus every diagonal
    (Dirichlet rows get diag 1, :344-347)."""
    te = prob.topo.tet_edges
    rows = np.concatenate([np.repeat(te, 6, axis=1).ravel(), np.arange(prob.n)])
    cols = np.concatenate([np.tile(te, (1, 6)).ravel(), np.arange(prob.n)])
    P = sp.coo_matrix((np.ones(rows.size), (rows, cols)), shape=(prob.n, prob.n)).tocsr()
    P.sum_duplicates()
    P.sort_indices()
    return P


def _on_pattern(P: sp.csr_matrix, A: sp.spmatrix) -> sp.csr_matrix:
    """Express A on pattern P (P must contain A's pattern); explicit zeros kept."""
    A = sp.csr_matrix(A)
    out = sp.csr_matrix((np.zeros(P.nnz, np.complex128), P.indices.copy(), P.indptr.copy()),
                        shape=P.shape)
    Acoo = A.tocoo()
    # locate each A entry in P
    pos = _slot_index(P, Acoo.row, Acoo.col)
    np.add.at(out.data, pos, Acoo.data)
    return out


def _slot_index(P: sp.csr_matrix, rows: np.ndarray, cols: np.ndarray) -> np.ndarray:
    """Position of each (row, col) in P's data array (row-major sorted keys)."""
    n = np.int64(P.shape[1])
    prow = np.repeat(np.arange(P.shape[0], dtype=np.int64), np.diff(P.indptr))
    pkey = prow * n + P.indices.astype(np.int64)
    key = rows.astype(np.int64) * n + cols.astype(np.int64)
    pos = np.searchsorted(pkey, key)
    if pos.size and (pos.max() >= pkey.size or np.any(pkey[pos] != key)):
        raise AssertionError("entry outside pattern")
    return pos


def assemble_km(prob: Problem, eps: np.ndarray, mu: Optional[np.ndarray] = None):
    """sweep.cpp:90-172 restated: K = sum K_loc/mu_r, M = sum eps_r M_loc
    (signed), both on the full pattern, Dirichlet: rows and columns zeroed,
    K diagonal 1, M diagonal 0."""
    mu = np.ones(prob.tets.shape[0], np.complex128) if mu is None else mu
    P = pattern(prob)
    K = _on_pattern(P, _scatter(prob, prob.Kloc / mu[:, None, None]))
    M = _on_pattern(P, _scatter(prob, prob.Mloc * eps[:, None, None]))
    for A, d in ((K, 1.0), (M, 0.0)):
        _apply_dirichlet(A, prob.pec, d)
    return K, M


def _apply_dirichlet(A: sp.csr_matrix, pec: np.ndarray, diag: complex) -> None:
    """assemble_maxwell.cpp:322-347: zero PEC rows and columns, keep the
    pattern, set the diagonal."""
    if pec.size == 0:
        return
    is_pec = np.zeros(A.shape[0], bool)
    is_pec[pec] = True
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    kill = is_pec[rows] | is_pec[A.indices]
    A.data[kill] = 0.0
    diag_mask = kill & (rows == A.indices) & is_pec[rows]
    A.data[diag_mask] = diag


def assemble_volume(prob: Problem, omega: float, eps: np.ndarray,
                    mu: Optional[np.ndarray] = None) -> sp.csr_matrix:
    """assemble_maxwell.cpp:114-207: A = sum (K_loc/mu_r - k0^2 eps_r M_loc) s_i s_j,
    no Dirichlet yet."""
    k0 = omega / C0
    mu = np.ones(prob.tets.shape[0], np.complex128) if mu is None else mu
    loc = prob.Kloc / mu[:, None, None] - (k0 * k0) * eps[:, None, None] * prob.Mloc
    return _on_pattern(pattern(prob), _scatter(prob, loc))


# ---------------------------------------------------------------------- ports

@dataclasses.dataclass
class WavePort:
    surface_tag: int
    edges: np.ndarray          # global edge ids (sorted, incl. PEC edges)
    weights: np.ndarray        # complex weights aligned with `edges`
    kc: float = 0.0
    Z0: complex = 0.0
    beta: complex = 0.0
    fc: float = 0.0


def solve_te10_mode(a: float, freq: float) -> dict:
    """port_eigensolve.cpp:45-65."""
    k = 2 * math.pi * freq / C0
    kc = math.pi / a
    beta = math.sqrt(max(0.0, k * k - kc * kc))
    return dict(fc=C0 / (2 * a), kc=kc, beta=beta, Z0=(ETA0_PORT * k / beta) if beta > 0 else 0.0)


def _tri_xyz(prob: Problem, sel: np.ndarray) -> np.ndarray:
    return prob.xyz[prob.node_lut[prob.tris[sel]]]


def port_mode_sign(prob: Problem, surface_tag: int, v_full: np.ndarray) -> float:
    """Sign convention: +1 or -1 so that integral of the mode field over the
    port face has a positive component on its dominant axis.  integral of
    N_e over a flat triangle = (A/3)(g_b - g_a) (lumped_port.cpp:86-87)."""
    sel = np.nonzero(prob.tri_phys == surface_tag)[0]
    v = _tri_xyz(prob, sel)
    g, _, area, ok = triangle_surface_curls(v)
    E = np.zeros(3)
    for le, (a, b) in enumerate(TRI_PAIRS):
        w = v_full[prob.topo.tri_edges[sel, le]] * prob.topo.tri_signs[sel, le] * ok
        E += np.einsum("s,sk->k", w * area / 3.0, g[:, b] - g[:, a])
    ax = int(np.argmax(np.abs(E)))
    return -1.0 if E[ax] < 0 else 1.0


def solve_port_mode_2d(prob: Problem, surface_tag: int, target_kc_sq: float):
    """wave_port.cpp:410-514: dense generalized eigenproblem K_s e = kc^2 M_s e
    on the free (non-PEC) port edges, eigenvalue closest to target with
    kc^2 >= 1e-6 max(target, 1).  Returns (v_full real (n,), kc_sq)."""
    is_pec = np.zeros(prob.n, bool)
    is_pec[prob.pec] = True
    sel = np.nonzero(prob.tri_phys == surface_tag)[0]
    local: Dict[int, int] = {}
    order: List[int] = []
    for s in sel.tolist():
        for le in range(3):
            ge = int(prob.topo.tri_edges[s, le])
            if is_pec[ge] or ge in local:
                continue
            local[ge] = len(order)
            order.append(ge)
    m = len(order)
    v_full = np.zeros(prob.n)
    if m == 0:
        return v_full, 0.0
    v = _tri_xyz(prob, sel)
    Mt = triangle_whitney_mass(v)
    _, curls, area, ok = triangle_surface_curls(v)
    K = np.zeros((m, m))
    M = np.zeros((m, m))
    for k, s in enumerate(sel.tolist()):
        if not ok[k]:
            continue
        for i in range(3):
            gi = int(prob.topo.tri_edges[s, i])
            if gi not in local:
                continue
            for j in range(3):
                gj = int(prob.topo.tri_edges[s, j])
                if gj not in local:
                    continue
                sg = prob.topo.tri_signs[s, i] * prob.topo.tri_signs[s, j]
                K[local[gi], local[gj]] += sg * curls[k, i] * curls[k, j] * area[k]
                M[local[gi], local[gj]] += sg * Mt[k, i, j]
    w, V = scipy.linalg.eigh(K, M)
    kc_min = 1e-6 * max(target_kc_sq, 1.0)
    best, best_d = -1, np.inf
    for i in range(m):
        if w[i] < kc_min:
            continue
        d = abs(w[i] - target_kc_sq)
        if d < best_d:
            best, best_d = i, d
    if best < 0:
        return v_full, 0.0
    v_full[np.array(order)] = V[:, best]
    v_full *= port_mode_sign(prob, surface_tag, v_full)
    return v_full, float(w[best])


def build_wave_port_2d(prob: Problem, surface_tag: int, mode: dict, target_kc_sq: float) -> WavePort:
    """wave_port.cpp:516-546: weights = discrete mode on the sorted set of
    all port-face edges (PEC edges carry weight 0); kc := sqrt(discrete kc^2)."""
    vf, kc_sq = solve_port_mode_2d(prob, surface_tag, target_kc_sq)
    kc = math.sqrt(kc_sq) if kc_sq > 0 else mode["kc"]
    sel = prob.tri_phys == surface_tag
    edges = np.unique(prob.topo.tri_edges[sel].ravel())
    return WavePort(surface_tag, edges, vf[edges].astype(np.complex128), kc=kc,
                    Z0=mode["Z0"], beta=mode["beta"], fc=mode["fc"])


def assemble_port_surface_mass(prob: Problem, surface_tag: int) -> sp.csr_matrix:
    """wave_port.cpp:548-585: signed triangle mass on the port face, PEC rows
    and columns omitted, global indexing, real."""
    is_pec = np.zeros(prob.n, bool)
    is_pec[prob.pec] = True
    sel = np.nonzero(prob.tri_phys == surface_tag)[0]
    Mt = triangle_whitney_mass(_tri_xyz(prob, sel))
    te = prob.topo.tri_edges[sel]
    ts = prob.topo.tri_signs[sel]
    rows = np.repeat(te, 3, axis=1).ravel()
    cols = np.tile(te, (1, 3)).ravel()
    vals = (Mt * ts[:, :, None] * ts[:, None, :]).ravel()
    keep = ~(is_pec[rows] | is_pec[cols])
    Ms = sp.coo_matrix((vals[keep], (rows[keep], cols[keep])), shape=(prob.n, prob.n)).tocsr()
    Ms.sum_duplicates()
    return Ms


def port_beta_tet(prob: Problem, surface_tag: int) -> int:
    """assemble_maxwell.cpp:660-684: index of the first tet (in mesh order)
    with a face on the port surface, or -1."""
    faces = set(tuple(sorted(f)) for f in prob.tris[prob.tri_phys == surface_tag].tolist())
    for t, c in enumerate(prob.tets.tolist()):
        for tf in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
            if tuple(sorted((c[tf[0]], c[tf[1]], c[tf[2]]))) in faces:
                return t
    return -1


# --------------------------------------------------------- eigenmode S-params

@dataclasses.dataclass
class EigenmodeSystem:
    A: sp.csr_matrix               # full system incl. j alpha beta M_s terms
    B: np.ndarray                  # (n, P) right-hand sides
    C: np.ndarray                  # (n, P) overlap vectors c_j = M_s,j e_j
    betas: np.ndarray
    beta_tets: List[int]
    Ms: List[sp.csr_matrix]
    e: List[np.ndarray]
    eps: np.ndarray
    evanescent: bool = False


def eigenmode_system(prob: Problem, omega: float, ports: Sequence[WavePort], eps: np.ndarray,
                     mu: Optional[np.ndarray] = None, port_abc_scale: float = 1.0) -> EigenmodeSystem:
    """assemble_maxwell.cpp:637-752 (one assembly shared by both active ports,
    which the reference rebuilds identically per port)."""
    mu = np.ones(prob.tets.shape[0], np.complex128) if mu is None else mu
    k0 = omega / C0
    P = len(ports)
    betas = np.zeros(P, np.complex128)
    btets = []
    evan = False
    for i, pt in enumerate(ports):
        t = port_beta_tet(prob, pt.surface_tag)
        btets.append(t)
        em = eps[t] * mu[t] if t >= 0 else 1.0 + 0j
        bsq = em * k0 * k0 - pt.kc * pt.kc
        if bsq.real <= 0:
            evan = True
        betas[i] = np.sqrt(bsq)
    A = assemble_volume(prob, omega, eps, mu)
    _apply_dirichlet(A, prob.pec, 1.0)
    Ms = [assemble_port_surface_mass(prob, pt.surface_tag) for pt in ports]
    es = []
    is_pec = np.zeros(prob.n, bool)
    is_pec[prob.pec] = True
    for i, pt in enumerate(ports):
        e = np.zeros(prob.n, np.complex128)
        keep = ~is_pec[pt.edges]
        e[pt.edges[keep]] = pt.weights[keep]
        nsq = np.real(np.vdot(e, Ms[i] @ e))
        if nsq > 1e-30:
            e = e / math.sqrt(nsq)
        es.append(e)
    Aport = sp.csr_matrix(A.shape, dtype=np.complex128)
    for i in range(P):
        Aport = Aport + (1j * port_abc_scale * betas[i]) * Ms[i]
    A = _on_pattern(pattern(prob), A + Aport)
    C = np.stack([Ms[i] @ es[i] for i in range(P)], axis=1)
    B = np.stack([2.0 * (1j * port_abc_scale * betas[i]) * C[:, i] for i in range(P)], axis=1)
    return EigenmodeSystem(A, B, C, betas, btets, Ms, es, eps, evan)


class EigenmodeSweep:
    """eigenmode_system at many frequencies from one K/M assembly: the
    reference's sweep split A(omega) = K - k0^2 M (src/sweep.cpp:82-172) with
    the eigenmode port terms j alpha beta_p(omega) M_s,p added per frequency
    (assemble_maxwell.cpp:637-752).  Frequency-independent permittivity
    only.  Equal to eigenmode_system up to the rounding of the split."""

    def __init__(self, prob: Problem, ports: Sequence[WavePort], eps: np.ndarray,
                 port_abc_scale: float = 1.0):
        self.prob, self.ports, self.eps, self.alpha = prob, list(ports), np.asarray(eps, np.complex128), port_abc_scale
        self.P = pattern(prob)
        self.K, self.M = assemble_km(prob, self.eps)
        self.beta_tets = [port_beta_tet(prob, pt.surface_tag) for pt in self.ports]
        is_pec = np.zeros(prob.n, bool)
        is_pec[prob.pec] = True
        self.Ms, self.Ms_on, self.e = [], [], []
        for pt in self.ports:
            Msp = assemble_port_surface_mass(prob, pt.surface_tag)
            e = np.zeros(prob.n, np.complex128)
            keep = ~is_pec[pt.edges]
            e[pt.edges[keep]] = pt.weights[keep]
            nsq = np.real(np.vdot(e, Msp @ e))
            if nsq > 1e-30:
                e = e / math.sqrt(nsq)
            self.Ms.append(Msp)
            self.Ms_on.append(_on_pattern(self.P, Msp).data)
            self.e.append(e)
        self.C = np.stack([self.Ms[i] @ self.e[i] for i in range(len(self.ports))], axis=1)

    def system(self, omega: float) -> EigenmodeSystem:
        k0 = omega / C0
        P = len(self.ports)
        betas = np.zeros(P, np.complex128)
        evan = False
        for i, t in enumerate(self.beta_tets):
            em = self.eps[t] if t >= 0 else 1.0 + 0j
            bsq = em * k0 * k0 - self.ports[i].kc ** 2
            evan |= bool(bsq.real <= 0)
            betas[i] = np.sqrt(bsq)
        data = self.K.data - (k0 * k0) * self.M.data
        for i in range(P):
            data = data + (1j * self.alpha * betas[i]) * self.Ms_on[i]
        A = sp.csr_matrix((data, self.K.indices, self.K.indptr), shape=self.K.shape)
        B = np.stack([2.0 * (1j * self.alpha * betas[i]) * self.C[:, i] for i in range(P)], axis=1)
        return EigenmodeSystem(A, B, self.C, betas, self.beta_tets, self.Ms, self.e, self.eps, evan)


def sparams_from_solution(sys_: EigenmodeSystem, X: np.ndarray) -> np.ndarray:
    """assemble_maxwell.cpp:771-783: S(j,a) = e_j^H M_s,j x_a - delta."""
    P = X.shape[1]
    S = np.empty((P, P), np.complex128)
    for a in range(P):
        for j in range(P):
            S[j, a] = np.vdot(sys_.e[j], sys_.Ms[j] @ X[:, a]) - (1.0 if j == a else 0.0)
    return S


def calculate_sparams_eigenmode(prob: Problem, omega: float, ports: Sequence[WavePort],
                                eps: np.ndarray, mu: Optional[np.ndarray] = None,
                                port_abc_scale: float = 1.0, return_solution: bool = False,
                                iterative_tol: Optional[float] = None, threads: int = 0):
    """Complex128 restatement of calculate_sparams_eigenmode: SuperLU direct
    solve, or with `iterative_tol` complex128 COCG with the auxiliary-space
    preconditioner to that relative residual (for systems whose direct
    factorisation is too slow on the CPU)."""
    sys_ = eigenmode_system(prob, omega, ports, eps, mu, port_abc_scale)
    P = len(ports)
    if sys_.evanescent:
        S = np.full((P, P), np.nan + 1j * np.nan)
        return (S, None, sys_) if return_solution else S
    if iterative_tol is None:
        X = spla.splu(sys_.A.tocsc()).solve(sys_.B)
    else:
        A = sys_.A.tocsr()
        inc = aux_incidence(prob)
        X = np.column_stack([cocg_aux_c(prob, A, sys_.B[:, k], tol=iterative_tol, inc=inc, threads=threads)["x"]
                             for k in range(sys_.B.shape[1])])
    S = sparams_from_solution(sys_, X)
    return (S, X, sys_) if return_solution else S


def waveguide_ports(prob: Problem, a: float, freq: float, tags=(2, 3)) -> List[WavePort]:
    """The port set-up of RectWaveguideDesign._setup_ports (waveguide.py:255-286)."""
    mode = solve_te10_mode(a, freq)
    kc_sq = (math.pi / a) ** 2
    return [build_wave_port_2d(prob, t, mode, kc_sq) for t in tags]


# ------------------------------------------------------------------- adjoint

def sparams_eigenmode_adjoint(prob: Problem, omega: float, ports: Sequence[WavePort],
                              eps: np.ndarray, out_j: int, in_i: int, iterative_tol: Optional[float] = None,
                              threads: int = 0):
    """Exact d|S_ji|^2 / d eps_e for real per-tet permittivity (mu = 1).

    S_ji = c_j^T x_i - delta, A x_i = b_i, A = A^T.  The adjoint vector
    lambda_j = A^{-1} c_j equals x_j / (2 j alpha beta_j) because
    b_j = 2 j alpha beta_j c_j.  Volume term: dA/deps_e = -k0^2 (signed M_loc,e).
    Port term: beta_p depends on eps of tet t_p, entering A (j alpha beta_p M_s,p)
    and b_p.  Returns (grad (T,), S); `iterative_tol` as in
    calculate_sparams_eigenmode."""
    S, X, sys_ = calculate_sparams_eigenmode(prob, omega, ports, eps, return_solution=True,
                                             iterative_tol=iterative_tol, threads=threads)
    k0 = omega / C0
    alpha = 1.0
    lam = X[:, out_j] / (2j * alpha * sys_.betas[out_j])
    xi = X[:, in_i]
    te, ts = prob.topo.tet_edges, prob.topo.tet_signs
    xl = xi[te] * ts
    ll = lam[te] * ts
    # dS/deps_e = -lam^T dA x = k0^2 lam_loc^T M_loc x_loc
    dS = (k0 * k0) * np.einsum("ti,tij,tj->t", ll, prob.Mloc, xl)
    for p, t in enumerate(sys_.beta_tets):
        if t < 0:
            continue
        dbeta = (k0 * k0) / (2.0 * sys_.betas[p])
        dA_x = (1j * alpha * dbeta) * (sys_.Ms[p] @ xi)
        term = -lam @ dA_x
        if p == in_i:
            term += lam @ ((2j * alpha * dbeta) * sys_.C[:, p])
        dS[t] += term
    Sji = S[out_j, in_i]
    grad = 2.0 * np.real(np.conj(Sji) * dS)
    return grad, S


# ------------------------------------------------ CPU iterative restatement

def aux_preconditioner(prob: Problem, A: sp.csr_matrix, vector: bool = False, omega: float = 0.5):
    """z = D^-1 r + G Dn^-1 G^T r: Jacobi plus Jacobi on the nodal gradient
    space (G = edge-node incidence with PEC rows removed, Dn = diag(G^T A G)),
    the preconditioner of the GPU solves, restated for the CPU baseline.
    With `vector`, also + omega Pi Dp^-1 Pi^T r on the vector-nodal space
    (Pi[e, (n, d)] = (x_head - x_tail)_d / 2 for both end nodes n of e,
    Dp = diag(Pi^T A Pi))."""
    n = prob.n
    e = prob.topo.edges
    i0 = prob.node_lut[e[:, 0]]
    i1 = prob.node_lut[e[:, 1]]
    keep = np.ones(n, bool)
    keep[prob.pec] = False
    rows = np.concatenate([np.arange(n)[keep]] * 2)
    cols = np.concatenate([i0[keep], i1[keep]])
    vals = np.concatenate([-np.ones(keep.sum()), np.ones(keep.sum())])
    G = sp.csr_matrix((vals, (rows, cols)), shape=(n, prob.xyz.shape[0]))
    GT = G.T.tocsr()
    dn = (GT @ A @ G).diagonal()
    mx = np.abs(dn).max()
    dninv = np.where(np.abs(dn) > 1e-12 * mx, 1.0 / np.where(dn == 0, 1, dn), 0.0)
    dinv = 1.0 / A.diagonal()
    dinv[~np.isfinite(dinv)] = 1.0
    if not vector:
        def apply(r):
            return dinv * r + G @ (dninv * (GT @ r))
        return apply
    nn = prob.xyz.shape[0]
    t = prob.xyz[i1] - prob.xyz[i0]
    prow, pcol, pval = [], [], []
    for d in range(3):
        for nd in (i0, i1):
            prow.append(np.arange(n)[keep])
            pcol.append(d * nn + nd[keep])
            pval.append(0.5 * t[keep, d])
    Pi = sp.csr_matrix((np.concatenate(pval), (np.concatenate(prow), np.concatenate(pcol))), shape=(n, 3 * nn))
    PiT = Pi.T.tocsr()
    dp = (PiT @ A @ Pi).diagonal()
    mp = np.abs(dp).max()
    dpinv = np.where(np.abs(dp) > 1e-12 * mp, omega / np.where(dp == 0, 1, dp), 0.0)

    def apply_v(r):
        return dinv * r + G @ (dninv * (GT @ r)) + Pi @ (dpinv * (PiT @ r))
    return apply_v


def cocg_jacobi(A: sp.csr_matrix, b: np.ndarray, tol: float = 1e-8, maxit: int = 100000,
                max_seconds: Optional[float] = None, prec=None):
    """Preconditioned COCG in complex128 on the CPU (Jacobi unless `prec`,
    e.g. aux_preconditioner, is given): the algorithm of the plain GPU path,
    restated for timing the CPU baseline.  Returns (x, iterations, relative
    residual, seconds per iteration).  With `max_seconds` it stops after that
    much wall time (a bounded sample)."""
    import time
    dinv = 1.0 / A.diagonal()
    dinv[~np.isfinite(dinv)] = 1.0
    if prec is None:
        def prec(v):
            return dinv * v
    x = np.zeros_like(b)
    r = b.copy()
    z = prec(r)
    p = z.copy()
    rho = r @ z
    nb = np.linalg.norm(b)
    t0 = time.perf_counter()
    it = 0
    rel = 1.0
    while it < maxit:
        q = A @ p
        alpha = rho / (p @ q)
        x += alpha * p
        r -= alpha * q
        it += 1
        rel = np.linalg.norm(r) / nb if nb > 0 else 0.0
        if rel < tol:
            break
        if max_seconds is not None and time.perf_counter() - t0 > max_seconds:
            break
        z = prec(r)
        rho_new = r @ z
        p = z + (rho_new / rho) * p
        rho = rho_new
    dt = time.perf_counter() - t0
    return x, it, rel, dt / max(it, 1)


# ----------------------------------------- C restatement of the COCG above

_CLIB = None


def _c_lib():
    """oracle/_build/liboracle_krylov.so (oracle/krylov_c.c), built on first
    use when absent."""
    global _CLIB
    if _CLIB is None:
        import ctypes as C
        import importlib.util
        import os
        here = os.path.dirname(os.path.abspath(__file__))
        spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(here, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        lib = C.CDLL(str(mod.build()))
        vp, i32, f64 = C.c_void_p, C.c_int, C.c_double
        lib.oracle_cocg_aux.restype = i32
        lib.oracle_cocg_aux.argtypes = [i32, vp, vp, vp, i32, vp, vp, vp, vp, vp, i32, f64, vp, vp, f64, f64, i32,
                                        i32, vp, vp, vp, vp, vp]
        lib.oracle_csr_matvec.restype = None
        lib.oracle_csr_matvec.argtypes = [i32, vp, vp, vp, vp, vp, i32]
        lib.oracle_max_threads.restype = i32
        _CLIB = lib
    return _CLIB


@dataclasses.dataclass
class AuxIncidence:
    """Edge-node incidence of the auxiliary spaces (aux_preconditioner):
    per edge its (tail, head) node index, -1 for PEC edges; per edge
    (x_head - x_tail)/2; per node its incident non-PEC edges in increasing
    order with sign -1 at the tail, +1 at the head."""
    enodes: np.ndarray
    piw: np.ndarray
    nptr: np.ndarray
    nedge: np.ndarray
    nsign: np.ndarray
    nn: int


def aux_incidence(prob: Problem) -> AuxIncidence:
    n = prob.n
    nn = prob.xyz.shape[0]
    i0 = prob.node_lut[prob.topo.edges[:, 0]]
    i1 = prob.node_lut[prob.topo.edges[:, 1]]
    keep = np.ones(n, bool)
    keep[prob.pec] = False
    enodes = np.stack([np.where(keep, i0, -1), np.where(keep, i1, -1)], 1).astype(np.int32)
    piw = np.where(keep[:, None], 0.5 * (prob.xyz[i1] - prob.xyz[i0]), 0.0)
    e = np.flatnonzero(keep)
    node = np.concatenate([i0[e], i1[e]])
    edge = np.concatenate([e, e])
    sign = np.concatenate([-np.ones(e.size, np.int8), np.ones(e.size, np.int8)])
    order = np.lexsort((edge, node))
    nptr = np.zeros(nn + 1, np.int32)
    np.add.at(nptr, node + 1, 1)
    return AuxIncidence(enodes.ravel(), np.ascontiguousarray(piw.ravel()), np.cumsum(nptr).astype(np.int32),
                        edge[order].astype(np.int32), sign[order], nn)


def cocg_aux_c(prob: Optional[Problem], A: sp.csr_matrix, b: np.ndarray, tol: float = 1e-8,
               maxit: int = 10 ** 6, level: int = 2, omega: float = 0.5, threads: int = 0,
               tol1: float = 0.0, inc: Optional[AuxIncidence] = None) -> dict:
    """cocg_jacobi with aux_preconditioner(prob, A, vector=level > 1, omega)
    (level 0: Jacobi alone), in C with OpenMP (krylov_c.c).  Returns a dict
    with x, iterations, relative residual, seconds (set-up included) and,
    when tol1 > 0, the iterations and seconds at which |r|/|b| first fell
    below tol1.  threads = 0 uses OpenMP's default."""
    import ctypes as C
    lib = _c_lib()
    A = sp.csr_matrix(A)
    n = A.shape[0]
    rp = np.ascontiguousarray(A.indptr, np.int64)
    ci = np.ascontiguousarray(A.indices, np.int32)
    va = np.ascontiguousarray(A.data, np.complex128)
    bb = np.ascontiguousarray(b, np.complex128)
    x = np.zeros(n, np.complex128)
    if level > 0 and inc is None:
        inc = aux_incidence(prob)
    it, rel, sec, it1, sec1 = C.c_int(), C.c_double(), C.c_double(), C.c_int(), C.c_double()

    def p(a):
        return None if a is None else a.ctypes.data_as(C.c_void_p)

    rc = lib.oracle_cocg_aux(n, p(rp), p(ci), p(va), inc.nn if level > 0 else 0,
                             p(inc.enodes) if level > 0 else None, p(inc.piw) if level > 0 else None,
                             p(inc.nptr) if level > 0 else None, p(inc.nedge) if level > 0 else None,
                             p(inc.nsign) if level > 0 else None, int(level), float(omega), p(bb), p(x),
                             float(tol1), float(tol), int(maxit), int(threads), C.byref(it), C.byref(rel),
                             C.byref(sec), C.byref(it1), C.byref(sec1))
    if rc < 0:
        raise RuntimeError("oracle_cocg_aux: bad arguments or out of memory")
    return {"x": x, "converged": rc == 0, "iterations": it.value, "relres": rel.value, "seconds": sec.value,
            "iterations_tol1": it1.value if tol1 > 0 else None, "seconds_tol1": sec1.value if tol1 > 0 else None,
            "threads": threads if threads > 0 else int(lib.oracle_max_threads())}


def csr_matvec_c(A: sp.csr_matrix, x: np.ndarray, threads: int = 0) -> np.ndarray:
    """A @ x in C (complex128, OpenMP over rows)."""
    import ctypes as C
    lib = _c_lib()
    A = sp.csr_matrix(A)
    rp = np.ascontiguousarray(A.indptr, np.int64)
    ci = np.ascontiguousarray(A.indices, np.int32)
    va = np.ascontiguousarray(A.data, np.complex128)
    xx = np.ascontiguousarray(x, np.complex128)
    y = np.empty(A.shape[0], np.complex128)
    lib.oracle_csr_matvec(A.shape[0], rp.ctypes.data_as(C.c_void_p), ci.ctypes.data_as(C.c_void_p),
                          va.ctypes.data_as(C.c_void_p), xx.ctypes.data_as(C.c_void_p),
                          y.ctypes.data_as(C.c_void_p), int(threads))
    return y


# -------------------------------------------------- w w^H (lumped) port path

# Constants of the port-ABC coefficients (assemble_maxwell.cpp:36-44).
MU0_ABC = 4.0 * math.pi * 1e-7
EPS0_ABC = 1.0 / (MU0_ABC * C0 * C0)
ETA0_ABC = MU0_ABC * C0


def port_abc_coeff(omega: float, kc: float, z0, abc_type: int):
    """assemble_maxwell.cpp:274-313: diagonal coefficient of the legacy port
    ABC (types 1 Beta j beta, 2 BetaNorm j beta/k0, 3 ImpedanceMatch
    j beta sqrt(Z0/eta0), 4 ModalAdmittance j omega eps0/Z0); None when the
    mode is cut off or the type is 0."""
    k0 = omega / C0
    bsq = k0 * k0 - kc * kc
    if abc_type == 0 or bsq <= 0:
        return None
    beta = math.sqrt(bsq)
    z = float(np.real(z0))
    return {1: 1j * beta, 2: 1j * beta / k0, 3: 1j * beta * math.sqrt(z / ETA0_ABC),
            4: 1j * omega * EPS0_ABC / z}[abc_type]


def assemble_maxwell(prob: Problem, omega: float, eps: np.ndarray, ports: Sequence[WavePort] = (),
                     active: int = -1, use_abc: bool = False, abc_tags: Sequence[int] = (),
                     mu: Optional[np.ndarray] = None, use_port_abc: bool = False, port_abc_type: int = 1):
    """assemble_maxwell.cpp:46-350 without PML: volume + w w^H/Z0 port blocks
    + 2w/sqrt(Z0) source + jk0 ABC diagonal + legacy port-ABC diagonal
    (use_port_abc) + Dirichlet.  Returns (A on a pattern that includes the
    port blocks, b)."""
    n = prob.n
    A = assemble_volume(prob, omega, eps, mu)
    is_pec = np.zeros(n, bool)
    is_pec[prob.pec] = True
    b = np.zeros(n, np.complex128)
    extra = []
    for i, pt in enumerate(ports):
        if pt.Z0 == 0:
            continue
        keep = ~is_pec[pt.edges]
        ed = pt.edges[keep]
        w = pt.weights[keep]
        blk = np.outer(w, np.conj(w)) / pt.Z0
        extra.append(sp.coo_matrix((blk.ravel(), (np.repeat(ed, ed.size), np.tile(ed, ed.size))),
                                   shape=(n, n)))
        if i == active:
            b[ed] += (2.0 / np.sqrt(complex(pt.Z0))) * w
    if use_abc:
        sel = np.ones(prob.tris.shape[0], bool) if not abc_tags else np.isin(prob.tri_phys, abc_tags)
        ab = np.unique(prob.topo.tri_edges[sel].ravel())
        ab = ab[~is_pec[ab]]
        extra.append(sp.coo_matrix((np.full(ab.size, 1j * omega / C0), (ab, ab)), shape=(n, n)))
    if use_port_abc:
        for pt in ports:
            if pt.Z0 == 0:
                continue
            c = port_abc_coeff(omega, pt.kc, pt.Z0, port_abc_type)
            if c is None:
                continue
            ed = pt.edges[~is_pec[pt.edges]]
            extra.append(sp.coo_matrix((np.full(ed.size, c), (ed, ed)), shape=(n, n)))
    if extra:
        Aall = A + sum(e.tocsr() for e in extra)
        P = pattern(prob)
        Pall = (P + sp.csr_matrix((np.ones(Aall.nnz), Aall.tocsr().indices, Aall.tocsr().indptr),
                                  shape=(n, n))).tocsr()
        Pall.sort_indices()
        A = _on_pattern(Pall, Aall)
    _apply_dirichlet(A, prob.pec, 1.0)
    b[is_pec] = 0.0
    return A, b


def calculate_sparams(prob: Problem, omega: float, eps: np.ndarray, ports: Sequence[WavePort],
                      use_abc=False, abc_tags=()):
    """assemble_maxwell.cpp:352-394 (direct solve)."""
    P = len(ports)
    S = np.empty((P, P), np.complex128)
    is_pec = np.zeros(prob.n, bool)
    is_pec[prob.pec] = True
    for i in range(P):
        A, b = assemble_maxwell(prob, omega, eps, ports, i, use_abc, abc_tags)
        x = spla.spsolve(A.tocsc(), b)
        vinc = np.sqrt(complex(ports[i].Z0))
        for j in range(P):
            keep = ~is_pec[ports[j].edges]
            Vj = np.sum(np.conj(ports[j].weights[keep]) * x[ports[j].edges[keep]])
            S[j, i] = (Vj - vinc) / vinc if i == j else Vj / vinc
    return S


def sparams_driven_adjoint(prob: Problem, omega: float, eps: np.ndarray, ports: Sequence[WavePort],
                           out_j: int, in_i: int, use_abc=False, abc_tags=(),
                           iterative_tol: Optional[float] = None, threads: int = 0):
    """Exact d|S_ji|^2 / d eps_t (real change of each tetrahedron's relative
    permittivity) of the driven-port S-parameters of calculate_sparams
    (assemble_maxwell.cpp:352-394): S_ji = (c_j^T x - delta_ji sqrt(Z0_i)) /
    sqrt(Z0_i), A x = b_i, c_j = conj(w_j) on the non-PEC port edges.  The
    adjoint system A^T lambda = c_j is solved as it stands (no symmetry
    assumed); dA/deps_t = -k0^2 (signed M_loc,t), the only term that depends
    on eps.  With `iterative_tol` both systems are solved by the C COCG with
    the auxiliary-space preconditioner to that relative residual instead of
    SuperLU; COCG needs a complex-symmetric matrix (real port weights, as
    normalised lumped ports have), and is given A^T as it stands.  Returns
    (grad (T,), S_ji)."""
    A, b = assemble_maxwell(prob, omega, eps, ports, in_i, use_abc, abc_tags)
    inc = aux_incidence(prob) if iterative_tol is not None else None

    def solve(M, rhs):
        if iterative_tol is None:
            return spla.spsolve(M.tocsc(), rhs)
        return cocg_aux_c(prob, M.tocsr(), rhs, tol=iterative_tol, threads=threads, inc=inc)["x"]

    x = solve(A, b)
    is_pec = np.zeros(prob.n, bool)
    is_pec[prob.pec] = True
    pj = ports[out_j]
    keep = ~is_pec[pj.edges]
    c = np.zeros(prob.n, np.complex128)
    np.add.at(c, pj.edges[keep], np.conj(pj.weights[keep]))
    vinc = np.sqrt(complex(ports[in_i].Z0))
    Sji = (c @ x - (vinc if out_j == in_i else 0.0)) / vinc
    lam = solve(A.T, c)
    k0 = omega / C0
    te, ts = prob.topo.tet_edges, prob.topo.tet_signs
    dS = (k0 * k0 / vinc) * np.einsum("ti,tij,tj->t", lam[te] * ts, prob.Mloc, x[te] * ts)
    return 2.0 * np.real(np.conj(Sji) * dS), Sji


def normalize_port_weights(prob: Problem, omega: float, eps: np.ndarray, ports: List[WavePort],
                           use_abc=False, abc_tags=()) -> List[WavePort]:
    """assemble_maxwell.cpp:396-494: scale w so |w^H A^{-1} w| = Re(Z0)."""
    A, _ = assemble_maxwell(prob, omega, eps, (), -1, use_abc, abc_tags)
    lu = spla.splu(A.tocsc())
    is_pec = np.zeros(prob.n, bool)
    is_pec[prob.pec] = True
    out = []
    for pt in ports:
        pt = dataclasses.replace(pt, weights=pt.weights.copy())
        if pt.Z0 != 0 and np.linalg.norm(pt.weights) >= 1e-15:
            keep = ~is_pec[pt.edges]
            rhs = np.zeros(prob.n, np.complex128)
            rhs[pt.edges[keep]] = pt.weights[keep]
            y = lu.solve(rhs)
            wAw = abs(np.sum(np.conj(pt.weights[keep]) * y[pt.edges[keep]]))
            tgt = float(np.real(pt.Z0))
            if wAw > 1e-15 and tgt > 1e-15:
                pt.weights *= math.sqrt(tgt / wAw)
        out.append(pt)
    return out


def build_lumped_port(prob: Problem, surface_tag: int, e_dir, z0: float = 50.0) -> WavePort:
    """lumped_port.cpp:21-160 (SurfaceIntegral weights).  The reference's edge
    order is unordered_set iteration order; here edges are sorted (the order
    does not change any S-parameter)."""
    sel = np.nonzero(prob.tri_phys == surface_tag)[0]
    if sel.size == 0:
        raise RuntimeError(f"build_lumped_port: no triangles found with surface_tag = {surface_tag}")
    edges = np.unique(prob.topo.tri_edges[sel].ravel())
    pos = {int(e): k for k, e in enumerate(edges)}
    e_dir = np.asarray(e_dir, float)
    e_dir = e_dir / np.linalg.norm(e_dir)
    v = _tri_xyz(prob, sel)
    g, _, area, ok = triangle_surface_curls(v)
    w = np.zeros(edges.size)
    for k in range(sel.size):
        if not ok[k]:
            continue
        for le, (a, b) in enumerate(TRI_PAIRS):
            ge = int(prob.topo.tri_edges[sel[k], le])
            w[pos[ge]] += prob.topo.tri_signs[sel[k], le] * (area[k] / 3.0) * np.dot(g[k, b] - g[k, a], e_dir)
    nrm = np.linalg.norm(w)
    if nrm > 1e-15:
        w *= math.sqrt(z0) / nrm
    return WavePort(surface_tag, edges, w.astype(np.complex128), Z0=z0)


# ------------------------------------------- network parameters, Touchstone

def compute_coupling(S, z0: float = 50.0):
    """coupling.cpp:9-50: Z = z0 (I+S)(I-S)^-1, Y = (I-S)(I+S)^-1 / z0; a
    rank-deficient factor is regularised by 1e-12 I (the full-rank
    pseudo-inverse there is the inverse)."""
    S = np.asarray(S, np.complex128)
    n = S.shape[0]
    I = np.eye(n)

    def inv(Mx):
        if np.linalg.matrix_rank(Mx) < n:
            Mx = Mx + 1e-12 * I
        return np.linalg.inv(Mx)

    return z0 * (I + S) @ inv(I - S), (I - S) @ inv(I + S) / z0


def mutual_coupling_db(S):
    """coupling.cpp:52-65."""
    return 20.0 * np.log10(np.maximum(np.abs(np.asarray(S)), 1e-20))


def active_reflection(S, a):
    """coupling.cpp:67-94."""
    S, a = np.asarray(S, np.complex128), np.asarray(a, np.complex128)
    num = S @ a
    return np.array([0.0 if abs(a[i]) < 1e-20 else num[i] / a[i] for i in range(a.size)], np.complex128)


def is_passive(S, tol=1e-6):
    """coupling.cpp:96-112: every singular value <= 1 + tol."""
    return bool(np.linalg.svd(np.asarray(S, np.complex128), compute_uv=False).max() <= 1.0 + tol)


def _is_approx(A, B, tol):
    # Eigen's isApprox: ||A - B||_F <= tol * min(||A||_F, ||B||_F)
    return bool(np.linalg.norm(A - B) <= tol * min(np.linalg.norm(A), np.linalg.norm(B)))


def is_lossless(S, tol=1e-6):
    """coupling.cpp:114-126."""
    S = np.asarray(S, np.complex128)
    return _is_approx(S.conj().T @ S, np.eye(S.shape[0]), tol)


def is_reciprocal(S, tol=1e-6):
    """coupling.cpp:128-136."""
    S = np.asarray(S, np.complex128)
    return _is_approx(S, S.T, tol)


def _g12(x: float) -> str:
    # an ostream with precision 12 in its default float format prints %.12g
    return "%.12g" % x


def _ts_value(v: complex, fmt: str) -> str:
    """touchstone.cpp:26-44."""
    v = complex(v)
    if fmt == "RI":
        return f"{_g12(v.real)} {_g12(v.imag)}"
    ang = math.atan2(v.imag, v.real) * 180.0 / math.pi
    if fmt == "MA":
        return f"{_g12(abs(v))} {_g12(ang)}"
    return f"{_g12(20.0 * math.log10(max(abs(v), 1e-20)))} {_g12(ang)}"


def touchstone_nport_text(freq, S_list, fmt: str = "RI", z0: float = 50.0) -> str:
    """touchstone.cpp:64-139: the text write_touchstone_nport produces."""
    n = np.asarray(S_list[0]).shape[0]
    out = ["! Touchstone file generated by EdgeFEM\n", f"! Number of ports: {n}\n",
           f"# Hz S {fmt} R {_g12(z0)}\n"]
    for f, S in zip(freq, S_list):
        S = np.asarray(S, np.complex128)
        line = _g12(f)
        k = 0
        for i in range(n):
            for j in range(n):
                if n > 2 and k > 0 and k % 4 == 0:
                    line += "\n"
                line += " " + _ts_value(S[i, j], fmt)
                k += 1
        out.append(line + "\n")
    return "".join(out)


def touchstone_2port_text(freq, S_list) -> str:
    """touchstone.cpp:48-60: legacy 2-port form (s11 s21 s12 s22, RI)."""
    out = ["# Hz S RI R 50\n"]
    for f, S in zip(freq, S_list):
        S = np.asarray(S, np.complex128)
        vals = [S[0, 0], S[1, 0], S[0, 1], S[1, 1]]
        out.append(_g12(f) + "".join(f" {_g12(v.real)} {_g12(v.imag)}" for v in vals) + "\n")
    return "".join(out)


# ------------------------------------------------------ field post-processing

def barycentric(V: np.ndarray, p: np.ndarray) -> np.ndarray:
    """edge_basis.cpp:131-151 for a batch: V (Q,4,3) vertices, p (Q,3) points;
    lambda_0..2 = T^-1 (p - v3), T = [v0-v3, v1-v3, v2-v3]."""
    T = np.stack([V[:, 0] - V[:, 3], V[:, 1] - V[:, 3], V[:, 2] - V[:, 3]], axis=2)
    l012 = np.linalg.solve(T, (p - V[:, 3])[..., None])[..., 0]
    return np.concatenate([l012, 1.0 - l012.sum(axis=1, keepdims=True)], axis=1)


def edge_field(prob: Problem, x: np.ndarray, tet_of=None, points=None) -> np.ndarray:
    """edge_basis.cpp:162-193 at many points: E = sum_e s_e x_e
    (lambda_a grad lambda_b - lambda_b grad lambda_a) over the six edges of
    the point's tet; the tet centroids when no points are given
    (vtk_export.cpp:33-41)."""
    tets = np.arange(prob.tets.shape[0]) if tet_of is None else np.asarray(tet_of)
    X = prob.xyz[prob.node_lut[prob.tets[tets]]]          # (Q,4,3)
    p = X.mean(axis=1) if points is None else np.asarray(points, float).reshape(-1, 3)
    lam = barycentric(X, p)
    g, _ = gradients_and_volume(X)
    dofs = x[prob.topo.tet_edges[tets]] * prob.topo.tet_signs[tets]
    E = np.zeros((tets.size, 3), np.complex128)
    for i, (a, b) in enumerate(TET_PAIRS):
        w = lam[:, a, None] * g[:, b] - lam[:, b, None] * g[:, a]
        E += dofs[:, i, None] * w
    return E


def _e8(v: float) -> str:
    # std::scientific with precision 8
    return "%.8e" % v


def vtu_text(prob: Problem, x: np.ndarray, magnitude=True, phase=True, real=False, imag=False,
             vector=True) -> str:
    """vtk_export.cpp:44-200: the .vtu export_fields_vtk writes."""
    E = edge_field(prob, x)
    T, NN = prob.tets.shape[0], prob.xyz.shape[0]
    o = ['<?xml version="1.0"?>\n',
         '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">\n',
         '  <UnstructuredGrid>\n', f'    <Piece NumberOfPoints="{NN}" NumberOfCells="{T}">\n',
         '      <Points>\n', '        <DataArray type="Float64" NumberOfComponents="3" format="ascii">\n']
    o += [f"          {_e8(a)} {_e8(b)} {_e8(c)}\n" for a, b, c in prob.xyz]
    o += ['        </DataArray>\n', '      </Points>\n', '      <Cells>\n',
          '        <DataArray type="Int32" Name="connectivity" format="ascii">\n']
    o += ["          " + "".join(f"{int(k)} " for k in prob.node_lut[t]) + "\n" for t in prob.tets]
    o += ['        </DataArray>\n', '        <DataArray type="Int32" Name="offsets" format="ascii">\n', "          "]
    for i in range(1, T + 1):
        o.append(f"{i * 4} ")
        if i % 20 == 0:
            o.append("\n          ")
    o += ["\n        </DataArray>\n", '        <DataArray type="UInt8" Name="types" format="ascii">\n', "          "]
    for i in range(T):
        o.append("10 ")
        if (i + 1) % 30 == 0:
            o.append("\n          ")
    o += ["\n        </DataArray>\n", "      </Cells>\n", "      <CellData>\n"]
    if magnitude:
        o.append('        <DataArray type="Float64" Name="E_magnitude" format="ascii">\n')
        o += [f"          {_e8(math.sqrt(sum(abs(c) ** 2 for c in e)))}\n" for e in E]
        o.append("        </DataArray>\n")
    if phase:
        o.append('        <DataArray type="Float64" Name="E_phase_rad" format="ascii">\n')
        for e in E:
            best, ph = 0.0, 0.0
            for c in e:
                if abs(c) > best:
                    best, ph = abs(c), math.atan2(c.imag, c.real)
            o.append(f"          {_e8(ph)}\n")
        o.append("        </DataArray>\n")
    for flag, name, part in ((real, "E_real", "real"), (imag, "E_imag", "imag"), (vector, "E_vector", "real")):
        if flag:
            o.append(f'        <DataArray type="Float64" Name="{name}" NumberOfComponents="3" format="ascii">\n')
            o += ["          " + " ".join(_e8(getattr(c, part)) for c in e) + "\n" for e in E]
            o.append("        </DataArray>\n")
    o += ['        <DataArray type="Int32" Name="PhysicalTag" format="ascii">\n', "          "]
    for i in range(T):
        o.append(f"{int(prob.tet_phys[i])} ")
        if (i + 1) % 20 == 0:
            o.append("\n          ")
    o += ["\n        </DataArray>\n", "      </CellData>\n", "    </Piece>\n", "  </UnstructuredGrid>\n",
          "</VTKFile>\n"]
    return "".join(o)


def vtk_legacy_text(prob: Problem, x: np.ndarray, magnitude=True, vector=True) -> str:
    """vtk_export.cpp:202-272: the legacy .vtk export_fields_vtk_legacy writes."""
    E = edge_field(prob, x)
    T, NN = prob.tets.shape[0], prob.xyz.shape[0]
    o = ["# vtk DataFile Version 3.0\n", "EdgeFEM Field Export\n", "ASCII\n", "DATASET UNSTRUCTURED_GRID\n",
         f"POINTS {NN} double\n"]
    o += [f"{_e8(a)} {_e8(b)} {_e8(c)}\n" for a, b, c in prob.xyz]
    o.append(f"CELLS {T} {T * 5}\n")
    o += ["4" + "".join(f" {int(k)}" for k in prob.node_lut[t]) + "\n" for t in prob.tets]
    o.append(f"CELL_TYPES {T}\n")
    o += ["10\n"] * T
    o.append(f"CELL_DATA {T}\n")
    if magnitude:
        o += ["SCALARS E_magnitude double 1\n", "LOOKUP_TABLE default\n"]
        o += [f"{_e8(math.sqrt(sum(abs(c) ** 2 for c in e)))}\n" for e in E]
    if vector:
        o.append("VECTORS E_vector double\n")
        o += [" ".join(_e8(c.real) for c in e) + "\n" for e in E]
    return "".join(o)
