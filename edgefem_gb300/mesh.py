"""Tetrahedral meshes: structured hex grids split into six tetrahedra, and
Gmsh v2 ASCII read/write.

The reference builds its meshes with gmsh from `.geo` scripts
(python/edgefem/designs/waveguide.py:109-241) and loads them through
`load_gmsh_v2` (src/mesh_gmsh.cpp:15-101).  gmsh is not available to this
package, so meshes of the same kind are synthesised here on a structured
grid: every hexahedral cell is cut along its main diagonal into the six
"path" tetrahedra of the Kuhn (Freudenthal) triangulation, which is
conforming across neighbouring cells because every cell uses the same
diagonal direction.

Physical tags follow the reference's waveguide design class
(waveguide.py:44-53): PEC walls 1, port 1 (z = 0) 2, port 2 (z = L) 3,
volume 100; a dielectric region inside the volume is tagged 101.

Node ids are 1-based like gmsh.  Tetrahedra are listed cell by cell with x
fastest, then y, then z, which fixes the reference's global edge numbering
(first appearance while scanning the tetrahedra, mesh_gmsh.cpp:104-147).
"""
from __future__ import annotations

import dataclasses
import itertools
from typing import Optional, Sequence

import numpy as np

PEC_TAG = 1
PORT1_TAG = 2
PORT2_TAG = 3
AIR_TAG = 100
DIELECTRIC_TAG = 101


@dataclasses.dataclass
class TetMesh:
    """Plain-array mesh: what `load_gmsh_v2` keeps for the volume path.

    Attributes:
        node_ids: (N,) int64 gmsh node ids.
        xyz: (N, 3) float64 node coordinates in metres.
        tets: (T, 4) int64 node ids of each tetrahedron.
        tet_phys: (T,) int32 physical tag of each tetrahedron.
        tris: (S, 3) int64 node ids of each boundary triangle.
        tri_phys: (S,) int32 physical tag of each triangle.
    """

    node_ids: np.ndarray
    xyz: np.ndarray
    tets: np.ndarray
    tet_phys: np.ndarray
    tris: np.ndarray
    tri_phys: np.ndarray

    @property
    def num_nodes(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def num_tets(self) -> int:
        return int(self.tets.shape[0])

    @property
    def num_tris(self) -> int:
        return int(self.tris.shape[0])

    def node_index(self) -> np.ndarray:
        """Map node id -> row of `xyz` as a dense lookup table."""
        lut = np.full(int(self.node_ids.max()) + 1, -1, dtype=np.int64)
        lut[self.node_ids] = np.arange(self.num_nodes, dtype=np.int64)
        return lut

    def tet_xyz(self) -> np.ndarray:
        """(T, 4, 3) vertex coordinates of every tetrahedron."""
        return self.xyz[self.node_index()[self.tets]]

    def centroids(self) -> np.ndarray:
        return self.tet_xyz().mean(axis=1)


# The six Kuhn path tetrahedra of the unit cube.  Cube corner (dx, dy, dz) has
# local index dx + 2*dy + 4*dz.  Each permutation (a, b, c) of the axes gives
# the path 000 -> e_a -> e_a + e_b -> 111.  Odd permutations have negative
# orientation; their first two vertices are swapped so every tetrahedron has
# det([v1-v0, v2-v0, v3-v0]) > 0.
def _kuhn_local_tets() -> np.ndarray:
    out = []
    for perm in itertools.permutations(range(3)):
        p = [0]
        cur = 0
        for ax in perm[:2]:
            cur |= 1 << ax
            p.append(cur)
        p.append(7)
        corners = np.array([[(c >> 0) & 1, (c >> 1) & 1, (c >> 2) & 1] for c in p], float)
        det = np.linalg.det(np.stack([corners[1] - corners[0], corners[2] - corners[0],
                                      corners[3] - corners[0]]))
        if det < 0:
            p[0], p[1] = p[1], p[0]
        out.append(p)
    return np.array(out, dtype=np.int64)


KUHN_TETS = _kuhn_local_tets()


def _axis_coords(n: int, length: float, grading: Optional[Sequence[float]] = None) -> np.ndarray:
    if grading is None:
        return np.linspace(0.0, length, n + 1)
    w = np.asarray(grading, dtype=np.float64)
    if w.shape != (n,):
        raise ValueError("grading needs one positive width per cell")
    c = np.concatenate([[0.0], np.cumsum(w)])
    return c * (length / c[-1])


def box_tet_mesh(
    nx: int,
    ny: int,
    nz: int,
    a: float,
    b: float,
    length: float,
    *,
    xs: Optional[np.ndarray] = None,
    ys: Optional[np.ndarray] = None,
    zs: Optional[np.ndarray] = None,
    jitter: float = 0.0,
    seed: int = 0,
    volume_tag_fn=None,
    wall_tag: int = PEC_TAG,
    port1_tag: int = PORT1_TAG,
    port2_tag: int = PORT2_TAG,
) -> TetMesh:
    """Box [0,a]x[0,b]x[0,length] on an nx*ny*nz hex grid, 6 tets per cell.

    Args:
        xs, ys, zs: optional explicit grid coordinates (length n+1, increasing)
            for graded grids; default uniform.
        jitter: interior nodes are moved by up to `jitter` times the local
            cell size in each direction (seeded); boundary nodes stay on the
            box faces.
        volume_tag_fn: optional callable(centroids (T,3)) -> (T,) int tags;
            default AIR_TAG everywhere.
    """
    xs = _axis_coords(nx, a) if xs is None else np.asarray(xs, np.float64)
    ys = _axis_coords(ny, b) if ys is None else np.asarray(ys, np.float64)
    zs = _axis_coords(nz, length) if zs is None else np.asarray(zs, np.float64)
    NX, NY, NZ = nx + 1, ny + 1, nz + 1
    K, J, I = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    I = I.ravel(); J = J.ravel(); K = K.ravel()
    xyz = np.stack([xs[I], ys[J], zs[K]], axis=1)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        hx = np.diff(xs).min(); hy = np.diff(ys).min(); hz = np.diff(zs).min()
        d = rng.uniform(-1.0, 1.0, size=xyz.shape) * jitter * np.array([hx, hy, hz])
        d[(I == 0) | (I == nx), 0] = 0.0
        d[(J == 0) | (J == ny), 1] = 0.0
        d[(K == 0) | (K == nz), 2] = 0.0
        xyz = xyz + d
    node_ids = np.arange(1, NX * NY * NZ + 1, dtype=np.int64)

    def nid(i, j, k):
        return 1 + i + NX * (j + NY * k)

    # cells, x fastest
    ck, cj, ci = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ci = ci.ravel(); cj = cj.ravel(); ck = ck.ravel()
    corner = np.stack([nid(ci + (c & 1), cj + ((c >> 1) & 1), ck + ((c >> 2) & 1))
                       for c in range(8)], axis=1)          # (C, 8)
    tets = corner[:, KUHN_TETS].reshape(-1, 4)              # (6C, 4)

    centroids = xyz[tets - 1].mean(axis=1)
    if volume_tag_fn is None:
        tet_phys = np.full(tets.shape[0], AIR_TAG, dtype=np.int32)
    else:
        tet_phys = np.asarray(volume_tag_fn(centroids), dtype=np.int32)

    tris = []
    phys = []

    def quad_tris(lo, e_a, e_b, hi):
        return [np.stack([lo, e_a, hi], 1), np.stack([lo, e_b, hi], 1)]

    # port faces z=0 and z=L (cells in x-y)
    qj, qi = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    qi = qi.ravel(); qj = qj.ravel()
    for k, tag in ((0, port1_tag), (nz, port2_tag)):
        t = quad_tris(nid(qi, qj, k), nid(qi + 1, qj, k), nid(qi, qj + 1, k), nid(qi + 1, qj + 1, k))
        tris += t; phys += [np.full(qi.size, tag)] * 2
    # walls y=0, y=b (cells in x-z)
    qk, qi2 = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    qk = qk.ravel(); qi2 = qi2.ravel()
    for j in (0, ny):
        t = quad_tris(nid(qi2, j, qk), nid(qi2 + 1, j, qk), nid(qi2, j, qk + 1), nid(qi2 + 1, j, qk + 1))
        tris += t; phys += [np.full(qk.size, wall_tag)] * 2
    # walls x=0, x=a (cells in y-z)
    qk3, qj3 = np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij")
    qk3 = qk3.ravel(); qj3 = qj3.ravel()
    for i in (0, nx):
        t = quad_tris(nid(i, qj3, qk3), nid(i, qj3 + 1, qk3), nid(i, qj3, qk3 + 1), nid(i, qj3 + 1, qk3 + 1))
        tris += t; phys += [np.full(qk3.size, wall_tag)] * 2
    tris = np.concatenate(tris, axis=0).astype(np.int64)
    tri_phys = np.concatenate(phys).astype(np.int32)
    return TetMesh(node_ids, xyz, tets.astype(np.int64), tet_phys, tris, tri_phys)


def waveguide_mesh(nx: int, ny: int, nz: int, a: float = 22.86e-3, b: float = 10.16e-3,
                   length: float = 50e-3, *, slab: Optional[tuple] = None, **kw) -> TetMesh:
    """Rectangular waveguide box; `slab=(z0, z1)` tags tets with centroid
    z in [z0, z1] as DIELECTRIC_TAG."""
    fn = None
    if slab is not None:
        z0, z1 = slab

        def fn(c):
            return np.where((c[:, 2] >= z0) & (c[:, 2] <= z1), DIELECTRIC_TAG, AIR_TAG)
    return box_tet_mesh(nx, ny, nz, a, b, length, volume_tag_fn=fn, **kw)


PATCH_TAG = 10
FEED_TAG = 20
ABC_TAG = 50


def _graded_axis(length: float, fine: tuple, feats: Sequence[float], h_fine: float, h_coarse: float,
                 growth: float = 1.2) -> np.ndarray:
    """Grid coordinates on [0, length]: spacing <= h_fine inside the zone
    `fine` = (lo, hi) with every feature coordinate a grid line, growing
    geometrically by `growth` up to h_coarse towards both ends."""
    lo, hi = fine
    pts = sorted(set([lo, hi] + [float(f) for f in feats if lo <= f <= hi]))
    xs = [pts[0]]
    for a, b in zip(pts, pts[1:]):
        n = max(1, int(np.ceil((b - a) / h_fine - 1e-9)))
        xs += list(np.linspace(a, b, n + 1)[1:])

    def ramp(gap):
        if gap <= 0:
            return np.zeros(0)
        h, w = h_fine, []
        while sum(w) < gap:
            h = min(h * growth, h_coarse)
            w.append(h)
        w = np.array(w) * (gap / sum(w))
        return np.cumsum(w)

    left = lo - ramp(lo)[::-1]
    right = hi + ramp(length - hi)
    out = np.concatenate([left[left < lo - 1e-12], xs, right[right > hi + 1e-12]])
    out[0], out[-1] = 0.0, length
    return np.unique(np.round(out, 12))


def patch_antenna_mesh(h_fine: float = 0.55e-3, h_coarse: float = 5e-3, *, box=(100e-3, 100e-3, 40e-3),
                       substrate: float = 1.6e-3, sub_cells: int = 4, patch=(38e-3, 29e-3),
                       feed_offset: float = -5e-3, feed_width: float = 1e-3, jitter: float = 0.15,
                       seed: int = 0, feed_x_offset: float = 0.0) -> TetMesh:
    """Probe-fed microstrip patch in an air box (the stacked-patch design's
    single-layer case, python/edgefem/designs/stacked_patch.py:184-463, built
    as a graded hex grid instead of a gmsh geometry).

    Box [0, box] with the ground plane at z = 0 (tag 1, PEC), the outer
    faces above it absorbing (tag 50), an FR-4 substrate 0 <= z <= substrate
    (tets tag 101), the patch (width x length = 38 x 29 mm: the resonant
    length along y, about 2.4 GHz on FR-4) as PEC triangles (tag 10) on
    z = substrate, centred in x and y, and a vertical lumped-port gap strip (tag 20) at
    y = centre + feed_offset, |x - centre - feed_x_offset| <= feed_width/2,
    between ground and patch.  Interior nodes move by up to `jitter` times the local spacing
    (seeded), except in the direction normal to a feature plane.
    """
    Lx, Ly, Lz = box
    cx, cy = Lx / 2, Ly / 2
    px0, px1 = cx - patch[0] / 2, cx + patch[0] / 2
    py0, py1 = cy - patch[1] / 2, cy + patch[1] / 2
    fy = cy + feed_offset
    fx0, fx1 = cx + feed_x_offset - feed_width / 2, cx + feed_x_offset + feed_width / 2
    m = 5e-3  # fine zone margin around the patch
    xs = _graded_axis(Lx, (px0 - m, px1 + m), [px0, px1, fx0, fx1], h_fine, h_coarse)
    ys = _graded_axis(Ly, (py0 - m, py1 + m), [py0, py1, fy], h_fine, h_coarse)
    zsub = np.linspace(0.0, substrate, sub_cells + 1)
    hz = substrate / sub_cells
    zup = substrate + np.cumsum(_ramp_widths(Lz - substrate, hz, h_coarse))
    zs = np.unique(np.round(np.concatenate([zsub, zup]), 12))
    zs[-1] = Lz

    def tag_fn(c):
        return np.where(c[:, 2] <= substrate, DIELECTRIC_TAG, AIR_TAG)

    mesh = box_tet_mesh(xs.size - 1, ys.size - 1, zs.size - 1, Lx, Ly, Lz, xs=xs, ys=ys, zs=zs,
                        volume_tag_fn=tag_fn, wall_tag=ABC_TAG, port1_tag=PEC_TAG, port2_tag=ABC_TAG)
    NX, NY = xs.size, ys.size

    def nid(i, j, k):
        return 1 + i + NX * (j + NY * k)

    def near(arr, v):
        return int(np.argmin(np.abs(arr - v)))

    tris, phys = [mesh.tris], [mesh.tri_phys]
    # patch: z = substrate, x in [px0, px1], y in [py0, py1] (same diagonal as the tet faces)
    k = near(zs, substrate)
    i0, i1, j0, j1 = near(xs, px0), near(xs, px1), near(ys, py0), near(ys, py1)
    qj, qi = np.meshgrid(np.arange(j0, j1), np.arange(i0, i1), indexing="ij")
    qi, qj = qi.ravel(), qj.ravel()
    lo, ea, eb, hi = nid(qi, qj, k), nid(qi + 1, qj, k), nid(qi, qj + 1, k), nid(qi + 1, qj + 1, k)
    tris += [np.stack([lo, ea, hi], 1), np.stack([lo, eb, hi], 1)]
    phys += [np.full(2 * qi.size, PATCH_TAG, np.int32)]
    # feed strip: y = fy, x in [fx0, fx1], z in [0, substrate]
    j = near(ys, fy)
    a0, a1 = near(xs, fx0), near(xs, fx1)
    qk, qi = np.meshgrid(np.arange(0, k), np.arange(a0, a1), indexing="ij")
    qi, qk = qi.ravel(), qk.ravel()
    lo, ea, eb, hi = nid(qi, j, qk), nid(qi + 1, j, qk), nid(qi, j, qk + 1), nid(qi + 1, j, qk + 1)
    tris += [np.stack([lo, ea, hi], 1), np.stack([lo, eb, hi], 1)]
    phys += [np.full(2 * qi.size, FEED_TAG, np.int32)]
    mesh.tris = np.concatenate(tris).astype(np.int64)
    mesh.tri_phys = np.concatenate(phys).astype(np.int32)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        n = mesh.num_nodes
        ijk = np.stack([(np.arange(n) % NX), (np.arange(n) // NX) % NY, np.arange(n) // (NX * NY)], 1)
        d = np.zeros((n, 3))
        for ax, g, feats in ((0, xs, [px0, px1, fx0, fx1]), (1, ys, [py0, py1, fy]), (2, zs, [substrate])):
            h = np.minimum(np.diff(g, prepend=np.inf), np.diff(g, append=np.inf))
            step = rng.uniform(-1.0, 1.0, n) * jitter * h[ijk[:, ax]]
            fixed = np.zeros(g.size, bool)
            fixed[[0, g.size - 1]] = True
            for f in feats:
                fixed[near(g, f)] = True
            step[fixed[ijk[:, ax]]] = 0.0
            d[:, ax] = step
        mesh.xyz = mesh.xyz + d
    return mesh


def _ramp_widths(gap: float, h0: float, h_max: float, growth: float = 1.2) -> np.ndarray:
    h, w = h0, []
    while sum(w) < gap:
        h = min(h * growth, h_max)
        w.append(h)
    return np.array(w) * (gap / sum(w))


# ---------------------------------------------------------------- Gmsh v2 I/O

def write_gmsh_v2(path: str, mesh: TetMesh) -> None:
    """Write a Gmsh v2.2 ASCII file with triangles (type 2) then tetrahedra
    (type 4), two tags each (physical, elementary)."""
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n")
        f.write(f"{mesh.num_nodes}\n")
        for nid, (x, y, z) in zip(mesh.node_ids.tolist(), mesh.xyz.tolist()):
            f.write(f"{nid} {x!r} {y!r} {z!r}\n")
        f.write("$EndNodes\n$Elements\n")
        f.write(f"{mesh.num_tris + mesh.num_tets}\n")
        eid = 1
        for (n0, n1, n2), ph in zip(mesh.tris.tolist(), mesh.tri_phys.tolist()):
            f.write(f"{eid} 2 2 {ph} {ph} {n0} {n1} {n2}\n")
            eid += 1
        for (n0, n1, n2, n3), ph in zip(mesh.tets.tolist(), mesh.tet_phys.tolist()):
            f.write(f"{eid} 4 2 {ph} {ph} {n0} {n1} {n2} {n3}\n")
            eid += 1
        f.write("$EndElements\n")


def read_gmsh_v2(path: str) -> TetMesh:
    """Parse a Gmsh v2 ASCII mesh the way `load_gmsh_v2` does
    (src/mesh_gmsh.cpp:15-101): nodes, triangles (type 2), tetrahedra
    (type 4); the first tag is the physical tag; line elements and other
    types are skipped.  Raises RuntimeError if the file cannot be opened."""
    try:
        with open(path) as f:
            lines = f.read().split("\n")
    except OSError as e:
        raise RuntimeError(f"Failed to open mesh file: {path}") from e
    node_ids, xyz, tets, tet_phys, tris, tri_phys = [], [], [], [], [], []
    i = 0
    while i < len(lines):
        line = lines[i].strip()
        if line == "$Nodes":
            n = int(lines[i + 1]); i += 2
            for k in range(n):
                p = lines[i + k].split()
                node_ids.append(int(p[0])); xyz.append([float(p[1]), float(p[2]), float(p[3])])
            i += n
        elif line == "$Elements":
            m = int(lines[i + 1]); i += 2
            for k in range(m):
                p = lines[i + k].split()
                typ, ntag = int(p[1]), int(p[2])
                phys = int(p[3]) if ntag > 0 else 0
                conn = [int(v) for v in p[3 + ntag:]]
                if typ == 2:
                    tris.append(conn[:3]); tri_phys.append(phys)
                elif typ == 4:
                    tets.append(conn[:4]); tet_phys.append(phys)
            i += m
        else:
            i += 1
    return TetMesh(np.array(node_ids, np.int64), np.array(xyz, np.float64).reshape(-1, 3),
                   np.array(tets, np.int64).reshape(-1, 4), np.array(tet_phys, np.int32),
                   np.array(tris, np.int64).reshape(-1, 3), np.array(tri_phys, np.int32))
