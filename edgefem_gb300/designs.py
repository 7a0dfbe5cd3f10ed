"""Design-class drop-ins for the reference's python/edgefem/designs/.

RectWaveguideDesign (waveguide.py): same constructor, tags, properties and
`sparams_at_freq` / `frequency_sweep` signatures and error behaviour
(ValueError below cutoff, RuntimeError without a mesh).

StackedPatchDesign (stacked_patch.py): same constructor, tag scheme,
`simulate` / `input_impedance` / `return_loss` / `frequency_sweep` /
`near_field` / `export_fields_vtk` / `export_touchstone` signatures; the
sweep runs on the batched engine.

gmsh is not available to this package, so `generate_mesh` builds structured
hex-to-tet meshes of mesh.py (the same boxes and features; only the element
layout differs from gmsh's Delaunay meshes), and `load_mesh` reads Gmsh v2
files as before.

Chosen forms beside the drop-ins:
  * `RectWaveguideDesign.sparams_sweep(freqs)`: every frequency and both
    ports in one batched double-float solve (FP32 pipes, about 48 bits,
    convergence confirmed on an FP64-accurate true residual);
  * `RectWaveguideDesign.sparams_adjoint(freq, out_j, in_i)`: d|S_ji|^2/d
    eps_r per tetrahedron.
"""
from __future__ import annotations

import math
from typing import List, Optional, Tuple

import numpy as np

from . import sdk as em
from .mesh import TetMesh, patch_antenna_mesh, waveguide_mesh

C0 = 299792458.0


class RectWaveguideDesign:
    def __init__(self, a: float, b: float, length: float, *, pec_tag: int = 1, port1_tag: int = 2,
                 port2_tag: int = 3, volume_tag: int = 100):
        self.a = a
        self.b = b
        self.length = length
        self._pec_tag = pec_tag
        self._port1_tag = port1_tag
        self._port2_tag = port2_tag
        self._volume_tag = volume_tag
        self._mesh: Optional[em.Mesh] = None
        self._mesh_path = None
        self._bc = None
        self._ports = None
        self._last_freq = None
        self._last_S = None
        self._fc = C0 / (2 * a)
        # material overrides: region tag -> eps_r, or per-tet eps_r array
        self.eps_r_regions = {}
        self.eps_r_tet: Optional[np.ndarray] = None
        self.solve_options: Optional[em.SolveOptions] = None

    @property
    def mesh(self):
        return self._mesh

    @property
    def ports(self):
        return self._ports

    @property
    def cutoff_frequency(self) -> float:
        return self._fc

    def _check_propagating(self, freq: float):
        if freq <= self._fc:
            raise ValueError(f"Frequency {freq/1e9:.3f} GHz is below TE10 cutoff {self._fc/1e9:.3f} GHz")

    def generate_mesh(self, density: float = 10.0, output_path: Optional[str] = None, gmsh_options=None) -> None:
        """Structured mesh with about `density` cells per wavelength at 1.5x
        cutoff (the reference's sizing rule, waveguide.py:128-132)."""
        lam = C0 / (1.5 * self._fc)
        h = lam / density
        nx = max(2, int(math.ceil(self.a / h)))
        ny = max(1, int(math.ceil(self.b / h)))
        nz = max(2, int(math.ceil(self.length / h)))
        self.set_mesh(waveguide_mesh(nx, ny, nz, self.a, self.b, self.length))
        if output_path:
            from .mesh import write_gmsh_v2
            path = output_path if output_path.endswith(".msh") else output_path + ".msh"
            write_gmsh_v2(path, self._mesh.arrays())
            self._mesh_path = path

    def set_mesh(self, mesh) -> None:
        """Use an in-memory mesh (TetMesh arrays or an sdk.Mesh)."""
        self._mesh = em.as_mesh(mesh)
        self._mesh_path = None
        self._bc = None
        self._ports = None

    def load_mesh(self, mesh_path: str) -> None:
        self._mesh = em.load_gmsh(mesh_path)
        self._mesh_path = mesh_path
        self._bc = None
        self._ports = None

    def _setup_ports(self, freq: float) -> None:
        if self._mesh is None:
            raise RuntimeError("Mesh not generated. Call generate_mesh() first.")
        if self._bc is None:
            self._bc = em.build_edge_pec(self._mesh, self._pec_tag)
        mode = em.solve_te10_mode(em.RectWaveguidePort(self.a, self.b), freq)
        kc_sq = (np.pi / self.a) ** 2
        if self._ports is None:
            pec = self._bc.dirichlet_edges
            self._ports = [em.build_wave_port_2d(self._mesh, self._port1_tag, mode, pec, kc_sq),
                           em.build_wave_port_2d(self._mesh, self._port2_tag, mode, pec, kc_sq)]
        else:
            # The 2D port mode does not depend on frequency; refresh the
            # analytic mode fields (beta, Z0) and keep the discrete kc.
            for pt in self._ports:
                kc = pt.mode.kc
                pt.mode = em.PortMode(**{**mode.__dict__, "kc": kc})

    def _params(self, freq: float, port_abc_scale: float = 1.0) -> em.MaxwellParams:
        p = em.MaxwellParams()
        p.omega = 2 * np.pi * freq
        p.port_abc_scale = port_abc_scale
        for tag, v in self.eps_r_regions.items():
            p.set_eps_r_region(tag, v)
        if self.eps_r_tet is not None:
            p.eps_r_tet = np.asarray(self.eps_r_tet, np.complex128)
        return p

    def sparams_at_freq(self, freq: float, *, use_eigenmode: bool = True, port_abc_scale: float = 1.0) -> np.ndarray:
        self._check_propagating(freq)
        self._setup_ports(freq)
        params = self._params(freq, port_abc_scale)
        if use_eigenmode:
            S = em.calculate_sparams_eigenmode(self._mesh, params, self._bc, self._ports, self.solve_options)
        else:
            S = em.calculate_sparams(self._mesh, params, self._bc, self._ports, self.solve_options)
        self._last_freq = freq
        self._last_S = S
        em.check_passivity(S)
        return np.array(S)

    def frequency_sweep(self, f_start: float, f_stop: float, n_points: int = 11, *, use_eigenmode: bool = True,
                        port_abc_scale: float = 1.0, verbose: bool = False) -> Tuple[np.ndarray, List[np.ndarray]]:
        freqs = np.linspace(f_start, f_stop, n_points)
        S_list = []
        for i, f in enumerate(freqs):
            if verbose:
                print(f"  {i+1}/{n_points}: {f/1e9:.3f} GHz")
            S_list.append(self.sparams_at_freq(f, use_eigenmode=use_eigenmode, port_abc_scale=port_abc_scale))
        return freqs, S_list

    # ----------------------------------------------------------- chosen forms
    def sparams_sweep(self, freqs, *, port_abc_scale: float = 1.0, opts: Optional[em.BatchOptions] = None):
        """All frequencies x both ports in one batched solve.  Returns
        (S[F,2,2], stats)."""
        freqs = np.asarray(freqs, np.float64)
        for f in freqs:
            self._check_propagating(float(f))
        self._setup_ports(float(freqs[0]))
        inst = em.BatchInstance(self._mesh, self._params(float(freqs[0]), port_abc_scale), self._bc, self._ports)
        S, stats = em.sparams_eigenmode_batched([inst], freqs, opts)
        return S[0], stats

    def sparams_adjoint(self, freq: float, out_j: int = 1, in_i: int = 0):
        """(d|S_ji|^2/d eps_r per tetrahedron, S) at one frequency."""
        self._check_propagating(freq)
        self._setup_ports(freq)
        return em.sparams_eigenmode_adjoint(self._mesh, self._params(freq), self._bc, self._ports, out_j, in_i,
                                            self.solve_options)

    def export_touchstone(self, path: str, freqs=None, S_matrices=None) -> None:
        """waveguide.py:436-464: write the given (or last) S matrices as .s2p."""
        if freqs is None:
            if self._last_freq is None:
                raise RuntimeError("No simulation data. Run sparams_at_freq() first.")
            freqs = np.array([self._last_freq])
            S_matrices = [self._last_S]
        if not path.endswith(".s2p"):
            path = path + ".s2p"
        em.write_touchstone_nport(path, list(freqs), [np.array(S, dtype=complex) for S in S_matrices])

    def export_fields_vtk(self, path: str, freq: Optional[float] = None, *, active_port: int = 0) -> None:
        """waveguide.py:466-509: solve the driven (w w^H) system with one port
        active and write E at the tet centroids as .vtu."""
        if self._mesh is None:
            raise RuntimeError("Mesh not generated. Call generate_mesh() first.")
        if freq is None:
            if self._last_freq is None:
                raise ValueError("No frequency specified and no prior simulation.")
            freq = self._last_freq
        else:
            self._setup_ports(freq)
        params = em.MaxwellParams()
        params.omega = 2 * np.pi * freq
        asm = em.assemble_maxwell(self._mesh, params, self._bc, self._ports, active_port)
        res = em.solve_linear(asm.A, asm.b)
        em.export_fields_vtk(self._mesh, res.x, path)

    def __repr__(self) -> str:
        return (f"RectWaveguideDesign(a={self.a*1000:.2f}mm, b={self.b*1000:.2f}mm, "
                f"length={self.length*1000:.2f}mm, fc={self._fc/1e9:.3f}GHz)")


class StackedPatchDesign:
    """Probe-fed (stacked) patch antenna: the drop-in for the reference's
    python/edgefem/designs/stacked_patch.py (StackedPatchDesign).

    Physical tags as there (stacked_patch.py:62-73): ground 1, cavity walls
    2, cavity bottom 3, probe 4, lumped port 5, patches 10, 11, ..., ABC 50,
    substrates 110, 111, ..., air 150.  Any mesh with these tags can be
    given to `set_mesh` / `load_mesh`.

    `generate_mesh` builds the single-patch, single-substrate case as a
    graded, jittered hex grid split into tets (mesh.patch_antenna_mesh): the
    ground plane (tag 1) over the whole box floor, the substrate (110), the
    patch (10) as PEC triangles on it, air (150) up to `air_box_height`
    above the patch with the absorbing faces (50), and the probe as a
    vertical lumped-port strip (5) between ground and patch at the probe
    offset, excited along z.  The cavity below the ground plane and the
    coaxial probe of the reference's gmsh geometry are not built (a gmsh
    geometry builder is outside this package); a loaded mesh uses the
    reference's port direction (x, across the coaxial gap).

    Extensions: `substrates[i]['debye'] = (eps_s, eps_inf, tau)` makes that
    substrate Debye-dispersive; `solve_options` replaces the solver options
    (GPU COCG, relative residual 1e-10); `use_batched_sweep = False` runs
    `frequency_sweep` one frequency at a time on the plain path.

    Port normalisation: the reference's `simulate` and `frequency_sweep`
    call normalize_port_weights and discard its result (its binding returns
    a normalised copy, pyedgefem.cpp:552-563), so they extract S11 with the
    unnormalised weights.  Here the normalised ports are used, as both
    methods' comments intend; `apply_normalization = False` reproduces the
    reference's literal behaviour.
    """

    _TAG_GROUND = 1
    _TAG_CAVITY_WALLS = 2
    _TAG_CAVITY_BOTTOM = 3
    _TAG_PROBE = 4
    _TAG_PORT = 5
    _TAG_PATCH_BASE = 10
    _TAG_ABC = 50
    _TAG_HUYGENS = 60
    _TAG_CAVITY_VOL = 100
    _TAG_SUBSTRATE_BASE = 110
    _TAG_AIR = 150

    def __init__(self, patches: List[dict], substrates: List[dict], cavity_size: float, cavity_depth: float,
                 probe_radius: float = 0.5e-3, probe_offset: Tuple[float, float] = (0.0, 0.0), z0: float = 50.0,
                 ground_plane_size: Optional[float] = None, air_box_height: Optional[float] = None):
        if len(patches) == 0:
            raise ValueError("At least one patch is required")
        if len(substrates) == 0:
            raise ValueError("At least one substrate is required")
        self.patches = patches
        self.substrates = substrates
        self.cavity_size = cavity_size
        self.cavity_depth = cavity_depth
        self.probe_radius = probe_radius
        self.probe_offset = probe_offset
        self.z0 = z0
        max_patch = max(max(p["width"], p["length"]) for p in patches)
        self.ground_plane_size = ground_plane_size or 3.0 * max_patch
        self._air_box_height = air_box_height
        self._mesh: Optional[em.Mesh] = None
        self._mesh_path = None
        self._bc = None
        self._ports = None
        self._last_solutions = {}
        self.port_e_direction = (1.0, 0.0, 0.0)
        self.solve_options: Optional[em.SolveOptions] = None
        self.batch_options: Optional[em.BatchOptions] = None
        self.use_batched_sweep = True
        self.apply_normalization = True

    @property
    def mesh(self):
        return self._mesh

    # ------------------------------------------------------------ meshes
    def generate_mesh(self, density: float = 12.0, output_path: Optional[str] = None,
                      design_freq: Optional[float] = None) -> None:
        """Mesh of the design with about `density` cells per wavelength at
        `design_freq` (default: the first patch's half-wave resonance,
        c0 / (2 L sqrt(eps_r)), stacked_patch.py:155-163) away from the
        patch and four times finer across it."""
        if len(self.patches) != 1 or len(self.substrates) != 1:
            raise NotImplementedError("generate_mesh builds one patch on one substrate; give a stacked "
                                      "design's mesh (reference tags) to set_mesh or load_mesh")
        patch, sub = self.patches[0], self.substrates[0]
        if design_freq is None:
            design_freq = C0 / (2 * patch["length"] * math.sqrt(sub["eps_r"]))
        lam = C0 / design_freq
        lc = lam / density
        if self._air_box_height is None:
            self._air_box_height = lam / 4
        t = float(sub["thickness"])
        gp = float(self.ground_plane_size)
        arrays = patch_antenna_mesh(h_fine=lc / 4, h_coarse=lc, box=(gp, gp, t + self._air_box_height),
                                    substrate=t, sub_cells=max(2, int(math.ceil(t / (lc / 4)))),
                                    patch=(patch["width"], patch["length"]),
                                    feed_offset=float(self.probe_offset[1]), feed_x_offset=float(self.probe_offset[0]),
                                    feed_width=max(2 * self.probe_radius, lc / 8))
        # mesh.py's tags -> the reference's tag scheme
        from . import mesh as M
        tp = np.asarray(arrays.tet_phys).copy()
        arrays.tet_phys = np.where(tp == M.DIELECTRIC_TAG, self._TAG_SUBSTRATE_BASE, self._TAG_AIR).astype(np.int32)
        rp = np.asarray(arrays.tri_phys)
        arrays.tri_phys = np.where(rp == M.FEED_TAG, self._TAG_PORT, rp).astype(np.int32)
        self.set_mesh(arrays)
        self.port_e_direction = (0.0, 0.0, 1.0)
        if output_path:
            from .mesh import write_gmsh_v2
            path = output_path if output_path.endswith(".msh") else output_path + ".msh"
            write_gmsh_v2(path, arrays)
            self._mesh_path = path

    def set_mesh(self, mesh) -> None:
        """Use an in-memory mesh (TetMesh arrays or an sdk.Mesh) with the
        reference's tags."""
        self._mesh = em.as_mesh(mesh)
        self._mesh_path = None
        self._bc = None
        self._ports = None
        self._last_solutions = {}

    def load_mesh(self, mesh_path: str) -> None:
        self._mesh = em.load_gmsh(mesh_path)
        self._mesh_path = mesh_path
        self._bc = None
        self._ports = None
        self._last_solutions = {}
        self.port_e_direction = (1.0, 0.0, 0.0)

    # ------------------------------------------------------- simulation
    def _setup_simulation(self, freq: float) -> None:
        """stacked_patch.py:469-501: PEC on every conductor tag present,
        merged; one lumped port on tag 5."""
        if self._mesh is None:
            raise RuntimeError("Mesh not generated. Call generate_mesh() first.")
        bc = em.BC()
        pec_tags = [self._TAG_GROUND, self._TAG_CAVITY_WALLS, self._TAG_CAVITY_BOTTOM, self._TAG_PROBE]
        pec_tags += [self._TAG_PATCH_BASE + i for i in range(len(self.patches))]
        for tag in pec_tags:
            if em.has_surface_tag(self._mesh, tag):
                bc.merge(em.build_edge_pec(self._mesh, tag))
        self._bc = bc
        self._ports = [em.build_lumped_port(self._mesh, self._TAG_PORT, self.z0, self.port_e_direction)]

    def _params(self, freq: float) -> em.MaxwellParams:
        p = em.MaxwellParams()
        p.omega = 2 * np.pi * freq
        p.use_abc = True
        p.abc_surface_tags = {self._TAG_ABC}
        for si, sub in enumerate(self.substrates):
            tag = self._TAG_SUBSTRATE_BASE + si
            if "debye" in sub:
                p.set_debye_region(tag, *sub["debye"])
            else:
                eps_r = sub["eps_r"]
                tan_d = sub.get("tan_d", 0.0)
                p.set_eps_r_region(tag, complex(eps_r, -eps_r * tan_d))
        return p

    def _opts(self) -> em.SolveOptions:
        return self.solve_options or em.SolveOptions(use_bicgstab=False, tolerance=1e-10, max_iterations=400000)

    def _normalized(self, params, opts):
        ports = em.normalize_port_weights(self._mesh, params, self._bc, self._ports, opts)
        return ports if self.apply_normalization else self._ports

    def simulate(self, freq: float) -> Tuple[complex, np.ndarray]:
        """stacked_patch.py:503-561: (S11, solution vector) at `freq`."""
        self._setup_simulation(freq)
        params = self._params(freq)
        opts = self._opts()
        ports = self._normalized(params, opts)
        S = em.calculate_sparams(self._mesh, params, self._bc, ports, opts)
        S11 = complex(S[0, 0])
        if abs(S11) > 1.01:
            import sys
            print(f"WARNING: |S11| = {abs(S11):.4f} > 1 at {freq/1e9:.3f} GHz "
                  f"(passivity violation \u2014 consider refining mesh)", file=sys.stderr)
        asm = em.assemble_maxwell(self._mesh, params, self._bc, ports, 0)
        res = em.solve_linear(asm.A, asm.b, opts)
        self._last_solutions[freq] = res.x
        return S11, res.x

    def input_impedance(self, freq: float) -> complex:
        S11, _ = self.simulate(freq)
        if abs(1 - S11) < 1e-30:
            return complex(1e6, 0)
        return self.z0 * (1 + S11) / (1 - S11)

    def return_loss(self, freq: float, z0: float = 50.0) -> float:
        S11, _ = self.simulate(freq)
        return 20 * np.log10(abs(S11) + 1e-30)

    def frequency_sweep(self, f_start: float, f_stop: float, n_points: int = 21,
                        verbose: bool = False) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """stacked_patch.py:652-717: ports normalised once at the middle
        frequency, then every frequency; returns (freqs, Z_in, S11).  All
        frequencies are solved together on the batched engine (driven-port
        formulation) unless use_batched_sweep is False."""
        freqs = np.linspace(f_start, f_stop, n_points)
        f_mid = (f_start + f_stop) / 2.0
        self._setup_simulation(f_mid)
        params = self._params(f_mid)
        opts = self._opts()
        ports = self._normalized(params, opts)
        if verbose:
            print(f"  Running {n_points}-point frequency sweep ({f_start/1e9:.3f}\u2013{f_stop/1e9:.3f} GHz)")
        if self.use_batched_sweep:
            sweep, _ = em.frequency_sweep_batched(self._mesh, params, self._bc, ports, freqs, self.batch_options)
        else:
            sweep = em.frequency_sweep(self._mesh, params, self._bc, ports, freqs, opts)
        S11 = np.array([complex(S[0, 0]) for S in sweep.S_matrices])
        Z = np.array([self.z0 * (1 + s) / (1 - s) if abs(1 - s) > 1e-30 else complex(1e6, 0) for s in S11])
        return freqs, Z, S11

    # ------------------------------------------------- post-processing
    def _locate(self, points: np.ndarray) -> np.ndarray:
        """Containing tetrahedron of each point (-1 outside the mesh)."""
        a = self._mesh.arrays()
        X = a.xyz[a.node_index()[a.tets]]
        out = np.full(points.shape[0], -1, np.int32)
        T = np.stack([X[:, 0] - X[:, 3], X[:, 1] - X[:, 3], X[:, 2] - X[:, 3]], axis=2)
        Tinv = np.linalg.inv(T)
        for i, p in enumerate(points):
            lam = np.einsum("tij,tj->ti", Tinv, p - X[:, 3])
            lam = np.concatenate([lam, 1.0 - lam.sum(axis=1, keepdims=True)], axis=1)
            hit = np.flatnonzero(np.all(lam >= -1e-10, axis=1))
            if hit.size:
                out[i] = hit[0]
        return out

    def near_field(self, freq: float, points: np.ndarray) -> np.ndarray:
        """stacked_patch.py:859-895: E at the given points (zero outside the
        mesh), from the last solution at `freq`; evaluated on the GPU."""
        if freq not in self._last_solutions:
            self.simulate(freq)
        pts = np.asarray(points, np.float64).reshape(-1, 3)
        tet_of = self._locate(pts)
        E = np.zeros((pts.shape[0], 3), np.complex128)
        inside = tet_of >= 0
        if inside.any():
            E[inside] = em.evaluate_field(self._mesh, self._last_solutions[freq], tet_of[inside], pts[inside])
        return E

    def export_fields_vtk(self, freq: float, path: str) -> None:
        if freq not in self._last_solutions:
            self.simulate(freq)
        em.export_fields_vtk(self._mesh, self._last_solutions[freq], path)

    def export_touchstone(self, path: str, freqs: np.ndarray, S11_array: np.ndarray) -> None:
        S_matrices = [np.array([[s]], dtype=complex) for s in S11_array]
        if not path.endswith(".s1p"):
            path = path + ".s1p"
        em.write_touchstone_nport(path, list(freqs), S_matrices)

    def __repr__(self) -> str:
        n_patches = len(self.patches)
        n_subs = len(self.substrates)
        return (f"StackedPatchDesign({n_patches} patch{'es' if n_patches > 1 else ''}, "
                f"{n_subs} substrate{'s' if n_subs > 1 else ''}, "
                f"cavity={self.cavity_size*1000:.1f}mm, z0={self.z0:.0f}ohm)")
