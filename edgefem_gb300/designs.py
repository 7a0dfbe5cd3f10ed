"""RectWaveguideDesign: the drop-in for the reference's
python/edgefem/designs/waveguide.py.

Same constructor, tags, properties and `sparams_at_freq` / `frequency_sweep`
signatures and error behaviour (ValueError below cutoff, RuntimeError
without a mesh).  gmsh is not available to this package, so
`generate_mesh` builds the structured hex-to-tet mesh of mesh.py (the box is
the same; only the element layout differs from gmsh's Delaunay mesh), and
`load_mesh` reads Gmsh v2 files as before.

Chosen forms beside the drop-in:
  * `sparams_sweep(freqs)`: every frequency and both ports in one batched
    complex64 solve with FP64 refinement;
  * `sparams_adjoint(freq, out_j, in_i)`: d|S_ji|^2/d eps_r per tetrahedron.
"""
from __future__ import annotations

import math
from typing import List, Optional, Tuple

import numpy as np

from . import sdk as em
from .mesh import TetMesh, waveguide_mesh

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
