"""edgefem-gb300: GB300-native frequency-domain Maxwell hot path of
jman4162/EdgeFEM (Nédélec assembly, sparse complex solve, S-parameters).

Importing the package loads libedgefem_gb300.so and fails if it is not
built (`python edgefem_gb300/build.py`).
"""
from .sdk import *  # noqa: F401,F403
from .sdk import (BC, BatchInstance, BatchOptions, BatchSolver, MaxwellParams, Mesh, PortMode,  # noqa: F401
                  RectWaveguidePort, SolveOptions, WavePort, as_mesh, assemble_maxwell, assemble_maxwell_km,
                  build_edge_pec, build_lumped_port, build_wave_port_2d, calculate_sparams,
                  calculate_sparams_eigenmode, check_passivity, device_count, frequency_sweep, load_gmsh,
                  normalize_port_weights, solve_linear, solve_te10_mode, sparams_eigenmode_adjoint, sparams_driven_adjoint,
                  sparams_eigenmode_batched, validate_mesh, validate_mesh_gpu, build_edges_gpu, CouplingMatrix, TouchstoneFormat, TouchstoneOptions,
                  active_reflection, compute_coupling, is_lossless, is_passive, is_reciprocal, mutual_coupling_db,
                  singular_values, touchstone_extension, write_touchstone, write_touchstone_nport,
                  VTKExportOptions, compute_barycentric, evaluate_edge_field, evaluate_field, export_fields_vtk,
                  export_fields_vtk_legacy, has_surface_tag, merge_bc, frequency_sweep_batched)
from .designs import RectWaveguideDesign, StackedPatchDesign  # noqa: F401
from .mesh import TetMesh, box_tet_mesh, read_gmsh_v2, waveguide_mesh, write_gmsh_v2  # noqa: F401

__version__ = "0.1.0"
