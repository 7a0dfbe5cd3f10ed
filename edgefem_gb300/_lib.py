"""ctypes binding of libedgefem_gb300.so (include/edgefem_gb300.h).

Loading fails loudly: if the in-tree library is missing the import raises,
there is no pure-Python or CPU stand-in for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libedgefem_gb300.so"

i32, i64, f64 = C.c_int32, C.c_int64, C.c_double
P = C.POINTER


class PortMode(C.Structure):
    _fields_ = [("fc", f64), ("kc", f64), ("omega", f64), ("eps", f64 * 2), ("mu", f64 * 2),
                ("beta", f64 * 2), ("Z0", f64 * 2)]


class WavePortC(C.Structure):
    _fields_ = [("surface_tag", i32), ("n_edges", i64), ("edges", P(i32)), ("weights", P(f64)),
                ("mode", PortMode)]


class MaxwellParamsC(C.Structure):
    _fields_ = [("omega", f64), ("eps_r", f64 * 2), ("mu_r", f64 * 2),
                ("n_eps_regions", i32), ("eps_region_tags", P(i32)), ("eps_region_vals", P(f64)),
                ("n_mu_regions", i32), ("mu_region_tags", P(i32)), ("mu_region_vals", P(f64)),
                ("n_debye", i32), ("debye_tags", P(i32)), ("debye_params", P(f64)),
                ("eps_tet", P(f64)), ("use_abc", i32), ("n_abc_tags", i32), ("abc_tags", P(i32)),
                ("port_abc_scale", f64), ("use_port_abc", i32), ("port_abc_type", i32)]


class VTKOptionsC(C.Structure):
    _fields_ = [("export_magnitude", i32), ("export_phase", i32), ("export_real", i32), ("export_imag", i32),
                ("export_vector", i32)]


class SolveOptionsC(C.Structure):
    _fields_ = [("use_bicgstab", i32), ("use_direct", i32), ("tolerance", f64),
                ("max_iterations", i32), ("verbose", i32), ("preconditioner", i32), ("use_ilut", i32)]


class SolveResultC(C.Structure):
    _fields_ = [("iters", i32), ("residual", f64), ("converged", i32), ("method", C.c_char * 64),
                ("error_message", C.c_char * 160)]


class BatchInstanceC(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("params", MaxwellParamsC), ("pec", P(i32)), ("n_pec", i64),
                ("ports", P(WavePortC)), ("n_ports", i32)]


class BatchOptionsC(C.Structure):
    _fields_ = [("tolerance", f64), ("max_iterations", i32), ("refine_interval", i32),
                ("rows_per_block", i32), ("use_graph", i32), ("verbose", i32), ("time_spmm", i32),
                ("precision", i32), ("formulation", i32), ("vector_aux", i32), ("reorder", i32),
                ("rb_samples", i32)]


class BatchStatsC(C.Structure):
    _fields_ = [("solve_ms", f64), ("setup_ms", f64), ("max_iters", i32), ("min_iters", i32),
                ("n_converged", i32), ("n_total", i32), ("max_residual", f64), ("spmm_launches", i64),
                ("spmm_ms", f64), ("spmm_timed", i64), ("kernel_launches", i64), ("rb_samples", i32),
                ("rb_basis", i32), ("rb_done_at_guess", i32), ("rb_reserved", i32), ("rb_ms", f64), ("rb_sample_ms", f64)]


# name -> (restype, argtypes)
_SIGS = {
    "efg_last_error": (C.c_char_p, []),
    "efg_abi_version": (C.c_int, []),
    "efg_device_count": (C.c_int, []),
    "efg_mesh_create": (C.c_int, [P(i64), P(f64), i64, P(i64), P(i32), i64, P(i64), P(i32), i64, P(C.c_void_p)]),
    "efg_mesh_load_gmsh_v2": (C.c_int, [C.c_char_p, P(C.c_void_p)]),
    "efg_mesh_destroy": (None, [C.c_void_p]),
    "efg_mesh_sizes": (C.c_int, [C.c_void_p, P(i64), P(i64), P(i64), P(i64)]),
    "efg_mesh_arrays": (C.c_int, [C.c_void_p, P(i64), P(f64), P(i64), P(i32), P(i64), P(i32)]),
    "efg_mesh_topology": (C.c_int, [C.c_void_p, P(i64), P(i32), P(C.c_int8), P(i32), P(C.c_int8)]),
    "efg_validate_mesh_gpu": (C.c_int, [C.c_void_p, P(i32), P(i32), P(C.c_double), P(C.c_double), P(C.c_int8),
                                        P(C.c_double)]),
    "efg_build_edges_gpu": (C.c_int, [i64, P(i64), i64, P(i32), i64, P(i32), P(i64), P(i32), P(C.c_int8),
                                      P(i32), P(C.c_int8), P(i64), P(C.c_double)]),
    "efg_validate_mesh": (C.c_int, [C.c_void_p, P(i32), P(i32), P(f64), P(f64)]),
    "efg_build_edge_pec": (C.c_int, [C.c_void_p, C.c_int, P(i32), i64, P(i64)]),
    "efg_pattern": (C.c_int, [C.c_void_p, P(i32), P(i32), P(i64), P(i32)]),
    "efg_element_matrices": (C.c_int, [P(f64), P(f64), P(f64)]),
    "efg_triangle_mass": (C.c_int, [P(f64), P(f64)]),
    "efg_solve_te10_mode": (C.c_int, [f64, f64, f64, P(PortMode)]),
    "efg_build_wave_port_2d": (C.c_int, [C.c_void_p, C.c_int, P(PortMode), P(i32), i64, f64, P(i32), P(f64),
                                         i64, P(i64), P(f64)]),
    "efg_build_lumped_port": (C.c_int, [C.c_void_p, C.c_int, f64, P(f64), C.c_int, P(i32), P(f64), i64, P(i64)]),
    "efg_maxwell_params_default": (None, [P(MaxwellParamsC)]),
    "efg_solve_options_default": (None, [P(SolveOptionsC)]),
    "efg_spmat_create": (C.c_int, [i32, i64, P(i32), P(i32), P(f64), P(C.c_void_p)]),
    "efg_spmat_info": (C.c_int, [C.c_void_p, P(i32), P(i64)]),
    "efg_spmat_export": (C.c_int, [C.c_void_p, P(i32), P(i32), P(f64)]),
    "efg_spmat_destroy": (None, [C.c_void_p]),
    "efg_assemble_maxwell": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(WavePortC), i32, i32,
                                       P(C.c_void_p), P(f64)]),
    "efg_solve_linear": (C.c_int, [C.c_void_p, P(f64), P(SolveOptionsC), P(f64), P(SolveResultC)]),
    "efg_calculate_sparams": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(WavePortC), i32,
                                        P(SolveOptionsC), P(f64)]),
    "efg_normalize_port_weights": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(WavePortC), i32,
                                             P(SolveOptionsC)]),
    "efg_calculate_sparams_eigenmode": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(WavePortC), i32,
                                                  P(SolveOptionsC), P(f64), P(SolveResultC)]),
    "efg_assemble_maxwell_km": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(C.c_void_p),
                                          P(C.c_void_p)]),
    "efg_frequency_sweep": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(WavePortC), i32, P(f64), i32,
                                      P(SolveOptionsC), P(f64)]),
    "efg_frequency_sweep_batched": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(WavePortC), i32,
                                              P(f64), i32, P(BatchOptionsC), P(f64), P(BatchStatsC)]),
    "efg_batch_options_default": (None, [P(BatchOptionsC)]),
    "efg_krylov_totals": (None, [i32, P(i64), P(i32), P(f64), P(f64)]),
    "efg_sparams_eigenmode_batched": (C.c_int, [P(BatchInstanceC), i32, P(f64), i32, P(BatchOptionsC), P(f64),
                                                P(BatchStatsC)]),
    "efg_batch_create": (C.c_int, [P(BatchInstanceC), i32, P(f64), i32, P(BatchOptionsC), P(C.c_void_p)]),
    "efg_batch_solve": (C.c_int, [C.c_void_p, P(f64), P(BatchStatsC)]),
    "efg_batch_info": (C.c_int, [C.c_void_p, P(i64), P(i64), P(i32), P(i32)]),
    "efg_batch_destroy": (None, [C.c_void_p]),
    "efg_transfer_counters": (None, [P(i64), P(i64)]),
    "efg_batch_rhs_stats": (C.c_int, [C.c_void_p, P(i32), P(i32), P(f64)]),
    "efg_sparams_eigenmode_adjoint": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(WavePortC), i32,
                                                i32, i32, P(SolveOptionsC), P(f64), P(f64)]),
    "efg_sparams_driven_adjoint": (C.c_int, [C.c_void_p, P(MaxwellParamsC), P(i32), i64, P(WavePortC), i32,
                                                i32, i32, P(SolveOptionsC), P(f64), P(f64)]),
    "efg_compute_barycentric": (C.c_int, [P(f64), P(f64), P(f64)]),
    "efg_evaluate_edge_field": (C.c_int, [P(f64), P(i32), P(f64), P(f64), P(f64)]),
    "efg_evaluate_field": (C.c_int, [C.c_void_p, P(f64), i64, P(i32), P(f64), P(f64)]),
    "efg_vtk_options_default": (None, [P(VTKOptionsC)]),
    "efg_export_fields_vtk": (C.c_int, [C.c_void_p, P(f64), C.c_char_p, P(VTKOptionsC), i32]),
    "efg_compute_coupling": (C.c_int, [i32, P(f64), f64, f64, P(f64), P(f64)]),
    "efg_mutual_coupling_db": (C.c_int, [i32, P(f64), P(f64)]),
    "efg_active_reflection": (C.c_int, [i32, P(f64), P(f64), P(f64)]),
    "efg_is_passive": (C.c_int, [i32, P(f64), f64]),
    "efg_check_passivity": (C.c_int, [i32, P(f64), f64]),
    "efg_is_lossless": (C.c_int, [i32, P(f64), f64]),
    "efg_is_reciprocal": (C.c_int, [i32, P(f64), f64]),
    "efg_singular_values": (C.c_int, [i32, P(f64), P(f64)]),
    "efg_write_touchstone_nport": (C.c_int, [C.c_char_p, i32, P(f64), i32, P(f64), i32, f64]),
    "efg_write_touchstone": (C.c_int, [C.c_char_p, i32, P(f64), P(f64)]),
    "efg_touchstone_extension": (C.c_int, [i32, C.c_char_p, i32]),
}


class EdgefemError(RuntimeError):
    pass


def _load():
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH.name} is not built; run `python edgefem_gb300/build.py` "
            "(there is no CPU fallback for this package)")
    lib = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_GLOBAL", 0))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(rc: int, what: str = "") -> int:
    """Raise EdgefemError on rc < 0 (message from efg_last_error)."""
    if rc < 0:
        msg = lib.efg_last_error().decode(errors="replace")
        raise EdgefemError(f"{what}: {msg}" if what else msg)
    return rc


def ptr(arr, ctype):
    """ctypes pointer to a contiguous numpy array (None for None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(P(ctype))
