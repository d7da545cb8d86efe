"""Loader of the in-tree C-ABI library ``libbiocfd_gb300.so``.

The library is the product: there is no fallback.  If it is missing this
module builds it (``bio-cfd_gb300/build.py``, nvcc for sm_103a); if it cannot
be built or loaded, import fails loudly.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
from pathlib import Path

_PKG = Path(__file__).resolve().parent.parent
_LIB = None

c_double = C.c_double
c_i64 = C.c_int64
c_int = C.c_int
P_d = C.POINTER(C.c_double)
P_i64 = C.POINTER(C.c_int64)


class BcfdError(RuntimeError):
    pass


# bcfd_status of include/biocfd_gb300.h
BCFD_OK = 0
BCFD_E_HANDLE = -1
BCFD_E_NOMEM = -2
BCFD_E_NONFINITE = -3
BCFD_E_NOTFOUND = -4
BCFD_E_TIMEOUT = -5
BCFD_E_ARG = -6
BCFD_E_CUDA = -7
BCFD_E_STATE = -8
BCFD_E_CAPACITY = -9


class StepConfig(C.Structure):
    """bcfd_step_config of include/biocfd_gb300.h."""
    _fields_ = [("deltat", c_double), ("re", c_double), ("uc", c_double), ("epsi", c_double),
                ("pc_ita_max", c_i64), ("precision", c_int), ("div_tol", c_double),
                ("use_graph", c_int)]


class ProfileReport(C.Structure):
    """bcfd_profile_report of include/biocfd_gb300.h."""
    _fields_ = [("sor_launches", c_i64), ("sor_ms", c_double), ("sor_bytes", c_double),
                ("sor_sweeps", c_i64), ("kernel_launches", c_i64)]


_SIGS = {
    "bcfd_block_get_divergence": [c_i64, P_d],
    "bcfd_block_set_mixed_params": [c_i64, c_i64, c_double, c_int],
    "bcfd_block_get_mixed_omega": [c_i64, P_d],
    "bcfd_block_set_solve_launch": [c_i64, c_int, c_int, c_int],
    "bcfd_set_batching": [c_int],
    "bcfd_set_warm_start": [c_int],
    "bcfd_set_wait_limit_ns": [c_i64],
    "bcfd_check_wait_limit": [C.POINTER(c_int), P_d],
    "bcfd_block_set_list_capacity": [c_i64, c_i64],
    "bcfd_adjoint_set_solver": [c_int],
    "bcfd_poisson_solve_zero_bc": [c_i64, P_d, P_d, c_double, c_i64],
    "bcfd_poisson_solve_adjoint": [c_i64, P_d, P_d, c_double, c_i64],
    "bcfd_coupling_apply": [c_i64, c_int, c_int, P_d, P_d],
    "bcfd_momentum_tangent": [c_i64, c_double, c_double, P_d, P_d, P_d, P_d, P_d, P_d, P_d, P_d, P_d, P_d],
    "bcfd_momentum_adjoint": [c_i64, c_double, c_double, P_d, P_d, P_d, P_d, P_d, P_d, P_d],
    "bcfd_momentum_adjoint_ts": [c_i64, c_double, c_double, P_d, P_d, P_d, P_d, P_d, P_d, P_d, P_d],
    "bcfd_forcing_ghost_adjoint": [c_i64, P_d, P_d, P_d, P_d, P_d, P_d, P_d, P_d],
    "bcfd_adjoint_run": [c_i64, C.POINTER(StepConfig), c_i64, c_i64, P_d, P_d, P_d, P_d, P_d, c_double, c_double,
                         c_double, c_i64, P_d, P_d, P_d, P_d, P_d, P_d, P_d],
    "bcfd_adjoint_run_motion": [c_i64, C.POINTER(StepConfig), c_i64, c_i64, P_d, P_d, P_d, P_d, P_d, c_double,
                                c_double, c_double, c_i64, P_d, P_d, P_d, P_d, P_d, P_d, P_d],
    "bcfd_block_set_body_motion": [c_i64, P_d],
    "bcfd_shift_surface_nodes_initial": [c_i64, c_double, c_double, c_i64, c_double, c_double, c_double],
    "bcfd_block_set_body_lag": [c_i64, c_double, c_double],
    "bcfd_compute_surface_variables": [c_i64, c_double, c_double, c_i64, c_double, c_double, c_double,
                                       c_double],
    "bcfd_set_motion_inputs": [c_double, c_double, c_double, c_double, c_i64, c_i64, c_double],
    "bcfd_get_time": [C.POINTER(c_i64), P_d],
    "bcfd_block_get_solve_launch": [c_i64, C.POINTER(c_int)],
    "bcfd_autotune": [C.POINTER(c_i64)],
    "bcfd_block_sor_sweeps": [c_i64, c_i64, c_int],
    "bcfd_profile_begin": [],
    "bcfd_profile_end": [C.POINTER(ProfileReport)],
    "bcfd_profile_phases": [P_d, c_int],
    "bcfd_measure_alu_rates": [P_d],
    "bcfd_init": [c_int], "bcfd_finalize": [], "bcfd_synchronize": [],
    "bcfd_get_stream": [C.POINTER(C.c_void_p)],
    "bcfd_block_create": [c_i64, c_i64, c_i64, P_d, P_d, P_d, P_d, P_d, P_d, P_i64],
    "bcfd_block_destroy": [c_i64],
    "bcfd_block_set_grid": [c_i64, P_d, P_d, P_d],
    "bcfd_block_set_scalars": [c_i64, c_double, c_double, c_double, c_double],
    "bcfd_block_set_search_box": [c_i64] + [c_i64] * 6,
    "bcfd_block_set_surface": [c_i64, c_i64, c_i64, P_i64, P_i64, P_i64, P_i64, P_d, P_d, P_d],
    "bcfd_block_set_nodes": [c_i64, P_d, P_d, P_d],
    "bcfd_block_set_kinematics": [c_i64, P_d],
    "bcfd_block_set_flags": [c_i64, c_i64, c_i64],
    "bcfd_block_set_role": [c_i64, c_int, c_int],
    "bcfd_block_upload_fields": [c_i64] + [P_d] * 7,
    "bcfd_block_download_fields": [c_i64] + [P_d] * 7,
    "bcfd_block_upload_tags": [c_i64] + [P_i64] * 5,
    "bcfd_block_download_tags": [c_i64] + [P_i64] * 5,
    "bcfd_block_get_counts": [c_i64, P_i64],
    "bcfd_block_get_sor_stats": [c_i64, P_i64, P_d, P_d],
    "bcfd_block_set_sor_iter": [c_i64, c_i64],
    "bcfd_block_read": [c_i64, C.c_char_p, C.c_void_p, c_i64, P_i64],
    "bcfd_block_write": [c_i64, C.c_char_p, P_d, c_i64],
    "bcfd_non_uni_coeff": [c_i64], "bcfd_coefficient_matrix": [c_i64, c_int],
    "bcfd_ns_momentum_2order": [c_i64, c_double, c_double],
    "bcfd_velocity_bc": [c_i64, c_double, c_double],
    "bcfd_solid_cell_bc": [c_i64], "bcfd_solid_cell_bc_move": [c_i64],
    "bcfd_velocity_forcing1": [c_i64], "bcfd_pressure_forcing1": [c_i64],
    "bcfd_velocity_forcing_field": [c_i64], "bcfd_pressure_forcing_field": [c_i64],
    "bcfd_velocity_forcing_ghost": [c_i64], "bcfd_pressure_forcing_ghost": [c_i64],
    "bcfd_compute_surface_norm": [c_i64, c_i64], "bcfd_tagging_th": [c_i64],
    "bcfd_selective_retagging_th": [c_i64], "bcfd_cellcount_solid": [c_i64],
    "bcfd_compute_norm_distance": [c_i64], "bcfd_find_ts_cells": [c_i64],
    "bcfd_cellcount_solid_coarse": [c_i64], "bcfd_fine_block_cell": [],
    "bcfd_compute_div": [c_i64], "bcfd_correct_pressure": [c_i64],
    "bcfd_correct_velocity": [c_i64, c_double],
    "bcfd_redblack_sor_linear": [c_i64, c_i64, c_double, c_double],
    "bcfd_update_velocity_newv": [c_i64],
    "bcfd_poisson_solver": [c_i64, c_double, c_i64, c_double, c_double, c_double, P_d, c_int, c_int, c_int],
    "bcfd_interface_create": [c_i64, c_i64, c_i64, c_i64, P_d, P_i64],
    "bcfd_interface_table": [c_i64, C.c_char_p, P_i64, c_i64, P_i64],
    "bcfd_fine_update_pc_bd": [], "bcfd_fine_update_newv_bd": [],
    "bcfd_fine_update_bd_mv": [c_i64], "bcfd_coarse_update": [],
    "bcfd_coarse_update_newv": [], "bcfd_coarse_update_pc": [],
    "bcfd_fine_update_mv": [c_i64],
    "bcfd_stress_calculation": [c_i64, c_double, c_double, P_d],
    "bcfd_stress_calculation_noalloc": [c_i64, c_double, c_double, P_d],
    "bcfd_run_steps": [C.POINTER(StepConfig), c_i64],
    "bcfd_block_move_stage": [P_i64],
    "bcfd_tagging_th_move": [c_i64],
    "bcfd_max_divergence": [c_i64, P_d],
}


def lib_path() -> Path:
    return _PKG / "lib" / "libbiocfd_gb300.so"


def _build_module():
    spec = importlib.util.spec_from_file_location("biocfd_gb300_build", _PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load(build_if_missing: bool = True):
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if build_if_missing:
        path = _build_module().build()
    if not path.exists():
        raise BcfdError(f"the CUDA library {path} is missing; run bio-cfd_gb300/build.py")
    L = C.CDLL(str(path))
    for name, args in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = c_int
    L.bcfd_status_string.restype = C.c_char_p
    L.bcfd_status_string.argtypes = [c_int]
    L.bcfd_kernel_launches.restype = c_i64
    L.bcfd_kernel_launches.argtypes = []
    _LIB = L
    return L


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = load().bcfd_status_string(status).decode()
        raise BcfdError(f"{what}: status {status} ({msg})")
