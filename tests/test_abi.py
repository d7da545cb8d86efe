"""The C-ABI library builds, loads and exports every symbol the header declares
(no compute calls: this runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "biocfd_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(bcfd_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert len(syms) > 50
    for must in ("bcfd_ns_momentum_2order", "bcfd_redblack_sor_linear", "bcfd_poisson_solver",
                 "bcfd_velocity_forcing1", "bcfd_selective_retagging_th", "bcfd_fine_update_newv_bd",
                 "bcfd_coarse_update_pc", "bcfd_run_steps"):
        assert must in syms


def test_library_exports_every_declared_symbol():
    from biocfd import _lib
    L = _lib.load()  # builds with nvcc if needed (cross-compiles without a GPU)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_status_strings_without_gpu():
    from biocfd import _lib
    L = _lib.load()
    assert L.bcfd_status_string(0) == b"ok"
    assert L.bcfd_status_string(-5) == b"device-side wait gave up"
    assert L.bcfd_kernel_launches() >= 0


def test_step_config_layout_matches_header():
    from biocfd._lib import StepConfig
    # deltat, re, uc, epsi (4 doubles) + pc_ita_max + precision(int, padded) + div_tol + use_graph
    assert C.sizeof(StepConfig) == 8 * 4 + 8 + 8 + 8 + 8


def test_fortran_shim_binds_only_declared_symbols():
    """Every C name the Fortran shim binds (bind(C, name=...)) is declared in
    the header, so the shim links against the library's exports."""
    shim = (ROOT / "bio-cfd_gb300" / "fortran" / "biocfd_gb300_shim.f90").read_text()
    bound = sorted(set(re.findall(r'name="(bcfd_[a-z0-9_]+)"', shim)))
    assert len(bound) > 30
    missing = [s for s in bound if s not in declared_symbols()]
    assert not missing, missing
    # the Search module carries the fine-block move sequence of app/main.F90
    for routine in ("block_move_check", "tagging_th_move", "selectiveRetagging_th", "computeSurfaceVariables"):
        assert re.search(rf"subroutine {routine}\b", shim), routine
