"""ctypes bridge to the CPU oracle (test infrastructure only).

Drives ``liborc.so`` (built by ``oracle/build.py``) with the same phase
sequence as the GPU library so that the two can be compared field by field.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from . import build as _build

_LIBS: Dict[tuple, C.CDLL] = {}

_f64 = C.c_double
_i64 = C.c_int64


def lib(checked: bool = True, dual: bool = False) -> C.CDLL:
    key = (checked, dual)
    if key not in _LIBS:
        L = C.CDLL(str(_build.build(checked=checked, dual=dual)))
        L.orc_lanes.restype = C.c_int
        L.orc_set_fd.argtypes = [_i64, C.c_char_p, C.c_int, _f64]
        L.orc_get_fd.restype = _f64
        L.orc_get_fd.argtypes = [_i64, C.c_char_p, C.c_int]
        L.orc_arg_tangent.argtypes = [C.c_char_p, C.c_int, _f64]
        L.orc_block_new.restype = _i64
        L.orc_block_new.argtypes = [_i64, _i64, _i64]
        L.orc_alloc_surface.argtypes = [_i64, _i64, _i64]
        L.orc_array.restype = C.c_void_p
        L.orc_array.argtypes = [_i64, C.c_char_p, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(C.c_int)]
        L.orc_set_f.argtypes = [_i64, C.c_char_p, _f64]
        L.orc_get_f.restype = _f64
        L.orc_get_f.argtypes = [_i64, C.c_char_p]
        L.orc_set_i.argtypes = [_i64, C.c_char_p, _i64]
        L.orc_get_i.restype = _i64
        L.orc_get_i.argtypes = [_i64, C.c_char_p]
        L.orc_err.argtypes = [_i64]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        L.orc_interface_new.restype = _i64
        L.orc_interface_new.argtypes = [_i64, _i64, _i64, _i64] + [_f64] * 6
        L.orc_interface_table.restype = C.POINTER(_i64)
        L.orc_interface_table.argtypes = [_i64, C.c_char_p, C.POINTER(_i64), C.POINTER(_i64)]
        for name, args in {
            "orc_derive_grids": [_i64], "orc_non_uni_coeff": [_i64],
            "orc_coefficient_matrix": [_i64, C.c_int], "orc_ns_momentum": [_i64, _f64, _f64],
            "orc_velocity_bc": [_i64, _f64, _f64], "orc_solid_cell_bc": [_i64],
            "orc_solid_cell_bc_move": [_i64], "orc_velocity_forcing1": [_i64],
            "orc_pressure_forcing1": [_i64], "orc_velocity_forcing_field": [_i64],
            "orc_pressure_forcing_field": [_i64], "orc_velocity_forcing_ghost": [_i64],
            "orc_pressure_forcing_ghost": [_i64], "orc_compute_surface_norm": [_i64, _i64],
            "orc_node_ids_from_elements": [_i64],
            "orc_find_dist_node": [_i64],
            "orc_block_move_stage": [],
            "orc_tagging_th_move": [_i64],
            "orc_shift_surface_nodes_initial": [_i64, _f64, _f64, _i64, _f64, _f64, _f64],
            "orc_compute_surface_variables": [_i64, _f64, _f64, _i64, _f64, _f64, _f64, _f64],
            "orc_tagging_th_core": [_i64], "orc_selective_retagging": [_i64],
            "orc_cellcount_solid": [_i64], "orc_cellcount_solid_coarse": [_i64],
            "orc_compute_norm_distance": [_i64], "orc_find_ts_cells": [_i64],
            "orc_update_velocity_newv": [_i64], "orc_compute_div": [_i64],
            "orc_correct_pressure": [_i64], "orc_correct_velocity": [_i64, _f64],
            "orc_redblack_sor": [_i64, _i64, _f64, _f64],
            "orc_poisson_solver": [_i64, _f64, _f64, _f64], "orc_fine_update_bd_mv": [_i64],
            "orc_fine_update_mv": [_i64], "orc_stress_calculation": [_i64, _f64, _f64],
        }.items():
            getattr(L, name).argtypes = args
        _LIBS[key] = L
    return _LIBS[key]


class Oracle:
    """One oracle instance (the oracle keeps module-global block/interface lists)."""

    def __init__(self, checked: bool = True, dual: bool = False):
        """``dual``: the tangent-linear build (``orc_lanes()`` tangents next
        to every value; ``arr`` then returns the value part, ``tangent`` a
        lane's tangent part, both as views into the oracle's storage)."""
        self.L = lib(checked, dual)
        self.lanes = int(self.L.orc_lanes())
        self.L.orc_reset()
        self.L.orc_clear_arg_tangents()
        # {(block, scalar name): [(lane, tangent)]}: seeds applied whenever
        # setf sets that scalar (set-up sets the motion parameters)
        self.scalar_seeds: Dict[tuple, list] = {}
        self.nblocks = 0
        self.case = None

    # ---- raw access -------------------------------------------------------
    def arr(self, g: int, name: str) -> np.ndarray:
        return self._view(g, name, 0)

    def tangent(self, g: int, name: str, lane: int) -> np.ndarray:
        """Lane ``lane``'s tangent of a floating-point array (dual build)."""
        assert 0 <= lane < self.lanes, lane
        return self._view(g, name, 1 + lane)

    def _view(self, g: int, name: str, part: int) -> np.ndarray:
        n, kind = _i64(), C.c_int()
        dims = (_i64 * 3)()
        p = self.L.orc_array(g, name.encode(), C.byref(n), dims, C.byref(kind))
        if not p:
            raise KeyError(name)
        shape = [int(d) for d in dims]
        while len(shape) > 1 and shape[-1] == 1:
            shape.pop()
        shape = tuple(shape)
        if n.value == 0:
            return np.zeros(shape, dtype=np.int64 if kind.value == 1 else np.float64, order="F")
        if kind.value == 2:
            # dual numbers: (1 + lanes) doubles per element, value first
            w = 1 + self.lanes
            buf = (_f64 * (n.value * w)).from_address(p)
            full = np.ndarray((w,) + shape, dtype=np.float64, buffer=buf, order="F")
            return full[part]
        assert part == 0, "tangents exist in the dual build only"
        ct = _f64 if kind.value == 0 else _i64
        buf = (ct * n.value).from_address(p)
        return np.ndarray(shape, dtype=np.float64 if kind.value == 0 else np.int64, buffer=buf, order="F")

    def geti(self, g, name):
        return int(self.L.orc_get_i(g, name.encode()))

    def getf(self, g, name):
        return float(self.L.orc_get_f(g, name.encode()))

    def seti(self, g, name, v):
        assert self.L.orc_set_i(g, name.encode(), int(v)) == 0, name

    def setf(self, g, name, v):
        assert self.L.orc_set_f(g, name.encode(), float(v)) == 0, name
        for lane, d in self.scalar_seeds.get((g, name), ()):
            self.setf_tangent(g, name, lane, d)

    def setf_tangent(self, g, name, lane, d):
        assert self.L.orc_set_fd(g, name.encode(), int(lane), float(d)) == 0, name

    def getf_tangent(self, g, name, lane):
        return float(self.L.orc_get_fd(g, name.encode(), int(lane)))

    def seed_arg(self, name, lane, d):
        """Tangent ``d`` in lane ``lane`` of a call argument ("uc",
        "phase_angle", "freq", "aoa", "piv_pt") for every later call."""
        assert self.L.orc_arg_tangent(name.encode(), int(lane), float(d)) == 0, name

    def err(self, g) -> int:
        return int(self.L.orc_err(g))

    def table(self, ih: int, name: str):
        ncols, cnt = _i64(), _i64()
        p = self.L.orc_interface_table(ih, name.encode(), C.byref(ncols), C.byref(cnt))
        a = np.ctypeslib.as_array(p, shape=(ncols.value, 3)).T.copy()
        return a, int(cnt.value)

    # ---- setup mirroring app/main.F90:43-127 ------------------------------
    def setup(self, case, with_fields: bool = True):
        L = self.L
        self.case = case
        for spec in case.blocks:
            g = L.orc_block_new(spec.nx, spec.ny, spec.nz)
            self.arr(g, "x1")[1:spec.nx + 2] = spec.x_faces
            self.arr(g, "y1")[1:spec.ny + 2] = spec.y_faces
            self.arr(g, "z1")[1:spec.nz + 2] = spec.z_faces
            L.orc_derive_grids(g)
            self.setf(g, "omega", spec.omega)
            self.setf(g, "dx", spec.x_faces[1] - spec.x_faces[0])
            self.setf(g, "dy", spec.y_faces[1] - spec.y_faces[0])
            self.setf(g, "dz", spec.z_faces[1] - spec.z_faces[0])
            for nm, v in (("xdot", spec.xdot), ("ydot", spec.ydot), ("yddot", spec.yddot),
                          ("piv_x", spec.piv[0]), ("piv_y", spec.piv[1]), ("piv_z", spec.piv[2])):
                self.setf(g, nm, v)
            if spec.has_body:
                m = spec.mesh
                L.orc_alloc_surface(g, len(m.tris), len(m.nodes))
                self.arr(g, "xnode1")[:] = m.nodes[:, 0]
                self.arr(g, "ynode1")[:] = m.nodes[:, 1]
                self.arr(g, "znode1")[:] = m.nodes[:, 2]
                self.arr(g, "ibElP1")[:] = m.tris[:, 0]
                self.arr(g, "ibElP2")[:] = m.tris[:, 1]
                self.arr(g, "ibElP3")[:] = m.tris[:, 2]
                self.arr(g, "ibSurfId")[:] = m.surf_id
                if spec.motion is not None:
                    # app/main.F90:64-69: body-frame nodes, initial placement
                    mo, mi = spec.motion, case.motion
                    self.arr(g, "xnode")[:] = m.nodes[:, 0]
                    self.arr(g, "ynode")[:] = m.nodes[:, 1]
                    self.arr(g, "znode")[:] = m.nodes[:, 2]
                    L.orc_node_ids_from_elements(g)
                    L.orc_find_dist_node(g)
                    for nm, v in (("a0", mo.a0_deg), ("bfreq", mo.bfreq), ("yamp", mo.yamp),
                                  ("xshift", mo.shift[0]), ("yshift", mo.shift[1]), ("zshift", mo.shift[2])):
                        self.setf(g, nm, v)
                    if mo.lag_deg != 0.0:
                        self.setf(g, "lag", mo.lag_deg * np.pi / 180.0)
                        self.setf(g, "lag_phase", mi.phase_deg * np.pi / 180.0)
                    L.orc_shift_surface_nodes_initial(g, mi.aoa_deg, mi.piv_pt, 0, case.dt, mi.dxmin, 0.0)
                for nm, v in zip(("i_startSearch", "i_endSearch", "j_startSearch", "j_endSearch",
                                  "k_startSearch", "k_endSearch"), spec.search_box):
                    self.seti(g, nm, v)
                L.orc_compute_surface_norm(g, m.inor)
        self.nblocks = len(case.blocks)
        for it in case.interfaces:
            L.orc_interface_new(it.a_blk, it.b_blk, it.a_msh, it.b_msh, *it.box)
        for g, spec in enumerate(case.blocks, 1):
            # app/main.F90:80-85: every block g /= 1 is tagged and counted (a
            # block without a surface is all fluid)
            if spec.has_body or (g != 1 and case.interfaces):
                L.orc_tagging_th_core(g)
                L.orc_cellcount_solid(g)
        if case.interfaces and not case.blocks[0].has_body:
            L.orc_fine_block_cell()
            L.orc_cellcount_solid_coarse(1)
        if not case.interfaces and not case.blocks[0].has_body:
            # a lone block without a body (not a configuration main.F90
            # builds): tagged all fluid and counted like a fine block
            L.orc_tagging_th_core(1)
            L.orc_cellcount_solid(1)
        if with_fields:
            for g, ini in enumerate(case.init, 1):
                for nm in ("u", "v", "w", "p"):
                    self.arr(g, nm)[...] = ini[nm]
                for nm in ("u", "v", "w"):
                    self.arr(g, nm + "t")[...] = ini[nm]
        for g, spec in enumerate(case.blocks, 1):
            if spec.has_body:
                L.orc_compute_norm_distance(g)
                L.orc_find_ts_cells(g)
            L.orc_coefficient_matrix(g, 1 if spec.is_coarse else 0)
        for g in range(1, self.nblocks + 1):
            L.orc_non_uni_coeff(g)
        # app/main.F90:45-46, 119: the time counters of the loop
        self.ita = 0
        self.totime = case.dt

    # ---- one time step, the phase order of app/main.F90:129-265 ------------
    def momentum_phase(self):
        c, L = self.case, self.L
        for g, spec in enumerate(c.blocks, 1):
            L.orc_ns_momentum(g, c.dt, c.re)
            if spec.is_coarse:
                L.orc_velocity_bc(g, c.dt, c.uc)
            if spec.has_body:
                L.orc_solid_cell_bc(g)
                L.orc_velocity_forcing1(g)
            if spec.is_coarse:
                L.orc_velocity_bc(g, c.dt, c.uc)

    def poisson_phase(self):
        c = self.case
        self.L.orc_poisson_solver(c.pc_ita_max, c.epsi, c.dt, c.uc)

    def research_phase(self):
        L, c = self.L, self.case
        for g, spec in enumerate(self.case.blocks, 1):
            if spec.has_body:
                L.orc_pressure_forcing1(g)
        # app/main.F90:169-230: moving bodies, the fine-block moves, the
        # surface normals, the re-tagging of moved blocks
        for g, spec in enumerate(self.case.blocks, 1):
            if spec.motion is not None:
                mi = c.motion
                self.seti(g, "blk_mv_tag", 0)
                L.orc_compute_surface_variables(g, mi.phase_deg * np.pi / 180.0, mi.piv_pt, self.ita, c.dt,
                                                mi.dxmin, mi.freq, self.totime)
        moving = c.motion is not None and any(s.motion is not None for s in self.case.blocks)
        if moving and c.interfaces:
            L.orc_block_move_stage()
        for g, spec in enumerate(self.case.blocks, 1):
            if spec.motion is not None:
                L.orc_compute_surface_norm(g, spec.mesh.inor)
        if moving and c.interfaces:
            for g in range(2, self.nblocks + 1):
                L.orc_tagging_th_move(g)
        for g, spec in enumerate(self.case.blocks, 1):
            if not spec.has_body:
                continue
            # app/main.F90:238-239: a block that moved this step was re-tagged
            # whole by tagging_th_move (blk_mv_tag = 1 skips the selective pass)
            L.orc_selective_retagging(g)
            self.seti(g, "blk_mv_tag", 0)
            L.orc_cellcount_solid(g)
            L.orc_solid_cell_bc_move(g)
            L.orc_update_velocity_newv(g)
            self.seti(g, "move_check", 0)
            L.orc_compute_norm_distance(g)
            L.orc_find_ts_cells(g)
            L.orc_velocity_forcing_field(g)
            L.orc_pressure_forcing_field(g)
            L.orc_velocity_forcing_ghost(g)
            L.orc_pressure_forcing_ghost(g)

    def step(self):
        # app/main.F90:130-131
        self.ita += 1
        self.totime += self.case.dt
        self.momentum_phase()
        self.poisson_phase()
        self.research_phase()

    def iters(self):
        return [self.geti(g, "nIterPcor") for g in range(1, self.nblocks + 1)]


# tangent lanes of drag_objective: the five motion parameters of the moving
# body (pitch and phase in degrees) and the inflow velocity
TANGENT_PARAMS = ("yamp", "a0_deg", "phase_deg", "freq", "bfreq", "uc")
STRESS_NAMES = ("viscous_drag", "pressure_drag", "viscous_lift", "pressure_lift")


def drag_objective(case, n_steps: int, block: int, stress_seed, mu_f: float, rho_f: float, dual: bool = False):
    """J = (1/n_steps) sum over the steps of sum_t stress_seed[t] * C_t, C_t
    the drag/lift coefficients of ``block`` (0-based) after each step, from
    a run of the oracle from the set-up.  With ``dual`` the run is the FP64
    tangent-linear model (the dual-number build) and the result is (J,
    {name: dJ/d name for TANGENT_PARAMS}); otherwise J."""
    o = Oracle(dual=dual)
    g = block + 1
    nl = len(TANGENT_PARAMS) if dual else 0
    if dual:
        assert o.lanes >= nl, o.lanes
        o.scalar_seeds = {(g, "yamp"): [(0, 1.0)], (g, "a0"): [(1, 1.0)], (g, "bfreq"): [(4, 1.0)]}
        o.seed_arg("phase_angle", 2, np.pi / 180.0)
        o.seed_arg("freq", 3, 1.0)
        o.seed_arg("uc", 5, 1.0)
    o.setup(case)
    J = 0.0
    dJ = np.zeros(nl)
    for _ in range(n_steps):
        o.step()
        o.L.orc_stress_calculation(g, mu_f, rho_f)
        for t, nm in enumerate(STRESS_NAMES):
            J += stress_seed[t] * o.getf(g, nm)
            if dual:
                dJ += stress_seed[t] * np.array([o.getf_tangent(g, nm, l) for l in range(nl)])
    for g2 in range(1, o.nblocks + 1):
        assert o.err(g2) == 0, (g2, o.err(g2))
    if not dual:
        return J / n_steps
    return J / n_steps, dict(zip(TANGENT_PARAMS, dJ / n_steps))
