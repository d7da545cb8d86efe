"""GPU solver over the C ABI: block registration, the reference's set-up
sequence (app/main.F90:43-127) and the per-step phases (app/main.F90:129-265).

Every call goes to ``libbiocfd_gb300.so``; the Python layer only moves host
mirrors in and out and sequences the module routines like the reference's
driver does.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from . import _lib
from ._lib import P_d, P_i64, check
from .synth import Case


def _pd(a: np.ndarray):
    return a.ctypes.data_as(P_d)


def _pi(a: np.ndarray):
    return a.ctypes.data_as(P_i64)


def full_grid(faces: np.ndarray):
    """x1(1..n+3) and deltax(1..n+2) from the faces x1(2..n+2) (src/ReadInput.f90:254-268)."""
    n = len(faces) - 1
    x1 = np.zeros(n + 3)
    x1[1:n + 2] = faces
    d = np.zeros(n + 2)
    d[1:n + 1] = x1[2:n + 2] - x1[1:n + 1]
    d[0] = d[1]
    d[n + 1] = d[n]
    x1[0] = x1[1] - d[0]
    x1[n + 2] = x1[n + 1] + d[n + 1]
    return x1, d


class Solver:
    """All blocks and interfaces of one case on the GPU."""

    def __init__(self, case: Case, device: int = 0):
        # The library keeps one block registry per process (block 1 is the
        # coarse block, as in the reference); a new Solver starts a fresh one.
        self.L = _lib.load()
        check(self.L.bcfd_finalize(), "bcfd_finalize")
        check(self.L.bcfd_init(device), "bcfd_init")
        self.case = case
        self.handles: List[int] = []
        self.ifaces: List[int] = []

    # ---- set-up --------------------------------------------------------------
    def setup(self, with_fields: bool = True):
        L, case = self.L, self.case
        if self.handles:
            raise _lib.BcfdError("setup called twice")
        for spec in case.blocks:
            x1, dx = full_grid(spec.x_faces)
            y1, dy = full_grid(spec.y_faces)
            z1, dz = full_grid(spec.z_faces)
            h = C.c_int64()
            check(L.bcfd_block_create(spec.nx, spec.ny, spec.nz, _pd(x1), _pd(y1), _pd(z1), _pd(dx),
                                      _pd(dy), _pd(dz), C.byref(h)), "block_create")
            g = h.value
            self.handles.append(g)
            check(L.bcfd_block_set_scalars(g, dx[1], dy[1], dz[1], spec.omega), "set_scalars")
            check(L.bcfd_block_set_role(g, int(spec.is_coarse), int(spec.has_body)), "set_role")
            kin = np.array([spec.xdot, spec.ydot, spec.yddot, 0, 0, 0, 0, 0, *spec.piv], dtype=np.float64)
            check(L.bcfd_block_set_kinematics(g, _pd(kin)), "set_kinematics")
            if spec.has_body:
                m = spec.mesh
                tri = np.ascontiguousarray(m.tris, dtype=np.int64)
                e1, e2, e3 = (np.ascontiguousarray(tri[:, q]) for q in range(3))
                sid = np.ascontiguousarray(m.surf_id, dtype=np.int64)
                xs, ys, zs = (np.ascontiguousarray(m.nodes[:, q]) for q in range(3))
                check(L.bcfd_block_set_surface(g, len(tri), len(xs), _pi(e1), _pi(e2), _pi(e3), _pi(sid),
                                               _pd(xs), _pd(ys), _pd(zs)), "set_surface")
                check(L.bcfd_block_set_search_box(g, *spec.search_box), "set_search_box")
                if spec.motion is not None:
                    # app/main.F90:64-69: the nodes above are the body frame
                    mo, mi = spec.motion, case.motion
                    p = np.array([mo.a0_deg, mo.bfreq, mo.yamp, *mo.shift], dtype=np.float64)
                    check(L.bcfd_block_set_body_motion(g, _pd(p)), "set_body_motion")
                    if mo.lag_deg != 0.0:
                        check(L.bcfd_block_set_body_lag(g, mo.lag_deg * np.pi / 180.0, mi.phase_deg * np.pi / 180.0),
                              "set_body_lag")
                    check(L.bcfd_shift_surface_nodes_initial(g, mi.aoa_deg, mi.piv_pt, 0, case.dt, mi.dxmin, 0.0),
                          "shift_surface_nodes_initial")
                check(L.bcfd_compute_surface_norm(g, m.inor), "compute_surface_norm")
        for it in case.interfaces:
            box = np.asarray(it.box, dtype=np.float64)
            h = C.c_int64()
            check(L.bcfd_interface_create(self.handles[it.a_blk - 1], self.handles[it.b_blk - 1],
                                          it.a_msh, it.b_msh, _pd(box), C.byref(h)), "interface_create")
            self.ifaces.append(h.value)
        for q, (g, spec) in enumerate(zip(self.handles, case.blocks)):
            # app/main.F90:80-85: every block g /= 1 is tagged and counted (a
            # block without a surface is all fluid)
            if spec.has_body or (q > 0 and case.interfaces):
                check(L.bcfd_tagging_th(g), "tagging_th")
                check(L.bcfd_cellcount_solid(g), "cellcount_solid")
        if case.interfaces and not case.blocks[0].has_body:
            check(L.bcfd_fine_block_cell(), "fine_block_cell")
            check(L.bcfd_cellcount_solid_coarse(self.handles[0]), "cellcount_solid_coarse")
        if not case.interfaces and not case.blocks[0].has_body:
            # a lone block without a body (not a configuration main.F90
            # builds): tagged all fluid and counted like a fine block
            check(L.bcfd_tagging_th(self.handles[0]), "tagging_th")
            check(L.bcfd_cellcount_solid(self.handles[0]), "cellcount_solid")
        if with_fields:
            for g, ini in zip(self.handles, case.init):
                self.upload_fields(g, ini)
        for g, spec in zip(self.handles, case.blocks):
            if spec.has_body:
                check(L.bcfd_compute_norm_distance(g), "compute_norm_distance")
                check(L.bcfd_find_ts_cells(g), "find_ts_cells")
            check(L.bcfd_coefficient_matrix(g, int(spec.is_coarse)), "coefficient_matrix")
        for g in self.handles:
            check(L.bcfd_non_uni_coeff(g), "non_uni_coeff")
        # app/main.F90:45-46, 119: ita = 0 and totime = deltat when the loop starts
        mi = case.motion
        inor = next((b.mesh.inor for b in case.blocks if b.mesh is not None), 1)
        check(L.bcfd_set_motion_inputs((mi.phase_deg * np.pi / 180.0) if mi else 0.0, mi.piv_pt if mi else 0.0,
                                       mi.freq if mi else 0.0, mi.dxmin if mi else 0.0, inor, 0, case.dt),
              "set_motion_inputs")
        self.sync()

    def upload_fields(self, g: int, ini: dict):
        u, v, w, p = (np.asfortranarray(ini[k], dtype=np.float64) for k in ("u", "v", "w", "p"))
        check(self.L.bcfd_block_upload_fields(g, _pd(u), _pd(v), _pd(w), _pd(p), _pd(u), _pd(v), _pd(w)),
              "upload_fields")

    # ---- per-step phases (routine by routine, for parity checks) -------------
    def momentum_phase(self):
        L, c = self.L, self.case
        for g, spec in zip(self.handles, c.blocks):
            check(L.bcfd_ns_momentum_2order(g, c.dt, c.re), "ns_momentum_2order")
            if spec.is_coarse:
                check(L.bcfd_velocity_bc(g, c.dt, c.uc), "velocity_bc")
            if spec.has_body:
                check(L.bcfd_solid_cell_bc(g), "solid_cell_bc")
                check(L.bcfd_velocity_forcing1(g), "velocity_forcing1")
            if spec.is_coarse:
                check(L.bcfd_velocity_bc(g, c.dt, c.uc), "velocity_bc")

    def poisson_phase(self):
        c = self.case
        tt = C.c_double(0.0)
        check(self.L.bcfd_poisson_solver(c.pc_ita_max, c.epsi, 0, c.dt, 0.0, c.uc, C.byref(tt), 1,
                                         len(self.handles), 1), "poisson_solver")

    def research_phase(self):
        L, c = self.L, self.case
        for g, spec in zip(self.handles, self.case.blocks):
            if spec.has_body:
                check(L.bcfd_pressure_forcing1(g), "pressure_forcing1")
        # app/main.F90:169-230: moving bodies, the fine-block moves, the
        # surface normals, the re-tagging of moved blocks
        if c.motion is not None:
            ita, tt = self.time()
            for g, spec in zip(self.handles, self.case.blocks):
                if spec.motion is not None:
                    mi = c.motion
                    check(L.bcfd_block_set_flags(g, -1, 0), "set_flags")
                    check(L.bcfd_compute_surface_variables(g, mi.phase_deg * np.pi / 180.0, mi.piv_pt, ita, c.dt,
                                                           mi.dxmin, mi.freq, tt), "compute_surface_variables")
            if c.interfaces:
                moved = np.zeros(1, np.int64)
                check(L.bcfd_block_move_stage(_pi(moved)), "block_move_stage")
            for g, spec in zip(self.handles, self.case.blocks):
                if spec.motion is not None:
                    check(L.bcfd_compute_surface_norm(g, spec.mesh.inor), "compute_surface_norm")
            if c.interfaces:
                for g in self.handles[1:]:
                    check(L.bcfd_tagging_th_move(g), "tagging_th_move")
        for g, spec in zip(self.handles, self.case.blocks):
            if not spec.has_body:
                continue
            # main.F90:238-249: blk_mv_tag clears after the re-tagging,
            # move_check after the moved block's solid cells and ut = u
            check(L.bcfd_selective_retagging_th(g), "selective_retagging_th")
            check(L.bcfd_block_set_flags(g, -1, 0), "set_flags")
            check(L.bcfd_cellcount_solid(g), "cellcount_solid")
            check(L.bcfd_solid_cell_bc_move(g), "solid_cell_bc_move")
            check(L.bcfd_update_velocity_newv(g), "update_velocity_newv")
            check(L.bcfd_block_set_flags(g, 0, -1), "set_flags")
            check(L.bcfd_compute_norm_distance(g), "compute_norm_distance")
            check(L.bcfd_find_ts_cells(g), "find_ts_cells")
            check(L.bcfd_velocity_forcing_field(g), "velocity_forcing_field")
            check(L.bcfd_pressure_forcing_field(g), "pressure_forcing_field")
            check(L.bcfd_velocity_forcing_ghost(g), "velocity_forcing_ghost")
            check(L.bcfd_pressure_forcing_ghost(g), "pressure_forcing_ghost")

    def kinematic(self, g: int, name: str) -> float:
        """A kinematic scalar of a block (xdot, ydot, yddot, thetaDot1, ..., piv_z)."""
        return float(self.read(g, name, 1)[0])

    def time(self):
        """(ita, totime) of the native driver's loop (app/main.F90:130-131)."""
        ita, tt = C.c_int64(), C.c_double()
        check(self.L.bcfd_get_time(C.byref(ita), C.byref(tt)), "get_time")
        return ita.value, tt.value

    def set_time(self, ita: int, totime: float):
        """Set the native driver's loop counters (a restart: lastConditions'
        ita and totime, then totime + deltat as app/main.F90:116 does)."""
        mi = self.case.motion
        inor = next((b.mesh.inor for b in self.case.blocks if b.mesh is not None), 1)
        check(self.L.bcfd_set_motion_inputs((mi.phase_deg * np.pi / 180.0) if mi else 0.0,
                                            mi.piv_pt if mi else 0.0, mi.freq if mi else 0.0,
                                            mi.dxmin if mi else 0.0, inor, int(ita), float(totime)),
              "set_motion_inputs")

    def step(self):
        # advance the loop counters as the native driver does
        ita, tt = self.time()
        mi = self.case.motion
        inor = next((b.mesh.inor for b in self.case.blocks if b.mesh is not None), 1)
        check(self.L.bcfd_set_motion_inputs((mi.phase_deg * np.pi / 180.0) if mi else 0.0,
                                            mi.piv_pt if mi else 0.0, mi.freq if mi else 0.0,
                                            mi.dxmin if mi else 0.0, inor, ita + 1, tt + self.case.dt),
              "set_motion_inputs")
        self.momentum_phase()
        self.poisson_phase()
        self.research_phase()
        self.sync()

    # ---- the native whole-step driver ---------------------------------------
    def config(self, precision: int = 0, div_tol: float = 1e-6, use_graph: int = 0) -> _lib.StepConfig:
        c = self.case
        return _lib.StepConfig(c.dt, c.re, c.uc, c.epsi, c.pc_ita_max, precision, div_tol, use_graph)

    def run(self, n_steps: int, precision: int = 0, div_tol: float = 1e-6, use_graph: int = 0):
        cfg = self.config(precision, div_tol, use_graph)
        check(self.L.bcfd_run_steps(C.byref(cfg), n_steps), "run_steps")

    # ---- host mirrors --------------------------------------------------------
    def sync(self):
        check(self.L.bcfd_synchronize(), "synchronize")

    def fields(self, g: int) -> dict:
        spec = self.case.blocks[self.handles.index(g)]
        out = {k: np.zeros(spec.shape, order="F") for k in ("u", "v", "w", "p", "ut", "vt", "wt")}
        check(self.L.bcfd_block_download_fields(g, *(_pd(out[k]) for k in ("u", "v", "w", "p", "ut", "vt", "wt"))),
              "download_fields")
        return out

    def tags(self, g: int) -> dict:
        spec = self.case.blocks[self.handles.index(g)]
        s2 = (spec.nx + 2, spec.ny + 2, spec.nz + 2)
        s3 = (spec.nx + 3, spec.ny + 3, spec.nz + 3)
        out = {"cell": np.zeros(s2, np.int64, order="F"), "cell2": np.zeros(s3, np.int64, order="F"),
               "nodeIdTag": np.zeros(s3, np.int64, order="F"), "cell_n": np.zeros(s2, np.int64, order="F"),
               "cell_pr": np.zeros(s3, np.int64, order="F")}
        check(self.L.bcfd_block_download_tags(g, *(_pi(out[k]) for k in ("cell", "cell2", "nodeIdTag", "cell_n", "cell_pr"))),
              "download_tags")
        return out

    def counts(self, g: int) -> dict:
        a = np.zeros(6, np.int64)
        check(self.L.bcfd_block_get_counts(g, _pi(a)), "get_counts")
        return dict(zip(("ibCellCount", "solidCellCount", "fluidCellCount", "redCellCount",
                         "blackCellCount", "TSCellCount"), (int(x) for x in a)))

    def sor_stats(self, g: int):
        n, d2, ds = C.c_int64(), C.c_double(), C.c_double()
        check(self.L.bcfd_block_get_sor_stats(g, C.byref(n), C.byref(d2), C.byref(ds)), "sor_stats")
        return n.value, d2.value, ds.value

    def read(self, g: int, name: str, n: int, dtype=np.float64) -> np.ndarray:
        out = np.zeros(max(n, 1), dtype=dtype)
        w = C.c_int64()
        check(self.L.bcfd_block_read(g, name.encode(), out.ctypes.data_as(C.c_void_p), n, C.byref(w)),
              f"block_read({name})")
        return out[:w.value]

    def read_list(self, g: int, name: str, count: int) -> np.ndarray:
        a = self.read(g, name, 3 * max(count, 1), np.int64)
        return a.reshape(3, -1).T if a.size else np.zeros((0, 3), np.int64)

    def max_divergence(self, g: int) -> float:
        d = C.c_double()
        check(self.L.bcfd_max_divergence(g, C.byref(d)), "max_divergence")
        return d.value

    def divergence(self, g: int):
        """(max |div ut| after the last correction, dt * max |Poisson residual| of the last solve)."""
        d = np.zeros(2)
        check(self.L.bcfd_block_get_divergence(g, _pd(d)), "get_divergence")
        return float(d[0]), float(d[1])

    def autotune(self) -> int:
        """Time the candidate launch shapes of the Poisson solves and keep the fastest."""
        n = C.c_int64()
        check(self.L.bcfd_autotune(C.byref(n)), "autotune")
        return n.value

    def solve_launch(self, g: int) -> dict:
        a = (C.c_int * 6)()
        check(self.L.bcfd_block_get_solve_launch(g, a), "get_solve_launch")
        return dict(zip(("fp64_threads", "fp64_ctas_per_sm", "fp64_sync", "fp32_threads", "fp32_ctas_per_sm",
                         "fp32_variant"), list(a)))

    def set_batching(self, on: bool):
        check(self.L.bcfd_set_batching(int(on)), "set_batching")

    def set_warm_start(self, on: bool):
        """Residual-target solves start from the previous step's correction (library-wide)."""
        check(self.L.bcfd_set_warm_start(int(on)), "set_warm_start")

    def set_solve_launch(self, threads: int = 0, ctas_per_sm: int = 0, fp64_sync: int = 0, block: int = None):
        for g in (self.handles if block is None else [self.handles[block]]):
            check(self.L.bcfd_block_set_solve_launch(g, threads, ctas_per_sm, fp64_sync), "set_solve_launch")

    def set_mixed_params(self, inner: int = 0, omega: float = 0.0, variant: int = 0, block: int = None):
        for g in (self.handles if block is None else [block]):
            check(self.L.bcfd_block_set_mixed_params(g, inner, omega, variant), "set_mixed_params")

    def profile_begin(self):
        check(self.L.bcfd_profile_begin(), "profile_begin")

    def profile_end(self) -> dict:
        r = _lib.ProfileReport()
        check(self.L.bcfd_profile_end(C.byref(r)), "profile_end")
        return {k: getattr(r, k) for k, _ in r._fields_}

    PHASES = ("momentum", "forcing", "poisson_solves", "coupling", "correction", "motion_search",
              "forcing_field")

    def profile_phases(self) -> dict:
        """Device ms per step phase of the eager steps of the last measurement window."""
        ms = np.zeros(len(self.PHASES))
        check(self.L.bcfd_profile_phases(_pd(ms), len(ms)), "profile_phases")
        return {k: float(v) for k, v in zip(self.PHASES, ms)}

    def stress(self, g: int, mu_f: float, rho_f: float = 1.0) -> np.ndarray:
        """stress_calculation (src/StressCalc.f90:14-208): viscous drag, pressure drag,
        viscous lift, pressure lift coefficients."""
        out = np.zeros(4, np.float64)
        check(self.L.bcfd_stress_calculation(g, mu_f, rho_f, _pd(out)), "stress_calculation")
        return out

    def stream_ptr(self) -> int:
        p = C.c_void_p()
        check(self.L.bcfd_get_stream(C.byref(p)), "get_stream")
        return p.value or 0

    def kernel_launches(self) -> int:
        return int(self.L.bcfd_kernel_launches())

    def close(self):
        for g in self.handles:
            self.L.bcfd_block_destroy(g)
        self.handles = []
