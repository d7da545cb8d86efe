"""Discrete adjoints of the solver as host calls and torch.autograd.Functions.

The Poisson solve:
  forward:  x = A^{-1} r      (bcfd_poisson_solve_zero_bc)
  backward: r_bar = A^{-T} x_bar (bcfd_poisson_solve_adjoint: the same SOR
            kernel with the transposed line tables and reversed colour order)
A is the Poisson operator of one block restricted to its fluid cells (zero
data on the other cells).

Whole runs of time steps: adjoint_run (fixed geometry), adjoint_run_motion
(moving bodies, gradients with respect to the motion parameters of the
objective's body) and
run_function, which wraps either as a torch.autograd.Function of the initial
state and the scalar parameters.

Arrays are natural-layout (nx+2, ny+2, nz+2) FP64, x-fastest, like the
block's fields.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check


def _solve(solver, g: int, r: np.ndarray, tol: float, itmax: int, adjoint: bool) -> np.ndarray:
    r = np.asfortranarray(r, dtype=np.float64)
    x = np.zeros_like(r, order="F")
    fn = solver.L.bcfd_poisson_solve_adjoint if adjoint else solver.L.bcfd_poisson_solve_zero_bc
    check(fn(g, r.ctypes.data_as(C.POINTER(C.c_double)), x.ctypes.data_as(C.POINTER(C.c_double)), tol, itmax),
          "poisson_solve_adjoint" if adjoint else "poisson_solve_zero_bc")
    return x


def poisson_solve(solver, g: int, r: np.ndarray, tol: float = 1e-12, itmax: int = 200000) -> np.ndarray:
    """x = A^{-1} r on block g (FP64 SOR to max|r - A x| <= tol)."""
    return _solve(solver, g, r, tol, itmax, False)


def poisson_solve_adjoint(solver, g: int, r: np.ndarray, tol: float = 1e-12, itmax: int = 200000) -> np.ndarray:
    """x = A^{-T} r on block g."""
    return _solve(solver, g, r, tol, itmax, True)


def poisson_function(solver, g: int, tol: float = 1e-12, itmax: int = 200000):
    """A torch.autograd.Function applying A^{-1} of block g to a float64 tensor
    of the block's point shape; its backward applies A^{-T}."""
    import torch

    class PoissonSolve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, r):
            x = poisson_solve(solver, g, r.detach().cpu().numpy(), tol, itmax)
            return torch.from_numpy(np.ascontiguousarray(x)).to(r)

        @staticmethod
        def backward(ctx, gx):
            gr = poisson_solve_adjoint(solver, g, gx.detach().cpu().numpy(), tol, itmax)
            return torch.from_numpy(np.ascontiguousarray(gr)).to(gx)

    return PoissonSolve


def momentum_tangent(solver, g: int, du, dv, dw, dp, dt: float | None = None, re: float | None = None):
    """Tangent-linear model of nsMomentum2order on block g at its current
    (u, v, w, p): returns (ut, vt, wt) -- bitwise the FP64 predictor -- and
    (dut, dvt, dwt), the predictor's derivative along (du, dv, dw, dp).
    Arrays are natural-layout FP64 of the block's point shape; only fluid
    interior cells (cell == 0) are written, the rest stay zero."""
    c = solver.case
    dt = c.dt if dt is None else dt
    re = c.re if re is None else re
    ins = [np.asfortranarray(a, dtype=np.float64) for a in (du, dv, dw, dp)]
    outs = [np.zeros_like(ins[0], order="F") for _ in range(6)]
    P = C.POINTER(C.c_double)
    check(solver.L.bcfd_momentum_tangent(g, dt, re, *(a.ctypes.data_as(P) for a in ins),
                                         *(a.ctypes.data_as(P) for a in outs)), "momentum_tangent")
    return tuple(outs[:3]), tuple(outs[3:])


def momentum_adjoint(solver, g: int, utb, vtb, wtb, dt: float | None = None, re: float | None = None):
    """Adjoint of nsMomentum2order on block g at its current (u, v, w, p):
    returns (ub, vb, wb, pb) = J^T (utb, vtb, wtb), the transpose of
    momentum_tangent (seeds off the fluid cells are ignored)."""
    c = solver.case
    dt = c.dt if dt is None else dt
    re = c.re if re is None else re
    ins = [np.asfortranarray(a, dtype=np.float64) for a in (utb, vtb, wtb)]
    outs = [np.zeros_like(ins[0], order="F") for _ in range(4)]
    P = C.POINTER(C.c_double)
    check(solver.L.bcfd_momentum_adjoint(g, dt, re, *(a.ctypes.data_as(P) for a in ins),
                                         *(a.ctypes.data_as(P) for a in outs)), "momentum_adjoint")
    return tuple(outs)


def adjoint_run(solver, weights: dict, n_steps: int, every: int = 20, uc: float | None = None,
                gradient: bool = True, adj_tol: float = 1e-13, adj_itmax: int = 200000,
                stress_seed=None, mu_f: float = 1.0, rho_f: float = 1.0, solve_precision: int | None = None):
    """Discrete adjoint of n_steps FP64 time steps of the solver's single
    block (domain BCs, optionally a stationary body), checkpointing every
    `every` steps.

    J = (1/N) sum_{n=1..N} (<W, x^n> + sum_t stress_seed[t] C_t(x^n)) with
    W = weights {"u","v","w","p"} (natural-layout arrays; missing fields weigh
    0) and C_t the four drag/lift coefficients of stress_calculation(mu_f,
    rho_f) (e.g. stress_seed = (1, 1, 0, 0) for the total drag coefficient).
    Returns J, or with `gradient` (J, dJ/duc, {"u","v","w","p"}: dJ/dx^0,
    "kin": dJ/d(xdot, ydot, yddot, thetaDot1, thetaDDot1, thetaDot2,
    thetaDDot2, alphaDot)} with the body's kinematic scalars constant and its
    geometry fixed).  The block advances by n_steps, exactly as
    solver.run(n_steps) would.  `solve_precision` selects the adjoint Poisson
    solver (0 FP64 SOR, 1 FP32 sweeps with FP64 defect correction; both to
    adj_tol), None keeps the library's setting."""
    c = solver.case
    g = solver.handles[0]
    shape = c.blocks[0].shape
    if solve_precision is not None:
        check(solver.L.bcfd_adjoint_set_solver(int(solve_precision)), "adjoint_set_solver")
    W = [np.asfortranarray(weights.get(k, np.zeros(shape)), dtype=np.float64) for k in ("u", "v", "w", "p")]
    cfg = solver.config(0)
    if uc is not None:
        cfg.uc = uc
    P = C.POINTER(C.c_double)
    J = C.c_double()
    duc = C.c_double()
    grads = [np.zeros(shape, order="F") for _ in range(4)] if gradient else None
    kin = np.zeros(8)
    null = C.cast(None, P)
    seed = None if stress_seed is None else np.ascontiguousarray(stress_seed, dtype=np.float64)
    check(solver.L.bcfd_adjoint_run(g, C.byref(cfg), n_steps, every, *(w.ctypes.data_as(P) for w in W),
                                    null if seed is None else seed.ctypes.data_as(P), mu_f, rho_f,
                                    adj_tol, adj_itmax, C.byref(J),
                                    C.byref(duc) if gradient else null,
                                    kin.ctypes.data_as(P) if gradient else null,
                                    *((a.ctypes.data_as(P) for a in grads) if gradient else (null,) * 4)),
          "adjoint_run")
    if not gradient:
        return J.value
    out = dict(zip(("u", "v", "w", "p"), grads))
    out["kin"] = kin
    return J.value, duc.value, out


# the motion parameters of adjoint_run_motion, in the units of synth.Motion /
# synth.MotionInputs (the C ABI's phase is in radians)
MOTION_PARAMS = ("yamp", "a0_deg", "phase_deg", "freq", "bfreq")


def adjoint_run_motion(solver, weights: dict, n_steps: int, every: int = 20, block: int = 0, uc: float | None = None,
                       gradient: bool = True, adj_tol: float = 1e-13, adj_itmax: int = 200000, stress_seed=None,
                       mu_f: float = 1.0, rho_f: float = 1.0):
    """adjoint_run through a moving body (bcfd_adjoint_run_motion): J of
    n_steps FP64 steps with the weights and drag/lift of block `block`, whose
    body moves (other moving bodies, e.g. a plate in tandem, move with the
    run and count towards the shared phase and pitch frequency).  Returns J,
    or with `gradient`
    (J, dJ/duc, {"u","v","w","p": dJ/dx^0 of the block, "motion": {name:
    dJ/d name for MOTION_PARAMS}}).  The body's tags, nodes and motion state
    are checkpointed with the fields; the block advances by n_steps exactly
    as solver.run(n_steps) would.  Thin-surface cells (surfaces 51/52) are
    differentiated; a fine-block move during the run is refused."""
    c = solver.case
    g = solver.handles[block]
    shape = c.blocks[block].shape
    W = [np.asfortranarray(weights.get(k, np.zeros(shape)), dtype=np.float64) for k in ("u", "v", "w", "p")]
    cfg = solver.config(0)
    if uc is not None:
        cfg.uc = uc
    P = C.POINTER(C.c_double)
    J = C.c_double()
    duc = C.c_double()
    grads = [np.zeros(shape, order="F") for _ in range(4)] if gradient else None
    dmot = np.zeros(5)
    null = C.cast(None, P)
    seed = None if stress_seed is None else np.ascontiguousarray(stress_seed, dtype=np.float64)
    check(solver.L.bcfd_adjoint_run_motion(g, C.byref(cfg), n_steps, every, *(w.ctypes.data_as(P) for w in W),
                                           null if seed is None else seed.ctypes.data_as(P), mu_f, rho_f,
                                           adj_tol, adj_itmax, C.byref(J),
                                           C.byref(duc) if gradient else null,
                                           dmot.ctypes.data_as(P) if gradient else null,
                                           *((a.ctypes.data_as(P) for a in grads) if gradient else (null,) * 4)),
          "adjoint_run_motion")
    if not gradient:
        return J.value
    dmot[2] *= np.pi / 180.0  # per radian -> per degree
    out = dict(zip(("u", "v", "w", "p"), grads))
    out["motion"] = dict(zip(MOTION_PARAMS, dmot))
    return J.value, duc.value, out


def run_function(make_solver, weights: dict, n_steps: int, every: int = 20, moving: bool = False, **kw):
    """A torch.autograd.Function J = f(u0, v0, w0, p0, params) of n_steps FP64
    time steps.  `params` is a float64 tensor: [uc], or with `moving`
    [uc, yamp, a0_deg, phase_deg, freq, bfreq]; make_solver(list of params)
    returns a set-up Solver for those values, and forward uploads the initial
    state (tensors of block 0's point shape) to its block 0 before the run.
    forward runs the forward steps and the reverse sweep in one call
    (adjoint_run / adjoint_run_motion) and keeps the gradient; backward scales
    it by the incoming gradient of J.  Remaining keywords go to the run
    (stress_seed, mu_f, rho_f, adj_tol, ...)."""
    import torch

    class AdjointRun(torch.autograd.Function):
        @staticmethod
        def forward(ctx, u, v, w, p, params):
            pv = [float(x) for x in params.detach().cpu().reshape(-1)]
            s = make_solver(pv)
            state = {k: np.asfortranarray(t.detach().cpu().numpy(), dtype=np.float64)
                     for k, t in zip(("u", "v", "w", "p"), (u, v, w, p))}
            s.upload_fields(s.handles[0], state)
            if moving:
                J, duc, g = adjoint_run_motion(s, weights, n_steps, every, uc=pv[0], **kw)
                gpar = [duc] + [g["motion"][k] for k in MOTION_PARAMS]
            else:
                J, duc, g = adjoint_run(s, weights, n_steps, every, uc=pv[0], **kw)
                gpar = [duc]
            ctx.grads = [torch.from_numpy(np.ascontiguousarray(g[k])).to(u) for k in ("u", "v", "w", "p")]
            ctx.gpar = torch.tensor(gpar, dtype=params.dtype, device=params.device)
            return torch.tensor(J, dtype=torch.float64, device=u.device)

        @staticmethod
        def backward(ctx, gJ):
            return (*(gJ * t for t in ctx.grads), gJ * ctx.gpar)

    return AdjointRun
