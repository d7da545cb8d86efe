"""Transposes of the thin-surface (TS) pieces of a step, one routine at a time.

A plate thinner than a cell (surface 51) on a 24^3 block, after one step (so
the ghost arrays hold velocityForcingGhost / pressureForcingGhost of the
block's state):
* the ghost calls G (bcfd_forcing_ghost_adjoint): a dot-product test, G is
  affine in (u, v, w, p, ut, vt, wt);
* the predictor with its TS overlay (bcfd_momentum_adjoint_ts), ghost arrays
  held fixed: J = <s, ut> + <r, (u, v, w, p) after the call> against central
  differences;
* the two composed as a step composes them (the ghost arrays G(x) of the
  state the predictor reads): the ghost adjoint the predictor returns, sent
  through G^T, against central differences of J(x) with G recomputed."""
import ctypes as C

import numpy as np
import pytest

from biocfd import synth
from biocfd._lib import check
from biocfd.solver import Solver

pytestmark = pytest.mark.gpu

P = C.POINTER(C.c_double)
FIELDS = ("u", "v", "w", "p", "ut", "vt", "wt")
GHOSTS = ("p_ghost", "pt_ghost", "u2_ghost", "u2t_ghost", "v2_ghost", "v2t_ghost", "w2_ghost", "w2t_ghost",
          "u1_ghost", "u1t_ghost", "v1_ghost", "v1t_ghost", "w1_ghost", "w1t_ghost")


def _pd(a):
    return a.ctypes.data_as(P)


@pytest.fixture(scope="module")
def plate():
    case = synth.plate_single_block(n=24, n_steps=1)
    s = Solver(case)
    s.setup()
    s.run(1)
    g = s.handles[0]
    nts = s.counts(g)["TSCellCount"]
    assert nts > 0
    x0 = {k: v.copy(order="F") for k, v in s.fields(g).items()}
    return case, s, g, nts, x0


def _upload(s, g, x):
    a = [np.asfortranarray(x[k]) for k in FIELDS]
    check(s.L.bcfd_block_upload_fields(g, *(_pd(v) for v in a)), "upload")


def _ghosts(s, g, nts, x):
    _upload(s, g, x)
    check(s.L.bcfd_velocity_forcing_ghost(g), "velocity_forcing_ghost")
    check(s.L.bcfd_pressure_forcing_ghost(g), "pressure_forcing_ghost")
    return np.stack([s.read(g, n, nts) for n in GHOSTS])


def _direction(case, s, g, rng):
    spec = case.blocks[0]
    m = np.zeros(spec.shape, bool, order="F")
    m[1:-1, 1:-1, 1:-1] = True
    return {k: np.asfortranarray(rng.normal(size=spec.shape) * m) for k in FIELDS}


def _restore(s, g, x0, ghosts):
    _upload(s, g, x0)
    check(s.L.bcfd_velocity_forcing_ghost(g), "velocity_forcing_ghost")
    check(s.L.bcfd_pressure_forcing_ghost(g), "pressure_forcing_ghost")


def test_ghost_calls_transpose(plate):
    case, s, g, nts, x0 = plate
    rng = np.random.default_rng(1)
    d = _direction(case, s, g, rng)
    gb = rng.normal(size=(14, nts))
    eps = 1.0  # G is affine: the central difference is exact up to rounding
    gp = _ghosts(s, g, nts, {k: x0[k] + eps * d[k] for k in FIELDS})
    gm = _ghosts(s, g, nts, {k: x0[k] - eps * d[k] for k in FIELDS})
    fd = float(np.sum(gb * (gp - gm))) / (2 * eps)
    out = {k: np.zeros(case.blocks[0].shape, order="F") for k in FIELDS}
    gbc = np.ascontiguousarray(gb)
    _ghosts(s, g, nts, x0)
    check(s.L.bcfd_forcing_ghost_adjoint(g, _pd(gbc), *(_pd(out[k]) for k in FIELDS)), "forcing_ghost_adjoint")
    ad = sum(float(np.sum(out[k] * d[k])) for k in FIELDS)
    assert abs(fd - ad) <= 1e-10 * max(abs(fd), 1.0), (fd, ad)


def _momentum_j(case, s, g, nts, x, st, r, ghosts_of_x):
    if ghosts_of_x:
        _ghosts(s, g, nts, x)
    else:
        _upload(s, g, x)
    check(s.L.bcfd_ns_momentum_2order(g, case.dt, case.re), "ns_momentum_2order")
    y = s.fields(g)
    return sum(float(np.sum(st[k] * y[k])) for k in ("ut", "vt", "wt")) + \
        sum(float(np.sum(r[k] * y[k])) for k in ("u", "v", "w", "p"))


def test_momentum_ts_adjoint_vs_fd(plate):
    """The direct part (ghost arrays held fixed) and the part through the
    ghost arrays (G recomputed from the perturbed state) separately."""
    case, s, g, nts, x0 = plate
    spec = case.blocks[0]
    rng = np.random.default_rng(2)
    cell = s.tags(g)["cell"]
    fluid = np.zeros(spec.shape, bool, order="F")
    fluid[1:-1, 1:-1, 1:-1] = True
    fluid &= cell == 0
    st = {k: np.asfortranarray(rng.normal(size=spec.shape) * fluid) for k in ("ut", "vt", "wt")}
    r = {k: np.asfortranarray(rng.normal(size=spec.shape)) for k in ("u", "v", "w", "p")}
    d = _direction(case, s, g, rng)
    for k in FIELDS:
        d[k] *= 1e-2 * max(float(np.sqrt(np.mean(x0[k] ** 2))), 1e-3)
    # adjoint at x0 with the ghost arrays of x0
    _ghosts(s, g, nts, x0)
    io = {k: r[k].copy(order="F") for k in ("u", "v", "w", "p")}
    gb = np.zeros((14, nts))
    check(s.L.bcfd_momentum_adjoint_ts(g, case.dt, case.re, *(_pd(st[k]) for k in ("ut", "vt", "wt")),
                                       *(_pd(io[k]) for k in ("u", "v", "w", "p")), _pd(gb)),
          "momentum_adjoint_ts")
    ad_direct = sum(float(np.sum(io[k] * d[k])) for k in ("u", "v", "w", "p"))
    gg = {k: np.zeros(spec.shape, order="F") for k in FIELDS}
    _ghosts(s, g, nts, x0)
    gbc = np.ascontiguousarray(gb)
    check(s.L.bcfd_forcing_ghost_adjoint(g, _pd(gbc), *(_pd(gg[k]) for k in FIELDS)), "ghost_adjoint")
    ad_ghost = sum(float(np.sum(gg[k] * d[k])) for k in FIELDS)
    eps = 1e-4
    xp = {k: x0[k] + eps * d[k] for k in FIELDS}
    xm = {k: x0[k] - eps * d[k] for k in FIELDS}
    _ghosts(s, g, nts, x0)
    jp = _momentum_j(case, s, g, nts, xp, st, r, False)
    _ghosts(s, g, nts, x0)
    jm = _momentum_j(case, s, g, nts, xm, st, r, False)
    fd_direct = (jp - jm) / (2 * eps)
    jp = _momentum_j(case, s, g, nts, xp, st, r, True)
    jm = _momentum_j(case, s, g, nts, xm, st, r, True)
    fd_ghost = (jp - jm) / (2 * eps) - fd_direct
    print("momentum_ts", {"fd_direct": fd_direct, "ad_direct": ad_direct, "fd_ghost": fd_ghost,
                          "ad_ghost": ad_ghost, "gb_abs": float(np.abs(gb).sum())})
    assert abs(fd_direct - ad_direct) <= 1e-6 * abs(fd_direct), (fd_direct, ad_direct)
    assert abs(fd_ghost) > 1e-6 * abs(fd_direct)  # the ghost path is exercised
    assert abs(fd_ghost - ad_ghost) <= 1e-6 * abs(fd_direct) + 1e-4 * abs(fd_ghost), (fd_ghost, ad_ghost)
