"""Thin-surface (TS) cells: a stationary plate (surface 51) thinner than a
cell.  The momentum predictor's in-place ghost substitution and restore
(src/NavierStokes.f90:310-490, 860-907) depend on the serial loop order; the
GPU must reproduce the oracle bit for bit, including the values the loop
leaves in u, v, w, p."""
import numpy as np
import pytest

from biocfd import synth
from biocfd.solver import Solver
from oracle.bridge import Oracle
from parity_util import compare_fields, compare_iters, compare_search, rel_l2

pytestmark = pytest.mark.gpu


def _pair(case):
    o = Oracle()
    o.setup(case)
    s = Solver(case)
    s.setup()
    return o, s


@pytest.mark.parametrize("n", [24, 32])
def test_plate_one_step_phases(n):
    case = synth.plate_single_block(n=n, n_steps=1)
    o, s = _pair(case)
    g = s.handles[0]
    assert s.counts(g)["TSCellCount"] > 0
    compare_search(o, s, "setup")
    o.momentum_phase()
    s.momentum_phase()
    compare_fields(o, s, "momentum phase")
    o.poisson_phase()
    s.poisson_phase()
    compare_fields(o, s, "poisson phase")
    compare_iters(o, s, "poisson phase")
    o.research_phase()
    s.research_phase()
    compare_search(o, s, "research phase")
    compare_fields(o, s, "research phase")


def test_plate_steps_native_driver():
    case = synth.plate_single_block(n=32, n_steps=3)
    o, s = _pair(case)
    for _ in range(3):
        o.step()
    s.run(3)
    compare_fields(o, s, "3 steps")
    compare_iters(o, s, "3 steps")
    compare_search(o, s, "3 steps")


def test_plate_mixed_path_close_to_fp64():
    case = synth.plate_single_block(n=32, n_steps=2)
    res = {}
    for prec in (2, 1):
        s = Solver(case)
        s.setup()
        s.run(2, precision=prec, div_tol=1e-6)
        res[prec] = s.fields(s.handles[0])
        assert s.divergence(s.handles[0])[1] <= 1e-6 * (1 + 1e-9)
        s.close()
    for nm in ("u", "v", "w", "p"):
        assert rel_l2(res[2][nm], res[1][nm]) < 1e-4, nm
