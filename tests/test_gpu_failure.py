"""Failure detection without a GPU fault.  Each failure is made on the host
or by a wait that nothing can satisfy; the device records a status, the call
returns it, and the context stays usable for the next step:

  * a bounded device-side wait that runs out (BCFD_E_TIMEOUT);
  * NaN or +-Inf in the velocity field (BCFD_E_NONFINITE, every precision);
  * the SOR iteration cap pcItaMax = 1 (not an error: the reference stops
    after its second iteration, src/PcorVcor.F90:373-375; bitwise vs oracle);
  * an IB list that outgrows its capacity (BCFD_E_CAPACITY);
  * a forcing probe outside the block, where find_index_in_array
    (src/Forcing.f90:1165-1183) finds no bracket (BCFD_E_NOTFOUND; the
    reference's result is undefined there, the oracle flags it too)."""
import ctypes as C

import numpy as np
import pytest

from biocfd import synth
from biocfd._lib import (BCFD_E_CAPACITY, BCFD_E_NONFINITE, BCFD_E_NOTFOUND, BCFD_E_TIMEOUT, check)
from biocfd.solver import Solver
from oracle.bridge import Oracle
from parity_util import compare_fields, compare_iters

pytestmark = pytest.mark.gpu


def _case(n=20):
    return synth.sphere_single_block(n=n, n_steps=2, diameter=0.3)


def _status(s, precision=0, steps=1):
    cfg = s.config(precision, 1e-6, 0)
    return s.L.bcfd_run_steps(C.byref(cfg), steps)


def test_bounded_wait_times_out_and_context_stays_usable():
    case = _case()
    s = Solver(case)
    try:
        s.setup()
        check(s.L.bcfd_set_wait_limit_ns(1_000_000), "set_wait_limit")  # 1 ms
        st, ms = C.c_int(0), C.c_double(0.0)
        check(s.L.bcfd_check_wait_limit(C.byref(st), C.byref(ms)), "check_wait_limit")
        assert st.value == BCFD_E_TIMEOUT, st.value
        assert 0.9 <= ms.value < 2000.0, ms.value  # gave up after the limit, not at once
        check(s.L.bcfd_set_wait_limit_ns(0), "set_wait_limit")  # back to 2 s
        # the next step at the normal limit runs and matches the oracle
        o = Oracle()
        o.setup(case)
        o.step()
        assert _status(s) == 0
        compare_fields(o, s, "step after a timed-out wait")
        compare_iters(o, s, "step after a timed-out wait")
    finally:
        s.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_nonfinite_velocity_is_reported(precision, bad):
    case = _case()
    s = Solver(case)
    try:
        s.setup()
        g = s.handles[0]
        ini = {k: np.array(v, order="F") for k, v in case.init[0].items()}
        ini["u"][5, 6, 7] = bad  # a fluid point away from the body
        s.upload_fields(g, ini)
        assert _status(s, precision) == BCFD_E_NONFINITE
        # the block is usable again with finite fields
        s.upload_fields(g, case.init[0])
        assert _status(s, precision) == 0
        assert all(np.all(np.isfinite(v)) for v in s.fields(g).values())
    finally:
        s.close()


def test_sor_iteration_cap_of_one_matches_oracle():
    case = synth.replace(_case(), pc_ita_max=1)
    o = Oracle()
    o.setup(case)
    s = Solver(case)
    try:
        s.setup()
        for _ in range(2):
            o.step()
        assert _status(s, 0, 2) == 0
        assert s.sor_stats(s.handles[0])[0] == o.geti(1, "nIterPcor") == 2
        compare_fields(o, s, "pcItaMax = 1")
        compare_iters(o, s, "pcItaMax = 1")
    finally:
        s.close()


def test_ib_list_over_capacity_is_reported():
    case = _case()
    s = Solver(case)
    try:
        s.setup()
        g = s.handles[0]
        nib = s.counts(g)["ibCellCount"]
        assert nib > 16
        check(s.L.bcfd_block_set_list_capacity(g, 16), "set_list_capacity")
        # the routine called alone, and a whole step, report the overflow
        assert s.L.bcfd_cellcount_solid(g) == BCFD_E_CAPACITY
        assert _status(s) == BCFD_E_CAPACITY
        # with the capacity back the lists are rebuilt whole
        check(s.L.bcfd_block_set_list_capacity(g, 0), "set_list_capacity")
        assert s.L.bcfd_tagging_th(g) == 0
        assert s.L.bcfd_cellcount_solid(g) == 0
        assert s.counts(g)["ibCellCount"] == nib
        assert _status(s) == 0
    finally:
        s.close()


def test_probe_outside_the_block_is_reported():
    # a sphere 1.3 cells from the block's low-x face: the probes of the IB cells
    # there (1.5 cell diagonals along the outward normal) leave the grid
    n = 32
    case = synth.sphere_single_block(n=n, n_steps=1, diameter=0.3, center=(0.15 + 1.3 / n, 0.5, 0.5))
    o = Oracle()
    o.setup(case)
    o.step()
    assert o.err(1) == BCFD_E_NOTFOUND
    s = Solver(case)
    try:
        s.setup()
        assert _status(s) == BCFD_E_NOTFOUND
    finally:
        s.close()
