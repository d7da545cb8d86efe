"""Allocation-free drag/lift entry point: bcfd_stress_calculation_noalloc
(fixed device scratch, no cudaMalloc/cudaFree) returns what
bcfd_stress_calculation returns, on two calls in a row.

Both entry points run the same two kernels with the same fixed summation
order, so the coefficients agree bit for bit.  A body with more surface
elements than the fixed scratch holds is refused with BCFD_E_CAPACITY before
any launch, and the allocating entry point still works on the same handle.

The file name sorts last so the test also runs after every other GPU test in
the same process; it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

from biocfd import synth
from biocfd._lib import BCFD_E_CAPACITY, check
from biocfd.solver import Solver

pytestmark = pytest.mark.gpu

MAX_ELEMS = 32768  # BCFD_STRESS_NOALLOC_MAX_ELEMS in include/biocfd_gb300.h


def _coeffs(fn, g, mu_f, rho_f):
    out = (C.c_double * 4)()
    check(fn(g, mu_f, rho_f, out), fn.__name__)
    return np.array(out[:])


def test_noalloc_stress_matches_allocating_entry_point():
    case = synth.sphere_single_block(n=32, n_steps=1)
    s = Solver(case)
    try:
        s.setup()
        s.run(1, precision=0)
        g = s.handles[0]
        mu_f, rho_f = 1.0 / case.re, 1.0
        ref = _coeffs(s.L.bcfd_stress_calculation, g, mu_f, rho_f)
        assert np.all(np.isfinite(ref)) and np.any(ref != 0.0), ref
        for _ in range(2):
            got = _coeffs(s.L.bcfd_stress_calculation_noalloc, g, mu_f, rho_f)
            np.testing.assert_array_equal(got, ref)
    finally:
        s.close()


def test_noalloc_stress_refuses_a_body_beyond_its_scratch():
    # a sphere whose Fibonacci markers give more triangles than the scratch holds
    case = synth.sphere_single_block(n=24, n_steps=1)
    spec = case.blocks[0]
    spec.mesh = synth.fibonacci_sphere((0.4, 0.5, 0.5), 0.25, 0.0034)
    ne = len(spec.mesh.tris)
    assert ne > MAX_ELEMS, ne
    s = Solver(case)
    try:
        s.setup()
        g = s.handles[0]
        mu_f, rho_f = 1.0 / case.re, 1.0
        out = (C.c_double * 4)(*([7.0] * 4))
        assert s.L.bcfd_stress_calculation_noalloc(g, mu_f, rho_f, out) == BCFD_E_CAPACITY
        assert list(out) == [7.0] * 4  # nothing written
        ref = _coeffs(s.L.bcfd_stress_calculation, g, mu_f, rho_f)
        assert np.all(np.isfinite(ref)), ref
    finally:
        s.close()
