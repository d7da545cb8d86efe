"""Allocation-free drag/lift entry point: bcfd_stress_calculation_noalloc
(fixed device scratch, no cudaMalloc/cudaFree) returns what
bcfd_stress_calculation returns, on two calls in a row.

The file name sorts last so the test also runs after every other GPU test in
the same process; it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

from biocfd import synth
from biocfd._lib import check
from biocfd.solver import Solver

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # same kernels and fixed summation order: agreement to rounding


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
            np.testing.assert_allclose(got, ref, rtol=RTOL, atol=0.0)
    finally:
        s.close()
