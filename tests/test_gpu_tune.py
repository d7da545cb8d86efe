"""The autotuner only picks launch shapes (threads per CTA, CTAs per SM, phase
synchronisation) of the Poisson solves, none of which changes the arithmetic:
tuned steps equal untuned steps bit for bit, and the solve state the trials
touch is restored."""
import pytest

from biocfd import synth
from biocfd.solver import Solver
from parity_util import assert_bitwise

pytestmark = pytest.mark.gpu


def _run(case, precision, tune):
    s = Solver(case)
    s.setup()
    n = s.autotune() if tune else 0
    shapes = [s.solve_launch(g) for g in s.handles]
    s.run(2, precision=precision, div_tol=1e-6)
    out = [(s.fields(g), s.sor_stats(g)[0]) for g in s.handles]
    s.close()
    return out, n, shapes


@pytest.mark.parametrize("precision", [0, 1])
def test_tuned_equals_untuned(precision):
    case = synth.small_two_block(n_steps=2)
    a, _, _ = _run(case, precision, False)
    b, n, shapes = _run(case, precision, True)
    assert all(sh["fp64_threads"] > 0 and sh["fp32_variant"] in (1, 3, 4) for sh in shapes), shapes
    for q, ((fa, ia), (fb, ib)) in enumerate(zip(a, b)):
        for k in ("u", "v", "w", "p"):
            assert_bitwise(f"block {q + 1} {k}", fa[k], fb[k])
        assert ia == ib
