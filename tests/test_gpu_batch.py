"""Several uneven fine blocks under one coarse block: GPU vs oracle bit for
bit, and the batched launches (one launch per phase over all blocks, the fine
blocks' Poisson solves side by side in one cooperative launch) give exactly
the results of one launch per block, with fewer launches."""
import numpy as np
import pytest

from biocfd import synth
from biocfd.solver import Solver
from oracle.bridge import Oracle
from parity_util import assert_bitwise, compare_fields, compare_iters, compare_search

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("plate", [False, True])
def test_multi_block_parity_vs_oracle(plate):
    case = synth.multi_block(n_steps=2, plate=plate)
    o = Oracle()
    o.setup(case)
    s = Solver(case)
    s.setup()
    for _ in range(2):
        o.step()
    s.run(2)
    compare_fields(o, s, "2 steps")
    compare_iters(o, s, "2 steps")
    compare_search(o, s, "2 steps")


@pytest.mark.parametrize("plate", [False, True])
def test_two_bodies_parity_vs_oracle(plate):
    # a body in each of two fine blocks (the tandem-plate layout in small):
    # fields, SOR iteration counts and every Search output bitwise after 2 steps
    case = synth.multi_block(n_steps=2, plate=plate, body=(0, 1))
    assert sum(b.has_body for b in case.blocks) == 2
    o = Oracle()
    o.setup(case)
    s = Solver(case)
    s.setup()
    for _ in range(2):
        o.step()
    s.run(2)
    compare_fields(o, s, "2 steps")
    compare_iters(o, s, "2 steps")
    compare_search(o, s, "2 steps")


def _run(case, precision, batching, steps):
    s = Solver(case)
    s.set_batching(batching)
    s.setup()
    k0 = s.kernel_launches()
    s.run(steps, precision=precision, div_tol=1e-6)
    n = s.kernel_launches() - k0
    out = [(s.fields(g), s.sor_stats(g)[0]) for g in s.handles]
    s.close()
    return out, n


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_equals_per_block(precision):
    case = synth.multi_block(n_steps=3)
    a, na = _run(case, precision, False, 3)
    b, nb = _run(case, precision, True, 3)
    for q, ((fa, ia), (fb, ib)) in enumerate(zip(a, b)):
        for k in ("u", "v", "w", "p"):
            assert_bitwise(f"block {q + 1} {k}", fa[k], fb[k])
        assert ia == ib, (q, ia, ib)
    assert nb < na, (na, nb)
