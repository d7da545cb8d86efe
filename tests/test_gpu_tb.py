"""Temporal-blocked FP32 sweeps (variant 4): the same corrections bit for bit
as the two-barrier tiled sweeps (variant 1), on both blocks of the two-block
sphere workload and on a stretched block, after one correction of an odd and
an even number of sweep pairs, and through whole mixed steps."""
import numpy as np
import pytest

from biocfd import synth
from biocfd.solver import Solver
from biocfd._lib import check

pytestmark = pytest.mark.gpu


def _pc(case, variant, pairs):
    s = Solver(case)
    s.setup()
    out = []
    for g in s.handles:
        s.set_mixed_params(variant=variant, block=g)
        check(s.L.bcfd_compute_div(g), "compute_div")
        check(s.L.bcfd_block_sor_sweeps(g, pairs, 1), "sor_sweeps")
        out.append(s.read(g, "pc", int(np.prod(case.blocks[s.handles.index(g)].shape))))
    s.close()
    return out


@pytest.mark.parametrize("pairs,odd", [(7, False), (16, False), (5, True)])
def test_tb_sweeps_bitwise_equal_to_tiled(pairs, odd):
    case = (synth.uniform_block(n=(23, 17, 13), lengths=(3.0, 2.0, 2.0)) if odd
            else synth.small_two_block(n_steps=1))
    ref = _pc(case, 1, pairs)
    got = _pc(case, 4, pairs)
    for a, b in zip(ref, got):
        assert np.any(a != 0.0)
        np.testing.assert_array_equal(a, b)


def test_tb_whole_mixed_steps_bitwise_equal():
    case = synth.small_two_block(n_steps=3)
    res = []
    for variant in (1, 4):
        s = Solver(case)
        s.setup()
        s.set_mixed_params(variant=variant)
        s.run(3, precision=1, div_tol=1e-6)
        res.append([s.fields(g) for g in s.handles])
        s.close()
    for fa, fb in zip(*res):
        for k in ("u", "v", "w", "p"):
            np.testing.assert_array_equal(fa[k], fb[k])
