"""Z-marching TMA sweeps (variant 5): two sweep pairs per pass over the block,
the correction staged plane by plane in shared memory by cp.async.bulk.tensor
loads.  The corrections are bitwise those of the tiled sweeps with grid-wide
barriers (variant 1): after one correction of an even and an odd number of
sweep pairs (an odd count ends with a one-pair pass), on both blocks of the
two-block sphere workload, on a stretched odd-sized block and on a block
large enough for several tiles along j and k; and through whole mixed
steps."""
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


@pytest.mark.parametrize("which,pairs", [("two_block", 8), ("two_block", 7), ("odd", 5), ("odd", 1),
                                         ("large", 6), ("large", 3)])
def test_zm_sweeps_bitwise_equal_to_tiled(which, pairs):
    if which == "two_block":
        case = synth.small_two_block(n_steps=1)
    elif which == "odd":
        case = synth.uniform_block(n=(23, 17, 13), lengths=(3.0, 2.0, 2.0))
    else:
        case = synth.uniform_block(n=(160, 96, 120), lengths=(4.0, 2.0, 3.0))
    ref = _pc(case, 1, pairs)
    got = _pc(case, 5, pairs)
    for a, b in zip(ref, got):
        assert np.any(a != 0.0)
        np.testing.assert_array_equal(a, b)


def test_zm_whole_mixed_steps_bitwise_equal():
    case = synth.small_two_block(n_steps=3)
    res = []
    for variant in (1, 5):
        s = Solver(case)
        s.setup()
        s.set_mixed_params(variant=variant)
        s.run(3, precision=1, div_tol=1e-6)
        res.append([s.fields(g) for g in s.handles])
        s.close()
    for fa, fb in zip(*res):
        for k in ("u", "v", "w", "p"):
            np.testing.assert_array_equal(fa[k], fb[k])
