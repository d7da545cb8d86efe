"""The oracle's OpenMP loops (sweeps of one colour, per-cell stencils without
thin-surface cells, the per-cell searches, maxima) give the serial loops'
results bit for bit: the same steps on one thread and on all threads."""
import numpy as np
import pytest

from biocfd import synth
from oracle.bridge import Oracle, lib
from parity_util import assert_bitwise

FIELDS = ("u", "v", "w", "p", "ut", "vt", "wt", "pc", "cell", "nodeIdTag")


def _run(case, steps, threads):
    L = lib(True)
    n0 = L.orc_get_threads()
    L.orc_set_threads(threads)
    try:
        o = Oracle()
        o.setup(case)
        for _ in range(steps):
            o.step()
        out = {(g, nm): np.array(o.arr(g, nm)) for g in range(1, len(case.blocks) + 1) for nm in FIELDS}
        out.update({(g, "nIterPcor"): o.geti(g, "nIterPcor") for g in range(1, len(case.blocks) + 1)})
        return out
    finally:
        L.orc_set_threads(n0)


@pytest.mark.parametrize("maker", [
    lambda: synth.sphere_single_block(n=20, n_steps=3, diameter=0.3),
    lambda: synth.small_two_block(n_steps=2),
    lambda: synth.moving_plate_single_block(n=24, n_steps=2),
], ids=["sphere", "two_block", "moving_plate"])
def test_parallel_oracle_equals_serial(maker):
    case = maker()
    steps = case.n_steps
    a = _run(case, steps, 1)
    b = _run(case, steps, 4)
    for key, ref in a.items():
        if isinstance(ref, int):
            assert ref == b[key], key
        else:
            assert_bitwise(f"{key}", ref, b[key])
