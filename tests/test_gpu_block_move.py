"""Fine-block moves (app/main.F90:178-230, src/Search.F90:916-1461): a
heaving, pitching, towed plate near the margins of its fine block's box, so
the block shifts by whole cells every step.  After each native step the
fields of both blocks, the moved grid, the interface tables and the tags are
bit for bit those of the oracle."""
import ctypes as C

import numpy as np
import pytest

from biocfd import synth
from biocfd._lib import check
from biocfd.solver import Solver
from oracle.bridge import Oracle
from parity_util import assert_bitwise, compare_fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("driver", ["native", "phases"])
def test_block_moves_match_oracle(driver):
    """`native`: the library's whole-step driver; `phases`: the per-subroutine
    entry points (block_move_stage, compute_surface_norm, tagging_th_move,
    selective_retagging_th, ...) in the reference's call order."""
    case = synth.moving_plate_block_move(n_steps=3)
    o = Oracle()
    o.setup(case)
    s = Solver(case)
    s.setup()
    gf = s.handles[1]
    spec = case.blocks[1]
    moves = []
    for step in range(3):
        o.step()
        if driver == "native":
            s.run(1)
        else:
            s.step()
        moves.append((o.geti(2, "move_amtx"), o.geti(2, "move_amty"), o.geti(2, "move_amtz")))
        compare_fields(o, s, f"step {step + 1}")
        assert_bitwise(f"step {step + 1} x1", o.arr(2, "x1"), s.read(gf, "x1", spec.nx + 3))
        assert_bitwise(f"step {step + 1} y1", o.arr(2, "y1"), s.read(gf, "y1", spec.ny + 3))
        for nm in ("px", "py", "pz", "ux", "uy", "uz", "vx", "vy", "vz", "wx", "wy", "wz"):
            ref, cnt = o.table(1, nm)
            out = np.zeros(3 * ref.shape[1], np.int64)
            c = C.c_int64()
            check(s.L.bcfd_interface_table(s.ifaces[0], nm.encode(), out.ctypes.data_as(C.POINTER(C.c_int64)),
                                           out.size, C.byref(c)), "interface_table")
            assert c.value == cnt, nm
            assert np.array_equal(ref[:, :cnt], out.reshape(-1, 3).T[:, :cnt]), (step, nm)
        for g, name in ((1, "cell"), (2, "cell_n")):
            t = s.tags(s.handles[g - 1])[name]
            np.testing.assert_array_equal(t, o.arr(g, name), err_msg=f"step {step + 1} {name} of block {g}")
    # the block did move (x and y), as the reference's margins demand
    assert any(m != (0, 0, 0) for m in moves), moves
