"""A heaving, pitching and towed plate (surface 51, thinner than a cell): the
per-step kinematics and node motion of computeSurfaceVariables
(src/Search.F90:126-208), the normals of the moved surface, the re-Search
and the forcing with the body velocity, bit for bit against the oracle."""
import numpy as np
import pytest

from biocfd import synth
from biocfd.solver import Solver
from oracle.bridge import Oracle
from parity_util import assert_bitwise, compare_fields, compare_iters, compare_search

pytestmark = pytest.mark.gpu


def _pair(case):
    o = Oracle()
    o.setup(case)
    s = Solver(case)
    s.setup()
    return o, s


def _nodes(o, s, tag):
    g = s.handles[0]
    nn = len(s.case.blocks[0].mesh.nodes)
    for nm in ("xnode1", "ynode1", "znode1"):
        assert_bitwise(f"{tag} {nm}", o.arr(1, nm), s.read(g, nm, nn))
    ne = len(s.case.blocks[0].mesh.tris)
    for nm in ("xcent", "ycent", "zcent", "cosAlpha", "cosBeta", "cosGamma"):
        assert_bitwise(f"{tag} {nm}", o.arr(1, nm), s.read(g, nm, ne))


def test_moving_plate_setup_and_steps():
    case = synth.moving_plate_single_block(n=32, n_steps=4)
    o, s = _pair(case)
    _nodes(o, s, "setup")
    # findDistnode's extreme nodes (the block-move checks read them)
    for nm in ("mk", "mkx1", "mkx2"):
        assert int(s.read(s.handles[0], nm, 1, np.int64)[0]) == o.geti(1, nm) > 0, nm
    compare_search(o, s, "setup")
    for q in range(4):
        o.step()
        s.run(1)
        _nodes(o, s, f"step {q + 1}")
        compare_fields(o, s, f"step {q + 1}")
        compare_iters(o, s, f"step {q + 1}")
        compare_search(o, s, f"step {q + 1}")
    for nm in ("xdot", "ydot", "yddot", "thetaDot1", "thetaDDot1", "piv_x", "piv_y"):
        assert s.kinematic(s.handles[0], nm) == o.getf(1, nm), nm


def test_lagging_plate_matches_oracle():
    # a body lagging 90 deg behind the shared kinematics (the tandem plates'
    # trailing plate): its initial placement at its own t = 0 state, then the
    # lagged heave and pitch, bitwise against the oracle's restatement
    case = synth.moving_plate_single_block(n=32, n_steps=3)
    spec = case.blocks[0]
    spec.motion = synth.dataclasses.replace(spec.motion, lag_deg=90.0)
    o, s = _pair(case)
    _nodes(o, s, "setup")
    assert s.kinematic(s.handles[0], "piv_y") == o.getf(1, "piv_y") != spec.motion.shift[1]
    for q in range(3):
        o.step()
        s.run(1)
        _nodes(o, s, f"step {q + 1}")
        compare_fields(o, s, f"step {q + 1}")
        compare_iters(o, s, f"step {q + 1}")
        compare_search(o, s, f"step {q + 1}")
    for nm in ("xdot", "ydot", "yddot", "thetaDot1", "thetaDDot1", "piv_x", "piv_y"):
        assert s.kinematic(s.handles[0], nm) == o.getf(1, nm), nm
