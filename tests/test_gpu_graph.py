"""A time step captured once as a CUDA graph and replayed gives bitwise the
same fields, Poisson iteration counts and residuals as the same steps issued
kernel by kernel; a changed solve parameter forces a new capture."""
import numpy as np
import pytest

from biocfd import synth
from biocfd.solver import Solver
from parity_util import assert_bitwise

pytestmark = pytest.mark.gpu


def _state(s):
    out = []
    for g in s.handles:
        f = s.fields(g)
        out.append(({k: f[k].copy() for k in ("u", "v", "w", "p")}, s.sor_stats(g), s.divergence(g)))
    return out


def _run(case, precision, use_graph, chunks, inner_change=None):
    s = Solver(case)
    s.setup()
    launches = []
    for q, n in enumerate(chunks):
        if inner_change is not None and q == 1:
            s.set_mixed_params(inner=inner_change)
        k0 = s.kernel_launches()
        s.run(n, precision=precision, div_tol=1e-6, use_graph=use_graph)
        launches.append(s.kernel_launches() - k0)
    st = _state(s)
    s.close()
    return st, launches


def _compare(a, b):
    for (fa, sa, da), (fb, sb, db) in zip(a, b):
        for k in ("u", "v", "w", "p"):
            assert_bitwise(k, fa[k], fb[k])
        assert sa[0] == sb[0], (sa, sb)
        assert np.array_equal(np.asarray(da), np.asarray(db)), (da, db)


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_matches_eager(precision):
    case = synth.small_two_block(n_steps=5)
    eager, le = _run(case, precision, 0, [5])
    graph, lg = _run(case, precision, 1, [5])
    _compare(eager, graph)
    # the replays count the captured kernels
    assert lg[0] == le[0], (le, lg)


def test_graph_recaptures_on_parameter_change():
    case = synth.small_two_block(n_steps=6)
    eager, _ = _run(case, 1, 0, [3, 3], inner_change=16)
    graph, _ = _run(case, 1, 1, [3, 3], inner_change=16)
    _compare(eager, graph)


def _kin(s, g):
    return [s.kinematic(g, k) for k in ("xdot", "ydot", "yddot", "thetaDot1", "thetaDDot1", "piv_x", "piv_y", "piv_z")]


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_moving_body_matches_eager(precision):
    """Steps with a heaving, pitching, towed plate replay from the graph: the
    host stages each step's kinematics before the launch, the captured node
    kernel applies them.  Fields, tags, kinematics and the loop counters equal
    the eager steps bit for bit."""
    case = synth.moving_plate_single_block(n=32, n_steps=6)
    out = []
    for use_graph in (0, 1):
        s = Solver(case)
        s.setup()
        s.run(6, precision=precision, div_tol=1e-6, use_graph=use_graph)
        g = s.handles[0]
        out.append((s.fields(g), s.tags(g), _kin(s, g), s.time(), s.sor_stats(g)[0]))
        s.close()
    (fa, ta, ka, tma, na), (fb, tb, kb, tmb, nb) = out
    for k in ("u", "v", "w", "p"):
        assert_bitwise(k, fa[k], fb[k])
    for k in ("cell", "cell2", "nodeIdTag"):
        assert np.array_equal(ta[k], tb[k]), k
    assert ka == kb
    assert tma == tmb
    assert na == nb


def test_graph_with_block_moves_matches_oracle():
    """Fine-block moves under the graph runner: a step whose staged motion
    reaches the margins runs eagerly (grids and tables change), the others
    replay; every step still equals the oracle bit for bit."""
    from oracle.bridge import Oracle
    from parity_util import compare_fields
    case = synth.moving_plate_block_move(n_steps=4)
    o = Oracle()
    o.setup(case)
    s = Solver(case)
    s.setup()
    t0 = s.time()[0]
    moves = []
    for step in range(4):
        o.step()
        s.run(1, use_graph=1)
        moves.append((o.geti(2, "move_amtx"), o.geti(2, "move_amty"), o.geti(2, "move_amtz")))
        compare_fields(o, s, f"step {step + 1}")
    assert s.time()[0] == t0 + 4
    assert any(m != (0, 0, 0) for m in moves), moves
    s.close()
