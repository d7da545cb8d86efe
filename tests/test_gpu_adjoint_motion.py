"""Discrete adjoint through a moving body (bcfd_adjoint_run_motion).

Two bodies on a 24^3 block, J = the body's time-averaged drag coefficient
over 6 FP64 steps from the set-up:
* a sphere (surface 50) that heaves and is towed; its nodes do not rotate,
  so only the pitch kinematics reach J from the pitch parameters;
* a plate thinner than a cell (surface 51) that heaves, pitches about x and
  is towed: every IB cell is a thin-surface (TS) cell, so the predictor's
  ghost substitution, the ghost calls and the node rotation are transposed;
* the same kind of plate in the fine block of a coarse/fine pair (the
  coupling transposes inside the moving run);
* two such plates in tandem, each in its own fine block, the trailing one
  90 degrees behind: J is the leading plate's drag, its own amplitudes and
  heave frequency are differentiated, and the shared phase angle and pitch
  frequency move both plates (both bodies' geometry transposed).
The gradients with respect to the motion parameters, the inflow velocity
and the initial state are checked against central finite differences of the
forward run at 1e-4 relative perturbations (bar: 1e-4 relative, plus an
absolute floor far below the gradients' scale for parameters J barely
depends on).  The plate's motion parameters use 1e-6: its forward run has
jumps (a probe changing its bracketing cell changes the 3-point derivative
stencil) within 1e-4 of the pitch amplitude, and central differences at
1e-5 and 1e-6 agree with the adjoint to ten digits.  The gradients do not depend on the checkpoint spacing; the
block ends at the state an ordinary run leaves (the next step agrees bit for
bit, so the ghost arrays do too); the torch.autograd.Function wrapper
returns the same gradients; a fine-block move inside the run is refused."""
import dataclasses

import numpy as np
import pytest

from biocfd import synth
from biocfd._lib import BCFD_E_STATE, BcfdError
from biocfd.adjoint import MOTION_PARAMS, adjoint_run_motion, run_function
from biocfd.solver import Solver

pytestmark = pytest.mark.gpu

N_STEPS = 6
DRAG = (1.0, 1.0, 0.0, 0.0)
BODIES = ("sphere", "plate")


def _base(body):
    if body == "sphere":
        return synth.heaving_sphere_single_block(n=24, n_steps=N_STEPS)
    if body == "pair":
        return synth.flapping_plate_pair(n_steps=N_STEPS, size="small")
    if body == "tandem":
        return synth.tandem_plates(n_steps=N_STEPS, moving=True, size="small")
    return synth.moving_plate_single_block(n=24, n_steps=N_STEPS)


def _mover(case):
    return next(q for q, b in enumerate(case.blocks) if b.motion is not None)


def _case(body, **motion):
    case = synth.replace(_base(body), epsi=1e-14, pc_ita_max=50000)
    q = _mover(case)
    blocks = list(case.blocks)
    own = {k: v for k, v in motion.items() if k in ("yamp", "a0_deg", "bfreq")}
    inputs = {k: v for k, v in motion.items() if k in ("phase_deg", "freq")}
    if own:
        blocks[q] = dataclasses.replace(blocks[q], motion=dataclasses.replace(blocks[q].motion, **own))
    mi = dataclasses.replace(case.motion, **inputs)
    return synth.replace(case, blocks=blocks, motion=mi)


def _params(case):
    mo, mi = case.blocks[_mover(case)].motion, case.motion
    return {"yamp": mo.yamp, "a0_deg": mo.a0_deg, "phase_deg": mi.phase_deg, "freq": mi.freq, "bfreq": mo.bfreq}


def _solver(case):
    # the run starts at the set-up: the initial fields and the ghost arrays
    # do not depend on the motion parameters there, only the placement does
    s = Solver(case)
    s.setup()
    return s


def _run(case, every=2, gradient=True, uc=None):
    return adjoint_run_motion(_solver(case), {}, N_STEPS, every=every, block=_mover(case), gradient=gradient,
                              stress_seed=DRAG, mu_f=1.0 / case.re, rho_f=1.0, uc=uc)


_BASE = {}


def _base_run(body):
    if body not in _BASE:
        case = _case(body)
        _BASE[body] = (case, _run(case))
    return _BASE[body]


@pytest.mark.parametrize("body", BODIES + ("pair", "tandem"))
def test_moving_body_gradients_vs_fd(body):
    case, (J, duc, g) = _base_run(body)
    assert np.isfinite(J) and J != 0.0
    if body != "sphere":
        s = _solver(case)
        assert s.counts(s.handles[_mover(case)])["TSCellCount"] > 0
    p0 = _params(case)
    gm = g["motion"]
    heave = abs(gm["yamp"]) * p0["yamp"]
    assert heave > 1e-6 * abs(J), gm  # the heave moves the drag
    rel = 1e-4 if body == "sphere" else 1e-6
    for name in MOTION_PARAMS:
        h = rel * abs(p0[name])
        jp = _run(_case(body, **{name: p0[name] + h}), gradient=False)
        jm = _run(_case(body, **{name: p0[name] - h}), gradient=False)
        fd = (jp - jm) / (2 * h)
        floor = 1e-7 * (heave + abs(J)) / abs(p0[name])
        assert abs(fd - gm[name]) <= 1e-4 * abs(fd) + floor, (name, fd, gm[name])
    h = 1e-4 * case.uc
    fd = (_run(case, gradient=False, uc=case.uc + h) - _run(case, gradient=False, uc=case.uc - h)) / (2 * h)
    assert abs(fd - duc) <= 1e-4 * abs(fd), (fd, duc)


@pytest.mark.parametrize("body", BODIES)
def test_moving_body_initial_state_vs_fd(body):
    case, (J, duc, g) = _base_run(body)
    s0 = _solver(case)
    g0 = s0.handles[0]
    state = {k: v.copy(order="F") for k, v in s0.fields(g0).items() if k in ("u", "v", "w", "p")}
    spec = case.blocks[0]
    m = np.zeros(spec.shape, bool, order="F")
    m[1:-1, 1:-1, 1:-1] = True
    m &= s0.tags(g0)["cell"] == 0
    rng = np.random.default_rng(5)
    eps = 1e-4

    def j_of(x):
        s = _solver(case)
        s.upload_fields(s.handles[0], x)
        return adjoint_run_motion(s, {}, N_STEPS, every=2, gradient=False, stress_seed=DRAG,
                                  mu_f=1.0 / case.re, rho_f=1.0)

    for field in ("u", "p"):
        scale = max(float(np.sqrt(np.mean(state[field] ** 2))), 1e-3)
        d = np.asfortranarray(rng.normal(size=spec.shape) * m * 1e-2 * scale)
        jp = j_of({**state, field: state[field] + eps * d})
        jm = j_of({**state, field: state[field] - eps * d})
        fd = (jp - jm) / (2 * eps)
        ad = float(np.sum(g[field] * d))
        assert abs(fd - ad) <= 1e-4 * abs(fd), (field, fd, ad)


@pytest.mark.parametrize("body", BODIES)
def test_checkpoint_spacing_and_final_state(body):
    case, (J, duc, g) = _base_run(body)
    for every in (1, N_STEPS):
        s = _solver(case)
        J2, duc2, g2 = adjoint_run_motion(s, {}, N_STEPS, every=every, stress_seed=DRAG, mu_f=1.0 / case.re,
                                          rho_f=1.0)
        assert J2 == J
        np.testing.assert_allclose(duc2, duc, rtol=1e-12)
        for k in MOTION_PARAMS:
            np.testing.assert_allclose(g2["motion"][k], g["motion"][k], rtol=1e-10, atol=1e-14 * abs(J))
        for k in ("u", "v", "w", "p"):
            np.testing.assert_allclose(g2[k], g[k], rtol=1e-10, atol=1e-14 * np.abs(g[k]).max())
        if every == N_STEPS:
            # the block is left where an ordinary run of the same steps ends,
            # ghost arrays included: one more step agrees bit for bit
            r = _solver(case)
            r.run(N_STEPS)
            for q in range(2):
                a, b = s.fields(s.handles[0]), r.fields(r.handles[0])
                for k in ("u", "v", "w", "p"):
                    np.testing.assert_array_equal(a[k], b[k])
                ta, tb = s.tags(s.handles[0]), r.tags(r.handles[0])
                np.testing.assert_array_equal(ta["cell"], tb["cell"])
                if q == 0:
                    s.run(1)
                    r.run(1)


def test_autograd_function_matches():
    torch = pytest.importorskip("torch")
    case, (J, duc, g) = _base_run("sphere")
    p0 = _params(case)

    def make(pv):
        c = _case("sphere", **dict(zip(MOTION_PARAMS, pv[1:])))
        return _solver(synth.replace(c, uc=pv[0]))

    s0 = _solver(case)
    st = s0.fields(s0.handles[0])
    x0 = [torch.from_numpy(np.ascontiguousarray(st[k])).requires_grad_(True) for k in ("u", "v", "w", "p")]
    params = torch.tensor([case.uc] + [p0[k] for k in MOTION_PARAMS], dtype=torch.float64, requires_grad=True)
    fn = run_function(make, {}, N_STEPS, every=2, moving=True, stress_seed=DRAG, mu_f=1.0 / case.re, rho_f=1.0)
    out = fn.apply(*x0, params)
    assert float(out.detach()) == J
    out.backward()
    want = [duc] + [g["motion"][k] for k in MOTION_PARAMS]
    np.testing.assert_allclose(params.grad.numpy(), want, rtol=1e-10, atol=1e-14 * abs(J))
    np.testing.assert_allclose(x0[0].grad.numpy(), np.ascontiguousarray(g["u"]), rtol=1e-10,
                               atol=1e-14 * np.abs(g["u"]).max())


def test_block_move_refused():
    case = synth.moving_plate_block_move(n_steps=3)
    s = Solver(case)
    s.setup()
    with pytest.raises(BcfdError, match=f"status {BCFD_E_STATE}"):
        adjoint_run_motion(s, {}, 3, every=1, block=1, stress_seed=DRAG, mu_f=1.0 / case.re, rho_f=1.0)
