"""The oracle's FP64 tangent-linear build (oracle/orc_real.h, -DORC_DUAL).

The dual-number build runs the same restated time step with a value and six
tangent lanes per floating-point number.  Checked here, on the CPU:
* its value part is bit for bit the plain oracle's (fields, tags, lists,
  iteration counts, drag/lift) over several steps of a moving thin plate
  (thin-surface cells, per-step re-Search) and of a coarse/fine pair whose
  fine block moves with its plate;
* its tangents of J = time-averaged drag with respect to the five motion
  parameters of the moving body and the inflow velocity equal central
  differences of the plain oracle (heaving sphere at 1e-4 relative steps;
  the plate at 1e-6, since its forward run has jumps within 1e-4 of the
  pitch amplitude where a probe changes its bracketing cell).
The GPU adjoint is compared with these tangents in
tests/test_gpu_adjoint_tlm.py."""
import dataclasses

import numpy as np
import pytest

from biocfd import synth
from oracle.bridge import TANGENT_PARAMS, Oracle, drag_objective

N_STEPS = 4
DRAG = (1.0, 1.0, 0.0, 0.0)


def _base(body):
    if body == "sphere":
        return synth.heaving_sphere_single_block(n=24, n_steps=N_STEPS)
    return synth.moving_plate_single_block(n=24, n_steps=N_STEPS)


def _case(body, **p):
    case = synth.replace(_base(body), epsi=1e-14, pc_ita_max=50000)
    spec = case.blocks[0]
    own = {k: v for k, v in p.items() if k in ("yamp", "a0_deg", "bfreq")}
    inputs = {k: v for k, v in p.items() if k in ("phase_deg", "freq")}
    if own:
        spec = dataclasses.replace(spec, motion=dataclasses.replace(spec.motion, **own))
    kw = {"uc": p["uc"]} if "uc" in p else {}
    return synth.replace(case, blocks=[spec], motion=dataclasses.replace(case.motion, **inputs), **kw)


def _params(case):
    mo, mi = case.blocks[0].motion, case.motion
    return {"yamp": mo.yamp, "a0_deg": mo.a0_deg, "phase_deg": mi.phase_deg, "freq": mi.freq,
            "bfreq": mo.bfreq, "uc": case.uc}


def _compare_runs(case, n_steps):
    a, b = Oracle(), Oracle(dual=True)
    for o in (a, b):
        o.setup(case)
    for _ in range(n_steps):
        for o in (a, b):
            o.step()
        assert a.iters() == b.iters()
        for g in range(1, a.nblocks + 1):
            for nm in ("u", "v", "w", "p", "ut", "vt", "wt", "pc"):
                np.testing.assert_array_equal(a.arr(g, nm), b.arr(g, nm), err_msg=nm)
            for nm in ("cell", "cell2", "nodeIdTag"):
                np.testing.assert_array_equal(a.arr(g, nm), b.arr(g, nm), err_msg=nm)
            for nm in ("ibCellCount", "fluidCellCount", "TSCellCount"):
                assert a.geti(g, nm) == b.geti(g, nm), nm
            assert a.getf(g, "derr2") == b.getf(g, "derr2")
    # no seed was set: every tangent stays zero
    for g in range(1, b.nblocks + 1):
        for lane in range(b.lanes):
            assert not np.any(b.tangent(g, "u", lane))


def test_dual_values_equal_plain_oracle_moving_plate():
    case = _case("plate")
    _compare_runs(case, 3)


def test_dual_values_equal_plain_oracle_block_moves():
    # a coarse/fine pair whose fine block moves with the plate (coupling,
    # fine-block moves and the moved block's re-tagging)
    case = synth.moving_plate_block_move(n_steps=3)
    _compare_runs(case, 3)


@pytest.mark.parametrize("body", ["sphere", "plate"])
def test_tangents_match_central_differences(body):
    case = _case(body)
    mu_f = 1.0 / case.re
    J, d = drag_objective(case, N_STEPS, 0, DRAG, mu_f, 1.0, dual=True)
    assert J == drag_objective(case, N_STEPS, 0, DRAG, mu_f, 1.0)
    p0 = _params(case)
    assert abs(d["yamp"]) * p0["yamp"] > 1e-6 * abs(J), d
    rel = 1e-4 if body == "sphere" else 1e-6
    for name in TANGENT_PARAMS:
        h = rel * abs(p0[name])
        jp = drag_objective(_case(body, **{name: p0[name] + h}), N_STEPS, 0, DRAG, mu_f, 1.0)
        jm = drag_objective(_case(body, **{name: p0[name] - h}), N_STEPS, 0, DRAG, mu_f, 1.0)
        fd = (jp - jm) / (2 * h)
        floor = 1e-8 * abs(J) / abs(p0[name])
        assert abs(fd - d[name]) <= 1e-5 * abs(fd) + floor, (name, fd, d[name])
