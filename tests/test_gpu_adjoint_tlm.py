"""The GPU discrete adjoint through a moving body against the FP64
tangent-linear model of the oracle.

The oracle's dual-number build (oracle/orc_real.h) differentiates the whole
restated time step in forward mode -- the predictor, the forcing, the
Poisson solves, the coupling and the moving geometry through the per-step
re-Search (node placement, normals, normal distances, probe points) -- on
the same discrete branch (tags, brackets, upwind switches and iteration
counts come from the values).  bcfd_adjoint_run_motion differentiates the
GPU's FP64 drop-in steps in reverse mode.  Both are exact derivatives of the
same discrete program up to the solves' stopping points (the forward solves
stop at the increment test with epsi 1e-14, the adjoint solves at a residual
of 1e-13), so the bar is 1e-7 relative, far below the 1e-4 of the
central-difference checks; a gradient J does not depend on (the sphere's
pitch parameters) must vanish on both sides."""
import dataclasses

import numpy as np
import pytest

from biocfd import synth
from biocfd.adjoint import MOTION_PARAMS, adjoint_run_motion
from biocfd.solver import Solver
from oracle.bridge import drag_objective

pytestmark = pytest.mark.gpu

N_STEPS = 6
DRAG = (1.0, 1.0, 0.0, 0.0)
LIFT = (0.0, 0.0, 1.0, 1.0)


def _case(body):
    if body == "sphere":
        base = synth.heaving_sphere_single_block(n=24, n_steps=N_STEPS)
    else:
        base = synth.moving_plate_single_block(n=24, n_steps=N_STEPS)
    return synth.replace(base, epsi=1e-14, pc_ita_max=50000)


@pytest.mark.parametrize("body,seed", [("sphere", DRAG), ("plate", DRAG), ("plate", LIFT)])
def test_adjoint_matches_tangent_linear_oracle(body, seed):
    case = _case(body)
    mu_f = 1.0 / case.re
    s = Solver(case)
    s.setup()
    J, duc, g = adjoint_run_motion(s, {}, N_STEPS, every=2, block=0, stress_seed=seed, mu_f=mu_f, rho_f=1.0)
    s.close()
    Jt, d = drag_objective(case, N_STEPS, 0, seed, mu_f, 1.0, dual=True)
    # the GPU's FP64 drop-in steps are bit for bit the oracle's; the drag/lift
    # sums differ in order only (a fixed-order tree on the GPU)
    assert abs(J - Jt) <= 1e-13 * abs(Jt), (J, Jt)
    scale = max(abs(d[k]) * max(abs(v), 1e-3) for k, v in (
        ("yamp", case.blocks[0].motion.yamp), ("uc", case.uc)))
    for name in MOTION_PARAMS:
        tol = 1e-7 * abs(d[name]) + 1e-10 * scale
        assert abs(g["motion"][name] - d[name]) <= tol, (name, g["motion"][name], d[name])
    assert abs(duc - d["uc"]) <= 1e-7 * abs(d["uc"]), (duc, d["uc"])
    if body == "sphere":
        for name in ("a0_deg", "phase_deg", "freq"):
            assert d[name] == 0.0
