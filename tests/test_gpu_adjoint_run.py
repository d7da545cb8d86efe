"""Discrete adjoint of whole FP64 time steps with checkpointing.

Body-free block with the domain BCs: J = (1/N) sum_n <W, x^n>, a momentum flux
through a mid plane plus the pressure difference across a control volume.
Stationary sphere (IB forcing in the step): J = the time-averaged drag
coefficient (viscous + pressure) of stress_calculation.  The adjoint
gradients with respect to the inflow velocity uc and to the initial state are
checked against central finite differences at a 1e-4 relative perturbation
(bar: 1e-4 relative), the gradients are independent of the checkpoint spacing
(bitwise: recomputation reproduces the forward run exactly), and the block
ends at the state an ordinary run leaves."""
import numpy as np
import pytest

from biocfd import synth
from biocfd.adjoint import adjoint_run
from biocfd.solver import Solver

pytestmark = pytest.mark.gpu

N_STEPS = 12


def _case():
    case = synth.uniform_block(n=(24, 16, 16), lengths=(3.0, 2.0, 2.0))
    return synth.replace(case, epsi=1e-14, pc_ita_max=50000)


def _solver(case, init=None):
    if init is not None:
        case = synth.replace(case, init=[init])
    s = Solver(case)
    s.setup()
    return s


def _weights(case):
    spec = case.blocks[0]
    shp = spec.shape
    nx, ny, nz = spec.nx, spec.ny, spec.nz
    wu = np.zeros(shp, order="F")
    wu[nx // 2, 1:ny + 1, 1:nz + 1] = 1.0 / (ny * nz)  # mean u through a mid plane
    wp = np.zeros(shp, order="F")
    box = (slice(5, 9), slice(5, 11))
    wp[8, box[0], box[1]] = 1.0 / 24.0  # upstream face of a control volume
    wp[14, box[0], box[1]] = -1.0 / 24.0  # downstream face
    return {"u": wu, "p": wp}


def test_adjoint_gradient_uc_and_initial_state_vs_fd():
    case = _case()
    W = _weights(case)
    s = _solver(case)
    J, duc, g = adjoint_run(s, W, N_STEPS, every=5)
    assert np.isfinite(J) and abs(duc) > 0.0

    # dJ/duc: central differences at 1e-4 relative
    h = 1e-4 * case.uc
    jp = adjoint_run(_solver(case), W, N_STEPS, every=5, uc=case.uc + h, gradient=False)
    jm = adjoint_run(_solver(case), W, N_STEPS, every=5, uc=case.uc - h, gradient=False)
    fd = (jp - jm) / (2 * h)
    assert abs(fd - duc) <= 1e-4 * abs(fd), (fd, duc)

    # dJ/dx0 along a random direction on the interior (1e-4 relative size)
    init = case.init[0]
    rng = np.random.default_rng(7)
    spec = case.blocks[0]
    m = np.zeros(spec.shape, bool, order="F")
    m[1:-1, 1:-1, 1:-1] = True
    # each field's direction scaled to the field's own size (p starts at 0):
    # a 1e-4 relative step stays clear of the upwind switches of v and w
    scale = {k: max(float(np.sqrt(np.mean(init[k] ** 2))), 1e-3) if k != "p" else 1.0 for k in ("u", "v", "w", "p")}
    d = {k: np.asfortranarray(rng.normal(size=spec.shape) * m * scale[k]) for k in ("u", "v", "w", "p")}
    eps = 1e-4
    xp = {k: init[k] + eps * d[k] for k in d}
    xm = {k: init[k] - eps * d[k] for k in d}
    jp = adjoint_run(_solver(case, xp), W, N_STEPS, every=5, gradient=False)
    jm = adjoint_run(_solver(case, xm), W, N_STEPS, every=5, gradient=False)
    fd = (jp - jm) / (2 * eps)
    ad = sum(float(np.sum(g[k] * d[k])) for k in d)
    assert abs(fd - ad) <= 1e-4 * abs(fd), (fd, ad)


def test_checkpoint_spacing_does_not_change_the_gradient():
    case = _case()
    W = _weights(case)
    out = [adjoint_run(_solver(case), W, N_STEPS, every=k) for k in (1, 5, N_STEPS)]
    J0, d0, g0 = out[0]
    for J, duc, g in out[1:]:
        assert J == J0 and duc == d0
        for k in g0:
            np.testing.assert_array_equal(g[k], g0[k])


def test_block_left_at_forward_final_state():
    case = _case()
    W = _weights(case)
    s = _solver(case)
    J = adjoint_run(s, W, N_STEPS, every=4)[0]
    fa = s.fields(s.handles[0])
    r = _solver(case)
    acc = 0.0
    g = r.handles[0]
    for _ in range(N_STEPS):
        r.run(1)
        f = r.fields(g)
        acc += sum(float(np.sum(W[k] * f[k])) for k in W)
    fb = r.fields(g)
    for k in ("u", "v", "w", "p"):
        np.testing.assert_array_equal(fa[k], fb[k])
    assert abs(J - acc / N_STEPS) <= 1e-12 * abs(J)


def test_refuses_a_stress_objective_without_a_body():
    case = _case()
    s = _solver(case)
    from biocfd._lib import BcfdError
    with pytest.raises(BcfdError):
        adjoint_run(s, {}, 2, every=1, stress_seed=(1.0, 1.0, 0.0, 0.0))


@pytest.mark.parametrize("field", ["u", "v", "w", "p"])
def test_initial_state_gradient_per_field(field):
    """dJ/dx0 along one field at a time (each scaled to the field's size)."""
    case = _case()
    W = _weights(case)
    J, duc, g = adjoint_run(_solver(case), W, 4, every=2)
    init = case.init[0]
    spec = case.blocks[0]
    m = np.zeros(spec.shape, bool, order="F")
    m[1:-1, 1:-1, 1:-1] = True
    rng = np.random.default_rng(11)
    scale = max(float(np.sqrt(np.mean(init[field] ** 2))), 1e-3) if field != "p" else 1.0
    d = np.asfortranarray(rng.normal(size=spec.shape) * m * scale)
    eps = 1e-4
    jp = adjoint_run(_solver(case, {**init, field: init[field] + eps * d}), W, 4, every=2, gradient=False)
    jm = adjoint_run(_solver(case, {**init, field: init[field] - eps * d}), W, 4, every=2, gradient=False)
    fd = (jp - jm) / (2 * eps)
    ad = float(np.sum(g[field] * d))
    assert abs(fd - ad) <= 1e-4 * abs(fd), (field, fd, ad)



# ---- stationary sphere: drag objective through the IB forcing ---------------

SPHERE_STEPS = 6
DRAG = (1.0, 1.0, 0.0, 0.0)


def _sphere_case():
    case = synth.sphere_single_block(n=24, n_steps=1, diameter=0.3)
    return synth.replace(case, epsi=1e-14, pc_ita_max=50000)


def _sphere_solver(case, state=None):
    s = Solver(case)
    s.setup()
    s.run(1)  # the per-step re-Search settles the tags of the set-up
    if state is not None:
        s.upload_fields(s.handles[0], state)
    return s


def _drag_run(s, case, **kw):
    return adjoint_run(s, {}, SPHERE_STEPS, every=kw.pop("every", 2), stress_seed=DRAG,
                       mu_f=1.0 / case.re, rho_f=1.0, **kw)


def test_sphere_drag_gradient_uc_vs_fd():
    case = _sphere_case()
    J, duc, g = _drag_run(_sphere_solver(case), case)
    assert np.isfinite(J) and J != 0.0
    h = 1e-4 * case.uc
    jp = _drag_run(_sphere_solver(case), case, uc=case.uc + h, gradient=False)
    jm = _drag_run(_sphere_solver(case), case, uc=case.uc - h, gradient=False)
    fd = (jp - jm) / (2 * h)
    assert abs(fd - duc) <= 1e-4 * abs(fd), (fd, duc)


@pytest.mark.parametrize("field", ["u", "v", "w", "p"])
def test_sphere_drag_gradient_state_vs_fd(field):
    case = _sphere_case()
    s0 = _sphere_solver(case)
    g0 = s0.handles[0]
    state = {k: v.copy(order="F") for k, v in s0.fields(g0).items() if k in ("u", "v", "w", "p")}
    J, duc, g = _drag_run(s0, case)
    spec = case.blocks[0]
    cell = s0.tags(g0)["cell"]
    m = np.zeros(spec.shape, bool, order="F")
    m[1:-1, 1:-1, 1:-1] = True
    m &= cell == 0
    rng = np.random.default_rng(21)
    scale = max(float(np.sqrt(np.mean(state[field] ** 2))), 1e-3)
    d = np.asfortranarray(rng.normal(size=spec.shape) * m * scale)
    eps = 1e-4
    jp = _drag_run(_sphere_solver(case, {**state, field: state[field] + eps * d}), case, gradient=False)
    jm = _drag_run(_sphere_solver(case, {**state, field: state[field] - eps * d}), case, gradient=False)
    fd = (jp - jm) / (2 * eps)
    ad = float(np.sum(g[field] * d))
    assert abs(fd - ad) <= 1e-4 * abs(fd), (field, fd, ad)


def test_sphere_checkpoint_spacing_does_not_change_the_gradient():
    case = _sphere_case()
    out = [_drag_run(_sphere_solver(case), case, every=k) for k in (1, 3, SPHERE_STEPS)]
    J0, d0, g0 = out[0]
    for J, duc, g in out[1:]:
        assert J == J0 and duc == d0
        for k in g0:
            np.testing.assert_array_equal(g[k], g0[k])


KIN0 = np.array([0.05, 0.1, 0.2, 0.0, 0.0, 0.0, 0.0, 0.0])


def _set_kin(s, case, kin):
    import ctypes as C
    spec = case.blocks[0]
    full = np.ascontiguousarray(np.concatenate([kin, np.asarray(spec.piv, dtype=np.float64)]))
    check = __import__("biocfd._lib", fromlist=["check"]).check
    check(s.L.bcfd_block_set_kinematics(s.handles[0], full.ctypes.data_as(C.POINTER(C.c_double))), "kin")


@pytest.mark.parametrize("p", [0, 1, 2])
def test_sphere_drag_gradient_kinematics_vs_fd(p):
    """dJ/d(xdot, ydot, yddot): the sphere's surface translating (and
    accelerating) at constant rates with its geometry fixed."""
    case = _sphere_case()

    def run(kin, gradient):
        s = _sphere_solver(case)
        _set_kin(s, case, kin)
        return _drag_run(s, case, gradient=gradient)

    J, duc, g = run(KIN0, True)
    h = 1e-4 * max(abs(KIN0[p]), 1.0)
    e = np.zeros(8)
    e[p] = h
    fd = (run(KIN0 + e, False) - run(KIN0 - e, False)) / (2 * h)
    assert abs(fd - g["kin"][p]) <= 1e-4 * abs(fd), (p, fd, g["kin"][p])


# ---- two blocks: coarse block with the domain BCs + fine block with the sphere ----

TWO_STEPS = 4


def _two_case():
    return synth.replace(synth.small_two_block(n_steps=1), epsi=1e-14, pc_ita_max=50000)


def _two_solver(case, state=None):
    s = Solver(case)
    s.setup()
    s.run(1)
    if state is not None:
        s.upload_fields(s.handles[1], state)
    return s


def _two_drag(s, case, **kw):
    """Time-averaged drag on the fine block's sphere; the inflow uc acts only
    through the coarse block's BCs, so its gradient crosses every coupling
    transpose (face fills, restrictions, the solves' boundary data)."""
    g = s.handles[1]
    from biocfd import adjoint as adj
    import ctypes as C
    spec = case.blocks[1]
    z = np.zeros(spec.shape, order="F")
    P = C.POINTER(C.c_double)
    cfg = s.config(0)
    if "uc" in kw:
        cfg.uc = kw.pop("uc")
    gradient = kw.pop("gradient", True)
    every = kw.pop("every", 2)
    seed = np.array(DRAG)
    J, duc = C.c_double(), C.c_double()
    grads = [np.zeros(spec.shape, order="F") for _ in range(4)]
    kin = np.zeros(8)
    null = C.cast(None, P)
    from biocfd._lib import check
    check(s.L.bcfd_adjoint_run(g, C.byref(cfg), TWO_STEPS, every, *(z.ctypes.data_as(P) for _ in range(4)),
                               seed.ctypes.data_as(P), 1.0 / case.re, 1.0, 1e-13, 200000, C.byref(J),
                               C.byref(duc) if gradient else null, kin.ctypes.data_as(P) if gradient else null,
                               *((a.ctypes.data_as(P) for a in grads) if gradient else (null,) * 4)), "adjoint_run")
    if not gradient:
        return J.value
    return J.value, duc.value, dict(zip("uvwp", grads))


def test_two_block_drag_gradient_uc_vs_fd():
    case = _two_case()
    J, duc, g = _two_drag(_two_solver(case), case)
    assert np.isfinite(J) and duc != 0.0
    h = 1e-4 * case.uc
    jp = _two_drag(_two_solver(case), case, uc=case.uc + h, gradient=False)
    jm = _two_drag(_two_solver(case), case, uc=case.uc - h, gradient=False)
    fd = (jp - jm) / (2 * h)
    assert abs(fd - duc) <= 1e-4 * abs(fd), (fd, duc)


@pytest.mark.parametrize("field", ["u", "p"])
def test_two_block_drag_gradient_fine_state_vs_fd(field):
    case = _two_case()
    s0 = _two_solver(case)
    g1 = s0.handles[1]
    state = {k: v.copy(order="F") for k, v in s0.fields(g1).items() if k in ("u", "v", "w", "p")}
    J, duc, g = _two_drag(s0, case)
    spec = case.blocks[1]
    cell = s0.tags(g1)["cell"]
    m = np.zeros(spec.shape, bool, order="F")
    m[1:-1, 1:-1, 1:-1] = True
    m &= cell == 0
    rng = np.random.default_rng(31)
    scale = max(float(np.sqrt(np.mean(state[field] ** 2))), 1e-3)
    d = np.asfortranarray(rng.normal(size=spec.shape) * m * scale)
    eps = 1e-4
    jp = _two_drag(_two_solver(case, {**state, field: state[field] + eps * d}), case, gradient=False)
    jm = _two_drag(_two_solver(case, {**state, field: state[field] - eps * d}), case, gradient=False)
    fd = (jp - jm) / (2 * eps)
    ad = float(np.sum(g[field] * d))
    assert abs(fd - ad) <= 1e-4 * abs(fd), (field, fd, ad)


def test_two_block_checkpoint_spacing_does_not_change_the_gradient():
    case = _two_case()
    out = [_two_drag(_two_solver(case), case, every=k) for k in (1, TWO_STEPS)]
    (J0, d0, g0), (J1, d1, g1) = out
    assert J0 == J1 and d0 == d1
    for k in g0:
        np.testing.assert_array_equal(g0[k], g1[k])


def test_adjoint_solver_precision_agrees():
    """The adjoint Poisson solves in FP64 SOR and in FP32 sweeps with FP64
    defect correction stop at the same FP64 residual target, so the
    gradients agree far inside the finite-difference bar."""
    case = _sphere_case()
    out = [_drag_run(_sphere_solver(case), case, solve_precision=sp) for sp in (0, 1)]
    (j0, d0, g0), (j1, d1, g1) = out
    assert j0 == j1  # the forward steps are the same FP64 steps
    assert abs(d0 - d1) <= 1e-8 * abs(d0), (d0, d1)
    for k in ("u", "v", "w", "p"):
        n = np.linalg.norm(g0[k])
        assert np.linalg.norm(g1[k] - g0[k]) <= 1e-8 * max(n, 1e-30), k
    assert np.allclose(g0["kin"], g1["kin"], rtol=1e-8, atol=1e-12 * np.abs(g0["kin"]).max())


# ---- stationary thin plate: the predictor's thin-surface ghost substitution ----

PLATE_STEPS = 6


def _plate_case():
    case = synth.plate_single_block(n=24, n_steps=1)
    return synth.replace(case, epsi=1e-14, pc_ita_max=50000)


def _plate_solver(case, state=None):
    s = Solver(case)
    s.setup()
    s.run(1)  # the ghost arrays of the run's start come from this step
    if state is not None:
        s.upload_fields(s.handles[0], state)
    return s


def _plate_run(s, case, **kw):
    return adjoint_run(s, {}, PLATE_STEPS, every=kw.pop("every", 2), stress_seed=DRAG,
                       mu_f=1.0 / case.re, rho_f=1.0, **kw)


def test_plate_drag_gradient_vs_fd():
    """Every IB cell of the plate is a thin-surface cell: the transposes of
    the ghost substitution, the final restore and the ghost calls carry the
    gradient through them.  The ghost arrays the run starts from are held
    fixed (they came from the step before), as in the forward runs of the
    finite differences."""
    case = _plate_case()
    s0 = _plate_solver(case)
    g0 = s0.handles[0]
    assert s0.counts(g0)["TSCellCount"] > 0
    state = {k: v.copy(order="F") for k, v in s0.fields(g0).items() if k in ("u", "v", "w", "p")}
    J, duc, g = _plate_run(s0, case)
    assert np.isfinite(J) and J != 0.0
    h = 1e-4 * case.uc
    jp = _plate_run(_plate_solver(case), case, uc=case.uc + h, gradient=False)
    jm = _plate_run(_plate_solver(case), case, uc=case.uc - h, gradient=False)
    fd = (jp - jm) / (2 * h)
    assert abs(fd - duc) <= 1e-4 * abs(fd), (fd, duc)
    spec = case.blocks[0]
    m = np.zeros(spec.shape, bool, order="F")
    m[1:-1, 1:-1, 1:-1] = True
    m &= s0.tags(g0)["cell"] == 0
    rng = np.random.default_rng(33)
    eps = 1e-4
    for field in ("u", "v", "p"):
        scale = max(float(np.sqrt(np.mean(state[field] ** 2))), 1e-3)
        d = np.asfortranarray(rng.normal(size=spec.shape) * m * scale)
        jp = _plate_run(_plate_solver(case, {**state, field: state[field] + eps * d}), case, gradient=False)
        jm = _plate_run(_plate_solver(case, {**state, field: state[field] - eps * d}), case, gradient=False)
        fd = (jp - jm) / (2 * eps)
        ad = float(np.sum(g[field] * d))
        assert abs(fd - ad) <= 1e-4 * abs(fd), (field, fd, ad)


def test_plate_checkpoint_spacing_does_not_change_the_gradient():
    case = _plate_case()
    out = [_plate_run(_plate_solver(case), case, every=k) for k in (1, 4, PLATE_STEPS)]
    J0, d0, g0 = out[0]
    for J, duc, g in out[1:]:
        assert J == J0 and duc == d0
        for k in g0:
            np.testing.assert_array_equal(g[k], g0[k])


PLATE_KIN0 = np.array([0.05, 0.1, 0.2, 0.3, 0.4, -0.3, -0.4, 0.0])


@pytest.mark.parametrize("p", [1, 3, 4])
def test_plate_drag_gradient_kinematics_vs_fd(p):
    """dJ/d(ydot, thetaDot1, thetaDDot1) of the thin plate (surface 51):
    rotation rates reach the surface velocities and dp/dn of the forcing, of
    the ghost calls and of the drag/lift."""
    case = _plate_case()

    def run(kin, gradient):
        s = _plate_solver(case)
        _set_kin(s, case, kin)
        return _plate_run(s, case, gradient=gradient)

    J, duc, g = run(PLATE_KIN0, True)
    # the plate's forward run jumps where a probe changes its bracketing cell
    # (within 1e-4 of these rates), so the differences take a smaller step
    h = 1e-6 * max(abs(PLATE_KIN0[p]), 1.0)
    e = np.zeros(8)
    e[p] = h
    fd = (run(PLATE_KIN0 + e, False) - run(PLATE_KIN0 - e, False)) / (2 * h)
    assert abs(fd - g["kin"][p]) <= 1e-4 * abs(fd), (p, fd, g["kin"][p])
