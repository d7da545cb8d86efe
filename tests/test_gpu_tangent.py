"""Tangent-linear model and adjoint of the momentum predictor
(nsMomentum2order in dual numbers).  The tangent's value part is bitwise the
FP64 predictor the drop-in path computes, and its tangent matches central
finite differences of that predictor along a random direction (the stencil
is quadratic in (u,v,w) and linear in p, so central differences are exact up
to round-off away from upwind switches).  The adjoint is the transpose of the
tangent: <J d, s> = <d, J^T s> field by field."""
import numpy as np
import pytest

from biocfd import synth
from biocfd._lib import BcfdError, check
from biocfd.adjoint import momentum_adjoint, momentum_tangent
from biocfd.solver import Solver

pytestmark = pytest.mark.gpu


def _sphere():
    case = synth.sphere_single_block(n=24, n_steps=1, diameter=0.3)
    s = Solver(case)
    s.setup()
    s.run(1)  # non-trivial p and a perturbed velocity field
    return s, case, s.handles[0]


def _mask(s, g, spec):
    cell = s.tags(g)["cell"]
    m = np.zeros(spec.shape, bool, order="F")
    m[1:-1, 1:-1, 1:-1] = True
    return m & (cell == 0)


def _predictor(s, g, case, fields):
    s.upload_fields(g, fields)
    check(s.L.bcfd_ns_momentum_2order(g, case.dt, case.re), "ns_momentum_2order")
    f = s.fields(g)
    return f["ut"], f["vt"], f["wt"]


def test_tangent_value_bitwise_and_fd():
    s, case, g = _sphere()
    spec = case.blocks[0]
    base = s.fields(g)
    x0 = {k: base[k].copy(order="F") for k in ("u", "v", "w", "p")}
    rng = np.random.default_rng(11)
    m = _mask(s, g, spec)
    assert m.sum() > 0.8 * spec.n_interior
    # the direction lives on fluid values that are not pinned to zero: the
    # boundary conditions hold v = 0 on a wall face, so |v(i) + v(i+1)| sits
    # on its kink at exactly zero, where central differences give 0 and the
    # tangent takes the + branch
    d = {k: np.asfortranarray(rng.normal(0.0, 1.0, spec.shape) * (m & (x0[k] != 0.0)))
         for k in ("u", "v", "w", "p")}

    # value part: bitwise the predictor at the same fields
    s.upload_fields(g, x0)
    val, tan = momentum_tangent(s, g, d["u"], d["v"], d["w"], d["p"])
    ref = _predictor(s, g, case, x0)
    for q in range(3):
        np.testing.assert_array_equal(val[q][m], ref[q][m])
        assert np.all(val[q][~m] == 0.0) and np.all(tan[q][~m] == 0.0)

    # tangent part: central differences of the FP64 predictor
    h = 1e-8
    fp = _predictor(s, g, case, {k: x0[k] + h * d[k] for k in x0})
    fm = _predictor(s, g, case, {k: x0[k] - h * d[k] for k in x0})
    for q in range(3):
        fd = (fp[q] - fm[q]) / (2 * h)
        scale = np.abs(tan[q][m]).max()
        err = np.abs(fd[m] - tan[q][m])
        # upwind switches inside [-h, h] are rare; the rest agree to round-off
        bad = err > 1e-6 * scale
        assert bad.sum() <= max(5, 1e-3 * m.sum()), (q, bad.sum(), err.max() / scale)
        assert np.median(err) < 1e-8 * scale


def test_tangent_linear_in_direction():
    s, case, g = _sphere()
    spec = case.blocks[0]
    rng = np.random.default_rng(5)
    d1 = [np.asfortranarray(rng.normal(size=spec.shape)) for _ in range(4)]
    d2 = [np.asfortranarray(rng.normal(size=spec.shape)) for _ in range(4)]
    _, t1 = momentum_tangent(s, g, *d1)
    _, t2 = momentum_tangent(s, g, *d2)
    _, t12 = momentum_tangent(s, g, *(2.0 * a - 3.0 * b for a, b in zip(d1, d2)))
    for q in range(3):
        np.testing.assert_allclose(t12[q], 2.0 * t1[q] - 3.0 * t2[q], rtol=1e-12, atol=1e-9)


def test_tangent_refuses_thin_surface_cells():
    case = synth.plate_single_block(n=24, n_steps=1)
    s = Solver(case)
    s.setup()
    g = s.handles[0]
    if s.counts(g)["TSCellCount"] == 0:
        pytest.skip("plate produced no thin-surface cells")
    z = np.zeros(case.blocks[0].shape, order="F")
    with pytest.raises(BcfdError):
        momentum_tangent(s, g, z, z, z, z)


@pytest.mark.parametrize("field", [0, 1, 2, 3])
def test_adjoint_is_transpose_of_tangent(field):
    s, case, g = _sphere()
    spec = case.blocks[0]
    rng = np.random.default_rng(100 + field)
    z = np.zeros(spec.shape, order="F")
    d = [z, z, z, z]
    d[field] = np.asfortranarray(rng.normal(size=spec.shape))
    seeds = [np.asfortranarray(rng.normal(size=spec.shape)) for _ in range(3)]
    _, tan = momentum_tangent(s, g, *d)
    adj = momentum_adjoint(s, g, *seeds)
    m = _mask(s, g, spec)
    lhs = sum(float(np.sum(tan[q][m] * seeds[q][m])) for q in range(3))
    rhs = float(np.sum(d[field] * adj[field]))
    scale = sum(float(np.sum(np.abs(tan[q][m] * seeds[q][m]))) for q in range(3))
    assert abs(lhs - rhs) <= 1e-12 * scale, (lhs, rhs, scale)
    # the adjoint is deterministic
    adj2 = momentum_adjoint(s, g, *seeds)
    for a, b in zip(adj, adj2):
        np.testing.assert_array_equal(a, b)


def test_adjoint_unit_columns():
    """J^T e_C at one fluid cell C equals the row of J read off by unit
    tangents at every input point of its stencil."""
    s, case, g = _sphere()
    spec = case.blocks[0]
    C = (6, 7, 8)  # natural-layout index of an interior fluid cell
    assert _mask(s, g, spec)[C]
    z = np.zeros(spec.shape, order="F")
    e = z.copy(order="F")
    e[C] = 1.0
    adj = momentum_adjoint(s, g, e, z, z)  # gradient of ut(C)
    for f in range(4):
        for off in ((0, 0, 0), (1, 0, 0), (-1, 0, 0), (2, 0, 0), (0, -1, 0), (1, -1, 0), (0, 0, 2)):
            X = tuple(c + o for c, o in zip(C, off))
            d = [z, z, z, z]
            d[f] = z.copy(order="F")
            d[f][X] = 1.0
            _, tan = momentum_tangent(s, g, *d)
            assert tan[0][C] == adj[f][X], (f, off, tan[0][C], adj[f][X])
