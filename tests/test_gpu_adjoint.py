"""Adjoint of the Poisson solve on a stretched coarse block (boundary folding,
non-uniform spacing: A is not symmetric): A^{-1} and A^{-T} against dense
solves of the same matrix assembled from the block's line tables, the
dot-product identity <A^{-1} r1, r2> = <r1, A^{-T} r2>, and torch's gradcheck
of the autograd wrapper."""
import numpy as np
import pytest

from biocfd import synth
from biocfd.adjoint import poisson_function, poisson_solve, poisson_solve_adjoint
from biocfd.solver import Solver

pytestmark = pytest.mark.gpu

TOL = 1e-13  # solver residual; the comparisons below hold to ~1e-9 relative


def _stretched(n, ratio):
    w = ratio ** np.arange(n)
    return np.concatenate([[0.0], np.cumsum(w / w.sum())])


def _block(nx, ny, nz):
    spec = synth.BlockSpec(nx, ny, nz, _stretched(nx, 1.15), _stretched(ny, 0.9), _stretched(nz, 1.05),
                           omega=1.6, is_coarse=True)
    case = synth.Case(name="stretched", blocks=[spec], dt=1e-3)
    case.init = [synth.noisy_initial(spec, 1.0, np.random.default_rng(3))]
    s = Solver(case)
    s.setup()
    g = s.handles[0]
    from biocfd._lib import check
    check(s.L.bcfd_tagging_th(g), "tagging")
    check(s.L.bcfd_cellcount_solid(g), "cellcount")
    return s, g, spec


def _dense(s, g, spec):
    nx, ny, nz = spec.nx, spec.ny, spec.nz
    ax = s.read(g, "Acx", 3 * nx).reshape(nx, 3, order="F")
    ay = s.read(g, "Acy", 3 * ny).reshape(ny, 3, order="F")
    az = s.read(g, "Acz", 3 * nz).reshape(nz, 3, order="F")
    idx = lambda i, j, k: (i - 2) + nx * ((j - 2) + ny * (k - 2))
    n = nx * ny * nz
    A = np.zeros((n, n))
    for k in range(2, nz + 2):
        for j in range(2, ny + 2):
            for i in range(2, nx + 2):
                r = idx(i, j, k)
                A[r, r] = ax[i - 2, 1] + ay[j - 2, 1] + az[k - 2, 1]
                for (a, b, e, coef) in ((-1, 0, 0, ax[i - 2, 0]), (1, 0, 0, ax[i - 2, 2]),
                                        (0, -1, 0, ay[j - 2, 0]), (0, 1, 0, ay[j - 2, 2]),
                                        (0, 0, -1, az[k - 2, 0]), (0, 0, 1, az[k - 2, 2])):
                    ii, jj, kk = i + a, j + b, k + e
                    if 2 <= ii <= nx + 1 and 2 <= jj <= ny + 1 and 2 <= kk <= nz + 1:
                        A[r, idx(ii, jj, kk)] = coef
    return A


def _interior(spec, rng):
    r = np.zeros(spec.shape, order="F")
    r[1:-1, 1:-1, 1:-1] = rng.standard_normal((spec.nx, spec.ny, spec.nz))
    return r


@pytest.mark.parametrize("precision", [0, 1])
def test_adjoint_solve_against_dense_transpose(precision):
    # 0: FP64 SOR; 1: FP32 sweeps (transposed FP32 tables) + FP64 correction
    s, g, spec = _block(6, 5, 4)
    s.L.bcfd_adjoint_set_solver(precision)
    A = _dense(s, g, spec)
    assert np.abs(A - A.T).max() > 1e-3 * np.abs(A).max()  # genuinely non-symmetric
    rng = np.random.default_rng(11)
    r = _interior(spec, rng)
    rv = r[1:-1, 1:-1, 1:-1].ravel(order="F")
    x = poisson_solve(s, g, r, TOL)[1:-1, 1:-1, 1:-1].ravel(order="F")
    y = poisson_solve_adjoint(s, g, r, TOL)[1:-1, 1:-1, 1:-1].ravel(order="F")
    xr, yr = np.linalg.solve(A, rv), np.linalg.solve(A.T, rv)
    assert np.linalg.norm(x - xr) <= 1e-9 * np.linalg.norm(xr)
    assert np.linalg.norm(y - yr) <= 1e-9 * np.linalg.norm(yr)
    s.L.bcfd_adjoint_set_solver(1)
    s.close()


def test_adjoint_dot_product_identity():
    s, g, spec = _block(24, 20, 16)
    rng = np.random.default_rng(5)
    r1, r2 = _interior(spec, rng), _interior(spec, rng)
    x1 = poisson_solve(s, g, r1, TOL)
    y2 = poisson_solve_adjoint(s, g, r2, TOL)
    lhs, rhs = np.vdot(x1, r2), np.vdot(r1, y2)
    assert abs(lhs - rhs) <= 1e-9 * abs(lhs), (lhs, rhs)
    s.close()


def test_autograd_gradcheck():
    torch = pytest.importorskip("torch")
    s, g, spec = _block(5, 4, 4)
    f = poisson_function(s, g, TOL)
    r = torch.zeros(spec.shape, dtype=torch.float64)
    r[1:-1, 1:-1, 1:-1] = torch.randn(spec.nx, spec.ny, spec.nz, dtype=torch.float64,
                                      generator=torch.Generator().manual_seed(2))
    mask = torch.zeros(spec.shape, dtype=torch.float64)
    mask[1:-1, 1:-1, 1:-1] = 1.0
    r = r.permute(2, 1, 0).contiguous().permute(2, 1, 0)  # x fastest in memory
    r.requires_grad_(True)
    w = torch.randn(spec.shape, dtype=torch.float64, generator=torch.Generator().manual_seed(4)) * mask
    loss = lambda rr: (f.apply(rr * mask) * w).sum()
    assert torch.autograd.gradcheck(loss, (r,), eps=1e-6, atol=1e-7, rtol=1e-6)
    s.close()


def _coupling(s, it, comp, op, x, out_shape):
    import ctypes as C
    from biocfd._lib import check
    x = np.asfortranarray(x, dtype=np.float64)
    out = np.zeros(out_shape, order="F")
    check(s.L.bcfd_coupling_apply(it, comp, op, x.ctypes.data_as(C.POINTER(C.c_double)),
                                  out.ctypes.data_as(C.POINTER(C.c_double))), "coupling_apply")
    return out


@pytest.mark.parametrize("comp", [0, 1, 2, 3])
def test_coupling_transposes_dot_product(comp):
    # <P c, f> = <c, P^T f> for the face fill, <R f, c> = <f, R^T c> for the
    # restriction (each map's transpose is a separate kernel)
    case = synth.small_two_block(n_steps=1)
    s = Solver(case)
    s.setup()
    it = s.ifaces[0]
    A, B = case.blocks[0].shape, case.blocks[1].shape
    rng = np.random.default_rng(7 + comp)
    c, f = rng.standard_normal(A), rng.standard_normal(B)
    Pc = _coupling(s, it, comp, 0, c, B)
    PTf = _coupling(s, it, comp, 1, f, A)
    assert np.count_nonzero(Pc) > 0 and np.count_nonzero(PTf) > 0
    lhs, rhs = np.vdot(Pc, f), np.vdot(c, PTf)
    assert abs(lhs - rhs) <= 1e-12 * np.sqrt(np.vdot(Pc, Pc) * np.vdot(f, f)), (lhs, rhs)
    Rf = _coupling(s, it, comp, 2, f, A)
    RTc = _coupling(s, it, comp, 3, c, B)
    assert np.count_nonzero(Rf) > 0 and np.count_nonzero(RTc) > 0
    lhs, rhs = np.vdot(Rf, c), np.vdot(f, RTc)
    assert abs(lhs - rhs) <= 1e-12 * np.sqrt(np.vdot(Rf, Rf) * np.vdot(c, c)), (lhs, rhs)
    s.close()
