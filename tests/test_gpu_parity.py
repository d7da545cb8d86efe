"""GPU parity against the CPU oracle, routine by routine, through the C ABI.

Bar: bit-exact for every tag, index list, donor element and interface
table; bit-exact FP64 fields and identical SOR iteration counts for the
drop-in path (the kernels round exactly like the serial reference build).
"""
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


def test_setup_single_block_sphere():
    case = synth.sphere_single_block(n=24, n_steps=1, diameter=0.3)
    o, s = _pair(case)
    compare_search(o, s, "setup")
    g = s.handles[0]
    for nm in ("xcent", "ycent", "zcent", "cosAlpha", "cosBeta", "cosGamma", "element_length"):
        assert_bitwise(nm, o.arr(1, nm), s.read(g, nm, len(case.blocks[0].mesh.tris)))
    for nm in ("Acx", "Acy", "Acz"):
        ref = o.arr(1, nm)
        assert_bitwise(nm, ref, s.read(g, nm, ref.size).reshape(ref.shape, order="F"))
    for t in ("uu", "vv", "ww", "uv", "uw", "vu", "vw", "wu", "wv"):
        for pre in ("ca_", "ck_"):
            ref = o.arr(1, pre + t)
            got = s.read(g, pre + t, ref.size).reshape(ref.shape, order="F")
            # columns 2..n are defined by the reference; the rest are unused
            assert_bitwise(pre + t, ref[:, 1:-2], got[:, 1:-2])


@pytest.mark.parametrize("n", [20, 32])
def test_one_step_single_block_phases(n):
    case = synth.sphere_single_block(n=n, n_steps=1, diameter=0.3)
    o, s = _pair(case)
    o.momentum_phase()
    s.momentum_phase()
    compare_fields(o, s, "momentum phase")
    o.poisson_phase()
    s.poisson_phase()
    compare_fields(o, s, "poisson phase")
    compare_iters(o, s, "poisson phase")
    g = s.handles[0]
    assert_bitwise("pc", o.arr(1, "pc"), s.read(g, "pc", o.arr(1, "pc").size).reshape(o.arr(1, "pc").shape, order="F"))
    o.research_phase()
    s.research_phase()
    compare_search(o, s, "research phase")
    compare_fields(o, s, "research phase")
    assert o.err(1) == 0


def test_steps_single_block_native_driver():
    case = synth.sphere_single_block(n=24, n_steps=3, diameter=0.3)
    o, s = _pair(case)
    for _ in range(3):
        o.step()
    s.run(3)
    compare_fields(o, s, "3 steps")
    compare_iters(o, s, "3 steps")
    compare_search(o, s, "3 steps")


def test_interface_tables():
    case = synth.small_two_block()
    o, s = _pair(case)
    for nm in ("px", "py", "pz", "ux", "uy", "uz", "vx", "vy", "vz", "wx", "wy", "wz"):
        ref, cnt = o.table(1, nm)
        out = np.zeros(3 * ref.shape[1], np.int64)
        import ctypes as C
        c = C.c_int64()
        from biocfd._lib import check
        check(s.L.bcfd_interface_table(s.ifaces[0], nm.encode(), out.ctypes.data_as(C.POINTER(C.c_int64)),
                                       out.size, C.byref(c)), "interface_table")
        assert c.value == cnt, nm
        got = out.reshape(-1, 3).T
        assert np.array_equal(ref[:, :cnt], got[:, :cnt]), nm


def test_two_block_steps():
    case = synth.small_two_block(n_steps=2)
    o, s = _pair(case)
    compare_search(o, s, "setup")
    for k in range(2):
        o.momentum_phase()
        s.momentum_phase()
        compare_fields(o, s, f"step {k} momentum")
        o.poisson_phase()
        s.poisson_phase()
        compare_fields(o, s, f"step {k} poisson")
        compare_iters(o, s, f"step {k} poisson")
        o.research_phase()
        s.research_phase()
        compare_fields(o, s, f"step {k} research")
        compare_search(o, s, f"step {k} research")


# the per-element contributions are the reference's expressions; only the
# summation order differs (element order on the CPU, a fixed tree on the GPU)
STRESS_RTOL = 1e-9


@pytest.mark.parametrize("maker", ["sphere", "plate"])
def test_stress_calculation(maker):
    case = (synth.sphere_single_block(n=24, n_steps=1, diameter=0.3) if maker == "sphere"
            else synth.plate_single_block(n=24, n_steps=1))
    o, s = _pair(case)
    o.step()
    s.run(1)
    mu_f, rho_f = 1.0 / case.re, 1.0
    o.L.orc_stress_calculation(1, mu_f, rho_f)
    ref = np.array([o.getf(1, k) for k in ("viscous_drag", "pressure_drag", "viscous_lift", "pressure_lift")])
    got = s.stress(s.handles[0], mu_f, rho_f)
    assert np.all(np.isfinite(ref)) and np.any(ref != 0.0)
    np.testing.assert_allclose(got, ref, rtol=STRESS_RTOL, atol=1e-14 * np.max(np.abs(ref)))


def test_steps_100_single_block_bitwise():
    # the drop-in path must stay within rel L2 1e-8 after 100 steps; it is bitwise
    case = synth.sphere_single_block(n=24, n_steps=100, diameter=0.3)
    o, s = _pair(case)
    for _ in range(100):
        o.step()
    s.run(100)
    compare_fields(o, s, "100 steps")
    compare_iters(o, s, "100 steps")
    compare_search(o, s, "100 steps")


@pytest.mark.parametrize("n", [(24, 16, 16), (23, 17, 13), (5, 4, 3)])
def test_steps_body_free_block(n):
    """A lone block with the domain BCs and no body (tagged all fluid and
    counted): three drop-in steps bitwise against the oracle, on even, odd
    (padded colour rows, ragged tiles) and minimal block sizes."""
    case = synth.replace(synth.uniform_block(n=n, lengths=(3.0, 2.0, 2.0)), n_steps=3, epsi=1e-8)
    o, s = _pair(case)
    for _ in range(3):
        o.step()
    s.run(3)
    compare_fields(o, s, "3 steps, body-free block")
    compare_iters(o, s, "3 steps, body-free block")


@pytest.mark.parametrize("workload", ["sphere_64", "two_block_bench"])
def test_full_size_steps_bitwise(workload):
    """The workloads at their full sizes: the 64^3 sphere block (D = 0.25 at
    (0.4, 0.5, 0.5), Re 100) and the bench's coarse 96x64x64 + fine 64^3
    two-block sphere (D = 0.5, Re 300).  Two drop-in steps bitwise against
    the oracle: fields, SOR iteration counts and Search tags."""
    if workload == "sphere_64":
        case = synth.sphere_single_block(n=64, n_steps=2)
    else:
        case = synth.sphere_two_block(n_steps=2)
    o, s = _pair(case)
    for _ in range(2):
        o.step()
    s.run(2)
    compare_fields(o, s, f"{workload}, 2 steps")
    compare_iters(o, s, f"{workload}, 2 steps")
    compare_search(o, s, f"{workload}, 2 steps")
