"""The mixed path's default relaxation factor, host mirror (synth.mixed_omega,
the expression the library evaluates for its FP32 sweeps): the SOR optimum
2 / (1 + sqrt(1 - rho^2)) with rho the mean of cos(pi/n) over the axes, at
most 1.99.  It is computed from sin^2(pi/2n) terms, so 1 - rho^2 carries no
cancellation; against a 50-digit evaluation it is within one ulp on the
workloads' block sizes."""
import pytest

from biocfd import synth

SIZES = [(8, 8, 8), (24, 16, 16), (96, 64, 64), (128, 96, 96), (256, 192, 192), (384, 256, 256)]


@pytest.mark.parametrize("dims", SIZES)
def test_mixed_omega_within_an_ulp_of_the_exact_optimum(dims):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    rho = sum(mpmath.cos(mpmath.pi / n) for n in dims) / 3
    exact = min(mpmath.mpf("1.99"), 2 / (1 + mpmath.sqrt(1 - rho ** 2)))
    got = synth.mixed_omega(*dims)
    assert 1.0 < got <= 1.99
    assert abs(mpmath.mpf(got) - exact) <= 2.3e-16 * exact, (dims, got, float(exact))


def test_mixed_omega_cap_and_copy():
    assert synth.mixed_omega(1024, 768, 512) == 1.99
    case = synth.small_two_block(n_steps=1)
    c2 = synth.with_mixed_omega(case)
    for b, b2 in zip(case.blocks, c2.blocks):
        assert b2.omega == synth.mixed_omega(b.nx, b.ny, b.nz) and b2.nx == b.nx
