"""Noise terms (pf/noise.go) on the device, checked statistically as the reference's tests do.

The device draws the Fourier transform of real white noise N(0, 2S) directly in
k space (Philox-4x32-10 + Box-Muller), so the realisations differ from Go's
math/rand; the distribution must not.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _white(dims, prec, strength, dt, seed=7):
    import gopf_gb300 as G

    m = G.Model(dims, prec, device=0)
    m.add_field("price")
    m.register_noise("WHITE_NOISE", "white", "price", strength, seed)
    m.add_equation("dprice/dt = WHITE_NOISE")
    m.init()
    m.set_stepper("euler", dt)
    m.upload(0, np.zeros(int(np.prod(dims))))
    return m


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_white_noise_variance(prec):
    """TestVariance (pf/noise_test.go:23-48): std of N(0, 2S) with S = 2 is 2; one step with dt = 1 from zero."""
    dims = [1024, 1024]
    m = _white(dims, prec, 2.0, 1.0)
    m.step(1)
    x = m.download_real(0)
    n = x.size
    assert abs(x.mean()) < 4 * 2.0 / math.sqrt(n)
    assert abs(x.std(ddof=1) - 2.0) < 4 * 2.0 / math.sqrt(2 * n)
    # Gaussian shape: fraction beyond one standard deviation ~ 0.3173
    frac = np.mean(np.abs(x) > 2.0)
    assert abs(frac - 0.3173) < 0.003
    # a second step draws new noise: increments are uncorrelated with the first draw
    m.step(1)
    y = m.download_real(0) - x
    assert abs(np.corrcoef(x, y)[0, 1]) < 0.01
    assert abs(y.std(ddof=1) - 2.0) < 4 * 2.0 / math.sqrt(2 * n)


def test_white_noise_3d_and_seed():
    a = _white([32, 32, 32], "fp64", 0.5, 1.0, seed=1)
    b = _white([32, 32, 32], "fp64", 0.5, 1.0, seed=1)
    c = _white([32, 32, 32], "fp64", 0.5, 1.0, seed=2)
    for m in (a, b, c):
        m.step(1)
    xa, xb, xc = a.download_real(0), b.download_real(0), c.download_real(0)
    assert np.array_equal(xa, xb)
    assert not np.array_equal(xa, xc)
    assert abs(xa.std(ddof=1) - 1.0) < 0.03


def test_conservative_noise():
    """TestConservativeNoise (pf/noise_test.go:50-94): 16x16, S = 1, dt = 0.1, 10 x 100 steps:
    the field stays real, its integral stays zero, and it is not trivially small."""
    import gopf_gb300 as G

    m = G.Model([16, 16], "fp64", device=0)
    m.add_field("myfield")
    m.register_noise("CONSERVATIVE_NOISE", "conservative", "myfield", 1.0, 3)
    m.add_equation("dmyfield/dt = CONSERVATIVE_NOISE")
    m.init()
    assert m.summary(0) == (1, 0)
    m.set_stepper("euler", 0.1)
    m.upload(0, np.zeros(256))
    for _ in range(10):
        m.step(100)
    d = m.download(0)
    assert np.all(d.imag == 0.0)
    assert abs(d.real.sum()) < 1e-10
    assert np.count_nonzero(np.abs(d.real) > math.sqrt(2.0)) > 0


def test_noise_with_cahn_hilliard_stays_finite():
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    m = G.Model([64, 64, 64], "fp32", device=0)
    m.add_field("conc")
    m.add_scalar("gamma", 0.5)
    m.add_scalar("m1", -1.0)
    m.register_noise("NOISE", "conservative", "conc", 1e-4, 5)
    m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc + NOISE")
    m.init()
    m.set_stepper("euler", 0.05)
    c0 = uniform_field(1, 64 ** 3, 0.0, 0.1)
    m.upload(0, c0)
    m.step(100)
    d = m.download_real(0)
    assert np.all(np.isfinite(d))
    assert abs(d.sum() - c0.sum()) / d.size < 1e-6


@pytest.mark.parametrize("kind", ["white", "conservative"])
def test_noise_in_a_model_of_two_fields(kind):
    """A noise term in the second equation of a two-field model draws exactly what the same term
    draws in a model of its own (the draws are keyed by seed, step and mode); the other field
    steps as without noise."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims, dt, n = [64, 64], 0.1, 64 * 64
    a0 = uniform_field(3, n, 0.2, 0.1)
    two = G.Model(dims, "fp64", device=0)
    two.add_field("a")
    two.add_field("b")
    two.add_scalar("m1", -1.0)
    two.register_noise("NOISE", kind, "b", 0.5, 11)
    two.add_equation("da/dt = m1*a")
    two.add_equation("db/dt = NOISE")
    two.init()
    two.set_stepper("euler", dt)
    two.upload(0, a0)
    two.upload(1, np.zeros(n))
    one = G.Model(dims, "fp64", device=0)
    one.add_field("b")
    one.register_noise("NOISE", kind, "b", 0.5, 11)
    one.add_equation("db/dt = NOISE")
    one.init()
    one.set_stepper("euler", dt)
    one.upload(0, np.zeros(n))
    for m in (two, one):
        m.step(7)
    assert np.array_equal(two.download(1), one.download(0))
    assert np.std(one.download_real(0)) > 0.0
    np.testing.assert_allclose(two.download_real(0), a0 / (1.0 + dt) ** 7, rtol=1e-12, atol=1e-14)
