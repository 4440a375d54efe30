"""Axis lengths with factors 5 and 7 (FFTW plans any length, pfutil/fftWrap.go:16-23).

The runtime Stockham plans take radix-5 and radix-7 stages beside 2, 3, 4, 8 and 16,
so grids such as 100^2, 250^2, 1000^2, 70 x 98 and 20^3 run on the device:
- the device FFT (pfutil.FourierTransform semantics) against numpy: FP64 1e-12, FP32 2e-6;
- Cahn-Hilliard Euler steps against the FP64 oracle: FP64 rel-L2 <= 1e-11, FP32 <= 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CH_EQ = "dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc"


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-6)])
@pytest.mark.parametrize("dims", [[100, 100], [250, 250], [1000, 1000], [70, 98], [49, 10], [20, 20, 20],
                                  [14, 14, 14], [30, 30, 30]])
def test_fft_radix5_radix7_matches_numpy(dims, prec, tol):
    import gopf_gb300 as G

    rng = np.random.default_rng(7)
    n = int(np.prod(dims))
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    m = G.Model(dims, prec, device=0)
    shape = tuple(dims) if len(dims) == 2 else (dims[2], dims[0], dims[1])
    ref = np.fft.fftn(x.reshape(shape)).ravel()
    y = m.fft(x, -1)
    assert np.abs(y - ref).max() <= tol * np.abs(ref).max()
    back = m.fft(y, +1) / n
    assert np.abs(back - x).max() <= tol * 10 * np.abs(x).max()
    m.close()


@pytest.mark.parametrize("dims,prec,steps,tol", [([100, 100], "fp64", 50, 1e-11), ([250, 250], "fp32", 30, 1e-4),
                                                 ([70, 98], "fp64", 40, 1e-11), ([20, 20, 20], "fp64", 20, 1e-11),
                                                 ([14, 14, 14], "fp32", 20, 1e-4)])
def test_cahn_hilliard_radix5_radix7_matches_oracle(oracle, dims, prec, steps, tol):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c0 = uniform_field(17, n, 0.5 if len(dims) == 2 else 0.0, 0.05 if len(dims) == 2 else 0.1)
    g = G.Model(dims, prec, device=0)
    g.add_field("conc")
    g.add_scalar("gamma", 1.0)
    g.add_scalar("m1", -1.0)
    g.add_equation(CH_EQ)
    g.init()
    g.set_stepper("euler", 0.1)
    g.upload(0, c0)
    g.step(steps)
    o = oracle.cahn_hilliard(dims, gamma=1.0)
    o.set_field(0, c0)
    o.step_euler(0.1, steps)
    ref = o.field(0).real
    err = np.linalg.norm(g.download_real(0) - ref) / np.linalg.norm(ref)
    assert err <= tol, err
    g.close()


def test_unsupported_prime_factor_is_rejected():
    """A length with a prime factor above 7 (here 11) has no device plan and is refused, never run on
    the CPU."""
    import gopf_gb300 as G

    with pytest.raises(G.GopfError) as e:
        G.Model([22, 22], "fp64", device=0)
    assert e.value.status == 6
