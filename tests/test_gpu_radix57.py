"""Axis lengths with factors 5 and 7, and odd column counts (FFTW plans any length,
pfutil/fftWrap.go:16-23).

The runtime Stockham plans take radix-5 and radix-7 stages beside 2, 3, 4, 8 and 16,
so grids such as 100^2, 250^2, 1000^2, 70 x 98 and 20^3 run on the device.  An odd
column count (35 x 49, 15^3) has no Nyquist column: the x pass transforms row pairs as
complex lines of the full odd length instead of packing each row into half a line.
- the device FFT (pfutil.FourierTransform semantics) against numpy: FP64 1e-12, FP32 2e-6;
- Cahn-Hilliard Euler steps against the FP64 oracle: FP64 rel-L2 <= 1e-11, FP32 <= 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CH_EQ = "dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc"


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-6)])
@pytest.mark.parametrize("dims", [[100, 100], [250, 250], [1000, 1000], [70, 98], [49, 10], [20, 20, 20],
                                  [14, 14, 14], [30, 30, 30], [35, 49], [49, 35], [8, 27], [15, 15, 15],
                                  [21, 21, 21]])
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
                                                 ([14, 14, 14], "fp32", 20, 1e-4), ([35, 49], "fp64", 50, 1e-11),
                                                 ([49, 35], "fp32", 30, 1e-4), ([63, 63], "fp64", 40, 1e-11),
                                                 ([15, 15, 15], "fp64", 20, 1e-11), ([21, 21, 21], "fp32", 20, 1e-4)])
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


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_odd_columns_upload_download_and_mass(prec):
    """Real field -> half spectrum -> real field and the FP64 reductions on 35 x 49 (odd rows and
    columns, so the last row pair of a tile holds one row)."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [35, 49]
    c = uniform_field(23, 35 * 49, 0.1, 0.5)
    m = G.Model(dims, prec, device=0)
    m.add_field("c")
    m.upload_real(0, c)
    tol = 1e-14 if prec == "fp64" else 2e-6
    assert np.abs(m.download_real(0) - c).max() <= tol
    assert abs(m.mass(0) - c.sum()) <= tol * 35 * 49
    assert abs(m.reduce(0, G.RED_MIN) - c.min()) <= tol and abs(m.reduce(0, G.RED_MAX) - c.max()) <= tol
    assert abs(m.reduce(0, G.RED_SUMSQ) - (c * c).sum()) <= tol * 35 * 49
    idx = np.array([0, 48, 49, 1000, 35 * 49 - 1])
    assert np.abs(m.point_values(0, idx) - c[idx]).max() <= tol * 10
    m.close()


def test_odd_columns_in_a_batch_equal_single_contexts():
    """Batched stepping of odd-sided instances (45, 63, 75) next to even ones: bitwise the fields of
    each instance stepped alone, FP64."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    def mk(side, i):
        m = G.Model([side, side], "fp64", device=0)
        m.add_field("conc")
        m.add_scalar("gamma", 0.6 + 0.1 * i)
        m.add_scalar("m1", -1.0)
        m.add_equation(CH_EQ)
        m.init()
        m.set_stepper("euler", 0.05)
        m.upload(0, uniform_field(70 + i, side * side, 0.5, 0.05))
        return m

    sides = [45, 63, 64, 75]
    a = [mk(s, i) for i, s in enumerate(sides)]
    b = [mk(s, i) for i, s in enumerate(sides)]
    G.Batch(a).step(25)
    for m in b:
        m.step(25)
    for x, y in zip(a, b):
        assert np.array_equal(x.download_real(0), y.download_real(0))
