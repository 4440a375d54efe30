"""CPU checks of the FP64 oracle against the reference's own known-answer tests.

Each test restates the specification (equation, sizes, steps, tolerance,
analytic solution) of one test in the reference and runs it on the oracle.
These pins are what make the oracle trustworthy as the GPU's checker.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O


# ---------------------------------------------------------------- FFT / Freq

@pytest.mark.parametrize("dims", [[8, 8], [8, 16], [9, 9], [12, 6], [128, 128], [384, 96], [8, 8, 8], [9, 9, 9],
                                  [6, 10, 14]])
def test_fft_matches_numpy(dims):
    """FFT sign/normalisation convention of pfutil/fftWrap.go:26-39 (pocketfft as the FFTW stand-in)."""
    rng = np.random.default_rng(1)
    n = int(np.prod(dims))
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    sh = O.mem_shape(dims)
    y = O.fftn(x, dims, -1)
    ref = np.fft.fftn(x.reshape(sh)).ravel()
    assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()
    back = O.fftn(y, dims, +1) / n
    assert np.abs(back - x).max() < 1e-12


def test_fft_real_input_data_i():
    """TestFFTWWrapConsistency (pfutil/fftwWrap_test.go:11-57): data[i] = i on 8x16, forward then backward."""
    nx, ny = 8, 16
    data = np.arange(nx * ny, dtype=np.complex128)
    y = O.fftn(data, [nx, ny], -1)
    assert np.allclose(y, np.fft.fft2(data.reshape(nx, ny)).ravel(), atol=1e-6)
    z = O.fftn(y, [nx, ny], +1)
    assert np.allclose(z, np.fft.ifft2(y.reshape(nx, ny)).ravel() * nx * ny, atol=1e-6)


def test_freq_convention():
    """Freq (pfutil/fftWrap.go:57-74): res[0]=row/n0, res[1]=col/n1, res[2]=depth/n2, folded to (-0.5, 0.5]."""
    dims = [4, 6, 8]
    for i in range(int(np.prod(dims))):
        col = i % 6
        row = (i // 6) % 4
        depth = i // 24
        exp = [row / 4, col / 6, depth / 8]
        exp = [e - 1 if e > 0.5 else e for e in exp]
        assert np.allclose(O.freq(dims, i), exp)
    # Nyquist stays +0.5
    assert O.freq([8, 8], 4 * 8 + 4)[0] == 0.5


@pytest.mark.parametrize("dims", [[8, 8], [9, 9], [8, 8, 8], [9, 9, 9]])
def test_conjugate_node(dims):
    """TestConjugateNode (pfutil/fftwWrap_test.go:59-90)."""
    for j in range(int(np.prod(dims))):
        f1 = O.freq(dims, j)
        f2 = O.freq(dims, O.conjugate_node(dims, j))
        for a, b in zip(f1, f2):
            assert abs(a + b) <= 1e-10 or abs(a) >= 0.5 - 1e-10


# ---------------------------------------------------------------- steppers

def _single(dims, init):
    m = O.Model(dims, 1)
    m.set_field(0, np.full(int(np.prod(dims)), init, dtype=np.complex128))
    return m


def test_exponential_decay():
    """TestExponentialDecay (pf/euler_test.go:10-49): dfield/dt = rate*field, 8x8, dt 1e-3, 1000 steps."""
    m = _single([8, 8], 1.0)
    m.add_term(0, -1.0, implicit=True)  # rate*field is bilinear -> Denum
    m.step_euler(1e-3, 1000, hooks=False)
    f = m.field(0)
    assert np.all(np.abs(f.real - math.exp(-1.0)) < 1e-3)
    assert np.all(np.abs(f.imag) < 1e-3)
    assert m.current_step == 1000


def test_euler_square_decay():
    """TestEulerSquareDecary (pf/euler_test.go:51-85): dfield/dt = rate*field^2 -> 1/(1+t)."""
    m = _single([8, 8], 1.0)
    d = m.add_product([0], [2])
    m.add_term(0, -1.0, src_kind=O.SRC_DERIVED, src=d)
    m.step_euler(1e-3, 1000, hooks=False)
    assert np.all(np.abs(m.field(0).real - 1.0 / 2.0) < 1e-3)


def test_rk4_simple_model():
    """TestSimpleModel (pf/rk4_test.go:14-54): RK4, dt 0.1, 10 steps, tolerance 1e-6."""
    m = _single([8, 8], 1.0)
    d = m.add_product([0], [2])
    m.add_term(0, -1.0, src_kind=O.SRC_DERIVED, src=d)
    m.step_rk4(0.1, 10, hooks=False)
    assert np.all(np.abs(m.field(0).real - 1.0 / 2.0) < 1e-6)


def test_rk4_with_implicit():
    """TestWithImplicit (pf/rk4_test.go:61-99): dfield/dt = field + rate*field^2, logistic, tolerance 1e-3."""
    c0 = 0.5
    m = _single([8, 8], c0)
    d = m.add_product([0], [2])
    m.add_term(0, 1.0, implicit=True)
    m.add_term(0, -1.0, src_kind=O.SRC_DERIVED, src=d)
    m.step_rk4(0.01, 100, hooks=False)
    A = 1.0 / c0 - 1.0
    exp = math.exp(1.0) / (A + math.exp(1.0))
    assert np.all(np.abs(m.field(0).real - exp) < 1e-3)


def test_solver_diffusion_mass():
    """TestSolverDiffusion (pf/solver_test.go:9-34): 16x16, delta at node 128, LAP conc, dt 0.1, 10x10 steps."""
    m = O.Model([16, 16], 1)
    f = np.zeros(256, dtype=np.complex128)
    f[128] = 1.0
    m.set_field(0, f)
    m.add_term(0, 1.0, lap=1, implicit=True)
    m.step_euler(0.1, 100)
    c = m.field(0).real
    assert abs(c.sum() - 1.0) < 1e-4
    assert np.all(c < 1.0) and np.all(c >= 0.0)


def test_laplacian_symbol():
    """TestLaplacianN (pf/diffOp_test.go:10-57): (-(2 pi f)^2)^p for p = 1, 2 at f = i."""
    # The oracle's symbol is exercised through an implicit term evaluated with a constant field.
    m = O.Model([4, 4], 1)
    m.add_term(0, 1.0, lap=1, implicit=True)
    den = m.eval_denum(0)
    for i in range(16):
        f = O.freq([4, 4], i)
        assert abs(den[i] - (-(2 * math.pi) ** 2 * (f @ f))) < 1e-10
    m2 = O.Model([4, 4], 1)
    m2.add_term(0, 1.0, lap=2, implicit=True)
    den2 = m2.eval_denum(0)
    for i in range(16):
        f = O.freq([4, 4], i)
        assert abs(den2[i] - ((2 * math.pi) ** 4 * (f @ f) ** 2)) < 1e-8


def test_homogeneous_rhs_with_mocked_displacement():
    """TestHomogeneousRHS (pf/homoLinElast_test.go:27-88): isotropic(60, 0.3), misfit eps_xx = 0.01,
    u_x = FFT((x(1-x))^2) injected, field = 0.5 -> RHS = C11 eps (e_xx - eps H) H' to 1e-4."""
    N = 16
    bulk, nu = 60.0, 0.3
    shear = 3.0 * bulk * (1.0 - 2.0 * nu) / (2.0 * (1.0 + nu))
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    v = 0.0
                    if i == j and k == l:
                        v += bulk - 2.0 * shear / 3.0
                    if i == k and j == l:
                        v += shear
                    if i == l and j == k:
                        v += shear
                    C[i, j, k, l] = v
    eps = 0.01
    misfit = np.zeros((3, 3))
    misfit[0, 0] = eps
    idx = np.arange(N * N)
    x = (idx // N) / N
    ux = (x * (1 - x)) ** 2 + 0j
    exx = 2 * x * (1 - x) * (1 - 2 * x) / N
    ux_hat = O.fftn(ux, [N, N], -1)
    m = O.Model([N, N], 1)
    e = m.add_elastic(0, 0, C, misfit)
    disp = np.zeros((N * N, 3), dtype=np.complex128)
    disp[:, 0] = ux_hat
    m.elastic_disp_override(e, disp)
    m.elastic_hfield(e)[:] = 0.5
    m.set_field(0, np.full(N * N, 0.5))
    rhs = m.eval_rhs(0)
    res = O.fftn(rhs, [N, N], +1) / (N * N)
    H = 3 * 0.25 - 2 * 0.125
    dH = 6 * 0.5 - 6 * 0.25
    expect = C[0, 0, 0, 0] * eps * (exx - eps * H) * dH
    assert np.abs(res.real - expect).max() < 1e-4
    assert np.abs(res.imag).max() < 1e-4


def test_vol_conserve_update_rule():
    """TestVolConserve (pf/volumeConserving_test.go:15-64): the Lagrange multiplier keeps the volume.

    The reference test drives VolumeConservingLP by hand with a zero Freq; the oracle
    restates the multiplier update, so the same loop is run here on a model whose
    step is exactly myfield += dt*(rate + lambda*indicator)."""
    N = 16
    dt, rate = 0.01, 0.01
    ind = np.zeros(N * N)
    ind[N * N // 2 + 1:] = 1.0
    field = np.ones(N * N)
    lam, cur, first = 0.0, 0.0, True
    for _ in range(100):
        field = field + dt * (rate + lam * ind)
        integ = field.sum()
        ind_int = ind.sum()  # real(FFT(indicator)[0])
        if first:
            cur, first = integ, False
        else:
            lam = lam - (integ - cur) / (dt * ind_int)
            cur = integ
    expect_change = 2.0 * dt * N * N * rate
    assert abs(field.sum() - expect_change - 256.0) < 1e-10


def test_vol_conserve_oracle_matches_rule():
    """The oracle's VolumeConservingLP (pf/volumeConserving.go:31-50) against the rule above,
    on an Allen-Cahn-like equation dphi/dt = -phi + VOLCONS (explicit) with indicator 1."""
    N = 8
    dt = 0.01
    m = O.Model([N, N], 1)
    phi = np.linspace(0.1, 0.9, N * N)
    m.set_field(0, phi)
    ind = m.add_poly(0, [1.0], [0])  # indicator == 1 everywhere
    m.add_term(0, -1.0, implicit=True)
    v = m.add_volcons(0, 0, ind, dt)
    m.step_euler(dt, 50)
    # the multiplier drives the volume back towards the value after the first step
    vol0 = None
    m2 = O.Model([N, N], 1)
    m2.set_field(0, phi)
    ind2 = m2.add_poly(0, [1.0], [0])
    m2.add_term(0, -1.0, implicit=True)
    m2.add_volcons(0, 0, ind2, dt)
    m2.step_euler(dt, 1)
    vol0 = m2.field(0).real.sum()
    assert abs(m.field(0).real.sum() - vol0) < 0.05 * abs(vol0)
    assert m.volcons_multiplier(v) != 0.0


def test_strain_from_displacement():
    """TestStrain (elasticity/linearElasticity_test.go:51-104) through the oracle's elastic term:
    e_xx of u_x = (x(1-x))^2 on 8x8 equals d u_x/dx / N to 1e-3."""
    N = 8
    idx = np.arange(N * N)
    x = (idx // N) / N
    ux = (x * (1 - x)) ** 2 + 0j
    expect = (2 * x * (1 - x) ** 2 - 2 * x * x * (1 - x)) / N
    uh = O.fftn(ux, [N, N], -1)
    # strain e_00 = i pi (f0 u0 + f0 u0) with Nyquist zeroed
    e = np.zeros(N * N, dtype=np.complex128)
    for i in range(N * N):
        f = O.freq([N, N], i)
        f0 = 0.0 if abs(abs(f[0]) - 0.5) < 1e-10 else f[0]
        e[i] = 2j * math.pi * f0 * uh[i]
    res = O.fftn(e, [N, N], +1) / (N * N)
    assert np.abs(res.real - expect).max() < 1e-3
    assert np.abs(res.imag).max() < 1e-3


def _ellipsoid(N, a, b, c):
    i, j, k = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    v = ((i - N // 2) / a) ** 2 + ((j - N // 2) / b) ** 2 + ((k - N // 2) / c) ** 2
    return (v <= 1.0).astype(np.complex128).ravel()


@pytest.mark.slow
@pytest.mark.parametrize("abc", [(10.0, 10.0, 10.0), (15.0, 7.0, 15.0), (7.0, 7.0, 15.0)])
def test_dilatational_misfit_eshelby(abc):
    """TestDilatationalMisfits (elasticity/linearElasticity_test.go:11-49): 64^3 ellipsoids,
    energy density within 5% of Eshelby's 2(1+nu) mu eps^2/(1-nu)."""
    N = 64
    nu, bulk = 0.3, 50.0
    shear = 3.0 * bulk * (1.0 - 2.0 * nu) / (2.0 * (1.0 + nu))
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    v = 0.0
                    if i == j and k == l:
                        v += bulk - 2.0 * shear / 3.0
                    if i == k and j == l:
                        v += shear
                    if i == l and j == k:
                        v += shear
                    C[i, j, k, l] = v
    eps = 0.05
    misfit = np.eye(3) * eps
    vox = _ellipsoid(N, *abc)
    energy = O.homogeneous_modulus_energy(vox, [N, N, N], misfit, C)
    expect = 2.0 * (1.0 + nu) * shear * eps * eps / (1.0 - nu)
    assert abs(energy - expect) <= 0.05 * expect


# ---------------------------------------------------------------- generator

def test_seeded_generator_matches_python():
    from gopf_gb300.synthetic import uniform_field

    a = uniform_field(3, 5000, 0.3, 0.02)
    b = O.uniform_field(3, 5000, 0.3, 0.02)
    assert np.array_equal(a, b)
    assert a.min() >= 0.28 and a.max() < 0.32


# ---------------------------------------------------------------- elastic symbol

def _cubic(c11, c12, c44):
    """elasticity.CubicMaterial (elasticity/rank4.go:113-128)."""
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        C[i, i, i, i] = c11
    for i in range(3):
        for j in range(i + 1, 3):
            C[i, i, j, j] = c12
            C[j, j, i, i] = c12
            C[i, j, i, j] = c44
            C[j, i, j, i] = c44
    return C


def _bsym(dims, C, mis):
    """The device's elastic symbol: b(k) = sum_{i<D} (A f~)_i (Gamma(f)^-1 A f)_i, symmetrised over k, -k."""
    D = len(dims)
    N = int(np.prod(dims))
    A = np.einsum("ijkl,kl->ij", C, mis)

    def bval(f):
        if np.all(np.abs(f) < 1e-10):
            return 0.0
        ft = f.copy()
        ft[np.abs(np.abs(ft) - 0.5) < 1e-10] = 0.0
        G = np.einsum("mjnl,j,l->mn", C, f, f)
        return float(np.dot((A @ ft)[:D], np.linalg.solve(G, A @ f)[:D]))

    b = np.zeros(N)
    for i in range(N):
        f = np.zeros(3)
        f[:D] = O.freq(dims, i)
        fm = np.zeros(3)
        fm[:D] = O.freq(dims, O.conjugate_node(dims, i))
        b[i] = 0.5 * (bval(f) + bval(fm))
    return b


@pytest.mark.parametrize("dims", [[16, 16], [8, 8, 8], [12, 12, 12]])
def test_elastic_symbol_is_hermitian_part_of_reference_term(dims):
    """The Khachaturyan term of pf/homoLinElast.go:47-99 (14 FFTs + per-k 3x3 solves in 3D) equals,
    in its Hermitian part, FFT[H'(h) (IFFT(b Hhat)/N - 2 e0 H(h))] with the symmetrised symbol b.
    The reference's anti-Hermitian remainder comes from f = +0.5 at both k and -k on Nyquist planes."""
    rng = np.random.default_rng(0)
    N = int(np.prod(dims))
    h = 0.3 + 0.2 * rng.random(N)
    C = _cubic(1.0, 0.6, 0.5)
    mis = np.eye(3) * 0.01
    mis[0, 1] = mis[1, 0] = 0.003
    m = O.Model(dims, 1)
    e = m.add_elastic(0, 0, C, mis)
    m.elastic_hfield(e)[:] = h
    m.set_field(0, h)
    ref = m.eval_rhs(0)
    conj = np.array([O.conjugate_node(dims, i) for i in range(N)])
    herm = 0.5 * (ref + np.conj(ref[conj]))
    A = np.einsum("ijkl,kl->ij", C, mis)
    e0 = 0.5 * np.einsum("ijkl,ij,kl->", C, mis, mis)
    H = 3 * h * h - 2 * h ** 3
    Hd = 6 * h - 6 * h * h
    w = (O.fftn(_bsym(dims, C, mis) * O.fftn(H.astype(complex), dims, -1), dims, +1) / N).real
    mine = O.fftn((Hd * (w - 2 * e0 * H)).astype(complex), dims, -1)
    assert np.abs(herm - mine).max() <= 1e-12 * np.abs(ref).max()
    del A


def test_oracle_polynomial_of_several_fields(oracle):
    """A derived field sum_t coef_t prod_f field_f^p_tf (a RegisterFunction closure that is a
    polynomial of two fields, examples/strain_single_precipitate/main.go:36-50) against numpy."""
    rng = np.random.default_rng(3)
    a, b = rng.random(64), rng.random(64)
    m = oracle.Model([8, 8], 2)
    m.set_field(0, a)
    m.set_field(1, b)
    d = m.add_mpoly([2.0, -1.5, 0.5], [[1, 2], [0, 3], [2, 0]])
    m.add_term(0, 1.0, src_kind=oracle.SRC_DERIVED, src=d)
    expect = np.fft.fft2((2.0 * a * b ** 2 - 1.5 * b ** 3 + 0.5 * a ** 2).reshape(8, 8)).ravel()
    assert np.max(np.abs(m.eval_rhs(0) - expect)) < 1e-12
