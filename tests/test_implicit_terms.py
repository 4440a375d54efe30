"""Implicit user terms with a per-frequency symbol: TensorialHessian (pf/tensorialHessian.go) and
SpectralViscosity (pf/spectralViscosity.go).

CPU: the oracle against the reference's unit tests (TestTensorialHessian's analytic derivatives,
TestInterpolation, TestSpectralViscosityTerm's symbol) and the term split of the equation parser
(TestHessianWithModel: one implicit, no explicit term).  GPU: trajectories against the FP64 oracle.
"""
import math

import numpy as np
import pytest


def hessian_data(N):
    i = np.arange(N * N)
    y = (i % N) / N
    x = (i // N) / N
    px = 16.0 * (x * x - 2 * x ** 3 + x ** 4)
    py = 16.0 * (y * y - 2 * y ** 3 + y ** 4)
    d = {"data": px * py}
    d["dx2"] = 16.0 * (2.0 - 12.0 * x + 12 * x * x) * py / (N * N)
    d["dy2"] = px * 16.0 * (2.0 - 12.0 * y + 12.0 * y * y) / (N * N)
    d["dxdy"] = 16.0 * (2 * x - 6 * x * x + 4 * x ** 3) * 16.0 * (2 * y - 6 * y * y + 4 * y ** 3) / (N * N)
    return d


@pytest.mark.parametrize("K,res,tol", [([1, 0, 0, 0], "dx2", 1e-3), ([0, 0, 0, 1], "dy2", 1e-3),
                                       ([0, 0.5, 0.5, 0], "dxdy", 1e-6)])
def test_oracle_tensorial_hessian(oracle, K, res, tol):
    """TestTensorialHessian (pf/tensorialHessian_test.go:42-104)."""
    N = 64
    d = hessian_data(N)
    m = oracle.Model([N, N], 1)
    m.add_hessian(0, K)
    sym = m.eval_denum(0)
    out = oracle.fftn(oracle.fftn(d["data"].astype(complex), [N, N]) * sym, [N, N], sign=1) / (N * N)
    assert np.max(np.abs(out.real - d[res])) < tol and np.max(np.abs(out.imag)) < tol


def test_oracle_spectral_viscosity(oracle):
    """TestInterpolation and TestSpectralViscosityTerm (pf/spectralViscosity_test.go)."""
    for k, e in [(0.19, 0.0), (0.66, 1.0), (0.4, 1.0 / 8.0)]:
        assert abs(oracle.sv_interpolant(k, 0.6) - e) < 1e-10
    N = 16
    m = oracle.Model([N, N], 1)
    m.add_viscosity(0, 1.0, 0.25, 2)
    sym = m.eval_denum(0)
    for i in range(N * N):
        f = oracle.freq([N, N], i)
        f2 = float(np.dot(f, f))
        expect = -1.0 * oracle.sv_interpolant(math.sqrt(f2), 0.25) * f2
        assert abs(sym[i].real - expect) < 1e-10 and abs(sym[i].imag) < 1e-10


def test_parser_treats_symbol_terms_as_implicit():
    """TestHessianWithModel / TestSpectralViscosityTerm: the terms join the denominator only."""
    import gopf_gb300 as G

    m = G.Model([16, 16], "fp64", device=-1)
    m.add_field("conc")
    m.register_hessian("HESSIAN", [1.0, 2.0, 2.0, 2.0])
    m.add_equation("dconc/dt = HESSIAN")
    m.init()
    assert m.summary(0) == (0, 1)
    v = G.Model([16, 16], "fp64", device=-1)
    v.add_field("conc")
    v.register_spectral_viscosity("SPECTRAL_VISC", 1.0, 0.25, 2)
    v.add_equation("dconc/dt = SPECTRAL_VISC")
    v.init()
    assert v.summary(0) == (0, 1)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("dims,K", [([32, 32], [1.0, 0.3, 0.3, 0.5]),
                                    ([16, 16, 16], [1.0, 0.2, 0.0, 0.2, 0.7, 0.1, 0.0, 0.1, 0.4])])
def test_anisotropic_cahn_hilliard_fp64(oracle, dims, K):
    """CH with the gradient energy replaced by an anisotropic Hessian (FP64, 40 steps).  On Nyquist
    lines the reference's symbol differs between k and -k (Freq keeps +1/2 for both), so its complex
    field grows an anti-Hermitian part; the device's real field follows the reference's step
    followed by taking the real part, which is what the oracle does here after every step."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c0 = uniform_field(6, n, 0.5, 0.05)
    g = G.Model(dims, "fp64", device=0)
    g.add_field("conc")
    g.add_scalar("m1", -1.0)
    g.register_hessian("HESS", K)
    g.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc - LAP HESS")
    g.init()
    assert g.summary(0) == (1, 2)
    g.set_stepper("euler", 0.05)
    g.upload(0, c0)
    g.step(40)
    o = oracle.Model(dims, 1)
    o.set_field(0, c0)
    d = o.add_product([0], [3])
    o.add_term(0, 1.0, lap=1, src_kind=oracle.SRC_DERIVED, src=d)
    o.add_term(0, -1.0, lap=1, implicit=True)
    o.add_hessian(0, K, coef=-1.0, lap=1)
    for _ in range(40):
        o.step_euler(0.05, 1)
        o.set_field(0, o.field(0).real.copy())
    assert rel_l2(g.download_real(0), o.field(0).real) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("stepper", ["euler", "rk4"])
def test_spectral_viscosity_fp64(oracle, stepper):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [64, 64]
    c0 = uniform_field(8, 64 * 64, 0.5, 0.05)
    g = G.Model(dims, "fp64", device=0)
    g.add_field("conc")
    g.add_scalar("gamma", 1.0)
    g.add_scalar("m1", -1.0)
    g.register_spectral_viscosity("SV", 0.5, 0.3, 2)
    g.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc + SV")
    g.init()
    g.set_stepper(stepper, 0.1)
    g.upload(0, c0)
    g.step(30)
    o = oracle.cahn_hilliard(dims, gamma=1.0)
    o.set_field(0, c0)
    o.add_viscosity(0, 0.5, 0.3, 2)
    if stepper == "euler":
        o.step_euler(0.1, 30)
    else:
        o.step_rk4(0.1, 30)
    assert rel_l2(g.download_real(0), o.field(0).real) <= 1e-11
