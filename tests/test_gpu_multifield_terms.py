"""The elastic and volume-conserving terms in models of several fields, and pointwise polynomials of
several fields, on the device against the oracle.

The model is examples/strain_single_precipitate/main.go: fields conc and phase; the chemical
potentials CHEMICALPOT and DERIV_PHASE_ORDER, Go closures of both fields (main.go:36-50), expanded
into their monomials; HomogeneousModulusLinElast on phase with CubicMaterial(110, 60, 30) and the
misfit diag(0.05, -0.01, 0) (main.go:92-95); VolumeConservingLP on phase with the indicator
SMEARING_DERIV = 6x - 6x^2 (main.go:51-54, 89-90); kappa = 0.1, dt = 0.1, the square precipitate
of main.go:64-72.  Euler updates conc first and phase second, in place (pf/euler.go:26-44); the
elastic term reads phase as it was after the previous step (OnStepFinished, pf/homoLinElast.go:130-134),
so it is zero on the first step.
Tolerances: FP64 rel-L2 <= 1e-11 per field (1e-10 for the 3D case without the elastic term, whose
rounding sensitivity is measured in its docstring) and 1e-9 on the multiplier, FP32 rel-L2 <= 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cubic(c11, c12, c44):
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


MISFIT = np.diag([0.05, -0.01, 0.0])


def chem_pot(A, B, M):
    """-M (A c (1 - H(x)) - B (1 - c) H(x)), H = 3x^2 - 2x^3, as monomials c^i x^j."""
    return ([-M * A, -3 * M * (B - A), 2 * M * (B - A), 3 * M * B, -2 * M * B],
            [[1, 0], [1, 2], [1, 3], [0, 2], [0, 3]])


def deriv_phase(A, B, W):
    """-(-A/2 c^2 H'(x) + B/2 (1 - c)^2 H'(x) + W L'(x)), H' = 6x - 6x^2, L' = 2x - 6x^2 + 4x^3."""
    return ([-3 * B - 2 * W, 3 * B + 6 * W, -4 * W, 6 * B, -6 * B, 3 * (A - B), -3 * (A - B)],
            [[0, 1], [0, 2], [0, 3], [1, 1], [1, 2], [2, 1], [2, 2]])


def square(dims):
    """main.go:64-72: conc = phase = 1 inside the central square (3/8, 5/8) of every axis."""
    M = dims[0]
    idx = np.indices(dims).reshape(len(dims), -1)
    inside = np.all((idx > 3 * M // 8) & (idx < 5 * M // 8), axis=0)
    return inside.astype(np.float64)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def precip_gpu(dims, prec, A=0.1, B=0.1, W=0.1, M=1.0, dt=0.1, elastic=True, volcons=True, init=None):
    import gopf_gb300 as G

    m = G.Model(dims, prec, device=0)
    m.add_scalar("kappa", 0.1)
    m.add_field("conc")
    m.add_field("phase")
    m.register_polynomial("CHEMICALPOT", *chem_pot(A, B, M))
    m.register_polynomial("DERIV_PHASE_ORDER", *deriv_phase(A, B, W))
    m.register_function("SMEARING_DERIV", G.DER_INDICATOR_D, "phase")
    eq = "dphase/dt = DERIV_PHASE_ORDER + kappa*LAP phase"
    if volcons:
        m.register_volcons("CONSERVE_PREC_VOL", "phase", "SMEARING_DERIV", dt)
        eq += " + CONSERVE_PREC_VOL"
    if elastic:
        m.register_elastic("LIN_ELAST", "phase", cubic(110.0, 60.0, 30.0), MISFIT)
        eq = eq.replace("DERIV_PHASE_ORDER +", "DERIV_PHASE_ORDER + LIN_ELAST +")
    m.add_equation("dconc/dt = CHEMICALPOT + kappa*LAP conc")
    m.add_equation(eq)
    m.init()
    m.set_stepper("euler", dt)
    c0, x0 = init if init is not None else (square(dims), square(dims))
    m.upload(0, c0)
    m.upload(1, x0)
    return m


def precip_oracle(O, dims, A=0.1, B=0.1, W=0.1, M=1.0, dt=0.1, elastic=True, volcons=True, init=None):
    o = O.Model(dims, 2)
    c0, x0 = init if init is not None else (square(dims), square(dims))
    o.set_field(0, c0)
    o.set_field(1, x0)
    cp = o.add_mpoly(*chem_pot(A, B, M))
    dp = o.add_mpoly(*deriv_phase(A, B, W))
    sm = o.add_indicator(1, O.DER_INDICATOR_D)
    o.add_term(0, 1.0, src_kind=O.SRC_DERIVED, src=cp)
    o.add_term(0, 0.1, lap=1, implicit=True)
    o.add_term(1, 1.0, src_kind=O.SRC_DERIVED, src=dp)
    if elastic:
        o.add_elastic(1, 1, cubic(110.0, 60.0, 30.0), MISFIT)
    o.add_term(1, 0.1, lap=1, implicit=True)
    v = o.add_volcons(1, 1, sm, dt) if volcons else None
    return o, v


@pytest.mark.parametrize("steps", [1, 2, 30])
def test_strain_single_precipitate_fp64(oracle, steps):
    dims = [64, 64]
    g = precip_gpu(dims, "fp64")
    g.step(steps)
    o, v = precip_oracle(oracle, dims)
    o.step_euler(0.1, steps)
    for f in range(2):
        assert rel(g.download(f).real, o.field(f).real) <= 1e-11, f
    assert abs(g.volcons_multiplier() - o.volcons_multiplier(v)) <= 1e-9 * max(1.0, abs(o.volcons_multiplier(v)))


def test_uneven_chemistry_fp64(oracle):
    """A != B makes every monomial of both chemical potentials non-zero; a perturbed start breaks
    the square's symmetry."""
    from gopf_gb300.synthetic import uniform_field

    dims = [32, 32]
    n = 32 * 32
    init = (square(dims) + uniform_field(11, n, 0.0, 0.05), square(dims) + uniform_field(12, n, 0.0, 0.05))
    g = precip_gpu(dims, "fp64", A=0.1, B=0.3, W=0.2, M=1.5, init=init)
    g.step(25)
    o, v = precip_oracle(oracle, dims, A=0.1, B=0.3, W=0.2, M=1.5, init=init)
    o.step_euler(0.1, 25)
    for f in range(2):
        assert rel(g.download(f).real, o.field(f).real) <= 1e-11, f
    assert abs(g.volcons_multiplier() - o.volcons_multiplier(v)) <= 1e-9 * max(1.0, abs(o.volcons_multiplier(v)))


def test_strain_single_precipitate_fp32(oracle):
    dims = [64, 64]
    g = precip_gpu(dims, "fp32")
    g.step(30)
    o, _ = precip_oracle(oracle, dims)
    o.step_euler(0.1, 30)
    for f in range(2):
        assert rel(g.download_real(f), o.field(f).real) <= 1e-4, f


@pytest.mark.parametrize("elastic,volcons", [(True, False), (False, True), (True, True)])
def test_precipitate_3d_fp64(oracle, elastic, volcons):
    """Without the elastic term this case amplifies rounding: the oracle against itself with conc's
    start perturbed by 1e-16 (relative) differs by 8e-12 after the 12 steps, hence 1e-10 there."""
    from gopf_gb300.synthetic import uniform_field

    dims = [16, 16, 16]
    n = 16 ** 3
    init = (square(dims) + uniform_field(21, n, 0.0, 0.05), square(dims) + uniform_field(22, n, 0.0, 0.05))
    g = precip_gpu(dims, "fp64", dt=0.05, elastic=elastic, volcons=volcons, init=init)
    g.step(12)
    o, v = precip_oracle(oracle, dims, dt=0.05, elastic=elastic, volcons=volcons, init=init)
    o.step_euler(0.05, 12)
    tol = 1e-11 if elastic else 1e-10
    for f in range(2):
        assert rel(g.download(f).real, o.field(f).real) <= tol, f
    if volcons:
        assert abs(g.volcons_multiplier() - o.volcons_multiplier(v)) <= 1e-9 * max(1.0, abs(o.volcons_multiplier(v)))


def test_elastic_on_the_first_field_of_the_second_equation(oracle):
    """The elastic term of conc's H(c) entering phase's equation (field and equation differ)."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [32, 32]
    n = 32 * 32
    c0, x0 = uniform_field(31, n, 0.4, 0.2), uniform_field(32, n, 0.5, 0.2)
    g = G.Model(dims, "fp64", device=0)
    g.add_field("conc")
    g.add_field("phase")
    g.add_scalar("m1", -1.0)
    g.register_elastic("LIN_ELAST", "conc", cubic(110.0, 60.0, 30.0), MISFIT)
    g.add_equation("dconc/dt = m1*LAP conc")
    g.add_equation("dphase/dt = m1*phase - LIN_ELAST + conc")
    g.init()
    g.set_stepper("euler", 0.01)
    g.upload(0, c0)
    g.upload(1, x0)
    g.step(20)
    o = oracle.Model(dims, 2)
    o.set_field(0, c0)
    o.set_field(1, x0)
    o.add_term(0, -1.0, lap=1, implicit=True)
    o.add_term(1, -1.0, implicit=True)
    o.add_elastic(1, 0, cubic(110.0, 60.0, 30.0), MISFIT, coef=-1.0)
    o.add_term(1, 1.0, src_kind=oracle.SRC_FIELD, src=0)
    o.step_euler(0.01, 20)
    for f in range(2):
        assert rel(g.download(f).real, o.field(f).real) <= 1e-11, f


def test_graph_replays_equal_eager_steps():
    import gopf_gb300 as G

    a = precip_gpu([32, 32], "fp64")
    b = precip_gpu([32, 32], "fp64")
    b.set_option(G._lib.OPT_USE_GRAPHS, 0)
    a.step(40)
    b.step(40)
    for f in range(2):
        assert np.array_equal(a.download(f), b.download(f))
    assert a.volcons_multiplier() == b.volcons_multiplier()


def test_polynomial_of_one_field_equals_register_function():
    """register_polynomial over one field steps exactly like the single-field polynomial kind."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    c0 = uniform_field(5, 64 * 64, 0.0, 0.1)
    out = []
    for how in ("poly", "mpoly"):
        m = G.Model([64, 64], "fp64", device=0)
        m.add_field("conc")
        if how == "poly":
            m.register_function("MU", G.DER_POLY, "conc", [1.0, -1.0], [3, 1])
        else:
            m.register_polynomial("MU", [1.0, -1.0], [[3], [1]])
        m.add_equation("dconc/dt = LAP MU - LAP^2 conc")
        m.init()
        m.set_stepper("euler", 0.01)
        m.upload(0, c0)
        m.step(20)
        out.append(m.download(0))
    assert np.array_equal(out[0], out[1])


def test_rejections():
    import gopf_gb300 as G

    m = precip_gpu([32, 32], "fp64")
    m.set_stepper("rk4", 0.1)
    with pytest.raises(G.GopfError):
        m.step(1)  # the elastic and volume-conserving terms are stepped with Euler
    m2 = G.Model([32, 32], "fp64", device=0)
    m2.add_field("conc")
    with pytest.raises(G.GopfError):
        m2.register_polynomial("P", [1.0], [[1, 1]])  # powers of a field that was not added
    with pytest.raises(G.GopfError):
        m2.register_polynomial("P", [1.0], [[-1]])
