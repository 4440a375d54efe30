"""ImplicitEuler (pf/implicitEuler.go): the oracle restatement against the reference's analytic tests,
and the device Newton-Krylov solve against the oracle and the same analytic tests.

TestImplicitEuler (pf/implicitEuler_test.go:10-108): 8x8 fields, dt = 0.01, 100 steps, tolerance 5e-3
against the ODE solutions, the two coupled fields included.  TestDissipatingHeatEquation (:160-223):
128^2, dt = 0.005, 10 steps, 1e-3.  Device against oracle (FP64, both solved to max|F| <= 1e-12):
rel-L2 <= 1e-9.
"""
import math

import numpy as np
import pytest

ODE_CASES = [
    # (device equation, oracle builder, c0, analytic solution at t)
    ("dconc/dt = -conc", "lin", 1.0, lambda t: math.exp(-t)),
    ("dconc/dt = -conc^2", "sq", 1.0, lambda t: 1.0 / (1.0 + t)),
    ("dconc/dt = conc - conc^2", "logistic", 0.5, lambda t: math.exp(t) / (1.0 + math.exp(t))),
]


def oracle_ode(O, kind, c0, n=8):
    m = O.Model([n, n], 1)
    m.set_field(0, np.full(n * n, c0))
    if kind == "lin":
        m.add_term(0, -1.0, implicit=True)
    elif kind == "sq":
        d = m.add_product([0], [2])
        m.add_term(0, -1.0, src_kind=O.SRC_DERIVED, src=d)
    elif kind == "logistic":
        m.add_term(0, 1.0, implicit=True)
        d = m.add_product([0], [2])
        m.add_term(0, -1.0, src_kind=O.SRC_DERIVED, src=d)
    return m


def heat_init(N):
    i = np.arange(N * N)
    x = (i // N) / N
    y = (i % N) / N
    return np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y), x, y


def heat_analytic(N, gamma, t, x, y):
    L = float(N)
    return np.exp(-(4.0 * np.pi / (L * L) + gamma) * t) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * x)


@pytest.mark.parametrize("eq,kind,c0,sol", ODE_CASES)
def test_oracle_implicit_euler_odes(oracle, eq, kind, c0, sol):
    from oracle.implicit_ref import implicit_euler_step

    m = oracle_ode(oracle, kind, c0)
    for _ in range(100):
        implicit_euler_step(m, [8, 8], 0.01)
    assert np.max(np.abs(m.field(0).real - sol(1.0))) < 5e-3


def test_oracle_implicit_euler_coupled_fields(oracle):
    """The two-field case of TestImplicitEuler: dconc1/dt = -conc1*conc2, dconc2/dt = -conc2.
    Only the oracle runs it (the device steps single-field models); restated directly in numpy."""
    dt, n = 0.01, 100
    c1, c2 = 1.0, 1.0
    for _ in range(n):
        # spatially uniform: the implicit step is the ETD scheme on the k = 0 mode (L = -1 for conc2,
        # L = 0 for conc1); solve the 2x2 fixed point by iteration
        x1, x2 = c1, c2
        for _ in range(200):
            f2 = math.exp(-dt)
            x2n = c2 * f2
            N1p, N1x = -c1 * c2, -x1 * x2n
            x1n = c1 + 0.5 * dt * (N1x + N1p)
            if abs(x1n - x1) < 1e-15 and abs(x2n - x2) < 1e-15:
                break
            x1, x2 = x1n, x2n
        c1, c2 = x1, x2
    t = dt * n
    assert abs(c1 - math.exp(math.exp(-t) - 1.0)) < 5e-3
    assert abs(c2 - math.exp(-t)) < 5e-3


def test_oracle_dissipating_heat_equation(oracle):
    from oracle.implicit_ref import implicit_euler_step

    N, gamma, dt = 128, 0.2, 0.005
    f0, x, y = heat_init(N)
    m = oracle.Model([N, N], 1)
    m.set_field(0, f0)
    m.add_term(0, 1.0, lap=1, implicit=True)
    d = m.add_poly(0, [-gamma], [1])
    m.add_term(0, 1.0, src_kind=oracle.SRC_DERIVED, src=d)
    for _ in range(10):
        implicit_euler_step(m, [N, N], dt)
    assert np.max(np.abs(m.field(0).real - heat_analytic(N, gamma, 10 * dt, x, y))) < 1e-3


# ---------------------------------------------------------------------------------------- device


def gpu_ode(eq, c0, prec="fp64", n=8):
    import gopf_gb300 as G

    m = G.Model([n, n], prec, device=0)
    m.add_field("conc")
    m.add_equation(eq)
    m.init()
    m.set_stepper("implicit_euler", 0.01)
    m.upload(0, np.full(n * n, c0))
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("eq,kind,c0,sol", ODE_CASES)
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_device_implicit_euler_odes(eq, kind, c0, sol, prec):
    m = gpu_ode(eq, c0, prec)
    m.step(100)
    assert np.max(np.abs(m.download_real(0) - sol(1.0))) < 5e-3
    _, _, _, conv = m.newton_stats()
    assert conv


@pytest.mark.gpu
def test_device_dissipating_heat_equation():
    import gopf_gb300 as G

    N, gamma, dt = 128, 0.2, 0.005
    f0, x, y = heat_init(N)
    m = G.Model([N, N], "fp64", device=0)
    m.add_field("temperature")
    m.register_function("DISSIPATE", G.DER_POLY, "temperature", [-gamma], [1])
    m.add_equation("dtemperature/dt = LAP temperature + DISSIPATE")
    m.init()
    m.set_stepper("implicit_euler", dt)
    m.upload(0, f0)
    m.step(10)
    assert np.max(np.abs(m.download_real(0) - heat_analytic(N, gamma, 10 * dt, x, y))) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [[32, 32], [16, 16, 16]])
def test_device_implicit_cahn_hilliard_matches_oracle(oracle, dims):
    """Cahn-Hilliard with ImplicitEuler, FP64: the device Newton-Krylov and the oracle's solve reach
    the same root (both to max|F| <= 1e-12), 5 steps."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field
    from oracle.implicit_ref import implicit_euler_step

    n = int(np.prod(dims))
    c0 = uniform_field(11, n, 0.0, 0.1)
    dt = 0.05
    g = G.Model(dims, "fp64", device=0)
    g.add_field("conc")
    g.add_scalar("gamma", 0.5)
    g.add_scalar("m1", -1.0)
    g.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    g.init()
    g.set_stepper("implicit_euler", dt)
    g.set_newton_krylov(tol=1e-12)
    g.upload(0, c0)
    o = oracle.cahn_hilliard(dims, gamma=0.5)
    o.set_field(0, c0)
    for _ in range(5):
        g.step(1)
        _, _, res, conv = g.newton_stats()
        assert conv and res <= 1e-12
        implicit_euler_step(o, dims, dt, tol=1e-12)
    ref = o.field(0).real
    assert np.linalg.norm(g.download_real(0) - ref) / np.linalg.norm(ref) <= 1e-9


def test_oracle_implicit_euler_coupled_fields_restatement(oracle):
    """The two-field case of TestImplicitEuler through the oracle's ImplicitEuler restatement (one
    Newton-Krylov solve over both fields per step)."""
    from oracle.implicit_ref import implicit_euler_step

    m = oracle.Model([8, 8], 2)
    m.set_field(0, np.ones(64))
    m.set_field(1, np.ones(64))
    m.add_term(0, -1.0, src_kind=oracle.SRC_DERIVED, src=m.add_product([0, 1], [1, 1]))
    m.add_term(1, -1.0, implicit=True)
    for _ in range(100):
        implicit_euler_step(m, [8, 8], 0.01)
    assert np.max(np.abs(m.field(0).real - math.exp(math.exp(-1.0) - 1.0))) < 5e-3
    assert np.max(np.abs(m.field(1).real - math.exp(-1.0))) < 5e-3


def gpu_coupled(prec, n=8):
    import gopf_gb300 as G

    m = G.Model([n, n], prec, device=0)
    m.add_field("conc1")
    m.add_field("conc2")
    m.add_equation("dconc1/dt = -conc1*conc2")
    m.add_equation("dconc2/dt = -conc2")
    m.init()
    m.set_stepper("implicit_euler", 0.01)
    m.upload(0, np.ones(n * n))
    m.upload(1, np.ones(n * n))
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_device_implicit_euler_coupled_fields(oracle, prec):
    """The two-field case of TestImplicitEuler on the device: the ODE solutions within 5e-3, and in
    FP64 the oracle's restatement within 1e-9."""
    from oracle.implicit_ref import implicit_euler_step

    m = gpu_coupled(prec)
    m.step(100)
    _, _, _, conv = m.newton_stats()
    assert conv
    assert np.max(np.abs(m.download_real(0) - math.exp(math.exp(-1.0) - 1.0))) < 5e-3
    assert np.max(np.abs(m.download_real(1) - math.exp(-1.0))) < 5e-3
    if prec == "fp64":
        o = oracle.Model([8, 8], 2)
        o.set_field(0, np.ones(64))
        o.set_field(1, np.ones(64))
        o.add_term(0, -1.0, src_kind=oracle.SRC_DERIVED, src=o.add_product([0, 1], [1, 1]))
        o.add_term(1, -1.0, implicit=True)
        for _ in range(100):
            implicit_euler_step(o, [8, 8], 0.01, tol=1e-12)
        for f in range(2):
            assert np.max(np.abs(m.download_real(f) - o.field(f).real)) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [[32, 32], [16, 16, 16]])
def test_device_implicit_two_fields_matches_oracle(oracle, dims):
    """Two spatially varying coupled fields, da/dt = LAP a - a b, db/dt = -b + a^2 (ImplicitEuler,
    FP64): the device and the oracle reach the same root every step (both to max|F| <= 1e-12)."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field
    from oracle.implicit_ref import implicit_euler_step

    n = int(np.prod(dims))
    a0, b0 = uniform_field(41, n, 0.3, 0.1), uniform_field(42, n, 0.2, 0.1)
    dt = 0.05
    g = G.Model(dims, "fp64", device=0)
    g.add_field("a")
    g.add_field("b")
    g.add_scalar("m1", -1.0)
    g.add_equation("da/dt = LAP a - a*b")
    g.add_equation("db/dt = m1*b + a^2")
    g.init()
    g.set_stepper("implicit_euler", dt)
    g.set_newton_krylov(tol=1e-12)
    g.upload(0, a0)
    g.upload(1, b0)
    o = oracle.Model(dims, 2)
    o.set_field(0, a0)
    o.set_field(1, b0)
    o.add_term(0, 1.0, lap=1, implicit=True)
    o.add_term(0, -1.0, src_kind=oracle.SRC_DERIVED, src=o.add_product([0, 1], [1, 1]))
    o.add_term(1, -1.0, implicit=True)
    o.add_term(1, 1.0, src_kind=oracle.SRC_DERIVED, src=o.add_product([0], [2]))
    for _ in range(3):
        g.step(1)
        _, _, res, conv = g.newton_stats()
        assert conv and res <= 1e-12
        implicit_euler_step(o, dims, dt, tol=1e-12)
    for f in range(2):
        ref = o.field(f).real
        assert np.linalg.norm(g.download_real(f) - ref) / np.linalg.norm(ref) <= 1e-9
