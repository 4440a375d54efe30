"""GPU parity of the semi-implicit spectral Euler step against the FP64 oracle.

Cases follow the reference's known-answer tests (pf/euler_test.go,
pf/solver_test.go) and the Cahn-Hilliard string of
examples/cahnHilliard/main.go:33, at sizes the oracle runs in seconds.
Tolerances: FP64 mode rel-L2 <= 1e-11 against the oracle; FP32 mode
rel-L2 <= 1e-4 (short trajectories) -- both written per test.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CH_EQ = "dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc"


def ch_gpu(dims, prec, gamma, dt, c0, M=1.0):
    import gopf_gb300 as G

    m = G.Model(dims, prec, device=0)
    m.add_field("conc")
    m.add_scalar("gamma", gamma)
    m.add_scalar("m1", -M)
    m.add_scalar("M", M)
    m.add_equation("dconc/dt = M*LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    m.init()
    m.set_stepper("euler", dt)
    m.upload(0, c0)
    return m


def ch_oracle(O, dims, gamma, c0, M=1.0):
    m = O.cahn_hilliard(dims, gamma=gamma, M=M)
    m.set_field(0, c0)
    return m


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_exponential_decay_gpu():
    """TestExponentialDecay (pf/euler_test.go:10-49) on the device, FP64."""
    import gopf_gb300 as G

    m = G.Model([8, 8], "fp64", device=0)
    m.add_field("field")
    m.add_scalar("rate", -1.0)
    m.add_equation("dfield/dt = rate*field")
    m.init()
    m.set_stepper("euler", 0.001)
    m.upload(0, np.ones(64))
    m.step(1000)
    f = m.download(0)
    assert np.all(np.abs(f.real - math.exp(-1.0)) < 1e-3)
    assert abs(m.time - 1.0) < 1e-10


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_square_decay_gpu(prec):
    """TestEulerSquareDecary (pf/euler_test.go:51-85): 1/(1+t) within 1e-3."""
    import gopf_gb300 as G

    m = G.Model([8, 8], prec, device=0)
    m.add_field("field")
    m.add_scalar("rate", -1.0)
    m.add_equation("dfield/dt = rate*field^2")
    m.init()
    m.set_stepper("euler", 0.001)
    m.upload(0, np.ones(64))
    m.step(1000)
    assert np.all(np.abs(m.download(0).real - 0.5) < 1e-3)


def test_solver_diffusion_gpu():
    """TestSolverDiffusion (pf/solver_test.go:9-34): mass 1 to 1e-4, values in [0, 1)."""
    import gopf_gb300 as G

    m = G.Model([16, 16], "fp64", device=0)
    m.add_field("conc")
    m.add_equation("dconc/dt = LAP conc")
    m.init()
    m.set_stepper("euler", 0.1)
    c = np.zeros(256)
    c[128] = 1.0
    m.upload(0, c)
    for _ in range(10):
        m.step(10)
    d = m.download(0).real
    assert abs(d.sum() - 1.0) < 1e-4
    assert np.all(d < 1.0) and np.all(d >= 0.0)


@pytest.mark.parametrize("dims,steps", [([64, 64], 50), ([128, 128], 1000), ([48, 96], 100)])
def test_cahn_hilliard_2d_fp64_parity(oracle, dims, steps):
    """2D CH, the plain splitting of examples/cahnHilliard, FP64 mode vs oracle: rel-L2 <= 1e-11."""
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c0 = uniform_field(0, n, 0.5, 0.05)
    g = ch_gpu(dims, "fp64", 1.0, 0.1, c0)
    g.step(steps)
    o = ch_oracle(oracle, dims, 1.0, c0)
    o.step_euler(0.1, steps)
    err = rel_l2(g.download(0).real, o.field(0).real)
    assert err <= 1e-11, err
    assert abs(g.mass(0) - o.field(0).real.sum()) <= 1e-9 * n


@pytest.mark.parametrize("dims,steps", [([16, 16, 16], 20), ([32, 32, 32], 50), ([24, 24, 24], 10)])
def test_cahn_hilliard_3d_fp64_parity(oracle, dims, steps):
    """3D CH (gamma 0.5, dt 0.05 as in the 256^3 configuration), FP64 mode vs oracle: rel-L2 <= 1e-11."""
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c0 = uniform_field(1, n, 0.0, 0.1)
    g = ch_gpu(dims, "fp64", 0.5, 0.05, c0)
    g.step(steps)
    o = ch_oracle(oracle, dims, 0.5, c0)
    o.step_euler(0.05, steps)
    err = rel_l2(g.download(0).real, o.field(0).real)
    assert err <= 1e-11, err


@pytest.mark.parametrize("dims,steps,gamma,dt,center,hw", [([128, 128], 100, 1.0, 0.1, 0.5, 0.05),
                                                            ([32, 32, 32], 50, 0.5, 0.05, 0.0, 0.1)])
def test_cahn_hilliard_fp32_parity(oracle, dims, steps, gamma, dt, center, hw):
    """FP32 mode vs the FP64 oracle on short trajectories: rel-L2 <= 1e-4."""
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c0 = uniform_field(2, n, center, hw)
    g = ch_gpu(dims, "fp32", gamma, dt, c0)
    g.step(steps)
    o = ch_oracle(oracle, dims, gamma, c0)
    o.step_euler(dt, steps)
    err = rel_l2(g.download(0).real, o.field(0).real)
    assert err <= 1e-4, err


def test_explicit_linear_splitting_matches_oracle(oracle):
    """The splitting mu = c^3 - c explicit, -gamma k^4 implicit (c_k <- (c_k - dt M k^2 mu_k) /
    (1 + dt M gamma k^4)), via a registered polynomial."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [64, 64]
    c0 = uniform_field(5, 64 * 64, 0.5, 0.05)
    m = G.Model(dims, "fp64", device=0)
    m.add_field("conc")
    m.add_scalar("mg", -1.3)
    m.add_scalar("M", 0.8)
    m.register_function("MU", G.DER_POLY, "conc", [1.0, -1.0], [3, 1])
    m.add_equation("dconc/dt = M*LAP MU + mg*M*LAP^2 conc")
    m.init()
    m.set_stepper("euler", 0.05)
    m.upload(0, c0)
    m.step(200)
    o = oracle.cahn_hilliard(dims, gamma=1.3, M=0.8, splitting="explicit_linear")
    o.set_field(0, c0)
    o.step_euler(0.05, 200)
    assert rel_l2(m.download(0).real, o.field(0).real) <= 1e-11


def test_graph_and_eager_paths_agree():
    """Steps replayed from CUDA graphs equal steps launched one by one (bitwise)."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [64, 64, 64]
    c0 = uniform_field(9, 64 ** 3, 0.0, 0.1)
    a = ch_gpu(dims, "fp32", 0.5, 0.05, c0)
    b = ch_gpu(dims, "fp32", 0.5, 0.05, c0)
    b.set_option(G._lib.OPT_USE_GRAPHS, 0)
    a.step(37)
    b.step(37)
    assert np.array_equal(a.download(0), b.download(0))


def test_nan_is_reported_not_trapped():
    """A blow-up is reported as GOPF_ERR_NAN by the host check (no device trap)."""
    import gopf_gb300 as G

    m = G.Model([8, 8], "fp32", device=0)
    m.add_field("f")
    m.add_equation("df/dt = f^4")
    m.init()
    m.set_stepper("euler", 1.0)
    m.upload(0, np.full(64, 10.0))
    with pytest.raises(G.GopfError) as e:
        m.step(10)
    assert e.value.status == 4


def test_mass_conserved_3d_256_fp32():
    """3D CH at 256^3 FP32 (the configuration of the benchmark): mass drift after 200 steps <= 1e-6 (absolute per cell)."""
    from gopf_gb300.synthetic import uniform_field

    n = 256 ** 3
    c0 = uniform_field(1, n, 0.0, 0.1)
    g = ch_gpu([256, 256, 256], "fp32", 0.5, 0.05, c0)
    m0 = g.mass(0)
    g.step(200)
    m1 = g.mass(0)
    assert abs(m1 - m0) / n <= 1e-6
    d = g.download(0).real
    assert np.all(np.isfinite(d))
    assert abs(d.sum() - c0.sum()) / n <= 1e-6


# ---------------------------------------------------------------- RK4 (pf/rk4.go)

def test_rk4_simple_model_gpu():
    """TestSimpleModel (pf/rk4_test.go:14-54): dfield/dt = rate*field^2, RK4 dt 0.1, 10 steps, 1e-6."""
    import gopf_gb300 as G

    m = G.Model([8, 8], "fp64", device=0)
    m.add_field("field")
    m.add_scalar("rate", -1.0)
    m.add_equation("dfield/dt = rate*field^2")
    m.init()
    m.set_stepper("rk4", 0.1)
    m.upload(0, np.ones(64))
    m.step(10)
    assert np.all(np.abs(m.download(0).real - 0.5) < 1e-6)


def test_rk4_with_implicit_gpu():
    """TestWithImplicit (pf/rk4_test.go:61-99): logistic growth, RK4 dt 0.01, 100 steps, 1e-3."""
    import gopf_gb300 as G

    m = G.Model([8, 8], "fp64", device=0)
    m.add_field("field")
    m.add_scalar("rate", -1.0)
    m.add_equation("dfield/dt = field + rate*field^2")
    m.init()
    m.set_stepper("rk4", 0.01)
    m.upload(0, np.full(64, 0.5))
    m.step(100)
    exp = math.exp(1.0) / (1.0 + math.exp(1.0))
    assert np.all(np.abs(m.download(0).real - exp) < 1e-3)


@pytest.mark.parametrize("dims,steps,prec,tol", [([64, 64], 100, "fp64", 1e-11), ([16, 16, 16], 20, "fp64", 1e-11),
                                                  ([32, 32, 32], 30, "fp32", 1e-4)])
def test_rk4_cahn_hilliard_parity(oracle, dims, steps, prec, tol):
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c0 = uniform_field(6, n, 0.5 if len(dims) == 2 else 0.0, 0.05 if len(dims) == 2 else 0.1)
    g = ch_gpu(dims, prec, 1.0, 0.1, c0)
    g.set_stepper("rk4", 0.1)
    g.step(steps)
    o = ch_oracle(oracle, dims, 1.0, c0)
    o.step_rk4(0.1, steps)
    assert rel_l2(g.download(0).real, o.field(0).real) <= tol


# ---------------------------------------------------------------- register-resident 256-point kernels

def _two_group_model(dims, prec, c0, fast):
    """Two explicit groups (LAP^1 and LAP^0) so that the fused passes carry two arrays."""
    import gopf_gb300 as G

    m = G.Model(dims, prec, device=0)
    m.set_option(G._lib.OPT_FAST_KERNELS, int(fast))
    m.add_field("conc")
    m.add_scalar("gamma", 0.5)
    m.add_scalar("m1", -1.0)
    m.add_scalar("eps", 0.05)
    m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc - eps*conc^2")
    m.init()
    m.set_stepper("euler", 0.05)
    m.upload(0, c0)
    return m


@pytest.mark.parametrize("dims", [[256, 256, 256], [256, 256], [384, 384], [512, 512], [768, 768], [1024, 1024]])
@pytest.mark.parametrize("two_groups", [False, True])
def test_fast_kernels_match_generic(dims, two_groups):
    """The register kernels (the 256-point engine, and the line engine for 2D sides 384 ... 1024)
    and the generic Stockham kernels agree (FP32, 20 steps)."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c0 = uniform_field(1, n, 0.0, 0.1)
    if two_groups:
        a = _two_group_model(dims, "fp32", c0, True)
        b = _two_group_model(dims, "fp32", c0, False)
    else:
        a = ch_gpu(dims, "fp32", 0.5, 0.05, c0)
        b = ch_gpu(dims, "fp32", 0.5, 0.05, c0)
        b.set_option(G._lib.OPT_FAST_KERNELS, 0)
    a.step(20)
    b.step(20)
    assert rel_l2(a.download(0).real, b.download(0).real) <= 2e-6


def test_fast_kernels_2d_256_vs_oracle(oracle):
    """FP32 fast path on 256^2 against the FP64 oracle, 100 steps: rel-L2 <= 1e-4."""
    from gopf_gb300.synthetic import uniform_field

    dims = [256, 256]
    c0 = uniform_field(0, 256 * 256, 0.5, 0.05)
    g = ch_gpu(dims, "fp32", 1.0, 0.1, c0)
    g.step(100)
    o = ch_oracle(oracle, dims, 1.0, c0)
    o.step_euler(0.1, 100)
    assert rel_l2(g.download(0).real, o.field(0).real) <= 1e-4


@pytest.mark.parametrize("two_groups", [False, True])
def test_tma_tiles_match_plain_loads(two_groups):
    """The x and z kernels that move their tiles with TMA compute exactly what the plain-load kernels
    do (same arithmetic, different data movement): bitwise equal after 10 steps, 256^3 FP32 (upload
    and download through the same kernels in both runs)."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [256, 256, 256]
    c0 = uniform_field(5, 256 ** 3, 0.0, 0.1)
    models = []
    for tma in (1, 0):
        if two_groups:
            m = _two_group_model(dims, "fp32", c0, True)
        else:
            m = ch_gpu(dims, "fp32", 0.5, 0.05, c0)
        m.set_option(G._lib.OPT_TMA, tma)
        m.step(10)
        m.set_option(G._lib.OPT_TMA, 1)  # the same transform back to real space for both
        models.append(m.download(0).real)
    assert np.array_equal(models[0], models[1])


def test_half_height_x_tiles_match():
    """The one-group 256-column x pass on 16-row tiles (128 threads, eight blocks per SM) computes
    exactly what the 32-row tiles do: bitwise equal after 10 steps, 256^3 and 256^2 FP32."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    for dims in ([256, 256, 256], [256, 256]):
        c0 = uniform_field(8, int(np.prod(dims)), 0.0, 0.1)
        out = []
        for rows in (16, 32):
            m = ch_gpu(dims, "fp32", 0.5, 0.05, c0)
            m.set_option(G._lib.OPT_X_ROWS, rows)
            m.step(10)
            out.append(m.download(0).real)
            m.close()
        assert np.array_equal(out[0], out[1])


def test_programmatic_dependent_launches_match():
    """The 3D step with its forward y, fused z and inverse y kernels launched as programmatic
    dependents (tables set up while the previous kernel finishes, data read after griddepcontrol.wait)
    steps exactly what plain stream order steps: bitwise after 1 and 21 steps (the 1-step and 16-step
    graphs), 256^3 FP32; and eagerly (no graphs) after 3 steps."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    c0 = uniform_field(10, 256 ** 3, 0.0, 0.1)
    a = ch_gpu([256, 256, 256], "fp32", 0.5, 0.05, c0)
    b = ch_gpu([256, 256, 256], "fp32", 0.5, 0.05, c0)
    b.set_option(G._lib.OPT_PDL, 0)
    for n in (1, 20):
        a.step(n)
        b.step(n)
        assert np.array_equal(a.download_real(0), b.download_real(0))
    a.set_option(G._lib.OPT_USE_GRAPHS, 0)
    b.set_option(G._lib.OPT_USE_GRAPHS, 0)
    a.step(3)
    b.step(3)
    assert np.array_equal(a.download_real(0), b.download_real(0))
    a.close()
    b.close()


def test_half_width_z_tiles_match():
    """The one-group 256-point z pass on 8-line tiles (128 threads, six blocks per SM) computes
    exactly what the 16-line tiles do: bitwise equal after 10 steps, 256^3 FP32."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    c0 = uniform_field(9, 256 ** 3, 0.0, 0.1)
    out = []
    for lines in (8, 16):
        m = ch_gpu([256, 256, 256], "fp32", 0.5, 0.05, c0)
        m.set_option(G._lib.OPT_Z_LINES, lines)
        m.step(10)
        out.append(m.download(0).real)
        m.close()
    assert np.array_equal(out[0], out[1])


def test_real_space_x_kernels_match_generic():
    """Upload (real -> spectrum), download (spectrum -> real) and the FP64 reductions through the
    256-column real-space kernels agree with the generic x pass to FP32 round-off."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [256, 256, 256]
    c0 = uniform_field(9, 256 ** 3, 0.2, 0.1)
    out = []
    for tma in (1, 0):
        m = G.Model(dims, "fp32", device=0)
        m.set_option(G._lib.OPT_TMA, tma)
        m.add_field("conc")
        m.add_scalar("gamma", 0.5)
        m.add_scalar("m1", -1.0)
        m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
        m.init()
        m.set_stepper("euler", 0.05)
        m.upload(0, c0)
        d = m.download_real(0)
        assert np.max(np.abs(d - c0)) < 2e-6  # the round trip
        out.append((d, m.mass(0), m.reduce(0, G.RED_MIN), m.reduce(0, G.RED_MAX), m.reduce(0, G.RED_SUMSQ)))
        m.step(5)
        out[-1] = out[-1] + (m.download_real(0),)
    (d1, s1, mn1, mx1, q1, e1), (d0, s0, mn0, mx0, q0, e0) = out
    assert rel_l2(d1, d0) < 1e-6 and rel_l2(e1, e0) < 1e-6
    # both sums are FP64 over FP32 cells; the FP32 field itself carries ~1e-8 relative error
    assert abs(s1 - s0) <= 1e-9 * abs(s0) and abs(s1 - c0.sum()) < 1e-7 * abs(c0.sum())
    assert abs(mn1 - c0.min()) < 2e-6 and abs(mx1 - c0.max()) < 2e-6
    assert abs(q1 - q0) <= 1e-6 * q0


def test_pinned_host_buffers_read_in_place():
    """Upload from and download to pinned host memory (read and written by kernels in place) give
    exactly what the staged path gives for pageable memory."""
    import ctypes

    import torch

    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [64, 64, 64]
    n = 64 ** 3
    c0 = uniform_field(4, n, 0.0, 0.1)
    m = ch_gpu(dims, "fp32", 0.5, 0.05, c0)
    L = G.load()
    pinned = torch.zeros(2 * n, dtype=torch.float64, pin_memory=True)
    pinned.numpy()[0::2] = c0
    dp = ctypes.cast(pinned.data_ptr(), ctypes.POINTER(ctypes.c_double))
    m._ck(L.gopf_field_upload(m.handle, 0, dp, n))
    m.step(3)
    m._ck(L.gopf_field_download(m.handle, 0, dp, n))
    a = pinned.numpy().copy()
    m.upload(0, c0)            # pageable numpy buffer: staged
    m.step(3)
    b = m.download(0)          # pageable
    assert np.array_equal(a[0::2], b.real) and np.all(a[1::2] == 0.0)


@pytest.mark.parametrize("dims,prec,tol", [([48, 32], "fp64", 1e-13), ([24, 24, 24], "fp64", 1e-13),
                                           ([64, 64, 64], "fp32", 2e-6)])
def test_point_monitor_matches_download(dims, prec, tol):
    """PointMonitor.Add (pf/monitor.go:27-30): the value at a node, read from the device state
    without downloading the field; node order of pfutil/indexPositionConversion.go:23-34."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    m = G.Model(dims, prec, device=0)
    m.add_field("conc")
    m.add_scalar("gamma", 0.5)
    m.add_scalar("m1", -1.0)
    m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    m.init()
    m.set_stepper("euler", 0.05)
    m.upload(0, uniform_field(5, n, 0.0, 0.1))
    m.step(7)
    full = m.download_real(0)
    sites = np.array([0, 1, n - 1, n // 2, 12345 % n, dims[1] - 1, dims[1]])
    vals = m.point_values(0, sites)
    assert np.max(np.abs(vals - full[sites])) <= tol * np.max(np.abs(full))
    with pytest.raises(G.GopfError) as e:
        m.point_values(0, [n])
    assert e.value.status == 1


@pytest.mark.parametrize("side", [384, 512, 768, 1024])
def test_line_engine_2d_vs_oracle(oracle, side):
    """2D FP32 Cahn-Hilliard on the line engine against the FP64 oracle (rel-L2 <= 1e-5, 10 steps)."""
    from gopf_gb300.synthetic import uniform_field

    dims = [side, side]
    c0 = uniform_field(7, side * side, 0.5, 0.05)
    g = ch_gpu(dims, "fp32", 0.5, 0.05, c0)
    g.step(10)
    o = oracle.cahn_hilliard(dims, gamma=0.5)
    o.set_field(0, c0)
    o.step_euler(0.05, 10)
    assert rel_l2(g.download_real(0), o.field(0).real) <= 1e-5
