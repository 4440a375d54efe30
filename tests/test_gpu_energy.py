"""Device energy monitors (gopf_free_energy, gopf_elastic_energy) against the oracle.

- The Cahn-Hilliard free energy sum (c^4/4 - c^2/2) + (gamma/2) sum |grad c|^2 of the
  stepped field, against the oracle's field after the same steps and against
  numpy on the device's own field: FP64 rel <= 1e-11, FP32 rel <= 1e-5.
- The energy falls at every step of the plain splitting (dt 0.05, gamma 0.5 in 3D;
  the benchmark's 256^3 FP32 run checked every 5 steps).
- HomogeneousModulusEnergy (elasticity/linearElasticity.go:101-165): the
  reference's own known answer, TestDilatationalMisfits
  (elasticity/linearElasticity_test.go:11-49: Eshelby's energy density within 5 %
  for 64^3 ellipsoids), and the oracle's restatement to rel 1e-10 in FP64 (1e-4
  in FP32), for the field and for its Indicator 3c^2 - 2c^3, in 2D and 3D.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CH_BULK = [0.0, 0.0, -0.5, 0.0, 0.25]
CH_EQ = "dconc/dt = M*LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc"


def ch_model(dims, prec, gamma, dt, c0):
    import gopf_gb300 as G

    m = G.Model(dims, prec, device=0)
    m.add_field("conc")
    m.add_scalar("gamma", gamma)
    m.add_scalar("M", 1.0)
    m.add_scalar("m1", -1.0)
    m.add_equation(CH_EQ)
    m.init()
    m.set_stepper("euler", dt)
    m.upload(0, c0)
    return m


def isotropic(bulk, nu):
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
    return C, shear


def cubic(c11, c12, c44):
    """CubicMaterial (elasticity/rank4.go:113-128), entry for entry."""
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        C[i, i, i, i] = c11
    for i in range(3):
        for j in range(i + 1, 3):
            C[i, i, j, j] = C[j, j, i, i] = c12
            C[i, j, i, j] = C[j, i, j, i] = c44
    return C


def ellipsoid(N, a, b, c):
    i, j, k = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    v = ((i - N // 2) / a) ** 2 + ((j - N // 2) / b) ** 2 + ((k - N // 2) / c) ** 2
    return (v <= 1.0).astype(np.float64).ravel()


@pytest.mark.parametrize("dims,prec,tol", [([32, 32, 32], "fp64", 1e-11), ([128, 128], "fp64", 1e-11),
                                           ([32, 32, 32], "fp32", 1e-5), ([256, 256], "fp32", 1e-5),
                                           # an odd axis (no Nyquist mode) and an even one of 2^2 3 5
                                           ([60, 45], "fp64", 1e-11), ([60, 45], "fp32", 1e-5)])
def test_free_energy_matches_oracle(oracle, dims, prec, tol):
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    gamma, dt = (0.5, 0.05) if len(dims) == 3 else (1.0, 0.1)
    c0 = uniform_field(21, n, 0.0 if len(dims) == 3 else 0.5, 0.1 if len(dims) == 3 else 0.05)
    g = ch_model(dims, prec, gamma, dt, c0)
    g.step(20)
    b, gr, tot = g.free_energy(0, CH_BULK, gamma)
    assert abs(tot - (b + gr)) <= 1e-14 * (abs(b) + abs(gr))
    o = oracle.cahn_hilliard(dims, gamma=gamma)
    o.set_field(0, c0)
    o.step_euler(dt, 20)
    ob, og = oracle.free_energy(o.field(0).real, dims, CH_BULK, gamma)
    scale = abs(ob) + abs(og)
    assert abs(b - ob) <= tol * scale and abs(gr - og) <= tol * scale
    # the monitor alone, on the device's own field
    db, dg = oracle.free_energy(g.download_real(0), dims, CH_BULK, gamma)
    own = 1e-12 if prec == "fp64" else 1e-6
    assert abs(b - db) <= own * scale and abs(gr - dg) <= own * scale
    g.close()


def test_free_energy_falls_every_step():
    """3D CH 64^3, gamma 0.5, dt 0.05, c0 = U(-0.1, 0.1), FP64: F decreases at each of 100 steps."""
    from gopf_gb300.synthetic import uniform_field

    dims = [64, 64, 64]
    g = ch_model(dims, "fp64", 0.5, 0.05, uniform_field(1, 64 ** 3, 0.0, 0.1))
    E = [g.free_energy(0, CH_BULK, 0.5)[2]]
    for _ in range(100):
        g.step(1)
        E.append(g.free_energy(0, CH_BULK, 0.5)[2])
    assert np.all(np.diff(E) < 0.0), np.diff(E).max()
    g.close()


def test_free_energy_falls_on_the_benchmark_run():
    """The benchmark's configuration (256^3, FP32, gamma 0.5, dt 0.05, seed 1): F decreases over
    each run of 5 steps for 60 steps."""
    from gopf_gb300.synthetic import uniform_field

    g = ch_model([256, 256, 256], "fp32", 0.5, 0.05, uniform_field(1, 256 ** 3, 0.0, 0.1))
    E = [g.free_energy(0, CH_BULK, 0.5)[2]]
    for _ in range(12):
        g.step(5)
        E.append(g.free_energy(0, CH_BULK, 0.5)[2])
    assert np.all(np.diff(E) < 0.0), np.diff(E).max()
    g.close()


@pytest.mark.parametrize("abc", [(10.0, 10.0, 10.0), (15.0, 7.0, 15.0), (7.0, 7.0, 15.0)])
def test_elastic_energy_eshelby(oracle, abc):
    """TestDilatationalMisfits on the device: 64^3 ellipsoids, isotropic (K 50, nu 0.3), dilatational
    misfit 0.05: within 5 % of 2(1+nu) mu eps^2/(1-nu), and within 1e-10 of the oracle."""
    import gopf_gb300 as G

    N, nu, bulk, eps = 64, 0.3, 50.0, 0.05
    C, shear = isotropic(bulk, nu)
    vox = ellipsoid(N, *abc)
    m = G.Model([N, N, N], "fp64", device=0)
    m.add_field("x")
    m.upload_real(0, vox)
    e = m.elastic_energy(C, np.eye(3) * eps)
    expect = 2.0 * (1.0 + nu) * shear * eps * eps / (1.0 - nu)
    assert abs(e - expect) <= 0.05 * expect
    ref = oracle.homogeneous_modulus_energy(vox, [N, N, N], np.eye(3) * eps, C)
    assert abs(e - ref) <= 1e-10 * abs(ref)
    m.close()


@pytest.mark.parametrize("dims,prec,tol", [([32, 32, 32], "fp64", 1e-10), ([64, 64], "fp64", 1e-10),
                                           ([32, 32, 32], "fp32", 1e-4),
                                           # Nyquist modes of a 2^3 3 axis; an odd axis
                                           ([24, 24, 24], "fp64", 1e-10), ([30, 45], "fp64", 1e-10),
                                           ([24, 24, 24], "fp32", 1e-4)])
@pytest.mark.parametrize("indicator", [False, True])
def test_elastic_energy_matches_oracle(oracle, dims, prec, tol, indicator):
    """A smooth random field (and its Indicator) under the cubic stiffness of the CH + elasticity
    configuration (C11 1.0, C12 0.6, C44 0.5) with an anisotropic misfit."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    x = uniform_field(31, n, 0.5, 0.5)
    C = cubic(1.0, 0.6, 0.5)
    misfit = np.array([[0.01, 0.002, 0.0], [0.002, -0.005, 0.001], [0.0, 0.001, 0.008]])
    m = G.Model(dims, prec, device=0)
    m.add_field("x")
    m.upload_real(0, x)
    e = m.elastic_energy(C, misfit, indicator=indicator)
    xin = 3 * x * x - 2 * x ** 3 if indicator else x
    ref = oracle.homogeneous_modulus_energy(xin, dims, misfit, C)
    assert abs(e - ref) <= tol * abs(ref)
    m.close()
