"""The oracle's shrinking-dimer dynamics (pf/sdd.go) against the reference's SDD tests.

Known answers of pf/sdd_test.go:
- TestHouseHolder (:409-451): the reflection of a 4x4 vector, golden values from numpy;
- TestHouseHolderDenum (:453-511): the Sherman-Morrison solve against a dense solve;
- TestDiagonalShermannMorrison (:273-323): (D + u v^T)^-1 b against a dense solve;
- TestFourierOuterProduct (:14-57): an outer product evaluated in Fourier space;
- TestDimerLengthTime (:59-66);
- TestDoubleWell (:68-108): the saddle of conc - conc^3 is 0 (1e-6);
- TestRevertOrientationVector (:343-381): v and -v give the same path (1e-10);
- TestClassicalNucleation (:165-271): the critical nucleus radius 2 sigma / rho (0.3).
"""
import math

import numpy as np
import pytest


def box_blur(a, width=2):
    """pfutil.Blur with a BoxKernel (pfutil/blur.go:38-70): the periodic mean over the
    (2 Cutoff + 1)^d box, Cutoff = width/2 + 1, of the shifts |s| <= width."""
    c = width // 2 + 1
    out = np.zeros_like(a)
    cnt = 0
    for dy in range(-c, c + 1):
        for dx in range(-c, c + 1):
            if abs(dy) <= width and abs(dx) <= width:
                out += np.roll(np.roll(a, -dy, axis=0), -dx, axis=1)
                cnt += 1
    return out / cnt


def circle(n, radius, inside=1.0, outside=-1.0):
    """insertCircleAtCenter (pf/sdd_test.go:153-163) on a field of `outside`."""
    r, c = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = np.full((n, n), outside)
    a[(r - n // 2) ** 2 + (c - n // 2) ** 2 <= radius * radius] = inside
    return a


def test_householder_known_answer(oracle):
    n = 4
    vec = np.arange(16, dtype=np.complex128)
    orient = np.array([i * i - 3 * i for i in range(16)], dtype=np.complex128)
    orient /= np.linalg.norm(orient)
    fv = oracle.fftn(vec, [n, n])
    fo = oracle.fftn(orient, [n, n])
    r = oracle.householder(fv, fo, 2.0, 16)
    out = oracle.fftn(r, [n, n], sign=+1) / 16
    expect = [0.0, 1.41446756, 2.41446756, 3.0, 3.17106489, 2.92766222, 2.26979199, 1.19745421, -0.28935113,
              -2.19062403, -4.50636448, -7.23657249, -10.38124806, -13.94039118, -17.91400186, -22.3020801]
    assert np.max(np.abs(out.real - expect)) < 1e-6


def test_householder_denum_against_dense_solve(oracle):
    n, dt, sigma = 16, 0.8, 1.0
    N = n * n
    orient = np.array([0.1 * (i * i - 4 * i) for i in range(N)])
    orient /= np.linalg.norm(orient)
    x = 0.1 * np.arange(N)
    A = np.eye(N) * (1.0 - dt) + dt * sigma * np.outer(orient, orient)
    res = np.linalg.solve(A, x)
    fo = oracle.fftn(orient.astype(np.complex128), [n, n])
    fx = oracle.fftn(x.astype(np.complex128), [n, n])
    y = oracle.sdd_denum_dot(np.ones(N), fo, sigma, dt, fx)
    out = oracle.fftn(y, [n, n], sign=+1) / N
    assert np.max(np.abs(out.real - res)) < 1e-10


def test_sherman_morrison_3x3(oracle):
    D = np.array([0.4, -0.2, 1.4])
    u = np.array([-1.0, 2.0, 3.0])
    v = np.array([2.0, 2.3, 1.2])
    b = np.array([4.0, 6.0, 8.2])
    res = np.linalg.solve(np.diag(D) + np.outer(u, v), b)
    out = oracle.dsm_dot(1.0 / D, u, v, b)
    assert np.max(np.abs(out.real - res)) < 1e-10


def test_fourier_outer_product(oracle):
    n = 8
    i = np.arange(n * n)
    data = (i / 10.0).astype(np.complex128)
    vector = ((i * i - i) / 10.0).astype(np.complex128)
    expect = vector.real * np.dot(data.real, vector.real)
    fd = oracle.fftn(data, [n, n])
    fv = oracle.fftn(vector, [n, n])
    dot = np.sum(np.conj(fv) * fd) / (n * n)
    out = oracle.fftn(fv * dot, [n, n], sign=+1) / (n * n)
    assert np.max(np.abs(out.real - expect)) < 1e-6
    assert np.max(np.abs(out.imag)) < 1e-6


def test_dimer_length_time(oracle):
    m = oracle.Model([4, 4], 1)
    s = oracle.SDD(m)
    s.set_params(0.1, init_len=5.0)
    t = 1.0 * math.log(5.0 / 0.5)  # RequiredDimerLengthTime (pf/sdd.go:364-367)
    assert abs(s.dimer_length(t) - 0.5) < 1e-10


def test_double_well_saddle(oracle):
    n = 4
    m = oracle.Model([n, n], 1)
    m.add_term(0, 1.0, implicit=True)  # conc (bilinear)
    c3 = m.add_product([0], [3])
    m.add_term(0, -1.0, src_kind=oracle.SRC_DERIVED, src=c3)
    init = np.full(16, -1.0)
    final = np.full(16, 1.5)
    m.set_field(0, 0.5 * (init + final))
    s = oracle.SDD(m)
    dt = 0.1
    s.set_params(dt)
    s.init(init, final)
    s.set_params(dt, init_len=0.1)
    final_time = 1.0 * math.log(0.1 / (1e-6 * 0.1))
    s.step(int(final_time / dt) + 1)
    assert np.max(np.abs(m.field(0))) < 1e-6


def example_model(oracle):
    """ExampleModel (pf/sdd_test.go:325-341): 'dconc/dt = conc^3 - conc + LAP conc', 16x16."""
    n = 16
    m = oracle.Model([n, n], 1)
    c3 = m.add_product([0], [3])
    m.add_term(0, 1.0, src_kind=oracle.SRC_DERIVED, src=c3)
    m.add_term(0, -1.0, implicit=True)
    m.add_term(0, 1.0, lap=1, implicit=True)
    f = np.where(np.arange(n * n) > 5, 0.1, 0.0)
    m.set_field(0, f)
    return m, f


def test_reverting_the_orientation_gives_the_same_path(oracle):
    orient = np.where(np.arange(256) > 5, -1.0, 1.0)
    runs = []
    for sign in (1.0, -1.0):
        m, _ = example_model(oracle)
        s = oracle.SDD(m)
        s.set_params(0.01)
        s.set_orientation(sign * orient)
        s.step(100)
        runs.append(m.field(0).copy())
    assert np.max(np.abs(runs[0] - runs[1])) < 1e-10


def nucleation_setup(n=64):
    init = box_blur(circle(n, 10))
    final = box_blur(circle(n, 15))
    field = box_blur(circle(n, 12))
    return init.ravel(), final.ravel(), field.ravel()


@pytest.mark.slow
def test_classical_nucleation_radius(oracle):
    """TestClassicalNucleation: phi^4 double well tilted by rho, gradient coefficient gamma; the
    dimer settles on the critical droplet, radius 2 sigma / rho with sigma = sqrt(gamma/2) 2/3."""
    n, gamma, rho = 64, 0.5, 0.05
    init, final, field = nucleation_setup(n)
    m = oracle.Model([n, n], 1)
    a = 3.0 * rho / 4.0
    mu = m.add_poly(0, [a, 1.0, -a, -1.0], [0, 1, 2, 3])  # (1 - phi^2)(phi + 3 rho/4)
    m.add_term(0, 1.0, src_kind=oracle.SRC_DERIVED, src=mu)
    m.add_term(0, gamma, lap=1, implicit=True)
    m.set_field(0, field)
    s = oracle.SDD(m)
    dt = 0.7
    s.set_params(dt, min_len=5e-6)
    s.init(init, final)
    s.step(int(1000.0 / dt))
    phi = m.field(0).real
    assert np.all(np.isfinite(phi))
    rc = 2.0 * math.sqrt(gamma / 2.0) * (2.0 / 3.0) / rho
    Rc = math.sqrt(np.sum(0.5 * (1.0 + phi)) / math.pi)
    assert abs(Rc - rc) <= 0.3
