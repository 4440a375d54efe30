"""Shrinking-dimer dynamics (pf/sdd.go) on the device against the oracle's SDD.

Cases from pf/sdd_test.go, run through the C ABI:
- TestDoubleWell (:68-108): 4x4, 'dconc/dt = conc - conc^3', the saddle at 0 (1e-6);
- TestRevertOrientationVector (:343-381) on ExampleModel (:325-341): v and -v agree (1e-10);
- TestClassicalNucleation (:165-271): the critical droplet radius 2 sigma / rho (0.3);
plus trajectory parity with the oracle (field, orientation and SDDMonitor; FP64 1e-10, or 1e-9 where
the dynamics amplify rounding, FP32 1e-4),
a two-field model, and the rejections.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def box_blur(a, width=2):
    c = width // 2 + 1
    out = np.zeros_like(a)
    cnt = 0
    for dy in range(-c, c + 1):
        for dx in range(-c, c + 1):
            if abs(dy) <= width and abs(dx) <= width:
                out += np.roll(np.roll(a, -dy, axis=0), -dx, axis=1)
                cnt += 1
    return out / cnt


def circle(n, radius):
    r, c = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = np.full((n, n), -1.0)
    a[(r - n // 2) ** 2 + (c - n // 2) ** 2 <= radius * radius] = 1.0
    return a


def test_double_well_saddle(oracle):
    import gopf_gb300 as G

    n = 4
    init = np.full(16, -1.0)
    final = np.full(16, 1.5)
    m = G.Model([n, n], "fp64", device=0)
    m.add_field("conc")
    m.add_equation("dconc/dt = conc - conc^3")
    m.init()
    dt = 0.1
    m.set_stepper("sdd", dt)
    m.upload(0, 0.5 * (init + final))
    m.sdd_init(init, final)
    m.sdd_set_params(init_length=0.1)
    nsteps = int(math.log(0.1 / 1e-7) / dt) + 1
    m.step(nsteps)
    assert np.max(np.abs(m.download(0).real)) < 1e-6
    o = oracle.Model([n, n], 1)
    o.add_term(0, 1.0, implicit=True)
    o.add_term(0, -1.0, src_kind=oracle.SRC_DERIVED, src=o.add_product([0], [3]))
    o.set_field(0, 0.5 * (init + final))
    s = oracle.SDD(o)
    s.set_params(dt)
    s.init(init, final)
    s.set_params(dt, init_len=0.1)
    s.step(nsteps)
    assert np.max(np.abs(m.download(0).real - o.field(0).real)) < 1e-12


def example_gpu(prec="fp64"):
    import gopf_gb300 as G

    m = G.Model([16, 16], prec, device=0)
    m.add_field("conc")
    m.add_equation("dconc/dt = conc^3 - conc + LAP conc")
    m.init()
    m.set_stepper("sdd", 0.01)
    m.upload(0, np.where(np.arange(256) > 5, 0.1, 0.0))
    return m


def example_oracle(O):
    o = O.Model([16, 16], 1)
    o.add_term(0, 1.0, src_kind=O.SRC_DERIVED, src=o.add_product([0], [3]))
    o.add_term(0, -1.0, implicit=True)
    o.add_term(0, 1.0, lap=1, implicit=True)
    o.set_field(0, np.where(np.arange(256) > 5, 0.1, 0.0))
    return o


def test_example_model_trajectory_and_monitor(oracle):
    orient = np.where(np.arange(256) > 5, -1.0, 1.0)
    m = example_gpu()
    m.sdd_set_orientation(orient)
    m.step(100)
    o = example_oracle(oracle)
    s = oracle.SDD(o)
    s.set_params(0.01)
    s.set_orientation(orient)
    s.step(100)
    assert rel(m.download(0).real, o.field(0).real) <= 1e-10
    assert rel(m.sdd_orientation(), s.orientation()) <= 1e-10
    mg, mo = m.sdd_monitor(), s.monitor()
    for k in ("max_force", "force_power_spectrum", "max_torque", "field_norm"):
        assert abs(mg[k] - mo[k]) <= 1e-9 * max(abs(mo[k]), 1e-12), k


def test_reverting_the_orientation_gives_the_same_path():
    orient = np.where(np.arange(256) > 5, -1.0, 1.0)
    runs = []
    for sign in (1.0, -1.0):
        m = example_gpu()
        m.sdd_set_orientation(sign * orient)
        m.step(100)
        runs.append(m.download(0))
    assert np.max(np.abs(runs[0] - runs[1])) < 1e-10


def nucleation_gpu(prec, gamma=0.5, rho=0.05, n=64):
    import gopf_gb300 as G

    init, final, field = (box_blur(circle(n, r)).ravel() for r in (10, 15, 12))
    m = G.Model([n, n], prec, device=0)
    m.add_field("phi")
    m.add_scalar("gamma", gamma)
    a = 3.0 * rho / 4.0
    m.register_function("MINUS_CHEM_POT", G.DER_POLY, "phi", [a, 1.0, -a, -1.0], [0, 1, 2, 3])
    m.add_equation("dphi/dt = MINUS_CHEM_POT + gamma*LAP phi")
    m.init()
    m.set_stepper("sdd", 0.7)
    m.upload(0, field)
    m.sdd_set_params(min_length=5e-6)
    m.sdd_init(init, final)
    return m, (init, final, field)


def nucleation_oracle(O, fields, gamma=0.5, rho=0.05, n=64):
    init, final, field = fields
    o = O.Model([n, n], 1)
    a = 3.0 * rho / 4.0
    o.add_term(0, 1.0, src_kind=O.SRC_DERIVED, src=o.add_poly(0, [a, 1.0, -a, -1.0], [0, 1, 2, 3]))
    o.add_term(0, gamma, lap=1, implicit=True)
    o.set_field(0, field)
    s = O.SDD(o)
    s.set_params(0.7, min_len=5e-6)
    s.init(init, final)
    return o, s


def test_example_model_fp32(oracle):
    orient = np.where(np.arange(256) > 5, -1.0, 1.0)
    m = example_gpu("fp32")
    m.sdd_set_orientation(orient)
    m.step(100)
    o = example_oracle(oracle)
    s = oracle.SDD(o)
    s.set_params(0.01)
    s.set_orientation(orient)
    s.step(100)
    assert rel(m.download_real(0), o.field(0).real) <= 1e-5
    assert rel(m.sdd_orientation(), s.orientation()) <= 1e-4


def test_nucleation_trajectory_parity(oracle):
    """150 steps of dt = 0.7 near the saddle amplify rounding: the oracle against itself with its
    start perturbed by 1e-16 (relative) differs by 3e-11 to 5e-11, hence 1e-9 here.  (FP32 is not
    run on this case: at MinDimerLength 5e-6 the dimer's ends differ by about 4e-8 per node,
    below FP32 resolution, and the torque is rounding noise.)"""
    m, fields = nucleation_gpu("fp64")
    m.step(150)
    o, s = nucleation_oracle(oracle, fields)
    s.step(150)
    assert rel(m.download_real(0), o.field(0).real) <= 1e-9
    assert rel(m.sdd_orientation(), s.orientation()) <= 1e-8


def test_classical_nucleation_radius():
    gamma, rho = 0.5, 0.05
    m, _ = nucleation_gpu("fp64")
    m.step(int(1000.0 / 0.7))
    phi = m.download_real(0)
    assert np.all(np.isfinite(phi))
    rc = 2.0 * math.sqrt(gamma / 2.0) * (2.0 / 3.0) / rho
    Rc = math.sqrt(np.sum(0.5 * (1.0 + phi)) / math.pi)
    assert abs(Rc - rc) <= 0.3, Rc
    assert m.sdd_dimer_length(1428 * 0.7) == pytest.approx(5e-6)


def test_two_field_model(oracle):
    """Two uniform fields (the potential of Test2DSurface, pf/sdd_test.go:110-151, on an 8x8
    grid): the device follows the oracle, including the reference's use of the first field's
    forces at the centre for every field."""
    import gopf_gb300 as G

    n = 64
    m = G.Model([8, 8], "fp64", device=0)
    m.add_field("xCrd")
    m.add_field("yCrd")
    m.add_scalar("FOUR", 4.0)
    m.add_scalar("TWO", 2.0)
    m.add_equation("dxCrd/dt = FOUR*xCrd - FOUR*xCrd^3")
    m.add_equation("dyCrd/dt = -TWO*yCrd")
    m.init()
    dt = 0.001
    m.set_stepper("sdd", dt)
    m.upload(0, np.full(n, 0.2))
    m.upload(1, np.full(n, 0.3))
    orient = np.concatenate([np.full(n, 0.1), np.full(n, 0.5)])
    m.sdd_set_orientation(orient)
    m.step(300)
    o = oracle.Model([8, 8], 2)
    o.set_field(0, np.full(n, 0.2))
    o.set_field(1, np.full(n, 0.3))
    o.add_term(0, 4.0, implicit=True)
    o.add_term(0, -4.0, src_kind=oracle.SRC_DERIVED, src=o.add_product([0], [3]))
    o.add_term(1, -2.0, implicit=True)
    s = oracle.SDD(o)
    s.set_params(dt)
    s.set_orientation(orient)
    s.step(300)
    for f in range(2):
        assert rel(m.download(f).real, o.field(f).real) <= 1e-10, f
    assert rel(m.sdd_orientation(), s.orientation()) <= 1e-10


def test_sdd_rejections():
    import gopf_gb300 as G

    m = example_gpu()
    with pytest.raises(G.GopfError) as e:
        m.step(1)  # no orientation yet
    assert e.value.status == 7
    m.sdd_set_orientation(np.ones(256))
    m.set_modal_filter(G.vandeven(4))
    with pytest.raises(G.GopfError) as e:
        m.step(1)  # SDD.SetFilter panics (pf/sdd.go:426-430)
    assert e.value.status == 6
    with pytest.raises(G.GopfError):
        m.sdd_set_orientation(np.ones(10))
