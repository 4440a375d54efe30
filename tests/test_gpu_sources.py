"""Point sources (Model.AddSource, pf/model.go:152-154; Source.Eval, pf/sourceTerm.go:25-30).

A source adds f(t) exp(-2 pi i Freq . pos) to its equation's right-hand side; f is a Go closure,
here a table of its values per step, shared by the device and the oracle.  Cases: a diffusing
point source (closed form at step 1), Cahn-Hilliard with sources in 2D and 3D, FP64 (1e-11) and
FP32 (1e-5), RK4, a two-field model, an off-grid position (the real field keeps the Hermitian
part, so the oracle is projected onto its real part after every step), and the coverage check.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def amp_table(n, dt, a=1.0, b=0.5, w=3.0):
    t = np.arange(n) * dt
    return a + b * np.sin(w * t)


def ch_with_sources(G, dims, prec, dt, c0, sources, stepper="euler"):
    m = G.Model(dims, prec, device=0)
    m.add_field("conc")
    m.add_scalar("gamma", 0.5)
    m.add_scalar("m1", -1.0)
    m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    m.init()
    for pos, _ in sources:
        m.add_source(0, pos)
    m.set_stepper(stepper, dt)
    m.upload(0, c0)
    return m


def test_point_source_first_step_closed_form():
    """One Euler step of 'dconc/dt = LAP conc' from zero with a unit source at (row 3, col 5):
    the field is dt / (1 + dt k^2) in k space, i.e. a smoothed spike whose sum is dt."""
    import gopf_gb300 as G

    m = G.Model([16, 16], "fp64", device=0)
    m.add_field("conc")
    m.add_equation("dconc/dt = LAP conc")
    m.init()
    m.add_source(0, [3.0, 5.0])
    m.set_stepper("euler", 0.1)
    m.upload(0, np.zeros(256))
    m.set_source_amplitudes(np.ones((1, 4)))
    m.step(1)
    f = m.download(0).real.reshape(16, 16)
    fy, fx = np.meshgrid(np.fft.fftfreq(16), np.fft.fftfreq(16), indexing="ij")
    k2 = 4 * np.pi ** 2 * (fx ** 2 + fy ** 2)
    S = np.exp(-2j * np.pi * (fy * 3.0 + fx * 5.0))
    expect = np.fft.ifft2(0.1 * S / (1 + 0.1 * k2)).real
    assert np.max(np.abs(f - expect)) < 1e-14
    assert abs(f.sum() - 0.1) < 1e-13


@pytest.mark.parametrize("dims,prec,tol", [([32, 32], "fp64", 1e-11), ([16, 16, 16], "fp64", 1e-11),
                                           ([64, 64], "fp32", 1e-5)])
def test_cahn_hilliard_with_sources(oracle, dims, prec, tol):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    dt, steps = 0.05, 30
    c0 = uniform_field(31, n, 0.0, 0.1)
    pos = [[float(d // 4) for d in dims], [float(d // 2 + 1) for d in dims]]
    amps = np.stack([amp_table(steps, dt), -0.5 * amp_table(steps, dt, w=1.0)])
    g = ch_with_sources(G, dims, prec, dt, c0, list(zip(pos, amps)))
    g.set_source_amplitudes(amps)
    g.step(steps)
    o = oracle.cahn_hilliard(dims, gamma=0.5)
    o.set_field(0, c0)
    for p, a in zip(pos, amps):
        o.add_source(0, p, a)
    o.step_euler(dt, steps)
    assert rel_l2(g.download_real(0), o.field(0).real) <= tol


def test_rk4_with_source(oracle):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims, dt, steps = [32, 32], 0.02, 20
    c0 = uniform_field(32, 1024, 0.0, 0.1)
    amps = amp_table(steps, dt)[None, :]
    g = ch_with_sources(G, dims, "fp64", dt, c0, [([5.0, 9.0], amps[0])], stepper="rk4")
    g.set_source_amplitudes(amps)
    g.step(steps)
    o = oracle.cahn_hilliard(dims, gamma=0.5)
    o.set_field(0, c0)
    o.add_source(0, [5.0, 9.0], amps[0])
    o.step_rk4(dt, steps)
    assert rel_l2(g.download_real(0), o.field(0).real) <= 1e-11


def test_off_grid_source_keeps_the_hermitian_part(oracle):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims, dt, steps = [32, 32], 0.05, 20
    c0 = uniform_field(33, 1024, 0.0, 0.1)
    amps = amp_table(steps, dt)[None, :]
    pos = [7.3, 11.6]
    g = ch_with_sources(G, dims, "fp64", dt, c0, [(pos, amps[0])])
    g.set_source_amplitudes(amps)
    g.step(steps)
    o = oracle.cahn_hilliard(dims, gamma=0.5)
    o.set_field(0, c0)
    o.add_source(0, pos, amps[0])
    for _ in range(steps):
        o.step_euler(dt, 1)
        f = o.field(0)
        f[:] = f.real
    assert rel_l2(g.download_real(0), o.field(0).real) <= 1e-11


def test_source_in_a_two_field_model(oracle):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims, dt, steps = [32, 32], 0.02, 25
    a0, b0 = uniform_field(34, 1024, 0.5, 0.05), uniform_field(35, 1024, 0.2, 0.05)
    m = G.Model(dims, "fp64", device=0)
    m.add_field("a")
    m.add_field("b")
    m.add_equation("da/dt = LAP a - a*b^2")
    m.add_equation("db/dt = LAP b + a*b^2 - b")
    m.init()
    m.add_source(1, [10.0, 20.0])
    m.set_stepper("euler", dt)
    m.upload(0, a0)
    m.upload(1, b0)
    amps = amp_table(steps, dt)[None, :]
    m.set_source_amplitudes(amps)
    m.step(steps)
    o = oracle.Model(dims, 2)
    o.set_field(0, a0)
    o.set_field(1, b0)
    ab2 = o.add_product([0, 1], [1, 2])
    o.add_term(0, 1.0, lap=1, implicit=True)
    o.add_term(0, -1.0, src_kind=oracle.SRC_DERIVED, src=ab2)
    o.add_term(1, 1.0, lap=1, implicit=True)
    o.add_term(1, 1.0, src_kind=oracle.SRC_DERIVED, src=ab2)
    o.add_term(1, -1.0, implicit=True)
    o.add_source(1, [10.0, 20.0], amps[0])
    o.step_euler(dt, steps)
    for f in range(2):
        assert rel_l2(m.download(f).real, o.field(f).real) <= 1e-11, f


def test_steps_beyond_the_amplitude_table_are_refused():
    import gopf_gb300 as G

    m = ch_with_sources(G, [16, 16], "fp64", 0.05, np.zeros(256), [([1.0, 1.0], None)])
    with pytest.raises(G.GopfError) as e:
        m.step(1)  # no table yet
    assert e.value.status == 7
    m.set_source_amplitudes(np.ones((1, 3)))
    m.step(3)
    with pytest.raises(G.GopfError) as e:
        m.step(1)
    assert e.value.status == 7
    m.set_source_amplitudes(np.ones((1, 20)))
    m.step(20)  # graphs of 16 steps and single steps both read the table
    with pytest.raises(G.GopfError):
        m.set_source_amplitudes(np.ones((2, 3)))  # one row per source
