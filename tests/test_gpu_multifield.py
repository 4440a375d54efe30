"""Multi-field models on the device against the FP64 oracle.

pf.Model holds several fields; Euler.Step and RK4.Step (pf/euler.go:16-47,
pf/rk4.go:29-127) evolve field i with equation i, every right-hand side seeing
every field at the start of the step or stage.  Derived fields may multiply
powers of different fields (pf/util.go:38-65).  Cases:
- TestReactionDiffusion's model (pf/model_test.go:45-110), 2A + 3B <-> C, stepped
  in 2D and 3D, FP64 (rel-L2 <= 1e-11) and FP32 (<= 1e-5 after 40 steps);
- TestConcreteTerm's model (pf/rhsBuilder_test.go:95-110) on uniform fields, where
  one Euler step has a closed form (the known answers 16 and 8 of its RHS table);
- TestDerivedFieldOrder's model (pf/rhsBuilder_test.go:250-270): 'solute*cluster'
  is the derived field cluster*solute;
- a coupled Cahn-Hilliard / Allen-Cahn pair with a cross LAP term, Euler and RK4;
- per-field reductions, file IO and the rejections (ImplicitEuler, batches).

Euler.Step updates the fields in place one after the other, in k space, before
the inverse transforms (pf/euler.go:31-42).  A term that is another field
itself ("LAP conc" in the phi equation) therefore sees that field already
updated when it comes earlier in m.Fields; products (derived fields) were
synced at the start of the step.  RK4 forms every stage of every field first.
The oracle follows both orders; test_euler_updates_fields_in_order pins the
first in closed form.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RD = [
    "dconcA/dt = LAP concA - kf*concA^2*concB^3 + kr*concC",
    "dconcB/dt = LAP concB - kf*concA^2*concB^3 + kr*concC",
    "dconcC/dt = LAP concC - kr*concC + kf*concA^2*concB^3",
]


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rd_fields(n):
    from gopf_gb300.synthetic import uniform_field

    return [uniform_field(11, n, 0.5, 0.05), uniform_field(12, n, 0.5, 0.05), uniform_field(13, n, 0.3, 0.05)]


def rd_gpu(dims, prec, fields, stepper="euler", dt=0.01):
    import gopf_gb300 as G

    m = G.Model(dims, prec, device=0)
    for name in ("concA", "concB", "concC"):
        m.add_field(name)
    m.add_scalar("kf", 2.0)
    m.add_scalar("kr", 0.2)
    for eq in RD:
        m.add_equation(eq)
    m.init()
    m.set_stepper(stepper, dt)
    for f, d in enumerate(fields):
        m.upload(f, d)
    return m


def rd_oracle(O, dims, fields):
    """The reaction-diffusion model written out term by term (pf.Build's split)."""
    o = O.Model(dims, 3)
    for f, d in enumerate(fields):
        o.set_field(f, d)
    ab = o.add_product([0, 1], [2, 3])
    for eq in (0, 1):
        o.add_term(eq, 1.0, lap=1, implicit=True)
        o.add_term(eq, -2.0, src_kind=O.SRC_DERIVED, src=ab)
        o.add_term(eq, 0.2, src_kind=O.SRC_FIELD, src=2)
    o.add_term(2, 1.0, lap=1, implicit=True)
    o.add_term(2, -0.2, implicit=True)
    o.add_term(2, 2.0, src_kind=O.SRC_DERIVED, src=ab)
    return o


@pytest.mark.parametrize("dims,steps", [([64, 64], 40), ([48, 32], 30), ([16, 16, 16], 20)])
def test_reaction_diffusion_euler_fp64(oracle, dims, steps):
    n = int(np.prod(dims))
    fields = rd_fields(n)
    g = rd_gpu(dims, "fp64", fields)
    assert [g.summary(e) for e in range(3)] == [(2, 1), (2, 1), (1, 2)]
    g.step(steps)
    o = rd_oracle(oracle, dims, fields)
    o.step_euler(0.01, steps)
    for f in range(3):
        assert rel_l2(g.download(f).real, o.field(f).real) <= 1e-11, f


@pytest.mark.parametrize("dims", [[32, 32], [8, 8, 8]])
def test_reaction_diffusion_rk4_fp64(oracle, dims):
    n = int(np.prod(dims))
    fields = rd_fields(n)
    g = rd_gpu(dims, "fp64", fields, stepper="rk4", dt=0.02)
    g.step(15)
    o = rd_oracle(oracle, dims, fields)
    o.step_rk4(0.02, 15)
    for f in range(3):
        assert rel_l2(g.download(f).real, o.field(f).real) <= 1e-11, f


@pytest.mark.parametrize("dims", [[256, 256], [64, 64, 64]])
def test_reaction_diffusion_fp32(oracle, dims):
    """FP32 (the 256-point y pass serves the 2D update) against the FP64 oracle."""
    n = int(np.prod(dims))
    fields = rd_fields(n)
    g = rd_gpu(dims, "fp32", fields)
    g.step(40)
    o = rd_oracle(oracle, dims, fields)
    o.step_euler(0.01, 40)
    for f in range(3):
        assert rel_l2(g.download_real(f), o.field(f).real) <= 1e-5, f


def test_concrete_term_uniform_fields_one_step():
    """TestConcreteTerm's equations: on uniform fields only k = 0 is excited, so one Euler step
    is c + dt * RHS with RHS = voltage^2 = 16, resistance*current^2 = 8 and
    current*magnetic^3 = 6.75 (pf/rhsBuilder_test.go:95-150)."""
    import gopf_gb300 as G

    dims = [16, 16]
    n = 256
    m = G.Model(dims, "fp64", device=0)
    for name in ("current", "voltage", "magnetic"):
        m.add_field(name)
    m.add_scalar("resistance", 2.0)
    m.add_equation("dcurrent/dt = voltage^2")
    m.add_equation("dvoltage/dt = resistance*current^2")
    m.add_equation("dmagnetic/dt = current*magnetic^3")
    m.init()
    assert [m.summary(e) for e in range(3)] == [(1, 0), (1, 0), (1, 0)]
    m.set_stepper("euler", 0.1)
    for f, v in enumerate((2.0, -4.0, 1.5)):
        m.upload(f, np.full(n, v))
    m.step(1)
    for f, v in enumerate((2.0 + 0.1 * 16.0, -4.0 + 0.1 * 8.0, 1.5 + 0.1 * 6.75)):
        assert np.allclose(m.download(f).real, v, rtol=0, atol=1e-13), f


def test_derived_field_order_cluster_solute():
    """'dsolute/dt = solute*cluster' is explicit in the derived field cluster*solute
    (pf/rhsBuilder_test.go:250-270): with cluster = 1 and solute = 2 one step adds dt * 2."""
    import gopf_gb300 as G

    m = G.Model([8, 8], "fp64", device=0)
    m.add_field("cluster")
    m.add_field("solute")
    m.add_equation("dcluster/dt = LAP cluster")
    m.add_equation("dsolute/dt = solute*cluster")
    m.init()
    assert m.summary(1) == (1, 0)
    m.set_stepper("euler", 0.25)
    m.upload(0, np.ones(64))
    m.upload(1, np.full(64, 2.0))
    m.step(1)
    assert np.allclose(m.download(0).real, 1.0, atol=1e-14)
    assert np.allclose(m.download(1).real, 2.5, atol=1e-14)


def test_euler_updates_fields_in_order():
    """'da/dt = b', 'db/dt = a' on uniform fields, one Euler step: a reads the old b, b reads
    the new a (1 + dt*2), so b = 2 + dt*1.2 and not 2 + dt*1 (pf/euler.go:31-42)."""
    import gopf_gb300 as G

    m = G.Model([8, 8], "fp64", device=0)
    m.add_field("a")
    m.add_field("b")
    m.add_equation("da/dt = b")
    m.add_equation("db/dt = a")
    m.init()
    assert [m.summary(e) for e in range(2)] == [(1, 0), (1, 0)]
    m.set_stepper("euler", 0.1)
    m.upload(0, np.ones(64))
    m.upload(1, np.full(64, 2.0))
    m.step(1)
    assert np.allclose(m.download(0).real, 1.2, atol=1e-14)
    assert np.allclose(m.download(1).real, 2.12, atol=1e-14)


CHAC = [
    "dconc/dt = LAP conc^3 + m1*LAP conc + m1*LAP^2 conc + LAP conc*phi^2",
    "dphi/dt = -phi + phi^3 + phi*conc^2 + kappa*LAP phi + LAP conc",
]


def chac_gpu(dims, prec, fields, stepper, dt):
    import gopf_gb300 as G

    m = G.Model(dims, prec, device=0)
    m.add_field("conc")
    m.add_field("phi")
    m.add_scalar("m1", -1.0)
    m.add_scalar("kappa", 0.5)
    for eq in CHAC:
        m.add_equation(eq)
    m.init()
    m.set_stepper(stepper, dt)
    for f, d in enumerate(fields):
        m.upload(f, d)
    return m


def chac_oracle(O, dims, fields):
    o = O.Model(dims, 2)
    for f, d in enumerate(fields):
        o.set_field(f, d)
    c3 = o.add_product([0], [3])
    cphi2 = o.add_product([0, 1], [1, 2])
    phi3 = o.add_product([1], [3])
    phic2 = o.add_product([0, 1], [2, 1])
    o.add_term(0, 1.0, lap=1, src_kind=O.SRC_DERIVED, src=c3)
    o.add_term(0, -1.0, lap=1, implicit=True)
    o.add_term(0, -1.0, lap=2, implicit=True)
    o.add_term(0, 1.0, lap=1, src_kind=O.SRC_DERIVED, src=cphi2)
    o.add_term(1, -1.0, implicit=True)
    o.add_term(1, 1.0, src_kind=O.SRC_DERIVED, src=phi3)
    o.add_term(1, 1.0, src_kind=O.SRC_DERIVED, src=phic2)
    o.add_term(1, 0.5, lap=1, implicit=True)
    o.add_term(1, 1.0, lap=1, src_kind=O.SRC_FIELD, src=0)
    return o


@pytest.mark.parametrize("stepper", ["euler", "rk4"])
@pytest.mark.parametrize("dims", [[32, 32], [12, 12, 12]])
def test_coupled_cahn_hilliard_allen_cahn_fp64(oracle, dims, stepper):
    """Two fields, cross products in both equations and an explicit 'LAP conc' in the phi
    equation: the x-pass writes groups of LAP power 0 and 1 for both equations."""
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    fields = [uniform_field(21, n, 0.5, 0.05), uniform_field(22, n, 0.1, 0.05)]
    g = chac_gpu(dims, "fp64", fields, stepper, 0.02)
    assert [g.summary(e) for e in range(2)] == [(2, 2), (3, 2)]
    g.step(25)
    o = chac_oracle(oracle, dims, fields)
    if stepper == "euler":
        o.step_euler(0.02, 25)
    else:
        o.step_rk4(0.02, 25)
    for f in range(2):
        assert rel_l2(g.download(f).real, o.field(f).real) <= 1e-11, f


def test_multifield_graph_equals_eager():
    import gopf_gb300 as G

    dims = [32, 32]
    fields = rd_fields(32 * 32)
    a = rd_gpu(dims, "fp32", fields)
    b = rd_gpu(dims, "fp32", fields)
    b.set_option(G._lib.OPT_USE_GRAPHS, 0)
    a.step(21)
    b.step(21)
    for f in range(3):
        assert np.array_equal(a.download_real(f), b.download_real(f))


def test_per_field_mass_and_file_io(tmp_path):
    """gopf_reduce and SaveFloat64/LoadFloat64 address each field (pf/fileIO.go:45-97)."""
    import gopf_gb300 as G

    dims = [32, 32]
    fields = rd_fields(32 * 32)
    g = rd_gpu(dims, "fp64", fields)
    for f in range(3):
        assert abs(g.mass(f) - fields[f].sum()) <= 1e-12 * abs(fields[f].sum())
    g.step(5)
    p = str(tmp_path / "concB_5.bin")
    g.save_float64(p, field=1)
    raw = np.fromfile(p, dtype=">f8")
    assert np.array_equal(raw, g.download(1).real)
    h = rd_gpu(dims, "fp64", [np.zeros(1024)] * 3)
    h.load_float64(p, field=2)
    assert np.allclose(h.download(2).real, raw, atol=1e-15)
    assert np.all(h.download(0).real == 0.0)
    with pytest.raises(G.GopfError):
        g.save_float64(p, field=3)


def test_multifield_rejections():
    """Batches take single-field contexts; ImplicitEuler steps the three-field model (one
    Newton-Krylov solve over all fields)."""
    import gopf_gb300 as G

    fields = rd_fields(16 * 16)
    g = rd_gpu([16, 16], "fp64", fields, stepper="implicit_euler")
    g.step(1)
    assert g.newton_stats()[3]
    h = rd_gpu([16, 16], "fp64", fields)
    with pytest.raises(G.GopfError) as e:
        G.Batch([h])
    assert e.value.status == 6
