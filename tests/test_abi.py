"""CPU-only checks of the C ABI: the library loads, exports every entry point
of include/gopf_gpu.h, and its equation front end makes the same term split
as pf.Build (pf/rhsBuilder.go).  Host-only contexts (device = -1) compile
models without touching a GPU."""
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "gopf_gpu.h")).read()
    return sorted(set(re.findall(r"\b(gopf_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_header_symbol(gpulib):
    syms = _header_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(gpulib, s), s


def test_status_strings(gpulib):
    assert gpulib.gopf_status_string(0) == b"ok"
    assert gpulib.gopf_status_string(4) == b"non-finite value in field"


def _host_model(dims=(16, 16)):
    import gopf_gb300 as G

    return G.Model(list(dims), "fp32", device=-1)


def test_cahn_hilliard_string_split():
    """examples/cahnHilliard/main.go:33 -> 1 explicit (LAP conc^3) + 2 implicit terms."""
    m = _host_model()
    m.add_field("conc")
    m.add_scalar("gamma", 2.0)
    m.add_scalar("m1", -1.0)
    m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    m.init()
    assert m.summary(0) == (1, 2)
    terms = m.terms()
    expl = [t for t in terms if not t["implicit"]]
    impl = sorted([t for t in terms if t["implicit"]], key=lambda t: t["lap"])
    assert expl[0]["coef"] == 1.0 and expl[0]["lap"] == 1 and expl[0]["source"] == 2
    assert impl[0]["coef"] == -1.0 and impl[0]["lap"] == 1
    assert impl[1]["coef"] == -2.0 and impl[1]["lap"] == 2
    der = m.derived()
    assert der == [dict(kind=0, field=[0], power=[3], coef=[1.0])]


def test_term_diffusion_is_implicit():
    """TestTermDiffusion (pf/model_test.go:17-43): 'dconc/dt = LAP conc' -> 0 terms, 1 denominator."""
    m = _host_model((2, 2))
    m.add_field("conc")
    m.add_equation("dconc/dt = LAP conc")
    m.init()
    assert m.summary(0) == (0, 1)
    t = m.terms()[0]
    assert t["implicit"] == 1 and t["coef"] == 1.0 and t["lap"] == 1


def test_decay_strings():
    """pf/euler_test.go: 'rate*field' is bilinear (implicit); 'rate*field^2' is explicit with a derived field."""
    m = _host_model((8, 8))
    m.add_field("field")
    m.add_scalar("rate", -1.0)
    m.add_equation("dfield/dt = rate*field")
    m.init()
    assert m.summary(0) == (0, 1)
    assert m.terms()[0]["coef"] == -1.0
    m2 = _host_model((8, 8))
    m2.add_field("field")
    m2.add_scalar("rate", -1.0)
    m2.add_equation("dfield/dt = rate*field^2")
    m2.init()
    assert m2.summary(0) == (1, 0)
    assert m2.derived()[0]["power"] == [2]


def test_logistic_string():
    """pf/rk4_test.go:79 'field + rate*field^2' -> 1 implicit (+1) and 1 explicit (-field^2)."""
    m = _host_model((8, 8))
    m.add_field("field")
    m.add_scalar("rate", -1.0)
    m.add_equation("dfield/dt = field + rate*field^2")
    m.init()
    assert m.summary(0) == (1, 1)
    t = {bool(t["implicit"]): t for t in m.terms()}
    assert t[True]["coef"] == 1.0 and t[True]["lap"] == 0
    assert t[False]["coef"] == -1.0


def test_negative_sign_and_prefixes():
    """Signs from the preceding delimiter (pf/rhsBuilder.go:126-130) and LAP^2 powers."""
    m = _host_model()
    m.add_field("c")
    m.add_scalar("k", 0.5)
    m.add_equation("dc/dt = -k*LAP^2 c - LAP c^3")
    m.init()
    terms = m.terms()
    imp = [t for t in terms if t["implicit"]][0]
    exp_ = [t for t in terms if not t["implicit"]][0]
    assert imp["coef"] == -0.5 and imp["lap"] == 2
    assert exp_["coef"] == -1.0 and exp_["lap"] == 1


def test_registered_function_as_brick():
    """RegisterFunction (pf/model.go:400-412): 'LAP MU' uses the function as the term's field."""
    import gopf_gb300 as G

    m = _host_model()
    m.add_field("conc")
    m.add_scalar("mg", -0.5)
    m.register_function("MU", G.DER_POLY, "conc", [1.0, -1.0], [3, 1])
    m.add_equation("dconc/dt = LAP MU + mg*LAP^2 conc")
    m.init()
    terms = m.terms()
    assert m.summary(0) == (1, 1)
    e = [t for t in terms if not t["implicit"]][0]
    assert e["source"] == G.SRC_DERIVED and e["lap"] == 1
    assert m.derived()[0]["power"] == [3, 1]


def test_unknown_name_is_a_parse_error():
    """TestPanicOnUnknownName (pf/rhsBuilder_test.go:158): unknown names are rejected."""
    import gopf_gb300 as G

    m = _host_model()
    m.add_field("conc")
    m.add_equation("dconc/dt = foo*LAP conc^3")
    with pytest.raises(G.GopfError) as e:
        m.init()
    assert e.value.status == 8


def test_reserved_names_rejected():
    """panicOnPrefixInName (pf/model.go:480-485)."""
    import gopf_gb300 as G

    m = _host_model()
    with pytest.raises(G.GopfError):
        m.add_field("LAPconc")


def test_bad_leibniz():
    import gopf_gb300 as G

    m = _host_model()
    m.add_field("conc")
    with pytest.raises(G.GopfError):
        m.add_equation("conc = LAP conc")


def test_cubic_3d_only():
    import gopf_gb300 as G

    with pytest.raises(G.GopfError) as e:
        G.Model([16, 16, 32], "fp32", device=-1)
    assert e.value.status == 6


def test_lengths_with_prime_factors_above_seven_rejected():
    """Odd column counts are accepted (8 x 9 has a plan); a factor of 11 or 13 has none."""
    import gopf_gb300 as G

    G.Model([8, 9], "fp32", device=-1).close()
    G.Model([25, 49], "fp64", device=-1).close()
    for dims in ([8, 11], [13, 8], [22, 22]):
        with pytest.raises(G.GopfError) as e:
            G.Model(dims, "fp32", device=-1)
        assert e.value.status == 6


def test_freq_and_conjugate_node_host_only():
    m = _host_model((8, 8))
    from oracle import oracle as O

    for i in range(64):
        assert np.allclose(m.freq(i), O.freq([8, 8], i))
        assert m.conjugate_node(i) == O.conjugate_node([8, 8], i)


def test_stepping_needs_a_device():
    import gopf_gb300 as G

    m = _host_model()
    m.add_field("conc")
    m.add_equation("dconc/dt = LAP conc")
    m.init()
    m.set_stepper("euler", 0.1)
    with pytest.raises(G.GopfError) as e:
        m.upload(0, np.zeros(256))
    assert e.value.status == 7


def test_size_mismatch_is_an_argument_error():
    """NewSolver panics on inconsistent sizes (pf/solver.go:55-60); the ABI returns GOPF_ERR_ARG."""
    import ctypes

    import gopf_gb300 as G

    m = _host_model()
    m.add_field("conc")
    a = np.zeros(2 * 100)
    rc = m._L.gopf_field_upload(m.handle, 0, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 100)
    assert rc == 1


def test_reaction_diffusion_split():
    """TestReactionDiffusion (pf/model_test.go:45-110): three fields, the derived field
    concA^2*concB^3, and (terms, denominators) = (2, 1), (2, 1), (1, 2)."""
    import gopf_gb300 as G

    m = _host_model()
    for f in ("concA", "concB", "concC"):
        m.add_field(f)
    m.add_scalar("kf", 2.0)
    m.add_scalar("kr", 0.2)
    m.add_equation("dconcA/dt = LAP concA - kf*concA^2*concB^3 + kr*concC")
    m.add_equation("dconcB/dt = LAP concB - kf*concA^2*concB^3 + kr*concC")
    m.add_equation("dconcC/dt = LAP concC - kr*concC + kf*concA^2*concB^3")
    m.init()
    assert [m.summary(e) for e in range(3)] == [(2, 1), (2, 1), (1, 2)]
    assert m.derived() == [dict(kind=0, field=[0, 1], power=[2, 3], coef=[1.0, 1.0])]
    field_terms = [t for t in m.terms() if t["source"] == G.SRC_FIELD and not t["implicit"]]
    assert [(t["eq"], t["src_index"], t["coef"]) for t in field_terms] == [(0, 2, 0.2), (1, 2, 0.2)]


def test_concrete_term_and_factor_order_split():
    """TestConcreteTerm (pf/rhsBuilder_test.go:95-110) and the factor-order case at :250-270:
    products of other fields are explicit derived fields named in sorted factor order."""
    m = _host_model()
    for f in ("current", "voltage", "magnetic"):
        m.add_field(f)
    m.add_scalar("resistance", 2.0)
    m.add_equation("dcurrent/dt = voltage^2")
    m.add_equation("dvoltage/dt = resistance*current^2")
    m.add_equation("dmagnetic/dt = current*magnetic^3")
    m.init()
    assert [m.summary(e) for e in range(3)] == [(1, 0), (1, 0), (1, 0)]
    assert [(d["field"], d["power"]) for d in m.derived()] == [([1], [2]), ([0], [2]), ([0, 2], [1, 3])]
    m2 = _host_model()
    m2.add_field("cluster")
    m2.add_field("solute")
    m2.add_equation("dcluster/dt = LAP cluster")
    m2.add_equation("dsolute/dt = solute*cluster")
    m2.init()
    assert m2.summary(1) == (1, 0)
    assert m2.derived() == [dict(kind=0, field=[0, 1], power=[1, 1], coef=[1.0, 1.0])]


def test_multifield_limits():
    """Several fields compile on the host, the elastic and noise terms included; what the device
    does not step in multi-field models (two noise terms, more than four fields) is rejected at
    init."""
    import gopf_gb300 as G

    m = _host_model()
    m.add_field("conc")
    m.add_field("phase")
    m.register_elastic("LIN_ELAST", "phase", np.zeros((3, 3, 3, 3)), np.eye(3) * 0.01)
    m.add_equation("dconc/dt = LAP conc")
    m.add_equation("dphase/dt = LAP phase + LIN_ELAST")
    m.init()
    assert m.summary(1) == (1, 1)
    mn = _host_model()
    mn.add_field("conc")
    mn.add_field("phase")
    mn.register_noise("NOISE", "conservative", "phase", 1e-3, 1)
    mn.register_noise("NOISE2", "conservative", "conc", 1e-3, 2)
    mn.add_equation("dconc/dt = LAP conc + NOISE2")
    mn.add_equation("dphase/dt = LAP phase + NOISE")
    with pytest.raises(G.GopfError) as e:
        mn.init()
    assert e.value.status == 6
    m5 = _host_model()
    for i in range(5):
        m5.add_field(f"f{i}")
    for i in range(5):
        m5.add_equation(f"df{i}/dt = LAP f{i}")
    with pytest.raises(G.GopfError) as e:
        m5.init()
    assert e.value.status == 6
