"""Committed golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the FP64 oracle).

CPU tests: the synthetic generator still yields each case's initial field (checksum) and the oracle
still reproduces every fixture.  GPU tests: the device, through the C ABI, against the fixtures --
FP64 mode to rel-L2 <= 1e-11, FP32 mode to rel-L2 <= 1e-4 (the tolerances of the 128^2 and 256^3
Cahn-Hilliard configurations).
"""
import numpy as np
import pytest

from tests.golden import make_golden as MG


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", sorted(MG.CASES))
def test_fixture_initial_field_checksum(name):
    case = MG.CASES[name]
    _, sha = MG.load(name)
    assert MG.checksum(MG.initial_field(case)) == sha


@pytest.mark.parametrize("name", sorted(MG.CASES))
def test_oracle_reproduces_fixture(oracle, name):
    field, _ = MG.load(name)
    got = MG.run_oracle(oracle, MG.CASES[name])
    assert rel_l2(got, field) <= 1e-13


def gpu_model(case, prec):
    import gopf_gb300 as G

    dims, dt = case["dims"], case["dt"]
    c0 = MG.initial_field(case)
    m = G.Model(dims, prec, device=0)
    if case["kind"] in ("ch", "elastic"):
        m.add_field("conc")
        m.add_scalar("gamma", case["gamma"])
        m.add_scalar("M", case["M"])
        m.add_scalar("m1", -case["M"])
        eq = "dconc/dt = M*LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc"
        if case["kind"] == "elastic":
            m.register_elastic("LIN_ELAST", "conc", MG.cubic(1.0, 0.6, 0.5), np.eye(3) * 0.01)
            eq += " - LAP LIN_ELAST"
        m.add_equation(eq)
    else:
        m.add_field("phi")
        m.add_scalar("m1", -1.0)
        m.register_function("IND", G.DER_INDICATOR_D, "phi")
        m.register_volcons("CONSERVE", "phi", "IND", dt)
        m.add_equation("dphi/dt = m1*phi + CONSERVE + phi^2")
    m.init()
    m.set_stepper(case["stepper"], dt)
    m.upload(0, c0)
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MG.CASES))
def test_device_fp64_matches_fixture(name):
    field, _ = MG.load(name)
    case = MG.CASES[name]
    m = gpu_model(case, "fp64")
    m.step(case["steps"])
    assert rel_l2(m.download_real(0), field) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ch2d_128", "ch3d_32", "rk4_ch2d_64", "elastic3d_16"])
def test_device_fp32_matches_fixture(name):
    field, _ = MG.load(name)
    case = MG.CASES[name]
    m = gpu_model(case, "fp32")
    m.step(case["steps"])
    assert rel_l2(m.download_real(0), field) <= 1e-4
