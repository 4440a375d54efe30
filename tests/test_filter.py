"""Modal filters (pf/vandeven.go, ApplyModalFilter pf/util.go:125-132, Euler/RK4 SetFilter).

CPU: the Vandeven table of the oracle and of the library reproduce TestVandeven
(pf/vandeven_test.go:8-40) and agree with each other.  GPU: Euler and RK4 with a Vandeven filter
against the FP64 oracle (FP64 mode to 1e-11, FP32 to 1e-4), and the 256-point kernels against the
generic ones with the filter on.
"""
import numpy as np
import pytest


@pytest.mark.parametrize("order", [3, 5, 10])
def test_vandeven_reference_points(oracle, order):
    import gopf_gb300 as G

    t_or = oracle.vandeven(order)
    t_lib = G.vandeven(order)
    assert np.max(np.abs(t_or - t_lib)) < 1e-14
    for x, y in [(0.0, 1.0), (0.5, 0.5), (1.0, 0.0)]:
        assert abs(oracle.filter_eval(t_or, x) - y) < 1e-4


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def ch_pair(oracle, dims, prec, table, stepper="euler", dt=0.1, fast=True, seed=0):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c0 = uniform_field(seed, n, 0.5, 0.05)
    g = G.Model(dims, prec, device=0)
    g.set_option(G._lib.OPT_FAST_KERNELS, int(fast))
    g.add_field("conc")
    g.add_scalar("gamma", 1.0)
    g.add_scalar("M", 1.0)
    g.add_scalar("m1", -1.0)
    g.add_equation("dconc/dt = M*LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    g.init()
    g.set_modal_filter(table)
    g.set_stepper(stepper, dt)
    g.upload(0, c0)
    o = None
    if oracle is not None:
        o = oracle.cahn_hilliard(dims, gamma=1.0, M=1.0)
        o.set_field(0, c0)
        o.set_filter(table)
    return g, o


@pytest.mark.gpu
@pytest.mark.parametrize("dims,steps", [([64, 64], 50), ([16, 16, 16], 20)])
def test_euler_with_filter_fp64(oracle, dims, steps):
    table = oracle.vandeven(5)
    g, o = ch_pair(oracle, dims, "fp64", table)
    g.step(steps)
    o.step_euler(0.1, steps)
    assert rel_l2(g.download_real(0), o.field(0).real) <= 1e-11
    # the filter changes the trajectory
    g2, _ = ch_pair(None, dims, "fp64", None)
    g2.step(steps)
    assert rel_l2(g2.download_real(0), o.field(0).real) > 1e-6


@pytest.mark.gpu
def test_rk4_with_filter_fp64(oracle):
    table = oracle.vandeven(3)
    g, o = ch_pair(oracle, [32, 32], "fp64", table, stepper="rk4")
    g.step(20)
    o.step_rk4(0.1, 20)
    assert rel_l2(g.download_real(0), o.field(0).real) <= 1e-11


@pytest.mark.gpu
def test_fast_2d_kernel_with_filter_fp32(oracle):
    """256^2 FP32: the 2D fused 256-point kernel applies the filter."""
    table = oracle.vandeven(5)
    g, o = ch_pair(oracle, [256, 256], "fp32", table)
    g.step(30)
    o.step_euler(0.1, 30)
    assert rel_l2(g.download_real(0), o.field(0).real) <= 1e-4


@pytest.mark.gpu
def test_fast_3d_kernels_with_filter_match_generic(oracle):
    table = oracle.vandeven(5)
    a, _ = ch_pair(None, [256, 256, 256], "fp32", table, dt=0.05, fast=True, seed=1)
    b, _ = ch_pair(None, [256, 256, 256], "fp32", table, dt=0.05, fast=False, seed=1)
    a.step(20)
    b.step(20)
    assert rel_l2(a.download_real(0), b.download_real(0)) <= 2e-6
