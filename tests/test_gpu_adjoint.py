"""The device adjoint of the semi-implicit Cahn-Hilliard step (gopf_adjoint_*).

Checked against (i) the FP64 numpy reference adjoint in oracle/adjoint_ref.py
(itself checked against finite differences on the CPU), (ii) central finite
differences of the FP64 forward (h = 1e-4), tolerance 1e-3 for the FP32
adjoint, and (iii) a short gamma/M fit through the torch.autograd.Function.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(dims, seed=4):
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    return uniform_field(seed, n, 0.5 if len(dims) == 2 else 0.0, 0.05 if len(dims) == 2 else 0.1)


@pytest.mark.parametrize("dims,T,every", [([64, 64], 40, 7), ([16, 16, 16], 20, 6)])
def test_fp64_adjoint_matches_reference(dims, T, every):
    from gopf_gb300.adjoint import AdjointCH
    from oracle import adjoint_ref as A

    c0 = _setup(dims)
    dt = 0.05
    target = A.forward(c0, dims, 1.3, 0.8, dt, T)
    run = AdjointCH(dims, "fp64", dt=dt, nsteps=T, every=every)
    loss, dg, dm, dc0 = run.loss_and_grad(c0, 1.0, 1.0, target)
    cT = A.forward(c0, dims, 1.0, 1.0, dt, T)
    rg, rm, rc0 = A.adjoint(c0, dims, 1.0, 1.0, dt, T, cT - target)
    assert abs(loss - 0.5 * np.sum((cT - target) ** 2)) <= 1e-9 * loss
    assert abs(dg - rg) <= 1e-9 * abs(rg)
    assert abs(dm - rm) <= 1e-9 * abs(rm)
    assert np.linalg.norm(dc0 - rc0) <= 1e-9 * np.linalg.norm(rc0)


def test_fp32_adjoint_matches_finite_differences():
    """FP32 adjoint gradient vs central differences of the FP64 forward (h = 1e-4): 1e-3."""
    from gopf_gb300.adjoint import AdjointCH
    from oracle import adjoint_ref as A

    dims, T, dt = [128, 128], 100, 0.05
    c0 = _setup(dims)
    target = A.forward(c0, dims, 1.3, 0.8, dt, T)
    run = AdjointCH(dims, "fp32", dt=dt, nsteps=T, every=20)
    _, dg, dm, dc0 = run.loss_and_grad(c0, 1.0, 1.0, target)
    h = 1e-4
    fdg = (A.loss(c0, dims, 1.0 + h, 1.0, dt, T, target) - A.loss(c0, dims, 1.0 - h, 1.0, dt, T, target)) / (2 * h)
    fdm = (A.loss(c0, dims, 1.0, 1.0 + h, dt, T, target) - A.loss(c0, dims, 1.0, 1.0 - h, dt, T, target)) / (2 * h)
    assert abs(dg - fdg) <= 1e-3 * abs(fdg)
    assert abs(dm - fdm) <= 1e-3 * abs(fdm)
    v = np.random.default_rng(0).standard_normal(c0.size)
    fdc = (A.loss(c0 + h * v, dims, 1.0, 1.0, dt, T, target) - A.loss(c0 - h * v, dims, 1.0, 1.0, dt, T, target)) / (2 * h)
    assert abs(dc0 @ v - fdc) <= 1e-3 * abs(fdc)


def test_autograd_function_and_fit():
    """The torch.autograd.Function gives the adjoint's gradients, and a few Adam steps reduce the loss."""
    import torch

    from gopf_gb300.adjoint import AdjointCH, fit_gamma_m, make_function
    from oracle import adjoint_ref as A

    dims, T, dt = [64, 64], 40, 0.05
    c0 = _setup(dims)
    target = A.forward(c0, dims, 1.3, 0.8, dt, T)
    run = AdjointCH(dims, "fp64", dt=dt, nsteps=T, every=10)
    CHSolve = make_function()
    c0t = torch.from_numpy(c0.copy()).requires_grad_(True)
    g = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    m = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    cT = CHSolve.apply(c0t, g, m, run)
    loss = 0.5 * torch.sum((cT - torch.from_numpy(target)) ** 2)
    loss.backward()
    rg, rm, rc0 = A.adjoint(c0, dims, 1.0, 1.0, dt, T, cT.detach().numpy() - target)
    assert abs(g.grad.item() - rg) <= 1e-9 * abs(rg)
    assert abs(m.grad.item() - rm) <= 1e-9 * abs(rm)
    assert np.linalg.norm(c0t.grad.numpy() - rc0) <= 1e-9 * np.linalg.norm(rc0)
    hist = fit_gamma_m(run, c0, target, 1.0, 1.0, iters=8, lr=0.05)
    assert hist[-1][0] < hist[0][0]


def test_c5_configuration_fp32_adjoint_matches_finite_differences():
    """The adjoint-fit configuration: 512^2, 200 steps, dt 0.05, c0 = 0.5 + U(-0.05, 0.05) from seed 4,
    checkpoints every 20, target from the FP64 forward at gamma* = 1.3, M* = 0.8.  The FP32 adjoint's
    dL/dgamma, dL/dM and dL/dc0 . v against central differences (h = 1e-4) of the FP64 device forward
    (the oracle-matching form): 1e-3."""
    from gopf_gb300.adjoint import AdjointCH

    dims, T, dt, every = [512, 512], 200, 0.05, 20
    c0 = _setup(dims, seed=4)
    ref = AdjointCH(dims, "fp64", dt=dt, nsteps=T, every=every)
    target = ref.forward(c0, 1.3, 0.8)
    run = AdjointCH(dims, "fp32", dt=dt, nsteps=T, every=every)
    _, dg, dm, dc0 = run.loss_and_grad(c0, 1.0, 1.0, target)

    def L(c, g, m):
        r = ref.forward(c, g, m) - target
        return 0.5 * float(r @ r)

    h = 1e-4
    fdg = (L(c0, 1.0 + h, 1.0) - L(c0, 1.0 - h, 1.0)) / (2 * h)
    fdm = (L(c0, 1.0, 1.0 + h) - L(c0, 1.0, 1.0 - h)) / (2 * h)
    assert abs(dg - fdg) <= 1e-3 * abs(fdg)
    assert abs(dm - fdm) <= 1e-3 * abs(fdm)
    v = np.random.default_rng(5).standard_normal(c0.size)
    fdc = (L(c0 + h * v, 1.0, 1.0) - L(c0 - h * v, 1.0, 1.0)) / (2 * h)
    assert abs(dc0 @ v - fdc) <= 1e-3 * abs(fdc)


def test_c5_fit_recovers_gamma_and_m():
    """Fitting gamma and M at the adjoint configuration: the FP32 adjoint's gradients drive L-BFGS (on
    log-parameters, from gamma = M = 1) to gamma* = 1.3 and M* = 0.8 within 1 % in at most 30
    evaluations, with the loss down by a factor of 1e4."""
    from gopf_gb300.adjoint import AdjointCH, fit_gamma_m

    dims, T, dt, every = [512, 512], 200, 0.05, 20
    c0 = _setup(dims, seed=4)
    target = AdjointCH(dims, "fp64", dt=dt, nsteps=T, every=every).forward(c0, 1.3, 0.8)
    run = AdjointCH(dims, "fp32", dt=dt, nsteps=T, every=every)
    hist = fit_gamma_m(run, c0, target, 1.0, 1.0, iters=30, method="lbfgs")
    loss, g, m = min(hist)
    assert abs(g - 1.3) <= 0.01 * 1.3, hist[-5:]
    assert abs(m - 0.8) <= 0.01 * 0.8, hist[-5:]
    assert loss <= 1e-4 * hist[0][0]
