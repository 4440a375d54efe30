"""Adjoint of the semi-implicit Cahn-Hilliard step: C-ABI wrapper, a
torch.autograd.Function and a small parameter fit.

Model (Euler, pf/euler.go:16-47, for "dconc/dt = M*LAP MU - M*gamma*LAP^2 conc",
MU = conc^3 - conc):
    c_{n+1} = D (c_n - dt M K f(c_n)),  K = -lap,  D = (1 + dt M gamma K^2)^-1.
The device computes c_T and, given dL/dc_T, the gradients of L with respect
to gamma, M and c0 by the hand-written adjoint with checkpoint-and-recompute
(gopf_adjoint_forward / gopf_adjoint_backward).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import GopfError, Model, _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class AdjointCH:
    """Forward/backward runner on one device context."""

    def __init__(self, domain_size, precision: str = "fp32", dt: float = 0.05, nsteps: int = 200, every: int = 20,
                 device: int = 0):
        self.model = Model(domain_size, precision, device=device)
        self.model.add_field("conc")
        self.N = self.model.N
        self.dt, self.nsteps, self.every = dt, nsteps, every
        self._L = _lib.load()
        self._params = None

    def forward(self, c0, gamma: float, M: float) -> np.ndarray:
        c = np.ascontiguousarray(np.asarray(c0, dtype=np.float64).reshape(-1))
        out = np.empty(self.N, dtype=np.float64)
        rc = self._L.gopf_adjoint_forward(self.model.handle, float(gamma), float(M), self.dt, self.nsteps, self.every,
                                          _dp(c), _dp(out))
        if rc != 0:
            raise GopfError(rc, self._L.gopf_last_error(self.model.handle).decode())
        self._params = (float(gamma), float(M))
        return out

    def backward(self, lam_T):
        lam = np.ascontiguousarray(np.asarray(lam_T, dtype=np.float64).reshape(-1))
        dg, dm = ctypes.c_double(), ctypes.c_double()
        dc0 = np.empty(self.N, dtype=np.float64)
        rc = self._L.gopf_adjoint_backward(self.model.handle, _dp(lam), ctypes.byref(dg), ctypes.byref(dm), _dp(dc0))
        if rc != 0:
            raise GopfError(rc, self._L.gopf_last_error(self.model.handle).decode())
        return dg.value, dm.value, dc0

    def loss_and_grad(self, c0, gamma: float, M: float, target):
        cT = self.forward(c0, gamma, M)
        r = cT - np.asarray(target, dtype=np.float64).reshape(-1)
        loss = 0.5 * float(r @ r)
        dg, dm, dc0 = self.backward(r)
        return loss, dg, dm, dc0


def make_function():
    """torch.autograd.Function: (c0, gamma, M) -> c_T on the device, gradients by the adjoint."""
    import torch

    class CHSolve(torch.autograd.Function):
        @staticmethod
        def forward(fctx, c0, gamma, M, runner):
            cT = runner.forward(c0.detach().cpu().double().numpy(), float(gamma), float(M))
            fctx.runner = runner
            fctx.shape = c0.shape
            return torch.from_numpy(cT).to(c0.dtype).reshape(c0.shape)

        @staticmethod
        def backward(fctx, grad_out):
            dg, dm, dc0 = fctx.runner.backward(grad_out.detach().cpu().double().numpy())
            return (torch.from_numpy(dc0).reshape(fctx.shape).to(grad_out.dtype),
                    torch.tensor(dg, dtype=grad_out.dtype), torch.tensor(dm, dtype=grad_out.dtype), None)

    return CHSolve


def fit_gamma_m(runner: AdjointCH, c0, target, gamma0: float, M0: float, iters: int = 20, lr: float = 0.05,
                method: str = "adam"):
    """Fit gamma and M to a target microstructure on log-parameters.  method "adam": `iters` Adam
    steps of rate lr; "lbfgs": L-BFGS with a strong-Wolfe line search, at most `iters` loss and
    gradient evaluations (one forward and one adjoint each).  Returns the history of
    (loss, gamma, M), one entry per evaluation."""
    import torch

    CHSolve = make_function()
    p = torch.tensor([np.log(gamma0), np.log(M0)], dtype=torch.float64, requires_grad=True)
    c0t = torch.from_numpy(np.asarray(c0, dtype=np.float64).reshape(-1))
    tgt = torch.from_numpy(np.asarray(target, dtype=np.float64).reshape(-1))
    hist = []

    def closure():
        opt.zero_grad()
        g, m = torch.exp(p[0]), torch.exp(p[1])
        cT = CHSolve.apply(c0t, g, m, runner)
        loss = 0.5 * torch.sum((cT - tgt) ** 2)
        loss.backward()
        hist.append((float(loss.detach()), float(g.detach()), float(m.detach())))
        return loss

    if method == "lbfgs":
        opt = torch.optim.LBFGS([p], lr=1.0, max_iter=iters, max_eval=iters, history_size=10,
                                line_search_fn="strong_wolfe", tolerance_grad=1e-14, tolerance_change=1e-16)
        opt.step(closure)
    elif method == "adam":
        opt = torch.optim.Adam([p], lr=lr)
        for _ in range(iters):
            closure()
            opt.step()
    else:
        raise ValueError(f"unknown method {method}")
    return hist
