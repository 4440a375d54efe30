"""CPU restatement of ImplicitEuler.Step (pf/implicitEuler.go:165-207) on the FP64 oracle model.

Test infrastructure only: it checks the device's ImplicitEuler and is never on the product path.

Per step, with c_n the field, N_n = GetRHS(c_n) and L = GetDenum (both in k space):
  F(x) = x - Re(IFFT(FFT(c_n) e^(L dt) + I(L, N(x), N_n)) / N)        updateEquation, :68-94
  I(L, N, N_n) = N_n (f - 1)/L + (N - N_n)/dt (f - L dt - 1)/L^2,  f = e^(L dt);
               = dt/2 (N + N_n f) when |L| < 1e-5                   nonlinearIntegral, :151-162
The root of F is found from one explicit Euler step (:182-190).  The reference's solver
(github.com/davidkleiven/gononlin v0.2.2, Newton-Krylov with GMRES) is a third-party dependency
that is not in the reference tree; any Newton-Krylov solve to a tight tolerance finds the same root,
so this restatement uses scipy.optimize.newton_krylov with a max-norm tolerance.
"""
from __future__ import annotations

import numpy as np


def residual_fn(model, dims, dt: float):
    """F for the model's current field (which becomes c_n); model's field is left at c_n."""
    from oracle import oracle as O

    c = model.field(0).real.copy()
    n = c.size
    chat = O.fftn(c.astype(np.complex128), dims)
    nprev = model.eval_rhs(0)
    L = model.eval_denum(0)
    f = np.exp(L * dt)
    small = np.abs(L) < 1e-5
    Ls = np.where(small, 1.0, L)
    c1 = (f - 1.0) / Ls
    c2 = (f - L * dt - 1.0) / (Ls * Ls)

    def F(x):
        model.set_field(0, np.asarray(x, dtype=np.float64))
        nx = model.eval_rhs(0)
        integral = np.where(small, 0.5 * dt * (nx + nprev * f), nprev * c1 + (nx - nprev) / dt * c2)
        upd = chat * f + integral
        r = O.fftn(np.asarray(x, dtype=np.complex128), dims) - upd
        out = O.fftn(r, dims, sign=1).real / n
        model.set_field(0, c)
        return out

    return F, c


def implicit_euler_step(model, dims, dt: float, tol: float = 1e-12) -> dict:
    """One ImplicitEuler step of a single-field oracle model, in place.  Returns solver info."""
    from scipy.optimize import newton_krylov

    F, c = residual_fn(model, dims, dt)
    model.step_euler(dt, 1, hooks=False)
    x0 = model.field(0).real.copy()
    model.set_field(0, c)
    if np.max(np.abs(F(x0))) <= tol:
        x = x0
    else:
        x = newton_krylov(F, x0, method="gmres", f_tol=tol, maxiter=100)
    res = float(np.max(np.abs(F(x))))
    model.set_field(0, x)
    return {"residual": res}
