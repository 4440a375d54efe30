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
    """F over x = [field 0 | field 1 | ...] for the model's current fields (which become c_n): every
    equation's right-hand side is evaluated from all fields of x (updateEquation, :68-94).  The
    model's fields are left at c_n."""
    from oracle import oracle as O

    nf = model.nfields
    cs = [model.field(f).real.copy() for f in range(nf)]
    n = cs[0].size
    chats = [O.fftn(c.astype(np.complex128), dims) for c in cs]
    nprevs = [model.eval_rhs(e) for e in range(nf)]
    parts = []
    for e in range(nf):
        L = model.eval_denum(e)
        f = np.exp(L * dt)
        small = np.abs(L) < 1e-5
        Ls = np.where(small, 1.0, L)
        parts.append((f, small, (f - 1.0) / Ls, (f - L * dt - 1.0) / (Ls * Ls)))

    def F(x):
        xs = np.asarray(x, dtype=np.float64).reshape(nf, n)
        for fi in range(nf):
            model.set_field(fi, xs[fi])
        out = []
        for e in range(nf):
            f, small, c1, c2 = parts[e]
            nx = model.eval_rhs(e)
            nprev = nprevs[e]
            integral = np.where(small, 0.5 * dt * (nx + nprev * f), nprev * c1 + (nx - nprev) / dt * c2)
            upd = chats[e] * f + integral
            r = O.fftn(xs[e].astype(np.complex128), dims) - upd
            out.append(O.fftn(r, dims, sign=1).real / n)
        for fi in range(nf):
            model.set_field(fi, cs[fi])
        return np.concatenate(out)

    return F, cs[0] if nf == 1 else cs


def implicit_euler_step(model, dims, dt: float, tol: float = 1e-12) -> dict:
    """One ImplicitEuler step of an oracle model (all its fields), in place.  Returns solver info."""
    from scipy.optimize import newton_krylov

    nf = model.nfields
    F, _ = residual_fn(model, dims, dt)
    cs = [model.field(f).real.copy() for f in range(nf)]
    model.step_euler(dt, 1, hooks=False)
    x0 = np.concatenate([model.field(f).real.copy() for f in range(nf)])
    for f in range(nf):
        model.set_field(f, cs[f])
    if np.max(np.abs(F(x0))) <= tol:
        x = x0
    else:
        x = newton_krylov(F, x0, method="gmres", f_tol=tol, maxiter=100)
    res = float(np.max(np.abs(F(x))))
    xs = np.asarray(x).reshape(nf, -1)
    for f in range(nf):
        model.set_field(f, xs[f])
    return {"residual": res}
