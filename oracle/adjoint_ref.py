"""FP64 numpy reference of the Cahn-Hilliard forward step and its adjoint.

Test infrastructure only (the reference computation for gopf_adjoint_*).  The forward step
restates Euler.Step (pf/euler.go:16-47) for "dconc/dt = M*LAP MU -
M*gamma*LAP^2 conc", MU = conc^3 - conc, with numpy's real FFTs; frequencies
follow Freq (pfutil/fftWrap.go:57-74): k^2 = (2 pi)^2 |f|^2.
"""
from __future__ import annotations

import numpy as np


def k2_grid(dims):
    dims = list(dims)
    if len(dims) == 2:
        fy = np.fft.fftfreq(dims[0])
        fx = np.fft.rfftfreq(dims[1])
        return (2 * np.pi) ** 2 * (fy[:, None] ** 2 + fx[None, :] ** 2)
    fz = np.fft.fftfreq(dims[2])
    fy = np.fft.fftfreq(dims[0])
    fx = np.fft.rfftfreq(dims[1])
    return (2 * np.pi) ** 2 * (fz[:, None, None] ** 2 + fy[None, :, None] ** 2 + fx[None, None, :] ** 2)


def _shape(dims):
    dims = list(dims)
    return tuple(dims) if len(dims) == 2 else (dims[2], dims[0], dims[1])


def forward(c0, dims, gamma, M, dt, nsteps, keep=False):
    sh = _shape(dims)
    k2 = k2_grid(dims)
    D = 1.0 / (1.0 + dt * M * gamma * k2 * k2)
    c = np.asarray(c0, dtype=np.float64).reshape(sh)
    traj = [c.ravel().copy()] if keep else None
    for _ in range(nsteps):
        f = c ** 3 - c
        ch = np.fft.rfftn(c)
        fh = np.fft.rfftn(f)
        c = np.fft.irfftn(D * (ch - dt * M * k2 * fh), s=sh)
        if keep:
            traj.append(c.ravel().copy())
    return (c.ravel(), traj) if keep else c.ravel()


def adjoint(c0, dims, gamma, M, dt, nsteps, lam_T):
    """Returns (dL/dgamma, dL/dM, dL/dc0) for the loss whose dL/dc_T is lam_T."""
    sh = _shape(dims)
    k2 = k2_grid(dims)
    D = 1.0 / (1.0 + dt * M * gamma * k2 * k2)
    _, traj = forward(c0, dims, gamma, M, dt, nsteps, keep=True)
    lam = np.asarray(lam_T, dtype=np.float64).reshape(sh)
    dg = dm = 0.0
    for n in range(nsteps - 1, -1, -1):
        cn = traj[n].reshape(sh)
        cn1 = traj[n + 1].reshape(sh)
        lh = np.fft.rfftn(lam)
        # <a, b> over real space = sum over the real spectrum with Hermitian weights / N
        N = cn.size
        w = np.full(lh.shape, 2.0)
        w[..., 0] = 1.0
        if sh[-1] % 2 == 0:
            w[..., -1] = 1.0
        c1h = np.fft.rfftn(cn1)
        fh = np.fft.rfftn(cn ** 3 - cn)
        s1 = np.sum(w * np.real(np.conj(lh) * k2 * k2 * D * c1h)) / N
        s2 = np.sum(w * np.real(np.conj(lh) * D * k2 * fh)) / N
        dg += -dt * M * s1
        dm += -dt * gamma * s1 - dt * s2
        mu = np.fft.irfftn(D * lh, s=sh)
        nu = np.fft.irfftn(D * k2 * lh, s=sh)
        lam = mu - dt * M * (3 * cn ** 2 - 1) * nu
    return dg, dm, lam.ravel()


def loss(c0, dims, gamma, M, dt, nsteps, target):
    r = forward(c0, dims, gamma, M, dt, nsteps) - np.asarray(target).ravel()
    return 0.5 * float(r @ r)
