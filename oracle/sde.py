"""Restatement of the reference's explicit Platen and Euler-Maruyama SODE steps (FP64, numpy).

TEST INFRASTRUCTURE ONLY: the checker for ``qg_sde_platen`` and ``qg_sde_euler``, never
the product.

Follows ``Platen.step`` (qutip/solver/sode/_sode.pyx:62-120) and ``Euler.step``
(_sode.pyx:32-55) on the drift and diffusion of ``StochasticClosedSystem``
(qutip/solver/sode/ssystem.pyx:141-166) and ``StochasticOpenSystem`` (ssystem.pyx:227-240),
in the same order of operations.  Pinned by tests/test_oracle_sde.py against the
reference's own ``run_from_experiment`` with a preset noise record (SSE Platen, SME Platen,
SSE and SME Euler: 1e-13 absolute per state entry).
"""
from __future__ import annotations

import numpy as np


def drift(L, C, M, x, open_):
    """ssystem.pyx:141-154 (closed) / 227-228 (open)."""
    out = L @ x
    if open_:
        return out
    for c, m in zip(C, M):
        e = np.vdot(x, m @ x)
        temp = c @ x
        out = out + (-0.125 * e * e) * x
        out = out + (0.5 * e) * temp
    return out


def diffusion(C, M, x, open_, d=None):
    """ssystem.pyx:156-166 (closed) / 230-240 (open: d = sqrt(len(x)))."""
    out = []
    for i, c in enumerate(C):
        v = c @ x
        if open_:
            dd = d or int(round(np.sqrt(len(x))))
            e = v[::dd + 1][:dd].sum()
            out.append(v + (-e) * x)
        else:
            e = np.vdot(x, M[i] @ x)
            out.append(v + (-0.5 * e) * x)
    return out


def platen_step(L, C, M, x, dW, dt, open_):
    """One step (_sode.pyx:62-120)."""
    m = len(C)
    sqrt_dt = np.sqrt(dt)
    sqrt_dt_inv = 0.25 / sqrt_dt
    d1 = x + dt * drift(L, C, M, x, open_)
    d2 = diffusion(C, M, x, open_)
    out = 0.5 * d1
    vt = d1.copy()
    vp, vm = [], []
    for i in range(m):
        vp.append(d1 + sqrt_dt * d2[i])
        vm.append(d1 + (-sqrt_dt) * d2[i])
        vt = vt + dW[i] * d2[i]
    out = out + (0.5 * dt) * drift(L, C, M, vt, open_)
    out = out + 0.5 * x
    for i in range(m):
        d2p = diffusion(C, M, vp[i], open_)
        d2m = diffusion(C, M, vm[i], open_)
        dw = dW[i] * 0.25
        out = out + (2 * dw) * d2[i]
        for j in range(m):
            if i == j:
                dw2 = sqrt_dt_inv * (dW[i] * dW[j] - dt)
                dw2p = dw2 + dw
                dw2m = -dw2 + dw
            else:
                dw2p = sqrt_dt_inv * dW[i] * dW[j]
                dw2m = -dw2p
            out = out + dw2p * d2p[j]
            out = out + dw2m * d2m[j]
    return out


def platen_steps(L, C, M, x, dW, dt, open_):
    """``len(dW)`` steps; ``dW[k]`` holds the increments of step k (one per operator)."""
    x = np.asarray(x, dtype=np.complex128)
    for k in range(len(dW)):
        x = platen_step(L, C, M, x, dW[k], dt, open_)
    return x


def euler_step(L, C, M, x, dW, dt, open_):
    """One Euler-Maruyama step (_sode.pyx:32-55)."""
    out = x + dt * drift(L, C, M, x, open_)
    d2 = diffusion(C, M, x, open_)
    for i in range(len(C)):
        out = out + dW[i] * d2[i]
    return out


def euler_steps(L, C, M, x, dW, dt, open_):
    x = np.asarray(x, dtype=np.complex128)
    for k in range(len(dW)):
        x = euler_step(L, C, M, x, dW[k], dt, open_)
    return x
