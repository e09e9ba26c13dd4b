"""Stochastic Schrodinger and master equations (``ssesolve`` / ``smesolve``) on the GPU.

The reference integrates one trajectory at a time with fixed-step SODE schemes, the
explicit Platen scheme by default (``PlatenSODE``, qutip/solver/sode/sode.py:235-251;
steps in qutip/solver/sode/_sode.pyx:58-120), drawing the Wiener increments of each
output interval from the trajectory's own generator (``Wiener.dW``,
qutip/solver/sode/_noise.py:22-30).  Here ``qg_sde_platen`` (``csrc/sde.cu``) runs all
the steps of an output interval in one launch, one warp or CTA per trajectory, with
increments drawn by the same ``Wiener`` object on the host: the trajectories are the
reference's, to rounding.  ``qg_sde_euler`` does the same with the Euler-Maruyama scheme
(``EulerSODE``, qutip/solver/sode/itotaylor.py:12-26).

:class:`SdeOperator` holds the drift and diffusion operators of one system on the device;
``IntegratorGpuPlaten`` / ``IntegratorGpuEuler`` in :mod:`qutip_gb300.qutip_plugin` are the
drop-in stochastic integrators (``method="gpu_platen"`` / ``"gpu_euler"``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from .operator import stream_ptr

__all__ = ["SdeOperator", "interval_steps", "SCHEMES"]

#: the reference's stochastic methods this module integrates, by name
SCHEMES = {"platen": "platen", "gpu_platen": "platen", "euler": "euler", "gpu_euler": "euler"}


def _csr_blocks(mats, device):
    """Row-stacked CSR (32-bit indices, complex128) of equally sized square matrices."""
    m = sp.csr_matrix(sp.vstack([sp.csr_matrix(a, dtype=np.complex128) for a in mats],
                                format="csr"))
    m.sort_indices()
    if m.nnz >= 2**31:
        raise ValueError("operator exceeds 32-bit indices")
    return (torch.from_numpy(m.indptr.astype(np.int32)).to(device),
            torch.from_numpy(m.indices.astype(np.int32)).to(device),
            torch.from_numpy(m.data.astype(np.complex128)).to(device))


class SdeOperator:
    """Drift and diffusion operators of a stochastic system (ssystem.pyx:119-250).

    ``open=False`` (ssesolve, kets of length d): ``L = -i H - 1/2 sum_i C_i^dag C_i``,
    ``C_i`` the stochastic operators, ``M_i = C_i + C_i^dag`` for their expectation values.
    ``open=True`` (smesolve, column-stacked rho of length d*d): ``L`` the Liouvillian of H,
    the stochastic and the deterministic collapse operators, ``C_i = spre(c_i) +
    spost(c_i^dag)``.  All matrices are scipy / numpy arrays (constant operators)."""

    def __init__(self, L, C_ops, M_ops=None, *, open: bool, d: int, device="cuda"):
        self.device = torch.device(device)
        self.open = bool(open)
        self.d = int(d)
        self.n = self.d * self.d if self.open else self.d
        self.n_sc = len(C_ops)
        if self.n_sc < 1 or self.n_sc > _lib.QG_MAX_COPS:
            raise ValueError(f"1..{_lib.QG_MAX_COPS} stochastic operators")
        if L.shape != (self.n, self.n) or any(c.shape != (self.n, self.n) for c in C_ops):
            raise ValueError("operators must act on the state vector")
        self.L = _csr_blocks([L], self.device)
        self.C = _csr_blocks(C_ops, self.device)
        self.M = _csr_blocks(M_ops, self.device) if not self.open else None
        if not self.open and (M_ops is None or len(M_ops) != self.n_sc):
            raise ValueError("the stochastic Schrodinger equation needs M_i = C_i + C_i^dag")
        self._work = None
        self._n_work = 0
        st = _lib.Sde()
        st.n, st.open, st.n_sc, st.d, st.reserved = self.n, int(self.open), self.n_sc, self.d, 0
        st.l_rp, st.l_col, st.l_val = (t.data_ptr() for t in self.L)
        st.c_rp, st.c_col, st.c_val = (t.data_ptr() for t in self.C)
        if self.M is not None:
            st.m_rp, st.m_col, st.m_val = (t.data_ptr() for t in self.M)
        self.struct = st

    @classmethod
    def sse(cls, H, sc_ops, device="cuda"):
        """ssesolve's system from H and the stochastic operators (StochasticClosedSystem,
        ssystem.pyx:131-139)."""
        H = sp.csr_matrix(H, dtype=np.complex128)
        cs = [sp.csr_matrix(c, dtype=np.complex128) for c in sc_ops]
        L = -1j * H
        for c in cs:
            L = L + (-0.5) * (c.conj().T @ c)
        return cls(L, cs, [c + c.conj().T for c in cs], open=False, d=H.shape[0], device=device)

    def _workspace(self, n_traj):
        need = int(_lib.load().qg_sde_work_values(self.n, self.n_sc)) * n_traj
        if self._work is None or self._n_work < need:
            self._work = torch.empty(need, dtype=torch.complex128, device=self.device)
            self._n_work = need
            self.struct.work = self._work.data_ptr()
        return self._work

    def advance(self, states: torch.Tensor, dW: torch.Tensor, n_steps: int, dt: float,
                scheme: str = "platen"):
        """``n_steps`` steps of every trajectory in ``states`` (n_traj x n, complex128, in
        place) with increments ``dW`` (n_traj x n_steps x n_sc, float64): the Platen scheme,
        or ``scheme="euler"`` for Euler-Maruyama."""
        n_traj = states.shape[0] if states.dim() == 2 else 1
        if states.dtype != torch.complex128 or states.numel() != n_traj * self.n:
            raise ValueError("states must be n_traj x n complex128")
        if dW.dtype != torch.float64 or dW.numel() != n_traj * n_steps * self.n_sc:
            raise ValueError("dW must be n_traj x n_steps x n_sc float64")
        if scheme not in ("platen", "euler"):
            raise ValueError("scheme must be 'platen' or 'euler'")
        self._workspace(n_traj)
        _lib.call(f"qg_sde_{scheme}", C.byref(self.struct), int(n_traj), states.data_ptr(),
                  dW.data_ptr(), int(n_steps), float(dt), stream_ptr())


def interval_steps(tlist, dt):
    """Fixed steps of each output interval as the reference's explicit SODE integrators
    count them (``_Explicit_Simple_Integrator.integrate``, qutip/solver/sode/sode.py:151-173):
    ``N`` whole steps of ``dt`` to the next output time, one more when the remainder exceeds
    half a step, none when the interval is under half a step; the integrator's time advances
    by ``dt * N``.  Returns the list of ``N`` (one per interval)."""
    steps, t_cur = [], float(tlist[0])
    for t in tlist[1:]:
        delta = float(t) - t_cur
        if delta < 0.5 * dt:
            steps.append(0)
            continue
        n, extra = np.divmod(delta, dt)
        n = int(n) + (1 if extra > 0.5 * dt else 0)
        steps.append(n)
        t_cur += dt * n
    return steps
