"""Restatement of the reference's mesolve / mcsolve drivers on top of ``oracle.vern7``.

TEST INFRASTRUCTURE ONLY: the checker for the GPU solvers, never the product.

* :func:`mesolve` follows ``Solver.run`` (qutip/solver/solver_base.py:159-226):
  integrate to each output time, restore the column-stacked state, normalise by
  the trace when the initial trace is 1 (``_restore_state``, :138-157) and take
  ``tr(op rho)`` per e_op (``_expect_csr_dense_dm``, qutip/core/data/expect.pyx:146-158).
* :func:`mc_trajectory` follows ``MCIntegrator`` (qutip/solver/mcsolve.py:228-418)
  with the option defaults of ``MCSolver`` (qutip/solver/mcsolve.py:449-466) and
  the per-trajectory generator ``numpy.random.default_rng(seed)``
  (qutip/solver/multitraj.py:382-393).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from .vern7 import Vern7

MC_DEFAULTS = dict(norm_steps=25, norm_t_tol=1e-6, norm_tol=1e-4, norm_min_step=0.1,
                   mc_corr_eps=1e-10)


def _coeff_fn(c):
    if c is None:
        return lambda t: 1.0
    return c


def make_deriv(terms):
    """``dy/dt = sum_k c_k(t) L_k y`` (``QobjEvo.matmul_data``, qobjevo.pyx:1103-1116)."""
    ops = [(sp.csr_matrix(op), _coeff_fn(c)) for op, c in terms]

    def deriv(t, y):
        out = np.zeros_like(y)
        for op, c in ops:
            out += c(t) * (op @ y)
        return out
    return deriv


def mesolve(terms, rho0_vec, tlist, e_ops, atol=1e-8, rtol=1e-6, nsteps=1000,
            return_states=False):
    ig = Vern7(make_deriv(terms), atol=atol, rtol=rtol, nsteps=nsteps)
    ig.set_initial_value(rho0_vec, tlist[0])
    d = int(round(np.sqrt(len(rho0_vec))))
    tr0 = np.trace(rho0_vec.reshape(d, d, order="F"))
    normalize = abs(tr0 - 1) <= 1e-12
    ops = [sp.csr_matrix(o) for o in e_ops]
    expect = np.zeros((len(ops), len(tlist)), dtype=np.complex128)
    states = []

    def record(i, y):
        rho = y.reshape(d, d, order="F")
        tr = np.trace(rho) if normalize else 1.0
        for k, op in enumerate(ops):
            expect[k, i] = (op.multiply(rho.T)).sum() / tr
        if return_states:
            states.append(y / tr)

    record(0, ig.y)
    for i, t in enumerate(tlist[1:], start=1):
        ig.integrate(t)
        ig.check()
        record(i, ig.y)
    return (expect, states, ig) if return_states else (expect, ig)


class MCTrajectory:
    """``MCIntegrator`` around :class:`oracle.vern7.Vern7` for one trajectory."""

    def __init__(self, heff_terms, c_ops, rng, atol=1e-8, rtol=1e-6, nsteps=1000, **opts):
        self.ig = Vern7(make_deriv(heff_terms), atol=atol, rtol=rtol, nsteps=nsteps)
        self.c_ops = [sp.csr_matrix(c) for c in c_ops]
        self.n_ops = [sp.csr_matrix(c.conj().T @ c) for c in self.c_ops]
        self.rng = rng
        self.opt = {**MC_DEFAULTS, **opts}
        self.collapses = []

    # mcsolve.py:245-281
    def set_state(self, t, psi):
        self.collapses = []
        self.target_norm = self.rng.random()
        self.ig.set_initial_value(psi, t)

    def _mcstep(self, t):
        # qutip_integrator.py:84-87 -> explicit_rk.pyx:278-331 with step=True
        self.ig.integrate(t, step=True)
        self.ig.check()
        return self.ig.t, self.ig.y

    @staticmethod
    def _prob(y):
        return float(np.linalg.norm(y)) ** 2

    # mcsolve.py:286-302
    def integrate(self, t):
        t_old, y_old = self.ig.t, self.ig.y
        norm_old = self._prob(y_old)
        while t_old < t:
            t_step, state = self._mcstep(t)
            norm = self._prob(state)
            if norm <= self.target_norm:
                t_col, state = self._find_collapse_time(norm_old, norm, t_old, t_step)
                self._do_collapse(t_col, state)
                t_old, y_old = self.ig.t, self.ig.y
                norm_old = 1.0
            else:
                t_old, y_old = t_step, state
                norm_old = norm
        return t_old, y_old / np.linalg.norm(y_old)

    # mcsolve.py:321-369
    def _find_collapse_time(self, norm_old, norm, t_prev, t_final):
        tries = 0
        cut = self.opt["norm_min_step"]
        while tries < self.opt["norm_steps"]:
            tries += 1
            if (t_final - t_prev) < self.opt["norm_t_tol"]:
                t_guess = t_final
                state = self.ig.y
                break
            dt = t_final - t_prev
            ratio = np.log(norm_old / self.target_norm) / np.log(norm_old / norm)
            if ratio < cut:
                ratio = cut
            if ratio > (1 - cut):
                ratio = 1 - cut
            t_guess = t_prev + dt * ratio
            if (t_guess - t_prev) < self.opt["norm_t_tol"]:
                t_guess = t_prev + self.opt["norm_t_tol"]
            _, state = self._mcstep(t_guess)
            norm2 = self._prob(state)
            if np.abs(self.target_norm - norm2) < self.opt["norm_tol"] * self.target_norm:
                break
            elif norm2 < self.target_norm:
                t_final = t_guess
                norm = norm2
            else:
                t_prev = t_guess
                norm_old = norm2
        if tries >= self.opt["norm_steps"]:
            raise RuntimeError("Could not find the collapse time within desired tolerance.")
        return t_guess, state.copy()

    # mcsolve.py:371-406
    def _do_collapse(self, t_col, state):
        num = len(self.n_ops)
        if num == 1:
            which = 0
        else:
            probs = [float(np.real(np.vdot(state, n @ state))) for n in self.n_ops]
            target = sum(probs) * self.rng.random() - probs[0]
            which = 0
            while target > 0 and which <= num:
                which += 1
                target -= probs[which]
        new = self.c_ops[which] @ state
        nn = np.linalg.norm(new)
        if nn < self.opt["mc_corr_eps"]:
            new = state / np.linalg.norm(state)
        else:
            new = new / nn
            self.collapses.append((t_col, which))
            self.target_norm = self.rng.random()
        self.ig.set_initial_value(new, t_col)


def mc_trajectory(heff_terms, c_ops, psi0, tlist, e_ops, seed, **opts):
    """Run one trajectory; returns ``(expect[n_e, n_t], collapses)``."""
    rng = np.random.default_rng(seed)
    tr = MCTrajectory(heff_terms, c_ops, rng, **opts)
    tr.set_state(tlist[0], np.asarray(psi0, dtype=np.complex128))
    ops = [sp.csr_matrix(o) for o in e_ops]
    ex = np.zeros((len(ops), len(tlist)), dtype=np.complex128)
    psi = np.asarray(psi0, dtype=np.complex128)
    for k, o in enumerate(ops):
        ex[k, 0] = np.vdot(psi, o @ psi)
    for i, t in enumerate(tlist[1:], start=1):
        _, psi = tr.integrate(t)
        for k, o in enumerate(ops):
            ex[k, i] = np.vdot(psi, o @ psi)
    return ex, list(tr.collapses)


def mesolve_matrix_form(h_terms, c_ops, rho0, tlist, e_ops, atol=1e-8, rtol=1e-6, nsteps=1000):
    """``mesolve`` with ``matrix_form=True`` (qutip/solver/mesolve.py:251-266): the state
    is rho itself (``_vectorize_state = False``) and the right-hand side
    ``LindbladMatrixForm.matmul_data`` (:func:`oracle.kernels.lindblad_matrix_form`).

    ``h_terms``: ``[(matrix, coefficient | None)]``; ``c_ops``: ``[(matrix, f | None)]``
    with ``f(t)`` the collapse operator's coefficient.  H_nh is formed as the reference
    does (lindblad_matrix_form.pyx:88-96).  Returns the e_op expectation values (traces,
    normalised when the initial trace is 1) at ``tlist``.
    """
    from .kernels import lindblad_matrix_form
    d = rho0.shape[0]
    hs = [(sp.csr_matrix(h), _coeff_fn(c)) for h, c in h_terms]
    cs = [(sp.csr_matrix(c), _coeff_fn(f)) for c, f in c_ops]

    def deriv(t, y):
        rho = y.reshape(d, d, order="F")
        h_nh = sum(c(t) * h for h, c in hs)
        for cm, f in cs:
            h_nh = h_nh - 0.5j * abs(f(t)) ** 2 * (cm.conj().T @ cm)
        cts = [f(t) * cm for cm, f in cs]
        return lindblad_matrix_form(h_nh, cts, rho).reshape(-1, order="F")

    ig = Vern7(deriv, atol=atol, rtol=rtol, nsteps=nsteps)
    ig.set_initial_value(np.asarray(rho0, dtype=np.complex128).reshape(-1, order="F"), tlist[0])
    normalize = abs(np.trace(rho0) - 1) <= 1e-12
    out = np.zeros((len(e_ops), len(tlist)), dtype=np.complex128)
    for i, t in enumerate(tlist):
        if i:
            ig.integrate(t)
            ig.check()
        rho = ig.y.reshape(d, d, order="F")
        tr = np.trace(rho) if normalize else 1.0
        for k, e in enumerate(e_ops):
            out[k, i] = np.trace(sp.csr_matrix(e) @ rho) / tr
    return out
