"""Restatement of the reference's adaptive explicit Runge-Kutta integrator (FP64).

TEST INFRASTRUCTURE ONLY: the checker for the GPU integrator, never the product.

Follows ``Explicit_RungeKutta`` in qutip/solver/integrator/explicit_rk.pyx with the
Verner-7 tableau (qutip/solver/integrator/verner7efficient.py) and the option
defaults of ``IntegratorVern7`` (qutip/solver/integrator/qutip_integrator.py:50-58).
The state is a flat complex128 vector; ``deriv(t, y)`` returns ``dy/dt``.
"""
from __future__ import annotations

import math

import numpy as np

from qutip_gb300 import vern7_tableau as T

AT_FRONT, INTERPOLATED, NORMAL = 2, 1, 0
TOO_MUCH_WORK, DT_UNDERFLOW, OUTSIDE_RANGE, NOT_INITIATED = -1, -2, -3, -4
MESSAGES = {
    TOO_MUCH_WORK: "Too much work done in one call. Try to increase the nsteps parameter "
                   "or increasing the tolerance.",
    DT_UNDERFLOW: "Step size becomes too small. Try increasing tolerance.",
    OUTSIDE_RANGE: "Step outside available range.",
    NOT_INITIATED: "Not initialized.",
}


class IntegrationError(Exception):
    pass


class Vern7:
    """``Explicit_RungeKutta`` (explicit_rk.pyx:47-530) with the Vern7 tableau."""

    def __init__(self, deriv, atol=1e-8, rtol=1e-6, nsteps=1000, first_step=0.0,
                 min_step=0.0, max_step=0.0, interpolate=True):
        self.deriv = deriv
        self.atol, self.rtol = atol, rtol
        self.max_numsteps = nsteps
        self.first_step = first_step
        self.min_step = min_step or 1e-15            # explicit_rk.pyx:133
        self.max_step = max_step
        self.interpolate = interpolate
        self.order = T.ORDER
        self.rk_step, self.rk_extra = T.RK_STEP, T.RK_EXTRA_STEP
        self.a = np.zeros((16, 16))
        for i, row in enumerate(T.A):
            self.a[i, :len(row)] = row
        self.b, self.c, self.e = np.array(T.B), np.array(T.C), np.array(T.E)
        self.bi = np.array(T.BI)
        self.dt_safe = atol
        self.y_prev = None
        self.status = NOT_INITIATED
        self.n_rhs = 0

    # explicit_rk.pyx:204-230
    def set_initial_value(self, y0, t):
        self.t = self.t_prev = self.t_front = t
        self.dt_int = 0.0
        self.y = np.array(y0, dtype=np.complex128)
        n = self.y.shape[0]
        self.k = [np.zeros(n, np.complex128) for _ in range(self.rk_extra if self.interpolate
                                                            else self.rk_step)]
        self.y_front = self.y.copy()
        self.y_prev = self.y.copy()
        self.status = NORMAL
        self.dt_safe = self._estimate_first_step(t, self.y) if not self.first_step \
            else self.first_step

    def _f(self, t, y):
        self.n_rhs += 1
        return self.deriv(t, y)

    # explicit_rk.pyx:232-276
    def _estimate_first_step(self, t, y0):
        norm = float(np.linalg.norm(y0))
        tol = self.atol + norm * self.rtol
        self.k[0] = self._f(t, y0)
        if norm <= self.atol:
            norm = 1
        tmp = float(np.linalg.norm(self.k[0]))
        fact = math.factorial(self.order)
        if tmp >= self.atol * 1e-6:
            dt1 = (tol * fact * norm ** self.order) ** (1 / (self.order + 1)) / tmp
        else:
            dt1 = (tol * fact) ** (1 / (self.order + 1)) * norm * 0.5
        t1 = t + dt1 / 100
        ytmp = y0 + (dt1 / 100) * self.k[0]
        self.k[1] = self._f(t1, ytmp)
        tmp = float(np.linalg.norm(self.k[1]))
        if tmp >= self.atol * 1e-6:
            dt2 = (tol * fact * norm ** self.order) ** (1 / (self.order + 1)) / tmp
        else:
            dt2 = dt1
        dt = min(dt1, dt2)
        if self.max_step:
            dt = min(self.max_step, dt)
        if self.min_step:
            dt = max(self.min_step, dt)
        return dt

    # explicit_rk.pyx:278-331
    def integrate(self, t, step=False):
        nsteps_left = self.max_numsteps
        if self.y_prev is None:
            self.status = NOT_INITIATED
            return
        if t == self.t:
            return
        if t < self.t_prev:
            self.status = OUTSIDE_RANGE
            return
        if self.interpolate and t < self.t_front:
            if self.status != INTERPOLATED:
                self._prep_dense_out()
                self.status = INTERPOLATED
            self.y = self._interpolate_step(t)
            self.t = t
            return
        self.status = NORMAL
        if step and self.t < self.t_front and t > self.t_front:
            t = self.t_front
        while self.t_front < t and self.status >= 0:
            self.y_prev = self.y_front.copy()
            self.t_prev = self.t_front
            nsteps_left -= self._step_in_err(t, nsteps_left)
            if step:
                break
        if self.status < 0:
            return
        if self.t_front > t:
            self._prep_dense_out()
            self.status = INTERPOLATED
            self.t = t
            self.y = self._interpolate_step(t)
        else:
            self.status = AT_FRONT
            self.t = self.t_front
            self.y = self.y_front.copy()

    # explicit_rk.pyx:333-356
    def _step_in_err(self, t, max_step):
        error = 1.0
        nsteps = 0
        while error >= 1:
            dt = self._get_timestep(t)
            error = self._compute_step(dt)
            self.dt_int = dt
            self._recompute_safe_step(error, dt)
            if dt == self.min_step and error > 1:
                self.status = DT_UNDERFLOW
                break
            nsteps += 1
            if nsteps > max_step:
                self.status = TOO_MUCH_WORK
                break
        return nsteps

    def _accumulate(self, target, factors, dt, size):
        # explicit_rk.pyx:432-437 with iadd_data skipping zero factors (:34-44)
        for i in range(size):
            f = dt * factors[i]
            if f != 0:
                target = target + f * self.k[i]
        return target

    # explicit_rk.pyx:358-389
    def _compute_step(self, dt):
        self.k[0] = self._f(self.t_prev, self.y_prev)
        for i in range(1, self.rk_step):
            ytmp = self._accumulate(self.y_prev.copy(), self.a[i], dt, i)
            self.k[i] = self._f(self.t_prev + self.c[i] * dt, ytmp)
        self.y_front = self._accumulate(self.y_prev.copy(), self.b, dt, self.rk_step)
        self.t_front = self.t_prev + dt
        return self._error(self.y_front, dt)

    # explicit_rk.pyx:391-397
    def _error(self, y_new, dt):
        diff = self._accumulate(np.zeros_like(y_new), self.e, dt, self.rk_step)
        return float(np.sqrt(np.mean((np.abs(diff) / (self.atol + self.rtol * np.abs(y_new))) ** 2)))

    # explicit_rk.pyx:399-410
    def _prep_dense_out(self):
        dt = self.dt_int
        for i in range(self.rk_step, self.rk_extra):
            ytmp = self._accumulate(self.y_prev.copy(), self.a[i], dt, i)
            self.k[i] = self._f(self.t_prev + self.c[i] * dt, ytmp)

    # explicit_rk.pyx:412-430
    def dense_factors(self, t):
        tau = (t - self.t_prev) / self.dt_int
        bf = np.zeros(self.rk_extra)
        for i in range(self.rk_extra):
            acc = 0.0
            for j in range(6, -1, -1):
                acc += self.bi[i, j]
                acc *= tau
            bf[i] = acc
        return bf

    def _interpolate_step(self, t):
        bf = self.dense_factors(t)
        return self._accumulate(self.y_prev.copy(), bf, self.dt_int, self.rk_extra)

    # explicit_rk.pyx:440-449
    def _get_timestep(self, t):
        dt_needed = t - self.t_prev
        if self.interpolate:
            return self.dt_safe
        if dt_needed <= self.dt_safe:
            return dt_needed
        return dt_needed / (int(dt_needed / self.dt_safe) + 1)

    # explicit_rk.pyx:451-467
    def _recompute_safe_step(self, err, dt):
        if err == 0:
            factor = 10.0
        else:
            factor = 0.9 * err ** (-1 / (self.order + 1))
            factor = min(10.0, factor)
            factor = max(0.2, factor)
        self.dt_safe = dt * factor
        if self.max_step:
            self.dt_safe = min(self.max_step, self.dt_safe)
        if self.min_step:
            self.dt_safe = max(self.min_step, self.dt_safe)

    def successful(self):
        return self.status >= 0

    def check(self):
        # qutip_integrator.py:89-92
        if not self.successful():
            raise IntegrationError(MESSAGES[self.status])
