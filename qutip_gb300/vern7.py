"""Adaptive Verner-7 integrator on the GPU for one (large) system.

The control flow mirrors ``Explicit_RungeKutta`` (qutip/solver/integrator/explicit_rk.pyx:47-530)
step for step -- first-step estimate, ``integrate`` with ``step=True`` for
Monte-Carlo stepping, ``_step_in_err`` retries, interpolation past the target
with the 7th-order dense output -- so that the step sequence, and therefore the
result, is the reference's.  The vector work runs in three kinds of launches:

* ``qg_vern7_stage`` -- one per stage: the matvec ``k_s = A(t_s) x_s`` fused
  with the next stage's input combination; the tenth fuses ``y_front`` and the
  FP64 WRMS error reduction (``wrmn_error_dense``, qutip/core/data/ode.pyx:27-52);
* ``qg_rk_combine`` -- dense-output stage input and materialised outputs;
* ``qg_norm2`` -- norms of the first-step estimate.

Precision forms: ``"double"`` (complex128 operator, stages and state),
``"mixed"`` (complex64 operator and stages with FP32 matvec accumulation, the
state ``y``, the stage combinations and the error control in FP64) and
``"single"`` (complex64 state as well; error control still FP64).  The scalar
step-size recurrences run on the host in IEEE double; the only per-step
device-to-host transfer is the 8-byte error norm.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from . import vern7_tableau as T
from .operator import DeviceOperator, qg_dtype, stream_ptr, torch_dtype

AT_FRONT, INTERPOLATED, NORMAL = 2, 1, 0
TOO_MUCH_WORK, DT_UNDERFLOW, OUTSIDE_RANGE, NOT_INITIATED = -1, -2, -3, -4
STATUS_MESSAGES = {
    AT_FRONT: "Internal state at the desired time.",
    INTERPOLATED: "Internal state past the desired time and interpolation to step done.",
    NORMAL: "No work done.",
    TOO_MUCH_WORK: ("Too much work done in one call. Try to increase the nsteps parameter or "
                    "increasing the tolerance."),
    DT_UNDERFLOW: "Step size becomes too small. Try increasing tolerance.",
    OUTSIDE_RANGE: "Step outside available range.",
    NOT_INITIATED: "Not initialized.",
}
PRECISIONS = {"double": ("c128", "c128"), "mixed": ("c128", "c64"), "single": ("c64", "c64")}


class IntegratorError(RuntimeError):
    """Integration failure; the plugin layer re-raises it as ``IntegratorException``."""


class GpuVern7:
    """Single-system adaptive Vern7 on device buffers.

    ``op`` is a :class:`DeviceOperator` or a
    :class:`~qutip_gb300.lindblad.LindbladOperator` whose dtype is the stage dtype
    of ``precision``.
    """

    def __init__(self, op: DeviceOperator, atol=1e-8, rtol=1e-6, nsteps=1000, first_step=0.0,
                 min_step=0.0, max_step=0.0, interpolate=True, precision="double"):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self.state_dt, self.stage_dt = PRECISIONS[precision]
        if op.dtype != self.stage_dt:
            raise TypeError(f"precision {precision!r} needs a {self.stage_dt} operator")
        if op.n_rows != op.n_cols:
            raise ValueError("the generator must be square")
        self.op = op
        self.precision = precision
        self.atol, self.rtol = float(atol), float(rtol)
        self.max_numsteps = int(nsteps)
        self.first_step = float(first_step)
        self.min_step = float(min_step) or 1e-15       # explicit_rk.pyx:133
        self.max_step = float(max_step)
        self.interpolate = bool(interpolate)
        self.order = T.ORDER
        self.a = np.zeros((16, 16))
        for i, row in enumerate(T.A):
            self.a[i, :len(row)] = row
        self.b, self.c, self.e, self.bi = np.array(T.B), np.array(T.C), np.array(T.E), np.array(T.BI)
        n = op.n_rows
        self.n = n
        dev = op.device
        sdt, kdt = torch_dtype(self.state_dt), torch_dtype(self.stage_dt)
        self._ya = torch.zeros(n, dtype=sdt, device=dev)
        self._yb = torch.zeros(n, dtype=sdt, device=dev)
        self.y_out = torch.zeros(n, dtype=sdt, device=dev)
        self.k = torch.zeros(16 * n, dtype=kdt, device=dev)
        self.ytmp = torch.zeros(2 * n, dtype=kdt, device=dev)
        self.scratch = torch.zeros(int(_lib.load().qg_scratch_doubles()), dtype=torch.float64,
                                   device=dev)
        self.counter = torch.zeros(4, dtype=torch.int32, device=dev)
        self.result = torch.zeros(4, dtype=torch.float64, device=dev)
        self._host = torch.zeros(4, dtype=torch.float64).pin_memory()
        self.y_prev, self.y_front = self._ya, self._yb
        # mixed form: complex64 copies of y_prev / y_front (stage inputs), swapped with them
        self.mixed = self.state_dt != self.stage_dt
        if self.mixed:
            self.y_prev_s = torch.zeros(n, dtype=kdt, device=dev)
            self.y_front_s = torch.zeros(n, dtype=kdt, device=dev)
        else:
            self.y_prev_s = self.y_front_s = None
        self._set = False
        self.status = NOT_INITIATED
        self.stats = {"steps": 0, "rejected": 0, "rhs": 0}
        self._out = ("front", None)  # how the state at self.t is obtained

    # -- buffers ---------------------------------------------------------
    def _rk(self) -> _lib.RkBuffers:
        ps = self.y_prev_s.data_ptr() if self.mixed else None
        fs = self.y_front_s.data_ptr() if self.mixed else None
        return _lib.RkBuffers(self.n, qg_dtype(self.state_dt), qg_dtype(self.stage_dt),
                              self.y_prev.data_ptr(), self.y_front.data_ptr(), ps, fs,
                              self.k.data_ptr(), self.ytmp.data_ptr(), self.scratch.data_ptr(),
                              self.counter.data_ptr(), self.result.data_ptr())

    def _swap(self):
        self.y_prev, self.y_front = self.y_front, self.y_prev
        if self.mixed:
            self.y_prev_s, self.y_front_s = self.y_front_s, self.y_prev_s

    def _view(self, base: torch.Tensor, factors=()) -> _lib.StateView:
        f = (C.c_double * 16)(*([float(x) for x in factors] + [0.0] * (16 - len(factors))))
        return _lib.StateView(self.n, qg_dtype(self.state_dt if base.dtype == torch_dtype(
            self.state_dt) else self.stage_dt), qg_dtype(self.stage_dt), base.data_ptr(),
            self.k.data_ptr(), len(factors), 0, f)

    def _combine(self, base, factors, out):
        v = self._view(base, factors)
        _lib.call("qg_rk_combine", C.byref(v), out.data_ptr(),
                  qg_dtype("c128" if out.dtype == torch.complex128 else "c64"), stream_ptr())

    def _read_result(self) -> float:
        self._host[:1].copy_(self.result[:1], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return float(self._host[0])

    def _norm(self, x: torch.Tensor) -> float:
        _lib.call("qg_norm2", x.data_ptr(), qg_dtype("c128" if x.dtype == torch.complex128 else "c64"),
                  x.numel(), self.scratch.data_ptr(), self.counter.data_ptr(),
                  self.result.data_ptr(), stream_ptr())
        return math.sqrt(self._read_result())

    def _k(self, j) -> torch.Tensor:
        return self.k[j * self.n:(j + 1) * self.n]

    def _ytmp(self, j) -> torch.Tensor:
        return self.ytmp[j * self.n:(j + 1) * self.n]

    def _deriv_into(self, t, x_stage: torch.Tensor, j: int):
        self.op.matvec(t, x_stage, self._k(j))
        self.stats["rhs"] += 1

    # -- reference algorithm ----------------------------------------------
    def set_initial_value(self, y0, t: float):
        """``set_initial_value`` (explicit_rk.pyx:204-230); copies ``y0``."""
        y0 = torch.as_tensor(y0)
        if y0.numel() != self.n:
            raise ValueError(f"state of size {y0.numel()} for a generator of size {self.n}")
        self.y_prev.copy_(y0.reshape(-1).to(self.y_prev.device, self.y_prev.dtype))
        self.y_front.copy_(self.y_prev)
        if self.mixed:
            self._combine(self.y_prev, (), self.y_prev_s)
            self.y_front_s.copy_(self.y_prev_s)
        self.t = self.t_prev = self.t_front = float(t)
        self.dt_int = 0.0
        self._out = ("front", None)
        self.status = NORMAL
        self._set = True
        self.dt_safe = self._estimate_first_step(self.t, self.y_prev) if not self.first_step \
            else self.first_step

    def _stage_input(self, y: torch.Tensor) -> torch.Tensor:
        if y.dtype == torch_dtype(self.stage_dt):
            return y
        self._combine(y, (), self._ytmp(0))
        return self._ytmp(0)

    def _stage_base(self) -> torch.Tensor:
        """Base of the stage combinations: y_prev, or its complex64 copy when mixed."""
        return self.y_prev_s if self.mixed else self.y_prev

    def _estimate_first_step(self, t, y0):
        # explicit_rk.pyx:232-276
        norm = self._norm(y0)
        tol = self.atol + norm * self.rtol
        self._deriv_into(t, self._stage_input(y0), 0)
        if norm <= self.atol:
            norm = 1
        tmp = self._norm(self._k(0))
        fact = math.factorial(self.order)
        if tmp >= self.atol * 1e-6:
            dt1 = (tol * fact * norm ** self.order) ** (1 / (self.order + 1)) / tmp
        else:
            dt1 = (tol * fact) ** (1 / (self.order + 1)) * norm * 0.5
        t1 = t + dt1 / 100
        self._combine(y0, [dt1 / 100], self._ytmp(1))
        self._deriv_into(t1, self._ytmp(1), 1)
        tmp = self._norm(self._k(1))
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

    def integrate(self, t: float, step: bool = False):
        """``integrate`` (explicit_rk.pyx:278-331)."""
        t = float(t)
        nsteps_left = self.max_numsteps
        if not self._set:
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
            self._set_interp(t)
            self.t = t
            return
        self.status = NORMAL
        if step and self.t < self.t_front and t > self.t_front:
            t = self.t_front
        while self.t_front < t and self.status >= 0:
            # y_prev <- y_front: swap the buffers (the old y_prev is dead)
            self._swap()
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
            self._set_interp(t)
        else:
            self.status = AT_FRONT
            self.t = self.t_front
            self._out = ("front", None)

    def _step_in_err(self, t, max_step):
        # explicit_rk.pyx:333-356
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
            self.stats["steps"] += 1
            if error >= 1:
                self.stats["rejected"] += 1
            if nsteps > max_step:
                self.status = TOO_MUCH_WORK
                break
        return nsteps

    def _compute_step(self, dt):
        # explicit_rk.pyx:358-397: ten fused stages; the last returns the error
        rk = self._rk()
        s = stream_ptr()
        for i in range(T.RK_STEP):
            self.op.vern7_stage(rk, i, self.t_prev, dt, self.atol, self.rtol, s)
        self.stats["rhs"] += T.RK_STEP
        self.t_front = self.t_prev + dt
        return self._read_result()

    def _prep_dense_out(self):
        # explicit_rk.pyx:399-410
        dt = self.dt_int
        rk = self._rk()
        self._combine(self._stage_base(), [dt * self.a[T.RK_STEP, j] for j in range(T.RK_STEP)],
                      self._ytmp(T.RK_STEP & 1))
        s = stream_ptr()
        for i in range(T.RK_STEP, T.RK_EXTRA_STEP):
            self.op.vern7_stage(rk, i, self.t_prev, dt, self.atol, self.rtol, s)
        self.stats["rhs"] += T.RK_EXTRA_STEP - T.RK_STEP

    def dense_factors(self, t):
        # explicit_rk.pyx:412-430 (Horner in tau, highest degree first)
        tau = (t - self.t_prev) / self.dt_int
        out = []
        for i in range(T.RK_EXTRA_STEP):
            acc = 0.0
            for j in range(T.DENSEOUT_ORDER - 1, -1, -1):
                acc += self.bi[i, j]
                acc *= tau
            out.append(self.dt_int * acc)
        return out

    def _set_interp(self, t):
        self._out = ("interp", self.dense_factors(t))

    def _get_timestep(self, t):
        # explicit_rk.pyx:440-449
        dt_needed = t - self.t_prev
        if self.interpolate:
            return self.dt_safe
        if dt_needed <= self.dt_safe:
            return dt_needed
        return dt_needed / (int(dt_needed / self.dt_safe) + 1)

    def _recompute_safe_step(self, err, dt):
        # explicit_rk.pyx:451-467
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

    # -- outputs ------------------------------------------------------------
    def successful(self) -> bool:
        return self.status >= 0

    def check(self):
        if not self.successful():
            raise IntegratorError(STATUS_MESSAGES[self.status])

    def state_view(self) -> _lib.StateView:
        """The state at ``self.t`` as a lazy view (valid until the next step)."""
        if self._out[0] == "front":
            return self._view(self.y_front)
        return self._view(self.y_prev, self._out[1])

    def get_state(self) -> torch.Tensor:
        """Materialise the state at ``self.t`` into ``self.y_out`` (state dtype)."""
        if self._out[0] == "front":
            self.y_out.copy_(self.y_front)
        else:
            self._combine(self.y_prev, self._out[1], self.y_out)
        return self.y_out
