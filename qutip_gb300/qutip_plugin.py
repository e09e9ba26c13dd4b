"""QuTiP plugin: the GB300 path behind QuTiP's own extension points.

Importing this module (QuTiP must be importable) registers:

* :class:`GpuDense`, a ``qutip.core.data.Data`` type whose matrix lives in device
  memory (complex128, column-major, so a column-stacked density matrix and its
  square form share one buffer).  Conversions to and from ``Dense`` and the
  alias ``"gpu"`` go through ``qutip.data.to.add_conversions`` /
  ``register_aliases`` (qutip/core/data/convert.pyx:208-331).
* Data-layer specialisations for ``GpuDense`` operands
  (qutip/core/data/dispatch.pyx:291-294 fixes their signatures): ``matmul``
  with a CSR, Dia or GpuDense left operand runs the library's SpMV
  (``qg_spmv_csr`` / ``qg_spmm_csr`` / ``qg_spmv_dia``; the reference's
  ``matmul_csr_dense_dense`` and ``matmul_dia_dense_dense``,
  qutip/core/data/matmul.pyx:226-272,429-507);
  ``expect`` / ``expect_super`` with a CSR or Dia operator run ``qg_expect_dm`` /
  ``qg_expect_ket`` (``expect_csr_dense`` and friends,
  qutip/core/data/expect.pyx:133-236); ``zeros``, ``add``, ``iadd``, ``sub``,
  ``mul``, ``imul``, ``neg``, ``trace``, ``trace_oper_ket``, ``norm.l2``,
  ``norm.frobenius``, ``column_stack``, ``column_unstack``, ``inner``,
  ``wrmn_error``, ``adjoint``, ``conj`` and ``transpose`` stay on the device
  (torch element-wise kernels; they are not on the integration hot path).
* :class:`IntegratorGpuVern7` as ``method="gpu_vern7"`` on ``MESolver``,
  ``SESolver``, ``MCSolver`` and ``BRSolver`` (``Solver.add_integrator``,
  qutip/solver/solver_base.py:475-492).  It takes the solver
  (``rhs_format = "solver"``), turns its ``QobjEvo`` right-hand side into one
  device operator with device-evaluated coefficients, and integrates with the
  fused Vern7 stage kernels; its options are the reference Vern7's
  (qutip/solver/integrator/qutip_integrator.py:51-59) plus ``precision``
  (``"double"`` or ``"mixed"``).
* :class:`IntegratorGpuPlaten` as ``method="gpu_platen"`` on ``SSESolver`` and
  ``SMESolver`` (``StochasticSolver.add_integrator``): the reference's Platen scheme,
  every step of an output interval in one ``qg_sde_platen`` launch, with the Wiener
  increments drawn by the reference's own ``Wiener`` object.
* ``map="gpu"`` for ``MCSolver`` (``qutip.solver.parallel._maps``,
  qutip/solver/parallel.py:541-559): all trajectories of a ``run`` -- with one
  initial state or a mixed initial ensemble -- go to one persistent
  ``qg_batch_vern7`` launch, and each comes back to ``MultiTrajResult.add`` as a
  trajectory result with its expectation values, collapse record and weight.

Nothing here computes on the host: a coefficient the device cannot evaluate, a
time-dependent collapse operator in a batched run, or a missing CUDA library is
an error, not a fallback.
"""
from __future__ import annotations

import ctypes as C
import math
from collections import OrderedDict

import numpy as np
import scipy.sparse as sp
import torch

import qutip
from qutip.core import data as _data
from qutip.core.cy import coefficient as _cyc
from qutip.core.data import CSR, Dense, Data, Dia
from qutip.core.data import ode as _ode
from qutip.solver.integrator import Integrator, IntegratorException
from qutip.solver.brmesolve import BRSolver
from qutip.solver.mcsolve import MCSolver
from qutip.solver.mesolve import MESolver
from qutip.solver.sesolve import SESolver
from qutip.solver import parallel as _parallel
from qutip.solver.stochastic import StochasticSolver
from qutip.solver.sode.sode import SIntegrator
from qutip.solver.sode._noise import PreSetWiener, Wiener

from . import _lib
from .coefficients import Coefficient, coefficient, interpolation
from .lindblad import LindbladOperator
from .operator import DeviceDia, DeviceOperator, stream_ptr
from .vern7 import GpuVern7, IntegratorError

__all__ = ["GpuDense", "IntegratorGpuVern7", "device_coefficient", "qobjevo_terms",
           "gpu_map", "register"]

_CDT = torch.complex128


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("GpuDense needs a CUDA device")
    return torch.device("cuda", torch.cuda.current_device())


# ------------------------------------------------------------------ data type --
class GpuDense(Data):
    """Dense complex128 matrix in device memory, column-major.

    ``buf`` is a flat torch CUDA tensor of length ``rows * cols`` holding the
    columns one after the other (the F order of ``qutip.core.data.Dense``).
    """

    def __init__(self, data, shape=None, copy=True):
        if isinstance(data, GpuDense):
            buf = data.buf.clone() if copy else data.buf
            shape = data.shape if shape is None else shape
        elif isinstance(data, torch.Tensor):
            t = data
            if t.dim() == 2:
                shape = tuple(t.shape) if shape is None else shape
                buf = t.transpose(0, 1).reshape(-1)
            else:
                if shape is None:
                    shape = (t.numel(), 1)
                buf = t.reshape(-1)
            buf = buf.to(_device(), _CDT)
            if copy and buf.data_ptr() == t.data_ptr():
                buf = buf.clone()
        else:
            arr = np.asarray(data, dtype=np.complex128)
            if arr.ndim == 1:
                arr = arr[:, None]
            if arr.ndim != 2:
                raise ValueError("GpuDense needs a 1-D or 2-D array")
            shape = arr.shape if shape is None else shape
            buf = torch.from_numpy(np.ascontiguousarray(arr.T).reshape(-1)).to(_device())
        shape = (int(shape[0]), int(shape[1]))
        if buf.numel() != shape[0] * shape[1]:
            raise ValueError(f"buffer of {buf.numel()} entries for shape {shape}")
        super().__init__(shape)
        self.buf = buf

    @classmethod
    def sparcity(cls):
        return "dense"

    # torch (rows, cols) view of the column-major buffer
    def matrix(self) -> torch.Tensor:
        return self.buf.view(self.shape[1], self.shape[0]).transpose(0, 1)

    def to_array(self):
        return self.buf.cpu().numpy().reshape(self.shape[1], self.shape[0]).T

    def trace(self):
        m, n = self.shape
        if m != n:
            raise ValueError("trace needs a square matrix")
        return complex(self.buf[::m + 1].sum().item())

    def copy(self):
        return GpuDense(self.buf.clone(), shape=self.shape, copy=False)

    def conj(self):
        return GpuDense(torch.conj(self.buf).resolve_conj(), shape=self.shape, copy=False)

    def transpose(self):
        return GpuDense(self.matrix().transpose(0, 1), copy=False)

    def adjoint(self):
        return GpuDense(torch.conj(self.matrix().transpose(0, 1)).resolve_conj(), copy=False)

    def __repr__(self):
        return f"GpuDense(shape={self.shape}, device={self.buf.device})"


def _wrap(buf: torch.Tensor, shape) -> GpuDense:
    return GpuDense(buf, shape=shape, copy=False)


def _dense_to_gpu(matrix):
    return GpuDense(matrix.to_array())


def _gpu_to_dense(matrix):
    return Dense(matrix.to_array(), copy=False)


# ------------------------------------------------------------ device operator --
class _OpCache:
    """Device copies of host operators, keyed by object identity (the object is kept
    alive by the cache, so an id is never reused while its entry exists)."""

    def __init__(self, size=64):
        self.size = size
        self._d = OrderedDict()

    def get(self, obj, build):
        key = id(obj)
        hit = self._d.get(key)
        if hit is not None and hit[0] is obj:
            self._d.move_to_end(key)
            return hit[1]
        val = build(obj)
        self._d[key] = (obj, val)
        if len(self._d) > self.size:
            self._d.popitem(last=False)
        return val


_OPS = _OpCache()
_SUPER_EOPS = _OpCache()


def _scipy(matrix) -> sp.csr_matrix:
    if isinstance(matrix, CSR):
        return matrix.as_scipy()
    if isinstance(matrix, Dia):
        return sp.csr_matrix(matrix.as_scipy())
    return sp.csr_matrix(matrix.to_array())


_DIAS = _OpCache()


def matmul_dia_gpu(left, right, scale=1, out=None):
    """Dia operator times a GpuDense matrix with the library's diagonal kernel
    (``qg_spmv_dia``; the reference's ``matmul_dia_dense_dense``,
    qutip/core/data/matmul.pyx:429-507), column by column."""
    if left.shape[1] != right.shape[0]:
        raise ValueError(f"incompatible matrix shapes {left.shape} and {right.shape}")
    op = _DIAS.get(left, lambda m: DeviceDia(m.as_scipy(), dtype="c128", device=_device()))
    rows, cols = left.shape[0], right.shape[1]
    y = torch.empty(rows * cols, dtype=_CDT, device=right.buf.device) if out is None else out.buf
    beta = 0.0 if out is None else 1.0
    for j in range(cols):
        op.matvec(right.buf[j * right.shape[0]:(j + 1) * right.shape[0]],
                  y[j * rows:(j + 1) * rows], alpha=scale, beta=beta)
    return out if out is not None else _wrap(y, (rows, cols))


def _device_op(matrix) -> DeviceOperator:
    return _OPS.get(matrix, lambda m: DeviceOperator([(_scipy(m), None)], dtype="c128",
                                                     device=_device(), fmt="csr"))


def matmul_csr_gpu(left, right, scale=1, out=None):
    if left.shape[1] != right.shape[0]:
        raise ValueError(f"incompatible matrix shapes {left.shape} and {right.shape}")
    op = _device_op(left)
    rows, cols = left.shape[0], right.shape[1]
    if out is None:
        y = torch.empty(rows * cols, dtype=_CDT, device=right.buf.device)
        beta = 0.0
    else:
        y, beta = out.buf, 1.0
    if cols == 1:
        op.matvec(0.0, right.buf, y, alpha=scale, beta=beta)
    else:
        op.matmat(0.0, right.buf.view(cols, right.shape[0]), y.view(cols, rows),
                  alpha=scale, beta=beta)
    return out if out is not None else _wrap(y, (rows, cols))


def matmul_gpu(left, right, scale=1, out=None):
    if left.shape[1] != right.shape[0]:
        raise ValueError(f"incompatible matrix shapes {left.shape} and {right.shape}")
    prod = (left.matrix() @ right.matrix()) * complex(scale)
    if out is not None:
        out.buf += prod.transpose(0, 1).reshape(-1)
        return out
    return GpuDense(prod, copy=False)


def zeros_gpu(rows, cols):
    return _wrap(torch.zeros(int(rows) * int(cols), dtype=_CDT, device=_device()), (rows, cols))


def _same_shape(a, b):
    if a.shape != b.shape:
        raise ValueError(f"incompatible matrix shapes {a.shape} and {b.shape}")


def add_gpu(left, right, scale=1):
    _same_shape(left, right)
    return _wrap(left.buf + complex(scale) * right.buf, left.shape)


def iadd_gpu(left, right, scale=1):
    _same_shape(left, right)
    left.buf.add_(right.buf, alpha=complex(scale))
    return left


def sub_gpu(left, right):
    _same_shape(left, right)
    return _wrap(left.buf - right.buf, left.shape)


def mul_gpu(matrix, value):
    return _wrap(matrix.buf * complex(value), matrix.shape)


def imul_gpu(matrix, value):
    matrix.buf.mul_(complex(value))
    return matrix


def neg_gpu(matrix):
    return _wrap(-matrix.buf, matrix.shape)


def trace_gpu(matrix):
    return matrix.trace()


def trace_oper_ket_gpu(matrix):
    n = matrix.shape[0]
    d = int(math.isqrt(n))
    if d * d != n or matrix.shape[1] != 1:
        raise ValueError("trace_oper_ket needs a column-stacked square operator")
    return complex(matrix.buf[::d + 1].sum().item())


def l2_gpu(matrix):
    if matrix.shape[0] != 1 and matrix.shape[1] != 1:
        raise ValueError("L2 norm is only defined on vectors")
    return float(torch.linalg.vector_norm(matrix.buf).item())


def frobenius_gpu(matrix):
    return float(torch.linalg.vector_norm(matrix.buf).item())


def column_stack_gpu(matrix):
    return _wrap(matrix.buf, (matrix.shape[0] * matrix.shape[1], 1))


def column_unstack_gpu(matrix, rows):
    rows = int(rows)
    if matrix.shape[1] != 1 or rows <= 0 or matrix.shape[0] % rows:
        raise ValueError(f"cannot unstack a {matrix.shape} vector into {rows} rows")
    return _wrap(matrix.buf, (rows, matrix.shape[0] // rows))


def inner_gpu(left, right, scalar_is_ket=False):
    if left.shape[0] == 1:      # bra
        return complex(torch.dot(left.buf, right.buf).item())
    return complex(torch.vdot(left.buf, right.buf).item())


def wrmn_error_gpu(diff, state, atol, rtol):
    w = torch.abs(diff.buf) / (atol + rtol * torch.abs(state.buf))
    return float(torch.sqrt(torch.mean(w * w)).item())


def isherm_gpu(matrix, tol=-1):
    """Hermitian up to an element-wise absolute tolerance: every pair satisfies
    ``|a_rc - conj(a_cr)|^2 < tol^2`` (isherm_dense and _conj_feq,
    qutip/core/data/properties.pyx:25-33,218-246), tested on the device."""
    rows, cols = matrix.shape
    if rows != cols:
        return False
    tol = float(tol) if tol >= 0 else float(qutip.settings.core["atol"])
    m = matrix.matrix()
    d = m - m.transpose(0, 1).conj()
    return bool(((d.real * d.real + d.imag * d.imag) < tol * tol).all().item())


def adjoint_gpu(matrix):
    return matrix.adjoint()


def conj_gpu(matrix):
    return matrix.conj()


def transpose_gpu(matrix):
    return matrix.transpose()


class _ExpectOp:
    """One operator as a single-group device operator for qg_expect_*."""

    def __init__(self, m: sp.csr_matrix):
        m = sp.csr_matrix(m, dtype=np.complex128)
        m.sort_indices()
        dev = _device()
        self.n = m.shape[0]
        self.row_ptr = torch.from_numpy(m.indptr.astype(np.int32)).to(dev)
        self.col = torch.from_numpy(m.indices.astype(np.int32)).to(dev)
        self.val = torch.from_numpy(m.data).to(dev)
        self.struct = _lib.CsrGroups(self.n, m.shape[1], 1, _lib.QG_C128,
                                     _lib.QG_LAYOUT_GROUP_MAJOR, 1, 0, 0,
                                     self.row_ptr.data_ptr(), self.col.data_ptr(),
                                     self.val.data_ptr(), None, None, None, None)
        self.out = torch.zeros(4, dtype=torch.float64, device=dev)


def _view(buf: torch.Tensor) -> _lib.StateView:
    return _lib.StateView(buf.numel(), _lib.QG_C128, _lib.QG_C128, buf.data_ptr(), None, 0, 0,
                          (C.c_double * 16)())


def _check_expect_shapes(op, state):
    if state.shape[1] == 1:
        if op.shape[1] != state.shape[0]:
            raise ValueError(f"incompatible shapes {op.shape} and {state.shape}")
    else:
        d = state.shape[0]
        if state.shape != (d, d) or op.shape != (d, d):
            raise ValueError(f"incompatible shapes {op.shape} and {state.shape}")


_MULTI = _OpCache(size=16)


class _MultiExpect:
    """Several e_ops as one operator with one coefficient group each, so that one
    ``qg_expect_dm`` / ``qg_expect_ket`` launch evaluates all of them."""

    def __init__(self, ops):
        from .solver import _wide_groups
        self.ops = ops                                   # keeps the ids below valid
        self.dev = _wide_groups([_scipy(o) for o in ops], "c128", _device())
        self.G = len(ops)


class _SuperRows:
    """Several super-operator e_ops as one operator whose row k is the sum of the
    diagonal-position rows of op k: one matvec gives every ``expect_super`` value."""

    def __init__(self, ops, d):
        self.ops = ops
        rows = [sp.csr_matrix(np.ones((1, d))) @ _scipy(o)[np.arange(d) * (d + 1)] for o in ops]
        self.e = _ExpectOp(sp.vstack(rows, format="csr"))


def _group_get(cache, ops, build):
    key = tuple(id(o) for o in ops)
    hit = cache._d.get(key)
    if hit is not None and all(a is b for a, b in zip(hit[1].ops, ops)):
        cache._d.move_to_end(key)
        return hit[1]
    val = build(tuple(ops))
    cache._d[key] = (None, val)
    if len(cache._d) > cache.size:
        cache._d.popitem(last=False)
    return val


def _launch_batch(batch, state, base_ptr):
    """Launch the kernels of every ``(kind, op)`` of ``batch`` against ``state``: the
    ``expect`` operators in launches of up to QG_MAX_EOPS groups, the ``super`` ones as
    one multi-row matvec.  Returns ``(kind, op, double offset)`` per operator."""
    place = []
    off = 0
    ex = [o for k, o in batch if k == "expect"]
    for i in range(0, len(ex), _lib.QG_MAX_EOPS):
        chunk = ex[i:i + _lib.QG_MAX_EOPS]
        m = _group_get(_MULTI, chunk, _MultiExpect)
        if state.shape[1] == 1:
            _lib.call("qg_expect_ket", C.byref(m.dev.struct), C.byref(_view(state.buf)),
                      base_ptr + 8 * off, stream_ptr())
        else:
            _lib.call("qg_expect_dm", C.byref(m.dev.struct), state.shape[0],
                      C.byref(_view(state.buf)), base_ptr + 8 * off, stream_ptr())
        place += [("expect", o, off + 2 * g) for g, o in enumerate(chunk)]
        off += 2 * (len(chunk) + 1)
    su = [o for k, o in batch if k == "super"]
    if su:
        d = int(math.isqrt(state.shape[0]))
        m = _group_get(_SUPER_EOPS, su, lambda ops: _SuperRows(ops, d))
        _lib.call("qg_spmv_csr", C.byref(m.e.struct), 0.0, state.buf.data_ptr(),
                  base_ptr + 8 * off, 1.0, 0.0, 0.0, 0.0, stream_ptr())
        place += [("super", o, off + 2 * g) for g, o in enumerate(su)]
        off += 2 * len(su)
    return place, off


def _fits(kind, op, state) -> bool:
    """Whether ``op`` can be evaluated against ``state`` as an e_op of this ``kind``."""
    n, m = state.shape
    if kind == "super":
        d = int(math.isqrt(n))
        return m == 1 and d * d == n and op.shape[1] == n
    return op.shape[1] == n if m == 1 else (n == m and op.shape == (n, n))


class _ExpectBatch:
    """Expectation values of one state against several operators with one read-back.

    ``Result.add`` asks for the e_ops of an output time one at a time, and each answer
    must be a host number, so computed one by one every e_op costs a launch and a
    blocking device-to-host read.  Here the first request against a new state launches
    the kernels of every operator asked for against the previous state (the e_ops of
    the previous output time) into one device buffer and reads it back once; the other
    requests against the same state are answered from that read.

    An answer is reused only while nothing can have changed the state: the same
    ``GpuDense`` object, the same torch version counter of its buffer, and no launch of
    the library since the read (every kernel that writes device memory counts)."""

    def __init__(self):
        self.state = None
        self.version = -1
        self.launch_mark = -1
        self.values = {}          # (kind, id(op)) -> complex
        self.keep = []            # the operators of ``values`` (their ids stay valid)
        self.prev = []            # (kind, op) asked for against the previous state
        self.cur = []
        self.buf = None
        self.host = None

    def _valid(self, state):
        return (state is self.state and state.buf._version == self.version
                and _lib.LAUNCHES[0] == self.launch_mark)

    def _buffers(self, k, device):
        size = 4 * k + 2 * (k // _lib.QG_MAX_EOPS + 2)    # values, traces / norms
        if self.buf is None or self.buf.numel() < size or self.buf.device != device:
            self.buf = torch.zeros(max(size, 64), dtype=torch.float64, device=device)
            self.host = torch.zeros(max(size, 64), dtype=torch.float64).pin_memory()

    def get(self, kind, op, state):
        key = (kind, id(op))
        if self._valid(state):
            if key in self.values:
                self.cur.append((kind, op))
                return self.values[key]
            batch = [(kind, op)]
        else:
            if self.state is not None:
                self.prev = self.cur
            self.cur = []
            self.values = {}
            self.keep = []
            batch = [(kind, op)]
            for k2, o2 in self.prev:
                if (k2, id(o2)) != key and _fits(k2, o2, state):
                    batch.append((k2, o2))
        self._buffers(len(batch), state.buf.device)
        place, used = _launch_batch(batch, state, self.buf.data_ptr())
        h = self.host[:used]
        h.copy_(self.buf[:used], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        v = h.numpy()
        for k2, o, at in place:
            self.values[(k2, id(o))] = complex(float(v[at]), float(v[at + 1]))
            self.keep.append(o)
        self.state = state
        self.version = state.buf._version
        self.launch_mark = _lib.LAUNCHES[0]
        self.cur.append((kind, op))
        return self.values[key]


_BATCH = _ExpectBatch()


def expect_csr_gpu(op, state):
    """``<psi|op|psi>`` for a ket, ``tr(op rho)`` for a square state."""
    _check_expect_shapes(op, state)
    return _BATCH.get("expect", op, state)


def expect_super_csr_gpu(op, state):
    """``tr(unvec(op @ vec(rho)))``: the rows of ``op`` on the diagonal of rho,
    summed (expect_super_csr_dense, qutip/core/data/expect.pyx:223-236)."""
    n = state.shape[0]
    d = int(math.isqrt(n))
    if d * d != n or state.shape[1] != 1 or op.shape[1] != n:
        raise ValueError(f"incompatible shapes {op.shape} and {state.shape}")
    return _BATCH.get("super", op, state)


# ---------------------------------------------------------- coefficients ------
def _cy_state(c):
    r = c.__reduce_ex__(2)
    if len(r) > 2 and r[2] is not None:
        return r[2]
    args = r[1]
    if len(args) > 2 and isinstance(args[2], tuple):
        return args[2]
    return ()


def _members(c):
    return [x for x in _cy_state(c) if isinstance(x, _cyc.Coefficient)]


def _decode(c) -> Coefficient:
    if isinstance(c, _cyc.ConstantCoefficient):
        return coefficient(complex(c(0.0)))
    if isinstance(c, _cyc.ConjCoefficient):
        (b,) = _members(c)
        return _decode(b).conj()
    if isinstance(c, _cyc.NormCoefficient):
        (b,) = _members(c)
        db = _decode(b)
        return db.conj() * db
    if isinstance(c, _cyc.SumCoefficient):
        a, b = _members(c)
        return _decode(a) + _decode(b)
    if isinstance(c, _cyc.MulCoefficient):
        a, b = _members(c)
        return _decode(a) * _decode(b)
    if isinstance(c, _cyc.InterCoefficient):
        _, (tl, poly, dt) = c.__reduce__()
        return interpolation(tl, poly, dt or 0.0)
    if isinstance(c, _cyc.StrFunctionCoefficient):
        base, args = c.__reduce__()[1]
        return coefficient(base, args)
    if type(c).__name__ == "StrCoefficient":
        # Cython-compiled string coefficient (qutip/core/coefficient.py:529-560):
        # its state holds the argument values, the source string, then the names.
        st = list(_cy_state(c))
        k = next(i for i, x in enumerate(st) if isinstance(x, str))
        names = [x for x in st[k + 1:] if isinstance(x, str)]
        values = [x for x in st[:k] if isinstance(x, (int, float, complex))]
        return coefficient(st[k], dict(zip(names, values[:len(names)])))
    raise TypeError(f"a {type(c).__name__} cannot be evaluated on the device")


_CHECK_TIMES = (0.0, 0.3183, 1.7321, 4.4721, 11.0)


def device_coefficient(c) -> Coefficient:
    """The device program of a QuTiP coefficient, checked against the coefficient
    itself at a few times; raises ``TypeError`` when it cannot be built."""
    try:
        prog = _decode(c)
    except (TypeError, ValueError, StopIteration) as exc:
        raise TypeError(f"coefficient {c!r} cannot be evaluated on the device: {exc}") from None
    for t in _CHECK_TIMES:
        want, got = complex(c(t)), complex(prog(t))
        if not (np.isclose(got, want, rtol=1e-12, atol=1e-12)
                or (np.isnan(got) and np.isnan(want))):
            raise TypeError(f"coefficient {c!r} cannot be evaluated on the device "
                            f"(device program gives {got} at t={t}, the coefficient {want})")
    return prog


def qobjevo_terms(evo):
    """``(scipy CSR, device Coefficient | None)`` terms of a QobjEvo or Qobj.

    A constant QobjEvo whose elements are not (operator, coefficient) pairs, e.g. a
    Bloch-Redfield tensor built from special elements (qutip/solver/brmesolve.py:323-333),
    becomes the single constant term ``evo(0)``, evaluated once by QuTiP itself."""
    if isinstance(evo, qutip.Qobj):
        return [(_scipy(evo.data), None)]
    try:
        return _decode_terms(evo)
    except TypeError:
        if evo.isconstant:
            return [(_scipy(evo(0).data), None)]
        raise


def _decode_terms(evo):
    out = []
    for el in evo.to_list():
        if isinstance(el, qutip.Qobj):
            out.append((_scipy(el.data), None))
        elif isinstance(el, (list, tuple)) and len(el) == 2 and isinstance(el[0], qutip.Qobj):
            c = el[1]
            if not isinstance(c, _cyc.Coefficient):
                c = qutip.coefficient(c)
            out.append((_scipy(el[0].data), device_coefficient(c)))
        else:
            raise TypeError("QobjEvo element of this kind cannot be evaluated on the device")
    return out


#: generators with at least this many rows are merged and laid out on the device
DEVICE_BUILD_ROWS = 1024


def device_operator(terms, dtype="c128") -> DeviceOperator:
    """The device operator of ``(scipy matrix, Coefficient | None)`` terms.

    Square generators of ``DEVICE_BUILD_ROWS`` rows or more -- every Liouvillian of a
    system of Hilbert dimension 32 or more -- are copied to the device term by term,
    merged per coefficient and laid out there (dictionary-coded sliced ELLPACK when the
    (column - row, value) pairs fit its tables, else sliced ELLPACK when its padding
    costs at most 15 %).  The host layouts of the same operator take seconds at a
    million rows (10 s for the L = 10 Ising Liouvillian).  Smaller or irregular
    generators keep the host layouts (row-major CSR with staged tiles)."""
    from .superop import device_term_groups, sliced_padding
    n_rows, n_cols = terms[0][0].shape
    if n_rows == n_cols and n_rows >= DEVICE_BUILD_ROWS and len(terms) <= _lib.QG_MAX_GROUPS * 4:
        groups = device_term_groups(terms, _device())
        if len(groups) <= _lib.QG_MAX_GROUPS and sliced_padding(groups) <= 1.15:
            return DeviceOperator.from_device_groups(groups, dtype, fmt="auto")
        del groups
    return DeviceOperator(terms, dtype=dtype, device=_device())


def _coefficient_groups(terms):
    """Term indices per coefficient group, in the order the operators merge them
    (:func:`qutip_gb300.systems.merge_terms`), with each group's coefficient."""
    keyed, out = {}, []
    for i, (_, c) in enumerate(terms):
        key = None if c is None else c.key()
        if key not in keyed:
            keyed[key] = len(out)
            out.append(([], c))
        out[keyed[key]][0].append(i)
    return [(tuple(idx), c) for idx, c in out]


def _is_matrix_form(rhs) -> bool:
    try:
        from qutip.core.cy.lindblad_matrix_form import LindbladMatrixForm
    except ImportError:
        return False
    return isinstance(rhs, LindbladMatrixForm)


def lindblad_operator(rhs, dtype="c128", dense="auto"):
    """The device generator of a ``LindbladMatrixForm`` (mesolve's ``matrix_form``
    option, qutip/solver/mesolve.py:251-266): A = -i H_nh from its ``H_nh``
    (lindblad_matrix_form.pyx:88-96) and one term per collapse operator.

    The dense small-dimension bucket (:class:`~qutip_gb300.dense.DenseLindbladOperator`,
    tensor-core GEMMs) takes the mixed form (complex64 stages) of a system with
    ``d <= 128`` whose operators are at least ``DENSE_FILL`` filled, or whenever
    ``dense=True``; sparse systems keep the matrix-free sparse kernel."""
    from .dense import DENSE_FILL, DenseLindbladOperator, dense_fill
    a_terms = [((-1j) * m, c) for m, c in qobjevo_terms(rhs.H_nh)]
    c_terms = []
    for c in rhs.c_ops:
        terms = qobjevo_terms(c)
        if len(terms) != 1:
            raise TypeError("matrix_form on the GPU needs each collapse operator to be a "
                            "single (possibly time-dependent) term")
        c_terms.append(terms[0])
    d = a_terms[0][0].shape[0]
    if dense is True and (dtype != "c64" or d > _lib.QG_DENSE_MAX_D):
        raise ValueError(f"the dense bucket runs the mixed form (precision='mixed') for "
                         f"d <= {_lib.QG_DENSE_MAX_D}")
    if dense is not False and dtype == "c64" and d <= _lib.QG_DENSE_MAX_D and (
            dense is True or dense_fill([m for m, _ in a_terms + c_terms]) >= DENSE_FILL):
        return DenseLindbladOperator(a_terms, c_terms, device=_device())
    return LindbladOperator(a_terms, c_terms, dtype=dtype, device=_device())


# ---------------------------------------------------------------- integrator --
def _as_gpu(state) -> GpuDense:
    if isinstance(state, GpuDense):
        return state
    return GpuDense(state.to_array())


class IntegratorGpuVern7(Integrator):
    """Verner 7(6) with dense output on the GPU: the reference's ``vern7`` control
    flow (qutip/solver/integrator/explicit_rk.pyx:204-467) on fused device stages.

    Usable with ``method="gpu_vern7"``; ``precision="mixed"`` keeps the operator and
    stage vectors in complex64 (FP32 accumulation) and the state, step control,
    stage combinations and norms in FP64.
    """
    integrator_options = {
        "atol": 1e-8,
        "rtol": 1e-6,
        "nsteps": 1000,
        "first_step": 0,
        "max_step": 0,
        "min_step": 0,
        "interpolate": True,
        "precision": "double",
        "dense": "auto",
        "hermitian_branch": "auto",
    }
    rhs_format = "solver"
    support_time_dependant = True
    supports_blackbox = False
    method = "gpu_vern7"

    def __init__(self, system, options):
        self.system = system
        self._is_set = False
        self._back = (np.inf, None)
        self._options = self.integrator_options.copy()
        self.options = options
        self._prepare()

    def _rhs(self):
        rhs = self.system.rhs
        return rhs if isinstance(rhs, (qutip.QobjEvo, qutip.Qobj)) else rhs()

    def _prepare(self):
        prec = self._options["precision"]
        if prec not in ("double", "mixed"):
            raise ValueError("precision must be 'double' or 'mixed'")
        dt = "c128" if prec == "double" else "c64"
        rhs = self._rhs()
        self._terms = None
        self._groups = None
        if _is_matrix_form(rhs):
            self._op = lindblad_operator(rhs, dt, self._options.get("dense", "auto"))
        else:
            self._terms = qobjevo_terms(rhs)
            self._groups = _coefficient_groups(self._terms)
            self._op = device_operator(self._terms, dt)
        self._blocks = {1: self._op}
        self._ode = self._integrator(self._op)
        self._shape = (self._op.n_rows, 1)
        self.name = f"{self.method} ({prec})"

    def _integrator(self, op):
        o = self._options
        return GpuVern7(op, atol=o["atol"], rtol=o["rtol"], nsteps=o["nsteps"],
                        first_step=o["first_step"], min_step=o["min_step"],
                        max_step=o["max_step"], interpolate=o["interpolate"],
                        precision=o["precision"])

    def _block_operator(self, m):
        """``I_m (x) A(t)``: the generator applied to each of the m columns of an
        operator-valued state (``propagator``'s identity, qutip/solver/propagator.py:201-213,
        evolved as ``rhs.matmul_data`` does on a matrix)."""
        if m not in self._blocks:
            if self._terms is None:
                raise ValueError("operator-valued states are not supported with matrix_form")
            eye = sp.identity(m, format="csr", dtype=np.complex128)
            dt = "c128" if self._options["precision"] == "double" else "c64"
            self._blocks[m] = DeviceOperator([(sp.kron(eye, a, format="csr"), c)
                                              for a, c in self._terms], dtype=dt,
                                             device=_device())
        return self._blocks[m]

    def set_state(self, t, state0):
        rows, cols = state0.shape
        if rows * cols == self._op.n_rows:
            op = self._op                      # a vector, or rho of the matrix form
        elif rows == self._op.n_rows:
            op = self._block_operator(cols)    # an operator-valued state, column by column
        else:
            raise ValueError(f"state of shape {state0.shape} for a generator of size "
                             f"{self._op.n_rows}")
        if self._ode.op is not op:
            self._ode = self._integrator(op)
        if isinstance(op, LindbladOperator):
            # the reference's branch choice: MESolver._prepare_state sets it from rho0.isherm
            # (qutip/solver/mesolve.py:270-277; lindblad_matrix_form.pyx:171-200); taken
            # where it is also the faster form
            op.hermitian = bool(getattr(self._rhs(), "assume_hermitian_state", False)) and \
                (self._options.get("hermitian_branch") is True or (
                    self._options.get("hermitian_branch") == "auto" and op.hermitian_pays()))
        self._ode.set_initial_value(_as_gpu(state0).buf, t)
        self._shape = state0.shape
        self._is_set = True

    def get_state(self, copy=True):
        y = self._ode.get_state()
        return self._ode.t, GpuDense(y.clone() if copy else y, shape=self._shape, copy=False)

    def _check(self):
        try:
            self._ode.check()
        except IntegratorError as exc:
            raise IntegratorException(str(exc)) from None

    def integrate(self, t, copy=True):
        self._ode.integrate(t, step=False)
        self._check()
        return self.get_state(copy)

    def mcstep(self, t, copy=True):
        self._ode.integrate(t, step=True)
        self._check()
        return self.get_state(copy)

    def reset(self, hard=False):
        if self._is_set:
            state = self.get_state()
        # The device coefficient programs hold the args they were decoded with, while the
        # reference's integrators read the rhs live: Solver._argument follows
        # rhs.arguments(args) with a soft reset (solver_base.py:457-460), so the
        # coefficients of a time-dependent rhs are decoded again.  The operator storage
        # stays: only the programs depend on the args.
        if hard:
            self._prepare()
        elif not getattr(self._rhs(), "isconstant", True):
            self._update_coefficients()
        if self._is_set:
            self.set_state(*state)

    def _update_coefficients(self):
        """New device coefficient programs for the same operator storage, or a full
        rebuild when the args regroup the terms (two coefficients become equal)."""
        if self._terms is None:                       # matrix form: rebuild
            self._prepare()
            return
        terms = qobjevo_terms(self._rhs())
        groups = _coefficient_groups(terms)
        if [idx for idx, _ in groups] != [idx for idx, _ in self._groups]:
            self._prepare()
            return
        coeffs = [c for _, c in groups]
        for op in self._blocks.values():
            op.set_coefficients(coeffs)
        self._terms, self._groups = terms, groups

    @property
    def options(self):
        """atol, rtol, nsteps, first_step, max_step, min_step, interpolate: as the
        reference ``vern7``; precision: ``"double"`` or ``"mixed"``; dense (matrix form
        only): ``"auto"`` sends small systems with dense operators in the mixed form to
        the tensor-core bucket, ``True`` forces it, ``False`` keeps the sparse kernel;
        hermitian_branch (matrix form only): with a Hermitian rho0, ``"auto"`` evaluates
        half the elements where that is faster (at least two 32 x 32 tiles per SM),
        ``True`` always, ``False``
        never."""
        return self._options

    @options.setter
    def options(self, new_options):
        Integrator.options.fset(self, new_options)


# ----------------------------------------------------------- stochastic (SODE) --
def sde_operator(rhs):
    """The device drift / diffusion operators of the reference's ``_StochasticRHS``
    (qutip/solver/stochastic.py:234-290), built as ``StochasticClosedSystem`` /
    ``StochasticOpenSystem`` build them (qutip/solver/sode/ssystem.pyx:131-139, 211-225)."""
    from .stochastic import SdeOperator
    evos = [rhs.H] + list(rhs.sc_ops) + list(rhs.c_ops)
    if not all(getattr(e, "isconstant", True) for e in evos):
        raise TypeError("method='gpu_platen' integrates constant H, sc_ops and c_ops")
    H = rhs.H(0)
    sc = [c(0) for c in rhs.sc_ops]
    if rhs.issuper:
        L = H + qutip.liouvillian(None, sc) if H.issuper else qutip.liouvillian(H, sc)
        if rhs.c_ops:
            L = L + qutip.liouvillian(None, [c(0) for c in rhs.c_ops])
        cs = [qutip.spre(c) + qutip.spost(c.dag()) for c in sc]
        d = int(round(np.sqrt(L.shape[0])))
        return SdeOperator(_scipy(L.data), [_scipy(c.data) for c in cs], open=True, d=d,
                           device=_device())
    L = -1j * H
    for c in sc:
        L = L + (-0.5 * c.dag() * c)
    ms = [c + c.dag() for c in sc]
    return SdeOperator(_scipy(L.data), [_scipy(c.data) for c in sc],
                       [_scipy(m.data) for m in ms], open=False, d=H.shape[0], device=_device())


class IntegratorGpuPlaten(SIntegrator):
    """The reference's explicit Platen scheme (``PlatenSODE``, strong order 1,
    qutip/solver/sode/sode.py:235-251) on the device: each ``integrate`` call runs the
    interval's fixed steps in one ``qg_sde_platen`` launch, with the increments the
    reference's ``Wiener`` draws from the trajectory's generator.  Options: ``dt``
    (default 0.001) and ``tol``, as the reference's."""
    integrator_options = {"dt": 0.001, "tol": 1e-10}
    N_dw = 1
    _stepper_options = []
    scheme = "platen"

    def __init__(self, rhs, options):
        self._options = self.integrator_options.copy()
        self.options = options
        self.rhs = rhs
        self._op = None

    def set_state(self, t, state0, generator):
        if self._op is None:
            self._op = sde_operator(self.rhs)
        self.t = t
        buf = _as_gpu(state0).buf
        if buf.numel() != self._op.n:
            raise ValueError(f"state of {buf.numel()} entries for a system of {self._op.n}")
        self._state = buf.clone()
        if isinstance(generator, PreSetWiener):
            if generator.is_measurement:
                raise NotImplementedError("gpu_platen does not support running the evolution "
                                          "from measurements")
            self.wiener = generator
        elif isinstance(generator, Wiener):
            self.wiener = generator
        else:
            self.wiener = Wiener(t, self.options["dt"], generator,
                                 (self.N_dw, len(self.rhs.sc_ops)))
        self.rhs._register_feedback(self.wiener)
        self._is_set = True

    def get_state(self, copy=True):
        buf = self._state.clone() if copy else self._state
        return self.t, GpuDense(buf, shape=(self._op.n, 1), copy=False), self.wiener

    def integrate(self, t, copy=True):
        """Reference control flow of ``_Explicit_Simple_Integrator.integrate``
        (sode.py:151-173): the number of dt steps to t, rounded up past half a step."""
        delta_t = t - self.t
        dt = self.options["dt"]
        if delta_t < 0:
            raise ValueError("Integration time, can't be negative.")
        elif delta_t < 0.5 * dt:
            import warnings
            warnings.warn(f"Step under minimum step ({dt}), skipped.", RuntimeWarning)
            return self.t, GpuDense(self._state, shape=(self._op.n, 1), copy=copy), \
                np.zeros(self.N_dw)
        N, extra = np.divmod(delta_t, dt)
        N = int(N)
        if extra > 0.5 * dt:
            N += 1
        dW = self.wiener.dW(self.t, N)
        dev = torch.from_numpy(np.ascontiguousarray(dW[:, 0, :], dtype=np.float64)).to(
            self._state.device, non_blocking=False)
        self._op.advance(self._state.view(1, -1), dev, N, dt, scheme=self.scheme)
        self.t += dt * N
        return self.t, GpuDense(self._state, shape=(self._op.n, 1), copy=copy), \
            np.sum(dW[:, 0, :], axis=0)

    def mcstep(self, t, copy=True):
        raise NotImplementedError

    @property
    def options(self):
        """dt : float, default 0.001 -- the fixed step; tol : float, default 1e-10."""
        return self._options

    @options.setter
    def options(self, new_options):
        Integrator.options.fset(self, new_options)


class IntegratorGpuEuler(IntegratorGpuPlaten):
    """The reference's Euler-Maruyama scheme (``EulerSODE``, strong order 0.5,
    qutip/solver/sode/itotaylor.py:12-26) on the device, as :class:`IntegratorGpuPlaten`."""
    scheme = "euler"


# ------------------------------------------------------------- trajectories ---
def _constant_matrix(op, what):
    if isinstance(op, qutip.QobjEvo):
        if not op.isconstant:
            raise TypeError(f"time-dependent {what} are not supported by map='gpu'")
        op = op(0)
    if not isinstance(op, qutip.Qobj):
        raise TypeError(f"{what} must be Qobj (map='gpu' records expectation values on the "
                        "device)")
    return _scipy(op.data)


def _collapse_term(op):
    """A collapse operator as ``(matrix, Coefficient | None)``: ``f(t) C`` for a
    one-term QobjEvo (mcsolve.py:168-170 wraps every c_op in one), ``C`` for a constant
    one.  The jump probabilities use ``|f(t)|^2 ||C psi||^2`` on the device; the solver's
    H_nh already carries the ``-1/2 conj(f) f C^dag C`` terms."""
    if isinstance(op, qutip.QobjEvo) and not op.isconstant:
        terms = qobjevo_terms(op)
        if len(terms) != 1:
            raise TypeError("map='gpu' needs each time-dependent collapse operator to be a "
                            "single term f(t) C")
        return terms[0]
    return (_constant_matrix(op, "collapse operators"), None)


def _mc_map_items(task, values, task_args, task_kwargs):
    """Decode the trajectory task an ``MCSolver`` hands to its map.

    Returns ``(solver, seeds, starts, floors, tlist, e_ops)`` where ``starts`` holds
    ``(initial state, weight)`` per trajectory and ``floors`` the improved-sampling
    jump-probability floor of each.  The forms follow the reference's call sites:

    * ``_run_one_traj`` over seeds (multitraj.py:169-258), with
      ``{'no_jump': False, 'jump_prob_floor': p}`` under improved sampling
      (mcsolve.py:716-747);
    * ``_run_one_traj_mixed`` over trajectory ids (multitraj.py:298-350);
    * ``_unpack_arguments(_run_one_traj_mixed, ('id', 'jump_prob_floor'))`` over
      ``(id, floor)`` pairs, improved sampling with mixed states (mcsolve.py:749-790).
    """
    kw = dict(task_kwargs or {})
    if kw.pop("no_jump", False):
        raise TypeError("map='gpu' does not run the no-jump trajectory as a map task")
    func, names = task, None
    if hasattr(task, "func") and hasattr(task, "argument_names"):
        func, names = task.func, tuple(task.argument_names)
    solver = getattr(func, "__self__", None)
    name = getattr(func, "__name__", "")
    if not isinstance(solver, MCSolver):
        raise TypeError("map='gpu' runs MCSolver trajectories only")
    if name == "_run_one_traj" and names is None:
        state0, tlist, e_ops = task_args
        floor = float(kw.pop("jump_prob_floor", 0.0))
        seeds = list(values)
        starts = [(state0, 1.0)] * len(seeds)
        floors = [floor] * len(seeds)
    elif name == "_run_one_traj_mixed" and names is None:
        all_seeds, ics, tlist, e_ops = task_args
        floor = float(kw.pop("jump_prob_floor", 0.0))
        ids = list(values)
        seeds = [all_seeds[i] for i in ids]
        starts = [ics.get_state_and_weight(i) for i in ids]
        floors = [floor] * len(ids)
    elif name == "_run_one_traj_mixed" and names == ("id", "jump_prob_floor"):
        all_seeds, ics, tlist, e_ops = (kw.pop(k) for k in ("seeds", "ics", "tlist", "e_ops"))
        pairs = [tuple(v) for v in values]
        seeds = [all_seeds[i] for i, _ in pairs]
        starts = [ics.get_state_and_weight(i) for i, _ in pairs]
        floors = [float(f) for _, f in pairs]
    else:
        raise TypeError(f"map='gpu' does not run the task {name or task!r}")
    if kw:
        raise TypeError(f"map='gpu' does not support the trajectory options {sorted(kw)}")
    return solver, seeds, starts, floors, tlist, e_ops


def _zero_trajectory(solver, e_ops, opts, tlist):
    """The all-zero trajectory of weight 0 the reference returns when improved
    sampling asks for a jump from a state that never jumps (mcsolve.py:544-558)."""
    traj = solver._trajectory_resultclass(e_ops, opts)
    traj.times = [float(t) for t in tlist]
    for key in traj.e_data:
        traj.e_data[key] = [0.0] * len(tlist)
    traj.collapse = []
    return traj


def gpu_map(task, values, task_args=None, task_kwargs=None, reduce_func=None, map_kw=None,
            progress_bar=None, progress_bar_kwargs={}):
    """``map="gpu"``: run every trajectory of an ``MCSolver.run`` in one persistent
    launch and hand each to ``reduce_func`` as the reference's trajectory result.

    The per-initial-state no-jump runs of improved sampling with mixed states
    (``_no_jump_simulation``, mcsolve.py:756-763) are single deterministic solves: they
    run one after another through the solver's own ``gpu_vern7`` integrator."""
    if isinstance(getattr(task, "__self__", None), StochasticSolver):
        return _gpu_map_sde(task, values, task_args, task_kwargs, reduce_func)
    if getattr(task, "__name__", "") == "_no_jump_simulation" and \
            isinstance(getattr(task, "__self__", None), MCSolver):
        out = [task(v, *(task_args or ()), **(task_kwargs or {})) for v in values]
        if reduce_func is not None:
            for r in out:
                reduce_func(r)
            return []
        return out
    from .batched import BatchProblem, MC_DEFAULTS
    solver, seeds, starts, floors, tlist, e_ops = _mc_map_items(
        task, values, task_args or (), task_kwargs)
    opts = solver.options
    if opts.get("method") not in ("vern7", "gpu_vern7"):
        raise TypeError(f"map='gpu' integrates with Vern7 on the device; method="
                        f"{opts.get('method')!r} is not available there (use 'vern7' or "
                        "'gpu_vern7')")
    if opts.get("bitgenerator") not in (None, "PCG64"):
        raise TypeError("map='gpu' draws from PCG64 streams (the default bit generator)")
    if opts.get("store_states") or opts.get("store_final_state"):
        raise TypeError("map='gpu' records expectation values only; pass e_ops and leave "
                        "store_states / store_final_state off")
    if isinstance(e_ops, dict):
        e_list = list(e_ops.values())
    elif e_ops is None:
        e_list = []
    elif isinstance(e_ops, (list, tuple)):
        e_list = list(e_ops)
    else:
        e_list = [e_ops]
    if not e_list:
        raise TypeError("map='gpu' needs e_ops")
    e_mats = [_constant_matrix(e, "e_ops") for e in e_list]
    c_mats = [_collapse_term(c) for c in solver._c_ops]
    terms = qobjevo_terms(solver.rhs())
    iopts = {**IntegratorGpuVern7.integrator_options,
             **{k: opts[k] for k in IntegratorGpuVern7.integrator_options if k in opts}}
    prec = iopts["precision"]
    tl = np.asarray(tlist, dtype=np.float64)
    mc = {k: opts[k] for k in MC_DEFAULTS if k in opts}
    max_jumps = int((map_kw or {}).get("max_jumps", 4096))
    # a floor at 1 - norm_tol or above: the state does not jump; the reference returns
    # a zero trajectory of weight 0 without integrating (mcsolve.py:544-558)
    dark = [f >= 1 - opts["norm_tol"] for f in floors]
    host_states = {}

    def launch(idx):
        """One persistent launch over the trajectories ``idx`` (dark ones skipped)."""
        bp = BatchProblem("c128" if prec == "double" else "c64")
        sid = bp.add_system(terms, e_mats, tl, "mc", c_ops=c_mats, atol=iopts["atol"],
                            rtol=iopts["rtol"], nsteps=iopts["nsteps"])
        for i in idx:
            if dark[i]:
                continue
            st = starts[i][0]
            if id(st) not in host_states:
                host_states[id(st)] = np.asarray(_as_gpu(st).to_array()).reshape(-1)
            bp.add_item(sid, host_states[id(st)], seed=seeds[i], jump_prob_floor=floors[i])
        if not bp.items:
            return iter(())
        bp.build(max_jumps=max_jumps, mc_options=mc)
        bp.launch()
        res = bp.results()
        gpu_map.launched_items += len(res)
        for r in res:
            if r["status"] == -5:
                raise RuntimeError("Could not find the collapse time within desired tolerance. "
                                   "Increase accuracy of the ODE solver or lower the tolerance "
                                   "with the options 'norm_steps', 'norm_tol', 'norm_t_tol'.")
            if r["status"] < 0:
                raise IntegratorException(f"trajectory failed with status {r['status']}")
        return iter(res)

    # With a target tolerance (multitrajresult.py:320-361) the reference stops the map as
    # soon as its reduce step estimates that no more trajectories are needed.  The
    # trajectories are then admitted in chunks: a first chunk, then as many as the
    # reduce step's own estimate asks for (at least ``min_chunk``), so no more are
    # integrated than the estimate needs.  Without one, every trajectory goes to one
    # launch.
    result = getattr(reduce_func, "__self__", None)
    early = getattr(result, "_target_tols", None) is not None
    total = len(seeds)
    min_chunk = int((map_kw or {}).get("min_chunk", 64))
    chunk = min(total, int((map_kw or {}).get("first_chunk", 256))) if early else total
    gpu_map.launched_items = 0
    pos = 0
    while pos < total:
        idx = range(pos, min(total, pos + max(chunk, 1)))
        res = launch(idx)
        left = None
        for i in idx:
            seed, (_, weight), f, d = seeds[i], starts[i], floors[i], dark[i]
            if d:
                traj, w = _zero_trajectory(solver, e_ops, opts, tlist), 0.0
            else:
                r = next(res)
                traj = solver._trajectory_resultclass(e_ops, opts)
                traj.times = [float(t) for t in tlist]
                for k, key in enumerate(traj.e_data):
                    traj.e_data[key] = list(r["expect"][:, k])
                traj.collapse = [(float(t), int(w)) for t, w in zip(r["col_times"],
                                                                      r["col_which"])]
                # MCSolver._run_one_traj scales by (1 - floor), _run_one_traj_mixed by the
                # initial state's weight (mcsolve.py:565, multitraj.py:297)
                w = weight * (1 - f)
            if reduce_func is not None:
                left = reduce_func((seed, traj, float(w)))
                if left is not None and left <= 0:
                    return None
        pos = idx.stop
        if early and left is not None and np.isfinite(left):
            chunk = max(min_chunk, int(math.ceil(left)))
        elif early:
            chunk = max(min_chunk, chunk)
    return None


gpu_map.launched_items = 0


def _sde_expect_rows(op_mats, n, open_, device):
    """Per operator E a vector w with <E> = sum_r conj(psi_r) (E psi)_r (kets: returned as
    the dense E) or Tr(E rho) = vec(E^T) . vec(rho) (column-stacked rho)."""
    out = []
    for m in op_mats:
        a = m.toarray() if sp.issparse(m) else np.asarray(m)
        herm = bool(np.allclose(a, a.conj().T, rtol=0, atol=1e-14 * max(1.0, np.abs(a).max())))
        w = a.T.reshape(-1, order="F") if open_ else a
        out.append((torch.from_numpy(np.ascontiguousarray(w, dtype=np.complex128)).to(device),
                    herm))
    return out


def _sde_expect(states, ops, open_):
    """Expectation values of every trajectory (rows of ``states``) for each operator."""
    vals = []
    for w, herm in ops:
        if open_:
            # element-wise product and row sums: a complex128 matrix-vector product through
            # torch took ~57 ms for 256 x 400 here (cuBLAS gemv path), this ~0.05 ms
            v = (states * w).sum(dim=1)
        else:
            v = (states.conj() * (states @ w.T)).sum(dim=1)
        v = v.cpu().numpy()
        vals.append(v.real.copy() if herm else v)
    return vals


def _gpu_map_sde(task, values, task_args, task_kwargs, reduce_func):
    """``map="gpu"`` for ``SSESolver`` / ``SMESolver``: every trajectory of a ``run`` in
    one ``qg_sde_platen`` launch per output interval (the reference's Platen scheme;
    ``_run_one_traj``, qutip/solver/multitraj.py:272-283).  Each trajectory's Wiener
    increments come from the reference's ``Wiener`` on the trajectory's own generator
    (``_get_generator``, multitraj.py:382-393), so the trajectories are the reference's;
    the results go to ``reduce_func`` as the reference's ``StochasticTrajResult``."""
    solver = task.__self__
    if getattr(task, "__name__", "") != "_run_one_traj":
        raise TypeError(f"map='gpu' does not run the task {getattr(task, '__name__', task)!r}")
    if task_kwargs:
        raise TypeError(f"map='gpu' does not support the trajectory options {sorted(task_kwargs)}")
    from .stochastic import SCHEMES, interval_steps
    opts = solver.options
    scheme = SCHEMES.get(opts.get("method"))
    if scheme is None:
        raise TypeError("map='gpu' integrates stochastic equations with the Platen or the "
                        "Euler-Maruyama scheme (method 'platen', 'euler', 'gpu_platen' or "
                        "'gpu_euler')")
    if opts.get("store_states") or opts.get("store_final_state"):
        raise TypeError("map='gpu' records expectation values and measurements only")
    state0, tlist, e_ops = task_args
    if isinstance(e_ops, dict):
        e_list = list(e_ops.values())
    elif e_ops is None:
        e_list = []
    elif isinstance(e_ops, (list, tuple)):
        e_list = list(e_ops)
    else:
        e_list = [e_ops]
    e_mats = [_constant_matrix(e, "e_ops") for e in e_list]
    op = sde_operator(solver.rhs)
    dt = float(solver._integrator.options["dt"])
    tl = np.asarray(tlist, dtype=np.float64)
    steps = interval_steps(tl, dt)
    total = int(sum(steps))
    m = op.n_sc
    seeds = list(values)
    n_traj = len(seeds)
    dW = np.empty((n_traj, total, m))
    for k, seed in enumerate(seeds):
        w = Wiener(float(tl[0]), dt, solver._get_generator(seed), (1, m))
        if total:
            dW[k] = w.dW(float(tl[0]), total)[:, 0, :]
    dev = _device()
    psi = _as_gpu(state0).buf
    states = psi.reshape(1, -1).repeat(n_traj, 1).contiguous()
    e_w = _sde_expect_rows(e_mats, op.n, op.open, dev)
    store_m = bool(opts.get("store_measurement"))
    m_w = _sde_expect_rows([_constant_matrix(mo, "m_ops") for mo in solver.m_ops], op.n,
                           op.open, dev) if store_m else []
    e_vals = [_sde_expect(states, e_w, op.open)]
    m_vals = [_sde_expect(states, m_w, op.open)] if store_m else []
    noise = []
    pos = 0
    for N in steps:
        if N:
            block = torch.from_numpy(np.ascontiguousarray(dW[:, pos:pos + N, :])).to(dev)
            op.advance(states, block, N, dt, scheme=scheme)
        noise.append(dW[:, pos:pos + N, :].sum(axis=1) if N else np.zeros((n_traj, 1)))
        pos += N
        e_vals.append(_sde_expect(states, e_w, op.open))
        if store_m:
            m_vals.append(_sde_expect(states, m_w, op.open))
    left = None
    for k, seed in enumerate(seeds):
        traj = solver._trajectory_resultclass(e_ops, opts)
        traj.times = [float(t) for t in tl]
        for j, key in enumerate(traj.e_data):
            traj.e_data[key] = [v[j][k] for v in e_vals]
        traj.noise = [nz[k] for nz in noise]
        if store_m:
            for j in range(len(traj.m_expect)):
                traj.m_expect[j][:] = [v[j][k] for v in m_vals]
        if reduce_func is not None:
            left = reduce_func((seed, traj, 1))
            if left is not None and left <= 0:
                break
    return None


# ---------------------------------------------------------------- register ----
_REGISTERED = False


def register():
    """Register the data type, specialisations, integrator and map (idempotent)."""
    global _REGISTERED
    if _REGISTERED:
        return
    _lib.load()
    _data.to.add_conversions([
        (GpuDense, Dense, _dense_to_gpu, 1),
        (Dense, GpuDense, _gpu_to_dense, 1),
    ])
    _data.to.register_aliases(["gpu", "GpuDense", "gpudense"], GpuDense)
    _data.zeros.add_specialisations([(GpuDense, zeros_gpu)])
    _data.matmul.add_specialisations([
        (CSR, GpuDense, GpuDense, matmul_csr_gpu),
        (Dia, GpuDense, GpuDense, matmul_dia_gpu),
        (GpuDense, GpuDense, GpuDense, matmul_gpu),
    ])
    _data.add.add_specialisations([(GpuDense, GpuDense, GpuDense, add_gpu)])
    _data.iadd.add_specialisations([(GpuDense, GpuDense, GpuDense, iadd_gpu)])
    _data.sub.add_specialisations([(GpuDense, GpuDense, GpuDense, sub_gpu)])
    _data.mul.add_specialisations([(GpuDense, GpuDense, mul_gpu)])
    _data.imul.add_specialisations([(GpuDense, GpuDense, imul_gpu)])
    _data.neg.add_specialisations([(GpuDense, GpuDense, neg_gpu)])
    # Dia operators go through the same expect kernels (converted once, cached)
    _data.expect.add_specialisations([(CSR, GpuDense, expect_csr_gpu),
                                      (Dia, GpuDense, expect_csr_gpu)])
    _data.expect_super.add_specialisations([(CSR, GpuDense, expect_super_csr_gpu),
                                            (Dia, GpuDense, expect_super_csr_gpu)])
    _data.trace.add_specialisations([(GpuDense, trace_gpu)])
    _data.trace_oper_ket.add_specialisations([(GpuDense, trace_oper_ket_gpu)])
    _data.norm.l2.add_specialisations([(GpuDense, l2_gpu)])
    _data.norm.frobenius.add_specialisations([(GpuDense, frobenius_gpu)])
    _data.column_stack.add_specialisations([(GpuDense, GpuDense, column_stack_gpu)])
    _data.column_unstack.add_specialisations([(GpuDense, GpuDense, column_unstack_gpu)])
    _data.inner.add_specialisations([(GpuDense, GpuDense, inner_gpu)])
    _ode.wrmn_error.add_specialisations([(GpuDense, GpuDense, wrmn_error_gpu)])
    _data.isherm.add_specialisations([(GpuDense, isherm_gpu)])
    _data.adjoint.add_specialisations([(GpuDense, GpuDense, adjoint_gpu)])
    _data.conj.add_specialisations([(GpuDense, GpuDense, conj_gpu)])
    _data.transpose.add_specialisations([(GpuDense, GpuDense, transpose_gpu)])
    for solver in (MESolver, SESolver, MCSolver, BRSolver):
        solver.add_integrator(IntegratorGpuVern7, "gpu_vern7")
    StochasticSolver.add_integrator(IntegratorGpuPlaten, "gpu_platen")
    StochasticSolver.add_integrator(IntegratorGpuEuler, "gpu_euler")
    _parallel._maps["gpu"] = gpu_map
    _REGISTERED = True


register()
