"""Host drivers: ``mesolve``-style evolution of one system on the GPU.

``mesolve`` mirrors the reference's ``Solver.run`` (qutip/solver/solver_base.py:159-226)
for the master equation: integrate to each output time, normalise the output by
the trace when the initial trace is 1 (``_restore_state``, :138-157) and record
``tr(op rho)`` for every e_op (``Result.add`` -> ``expect``, qutip/core/expect.py:91).
Expectation values are evaluated on the device directly from the interpolated
Runge-Kutta data (only the entries each e_op touches are formed) into a device
array that is read back once at the end.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from .coefficients import Coefficient, coefficient
from .lindblad import LindbladOperator
from .operator import DeviceOperator, stream_ptr
from .systems import OpenSystem, lindblad_dissipator, merge_terms, spost, spre
from .vern7 import GpuVern7, PRECISIONS

__all__ = ["MEResult", "mesolve", "solve_system", "liouvillian_terms", "ExpectOps"]

ME_DEFAULTS = dict(atol=1e-8, rtol=1e-6, nsteps=1000, first_step=0.0, min_step=0.0,
                   max_step=0.0, interpolate=True, precision="double", store_states=False,
                   store_final_state=False, normalize_output=True, matrix_form=False,
                   hermitian_branch="auto")


@dataclass
class MEResult:
    times: np.ndarray
    expect: list
    states: list = field(default_factory=list)
    final_state: np.ndarray | None = None
    stats: dict = field(default_factory=dict)


class ExpectOps:
    """e_ops resident on the device, one CSR group per operator."""

    def __init__(self, e_ops, dtype="c128", device="cuda"):
        self.ops = [sp.csr_matrix(o) for o in e_ops]
        self.n = len(self.ops)
        if self.n > _lib.QG_MAX_EOPS:
            raise ValueError(f"at most {_lib.QG_MAX_EOPS} e_ops per launch")
        # each operator is its own CSR group (no merging, coefficient 1)
        self.dev = _wide_groups(self.ops, dtype, device) if self.n else None

    def expect_dm(self, d: int, view: _lib.StateView, out: torch.Tensor):
        _lib.call("qg_expect_dm", C.byref(self.dev.struct), d, C.byref(view), out.data_ptr(),
                  stream_ptr())

    def expect_ket(self, view: _lib.StateView, out: torch.Tensor):
        _lib.call("qg_expect_ket", C.byref(self.dev.struct), C.byref(view), out.data_ptr(),
                  stream_ptr())


def _wide_groups(ops, dtype, device):
    """A DeviceOperator-like holder with up to QG_MAX_EOPS groups (expect only)."""
    class _Wide:
        pass
    w = _Wide()
    rps, cols, vals, off = [], [], [], 0
    for o in ops:
        m = sp.csr_matrix(o, dtype=np.complex128)
        m.sort_indices()
        rps.append(m.indptr.astype(np.int64) + off)
        cols.append(m.indices.astype(np.int32))
        vals.append(m.data)
        off += m.nnz
    tdt = torch.complex128 if dtype == "c128" else torch.complex64
    w.row_ptr = torch.from_numpy(np.concatenate(rps).astype(np.int32)).to(device)
    w.col = torch.from_numpy(np.concatenate(cols)).to(device)
    w.val = torch.from_numpy(np.concatenate(vals)).to(device, tdt)
    n = ops[0].shape[0]
    w.struct = _lib.CsrGroups(n, n, len(ops), 0 if dtype == "c128" else 1,
                              _lib.QG_LAYOUT_GROUP_MAJOR, 1, 0, 0, w.row_ptr.data_ptr(),
                              w.col.data_ptr(), w.val.data_ptr(), None, None, None, None)
    return w


def _as_terms(H, args=None):
    """H as a list of (matrix, Coefficient|None); accepts QobjEvo-like list syntax."""
    if isinstance(H, (list, tuple)):
        out = []
        for item in H:
            if isinstance(item, (list, tuple)):
                op, c = item
                out.append((sp.csr_matrix(op), c if isinstance(c, Coefficient)
                            else coefficient(c, args)))
            else:
                out.append((sp.csr_matrix(item), None))
        return out
    return [(sp.csr_matrix(H), None)]


def liouvillian_terms(H, c_ops=(), args=None):
    """Liouvillian terms of ``H`` (matrix or list form) and constant collapse operators."""
    terms = [((-1j) * (spre(h) - spost(h)), c) for h, c in _as_terms(H, args)]
    for c in c_ops:
        terms.append((lindblad_dissipator(sp.csr_matrix(c)), None))
    return merge_terms(terms)


def _evolve(ig: GpuVern7, tlist, ex: ExpectOps, d: int, store_states, store_final, normalize,
            kind="me"):
    nt = len(tlist)
    G = ex.n
    raw = torch.zeros((nt, 2 * (G + 1)), dtype=torch.float64, device=ig.op.device)
    states = []

    def record(i):
        if G:
            if kind == "me":
                ex.expect_dm(d, ig.state_view(), raw[i])
            else:
                ex.expect_ket(ig.state_view(), raw[i])
        if store_states:
            states.append(ig.get_state().clone())

    record(0)
    for i in range(1, nt):
        ig.integrate(float(tlist[i]))
        ig.check()
        record(i)
    final = ig.get_state().clone() if store_final else None
    r = raw.cpu().numpy()
    vals = r[:, 0:2 * G:2] + 1j * r[:, 1:2 * G:2]
    norm = r[:, 2 * G] + 1j * r[:, 2 * G + 1]
    if G and normalize:
        vals = vals / norm[:, None]
    return [vals[:, k] for k in range(G)], states, final, norm


def solve_system(system: OpenSystem, tlist, options=None, op: DeviceOperator | None = None,
                 ex: ExpectOps | None = None) -> MEResult:
    """Evolve an :class:`~qutip_gb300.systems.OpenSystem` of kind ``"me"``.

    ``matrix_form=True`` applies the Lindblad generator without its superoperator
    (:class:`~qutip_gb300.lindblad.LindbladOperator`, from the system's ``h_terms`` and
    ``c_ops``), as the reference's ``matrix_form`` option (qutip/solver/mesolve.py:251-266).
    """
    opt = {**ME_DEFAULTS, **(options or {})}
    prec = opt["precision"]
    if prec not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
    stage_dt = PRECISIONS[prec][1]
    t0 = time.perf_counter()
    if op is None and opt["matrix_form"]:
        if not system.h_terms:
            raise ValueError("matrix_form needs the system's Hamiltonian terms")
        op = LindbladOperator.from_hamiltonian(system.h_terms, system.c_ops, dtype=stage_dt)
    elif op is None:
        op = DeviceOperator(system.terms, dtype=stage_dt)
    if ex is None:
        ex = ExpectOps(system.e_ops)
    ig = GpuVern7(op, atol=opt["atol"], rtol=opt["rtol"], nsteps=opt["nsteps"],
                  first_step=opt["first_step"], min_step=opt["min_step"],
                  max_step=opt["max_step"], interpolate=opt["interpolate"], precision=prec)
    rho0 = np.asarray(system.state0, dtype=np.complex128)
    d = system.dim
    if isinstance(op, LindbladOperator):
        # the reference's branch: A + A^dag when rho0 is Hermitian (mesolve.py:270-277;
        # Qobj.isherm at the default atol 1e-12)
        r = rho0.reshape(d, d, order="F")
        branch = opt.get("hermitian_branch", "auto")
        op.hermitian = bool(np.all(np.abs(r - r.conj().T) <= 1e-12)) and (
            branch is True or (branch == "auto" and op.hermitian_pays()))
    tr0 = np.trace(rho0.reshape(d, d, order="F"))
    normalize = opt["normalize_output"] and abs(tr0 - 1) <= 1e-12
    ig.set_initial_value(torch.from_numpy(rho0).to(op.device), float(tlist[0]))
    prep = time.perf_counter() - t0
    expect, states, final, _ = _evolve(ig, tlist, ex, d, opt["store_states"],
                                       opt["store_final_state"], normalize)
    if normalize and final is not None:
        final = final / torch.trace(final.reshape(d, d).T)
    res = MEResult(np.asarray(tlist), expect,
                   [s.cpu().numpy() for s in states],
                   None if final is None else final.cpu().numpy(),
                   {"preparation time": prep, "run time": time.perf_counter() - t0 - prep,
                    **ig.stats, "method": f"gpu_vern7[{prec}]"})
    return res


def mesolve(H, rho0, tlist, c_ops=None, e_ops=None, args=None, options=None) -> MEResult:
    """Lindblad master equation on the GPU, ``mesolve``'s calling convention
    (qutip/solver/mesolve.py:24-166) with numpy/scipy inputs.

    ``H`` is a matrix or a list ``[H0, [H1, coeff], ...]`` with string/number
    coefficients; ``rho0`` a ket or a density matrix; ``e_ops`` matrices.
    """
    c_ops = list(c_ops or [])
    rho0 = np.asarray(rho0, dtype=np.complex128)
    if rho0.ndim == 1 or rho0.shape[1] == 1:
        psi = rho0.reshape(-1)
        rho0 = np.outer(psi, psi.conj())
    d = rho0.shape[0]
    if (options or {}).get("matrix_form"):
        system = OpenSystem("user", "me", d, None, rho0.reshape(-1, order="F").copy(),
                            list(e_ops or []), [sp.csr_matrix(c) for c in c_ops],
                            _as_terms(H, args))
    else:
        system = OpenSystem("user", "me", d, liouvillian_terms(H, c_ops, args),
                            rho0.reshape(-1, order="F").copy(), list(e_ops or []))
    return solve_system(system, tlist, options)
