"""The Lindblad generator on the device without its superoperator.

The reference's matrix form (``mesolve(..., options={"matrix_form": True})``,
qutip/solver/mesolve.py:251-266; qutip/core/cy/lindblad_matrix_form.pyx:105-204)
keeps rho as a d x d matrix and evaluates

    L[rho] = A rho + rho A^dag + sum_i |f_i(t)|^2 C_i rho C_i^dag,
    A = -i H_nh,   H_nh = H - (i/2) sum_i |f_i(t)|^2 C_i^dag C_i,

with matrix products.  Here one kernel (``qg_lindblad_apply`` / ``qg_lindblad_stage``)
evaluates every element of L[rho] from the d x d operators and vec(rho) directly, so a
stage reads the small operators (L1-resident) and the state (L2-resident) instead of
streaming a d^2 x d^2 superoperator from HBM.  The state is vec(rho) in column-major
order, the same vector as the superoperator form, so the integrator, the expectation
values and the outputs are shared with it.

The reference computes ``A + A^dag`` when rho is Hermitian and the full form otherwise
(lindblad_matrix_form.pyx:160-200); both are the same generator and this kernel always
evaluates the full form, which also evolves non-Hermitian rho.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from .coefficients import Coefficient, pack_programs
from .operator import DeviceOperator, _ptr, _QG, _TORCH, stream_ptr

__all__ = ["LindbladOperator"]


class LindbladOperator:
    """Matrix-free Lindblad generator acting on vec(rho) (length d*d).

    ``a_terms``: ``[(d x d matrix, Coefficient | None)]``, the terms of A = -i H_nh.
    ``c_terms``: ``[(d x d matrix, Coefficient | None)]``, one per collapse operator
    f_i(t) C_i.  Exposes the interface the Vern7 driver uses (``n_rows``, ``dtype``,
    ``device``, ``matvec``, ``vern7_stage``).
    """

    def __init__(self, a_terms, c_terms, dtype: str = "c128", device="cuda"):
        if dtype not in _TORCH:
            raise TypeError(f"unsupported dtype {dtype!r}")
        if not a_terms:
            raise ValueError("the generator needs at least one Hamiltonian term")
        if len(c_terms) > _lib.QG_MAX_COPS:
            raise ValueError(f"at most {_lib.QG_MAX_COPS} collapse operators")
        d = a_terms[0][0].shape[0]
        for m, c in list(a_terms) + list(c_terms):
            if m.shape != (d, d):
                raise ValueError("all operators must be d x d")
            if c is not None and not isinstance(c, Coefficient):
                raise TypeError("coefficients must be qutip_gb300.coefficients.Coefficient")
        if d * d >= 2**31:
            raise ValueError("d*d must stay below 2^31")
        self.d = d
        self.n_rows = self.n_cols = d * d
        self.shape = (d * d, d * d)
        self.dtype = dtype
        self.device = torch.device(device)
        self.fmt = "lindblad"
        self.a_terms = [(sp.csr_matrix(m), c) for m, c in a_terms]
        self.c_terms = [(sp.csr_matrix(m), c) for m, c in c_terms]
        self.a = DeviceOperator(a_terms, dtype=dtype, device=device, fmt="csr")
        self.coeffs = list(self.a.coeffs) + [c for _, c in c_terms]
        mats = [sp.csr_matrix(m, dtype=np.complex128) for m, _ in c_terms]
        for m in mats:
            m.sort_indices()
        self.n_cops = len(mats)
        self.c_coeffs = [c for _, c in c_terms]
        self.c_nnz = [int(m.nnz) for m in mats]
        P = DeviceOperator.PAD
        if mats:
            rps, off = [], 0
            for m in mats:
                rps.append(m.indptr.astype(np.int64) + off)
                off += m.nnz
            rp = np.concatenate(rps)
            if rp[-1] >= 2**31 - 16:
                raise ValueError("collapse operators beyond 2^31 entries")
            self.c_row_ptr = torch.from_numpy(rp.astype(np.int32)).to(self.device)
            col = np.concatenate([m.indices.astype(np.int32) for m in mats] + [np.zeros(P, np.int32)])
            val = np.concatenate([m.data for m in mats] + [np.zeros(P, np.complex128)])
            self.c_col = torch.from_numpy(col).to(self.device)
            self.c_val = torch.from_numpy(val).to(self.device, _TORCH[dtype])
        else:
            self.c_row_ptr = self.c_col = self.c_val = None
        if any(c is not None for c in self.c_coeffs):
            code, starts, consts = pack_programs(self.c_coeffs)
            self.c_code = torch.from_numpy(code).to(self.device)
            self.c_start = torch.from_numpy(starts).to(self.device)
            self.c_consts = torch.from_numpy(consts).to(self.device)
        else:
            self.c_code = self.c_start = self.c_consts = None
        self.struct = self._make_struct()

    def _make_struct(self) -> _lib.Lindblad:
        a = self.a
        d = self.d
        a_s = _lib.CsrGroups(d, d, a.n_groups, _QG[self.dtype], _lib.QG_LAYOUT_ROW_MAJOR,
                             1, 0, 0, _ptr(a.row_ptr), _ptr(a.col), _ptr(a.val), None,
                             _ptr(a.coef_code), _ptr(a.coef_start), _ptr(a.coef_consts))
        c_s = _lib.CsrGroups(d, d, self.n_cops, _QG[self.dtype], _lib.QG_LAYOUT_GROUP_MAJOR, 1, 0,
                             0, _ptr(self.c_row_ptr), _ptr(self.c_col), _ptr(self.c_val), None,
                             _ptr(self.c_code), _ptr(self.c_start), _ptr(self.c_consts))
        return _lib.Lindblad(d, a_s, c_s)

    # -- constructors -------------------------------------------------------
    @classmethod
    def from_hamiltonian(cls, h_terms, c_ops, dtype: str = "c128", device="cuda"):
        """From ``H(t) = sum_g h_g(t) H_g`` (``[(matrix, Coefficient | None)]``) and the
        collapse operators (matrices, or ``(matrix, Coefficient | None)`` pairs):
        A = -i H - 1/2 sum_i |f_i|^2 C_i^dag C_i, as LindbladMatrixForm builds H_nh
        (lindblad_matrix_form.pyx:88-96)."""
        cops = [c if isinstance(c, tuple) else (c, None) for c in c_ops]
        a_terms = [((-1j) * sp.csr_matrix(h), c) for h, c in h_terms]
        for m, f in cops:
            m = sp.csr_matrix(m)
            a_terms.append((-0.5 * (m.conj().T @ m), None if f is None else f.conj() * f))
        return cls(a_terms, [(sp.csr_matrix(m), f) for m, f in cops], dtype=dtype, device=device)

    # -- properties ---------------------------------------------------------
    @property
    def n_groups(self) -> int:
        return self.a.n_groups

    @property
    def isconstant(self) -> bool:
        return all(c is None for c in self.coeffs)

    @property
    def launch(self):
        return ("lindblad", 0, 1)

    def launch_desc(self) -> str:
        return f"matrix-free Lindblad (d={self.d}, {self.n_cops} collapse operators)"

    def tune(self, *args, **kwargs):
        """One launch shape (one thread per element, grid from the occupancy query)."""
        return self.launch

    def value_bytes(self) -> int:
        es = 16 if self.dtype == "c128" else 8
        return (self.a.stored + sum(self.c_nnz)) * (es + 4)

    def state_bytes(self) -> int:
        """Bytes of one vec(rho) in the stage dtype."""
        return self.n_rows * (16 if self.dtype == "c128" else 8)

    # -- application --------------------------------------------------------
    def matvec(self, t: float, x: torch.Tensor, y: torch.Tensor, alpha=1.0, beta=0.0):
        """``y = alpha * L(t)[x] + beta * y`` (x, y: vec(rho) in this dtype)."""
        if x.numel() != self.n_rows or y.numel() != self.n_rows:
            raise ValueError("vector length must be d*d")
        a, b = complex(alpha), complex(beta)
        _lib.call("qg_lindblad_apply", C.byref(self.struct), float(t), x.data_ptr(), y.data_ptr(),
                  a.real, a.imag, b.real, b.imag, stream_ptr())

    def vern7_stage(self, rk, stage: int, t_prev: float, dt: float, atol: float, rtol: float,
                    stream: int):
        lib = _lib.load()
        _lib.check(lib.qg_lindblad_stage(C.byref(self.struct), C.byref(rk), stage, t_prev, dt,
                                         atol, rtol, stream), "qg_lindblad_stage")
