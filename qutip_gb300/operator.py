"""Device-resident operators: coefficient-grouped CSR and Dia matrices in HBM.

A :class:`DeviceOperator` is the GPU form of a ``QobjEvo`` generator
(qutip/core/cy/qobjevo.pyx:189-245): its terms are merged per coefficient
(``QobjEvo.compress``, qobjevo.pyx:816) and stored as one set of concatenated
CSR arrays -- ``row_ptr`` int32 ``[G, n+1]`` (absolute offsets), ``col`` int32
``[nnz]`` and ``val`` complex128 or complex64 ``[nnz]`` -- plus the coefficient
programs the kernels evaluate on the device.  Layout and index width follow the
reference's CSR (qutip/core/data/csr.pxd:17-30, 32-bit ``idxint``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from .coefficients import Coefficient, pack_programs
from .systems import merge_terms

__all__ = ["DeviceOperator", "DeviceDia", "torch_dtype", "qg_dtype"]

_TORCH = {"c128": torch.complex128, "c64": torch.complex64}
_QG = {"c128": _lib.QG_C128, "c64": _lib.QG_C64}


def torch_dtype(dt: str):
    return _TORCH[dt]


def qg_dtype(dt: str) -> int:
    return _QG[dt]


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


class DeviceOperator:
    """``A(t) = sum_g c_g(t) A_g`` resident on the GPU.

    ``terms`` is a list of ``(scipy matrix, Coefficient | None)``.
    """

    def __init__(self, terms, dtype: str = "c128", device="cuda", merge: bool = True):
        if dtype not in _TORCH:
            raise TypeError(f"unsupported dtype {dtype!r}")
        terms = merge_terms(terms) if merge else [(sp.csr_matrix(o), c) for o, c in terms]
        if not terms:
            raise ValueError("operator needs at least one term")
        if len(terms) > _lib.QG_MAX_GROUPS:
            raise ValueError(f"at most {_lib.QG_MAX_GROUPS} coefficient groups are supported")
        shape = terms[0][0].shape
        for op, c in terms:
            if op.shape != shape:
                raise ValueError("all terms must have the same shape")
            if c is not None and not isinstance(c, Coefficient):
                raise TypeError("coefficients must be qutip_gb300.coefficients.Coefficient")
        self.shape = shape
        self.n_rows, self.n_cols = shape
        self.dtype = dtype
        self.coeffs = [c for _, c in terms]
        self.device = torch.device(device)
        rps, cols, vals = [], [], []
        off = 0
        for op, _ in terms:
            m = sp.csr_matrix(op, dtype=np.complex128)
            m.sort_indices()
            rps.append(m.indptr.astype(np.int64) + off)
            cols.append(m.indices.astype(np.int32))
            vals.append(m.data)
            off += m.nnz
        if off >= 2**31:
            raise ValueError("operators beyond 2^31 stored entries need 64-bit indices")
        self.nnz = off
        self.group_nnz = [len(c) for c in cols]
        self.row_ptr = torch.from_numpy(np.concatenate(rps).astype(np.int32)).to(self.device)
        self.col = torch.from_numpy(np.concatenate(cols)).to(self.device)
        self.val = torch.from_numpy(np.concatenate(vals)).to(self.device, _TORCH[dtype])
        if all(c is None for c in self.coeffs):
            self.coef_code = self.coef_start = self.coef_consts = None
        else:
            code, starts, consts = pack_programs(self.coeffs)
            self.coef_code = torch.from_numpy(code).to(self.device)
            self.coef_start = torch.from_numpy(starts).to(self.device)
            self.coef_consts = torch.from_numpy(consts).to(self.device)
        self.struct = _lib.CsrGroups(
            self.n_rows, self.n_cols, len(terms), _QG[dtype], _ptr(self.row_ptr), _ptr(self.col),
            _ptr(self.val), _ptr(self.coef_code), _ptr(self.coef_start), _ptr(self.coef_consts))
        self.lanes = self.default_lanes()

    def device_arrays(self):
        return [t for t in (self.row_ptr, self.col, self.val, self.coef_code, self.coef_start,
                            self.coef_consts) if t is not None]

    def host_copy(self, pinned: bool = True):
        """Host copies of the device arrays (pinned), for end-to-end transfer timing."""
        out = []
        for t in self.device_arrays():
            h = torch.empty(t.shape, dtype=t.dtype, pin_memory=pinned)
            h.copy_(t)
            out.append(h)
        return out

    def upload(self, host_arrays) -> int:
        """Copy host arrays (from :meth:`host_copy`) into the resident device arrays."""
        nbytes = 0
        for d, h in zip(self.device_arrays(), host_arrays):
            d.copy_(h, non_blocking=True)
            nbytes += h.numel() * h.element_size()
        return nbytes

    @property
    def n_groups(self) -> int:
        return len(self.coeffs)

    @property
    def isconstant(self) -> bool:
        return all(c is None for c in self.coeffs)

    def default_lanes(self) -> int:
        """Threads per row: the power of two nearest half the largest group's mean row length."""
        mean = max(g / max(self.n_rows, 1) for g in self.group_nnz)
        lanes = 2
        while lanes < 32 and lanes * 2 <= max(mean / 1.5, 2):
            lanes *= 2
        return lanes

    def value_bytes(self) -> int:
        return 16 if self.dtype == "c128" else 8

    def spmv_bytes(self, accumulate: bool = False) -> int:
        """Algorithmic HBM bytes of one matvec: values + indices + row pointers + x + y."""
        sv, sx = self.value_bytes(), self.value_bytes()
        return (self.nnz * (sv + 4) + self.n_groups * (self.n_rows + 1) * 4 + self.n_cols * sx
                + self.n_rows * sx * (2 if accumulate else 1))

    def matvec(self, t: float, x: torch.Tensor, y: torch.Tensor, alpha=1.0, beta=0.0,
               lanes: int | None = None):
        """``y = alpha A(t) x + beta y`` on the current stream (vectors in ``self.dtype``)."""
        if x.dtype != _TORCH[self.dtype] or y.dtype != _TORCH[self.dtype]:
            raise TypeError("vector dtype must match the operator dtype")
        if x.numel() != self.n_cols or y.numel() != self.n_rows:
            raise ValueError("incompatible shapes")
        if not (x.is_contiguous() and y.is_contiguous()):
            raise ValueError("vectors must be contiguous")
        a, b = complex(alpha), complex(beta)
        _lib.call("qg_spmv_csr", C.byref(self.struct), float(t), x.data_ptr(), y.data_ptr(),
                  a.real, a.imag, b.real, b.imag, int(lanes or self.lanes), stream_ptr())
        return y

    def matmat(self, t: float, X: torch.Tensor, Y: torch.Tensor, alpha=1.0, beta=0.0):
        """``Y = alpha A(t) X + beta Y`` for F-ordered column blocks stored as ``[n_vec, n]``."""
        if X.dtype != _TORCH[self.dtype] or Y.dtype != _TORCH[self.dtype]:
            raise TypeError("vector dtype must match the operator dtype")
        if X.dim() != 2 or X.shape[1] != self.n_cols or Y.shape != (X.shape[0], self.n_rows):
            raise ValueError("incompatible shapes")
        a, b = complex(alpha), complex(beta)
        _lib.call("qg_spmm_csr", C.byref(self.struct), float(t), X.data_ptr(), Y.data_ptr(),
                  X.shape[0], X.stride(0), a.real, a.imag, b.real, b.imag, stream_ptr())
        return Y

    def tune_lanes(self, candidates=(2, 4, 8, 16, 32), reps: int = 5) -> int:
        """Time the matvec for each sub-warp width on this device and keep the fastest."""
        x = torch.randn(self.n_cols, dtype=_TORCH[self.dtype], device=self.device)
        y = torch.empty(self.n_rows, dtype=_TORCH[self.dtype], device=self.device)
        best, best_t = self.lanes, float("inf")
        for lanes in candidates:
            self.matvec(0.37, x, y, lanes=lanes)
            st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            st.record()
            for _ in range(reps):
                self.matvec(0.37, x, y, lanes=lanes)
            en.record()
            en.synchronize()
            ms = st.elapsed_time(en) / reps
            if ms < best_t:
                best, best_t = lanes, ms
        self.lanes = best
        return best


class DeviceDia:
    """A Dia matrix (qutip/core/data/dia.pxd:17-38) resident on the GPU."""

    def __init__(self, mat, dtype: str = "c128", device="cuda"):
        m = sp.dia_matrix(mat)
        m.sum_duplicates()
        self.shape = m.shape
        self.dtype = dtype
        n_cols = m.shape[1]
        data = np.zeros((len(m.offsets), n_cols), dtype=np.complex128)
        data[:, : min(n_cols, m.data.shape[1])] = m.data[:, :n_cols]
        self.offsets = torch.from_numpy(m.offsets.astype(np.int32)).to(device)
        self.data = torch.from_numpy(data).to(device, _TORCH[dtype])
        self.struct = _lib.Dia(m.shape[0], m.shape[1], len(m.offsets), _QG[dtype],
                               _ptr(self.offsets), _ptr(self.data))

    def matvec(self, x: torch.Tensor, y: torch.Tensor, alpha=1.0, beta=0.0):
        if x.numel() != self.shape[1] or y.numel() != self.shape[0]:
            raise ValueError("incompatible shapes")
        a, b = complex(alpha), complex(beta)
        _lib.call("qg_spmv_dia", C.byref(self.struct), x.data_ptr(), y.data_ptr(), a.real, a.imag,
                  b.real, b.imag, stream_ptr())
        return y
