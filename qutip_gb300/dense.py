"""Dense small-dimension bucket: the Lindblad generator of a small system with dense
operators, applied as GEMMs on the tensor cores.

The reference's matrix form (``LindbladMatrixForm``,
qutip/core/cy/lindblad_matrix_form.pyx:105-204) applies ``A rho + rho A^dag +
sum_i C_i rho C_i^dag`` with ``A = -i H_nh`` through sparse or dense matmuls.  For a
system of Hilbert dimension ``d <= 128`` whose operators are dense, those products are
small dense GEMMs: :class:`DenseLindbladOperator` keeps ``A_g`` and ``C_i`` as complex64
``d x d`` matrices and applies the generator in one CTA with ``tcgen05`` tensor-core
MMAs (TF32 inputs split hi + lo, FP32 accumulation in tensor memory; ``qg_dense_lindblad_*``
in ``csrc/dense.cu``; one CTA per 16 output columns; each K chunk of 32 in fresh
accumulators, the large hi*hi part and the small hi*lo + lo*hi corrections apart, summed
on the CUDA cores with round-to-nearest).  The stages are
complex64, so it serves the mixed form
(``precision="mixed"``: FP64 state, step control and expectation values).

Sparse operators (a Jaynes-Cummings system has three entries per row) keep the sparse
paths: a dense GEMM multiplies every zero, so :func:`dense_fill` gates the bucket.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from .coefficients import pack_programs
from .operator import stream_ptr

__all__ = ["DenseLindbladOperator", "dense_fill", "DENSE_FILL"]

#: fraction of nonzero entries of A = -i H_nh and the collapse operators from which the
#: dense bucket takes a matrix-form generator (below it the sparse kernels do less work)
DENSE_FILL = 0.5


def dense_fill(mats) -> float:
    """Nonzero fraction of the union of the matrices' patterns."""
    mats = [sp.csr_matrix(m) for m in mats]
    d = mats[0].shape[0]
    pattern = sum((abs(m) > 0).astype(np.int8) for m in mats)
    return sp.csr_matrix(pattern).nnz / float(d * d)


def _ptr(t):
    return None if t is None else t.data_ptr()


class DenseLindbladOperator:
    """``L(t)[rho] = A(t) rho + rho A(t)^dag + sum_i |f_i(t)|^2 C_i rho C_i^dag`` for
    ``d <= 128`` with dense complex64 operators, on ``vec(rho)`` (column-stacked, length
    ``d*d``), for :class:`qutip_gb300.vern7.GpuVern7` (``precision="mixed"``).

    ``a_terms``: ``[(A_g, Coefficient | None)]`` with ``A = sum_g a_g(t) A_g = -i H_nh``;
    ``c_terms``: ``[(C_i, Coefficient | None)]`` (the coefficient multiplies C_i)."""

    def __init__(self, a_terms, c_terms, device="cuda"):
        if not a_terms:
            raise ValueError("the generator needs at least one A term")
        d = a_terms[0][0].shape[0]
        if not 1 <= d <= _lib.QG_DENSE_MAX_D:
            raise ValueError(f"the dense bucket takes 1 <= d <= {_lib.QG_DENSE_MAX_D}, not {d}")
        if len(a_terms) > _lib.QG_MAX_GROUPS or len(c_terms) > _lib.QG_MAX_COPS:
            raise ValueError("too many coefficient groups or collapse operators")
        self.d = d
        self.n_rows = self.n_cols = d * d
        self.shape = (d * d, d * d)
        self.dtype = "c64"
        self.device = torch.device(device)
        self.fmt = "dense"

        def dense(m):
            a = m.toarray() if sp.issparse(m) else np.asarray(m)
            if a.shape != (d, d):
                raise ValueError("all operators must be d x d")
            return a.astype(np.complex64)
        self.a_coeffs = [c for _, c in a_terms]
        self.c_coeffs = [c for _, c in c_terms]
        self.a = torch.from_numpy(np.stack([dense(m) for m, _ in a_terms])).to(self.device)
        self.c = (torch.from_numpy(np.stack([dense(m) for m, _ in c_terms])).to(self.device)
                  if c_terms else None)
        self._a_prog = self._programs(self.a_coeffs)
        self._c_prog = self._programs(self.c_coeffs)
        self.coeffs = self.a_coeffs + self.c_coeffs
        st = _lib.DenseLindblad()
        st.d, st.n_groups, st.n_cops, st.reserved = d, len(a_terms), len(c_terms), 0
        st.a, st.c = _ptr(self.a), _ptr(self.c)
        st.a_coef_code, st.a_coef_start, st.a_coef_consts = (_ptr(v) for v in self._a_prog)
        st.c_coef_code, st.c_coef_start, st.c_coef_consts = (_ptr(v) for v in self._c_prog)
        self.struct = st

    def _programs(self, coeffs):
        if all(c is None for c in coeffs):
            return (None, None, None)
        code, starts, consts = pack_programs(coeffs)
        return tuple(torch.from_numpy(a).to(self.device) for a in (code, starts, consts))

    @classmethod
    def from_hamiltonian(cls, h_terms, c_ops, device="cuda"):
        """From ``H(t) = sum_g h_g(t) H_g`` and collapse operators (matrices or
        ``(matrix, Coefficient | None)`` pairs): A = -i H - 1/2 sum_i |f_i|^2 C_i^dag C_i,
        as LindbladMatrixForm builds H_nh (lindblad_matrix_form.pyx:88-96)."""
        cops = [c if isinstance(c, tuple) else (c, None) for c in c_ops]
        a_terms = [((-1j) * sp.csr_matrix(h), c) for h, c in h_terms]
        for m, f in cops:
            m = sp.csr_matrix(m)
            a_terms.append((-0.5 * (m.conj().T @ m), None if f is None else f.conj() * f))
        return cls(a_terms, [(sp.csr_matrix(m), f) for m, f in cops], device=device)

    # -- the integrator's view --------------------------------------------------------
    @property
    def n_groups(self) -> int:
        return len(self.a_coeffs)

    @property
    def n_cops(self) -> int:
        return len(self.c_coeffs)

    @property
    def isconstant(self) -> bool:
        return all(c is None for c in self.coeffs)

    @property
    def launch(self):
        return ("dense", 0, 1)

    def launch_desc(self) -> str:
        return (f"dense tensor-core Lindblad (d={self.d}, {self.n_groups} A groups, "
                f"{self.n_cops} collapse operators, tcgen05 TF32x3)")

    def tune(self, *args, **kwargs):
        return self.launch

    def value_bytes(self) -> int:
        return 8

    def operator_bytes(self) -> int:
        """Bytes of the dense operators (complex64)."""
        return 8 * self.d * self.d * (self.n_groups + self.n_cops)

    @property
    def n_ctas(self) -> int:
        """CTAs (one per SM) of one application: one per 16 output columns."""
        return (self.d + 15) // 16

    def gemm_flops(self) -> int:
        """Real multiply-adds x 2 of one application as issued: per complex product of two
        d x d matrices (padded to 128 rows, 16-column blocks, 8-wide K steps) four real
        products in three TF32 terms."""
        d = self.d
        np_ = (d + 15) // 16 * 16
        k = (d + 7) // 8 * 8
        products = 2 + 2 * self.n_cops
        return 2 * 128 * np_ * k * 12 * products

    def matvec(self, t: float, x: torch.Tensor, y: torch.Tensor, alpha=1.0, beta=0.0):
        """``y = alpha * L(t)[x] + beta * y`` (complex64 vec(rho))."""
        if x.numel() != self.n_rows or y.numel() != self.n_rows:
            raise ValueError("vector length must be d*d")
        if x.dtype != torch.complex64 or y.dtype != torch.complex64:
            raise TypeError("the dense bucket applies to complex64 vectors")
        a, b = complex(alpha), complex(beta)
        _lib.call("qg_dense_lindblad_apply", C.byref(self.struct), float(t), x.data_ptr(),
                  y.data_ptr(), a.real, a.imag, b.real, b.imag, stream_ptr())

    def vern7_stage(self, rk, stage: int, t_prev: float, dt: float, atol: float, rtol: float,
                    stream: int):
        lib = _lib.load()
        _lib.check(lib.qg_dense_lindblad_stage(C.byref(self.struct), C.byref(rk), stage, t_prev,
                                               dt, atol, rtol, stream), "qg_dense_lindblad_stage")
