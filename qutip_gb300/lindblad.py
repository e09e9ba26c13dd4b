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
(lindblad_matrix_form.pyx:160-200).  ``hermitian = True`` is that branch here: the kernel
evaluates the elements on and below the diagonal only and writes each one's conjugate to
its mirror (real diagonal), half the generator's work; ``False`` evaluates every element
and also evolves non-Hermitian rho.  Both give the same generator on a Hermitian rho; the
plugin takes the branch where the reference would (``assume_hermitian_state``, set by
mesolve from ``rho0.isherm``) and where it is the faster form
(:meth:`LindbladOperator.hermitian_pays`).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from .coefficients import Coefficient, pack_programs
from .operator import DeviceOperator, _ptr, _QG, _TORCH, stream_ptr
from .systems import merge_terms

__all__ = ["LindbladOperator", "ell_block"]


def ell_block(m: sp.csr_matrix):
    """``(width, col[width*d], val[width*d])`` of a d x d CSR matrix in the ELL layout
    the kernel reads: entry j of row r at ``j*d + r``; padding has value 0 and column r."""
    m = sp.csr_matrix(m, dtype=np.complex128)
    m.sort_indices()
    d = m.shape[0]
    lens = np.diff(m.indptr)
    W = int(lens.max()) if m.nnz else 0
    col = np.tile(np.arange(d, dtype=np.int32), W).reshape(W, d)
    val = np.zeros((W, d), dtype=np.complex128)
    if m.nnz:
        rows = np.repeat(np.arange(d), lens)
        pos = np.arange(m.nnz) - m.indptr[rows]
        col[pos, rows] = m.indices
        val[pos, rows] = m.data
    return W, col.reshape(-1), val.reshape(-1)


def _is_diagonal(m: sp.csr_matrix) -> bool:
    m = sp.coo_matrix(m)
    return bool(np.all(m.row[m.data != 0] == m.col[m.data != 0]))


class LindbladOperator:
    """Matrix-free Lindblad generator acting on vec(rho) (length d*d).

    ``a_terms``: ``[(d x d matrix, Coefficient | None)]``, the terms of A = -i H_nh
    (merged per coefficient).  ``c_terms``: ``[(d x d matrix, Coefficient | None)]``, one
    per collapse operator f_i(t) C_i.  Exposes the interface the Vern7 driver uses
    (``n_rows``, ``dtype``, ``device``, ``matvec``, ``vern7_stage``).
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
        a_terms = merge_terms([(sp.csr_matrix(m, dtype=np.complex128), c) for m, c in a_terms])
        if len(a_terms) > _lib.QG_MAX_GROUPS:
            raise ValueError(f"at most {_lib.QG_MAX_GROUPS} coefficient groups in H_nh")
        self.d = d
        self.n_rows = self.n_cols = d * d
        self.shape = (d * d, d * d)
        self.dtype = dtype
        self.device = torch.device(device)
        self.fmt = "lindblad"
        tdt = _TORCH[dtype]
        # A: per group its diagonal and an ELL block of its off-diagonal entries
        self.a_terms = a_terms
        self.a_coeffs = [c for _, c in a_terms]
        diag, widths, cols, vals = [], [], [], []
        for m, _ in a_terms:
            dg = m.diagonal()
            diag.append(dg)
            W, col, val = ell_block(m - sp.diags(dg, format="csr"))
            widths.append(W)
            cols.append(col)
            vals.append(val)
        self.a_width = widths
        # collapse operators: the all-diagonal ones first (constant before time-dependent),
        # then ELL blocks of the others
        def rank(i):
            m, f = c_terms[i]
            if _is_diagonal(m):
                return 0 if f is None else 1
            return 2 if np.diff(sp.csr_matrix(m).indptr).max() == 1 else 3
        order = sorted(range(len(c_terms)), key=rank)   # width-1 general operators lead
        self.c_terms = [(sp.csr_matrix(c_terms[i][0], dtype=np.complex128), c_terms[i][1])
                        for i in order]
        self.c_order = order
        self.n_cops = len(order)
        self.n_diag_cops = sum(1 for m, _ in self.c_terms if _is_diagonal(m))
        cdiag = [m.diagonal() for m, _ in self.c_terms[:self.n_diag_cops]]
        cw, ccols, cvals = [], [], []
        for m, _ in self.c_terms[self.n_diag_cops:]:
            W, col, val = ell_block(m)
            cw.append(W)
            ccols.append(col)
            cvals.append(val)
        self.c_width = cw
        if sum(widths) * d >= 2**31 or sum(cw) * d >= 2**31:
            raise ValueError("ELL storage beyond 2^31 entries")
        P = DeviceOperator.PAD
        dev = self.device

        def up(arrs, np_dt, t_dt):
            a = np.concatenate(arrs + [np.zeros(P, np_dt)]) if arrs else np.zeros(P, np_dt)
            return torch.from_numpy(a.astype(np_dt)).to(dev, t_dt)
        self.a_diag = up(diag, np.complex128, tdt)
        self.a_col = up(cols, np.int32, torch.int32)
        self.a_val = up(vals, np.complex128, tdt)
        self.c_diag = up(cdiag, np.complex128, tdt)
        self.c_col = up(ccols, np.int32, torch.int32)
        self.c_val = up(cvals, np.complex128, tdt)
        self.c_coeffs = [c for _, c in self.c_terms]
        # constant diagonal part D0(r, c) at r + c*d, precomputed once
        self.a_diag_const = 0
        for g, (m, c) in enumerate(a_terms):
            if c is None and np.any(diag[g] != 0):
                self.a_diag_const |= 1 << g
        self.n_const_diag = sum(1 for m, c in self.c_terms[:self.n_diag_cops] if c is None)
        self.d_const = None
        if self.a_diag_const or self.n_const_diag:
            self.d_const = self._constant_diagonal(diag, cdiag).to(tdt)
        self._a_prog = self._programs(self.a_coeffs)
        self._c_prog = self._programs(self.c_coeffs)
        self.coeffs = self.a_coeffs + self.c_coeffs
        self.stored = sum(widths) * d + sum(cw) * d
        self.struct = self._make_struct()

    def _constant_diagonal(self, a_diag, c_diag):
        """D0 as a (d, d) tensor M with M[c, r] = D0(r, c), i.e. vec order r + c*d."""
        d, dev = self.d, self.device
        a = np.zeros(d, dtype=np.complex128)
        for g in range(len(a_diag)):
            if (self.a_diag_const >> g) & 1:
                a += a_diag[g]
        av = torch.from_numpy(a).to(dev)
        M = av[None, :] + av.conj()[:, None]
        if self.n_const_diag:
            V = torch.from_numpy(np.stack(c_diag[:self.n_const_diag])).to(dev)  # (m, d)
            M = M + V.conj().T @ V     # [c, r] = sum_i conj(v_i[c]) v_i[r]
        return M.reshape(-1)

    def _programs(self, coeffs):
        if all(c is None for c in coeffs):
            return (None, None, None)
        code, starts, consts = pack_programs(coeffs)
        return tuple(torch.from_numpy(a).to(self.device) for a in (code, starts, consts))

    def _make_struct(self) -> _lib.Lindblad:
        st = _lib.Lindblad()
        st.d = self.d
        st.dtype = _QG[self.dtype]
        st.n_groups = len(self.a_terms)
        st.n_diag_cops = self.n_diag_cops
        st.n_cops = self.n_cops
        st.a_diag_const = self.a_diag_const
        st.n_const_diag = self.n_const_diag
        st.hermitian = int(getattr(self, "_hermitian", False))
        st.d_const = _ptr(self.d_const)
        for g, w in enumerate(self.a_width):
            st.a_width[g] = w
        for i, w in enumerate(self.c_width):
            st.c_width[i] = w
        st.a_diag, st.a_col, st.a_val = _ptr(self.a_diag), _ptr(self.a_col), _ptr(self.a_val)
        st.c_diag, st.c_col, st.c_val = _ptr(self.c_diag), _ptr(self.c_col), _ptr(self.c_val)
        st.a_coef_code, st.a_coef_start, st.a_coef_consts = (_ptr(v) for v in self._a_prog)
        st.c_coef_code, st.c_coef_start, st.c_coef_consts = (_ptr(v) for v in self._c_prog)
        return st

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
    def hermitian(self) -> bool:
        """Evaluate only the elements r >= c and mirror them (rho Hermitian)."""
        return bool(getattr(self, "_hermitian", False))

    @hermitian.setter
    def hermitian(self, value: bool):
        self._hermitian = bool(value)
        self.struct.hermitian = int(self._hermitian)

    def hermitian_pays(self) -> bool:
        """Whether the Hermitian branch is the faster form for this size.  It halves the
        generator's arithmetic and writes the mirrored half through 32 x 32 shared-memory
        tiles, one CTA per tile on or below the diagonal: measured on the Ising chain
        (mixed form), 58 -> 43 us per stage at L = 10 (528 tiles) and 4.8 -> 2.6 ms at
        L = 13.  With fewer tiles than two per SM the GPU idles (dense random d = 128,
        10 tiles: 534 -> 2133 ms per solve), so the full form stays there."""
        n_t = (self.d + 31) // 32
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        return n_t * (n_t + 1) // 2 >= 2 * sms

    @property
    def n_groups(self) -> int:
        return len(self.a_terms)

    @property
    def isconstant(self) -> bool:
        return all(c is None for c in self.coeffs)

    @property
    def launch(self):
        return ("lindblad", 0, 1)

    def launch_desc(self) -> str:
        half = ", Hermitian rho: half the elements" if self.hermitian else ""
        return f"matrix-free Lindblad (d={self.d}, {self.n_cops} collapse operators{half})"

    def tune(self, *args, **kwargs):
        """One launch shape (one thread per element, grid from the occupancy query)."""
        return self.launch

    def value_bytes(self) -> int:
        """Bytes of one value in the stage dtype."""
        return 16 if self.dtype == "c128" else 8

    def operator_bytes(self) -> int:
        """Bytes of the generator's storage: ELL blocks, diagonals and the precomputed
        constant diagonal factor (d*d values)."""
        es = self.value_bytes()
        b = self.stored * (es + 4) + (self.n_groups + self.n_diag_cops) * self.d * es
        return b + (self.n_rows * es if self.d_const is not None else 0)

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
