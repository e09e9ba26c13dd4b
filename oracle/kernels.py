"""Restatement of the reference's data-layer kernels (FP64, numpy).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA kernels, never the product.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def spmv_csr(data, col, row_ptr, x, scale=1.0, out=None):
    """``out += scale * A @ x`` for CSR ``A``.

    Follows ``_matmul_csr_vector`` (qutip/core/data/src/matmul_csr_vector.cpp:107-149):
    each row's dot product is accumulated first and then scaled and added to
    ``out``.
    """
    n = len(row_ptr) - 1
    prod = np.asarray(data) * np.asarray(x)[np.asarray(col)]
    row_ids = np.repeat(np.arange(n), np.diff(row_ptr))
    dot = np.zeros(n, dtype=np.complex128)
    np.add.at(dot, row_ids, prod)
    if out is None:
        out = np.zeros(n, dtype=np.complex128)
    out += scale * dot
    return out


def spmv_dia(data, offsets, n_rows, n_cols, x, scale=1.0, out=None):
    """``out += scale * A @ x`` for a Dia matrix stored as ``data[ndiag, n_cols]``.

    Follows ``matmul_dia_dense_dense`` / ``_matmul_diag_vector``
    (qutip/core/data/matmul.pyx:429-507, qutip/core/data/src/matmul_diag_vector.cpp:13-39):
    diagonal ``d`` with offset ``o`` multiplies ``x[col]`` into ``out[col - o]``
    where the entry is stored at ``data[d, col]``.
    """
    if out is None:
        out = np.zeros(n_rows, dtype=np.complex128)
    acc = np.zeros(n_rows, dtype=np.complex128)
    for d, off in enumerate(offsets):
        start = max(0, off)
        end = min(n_cols, n_rows + off)
        if end <= start:
            continue
        cols = np.arange(start, end)
        acc[cols - off] += data[d, cols] * x[cols]
    out += scale * acc
    return out


def expect_csr_dm(op: sp.csr_matrix, rho_vec: np.ndarray) -> complex:
    """``tr(op @ rho)`` with ``rho`` column-stacked (F order).

    Follows ``_expect_csr_dense_dm`` (qutip/core/data/expect.pyx:146-158).
    """
    d = op.shape[0]
    rho = rho_vec.reshape(d, d, order="F")
    op = sp.csr_matrix(op)
    out = 0j
    for r in range(d):
        s, e = op.indptr[r], op.indptr[r + 1]
        for p in range(s, e):
            out += op.data[p] * rho[op.indices[p], r]
    return out


def expect_csr_ket(op: sp.csr_matrix, psi: np.ndarray) -> complex:
    """``<psi|op|psi>``; follows ``_expect_csr_dense_ket`` (qutip/core/data/expect.pyx:133-144)."""
    return complex(np.vdot(psi, op @ psi))


def expect_super_csr(op: sp.csr_matrix, vec: np.ndarray) -> complex:
    """``tr(op @ rho)`` for a super-operator ``op`` and column-stacked ``vec``.

    Follows ``expect_super_csr_dense`` (qutip/core/data/expect.pyx:223-236): the
    rows ``0, n+1, 2(n+1), ...`` of ``op @ vec`` are summed.
    """
    n = int(round(np.sqrt(vec.shape[0])))
    rows = np.arange(n) * (n + 1)
    return complex((op[rows] @ vec).sum())


def wrmn_error(diff, state, atol, rtol) -> float:
    """Weighted RMS norm; ``wrmn_error_dense`` (qutip/core/data/ode.pyx:27-52)."""
    diff = np.asarray(diff).ravel()
    state = np.asarray(state).ravel()
    return float(np.sqrt(np.mean((np.abs(diff) / (atol + rtol * np.abs(state))) ** 2)))


def lindblad_matrix_form(h_nh, c_ops, rho, scale=1.0, hermitian=False, out=None):
    """``out += scale * L[rho]`` with rho a d x d matrix, the reference's matrix form
    (``LindbladMatrixForm.matmul_data``, qutip/core/cy/lindblad_matrix_form.pyx:105-204).

    ``h_nh`` is the non-Hermitian Hamiltonian ``H - (i/2) sum c^dag c`` at the time of
    the call and ``c_ops`` the collapse operators at that time (d x d, sparse or dense).
    ``hermitian=True`` takes the reference's Hermitian branch: ``A + A^dag`` with
    ``A = -i H_nh rho + 1/2 sum c rho c^dag`` (:160-182); otherwise the full form
    ``-i (H_nh rho - rho H_nh^dag) + sum c rho c^dag`` (:183-200).
    """
    rho = np.asarray(rho, dtype=np.complex128)
    h = sp.csr_matrix(h_nh)
    if out is None:
        out = np.zeros_like(rho)
    if hermitian:
        acc = (-1j * scale) * (h @ rho)
        for c in c_ops:
            c = sp.csr_matrix(c)
            tmp = (0.5 * scale) * (c @ rho)
            acc = acc + (c.conj() @ tmp.T).T          # tmp @ c^dag
        out += acc + acc.conj().T
    else:
        out += (-1j * scale) * (h @ rho)
        out += (1j * scale) * (h.conj() @ rho.T).T    # rho @ h^dag
        for c in c_ops:
            c = sp.csr_matrix(c)
            tmp = scale * (c @ rho)
            out += (c.conj() @ tmp.T).T
    return out
