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


try:  # the raw current stream without torch.cuda.current_stream()'s Python overhead
    _raw_stream = torch._C._cuda_getCurrentRawStream
    _cur_device = torch._C._cuda_getDevice
except AttributeError:  # pragma: no cover - older or newer torch without these bindings
    _raw_stream = _cur_device = None


def stream_ptr() -> int:
    """``cudaStream_t`` of torch's current stream on the current device, as an int."""
    if _raw_stream is not None:
        return _raw_stream(_cur_device())
    return torch.cuda.current_stream().cuda_stream


def row_major_layout(mats):
    """Interleave coefficient groups row by row.

    Returns ``(row_ptr[n*G+1], col[nnz], val[nnz])`` with the entries of row r
    stored contiguously, group 0 first: group g of row r spans
    ``[row_ptr[r*G+g], row_ptr[r*G+g+1])``.
    """
    mats = [sp.csr_matrix(m, dtype=np.complex128) for m in mats]
    for m in mats:
        m.sort_indices()
    n, m_cols = mats[0].shape
    G = len(mats)
    if G == 1:  # one group: the row-major layout is the CSR itself
        m = mats[0]
        return m.indptr.astype(np.int64), m.indices.astype(np.int32), m.data.copy()
    counts = np.stack([np.diff(m.indptr) for m in mats], axis=1).reshape(-1)
    rp = np.zeros(n * G + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    nnz = int(rp[-1])
    col = np.empty(nnz, dtype=np.int32)
    val = np.empty(nnz, dtype=np.complex128)
    # destination of entry q of group g, row r: rp[r*G+g] + (q - indptr_g[r])
    for g, m in enumerate(mats):
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(m.indptr))
        dst = rp[rows * G + g] + (np.arange(m.nnz, dtype=np.int64) - m.indptr[rows])
        col[dst] = m.indices
        val[dst] = m.data
    return rp, col, val


def sliced_layout(mats, n_cols):
    """Sliced ELLPACK (32-row slices) of coefficient groups.

    Entries of each row and group are ordered by ``col XOR row``; in Kronecker-
    structured Liouvillians entry j of every row then flips the same index bits,
    so a warp's gathers land in the same few cache lines.  Returns
    ``(slice_ptr[S+1], widths[S*G], col, val, padded_entries)``.
    """
    mats = [sp.csr_matrix(m, dtype=np.complex128) for m in mats]
    n = mats[0].shape[0]
    G = len(mats)
    S = (n + 31) // 32
    counts = np.zeros((S * 32, G), dtype=np.int64)
    for g, m in enumerate(mats):
        counts[:n, g] = np.diff(m.indptr)
    widths = counts.reshape(S, 32, G).max(axis=1)                 # [S, G]
    slice_size = 32 * widths.sum(axis=1)
    slice_ptr = np.zeros(S + 1, dtype=np.int64)
    np.cumsum(slice_size, out=slice_ptr[1:])
    total = int(slice_ptr[-1])
    # padding: value 0, column = the row's own index (clipped) so gathers stay coalesced
    pos_slice = np.repeat(np.arange(S, dtype=np.int64), slice_size)
    lane = (np.arange(total, dtype=np.int64) - slice_ptr[pos_slice]) % 32
    col = np.minimum(pos_slice * 32 + lane, n_cols - 1).astype(np.int32)
    val = np.zeros(total, dtype=np.complex128)
    gprefix = np.concatenate([np.zeros((S, 1), np.int64), np.cumsum(widths, axis=1)[:, :-1]], 1)
    for g, m in enumerate(mats):
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(m.indptr))
        key = m.indices.astype(np.int64) ^ rows
        order = np.lexsort((key, rows))
        ci, dv = m.indices[order], m.data[order]
        q = np.arange(m.nnz, dtype=np.int64) - m.indptr[rows]
        sl = rows // 32
        dst = slice_ptr[sl] + 32 * (gprefix[sl, g] + q) + rows % 32
        col[dst] = ci
        val[dst] = dv
    return slice_ptr, widths.reshape(-1).astype(np.int32), col, val, total


def split_entries(m):
    """The real/imaginary split of a CSR matrix's entries: every entry becomes its nonzero
    real part ``(off << 1, a)`` and its nonzero imaginary part ``((off << 1) | 1, a)``, in
    row order, then ``col XOR row`` order, real part first.  ``off`` is column - row.
    Returns ``(rows, off2, a)``: int64, int64, float64."""
    m = sp.csr_matrix(m, dtype=np.complex128)
    n = m.shape[0]
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(m.indptr))
    order = np.lexsort((m.indices.astype(np.int64) ^ rows, rows))
    ci = m.indices[order].astype(np.int64)
    dv = m.data[order]
    r2 = np.repeat(rows, 2)
    off2 = np.repeat(ci - rows, 2) * 2 + np.tile(np.array([0, 1], np.int64), len(dv))
    a = np.stack([dv.real, dv.imag], axis=1).reshape(-1)
    keep = a != 0
    return r2[keep], off2[keep], a[keep]


def split_table_values(off2, a):
    """Table values of split entries: ``(a, a)`` for a real part (the product is
    ``a x``), ``(-a, a)`` for an imaginary part, whose product ``i a x`` is formed from x
    with its real and imaginary parts exchanged."""
    imag = (off2 & 1) == 1
    return np.where(imag, -a, a) + 1j * a


def dict_sliced_layout(mats, n_cols, dtype: str, max_table: int = _lib.QG_DICT_MAX,
                       split: bool = False):
    """Dictionary-coded sliced ELLPACK of coefficient groups, or ``None`` when the groups'
    (column - row, value) pairs do not fit ``max_table`` table entries.

    Rows are grouped in 32-row slices as in :func:`sliced_layout` (entries of a row ordered
    by ``col XOR row``); each group has its own code section, widths rounded up to a
    multiple of 4, and the codes of lane l are stored four at a time (entries 4q..4q+3 at
    ``base + 128 q + 4 l``).  Code 0 of every group is padding (offset 0, value 0).
    Values are deduplicated in the operator's dtype.  Returns ``(row_ptr[G*(S+1)],
    widths[S*G], codes, code_bytes, table_off, table_val, table_start[G+1], stored)``.

    ``split=True`` (complex128, ``QG_LAYOUT_SLICED_DICT_RI``) codes the real and the
    imaginary part of every entry separately (:func:`split_entries`), so that each code
    costs two FP64 multiply-adds instead of four; table offsets are then ``off << 1``
    with the low bit set for an imaginary part.
    """
    if split:
        return _dict_split_layout(mats, n_cols, max_table)
    mats = [sp.csr_matrix(m, dtype=np.complex128) for m in mats]
    n = mats[0].shape[0]
    G = len(mats)
    S = (n + 31) // 32
    vdt = np.complex64 if dtype == "c64" else np.complex128
    widths = np.zeros((S, G), dtype=np.int64)
    for g, m in enumerate(mats):
        c = np.zeros(S * 32, dtype=np.int64)
        c[:n] = np.diff(m.indptr)
        widths[:, g] = c.reshape(S, 32).max(axis=1)      # exact: the kernel skips the rest
    sect = 32 * ((widths + 3) // 4 * 4)                  # codes per (slice, group)
    gsize = sect.sum(axis=0)                             # codes per group
    gbase = np.concatenate([[0], np.cumsum(gsize)[:-1]])
    row_ptr = np.zeros((G, S + 1), dtype=np.int64)
    for g in range(G):
        row_ptr[g, 1:] = np.cumsum(sect[:, g])
        row_ptr[g] += gbase[g]
    total = int(gsize.sum())
    if total >= 2**31 - 16:
        return None
    codes = np.zeros(total, dtype=np.int32)
    t_off, t_val, t_start = [], [], [0]
    for g, m in enumerate(mats):
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(m.indptr))
        order = np.lexsort((m.indices.astype(np.int64) ^ rows, rows))
        ci = m.indices[order].astype(np.int64)
        dv = m.data[order].astype(vdt)
        off = ci - rows
        nz = dv != 0
        vals, vcode = np.unique(dv[nz], return_inverse=True)
        key = off[nz] * max(len(vals), 1) + vcode.reshape(-1)
        ukey, kcode = np.unique(key, return_inverse=True)
        if len(ukey) + 1 > max_table:
            return None
        voff = ukey // max(len(vals), 1)
        t_off.append(np.concatenate([[0], voff]).astype(np.int32))
        t_val.append(np.concatenate([np.zeros(1, vdt), vals[ukey - voff * max(len(vals), 1)]]))
        t_start.append(t_start[-1] + len(ukey) + 1)
        code = np.zeros(m.nnz, dtype=np.int32)
        code[nz] = kcode.reshape(-1) + 1
        q = np.arange(m.nnz, dtype=np.int64) - m.indptr[rows]
        sl = rows // 32
        dst = row_ptr[g, sl] + 128 * (q // 4) + 4 * (rows % 32) + q % 4
        codes[dst] = code
    if t_start[-1] > max_table:
        return None
    cb = 1 if max(b - a for a, b in zip(t_start[:-1], t_start[1:])) <= 256 else 2
    if cb == 2 and max(b - a for a, b in zip(t_start[:-1], t_start[1:])) > 65536:
        return None
    return (row_ptr.reshape(-1), widths.reshape(-1).astype(np.int32),
            codes.astype(np.uint8 if cb == 1 else np.uint16), cb,
            np.concatenate(t_off), np.concatenate(t_val), np.asarray(t_start, np.int32), total)


def _dict_split_layout(mats, n_cols, max_table):
    """:func:`dict_sliced_layout` of the real/imaginary split entries (complex128)."""
    n = mats[0].shape[0]
    G = len(mats)
    S = (n + 31) // 32
    ents = [split_entries(m) for m in mats]
    widths = np.zeros((S, G), dtype=np.int64)
    for g, (r, _, _) in enumerate(ents):
        c = np.zeros(S * 32, dtype=np.int64)
        c[:n] = np.bincount(r, minlength=n)
        widths[:, g] = c.reshape(S, 32).max(axis=1)
    sect = 32 * ((widths + 3) // 4 * 4)
    gsize = sect.sum(axis=0)
    gbase = np.concatenate([[0], np.cumsum(gsize)[:-1]])
    row_ptr = np.zeros((G, S + 1), dtype=np.int64)
    for g in range(G):
        row_ptr[g, 1:] = np.cumsum(sect[:, g])
        row_ptr[g] += gbase[g]
    total = int(gsize.sum())
    if total >= 2**31 - 16:
        return None
    codes = np.zeros(total, dtype=np.int32)
    t_off, t_val, t_start = [], [], [0]
    for g, (r, off2, a) in enumerate(ents):
        vals, vcode = np.unique(a, return_inverse=True)
        V = max(len(vals), 1)
        ukey, kcode = np.unique(off2 * V + vcode.reshape(-1), return_inverse=True)
        if len(ukey) + 1 > max_table:
            return None
        uoff = np.floor_divide(ukey, V)
        ua = vals[ukey - uoff * V]
        t_off.append(np.concatenate([[0], uoff]).astype(np.int32))
        t_val.append(np.concatenate([np.zeros(1, np.complex128), split_table_values(uoff, ua)]))
        t_start.append(t_start[-1] + len(ukey) + 1)
        start = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(np.bincount(r, minlength=n), out=start[1:])
        q = np.arange(len(r), dtype=np.int64) - start[r]
        sl = r // 32
        dst = row_ptr[g, sl] + 128 * (q // 4) + 4 * (r % 32) + q % 4
        codes[dst] = kcode.reshape(-1) + 1
    if t_start[-1] > max_table:
        return None
    longest = max(b - a for a, b in zip(t_start[:-1], t_start[1:]))
    if longest > 65536:
        return None
    cb = 1 if longest <= 256 else 2
    return (row_ptr.reshape(-1), widths.reshape(-1).astype(np.int32),
            codes.astype(np.uint8 if cb == 1 else np.uint16), cb,
            np.concatenate(t_off), np.concatenate(t_val), np.asarray(t_start, np.int32), total)


def row_tiles(row_start, tile_nnz, max_rows):
    """Greedy row tiles holding at most ``tile_nnz - 8`` entries and ``max_rows`` rows.

    ``row_start`` is the entry offset of each row (length n+1).  Returns the
    first row of each tile (length n_tiles+1) or ``None`` if a row is too long.
    """
    n = len(row_start) - 1
    cap = tile_nnz - 8
    if n == 0 or np.max(np.diff(row_start)) > cap:
        return None
    out = [0]
    r = 0
    while r < n:
        r1 = int(np.searchsorted(row_start, row_start[r] + cap, side="right")) - 1
        r1 = min(r1, r + max_rows, n)
        out.append(r1)
        r = r1
    return np.asarray(out, dtype=np.int32)


class DeviceOperator:
    """``A(t) = sum_g c_g(t) A_g`` resident on the GPU.

    ``terms`` is a list of ``(scipy matrix, Coefficient | None)``.  Entries are
    stored row-major (all groups of a row contiguous) with 8 entries of padding
    so that row tiles can be bulk-copied in 16-byte units; the launch shape
    (direct sub-warp kernel or shared-memory staged tiles, threads per row) is
    chosen by :meth:`tune`.
    """

    PAD = 8

    def __init__(self, terms, dtype: str = "c128", device="cuda", merge: bool = True,
                 fmt: str = "auto"):
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
        G = len(terms)
        mats = [sp.csr_matrix(op) for op, _ in terms]
        self.group_nnz = [int(m.nnz) for m in mats]
        self.nnz = sum(self.group_nnz)
        lay = None
        self.dict_split = False
        if fmt == "auto":
            fmt = self._choose_format(mats)
            if fmt == "sliced":  # prefer the dictionary-coded form when the tables fit
                lay, self.dict_split = self._dict_layout(mats, dtype)
                fmt = "dict" if lay is not None else "sliced"
        elif fmt == "dict":
            lay, self.dict_split = self._dict_layout(mats, dtype)
            if lay is None:
                raise ValueError("the (column - row, value) pairs exceed the dictionary size")
        if fmt not in ("csr", "sliced", "dict"):
            raise ValueError("fmt must be 'auto', 'csr', 'sliced' or 'dict'")
        self.fmt = fmt
        P = self.PAD
        self._tiles = {}
        self.dict_off = self.dict_start = None
        self.code_bytes = 0
        if fmt == "dict":
            rp, widths, codes, cb, t_off, t_val, t_start, total = lay
            self.stored = total
            self.code_bytes = cb
            self.slice_width = torch.from_numpy(widths).to(self.device)
            self.row_ptr = torch.from_numpy(rp.astype(np.int32)).to(self.device)
            self.col = torch.from_numpy(codes if cb == 1 else codes.view(np.int16)).to(self.device)
            self.val = torch.from_numpy(t_val).to(self.device, _TORCH[dtype])
            self.dict_off = torch.from_numpy(t_off).to(self.device)
            self.dict_start = torch.from_numpy(t_start).to(self.device)
            self._finish(G)
            return
        if fmt == "sliced":
            rp, widths, col, val, total = sliced_layout(mats, self.n_cols)
            self.stored = total
            self.slice_width = torch.from_numpy(widths).to(self.device)
        else:
            rp, col, val = row_major_layout(mats)
            self.stored = len(col)
            self.slice_width = None
        if self.stored >= 2**31 - 16 or self.n_rows * G >= 2**31 - 16:
            raise ValueError("operators beyond 2^31 stored entries need 64-bit indices")
        self.row_ptr = torch.zeros(len(rp) + P, dtype=torch.int32, device=self.device)
        self.row_ptr[:len(rp)] = torch.from_numpy(rp.astype(np.int32)).to(self.device)
        self.col = torch.zeros(self.stored + P, dtype=torch.int32, device=self.device)
        self.col[:self.stored] = torch.from_numpy(col).to(self.device)
        self.val = torch.zeros(self.stored + P, dtype=_TORCH[dtype], device=self.device)
        self.val[:self.stored] = torch.from_numpy(val).to(self.device, _TORCH[dtype])
        if fmt == "csr":
            row_start = rp[::G]
            for tn in (2048, 4096):
                t = row_tiles(row_start, tn, _lib.QG_TILE_ROWS)
                if t is not None:
                    self._tiles[tn] = torch.from_numpy(t).to(self.device)
        self._finish(G)

    def _dict_layout(self, mats, dtype):
        """Dictionary layout of host groups: real/imaginary split for complex128 (two FP64
        multiply-adds per code instead of four), falling back to whole complex values when
        the split tables do not fit.  Returns ``(layout or None, split)``."""
        if dtype == "c128":
            lay = dict_sliced_layout(mats, self.n_cols, dtype, split=True)
            if lay is not None:
                return lay, True
        return dict_sliced_layout(mats, self.n_cols, dtype), False

    @classmethod
    def from_device_groups(cls, groups, dtype: str = "c64", fmt: str = "auto"):
        """Sliced operator from device CSR groups ``[(indptr, indices, data,
        Coefficient | None), ...]`` (for example from
        :func:`qutip_gb300.superop.liouvillian_groups`), laid out on the device:
        dictionary-coded when the groups' (column - row, value) pairs fit the tables
        (``fmt="auto"`` or ``"dict"``), plain sliced ELLPACK otherwise (or ``"sliced"``)."""
        from .superop import device_dict_layout, device_sliced_layout
        if fmt not in ("auto", "dict", "sliced"):
            raise ValueError("fmt must be 'auto', 'dict' or 'sliced'")
        if dtype not in _TORCH:
            raise TypeError(f"unsupported dtype {dtype!r}")
        if not groups or len(groups) > _lib.QG_MAX_GROUPS:
            raise ValueError(f"1..{_lib.QG_MAX_GROUPS} coefficient groups are supported")
        self = cls.__new__(cls)
        indptr0 = groups[0][0]
        n = indptr0.numel() - 1
        self.shape = (n, n)
        self.n_rows = self.n_cols = n
        self.dtype = dtype
        self.coeffs = [c for _, _, _, c in groups]
        for c in self.coeffs:
            if c is not None and not isinstance(c, Coefficient):
                raise TypeError("coefficients must be qutip_gb300.coefficients.Coefficient")
        self.device = indptr0.device
        self.group_nnz = [int(ix.numel()) for _, ix, _, _ in groups]
        self.nnz = sum(self.group_nnz)
        self._tiles = {}
        self.dict_off = self.dict_start = None
        self.code_bytes = 0
        self.dict_split = False
        lay = None
        if fmt != "sliced" and dtype == "c128":
            lay = device_dict_layout(groups, n, dtype, split=True)
            self.dict_split = lay is not None
        if lay is None and fmt != "sliced":
            lay = device_dict_layout(groups, n, dtype)
        if lay is None and fmt == "dict":
            raise ValueError("the (column - row, value) pairs exceed the dictionary size")
        if lay is not None:
            rp, widths, codes, cb, t_off, t_val, t_start, total = lay
            self.fmt = "dict"
            self.stored = total
            self.code_bytes = cb
            self.slice_width = widths
            self.row_ptr, self.col, self.val = rp, codes, t_val.to(_TORCH[dtype])
            self.dict_off, self.dict_start = t_off, t_start
            self._finish(len(groups))
            return self
        self.fmt = "sliced"
        P = self.PAD
        rp, widths, col, val, total = device_sliced_layout(groups, n)
        if total >= 2**31 - 16 or n * len(groups) >= 2**31 - 16:
            raise ValueError("operators beyond 2^31 stored entries need 64-bit indices")
        self.stored = total
        self.slice_width = widths
        self.row_ptr = torch.zeros(rp.numel() + P, dtype=torch.int32, device=self.device)
        self.row_ptr[:rp.numel()] = rp.to(torch.int32)
        self.col = torch.zeros(total + P, dtype=torch.int32, device=self.device)
        self.col[:total] = col
        del col
        self.val = torch.zeros(total + P, dtype=_TORCH[dtype], device=self.device)
        self.val[:total] = val.to(_TORCH[dtype])
        del val
        self._finish(len(groups))
        return self

    def astype(self, dtype: str):
        """The same operator and layout with values in ``dtype`` (device copy).  The
        real/imaginary split tables exist for complex128 only."""
        if getattr(self, "dict_split", False) and dtype != "c128":
            raise TypeError("the real/imaginary split dictionary is a complex128 layout; "
                            "build the complex64 operator from the terms")
        other = self.__class__.__new__(self.__class__)
        other.__dict__.update(self.__dict__)
        other.dtype = dtype
        other.val = self.val.to(_TORCH[dtype])
        other._finish(self.n_groups)
        other.set_launch(self.launch)
        return other

    def _pack_coefficients(self):
        if all(c is None for c in self.coeffs):
            self.coef_code = self.coef_start = self.coef_consts = None
        else:
            code, starts, consts = pack_programs(self.coeffs)
            self.coef_code = torch.from_numpy(code).to(self.device)
            self.coef_start = torch.from_numpy(starts).to(self.device)
            self.coef_consts = torch.from_numpy(consts).to(self.device)

    def set_coefficients(self, coeffs):
        """Replace the groups' coefficient programs (new args), keeping the storage."""
        if len(coeffs) != self.n_groups:
            raise ValueError(f"{len(coeffs)} coefficients for {self.n_groups} groups")
        if [c is None for c in coeffs] != [c is None for c in self.coeffs]:
            raise ValueError("constant and time-dependent groups cannot swap places")
        self.coeffs = list(coeffs)
        self._pack_coefficients()
        self.struct.coef_code = _ptr(self.coef_code)
        self.struct.coef_start = _ptr(self.coef_start)
        self.struct.coef_consts = _ptr(self.coef_consts)

    def _finish(self, G):
        fmt = self.fmt
        dtype = self.dtype
        self._pack_coefficients()
        layout = {"sliced": _lib.QG_LAYOUT_SLICED, "dict": _lib.QG_LAYOUT_SLICED_DICT}.get(
            fmt, _lib.QG_LAYOUT_ROW_MAJOR)
        if fmt == "dict" and getattr(self, "dict_split", False):
            layout = _lib.QG_LAYOUT_SLICED_DICT_RI
        self.struct = _lib.CsrGroups(
            self.n_rows, self.n_cols, G, _QG[dtype], layout, 4, 0, 0,
            _ptr(self.row_ptr), _ptr(self.col), _ptr(self.val), None, _ptr(self.coef_code),
            _ptr(self.coef_start), _ptr(self.coef_consts), _ptr(self.dict_off),
            _ptr(self.dict_start))
        self.set_launch(self.default_launch())

    def _choose_format(self, mats) -> str:
        """Sliced ELLPACK when its padding costs at most 15 % more entries, else CSR."""
        n = self.n_rows
        if n < 1024:
            return "csr"
        S = (n + 31) // 32
        padded = 0
        for m in mats:
            c = np.zeros(S * 32, dtype=np.int64)
            c[:n] = np.diff(m.indptr)
            padded += 32 * int(c.reshape(S, 32).max(axis=1).sum())
        return "sliced" if padded <= 1.15 * max(self.nnz, 1) else "csr"

    # -- launch shape ------------------------------------------------------
    def default_launch(self):
        """Staged tiles for short rows, a sub-warp per row otherwise (before tuning)."""
        if self.fmt == "sliced":
            return ("sliced", 0, 1)
        if self.fmt == "dict":
            return ("dict", 0, 1)
        mean = self.nnz / max(self.n_rows, 1)
        tn = 4096 if self.dtype == "c64" else 2048
        if tn in self._tiles and mean <= 64:
            return ("staged", tn, 4 if mean >= 12 else 2)
        lanes = 2
        while lanes < 32 and lanes * 2 <= max(mean / self.n_groups / 1.5, 2):
            lanes *= 2
        return ("direct", 0, lanes)

    def set_launch(self, launch):
        kind, tile_nnz, lanes = launch
        if (kind in ("sliced", "dict") or self.fmt in ("sliced", "dict")) and kind != self.fmt:
            raise ValueError(f"launch {kind!r} does not match the {self.fmt!r} storage")
        if kind == "dict":
            self.struct.n_tiles = (self.n_rows + 31) // 32
            self.struct.tile_nnz = self.code_bytes
            self.struct.tile_row = self.slice_width.data_ptr()
            self.struct.lanes = int(self.val.numel())
            self.launch = launch
            return
        if kind == "sliced":
            self.struct.n_tiles = (self.n_rows + 31) // 32
            self.struct.tile_nnz = 0
            self.struct.tile_row = self.slice_width.data_ptr()
        elif kind == "staged":
            if tile_nnz not in self._tiles:
                raise ValueError(f"no {tile_nnz}-entry tiling (a row is too long)")
            t = self._tiles[tile_nnz]
            self.struct.n_tiles = len(t) - 1
            self.struct.tile_nnz = tile_nnz
            self.struct.tile_row = t.data_ptr()
        else:
            self.struct.n_tiles = 0
            self.struct.tile_nnz = 0
            self.struct.tile_row = None
        self.struct.lanes = lanes
        self.launch = (kind, tile_nnz, lanes)

    def launch_desc(self) -> str:
        kind, tn, lanes = self.launch
        if kind == "dict":
            split = ", real/imaginary split" if getattr(self, "dict_split", False) else ""
            return (f"dict(32-row slices, {self.code_bytes}-byte codes, "
                    f"{self.val.numel()} table entries{split}, "
                    f"{self.stored / max(self.nnz, 1):.3f}x stored/nnz)")
        if kind == "sliced":
            return f"sliced(32-row slices, {self.stored / max(self.nnz, 1):.3f}x stored/nnz)"
        return f"{kind}(lanes={lanes}" + (f", tile_nnz={tn})" if kind == "staged" else ")")

    def candidates(self):
        if self.fmt in ("sliced", "dict"):
            return [(self.fmt, 0, 1)]
        out = [("direct", 0, l) for l in (1, 2, 4, 8, 16, 32)]
        for tn in sorted(self._tiles):
            out += [("staged", tn, l) for l in (1, 2, 4, 8, 16)]
        return out

    def tune(self, reps: int = 5, candidates=None):
        """Time the matvec for every launch shape on this device and keep the fastest."""
        x = torch.randn(self.n_cols, dtype=_TORCH[self.dtype], device=self.device)
        y = torch.empty(self.n_rows, dtype=_TORCH[self.dtype], device=self.device)
        results = {}
        for cand in candidates or self.candidates():
            self.set_launch(cand)
            self.matvec(0.37, x, y)
            st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            st.record()
            for _ in range(reps):
                self.matvec(0.37, x, y)
            en.record()
            en.synchronize()
            results[cand] = st.elapsed_time(en) / reps
        best = min(results, key=results.get)
        self.set_launch(best)
        self.tune_results = results
        return best

    tune_lanes = tune

    def device_arrays(self):
        return [t for t in (self.row_ptr, self.col, self.val, self.slice_width, self.coef_code,
                            self.coef_start, self.coef_consts, self.dict_off, self.dict_start)
                if t is not None]

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

    def value_bytes(self) -> int:
        return 16 if self.dtype == "c128" else 8

    def operator_bytes(self) -> int:
        """Algorithmic HBM bytes of the operator stream of one application: values and
        int32 indices plus row pointers, or for the dictionary form its codes (padding
        included), slice pointers and widths, and the tables."""
        sv = self.value_bytes()
        if self.fmt == "dict":
            S = (self.n_rows + 31) // 32
            return (self.stored * self.code_bytes + 8 * self.n_groups * (S + 1)
                    + int(self.val.numel()) * (sv + 4))
        return self.nnz * (sv + 4) + (self.n_groups * self.n_rows + 1) * 4

    def spmv_bytes(self, accumulate: bool = False) -> int:
        """Algorithmic HBM bytes of one matvec: the operator stream + x + y."""
        sv = self.value_bytes()
        return (self.operator_bytes() + self.n_cols * sv
                + self.n_rows * sv * (2 if accumulate else 1))

    def matvec(self, t: float, x: torch.Tensor, y: torch.Tensor, alpha=1.0, beta=0.0):
        """``y = alpha A(t) x + beta y`` on the current stream (vectors in ``self.dtype``)."""
        if x.dtype != _TORCH[self.dtype] or y.dtype != _TORCH[self.dtype]:
            raise TypeError("vector dtype must match the operator dtype")
        if x.numel() != self.n_cols or y.numel() != self.n_rows:
            raise ValueError("incompatible shapes")
        if not (x.is_contiguous() and y.is_contiguous()):
            raise ValueError("vectors must be contiguous")
        a, b = complex(alpha), complex(beta)
        _lib.call("qg_spmv_csr", C.byref(self.struct), float(t), x.data_ptr(), y.data_ptr(),
                  a.real, a.imag, b.real, b.imag, stream_ptr())
        return y

    def vern7_stage(self, rk, stage: int, t_prev: float, dt: float, atol: float, rtol: float,
                    stream: int):
        """One fused Vern7 stage (``qg_vern7_stage``) on the buffers ``rk``."""
        lib = _lib.load()
        _lib.check(lib.qg_vern7_stage(C.byref(self.struct), C.byref(rk), stage, t_prev, dt,
                                      atol, rtol, stream), "qg_vern7_stage")

    def matmat(self, t: float, X: torch.Tensor, Y: torch.Tensor, alpha=1.0, beta=0.0):
        """``Y = alpha A(t) X + beta Y`` for F-ordered column blocks stored as ``[n_vec, n]``."""
        if X.dtype != _TORCH[self.dtype] or Y.dtype != _TORCH[self.dtype]:
            raise TypeError("vector dtype must match the operator dtype")
        if X.dim() != 2 or X.shape[1] != self.n_cols or Y.shape != (X.shape[0], self.n_rows):
            raise ValueError("incompatible shapes")
        if self.fmt != "csr":
            raise TypeError("multi-vector products need the CSR storage (fmt='csr')")
        a, b = complex(alpha), complex(beta)
        _lib.call("qg_spmm_csr", C.byref(self.struct), float(t), X.data_ptr(), Y.data_ptr(),
                  X.shape[0], X.stride(0), a.real, a.imag, b.real, b.imag, stream_ptr())
        return Y


class DeviceDia:
    """A Dia matrix (qutip/core/data/dia.pxd:17-38) resident on the GPU."""

    def __init__(self, mat, dtype: str = "c128", device="cuda"):
        m = sp.dia_matrix(sp.csr_matrix(mat))  # duplicates summed by the CSR conversion
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
