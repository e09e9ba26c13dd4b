"""Liouvillians assembled in device memory from Hilbert-space operators.

The reference forms superoperators on the host with sparse Kronecker products:
``spre`` / ``spost`` / ``sprepost`` (qutip/core/superoperator.py:357-440) and
``lindblad_dissipator`` / ``liouvillian`` (:36-200), in the column-stacking
convention ``vec(A rho B) = (B^T (x) A) vec(rho)``.  At the L = 12 Ising chain
(16,777,216 rows, about 4.8e8 entries) that takes minutes and tens of GB of host
memory.

Here every term ``c * (B^T (x) A)`` is expanded as the outer product of its two
factors' COO entries on the device. Duplicate positions within a coefficient
group are summed after one device sort of the ``row * N + col`` keys, and exact
zeros are dropped (as scipy's sparse sum does). The result goes straight into
the sliced-ELLPACK layout of
:class:`~qutip_gb300.operator.DeviceOperator` (:func:`device_sliced_layout`, the
device twin of :func:`~qutip_gb300.operator.sliced_layout`).  The host only holds
the ``d x d`` Hilbert-space operators.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

__all__ = ["kron_coo", "coalesce", "liouvillian_groups", "device_sliced_layout",
           "device_term_groups", "sliced_padding"]


def _coo(m, device):
    m = sp.coo_matrix(m)
    return (torch.from_numpy(m.row.astype(np.int64)).to(device),
            torch.from_numpy(m.col.astype(np.int64)).to(device),
            torch.from_numpy(m.data.astype(np.complex128)).to(device))


def kron_coo(a, b, scale=1.0, device="cuda"):
    """COO entries of ``scale * (a (x) b)`` (a, b: square scipy matrices)."""
    ra, ca, va = _coo(a, device)
    rb, cb, vb = _coo(b, device)
    nb = b.shape[0]
    rows = (ra[:, None] * nb + rb[None, :]).reshape(-1)
    cols = (ca[:, None] * nb + cb[None, :]).reshape(-1)
    vals = (va[:, None] * vb[None, :]).reshape(-1) * complex(scale)
    return rows, cols, vals


def coalesce(terms, n, device="cuda"):
    """Sum of Kronecker terms ``[(a, b, scale), ...]`` as CSR: keys ``row * n + col``
    are written term by term into one buffer (no per-term index arrays are kept),
    sorted once, duplicates summed, exact zeros dropped.

    Returns ``(indptr int64[n+1], indices int64[nnz], data complex128[nnz])`` with
    rows ascending and columns ascending within each row."""
    sizes = [sp.csr_matrix(a).nnz * sp.csr_matrix(b).nnz for a, b, _ in terms]
    total = sum(sizes)
    keys = torch.empty(total, dtype=torch.int64, device=device)
    vals = torch.empty(total, dtype=torch.complex128, device=device)
    off = 0
    for (a, b, scale), size in zip(terms, sizes):
        r, c, v = kron_coo(a, b, scale, device)
        keys[off:off + size] = r * n + c
        vals[off:off + size] = v
        off += size
        del r, c, v
    keys, order = torch.sort(keys)
    vals = vals[order]
    del order
    uniq, inv = torch.unique_consecutive(keys, return_inverse=True)
    del keys
    summed = torch.zeros(uniq.numel(), dtype=vals.dtype, device=device)
    summed.index_add_(0, inv, vals)
    del inv, vals
    keep = summed != 0
    uniq, summed = uniq[keep], summed[keep]
    rows = torch.div(uniq, n, rounding_mode="floor")
    cols = uniq - rows * n
    del uniq
    counts = torch.bincount(rows, minlength=n)
    indptr = torch.zeros(n + 1, dtype=torch.int64, device=device)
    torch.cumsum(counts, 0, out=indptr[1:])
    return indptr, cols, summed


def liouvillian_groups(h_terms, c_ops=(), device="cuda"):
    """Coefficient groups of the Lindblad generator, assembled on the device.

    ``h_terms``: list of ``(H_k, Coefficient | None)`` (d x d scipy);
    ``c_ops``: constant collapse operators.  Group order follows the first
    appearance of each coefficient, the constant group first if present, which
    matches :func:`qutip_gb300.systems.merge_terms` of the host construction.

    Returns ``[(indptr, indices, data, coefficient), ...]`` (device CSR).
    """
    d = (h_terms[0][0] if h_terms else c_ops[0]).shape[0]
    n = d * d
    eye = sp.identity(d, dtype=np.complex128, format="csr")
    groups: dict = {}
    order = []

    def add(key, coeff, term):
        if key not in groups:
            groups[key] = (coeff, [])
            order.append(key)
        groups[key][1].append(term)

    for h, coeff in h_terms:
        key = None if coeff is None else coeff.key()
        h = sp.csr_matrix(h, dtype=np.complex128)
        add(key, coeff, (eye, h, -1j))          # -i spre(H)
        add(key, coeff, (h.T.tocsr(), eye, 1j))  # +i spost(H)
    for c in c_ops:
        c = sp.csr_matrix(c, dtype=np.complex128)
        cdc = (c.conj().T @ c).tocsr()
        add(None, None, (c.conj(), c, 1.0))      # sprepost(c, c^dag)
        add(None, None, (eye, cdc, -0.5))        # -1/2 spre(c^dag c)
        add(None, None, (cdc.T.tocsr(), eye, -0.5))  # -1/2 spost(c^dag c)
    if None in groups:                           # constant group first
        order.remove(None)
        order.insert(0, None)
    out = []
    for key in order:
        coeff, terms = groups[key]
        indptr, indices, data = coalesce(terms, n, device)
        out.append((indptr, indices, data, coeff))
    return out


def _upload_csr(m, device):
    """Device copies of a CSR matrix's arrays, indices widened on the device (the host
    arrays are sent as stored: 32-bit indices, complex128 values)."""
    m = sp.csr_matrix(m)

    def idx(a):
        a = np.asarray(a)
        if a.dtype not in (np.int32, np.int64):
            a = a.astype(np.int64)
        return torch.from_numpy(np.ascontiguousarray(a)).to(device).to(torch.int64)
    return (idx(m.indptr), idx(m.indices),
            torch.from_numpy(np.ascontiguousarray(m.data, dtype=np.complex128)).to(device))


def _sum_in_order(parts, n):
    """Sum of device CSR matrices ``parts`` (same shape) with each position summed
    left to right in list order, as chained scipy ``+`` does, and exact zeros dropped.
    The order is fixed, so equal inputs give equal bits (a dictionary of the values
    then deduplicates them)."""
    keys = torch.cat([torch.repeat_interleave(torch.arange(n, device=ip.device), ip[1:] - ip[:-1])
                      * n + ix for ip, ix, _ in parts])
    vals = torch.cat([v for _, _, v in parts])
    keys, perm = torch.sort(keys, stable=True)        # stable: list order within a position
    vals = vals[perm]
    del perm
    first = torch.ones_like(keys, dtype=torch.bool)
    first[1:] = keys[1:] != keys[:-1]
    seg = torch.cumsum(first, 0) - 1
    starts = torch.nonzero(first).reshape(-1)
    rank = torch.arange(keys.numel(), device=keys.device) - starts[seg]
    uniq = keys[first]
    del keys, first
    summed = vals[starts].clone()
    for r in range(1, len(parts)):
        m = rank == r
        if not bool(m.any()):
            break
        summed[seg[m]] += vals[m]                     # one entry per position: no races
    keep = summed != 0
    uniq, summed = uniq[keep], summed[keep]
    rows = torch.div(uniq, n, rounding_mode="floor")
    counts = torch.bincount(rows, minlength=n)
    indptr = torch.zeros(n + 1, dtype=torch.int64, device=uniq.device)
    torch.cumsum(counts, 0, out=indptr[1:])
    return indptr, uniq - rows * n, summed


def device_term_groups(terms, device="cuda"):
    """Coefficient groups of ``(scipy matrix, Coefficient | None)`` terms as device CSR
    ``[(indptr, indices, data, coefficient), ...]``: each term's arrays are copied to the
    device once and the terms sharing a coefficient are summed there, in the group order
    of :func:`qutip_gb300.systems.merge_terms` (``QobjEvo.compress``,
    qutip/core/cy/qobjevo.pyx:816).  This is the device twin of the host merge that
    :class:`~qutip_gb300.operator.DeviceOperator` runs before its layouts, for generators
    too large to lay out on the host in reasonable time."""
    n = terms[0][0].shape[0]
    keyed: dict = {}
    order = []
    for m, c in terms:
        key = None if c is None else c.key()
        if key not in keyed:
            keyed[key] = (c, [])
            order.append(key)
        keyed[key][1].append(m)
    out = []
    for key in order:
        c, mats = keyed[key]
        parts = [_upload_csr(m, device) for m in mats]
        if len(parts) == 1:
            ip, ix, v = parts[0]
            if bool((v == 0).any()):                 # drop stored zeros, as the host merge does
                ip, ix, v = _sum_in_order(parts, n)
        else:
            ip, ix, v = _sum_in_order(parts, n)
        out.append((ip, ix, v, c))
    return out


def sliced_padding(groups) -> float:
    """Entries the sliced layout of device CSR ``groups`` stores (32-row slices padded to
    their longest row) per structural entry."""
    n = groups[0][0].numel() - 1
    S = (n + 31) // 32
    padded = 0
    nnz = 0
    for indptr, ix, _, _ in groups:
        c = torch.zeros(S * 32, dtype=torch.int64, device=indptr.device)
        c[:n] = indptr[1:] - indptr[:-1]
        padded += 32 * int(c.view(S, 32).amax(dim=1).sum().item())
        nnz += ix.numel()
    return padded / max(nnz, 1)


def device_sliced_layout(groups, n_cols):
    """Sliced ELLPACK of device CSR groups: the layout of
    :func:`qutip_gb300.operator.sliced_layout` computed with device sorts and
    scatters.  Returns ``(slice_ptr, widths, col int32, val complex128, total)``."""
    indptr0 = groups[0][0]
    device = indptr0.device
    n = indptr0.numel() - 1
    G = len(groups)
    S = (n + 31) // 32
    counts = torch.zeros((S * 32, G), dtype=torch.int64, device=device)
    for g, (indptr, _, _, _) in enumerate(groups):
        counts[:n, g] = indptr[1:] - indptr[:-1]
    widths = counts.view(S, 32, G).amax(dim=1)                   # [S, G]
    slice_size = 32 * widths.sum(dim=1)
    slice_ptr = torch.zeros(S + 1, dtype=torch.int64, device=device)
    torch.cumsum(slice_size, 0, out=slice_ptr[1:])
    total = int(slice_ptr[-1].item())
    pos_slice = torch.repeat_interleave(torch.arange(S, device=device), slice_size)
    lane = (torch.arange(total, device=device) - slice_ptr[pos_slice]) % 32
    col = torch.clamp(pos_slice * 32 + lane, max=n_cols - 1).to(torch.int32)
    del pos_slice, lane
    val = torch.zeros(total, dtype=torch.complex128, device=device)
    gprefix = torch.zeros((S, G), dtype=torch.int64, device=device)
    if G > 1:
        gprefix[:, 1:] = torch.cumsum(widths, dim=1)[:, :-1]
    for g, (indptr, indices, data, _) in enumerate(groups):
        nnz = indices.numel()
        cnt = indptr[1:] - indptr[:-1]
        rows = torch.repeat_interleave(torch.arange(n, device=device), cnt)
        # order each row's entries by (col XOR row): rows stay grouped, key < 2^31
        key = (rows << 32) | (indices ^ rows)
        key, perm = torch.sort(key)
        del key
        ci, dv = indices[perm], data[perm]
        del perm
        q = torch.arange(nnz, device=device) - indptr[rows]
        sl = torch.div(rows, 32, rounding_mode="floor")
        dst = slice_ptr[sl] + 32 * (gprefix[sl, g] + q) + rows % 32
        del q, sl
        col[dst] = ci.to(torch.int32)
        val[dst] = dv
        del dst, ci, dv, rows
    return slice_ptr, widths.reshape(-1).to(torch.int32), col, val, total


def _device_split_entries(indptr, indices, data, n):
    """Device twin of :func:`qutip_gb300.operator.split_entries`: ``(rows, off2, a)``."""
    device = indptr.device
    cnt = indptr[1:] - indptr[:-1]
    rows = torch.repeat_interleave(torch.arange(n, device=device), cnt)
    idx = indices.to(torch.int64)
    _, perm = torch.sort((rows << 32) | (idx ^ rows))
    off = idx[perm] - rows
    dv = data[perm].to(torch.complex128)
    del perm, idx
    r2 = rows.repeat_interleave(2)
    off2 = off.repeat_interleave(2) * 2 + torch.tensor([0, 1], device=device).repeat(dv.numel())
    a = torch.view_as_real(dv).reshape(-1)
    keep = a != 0
    return r2[keep], off2[keep], a[keep]


def _device_dict_split_layout(groups, n, max_table):
    """Device twin of the real/imaginary split dictionary layout (complex128)."""
    device = groups[0][0].device
    G = len(groups)
    S = (n + 31) // 32
    ents = [_device_split_entries(ip, ix, v, n) for ip, ix, v, _ in groups]
    counts = torch.zeros((G, S * 32), dtype=torch.int64, device=device)
    for g, (r, _, _) in enumerate(ents):
        counts[g, :n] = torch.bincount(r, minlength=n)
    widths = counts.view(G, S, 32).amax(dim=2)          # exact: the kernel skips the rest
    sect = 32 * ((widths + 3) // 4 * 4)
    gsize = sect.sum(dim=1)
    gbase = torch.cumsum(gsize, 0) - gsize
    row_ptr = torch.zeros((G, S + 1), dtype=torch.int64, device=device)
    row_ptr[:, 1:] = torch.cumsum(sect, dim=1)
    row_ptr += gbase[:, None]
    total = int(gsize.sum().item())
    if total >= 2**31 - 16:
        return None
    codes = torch.zeros(total, dtype=torch.int32, device=device)
    t_off, t_val, t_start = [], [], [0]
    for g, (r, off2, a) in enumerate(ents):
        vbits, vcode = torch.unique(a.view(torch.int64), return_inverse=True)
        V = max(int(vbits.numel()), 1)
        ukey, kcode = torch.unique(off2 * V + vcode, return_inverse=True)
        del vcode
        if ukey.numel() + 1 > max_table:
            return None
        uoff = torch.div(ukey, V, rounding_mode="floor")
        ua = vbits[ukey - uoff * V].view(torch.float64)
        tv = torch.complex(torch.where((uoff & 1) == 1, -ua, ua), ua)
        t_off.append(torch.cat([torch.zeros(1, dtype=torch.int64, device=device), uoff]))
        t_val.append(torch.cat([torch.zeros(1, dtype=torch.complex128, device=device), tv]))
        t_start.append(t_start[-1] + ukey.numel() + 1)
        start = torch.zeros(n + 1, dtype=torch.int64, device=device)
        torch.cumsum(counts[g, :n], 0, out=start[1:])
        q = torch.arange(r.numel(), device=device) - start[r]
        sl = torch.div(r, 32, rounding_mode="floor")
        dst = row_ptr[g, sl] + 128 * torch.div(q, 4, rounding_mode="floor") + 4 * (r % 32) + q % 4
        codes[dst] = kcode.to(torch.int32) + 1
        del q, sl, dst, kcode, start
    if t_start[-1] > max_table:
        return None
    longest = max(b - a for a, b in zip(t_start[:-1], t_start[1:]))
    if longest > 65536:
        return None
    cb = 1 if longest <= 256 else 2
    codes = codes.to(torch.uint8) if cb == 1 else codes.to(torch.int16)
    return (row_ptr.reshape(-1).to(torch.int32), widths.t().reshape(-1).to(torch.int32), codes,
            cb, torch.cat(t_off).to(torch.int32), torch.cat(t_val),
            torch.tensor(t_start, dtype=torch.int32, device=device), total)


def device_dict_layout(groups, n_cols, dtype: str, max_table: int = 4096, split: bool = False):
    """Dictionary-coded sliced layout of device CSR groups: the layout of
    :func:`qutip_gb300.operator.dict_sliced_layout` computed with device sorts, uniques
    and scatters (tables in a different but equivalent order).  Returns
    ``(row_ptr, widths, codes, code_bytes, table_off, table_val, table_start, stored)``
    as device tensors, or ``None`` when the (column - row, value) pairs do not fit
    ``max_table`` table entries.  ``split=True``: the real/imaginary split of complex128
    entries (``QG_LAYOUT_SLICED_DICT_RI``)."""
    if split:
        return _device_dict_split_layout(groups, groups[0][0].numel() - 1, max_table)
    indptr0 = groups[0][0]
    device = indptr0.device
    n = indptr0.numel() - 1
    G = len(groups)
    S = (n + 31) // 32
    vdt = torch.complex64 if dtype == "c64" else torch.complex128
    counts = torch.zeros((G, S * 32), dtype=torch.int64, device=device)
    for g, (indptr, _, _, _) in enumerate(groups):
        counts[g, :n] = indptr[1:] - indptr[:-1]
    widths = counts.view(G, S, 32).amax(dim=2)                    # [G, S], exact
    del counts
    sect = 32 * ((widths + 3) // 4 * 4)
    gsize = sect.sum(dim=1)
    gbase = torch.cumsum(gsize, 0) - gsize
    row_ptr = torch.zeros((G, S + 1), dtype=torch.int64, device=device)
    row_ptr[:, 1:] = torch.cumsum(sect, dim=1)
    row_ptr += gbase[:, None]
    total = int(gsize.sum().item())
    if total >= 2**31 - 16:
        return None
    codes = torch.zeros(total, dtype=torch.int32, device=device)
    t_off, t_val, t_start = [], [], [0]
    for g, (indptr, indices, data, _) in enumerate(groups):
        nnz = indices.numel()
        cnt = indptr[1:] - indptr[:-1]
        rows = torch.repeat_interleave(torch.arange(n, device=device), cnt)
        idx = indices.to(torch.int64)
        key = (rows << 32) | (idx ^ rows)              # rows stay grouped, (col XOR row) within
        _, perm = torch.sort(key)
        del key
        off = idx[perm] - rows
        dv = data[perm].to(vdt)
        del perm, idx
        nz = dv != 0
        # distinct values by their bit patterns, with one-dimensional uniques only
        parts = torch.view_as_real(dv[nz]).contiguous()
        if dtype == "c64":
            vbits, vcode = torch.unique(parts.view(torch.int64).view(-1), return_inverse=True)
        else:
            pb = parts.view(torch.int64)                 # [m, 2]: real and imaginary bits
            ure, ire = torch.unique(pb[:, 0], return_inverse=True)
            uim, iim = torch.unique(pb[:, 1], return_inverse=True)
            del pb
            vkey, vcode = torch.unique(ire * uim.numel() + iim, return_inverse=True)
            del ire, iim
            q_re = torch.div(vkey, uim.numel(), rounding_mode="floor")
            vbits = torch.stack([ure[q_re], uim[vkey - q_re * uim.numel()]], dim=1)
            del ure, uim, vkey, q_re
        del parts
        V = max(int(vbits.shape[0]), 1)
        ukey, kcode = torch.unique(off[nz] * V + vcode, return_inverse=True)
        del vcode
        if ukey.numel() + 1 > max_table:
            return None
        voff = torch.div(ukey, V, rounding_mode="floor")
        vals = vbits[ukey - voff * V].contiguous()
        if dtype == "c64":
            vals = vals.view(torch.complex64)
        else:
            vals = torch.view_as_complex(vals.view(torch.float64))
        t_off.append(torch.cat([torch.zeros(1, dtype=torch.int64, device=device), voff]))
        t_val.append(torch.cat([torch.zeros(1, dtype=vdt, device=device), vals.reshape(-1)]))
        t_start.append(t_start[-1] + ukey.numel() + 1)
        code = torch.zeros(nnz, dtype=torch.int32, device=device)
        code[nz] = kcode.to(torch.int32) + 1
        del kcode, nz, off, dv
        q = torch.arange(nnz, device=device) - indptr[rows]
        sl = torch.div(rows, 32, rounding_mode="floor")
        dst = row_ptr[g, sl] + 128 * torch.div(q, 4, rounding_mode="floor") + 4 * (rows % 32) + q % 4
        codes[dst] = code
        del q, sl, dst, code, rows
    if t_start[-1] > max_table:
        return None
    longest = max(b - a for a, b in zip(t_start[:-1], t_start[1:]))
    cb = 1 if longest <= 256 else 2
    codes = codes.to(torch.uint8) if cb == 1 else codes.to(torch.int16)
    return (row_ptr.reshape(-1).to(torch.int32), widths.t().reshape(-1).to(torch.int32), codes,
            cb, torch.cat(t_off).to(torch.int32), torch.cat(t_val),
            torch.tensor(t_start, dtype=torch.int32, device=device), total)
