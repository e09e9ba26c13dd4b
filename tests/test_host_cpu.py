"""Host-side checks that need no GPU: the C-ABI library loads and exports every
declared symbol, the compiled-in tableau is the reference's, coefficients compile."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden

from qutip_gb300 import coefficients as CF


def _header_functions():
    src = open(os.path.join(ROOT, "include", "qutip_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:int|int64_t|const char\s*\*)\s*(qg_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    from qutip_gb300 import _lib
    lib = _lib.load()
    declared = _header_functions()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in include/qutip_gb300.h but not exported"
    assert set(_lib.declared_symbols()) <= set(declared)
    assert lib.qg_version() >= 1


def test_compiled_tableau_matches_reference():
    import ctypes as C
    from qutip_gb300 import _lib
    g = golden("vern7_tableau.npz")
    a, b, c, e, bi = (np.zeros(256), np.zeros(10), np.zeros(16), np.zeros(10), np.zeros(112))
    rc = _lib.load().qg_vern7_tableau(*(x.ctypes.data_as(C.c_void_p) for x in (a, b, c, e, bi)))
    assert rc == 0
    assert np.array_equal(a.reshape(16, 16), g["a"])
    assert np.array_equal(b, g["b"]) and np.array_equal(c, g["c"]) and np.array_equal(e, g["e"])
    assert np.array_equal(bi.reshape(16, 7), g["bi"])


@pytest.mark.parametrize("expr,args", [
    ("cos(w*t)", {"w": 1.3}),
    ("exp(-1j*w*t) + 0.5*sin(t)**2", {"w": 2.0}),
    ("sqrt(t+1)*conj(exp(1j*t))/(1+t)", {}),
    ("np.cos(2*np.pi*f*t) - a", {"f": 0.3, "a": 0.1}),
    ("tanh(t-2) + arctan(t) - log(t + 2) + abs(-t) + real(1j*t+3)", {}),
])
def test_coefficient_programs(expr, args):
    c = CF.coefficient(expr, args)
    ns = {"cos": np.cos, "sin": np.sin, "exp": np.exp, "sqrt": np.sqrt, "conj": np.conj,
          "np": np, "tanh": np.tanh, "arctan": np.arctan, "log": np.log, "abs": np.abs,
          "real": np.real, **args}
    for t in (0.0, 0.37, 2.5, 9.9):
        want = complex(eval(expr, ns, {"t": t}))
        assert abs(c(t) - want) <= 1e-12 * max(1.0, abs(want))
    assert (c.conj()(0.7)) == c(0.7).conjugate()
    assert abs((c + 2.0)(0.7) - (c(0.7) + 2.0)) < 1e-15


def test_coefficient_rejects_unknown_names():
    with pytest.raises(ValueError):
        CF.coefficient("cos(w*t)")
    with pytest.raises(ValueError):
        CF.coefficient("__import__('os')")
    with pytest.raises(TypeError):
        CF.coefficient(lambda t: t)


def test_pack_programs_layout():
    code, starts, consts = CF.pack_programs([None, CF.coefficient("cos(w*t)", {"w": 2.0})])
    assert starts[0] == 0 and starts[-1] == len(code)
    assert code[starts[1] - 1] == CF.OPCODES["END"]
    assert consts.dtype == np.float64 and len(consts) % 2 == 0


def test_struct_layouts_match_the_library():
    """ctypes / numpy mirrors of the ABI structs have the library's sizes."""
    import ctypes as C
    from qutip_gb300 import _lib
    from qutip_gb300.batched import ITEM_DTYPE, SYSTEM_DTYPE, BatchStruct
    out = np.zeros(10, dtype=np.int64)
    n = _lib.load().qg_abi_sizes(out.ctypes.data_as(C.c_void_p), 10)
    assert n == 10
    mine = [C.sizeof(_lib.CsrGroups), C.sizeof(_lib.Dia), C.sizeof(_lib.RkBuffers),
            C.sizeof(_lib.StateView), SYSTEM_DTYPE.itemsize, ITEM_DTYPE.itemsize,
            C.sizeof(BatchStruct), C.sizeof(_lib.Lindblad), C.sizeof(_lib.DenseLindblad),
            C.sizeof(_lib.Sde)]
    assert list(out) == mine


def test_sliced_layout_host_builder():
    """The sliced-ELLPACK builder reproduces A @ x and keeps warps' gathers local."""
    import scipy.sparse as sp
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import sliced_layout
    s = S.ising_chain(5)
    mats = [m for m, _ in s.terms]
    rp, w, col, val, total = sliced_layout(mats, mats[0].shape[1])
    n, G = mats[0].shape[0], len(mats)
    x = np.random.default_rng(0).normal(size=n) + 0.5j
    for g in range(G):
        y = np.zeros(n, complex)
        for sl in range(len(rp) - 1):
            off = rp[sl] + 32 * int(w[sl * G:sl * G + g].sum())
            for j in range(w[sl * G + g]):
                idx = off + 32 * j + np.arange(32)
                rows = sl * 32 + np.arange(32)
                ok = rows < n
                y[rows[ok]] += val[idx[ok]] * x[col[idx[ok]]]
        np.testing.assert_allclose(y, mats[g] @ x, atol=1e-13)
    assert total <= 1.15 * sum(m.nnz for m in mats)


def test_batch_argument_validation_before_any_device_call():
    """qg_batch_vern7 rejects malformed launches on the host, before any CUDA call."""
    import ctypes as C
    from qutip_gb300 import _lib
    from qutip_gb300.batched import BatchStruct
    lib = _lib.load()
    assert lib.qg_batch_vern7(None, None) == _lib.QG_ERR_ARG
    fake = 256  # never dereferenced on the host
    b = BatchStruct()
    for f in ("systems", "items", "op_rp", "op_col", "op_val", "tlist", "y0", "out", "status",
              "work", "queue"):
        setattr(b, f, fake)
    b.n_systems, b.n_items, b.dtype, b.max_n, b.n_slots = 1, 0, _lib.QG_C64, 16, 1
    assert lib.qg_batch_vern7(C.byref(b), None) == _lib.QG_OK        # nothing to do
    b.group = 7
    assert lib.qg_batch_vern7(C.byref(b), None) == _lib.QG_ERR_ARG   # unknown group
    b.group = _lib.QG_GROUP_CLUSTER
    b.stage_op_entries, b.stage_op_rp = 100, 17
    assert lib.qg_batch_vern7(C.byref(b), None) == _lib.QG_ERR_ARG   # staging needs warp/CTA
    b.group, b.n_systems = _lib.QG_GROUP_CTA, 2
    assert lib.qg_batch_vern7(C.byref(b), None) == _lib.QG_ERR_ARG   # staging needs 1 system
    b.n_systems, b.stage_op_entries = 1, 10 ** 6
    assert lib.qg_batch_vern7(C.byref(b), None) == _lib.QG_ERR_ARG   # exceeds shared memory
    b.stage_op_entries, b.dtype = 0, 5
    assert lib.qg_batch_vern7(C.byref(b), None) == _lib.QG_ERR_UNSUPPORTED
    assert b"dtype" in lib.qg_last_error()


def _banded(n, offsets, values, empty_every=7, seed=5):
    """n x n matrix with entries on a few diagonals, values from a small set, and every
    ``empty_every``-th row empty."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for r in range(n):
        if r % empty_every == 0:
            continue
        for o in offsets:
            c = r + o
            if 0 <= c < n and rng.random() < 0.8:
                rows.append(r)
                cols.append(c)
                vals.append(values[rng.integers(len(values))])
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n), dtype=np.complex128)


def _emulate_dict(lay, n, x, coefs, split=False):
    """The dictionary kernel's indexing on the host: codes of lane l, chunk q of slice s
    and group g at row_ptr[g*(S+1)+s] + 128 q + 4 l + u.  ``split``: the real/imaginary
    split tables (offset << 1 with the low bit marking an imaginary part, value pair
    (c1, c2) applied as (c1 p, c2 q) to x with real and imaginary parts exchanged for an
    imaginary part)."""
    rp, widths, codes, cb, t_off, t_val, t_start, total = lay
    G = len(t_start) - 1
    S = (n + 31) // 32
    y = np.zeros(S * 32, dtype=complex)
    for s in range(S):
        for lane in range(32):
            row = 32 * s + lane
            acc = 0j
            for g in range(G):
                w = widths[s * G + g]
                base = rp[g * (S + 1) + s]
                part = 0j
                for q in range((w + 3) // 4):
                    for u in range(min(4, w - 4 * q)):
                        k = int(codes[base + 128 * q + 4 * lane + u])
                        k = t_start[g] + (k if k < t_start[g + 1] - t_start[g] else 0)
                        if split:
                            oc = int(t_off[k])
                            col = min(max(row + (oc >> 1), 0), n - 1)
                            xv = x[col]
                            p, r = (xv.imag, xv.real) if oc & 1 else (xv.real, xv.imag)
                            part += complex(t_val[k].real * p, t_val[k].imag * r)
                            continue
                        col = min(max(row + t_off[k], 0), n - 1)
                        part += t_val[k] * x[col]
                acc += coefs[g] * part
            y[row] = acc
    return y[:n]


def test_dict_layout_reproduces_the_matvec():
    """The dictionary-coded sliced layout, walked with the kernel's indexing, gives A @ x:
    the Ising chain's Liouvillian (two groups) and a banded matrix with empty rows, a
    row count that is not a multiple of 32 and an all-zero group."""
    import scipy.sparse as sp
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import dict_sliced_layout
    rng = np.random.default_rng(1)
    s = S.ising_chain(3)
    mats = [m for m, _ in s.terms]
    n = mats[0].shape[0]
    lay = dict_sliced_layout(mats, n, "c128")
    assert lay is not None and lay[3] == 1          # one-byte codes
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    coefs = [1.0, 0.3 - 0.2j]
    want = mats[0] @ x + coefs[1] * (mats[1] @ x)
    np.testing.assert_allclose(_emulate_dict(lay, n, x, coefs), want, atol=1e-12)
    n = 101
    b = _banded(n, [-5, -1, 0, 2, 31], [1.0, -0.5j, 0.25 + 1j])
    lay = dict_sliced_layout([b, sp.csr_matrix((n, n), dtype=complex)], n, "c64")
    assert lay is not None
    rp, widths, codes, cb, t_off, t_val, t_start, total = lay
    assert list(np.diff(t_start)) == [len(set(zip(b.tocoo().col - b.tocoo().row,
                                                    b.tocoo().data))) + 1, 1]
    assert all(r % 128 == 0 for r in rp)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    np.testing.assert_allclose(_emulate_dict(lay, n, x, [1.0, 5.0]), b @ x, atol=1e-6)


def test_dict_layout_declines_incompressible_operators():
    import scipy.sparse as sp
    from qutip_gb300.operator import dict_sliced_layout
    m = sp.random(3000, 3000, density=0.01, random_state=3, format="csr")
    assert dict_sliced_layout([m], 3000, "c128") is None


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_device_dict_layout_reproduces_the_matvec(dtype):
    """The device-side dictionary builder (torch, run here on CPU tensors) gives a layout
    whose kernel walk reproduces the Liouvillian matvec, as the host builder does."""
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.superop import device_dict_layout, liouvillian_groups
    s = S.ising_chain(3, build_terms=False)
    groups = liouvillian_groups(s.h_terms, s.c_ops, device="cpu")
    n = groups[0][0].numel() - 1
    lay = device_dict_layout(groups, n, dtype)
    assert lay is not None
    host = tuple(v.numpy() if isinstance(v, torch.Tensor) else v for v in lay)
    rng = np.random.default_rng(4)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    coefs = [1.0 if c is None else c(0.8) for _, _, _, c in groups]
    mats = [sp_from(g, n) for g in groups]
    want = sum(c * (m @ x) for c, m in zip(coefs, mats))
    tol = 1e-12 if dtype == "c128" else 1e-6
    np.testing.assert_allclose(_emulate_dict(host, n, x, coefs), want, atol=tol * np.abs(want).max())


def test_split_dict_layout_reproduces_the_matvec():
    """The real/imaginary split tables (complex128): the Ising chain's Liouvillian, whose
    diagonal entries are complex and split in two codes, and a banded matrix with real,
    imaginary and complex entries; host and device builders agree with A @ x."""
    import scipy.sparse as sp
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import dict_sliced_layout
    from qutip_gb300.superop import device_dict_layout
    rng = np.random.default_rng(2)
    s = S.ising_chain(3)
    mats = [sp.csr_matrix(m) for m, _ in s.terms]
    n = mats[0].shape[0]
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    coefs = [1.0, 0.3 - 0.2j]
    want = mats[0] @ x + coefs[1] * (mats[1] @ x)
    lay = dict_sliced_layout(mats, n, "c128", split=True)
    assert lay is not None
    rp, widths, codes, cb, t_off, t_val, t_start, total = lay
    pad = np.zeros(len(t_val), dtype=bool)
    pad[t_start[:-1]] = True                       # code 0 of each group
    imag = ((t_off & 1) == 1) & ~pad
    real = ((t_off & 1) == 0) & ~pad
    assert np.all(t_val.imag[~pad] != 0) and np.all(t_val[pad] == 0)
    assert np.all(t_val.real[imag] == -t_val.imag[imag])
    assert np.all(t_val.real[real] == t_val.imag[real])
    n_parts = sum(int(np.count_nonzero(m.data.real) + np.count_nonzero(m.data.imag)) for m in mats)
    assert int(np.count_nonzero(codes)) == n_parts
    np.testing.assert_allclose(_emulate_dict(lay, n, x, coefs, split=True), want, atol=1e-12)
    groups = [(torch.from_numpy(m.indptr.astype(np.int64)), torch.from_numpy(m.indices.astype(np.int64)),
               torch.from_numpy(m.data), None) for m in mats]
    dl = device_dict_layout(groups, n, "c128", split=True)
    dh = tuple(v.numpy() if isinstance(v, torch.Tensor) else v for v in dl)
    assert dh[-1] == total and list(dh[6]) == list(t_start)
    np.testing.assert_allclose(_emulate_dict(dh, n, x, coefs, split=True), want, atol=1e-12)
    n = 101
    b = _banded(n, [-5, -1, 0, 2, 31], [1.0, -0.5j, 0.25 + 1j])
    z = sp.csr_matrix((n, n), dtype=complex)
    lay = dict_sliced_layout([b, z], n, "c128", split=True)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    np.testing.assert_allclose(_emulate_dict(lay, n, x, [1.0, 5.0], split=True), b @ x,
                               atol=1e-12)


def sp_from(group, n):
    import scipy.sparse as sp
    indptr, indices, data, _ = group
    return sp.csr_matrix((data.numpy(), indices.numpy(), indptr.numpy()), shape=(n, n))


def test_device_groups_operator_prefers_the_dictionary():
    """``DeviceOperator.from_device_groups`` (device assembly path, run on CPU tensors)
    builds the dictionary-coded storage and its struct, and keeps sliced on request."""
    from qutip_gb300 import _lib
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.superop import liouvillian_groups
    s = S.ising_chain(3, build_terms=False)
    groups = liouvillian_groups(s.h_terms, s.c_ops, device="cpu")
    op = DeviceOperator.from_device_groups(groups, "c128")
    assert op.fmt == "dict" and op.struct.layout == _lib.QG_LAYOUT_SLICED_DICT_RI
    assert op.dict_split
    assert op.struct.tile_nnz == op.code_bytes == 1 and op.struct.lanes == op.val.numel()
    assert op.struct.dict_off and op.struct.dict_start
    with pytest.raises(TypeError):
        op.astype("c64")                            # the split tables are complex128 only
    op64 = DeviceOperator.from_device_groups(groups, "c64")
    assert op64.fmt == "dict" and op64.struct.layout == _lib.QG_LAYOUT_SLICED_DICT
    op128 = op64.astype("c128")
    assert op128.val.dtype.is_complex and op128.struct.lanes == op64.struct.lanes
    sl = DeviceOperator.from_device_groups(groups, "c64", fmt="sliced")
    assert sl.fmt == "sliced" and sl.struct.layout == _lib.QG_LAYOUT_SLICED


def _groups(layout, **kw):
    from qutip_gb300 import _lib
    g = _lib.CsrGroups(64, 64, 1, _lib.QG_C64, layout, 1, 0, 0, 8, 8, 8, None, None, None, None,
                       None, None)
    for k, v in kw.items():
        setattr(g, k, v)
    return g


def test_layout_validation_before_any_device_call():
    """The entry points reject storage they cannot read before touching the device:
    spmm and expect need a CSR layout; the dictionary layout needs its tables, 1- or
    2-byte codes and a table size within QG_DICT_MAX."""
    import ctypes as C
    from qutip_gb300 import _lib
    lib = _lib.load()
    x = C.c_void_p(8)
    for layout in (_lib.QG_LAYOUT_SLICED, _lib.QG_LAYOUT_SLICED_DICT):
        g = _groups(layout)
        assert lib.qg_spmm_csr(C.byref(g), 0.0, x, x, 1, 64, 1.0, 0.0, 0.0, 0.0,
                               None) == _lib.QG_ERR_UNSUPPORTED
        v = _lib.StateView(64 * 64, 0, 0, 8, 8, 0, 0)
        assert lib.qg_expect_dm(C.byref(g), 64, C.byref(v), x, None) == _lib.QG_ERR_UNSUPPORTED
    base = dict(n_tiles=2, tile_row=8, dict_off=8, dict_start=8, tile_nnz=1)
    bad = [dict(dict_off=None), dict(dict_start=None), dict(tile_row=None), dict(n_tiles=1),
           dict(tile_nnz=4), dict(lanes=0), dict(lanes=_lib.QG_DICT_MAX + 1)]
    for change in bad:
        g = _groups(_lib.QG_LAYOUT_SLICED_DICT, **{**base, **change})
        assert lib.qg_spmv_csr(C.byref(g), 0.0, x, x, 1.0, 0.0, 0.0, 0.0, None) == \
            _lib.QG_ERR_ARG, change


def test_lindblad_validation_before_any_device_call():
    import ctypes as C
    from qutip_gb300 import _lib
    lib = _lib.load()
    x = C.c_void_p(8)

    def make(**kw):
        L = _lib.Lindblad()
        L.d, L.dtype, L.n_groups, L.n_diag_cops, L.n_cops = 4, _lib.QG_C64, 1, 0, 1
        L.a_width[0], L.c_width[0] = 1, 1
        L.a_diag = L.a_col = L.a_val = L.c_col = L.c_val = 8
        for k, v in kw.items():
            setattr(L, k, v)
        return L
    assert lib.qg_lindblad_apply(None, 0.0, x, x, 1.0, 0.0, 0.0, 0.0, None) == _lib.QG_ERR_ARG
    bad = [dict(d=0), dict(d=46341), dict(dtype=7), dict(n_groups=0), dict(n_groups=9),
           dict(n_cops=65), dict(n_diag_cops=2), dict(a_diag=None), dict(a_diag_const=1),
           dict(n_const_diag=1), dict(a_col=None), dict(c_val=None)]
    for change in bad:
        L = make(**change)
        rc = lib.qg_lindblad_apply(C.byref(L), 0.0, x, x, 1.0, 0.0, 0.0, 0.0, None)
        assert rc in (_lib.QG_ERR_ARG, _lib.QG_ERR_UNSUPPORTED), change
    L = make()
    L.a_width[0] = -1
    assert lib.qg_lindblad_apply(C.byref(L), 0.0, x, x, 1.0, 0.0, 0.0, 0.0, None) == _lib.QG_ERR_ARG
    rk = _lib.RkBuffers(16, 0, 1, 8, 8, None, None, 8, 8, 8, 8, 8)
    L = make()
    assert lib.qg_lindblad_stage(C.byref(L), C.byref(rk), 0, 0.0, 0.1, 1e-8, 1e-6, None) == \
        _lib.QG_ERR_ARG          # mixed form without its complex64 shadows
    rk = _lib.RkBuffers(15, 1, 1, 8, 8, None, None, 8, 8, 8, 8, 8)
    assert lib.qg_lindblad_stage(C.byref(L), C.byref(rk), 0, 0.0, 0.1, 1e-8, 1e-6, None) == \
        _lib.QG_ERR_ARG          # n != d*d


def test_conj_of_a_real_coefficient_is_itself():
    """A coefficient program that is real for every real t is its own conjugate, so the
    reference's ConjCoefficient of it (the spost part of a Liouvillian) shares its group;
    programs that can turn complex keep an explicit conj."""
    from qutip_gb300.coefficients import coefficient
    real = ["cos(w*t)", "amp * sin(2*t) + exp(-t)", "abs(sqrt(t - 1))", "real(exp(1j*t)) * t",
            "tanh(t) / (1 + t)"]
    maybe = ["exp(1j*w*t)", "sqrt(t)", "t**2", "log(t)", "1j * cos(t)"]
    for e in real:
        c = coefficient(e, args={"w": 1.3, "amp": 0.5})
        assert c.is_real() and c.conj() is c, e
        for t in (0.0, 0.7, 3.1):
            assert abs(c(t).imag) == 0.0
    for e in maybe:
        c = coefficient(e, args={"w": 1.3})
        assert not c.is_real() and c.conj().key() != c.key(), e
        for t in (0.3, 2.2):
            assert c.conj()(t) == c(t).conjugate()
