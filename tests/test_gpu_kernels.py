"""GPU kernels through the C ABI against the CPU oracle and the reference's golden vectors."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda")


def _t(a, dtype=torch.complex128):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


@pytest.mark.parametrize("i", [0, 1, 2])
def test_spmv_c128_matches_reference_every_launch_shape(dev, i):
    from qutip_gb300.operator import DeviceOperator
    g = golden("kernels.npz")
    n = len(g[f"spmv{i}_x"])
    A = sp.csr_matrix((g[f"spmv{i}_data"], g[f"spmv{i}_indices"], g[f"spmv{i}_indptr"]), shape=(n, n))
    op = DeviceOperator([(A, None)])
    cands = op.candidates()
    assert any(c[0] == "staged" for c in cands)
    for cand in cands:
        op.set_launch(cand)
        y = _t(g[f"spmv{i}_out0"])
        op.matvec(0.0, _t(g[f"spmv{i}_x"]), y, alpha=0.5j, beta=1.0)
        np.testing.assert_allclose(y.cpu().numpy(), g[f"spmv{i}_res"], rtol=1e-13, atol=1e-13,
                                   err_msg=str(cand))


def test_staged_tiles_cover_many_tiles_and_groups(dev):
    """A multi-tile, two-group operator: every launch shape equals the scipy result."""
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    s = S.ising_chain(6)
    rng = np.random.default_rng(5)
    for dt, tol in (("c128", 1e-12), ("c64", 2e-5)):
        op = DeviceOperator(s.terms, dtype=dt, fmt="csr")
        assert len(op._tiles[2048]) > 10
        x = rng.normal(size=op.n_cols) + 1j * rng.normal(size=op.n_cols)
        want = sum((m * (1 if c is None else c(0.9))) @ x for m, c in s.terms)
        xt = _t(x, torch.complex128 if dt == "c128" else torch.complex64)
        for cand in op.candidates():
            op.set_launch(cand)
            y = torch.zeros(op.n_rows, dtype=xt.dtype, device="cuda")
            op.matvec(0.9, xt, y)
            np.testing.assert_allclose(y.cpu().numpy(), want, rtol=tol, atol=tol * np.abs(want).max(),
                                       err_msg=f"{dt} {cand}")
    from qutip_gb300 import _lib
    assert _lib.load().qg_device_fault() == 0


@pytest.mark.parametrize("i", [0, 1, 2])
def test_spmv_c64_error_bound(dev, i):
    from oracle.kernels import spmv_csr
    from qutip_gb300.operator import DeviceOperator
    g = golden("kernels.npz")
    n = len(g[f"spmv{i}_x"])
    A = sp.csr_matrix((g[f"spmv{i}_data"], g[f"spmv{i}_indices"], g[f"spmv{i}_indptr"]), shape=(n, n))
    op = DeviceOperator([(A, None)], dtype="c64")
    op.tune()
    x = g[f"spmv{i}_x"]
    y = torch.zeros(n, dtype=torch.complex64, device="cuda")
    op.matvec(0.0, _t(x, torch.complex64), y)
    want = spmv_csr(A.data, A.indices, A.indptr, x)
    # FP32 accumulation: |err| <= ~nnz_row * eps32 * sum|a||x|
    bound = 8 * np.finfo(np.float32).eps * (abs(A) @ np.abs(x)) + 1e-30
    assert np.all(np.abs(y.cpu().numpy() - want) <= bound)


@pytest.mark.parametrize("L", [5, 7])
def test_sliced_layout_matches_scipy(dev, L):
    """Sliced ELLPACK storage (32-row slices, XOR-ordered rows) for both dtypes and
    both epilogues: AXPBY against scipy, and a Vern7 step against the CSR storage."""
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.vern7 import GpuVern7
    s = S.ising_chain(L)
    rng = np.random.default_rng(L)
    x = rng.normal(size=4 ** L) + 1j * rng.normal(size=4 ** L)
    want = sum((m * (1 if c is None else c(1.7))) @ x for m, c in s.terms)
    for fmt in ("sliced", "dict"):
        for dt, tol in (("c128", 1e-12), ("c64", 2e-5)):
            op = DeviceOperator(s.terms, dtype=dt, fmt=fmt)
            assert op.launch[0] == fmt and op.stored >= op.nnz
            xt = _t(x, torch.complex128 if dt == "c128" else torch.complex64)
            y = _t(np.ones(op.n_rows), xt.dtype)
            op.matvec(1.7, xt, y, alpha=2.0, beta=-1.0)
            np.testing.assert_allclose(y.cpu().numpy(), 2 * want - 1, rtol=tol,
                                       atol=tol * np.abs(want).max(), err_msg=f"{fmt} {dt}")
    outs = []
    for fmt in ("sliced", "csr", "dict"):
        op = DeviceOperator(s.terms, dtype="c128", fmt=fmt)
        assert fmt != "dict" or op.dict_split      # complex128: real/imaginary split tables
        ig = GpuVern7(op)
        ig.set_initial_value(torch.from_numpy(s.state0).cuda(), 0.0)
        ig.integrate(0.7)
        outs.append(ig.get_state().cpu().numpy())
    np.testing.assert_allclose(outs[0], outs[1], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(outs[2], outs[1], rtol=1e-12, atol=1e-14)


def test_split_dictionary_with_complex_coefficients_and_entries(dev):
    """The complex128 real/imaginary split dictionary: complex, real and imaginary
    entries (a banded matrix and the Ising Liouvillian, whose diagonal is complex), a
    complex time-dependent coefficient (the general coefficient product) and a real one
    (its two-multiply-add path), a row count that is not a multiple of 32; matvec and a
    Vern7 step against the CSR storage."""
    from qutip_gb300 import _lib
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.vern7 import GpuVern7
    n = 1100
    rng = np.random.default_rng(11)
    diags = {-33: 0.5, -1: -0.25j, 0: 0.3 + 0.7j, 2: 1.1, 31: -0.2 - 0.4j}
    band = sp.diags([np.full(n - abs(k), v) for k, v in diags.items()], list(diags), shape=(n, n),
                    format="csr", dtype=np.complex128)
    other = sp.diags([np.full(n - 5, 0.9j), np.full(n, -0.1)], [5, 0], shape=(n, n), format="csr",
                     dtype=np.complex128)
    terms = [(band, None), (other, coefficient("exp(1j*w*t)", args={"w": 0.8})),
             (band.T.tocsr() * 0.5, coefficient("cos(w*t)", args={"w": 1.3}))]
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    t = 0.77
    want = sum((m * (1 if c is None else c(t))) @ x for m, c in terms)
    op = DeviceOperator(terms, dtype="c128", fmt="dict")
    assert op.dict_split and op.struct.layout == _lib.QG_LAYOUT_SLICED_DICT_RI
    y = _t(np.ones(n))
    op.matvec(t, _t(x), y, alpha=1.5 - 0.5j, beta=0.25)
    np.testing.assert_allclose(y.cpu().numpy(), (1.5 - 0.5j) * want + 0.25, rtol=1e-12,
                               atol=1e-12 * np.abs(want).max())
    outs = []
    for fmt in ("csr", "dict"):
        o = DeviceOperator(terms, dtype="c128", fmt=fmt)
        ig = GpuVern7(o, atol=1e-10, rtol=1e-9)
        ig.set_initial_value(_t(x / np.linalg.norm(x)), 0.0)
        ig.integrate(0.4)
        outs.append(ig.get_state().cpu().numpy())
    np.testing.assert_allclose(outs[1], outs[0], rtol=1e-12, atol=1e-14)


def test_grouped_coefficients_match_scipy(dev):
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    s = S.ising_chain(4)
    op = DeviceOperator(s.terms)
    assert op.n_groups == 2
    rng = np.random.default_rng(3)
    x = rng.normal(size=op.n_cols) + 1j * rng.normal(size=op.n_cols)
    for t in (0.0, 0.37, 5.1):
        y = torch.zeros(op.n_rows, dtype=torch.complex128, device="cuda")
        op.matvec(t, _t(x), y)
        want = sum((m * (1 if c is None else c(t))) @ x for m, c in s.terms)
        np.testing.assert_allclose(y.cpu().numpy(), want, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("expr,args", [("cos(w*t)", {"w": 1.3}),
                                       ("exp(-1j*w*t)*sqrt(t+1)", {"w": 2.0}),
                                       ("tanh(t-2)+arctan(t)-log(t+2)", {}),
                                       ("conj(exp(1j*t))**2/(1+t)", {})])
def test_device_coefficient_interpreter(dev, expr, args):
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.operator import DeviceOperator
    c = coefficient(expr, args)
    op = DeviceOperator([(sp.identity(1, format="csr"), c)])
    x = _t(np.ones(1))
    for t in (0.0, 0.37, 3.3):
        y = torch.zeros(1, dtype=torch.complex128, device="cuda")
        op.matvec(t, x, y)
        assert abs(complex(y.cpu().numpy()[0]) - c(t)) <= 1e-13 * max(1.0, abs(c(t)))


@pytest.mark.parametrize("i", [0, 1, 2])
def test_dia_matches_reference(dev, i):
    from qutip_gb300.operator import DeviceDia
    g = golden("kernels.npz")
    n = len(g[f"spmv{i}_x"])
    m = sp.dia_matrix((g[f"dia{i}_data"], g[f"dia{i}_offsets"]), shape=(n, n))
    op = DeviceDia(m)
    y = torch.zeros(n, dtype=torch.complex128, device="cuda")
    op.matvec(_t(g[f"spmv{i}_x"]), y)
    np.testing.assert_allclose(y.cpu().numpy(), g[f"dia{i}_res"], rtol=1e-13, atol=1e-13)


def test_spmm_matches_columnwise(dev):
    from qutip_gb300.operator import DeviceOperator
    g = golden("kernels.npz")
    n = len(g["spmv1_x"])
    A = sp.csr_matrix((g["spmv1_data"], g["spmv1_indices"], g["spmv1_indptr"]), shape=(n, n))
    op = DeviceOperator([(A, None)])
    rng = np.random.default_rng(0)
    X = rng.normal(size=(7, n)) + 1j * rng.normal(size=(7, n))
    Y = torch.zeros((7, n), dtype=torch.complex128, device="cuda")
    op.matmat(0.0, _t(X), Y)
    np.testing.assert_allclose(Y.cpu().numpy(), (A @ X.T).T, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("i", [0, 1])
def test_expect_dm_and_ket_match_reference(dev, i):
    from qutip_gb300 import _lib
    from qutip_gb300.solver import ExpectOps
    g = golden("kernels.npz")
    n = len(g[f"spmv{i}_x"])
    A = sp.csr_matrix((g[f"spmv{i}_data"], g[f"spmv{i}_indices"], g[f"spmv{i}_indptr"]), shape=(n, n))
    ex = ExpectOps([A, sp.identity(n)])
    rho = _t(g[f"exp{i}_rho"])
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    f = (C.c_double * 16)()
    v = _lib.StateView(n * n, 0, 0, rho.data_ptr(), rho.data_ptr(), 0, 0, f)
    ex.expect_dm(n, v, out)
    o = out.cpu().numpy()
    np.testing.assert_allclose(o[0] + 1j * o[1], g[f"exp{i}_dm"], rtol=1e-12)
    np.testing.assert_allclose(o[4] + 1j * o[5], np.trace(g[f"exp{i}_rho"].reshape(n, n, order="F")),
                               rtol=1e-12)
    psi = _t(g[f"spmv{i}_x"])
    v = _lib.StateView(n, 0, 0, psi.data_ptr(), psi.data_ptr(), 0, 0, f)
    ex.expect_ket(v, out)
    o = out.cpu().numpy()
    np.testing.assert_allclose(o[0] + 1j * o[1], g[f"exp{i}_ket"], rtol=1e-12)
    np.testing.assert_allclose(o[4], np.vdot(g[f"spmv{i}_x"], g[f"spmv{i}_x"]).real, rtol=1e-12)


def test_norm2_and_combine(dev):
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.vern7 import GpuVern7
    n = 1000
    op = DeviceOperator([(sp.identity(n, format="csr"), None)])
    ig = GpuVern7(op)
    rng = np.random.default_rng(1)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    assert abs(ig._norm(_t(x)) - np.linalg.norm(x)) < 1e-12 * np.linalg.norm(x)
    ks = rng.normal(size=(16, n)) + 1j * rng.normal(size=(16, n))
    ig.k.copy_(_t(ks.reshape(-1)))
    f = rng.normal(size=16)
    f[3] = 0.0
    out = torch.zeros(n, dtype=torch.complex128, device="cuda")
    ig._combine(_t(x), list(f), out)
    np.testing.assert_allclose(out.cpu().numpy(), x + f @ ks, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("order,uniform", [(0, True), (1, False), (3, True), (3, False)])
def test_device_interpolated_coefficient(dev, order, uniform):
    """Piecewise polynomials (the reference's InterCoefficient form) on the device vs
    the host evaluation, inside, at and outside the breakpoints."""
    from qutip_gb300.coefficients import interpolation
    from qutip_gb300.operator import DeviceOperator
    rng = np.random.default_rng(order)
    n = 9
    tl = np.linspace(0.0, 4.0, n) if uniform else np.sort(rng.uniform(0, 4, n))
    poly = rng.normal(size=(order + 1, n)) + 1j * rng.normal(size=(order + 1, n))
    c = interpolation(tl, poly, (tl[1] - tl[0]) if uniform else 0.0) * 2.0 + 0.5j
    op = DeviceOperator([(sp.identity(1, format="csr"), c)])
    x = _t(np.ones(1))
    for t in list(tl) + [-1.0, 0.123, 1.9, 3.999, 7.0]:
        y = torch.zeros(1, dtype=torch.complex128, device="cuda")
        op.matvec(t, x, y)
        assert abs(complex(y.cpu().numpy()[0]) - c(t)) <= 1e-13 * max(1.0, abs(c(t)))


@pytest.mark.parametrize("fmt", ["csr", "sliced"])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_spmv_ragged_rows_and_empty_group(dev, fmt, dtype):
    """Rows without entries, a coefficient group that is all zero, and a row count
    that is not a multiple of the 32-row slice."""
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.operator import DeviceOperator
    rng = np.random.default_rng(5)
    n = 1061
    a = (sp.random(n, n, density=0.01, random_state=1, format="csr", dtype=np.complex128)
         + 1j * sp.random(n, n, density=0.002, random_state=2, format="csr"))
    keep = np.ones(n)
    keep[::7] = 0                                   # every 7th row empty
    a = sp.csr_matrix(sp.diags(keep) @ a)
    a.eliminate_zeros()
    empty = sp.csr_matrix((n, n), dtype=np.complex128)
    c = coefficient("cos(t)")
    op = DeviceOperator([(a, None), (empty, c)], dtype=dtype, merge=False, fmt=fmt)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    tdt = torch.complex128 if dtype == "c128" else torch.complex64
    y = torch.full((n,), 7.0 + 7.0j, dtype=tdt, device="cuda")
    op.matvec(0.4, _t(x, tdt), y)
    want = a @ x
    tol = 1e-12 if dtype == "c128" else 3e-6
    np.testing.assert_allclose(y.cpu().numpy(), want, rtol=tol, atol=tol * np.abs(want).max())
    assert np.all(y.cpu().numpy()[::7] == 0)


def test_spmv_one_by_one(dev):
    from qutip_gb300.operator import DeviceOperator
    op = DeviceOperator([(sp.csr_matrix(np.array([[2.0 - 1.0j]])), None)])
    y = torch.zeros(1, dtype=torch.complex128, device="cuda")
    op.matvec(0.0, _t(np.array([3.0 + 0.5j])), y, alpha=2.0, beta=0.0)
    assert complex(y.item()) == pytest.approx(2 * (2.0 - 1.0j) * (3.0 + 0.5j), abs=1e-14)


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_spmv_dict_ragged_rows_and_empty_group(dev, dtype):
    """Dictionary-coded storage: entries on a few diagonals with values from a small
    set, every 7th row empty, a row count that is not a multiple of 32, an all-zero
    coefficient group, columns near both edges, and both Vern7 epilogues."""
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.vern7 import GpuVern7
    rng = np.random.default_rng(9)
    n = 1061
    rows, cols, vals = [], [], []
    choices = [1.0, -0.5j, 0.25 + 1j, -2.0]
    for r in range(n):
        if r % 7 == 0:
            continue
        for o in (-40, -1, 0, 3, 33):
            if 0 <= r + o < n and rng.random() < 0.8:
                rows.append(r)
                cols.append(r + o)
                vals.append(choices[rng.integers(4)])
    a = sp.csr_matrix((vals, (rows, cols)), shape=(n, n), dtype=np.complex128)
    empty = sp.csr_matrix((n, n), dtype=np.complex128)
    c = coefficient("cos(t)")
    op = DeviceOperator([(a, None), (empty, c)], dtype=dtype, merge=False, fmt="dict")
    assert op.launch[0] == "dict" and op.code_bytes == 1
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    tdt = torch.complex128 if dtype == "c128" else torch.complex64
    y = torch.full((n,), 7.0 + 7.0j, dtype=tdt, device="cuda")
    op.matvec(0.4, _t(x, tdt), y)
    want = a @ x
    tol = 1e-12 if dtype == "c128" else 3e-6
    np.testing.assert_allclose(y.cpu().numpy(), want, rtol=tol, atol=tol * np.abs(want).max())
    assert np.all(y.cpu().numpy()[::7] == 0)
    # a Vern7 integration through the fused stages agrees with the CSR storage
    gen = [((-0.1j) * (a + a.conj().T), None), (empty, c)]
    outs = []
    for fmt in ("csr", "dict"):
        ig = GpuVern7(DeviceOperator(gen, dtype="c128", merge=False, fmt=fmt))
        ig.set_initial_value(_t(x / np.linalg.norm(x)), 0.0)
        ig.integrate(0.5)
        outs.append(ig.get_state().cpu().numpy())
    np.testing.assert_allclose(outs[1], outs[0], rtol=1e-12, atol=1e-14)
