"""Host-side checks of the matrix-free Lindblad generator (mesolve's matrix form):
the oracle restatement against the reference's ``LindbladMatrixForm`` and against
the superoperator, and the operator the host builds for the kernel."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle.kernels import lindblad_matrix_form
from oracle.ref_workloads import reference_available
from qutip_gb300 import systems as S


def _kron_generator(a_terms, c_terms, t):
    """d^2 x d^2 matrix of rho -> A rho + rho A^dag + sum |f|^2 C rho C^dag on the
    column-major vec(rho): I (x) A + conj(A) (x) I + sum |f|^2 conj(C) (x) C."""
    d = a_terms[0][0].shape[0]
    eye = sp.identity(d, format="csr")
    A = sum((1.0 if c is None else c(t)) * m for m, c in a_terms)
    out = sp.kron(eye, A) + sp.kron(A.conj(), eye)
    for m, f in c_terms:
        w = 1.0 if f is None else abs(f(t)) ** 2
        out = out + w * sp.kron(m.conj(), m)
    return sp.csr_matrix(out)


def _superop(terms, t):
    return sp.csr_matrix(sum((1.0 if c is None else c(t)) * m for m, c in terms))


@pytest.mark.parametrize("system", ["jc", "ising"])
def test_host_generator_equals_the_superoperator(system):
    """The A = -i H_nh terms and collapse terms the host hands the kernel describe the
    same generator as the superoperator Liouvillian."""
    from qutip_gb300.lindblad import LindbladOperator
    s = S.jaynes_cummings(n_cav=4) if system == "jc" else S.ising_chain(3)
    lop = LindbladOperator.from_hamiltonian(s.h_terms, s.c_ops, device="cpu")
    assert lop.n_rows == s.dim ** 2 and lop.n_cops == len(s.c_ops)
    for t in (0.0, 0.37, 2.1):
        want = _superop(s.terms, t)
        got = _kron_generator(lop.a_terms, lop.c_terms, t)
        assert abs(got - want).max() < 1e-13


def test_host_struct_layout():
    from qutip_gb300 import _lib
    from qutip_gb300.lindblad import LindbladOperator
    s = S.ising_chain(3)
    lop = LindbladOperator.from_hamiltonian(s.h_terms, s.c_ops, dtype="c64", device="cpu")
    st = lop.struct
    assert st.d == 8 and st.dtype == _lib.QG_C64
    # H_nh: a diagonal constant group (zz couplings, c^dag c) and the driven sx group
    assert st.n_groups == 2 and sorted(st.a_width[:2]) == [0, 3]
    assert st.a_coef_code and not st.c_coef_code
    # sz dephasing is diagonal, s- is one entry per row
    assert st.n_cops == 6 and st.n_diag_cops == 3 and list(st.c_width[:3]) == [1, 1, 1]
    assert lop.a_col.numel() == 3 * 8 + 8 and lop.c_val.numel() == 3 * 8 + 8


def test_ell_block_layout():
    from qutip_gb300.lindblad import ell_block
    rng = np.random.default_rng(2)
    m = sp.random(13, 13, density=0.3, random_state=rng, format="csr")
    m.data = m.data + 1j
    W, col, val = ell_block(m)
    assert W == np.diff(m.indptr).max()
    back = np.zeros((13, 13), dtype=complex)
    for j in range(W):
        for r in range(13):
            back[r, col[j * 13 + r]] += val[j * 13 + r]
    np.testing.assert_allclose(back, m.toarray())
    assert np.all((col >= 0) & (col < 13))


def test_host_rejects_bad_operators():
    from qutip_gb300.lindblad import LindbladOperator
    h = sp.identity(4, format="csr")
    with pytest.raises(ValueError):
        LindbladOperator([(h, None)], [(sp.identity(3, format="csr"), None)], device="cpu")
    with pytest.raises(ValueError):
        LindbladOperator([(h, None)], [(h, None)] * 65, device="cpu")
    with pytest.raises(TypeError):
        LindbladOperator([(h, lambda t: 1.0)], [], device="cpu")


@pytest.mark.parametrize("hermitian", [True, False])
def test_oracle_matches_the_superoperator(hermitian):
    rng = np.random.default_rng(5)
    s = S.jaynes_cummings(n_cav=4)
    d = s.dim
    m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    rho = m @ m.conj().T if hermitian else m
    h = s.h_terms[0][0]
    h_nh = h - 0.5j * sum(c.conj().T @ c for c in s.c_ops)
    got = lindblad_matrix_form(h_nh, s.c_ops, rho, hermitian=hermitian)
    want = (_superop(s.terms, 0.0) @ rho.reshape(-1, order="F")).reshape(d, d, order="F")
    np.testing.assert_allclose(got, want, atol=1e-12)


def test_oracle_matches_the_reference_matrix_form():
    """The oracle restatement reproduces LindbladMatrixForm.matmul_data of the
    reference itself, both branches."""
    if not reference_available():
        pytest.skip("reference QuTiP not built (oracle/build_ref.py)")
    from oracle.ref_workloads import import_reference
    qt = import_reference()
    from qutip.core.cy.lindblad_matrix_form import LindbladMatrixForm
    N = 5
    a = qt.destroy(N)
    H = qt.QobjEvo([a.dag() * a, [a + a.dag(), "cos(2*t)"]])
    c_ops = [qt.QobjEvo(np.sqrt(0.3) * a), qt.QobjEvo([a.dag() * a, "0.2*exp(-t)"])]
    rng = np.random.default_rng(11)
    m = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    t = 0.6
    h_t = H(t).full()
    cs = [c(t).full() for c in c_ops]
    h_nh = h_t - 0.5j * sum(c.conj().T @ c for c in cs)
    for hermitian, rho in ((True, m @ m.conj().T), (False, m)):
        lmf = LindbladMatrixForm(H, c_ops, assume_hermitian_state=hermitian)
        want = lmf.matmul_data(t, qt.data.Dense(rho)).to_array()
        got = lindblad_matrix_form(h_nh, cs, rho, hermitian=hermitian)
        np.testing.assert_allclose(got, want, atol=1e-12)


def test_oracle_matrix_form_solver_matches_the_superoperator_solver():
    from oracle.solvers import mesolve as me_super, mesolve_matrix_form
    s = S.jaynes_cummings(n_cav=4)
    tl = np.linspace(0, 3, 7)
    want, _ = me_super(s.terms, s.state0, tl, s.e_ops)
    rho0 = s.state0.reshape(s.dim, s.dim, order="F")
    got = mesolve_matrix_form(s.h_terms, [(c, None) for c in s.c_ops], rho0, tl, s.e_ops)
    np.testing.assert_allclose(got, want, atol=1e-7)


def _emulate_kernel(lop, x, t):
    """The element formula of the matrix-free kernel, read from the arrays it reads with
    its indexing (ELL entry j of row r at base + j*d + r)."""
    d = lop.d
    ca = [1.0 if c is None else c(t) for c in lop.a_coeffs]
    wc = [1.0 if c is None else abs(c(t)) ** 2 for c in lop.c_coeffs]
    adiag, acol, aval = lop.a_diag.numpy(), lop.a_col.numpy(), lop.a_val.numpy()
    cdiag, ccol, cval = lop.c_diag.numpy(), lop.c_col.numpy(), lop.c_val.numpy()
    ND = lop.n_diag_cops
    dconst = None if lop.d_const is None else lop.d_const.numpy()
    st = lop.struct
    out = np.zeros(d * d, dtype=complex)
    for idx in range(d * d):
        c, r = divmod(idx, d)
        D = dconst[idx] if dconst is not None else 0.0
        D += sum(k * adiag[g * d + r] + np.conj(k * adiag[g * d + c])
                 for g, k in enumerate(ca) if not (st.a_diag_const >> g) & 1)
        D += sum(wc[i] * cdiag[i * d + r] * np.conj(cdiag[i * d + c])
                 for i in range(st.n_const_diag, ND))
        acc = D * x[idx]
        base = 0
        for g, k in enumerate(ca):
            W = lop.a_width[g]
            for j in range(W):
                e = base + j * d
                acc += k * aval[e + r] * x[acol[e + r] + c * d]
                acc += np.conj(k * aval[e + c]) * x[r + acol[e + c] * d]
            base += W * d
        base = 0
        for i, W in enumerate(lop.c_width):
            for q in range(W):
                for p in range(W):
                    b, v = cval[base + q * d + c], cval[base + p * d + r]
                    kc, kr = ccol[base + q * d + c], ccol[base + p * d + r]
                    acc += wc[ND + i] * v * np.conj(b) * x[kr + kc * d]
            base += W * d
        out[idx] = acc
    return out


def test_layout_reproduces_the_generator():
    """Walking the device arrays as the kernel does gives the superoperator's matvec:
    a random generator with ragged rows, time-dependent groups and collapse operators,
    diagonal and non-diagonal collapse operators and an empty one."""
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.lindblad import LindbladOperator
    rng = np.random.default_rng(7)
    d = 9

    def rand(density):
        m = sp.random(d, d, density=density, random_state=rng, format="csr")
        m.data = rng.normal(size=m.nnz) + 1j * rng.normal(size=m.nnz)
        return m
    h0, h1 = rand(0.3), rand(0.2)
    cops = [(rand(0.2), None), (sp.diags(rng.normal(size=d)).tocsr(), coefficient("0.5+0.1*t")),
            (sp.csr_matrix((d, d), dtype=complex), None), (rand(0.1), coefficient("cos(t)"))]
    lop = LindbladOperator.from_hamiltonian([(h0 + h0.conj().T, None),
                                             (h1 + h1.conj().T, coefficient("sin(2*t)"))],
                                            cops, device="cpu")
    assert lop.n_diag_cops == 2            # the diagonal one and the empty one
    assert lop.n_const_diag == 1 and lop.d_const is not None
    x = rng.normal(size=d * d) + 1j * rng.normal(size=d * d)
    for t in (0.0, 0.9):
        want = _kron_generator(lop.a_terms, lop.c_terms, t) @ x
        np.testing.assert_allclose(_emulate_kernel(lop, x, t), want, atol=1e-12)
