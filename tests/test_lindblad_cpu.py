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
    assert st.d == 8
    assert st.a.layout == _lib.QG_LAYOUT_ROW_MAJOR and st.a.n_tiles == 0
    assert st.a.n_rows == st.a.n_cols == 8 and st.a.dtype == _lib.QG_C64
    assert st.a.n_groups == 2 and st.a.coef_code  # constant group + cos(w t) group
    assert st.cops.layout == _lib.QG_LAYOUT_GROUP_MAJOR and st.cops.n_groups == 6
    assert not st.cops.coef_code                    # constant collapse operators
    rp = lop.c_row_ptr.numpy()
    assert len(rp) == 6 * 9 and rp[-1] == sum(lop.c_nnz)


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
