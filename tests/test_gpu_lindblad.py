"""The matrix-free Lindblad generator (mesolve's matrix form) on the GPU through the
C ABI, against the superoperator on the same vec(rho), the CPU oracle, and the
reference's own ``matrix_form=True`` runs.

Tolerances: one application in complex128 within 1e-12 of the row scale; complex64
within 2e-6 of the largest output entry (FP32 accumulation); solves in complex128
within atol 1e-8 / rtol 1e-6 of the oracle and the reference; the mixed form within
1e-6 of the complex128 solve."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle.ref_workloads import reference_available

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda")


def _kron_generator(a_terms, c_terms, t):
    d = a_terms[0][0].shape[0]
    eye = sp.identity(d, format="csr")
    A = sum((1.0 if c is None else c(t)) * m for m, c in a_terms)
    out = sp.kron(eye, A) + sp.kron(A.conj(), eye)
    for m, f in c_terms:
        w = 1.0 if f is None else abs(f(t)) ** 2
        out = out + w * sp.kron(m.conj(), m)
    return sp.csr_matrix(out)


def _random_generator(d, seed):
    """Ragged rows (including empty ones), a time-dependent Hamiltonian group, a
    time-dependent collapse operator and an empty one."""
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.lindblad import LindbladOperator
    rng = np.random.default_rng(seed)

    def rand(density):
        m = sp.random(d, d, density=density, random_state=rng, format="csr")
        m.data = rng.normal(size=m.nnz) + 1j * rng.normal(size=m.nnz)
        return m
    h0 = rand(0.15)
    h0 = h0 + h0.conj().T
    h1 = rand(0.05)
    h1 = h1 + h1.conj().T
    c0, c1 = rand(0.08), rand(0.04)
    mask = np.ones(d)
    mask[:5] = 0.0
    c1 = sp.csr_matrix(sp.diags(mask) @ c1)   # empty first rows
    c1.eliminate_zeros()
    empty = sp.csr_matrix((d, d), dtype=np.complex128)
    cops = [(c0, None), (c1, coefficient("0.7*exp(-t/3) + 0.2j")), (empty, None)]
    h_terms = [(h0, None), (h1, coefficient("cos(1.3*t)"))]
    return h_terms, cops, LindbladOperator


@pytest.mark.parametrize("dtype", ["c128", "c64"])
@pytest.mark.parametrize("case", ["jc", "ising", "random37", "random100"])
def test_apply_matches_the_superoperator(dev, dtype, case):
    from qutip_gb300 import systems as S
    from qutip_gb300.lindblad import LindbladOperator
    if case == "jc":
        s = S.jaynes_cummings(n_cav=6)
        lop = LindbladOperator.from_hamiltonian(s.h_terms, s.c_ops, dtype=dtype)
    elif case == "ising":
        s = S.ising_chain(5)
        lop = LindbladOperator.from_hamiltonian(s.h_terms, s.c_ops, dtype=dtype)
    else:
        h_terms, cops, LO = _random_generator(int(case[6:]), seed=int(case[6:]))
        lop = LO.from_hamiltonian(h_terms, cops, dtype=dtype)
    n = lop.n_rows
    rng = np.random.default_rng(3)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    y0 = rng.normal(size=n) + 1j * rng.normal(size=n)
    tdt = torch.complex128 if dtype == "c128" else torch.complex64
    for t in (0.0, 0.83):
        L = _kron_generator(lop.a_terms, lop.c_terms, t)
        xs = x.astype(np.complex64).astype(np.complex128) if dtype == "c64" else x
        want = 0.5j * (L @ xs) + 2.0 * y0
        y = torch.from_numpy(y0).to(dev, tdt)
        lop.matvec(t, torch.from_numpy(x).to(dev, tdt), y, alpha=0.5j, beta=2.0)
        got = y.cpu().numpy().astype(np.complex128)
        scale = (abs(L) @ abs(xs)).max() + abs(y0).max()
        tol = 1e-12 if dtype == "c128" else 2e-6
        assert np.abs(got - want).max() <= tol * scale, (case, t)


@pytest.mark.parametrize("dtype", ["c128", "c64"])
@pytest.mark.parametrize("case", ["jc", "random37", "random100"])
def test_hermitian_half_matches_the_superoperator(dev, dtype, case):
    """The Hermitian branch (elements r >= c evaluated, mirrored as conjugates): on a
    Hermitian rho it equals the superoperator product within the full form's tolerance,
    its output is exactly Hermitian with a real diagonal, and it agrees with the full form."""
    from qutip_gb300 import systems as S
    from qutip_gb300.lindblad import LindbladOperator
    if case == "jc":
        s = S.jaynes_cummings(n_cav=6)
        lop = LindbladOperator.from_hamiltonian(s.h_terms, s.c_ops, dtype=dtype)
    else:
        h_terms, cops, LO = _random_generator(int(case[6:]), seed=int(case[6:]))
        lop = LO.from_hamiltonian(h_terms, cops, dtype=dtype)
    d = lop.d
    rng = np.random.default_rng(5)
    m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    rho = (m + m.conj().T).astype(np.complex64 if dtype == "c64" else np.complex128)
    x = torch.from_numpy(rho.reshape(-1, order="F").copy()).to(dev)
    xs = rho.astype(np.complex128).reshape(-1, order="F")
    tol = 1e-12 if dtype == "c128" else 2e-6
    for t in (0.0, 0.83):
        L = _kron_generator(lop.a_terms, lop.c_terms, t)
        want = L @ xs
        scale = (abs(L) @ abs(xs)).max()
        lop.hermitian = True
        yh = torch.empty_like(x)
        lop.matvec(t, x, yh)
        lop.hermitian = False
        yf = torch.empty_like(x)
        lop.matvec(t, x, yf)
        gh = yh.cpu().numpy().astype(np.complex128)
        gf = yf.cpu().numpy().astype(np.complex128)
        assert np.abs(gh - want).max() <= tol * scale, (case, t)
        assert np.abs(gh - gf).max() <= tol * scale, (case, t)
        M = gh.reshape(d, d, order="F")
        np.testing.assert_array_equal(M, M.conj().T)
        assert np.all(np.diag(M).imag == 0)


@pytest.mark.parametrize("case", ["jc", "ising"])
def test_matrix_form_solve_matches_the_oracle(dev, case):
    from oracle.solvers import mesolve as oracle_mesolve
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import solve_system
    s = S.jaynes_cummings(n_cav=6) if case == "jc" else S.ising_chain(4)
    tl = np.linspace(0, 4, 21)
    got = solve_system(s, tl, {"matrix_form": True})
    want, _ = oracle_mesolve(s.terms, s.state0, tl, s.e_ops)
    for k in range(len(s.e_ops)):
        err = np.abs(got.expect[k] - want[k])
        assert np.all(err <= 1e-8 + 1e-6 * np.abs(want[k])), (k, err.max())
    assert got.stats["method"].startswith("gpu_vern7")


def test_matrix_form_mixed_precision_error(dev):
    """The mixed form (complex64 generator and stages, FP64 state and control)
    stays within 1e-6 of the complex128 matrix-form solve."""
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import solve_system
    s = S.ising_chain(6)
    tl = np.linspace(0, 5, 26)
    ref = solve_system(s, tl, {"matrix_form": True})
    mix = solve_system(s, tl, {"matrix_form": True, "precision": "mixed"})
    err = max(np.abs(a - b).max() for a, b in zip(ref.expect, mix.expect))
    assert err <= 1e-6, err


def test_matrix_form_agrees_with_the_superoperator_path(dev):
    """Ising L=8 (d^2 = 65,536): the matrix-free generator and the sliced-ELLPACK
    superoperator give the same solve."""
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import solve_system
    s = S.ising_chain(8)
    tl = np.linspace(0, 2, 11)
    a = solve_system(s, tl, {"matrix_form": True})
    b = solve_system(s, tl)
    for x, y in zip(a.expect, b.expect):
        np.testing.assert_allclose(x, y, atol=1e-8, rtol=1e-6)


# ---- through QuTiP: mesolve(..., options={"matrix_form": True}) -------------
@pytest.fixture(scope="module")
def qt(dev):
    if not reference_available():
        pytest.skip("reference QuTiP not built (oracle/build_ref.py)")
    from oracle.ref_workloads import import_reference
    qt = import_reference()
    from qutip_gb300 import qutip_plugin  # noqa: F401  (registers gpu_vern7)
    return qt


N, KAPPA = 10, 0.2
TL = np.linspace(0, 10, 101)


def _both(qt, H, rho0, c_ops, e_ops=None, args=None, tlist=TL, extra=None):
    opts = {"progress_bar": None, "matrix_form": True, "method": "vern7"}
    ref = qt.mesolve(H, rho0, tlist, c_ops, e_ops=e_ops, args=args, options=opts)
    got = qt.mesolve(H, rho0, tlist, c_ops, e_ops=e_ops, args=args,
                     options={**opts, "method": "gpu_vern7", **(extra or {})})
    return ref, got


def test_plugin_constant_decay(qt):
    """Known answer 9 exp(-kappa t) (test_mesolve.py:97-108)."""
    a = qt.destroy(N)
    H = a.dag() * a
    ref, got = _both(qt, H, qt.basis(N, 9), [np.sqrt(KAPPA) * a], e_ops=[H])
    np.testing.assert_allclose(got.expect[0], 9.0 * np.exp(-KAPPA * TL), atol=1e-6)
    np.testing.assert_allclose(got.expect[0], ref.expect[0], atol=1e-8, rtol=1e-6)


def test_plugin_time_dependent_decay(qt):
    """Known answer 9 exp(-kappa (1 - exp(-t))) (test_mesolve.py:125-136)."""
    a = qt.destroy(N)
    H = a.dag() * a
    c_ops = [[a, "sqrt(kappa * exp(-t))"]]
    ref, got = _both(qt, H, qt.basis(N, 9), c_ops, e_ops=[H], args={"kappa": KAPPA})
    want = 9.0 * np.exp(-KAPPA * (1.0 - np.exp(-TL)))
    np.testing.assert_allclose(got.expect[0], want, rtol=1e-5)
    np.testing.assert_allclose(got.expect[0], ref.expect[0], atol=1e-8, rtol=1e-6)


def test_plugin_time_dependent_h_and_decay(qt):
    """test_mesolve.py:166-178: H = [a^dag a, '1'] with the time-dependent decay."""
    a = qt.destroy(N)
    ada = a.dag() * a
    ref, got = _both(qt, [ada, "1"], qt.basis(N, 9), [[a, "sqrt(kappa * exp(-t))"]],
                     e_ops=[ada], args={"kappa": KAPPA})
    want = 9.0 * np.exp(-KAPPA * (1.0 - np.exp(-TL)))
    np.testing.assert_allclose(got.expect[0], want, atol=5e-6)
    np.testing.assert_allclose(got.expect[0], ref.expect[0], atol=1e-8, rtol=1e-6)


def test_plugin_non_hermitian_rho(qt):
    """A transition matrix |0><1| (test_mesolve.py:180-200): states of the matrix
    form against the reference's superoperator and matrix-form runs."""
    a = qt.destroy(N)
    rho0 = qt.basis(N, 0) * qt.basis(N, 1).dag()
    tl = np.linspace(0, 5, 51)
    ref, got = _both(qt, a.dag() * a, rho0, [np.sqrt(KAPPA) * a], tlist=tl)
    sup = qt.mesolve(a.dag() * a, rho0, tl, [np.sqrt(KAPPA) * a],
                     options={"progress_bar": None, "method": "vern7"})
    exact = np.exp(1j * tl - KAPPA * tl / 2)   # <0|rho|1>
    for g, r, s, e in zip(got.states, ref.states, sup.states, exact):
        assert g.shape == (N, N)
        np.testing.assert_allclose(g.full(), r.full(), atol=1e-7)
        np.testing.assert_allclose(g.full(), s.full(), atol=1e-7)
        assert abs(g.full()[0, 1] - e) <= 1e-6


def test_plugin_follows_the_references_hermitian_branch(qt):
    """mesolve's matrix form takes the reference's A + A^dag branch for a Hermitian rho0
    and the full form for a non-Hermitian one (MESolver._prepare_state sets
    assume_hermitian_state from rho0.isherm), when asked to (hermitian_branch=True; "auto"
    takes it only for large rho); both match the reference's own runs."""
    a = qt.destroy(N)
    H, c_ops = a.dag() * a + 0.3 * (a + a.dag()), [np.sqrt(KAPPA) * a]
    opts = {"method": "gpu_vern7", "matrix_form": True, "progress_bar": None,
            "hermitian_branch": True}
    tl = np.linspace(0, 3, 31)
    for rho0, herm in ((qt.coherent_dm(N, 0.8), True),
                       (qt.basis(N, 0) * qt.basis(N, 1).dag(), False)):
        solver = qt.MESolver(H, c_ops, options=opts)
        got = solver.run(rho0, tl)
        assert solver._integrator._op.hermitian is herm
        # "auto" takes it only where it is the faster form: not at d = 10
        auto = qt.MESolver(H, c_ops, options={**opts, "hermitian_branch": "auto"})
        auto.run(rho0, tl[:3])
        assert auto._integrator._op.hermitian is False
        ref = qt.mesolve(H, rho0, tl, c_ops, options={"method": "vern7", "matrix_form": True,
                                                      "progress_bar": None})
        for g, r in zip(got.states, ref.states):
            np.testing.assert_allclose(g.full(), r.full(), atol=1e-7)


def test_plugin_jaynes_cummings_mixed_precision(qt):
    """A driven, dissipative JC model: complex128 against the reference, the mixed form
    within 1e-6 of it."""
    Nc = 8
    a = qt.tensor(qt.destroy(Nc), qt.qeye(2))
    sm = qt.tensor(qt.qeye(Nc), qt.sigmam())
    H = [2 * np.pi * (a.dag() * a + 0.5 * sm.dag() * sm)
         + 2 * np.pi * 0.1 * (a.dag() * sm + a * sm.dag()),
         [a + a.dag(), "0.3*cos(2*pi*t)"]]
    c_ops = [np.sqrt(0.05) * a, np.sqrt(0.02) * sm, np.sqrt(0.01) * sm.dag() * sm]
    rho0 = qt.ket2dm(qt.tensor(qt.basis(Nc, 2), qt.basis(2, 0)))
    e_ops = [a.dag() * a, sm.dag() * sm]
    tl = np.linspace(0, 10, 51)
    ref, got = _both(qt, H, rho0, c_ops, e_ops=e_ops, tlist=tl)
    for g, r in zip(got.expect, ref.expect):
        np.testing.assert_allclose(g, r, atol=1e-8, rtol=1e-6)
    _, mix = _both(qt, H, rho0, c_ops, e_ops=e_ops, tlist=tl, extra={"precision": "mixed"})
    for m, r in zip(mix.expect, ref.expect):
        assert np.abs(np.asarray(m) - np.asarray(r)).max() <= 1e-6
