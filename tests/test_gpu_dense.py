"""The dense small-dimension bucket (tcgen05 tensor-core Lindblad generator) against
complex128 references.

Tolerances: the generator is applied with TF32 inputs split hi + lo and FP32
accumulation, so one application agrees with the complex128 product to FP32 level
(2e-5 of the largest entry, for sums of up to 2 x 128 products per entry); solves in
the mixed form (complex64 stages, FP64 state and step control) keep the mixed form's
bound, 2e-6 on the Jaynes-Cummings expectation values of the reference's own solve."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _rand(d, rng, herm=False):
    m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    return (m + m.conj().T) / 2 if herm else m


def _generator(a_list, a_coef, c_list, c_coef, X):
    """L[X] with A = sum_g a_g A_g, C_i scaled by f_i (complex128)."""
    A = sum(a * m for a, m in zip(a_coef, a_list))
    out = A @ X + X @ A.conj().T
    for f, c in zip(c_coef, c_list):
        out = out + abs(f) ** 2 * (c @ X @ c.conj().T)
    return out


@pytest.mark.parametrize("d", [5, 16, 40, 100, 128])
def test_dense_apply_matches_complex128(d):
    """Two A groups (one with a complex time-dependent coefficient), two collapse
    operators (one time-dependent), a non-Hermitian argument, alpha / beta epilogue."""
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.dense import DenseLindbladOperator
    rng = np.random.default_rng(d)
    a0, a1 = -1j * _rand(d, rng, herm=True), 0.3 * _rand(d, rng)
    c0, c1 = 0.2 * _rand(d, rng), 0.1 * _rand(d, rng)
    ca = coefficient("exp(1j*w*t)", args={"w": 0.7})
    cc = coefficient("cos(t) + 0.5")
    op = DenseLindbladOperator([(a0, None), (a1, ca)], [(c0, None), (c1, cc)])
    X = _rand(d, rng)
    t = 0.37
    want = _generator([a0, a1], [1.0, ca(t)], [c0, c1], [1.0, cc(t)], X)
    x = torch.from_numpy(X.reshape(-1, order="F").astype(np.complex64)).cuda()
    y0 = _rand(d, rng).reshape(-1, order="F").astype(np.complex64)
    y = torch.from_numpy(y0.copy()).cuda()
    alpha, beta = 0.75 - 0.25j, 0.5
    op.matvec(t, x, y, alpha=alpha, beta=beta)
    got = y.cpu().numpy().reshape(d, d, order="F")
    ref = alpha * want + beta * y0.reshape(d, d, order="F")
    err = np.abs(got - ref).max() / np.abs(ref).max()
    print(f"\ndense bucket d={d}: max |L[X] - complex128| / max |L[X]| = {err:.2e}")
    assert err <= 2e-5
    from qutip_gb300 import _lib
    assert _lib.load().qg_device_fault() == 0


def test_dense_bucket_mixed_solve_matches_the_reference():
    """The Jaynes-Cummings mesolve (N = 10, d = 20) through the dense bucket in the mixed
    form against the reference's own complex128 solve (golden)."""
    from qutip_gb300 import systems as S
    from qutip_gb300.dense import DenseLindbladOperator
    from qutip_gb300.solver import solve_system
    g = golden("jc_mesolve.npz")
    s = S.jaynes_cummings()
    op = DenseLindbladOperator.from_hamiltonian(s.h_terms, s.c_ops)
    res = solve_system(s, g["tlist"], {"precision": "mixed"}, op=op)
    err = max(np.abs(res.expect[k].real - g["expect"][k]).max() for k in range(2))
    print(f"\ndense bucket JC mixed: max |<e_op> - reference| = {err:.2e}, "
          f"{res.stats['steps']} steps")
    assert err <= 2e-6


def test_dense_bucket_random_system_against_sparse_complex128():
    """A dense random system (d = 48, Hermitian H with a cos(t) drive, two dense collapse
    operators, |H| ~ 10): the dense bucket's mixed solve against the matrix-free complex128
    solve.  Its error is the mixed form's, set by complex64 stages on this stiffer system:
    at most twice that of the sparse matrix-free kernel's own mixed solve (FP32 SIMT
    arithmetic), and below 5e-5."""
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.dense import DenseLindbladOperator
    from qutip_gb300.lindblad import LindbladOperator
    from qutip_gb300.solver import ExpectOps, solve_system
    from qutip_gb300.systems import OpenSystem
    d = 48
    rng = np.random.default_rng(7)
    h0, h1 = _rand(d, rng, herm=True), 0.3 * _rand(d, rng, herm=True)
    c_ops = [0.15 * _rand(d, rng), 0.05 * _rand(d, rng)]
    h_terms = [(sp.csr_matrix(h0), None), (sp.csr_matrix(h1), coefficient("cos(1.1*t)"))]
    psi = rng.normal(size=d) + 1j * rng.normal(size=d)
    psi /= np.linalg.norm(psi)
    rho0 = np.outer(psi, psi.conj()).reshape(-1, order="F")
    e_ops = [sp.csr_matrix(_rand(d, rng, herm=True)) for _ in range(3)]
    s = OpenSystem("dense_random", "me", d, None, rho0, e_ops, [sp.csr_matrix(c) for c in c_ops],
                   h_terms)
    tl = np.linspace(0, 2.0, 21)
    ex = ExpectOps(e_ops)
    ref = solve_system(s, tl, {"precision": "double"},
                       op=LindbladOperator.from_hamiltonian(h_terms, s.c_ops, dtype="c128"), ex=ex)
    got = solve_system(s, tl, {"precision": "mixed"},
                       op=DenseLindbladOperator.from_hamiltonian(h_terms, s.c_ops), ex=ex)
    simt = solve_system(s, tl, {"precision": "mixed"},
                        op=LindbladOperator.from_hamiltonian(h_terms, s.c_ops, dtype="c64"), ex=ex)

    def rel(res):
        return max(float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
                   for a, b in zip(res.expect, ref.expect))
    r_tc, r_simt = rel(got), rel(simt)
    print(f"\ndense bucket d={d} random system: relative error vs complex128 {r_tc:.2e} "
          f"(sparse kernel, mixed: {r_simt:.2e}), {got.stats['steps']} / {ref.stats['steps']} steps")
    assert r_tc <= max(2 * r_simt, 1e-6) and r_tc <= 5e-5


def test_plugin_routes_dense_matrix_form_to_the_tensor_cores():
    """mesolve(..., options={"matrix_form": True, "precision": "mixed"}) of a small system
    with dense operators runs on the dense bucket (chosen by fill, or forced with
    dense=True); the reference's own matrix-form solve is the check.  A sparse system
    (Jaynes-Cummings) stays on the sparse kernel unless forced."""
    from oracle.ref_workloads import import_reference, reference_available
    if not reference_available():
        pytest.skip("reference QuTiP not built")
    qt = import_reference()
    from qutip_gb300 import qutip_plugin
    from qutip_gb300.dense import DenseLindbladOperator
    d = 24
    H = qt.rand_herm(d, density=1.0, seed=3)
    c_ops = [0.2 * qt.rand_unitary(d, seed=4), 0.1 * qt.destroy(d)]
    rho0 = qt.rand_dm(d, seed=5)
    e_ops = [qt.rand_herm(d, density=1.0, seed=6), qt.num(d)]
    tl = np.linspace(0, 2, 21)
    ref = qt.mesolve(H, rho0, tl, c_ops, e_ops=e_ops,
                     options={"method": "vern7", "matrix_form": True})
    opts = {"method": "gpu_vern7", "matrix_form": True, "precision": "mixed"}
    solver = qt.MESolver(H, c_ops, options=opts)
    assert isinstance(solver._integrator._op, DenseLindbladOperator)
    got = solver.run(rho0, tl, e_ops=e_ops)
    for g, w in zip(got.expect, ref.expect):
        np.testing.assert_allclose(np.asarray(g), np.asarray(w), atol=2e-6)
    a = qt.tensor(qt.destroy(6), qt.qeye(2))
    H_jc = a.dag() * a + 0.1 * (a + a.dag())
    sparse = qt.MESolver(H_jc, [0.1 * a], options=opts)
    assert not isinstance(sparse._integrator._op, DenseLindbladOperator)
    forced = qt.MESolver(H_jc, [0.1 * a], options={**opts, "dense": True})
    assert isinstance(forced._integrator._op, DenseLindbladOperator)
    assert qutip_plugin.IntegratorGpuVern7.integrator_options["dense"] == "auto"
