"""Stochastic Schrodinger / master equations on the GPU (``method="gpu_platen"``) against
the reference's own Platen runs (qutip/solver/sode/_sode.pyx:58-120) with the same seeds.

The device integrator draws the Wiener increments with the reference's ``Wiener`` object
from the trajectory's generator, so each trajectory is the reference's trajectory, to
rounding: the tolerance is 1e-8 on every trajectory's expectation values and measurement
record (complex128, about 1e3 steps of dt = 1e-3), far below the scheme's own error."""
import numpy as np
import pytest

from oracle.ref_workloads import reference_available

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def qt():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not reference_available():
        pytest.skip("reference QuTiP not built (oracle/build_ref.py)")
    from oracle.ref_workloads import import_reference
    q = import_reference()
    from qutip_gb300 import qutip_plugin  # noqa: F401  (registers gpu_platen)
    return q


def _opts(method):
    return {"method": method, "keep_runs_results": True, "store_measurement": "end",
            "progress_bar": None, "dt": 1e-3}


def _same(got, ref, tol=1e-8):
    for g, r in zip(got.runs_expect, ref.runs_expect):
        np.testing.assert_allclose(np.asarray(g), np.asarray(r), atol=tol, rtol=0)
    if ref.measurement is not None:
        np.testing.assert_allclose(np.asarray(got.measurement), np.asarray(ref.measurement),
                                   atol=tol * 1e3, rtol=0)


@pytest.mark.parametrize("heterodyne", [False, True])
def test_ssesolve_matches_the_reference(qt, heterodyne):
    N = 8
    a = qt.destroy(N)
    H = a.dag() * a + 0.4 * (a + a.dag())
    sc_ops = [np.sqrt(0.3) * a]
    psi0 = qt.basis(N, 2)
    e_ops = [a.dag() * a, a + a.dag()]
    tl = np.linspace(0, 1, 11)
    ref = qt.ssesolve(H, psi0, tl, sc_ops, e_ops=e_ops, ntraj=3, seeds=[11, 12, 13],
                      heterodyne=heterodyne, options=_opts("platen"))
    got = qt.ssesolve(H, psi0, tl, sc_ops, e_ops=e_ops, ntraj=3, seeds=[11, 12, 13],
                      heterodyne=heterodyne, options=_opts("gpu_platen"))
    _same(got, ref)


@pytest.mark.parametrize("heterodyne", [False, True])
def test_smesolve_matches_the_reference(qt, heterodyne):
    N = 6
    a = qt.destroy(N)
    H = a.dag() * a + 0.3 * (a + a.dag())
    sc_ops = [np.sqrt(0.2) * a]
    c_ops = [np.sqrt(0.1) * a.dag() * a]
    rho0 = qt.coherent_dm(N, 0.7)
    e_ops = [a.dag() * a, a + a.dag()]
    tl = np.linspace(0, 1, 11)
    ref = qt.smesolve(H, rho0, tl, c_ops=c_ops, sc_ops=sc_ops, e_ops=e_ops, ntraj=3,
                      seeds=[5, 6, 7], heterodyne=heterodyne, options=_opts("platen"))
    got = qt.smesolve(H, rho0, tl, c_ops=c_ops, sc_ops=sc_ops, e_ops=e_ops, ntraj=3,
                      seeds=[5, 6, 7], heterodyne=heterodyne, options=_opts("gpu_platen"))
    _same(got, ref)


@pytest.mark.parametrize("d", [7, 520])
def test_sde_kernel_matches_the_oracle_restatement(qt, d):
    """qg_sde_platen on a batch of trajectories (d = 7: one warp each; d = 520: one CTA
    each), two stochastic operators, an odd number of steps, against the numpy
    restatement of the Platen step."""
    import scipy.sparse as sp
    from oracle.sde import platen_steps
    from qutip_gb300.stochastic import SdeOperator
    rng = np.random.default_rng(3)
    dens = 1.0 if d < 64 else 0.02

    def rand():
        m = sp.random(d, d, density=dens, random_state=rng, format="csr")
        m.data = rng.normal(size=m.nnz) + 1j * rng.normal(size=m.nnz)
        return m
    h = rand()
    H = sp.csr_matrix(h + h.conj().T)
    cs = [0.3 * rand() for _ in range(2)]
    op = SdeOperator.sse(H, cs)
    n_traj, n_steps, dt = 5, 37, 1e-3
    psi = rng.normal(size=(n_traj, d)) + 1j * rng.normal(size=(n_traj, d))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    dW = rng.normal(0, np.sqrt(dt), size=(n_traj, n_steps, 2))
    states = torch.from_numpy(psi.copy()).cuda()
    op.advance(states, torch.from_numpy(dW).cuda(), n_steps, dt)
    got = states.cpu().numpy()
    L = -1j * H - 0.5 * sum(c.conj().T @ c for c in cs)
    for k in range(n_traj):
        want = platen_steps(L, cs, [c + c.conj().T for c in cs], psi[k], dW[k], dt, open_=False)
        np.testing.assert_allclose(got[k], want, atol=1e-12, rtol=0)


@pytest.mark.parametrize("solver", ["sse", "sme"])
def test_gpu_map_runs_every_trajectory_in_one_batch(qt, solver):
    """map="gpu": all trajectories of a run in one launch per output interval, noise from
    the reference's Wiener on each trajectory's generator; every trajectory equals the
    reference's serial run with the same seeds (expectation values and measurements)."""
    N = 6
    a = qt.destroy(N)
    H = a.dag() * a + 0.3 * (a + a.dag())
    e_ops = [a.dag() * a, a + a.dag()]
    tl = np.linspace(0, 0.5, 6)
    seeds = [21, 22, 23, 24, 25]
    if solver == "sse":
        def run(opts):
            return qt.ssesolve(H, qt.basis(N, 1), tl, [np.sqrt(0.3) * a], e_ops=e_ops,
                               ntraj=len(seeds), seeds=seeds, options=opts)
    else:
        def run(opts):
            return qt.smesolve(H, qt.coherent_dm(N, 0.6), tl, c_ops=[np.sqrt(0.1) * a],
                               sc_ops=[np.sqrt(0.2) * a], e_ops=e_ops, ntraj=len(seeds),
                               seeds=seeds, options=opts)
    ref = run(_opts("platen"))
    got = run({**_opts("platen"), "map": "gpu"})
    _same(got, ref)
    assert len(got.runs_expect[0]) == len(seeds)


@pytest.mark.parametrize("solver", ["sse", "sme"])
def test_euler_matches_the_reference(qt, solver):
    """method="gpu_euler" (one trajectory at a time) and map="gpu" with method="euler"
    against the reference's Euler-Maruyama runs with the same seeds."""
    N = 6
    a = qt.destroy(N)
    H = a.dag() * a + 0.3 * (a + a.dag())
    e_ops = [a.dag() * a, a + a.dag()]
    tl = np.linspace(0, 0.5, 6)
    seeds = [31, 32, 33]
    if solver == "sse":
        def run(opts):
            return qt.ssesolve(H, qt.basis(N, 1), tl, [np.sqrt(0.3) * a], e_ops=e_ops,
                               ntraj=len(seeds), seeds=seeds, options=opts)
    else:
        def run(opts):
            return qt.smesolve(H, qt.coherent_dm(N, 0.6), tl, c_ops=[np.sqrt(0.1) * a],
                               sc_ops=[np.sqrt(0.2) * a], e_ops=e_ops, ntraj=len(seeds),
                               seeds=seeds, options=opts)
    ref = run(_opts("euler"))
    _same(run(_opts("gpu_euler")), ref)
    _same(run({**_opts("euler"), "map": "gpu"}), ref)
