"""The numpy restatement of the Platen and Euler SODE steps (oracle/sde.py) pinned to the reference's
own stochastic solvers: ``run_from_experiment`` with a preset noise record integrates one
step per output interval, which the restatement reproduces to rounding."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle.ref_workloads import import_reference, reference_available
from oracle.sde import euler_steps, platen_steps


@pytest.fixture(scope="module")
def qt():
    if not reference_available():
        pytest.skip("reference QuTiP not built (oracle/build_ref.py)")
    return import_reference()


def _csr(q):
    return sp.csr_matrix(q.full())


def test_sse_platen_restatement_matches_the_reference(qt):
    N = 6
    a = qt.destroy(N)
    H = a.dag() * a + 0.4 * (a + a.dag())
    sc = [np.sqrt(0.3) * a, np.sqrt(0.1) * a.dag() * a]
    psi0 = qt.basis(N, 1)
    dt = 1e-3
    tl = np.arange(21) * dt
    noise = np.random.default_rng(4).normal(0, np.sqrt(dt), size=(len(sc), len(tl) - 1))
    solver = qt.SSESolver(H, sc, heterodyne=False,
                          options={"method": "platen", "dt": dt, "store_states": True,
                                   "progress_bar": None})
    res = solver.run_from_experiment(psi0, tl, noise)
    C = [_csr(c) for c in sc]
    L = -1j * _csr(H) - 0.5 * sum(c.conj().T @ c for c in C)
    M = [c + c.conj().T for c in C]
    x = psi0.full()[:, 0]
    for k in range(1, len(tl)):
        x = platen_steps(L, C, M, x, noise[:, k - 1][None, :], dt, open_=False)
        np.testing.assert_allclose(x, res.states[k].full()[:, 0], atol=1e-13, rtol=0)


def test_sme_platen_restatement_matches_the_reference(qt):
    N = 5
    a = qt.destroy(N)
    H = a.dag() * a + 0.3 * (a + a.dag())
    sc = [np.sqrt(0.2) * a]
    cops = [np.sqrt(0.1) * a.dag() * a]
    rho0 = qt.coherent_dm(N, 0.7)
    dt = 1e-3
    tl = np.arange(16) * dt
    noise = np.random.default_rng(8).normal(0, np.sqrt(dt), size=(1, len(tl) - 1))
    solver = qt.SMESolver(H, sc, heterodyne=False, c_ops=cops,
                          options={"method": "platen", "dt": dt, "store_states": True,
                                   "progress_bar": None})
    res = solver.run_from_experiment(rho0, tl, noise)
    L = _csr(qt.liouvillian(H, sc) + qt.liouvillian(None, cops))
    C = [_csr(qt.spre(c) + qt.spost(c.dag())) for c in sc]
    x = rho0.full().reshape(-1, order="F")
    for k in range(1, len(tl)):
        x = platen_steps(L, C, None, x, noise[:, k - 1][None, :], dt, open_=True)
        np.testing.assert_allclose(x, res.states[k].full().reshape(-1, order="F"),
                                   atol=1e-13, rtol=0)


def test_sse_euler_restatement_matches_the_reference(qt):
    N = 6
    a = qt.destroy(N)
    H = a.dag() * a + 0.4 * (a + a.dag())
    sc = [np.sqrt(0.3) * a]
    psi0 = qt.basis(N, 1)
    dt = 1e-3
    tl = np.arange(21) * dt
    noise = np.random.default_rng(5).normal(0, np.sqrt(dt), size=(1, len(tl) - 1))
    solver = qt.SSESolver(H, sc, heterodyne=False,
                          options={"method": "euler", "dt": dt, "store_states": True,
                                   "progress_bar": None})
    res = solver.run_from_experiment(psi0, tl, noise)
    C = [_csr(c) for c in sc]
    L = -1j * _csr(H) - 0.5 * sum(c.conj().T @ c for c in C)
    M = [c + c.conj().T for c in C]
    x = psi0.full()[:, 0]
    for k in range(1, len(tl)):
        x = euler_steps(L, C, M, x, noise[:, k - 1][None, :], dt, open_=False)
        np.testing.assert_allclose(x, res.states[k].full()[:, 0], atol=1e-13, rtol=0)


def test_sme_euler_restatement_matches_the_reference(qt):
    N = 5
    a = qt.destroy(N)
    H = a.dag() * a + 0.3 * (a + a.dag())
    sc = [np.sqrt(0.2) * a, np.sqrt(0.05) * a.dag() * a]
    cops = [np.sqrt(0.1) * a]
    rho0 = qt.coherent_dm(N, 0.5)
    dt = 1e-3
    tl = np.arange(16) * dt
    noise = np.random.default_rng(9).normal(0, np.sqrt(dt), size=(len(sc), len(tl) - 1))
    solver = qt.SMESolver(H, sc, heterodyne=False, c_ops=cops,
                          options={"method": "euler", "dt": dt, "store_states": True,
                                   "progress_bar": None})
    res = solver.run_from_experiment(rho0, tl, noise)
    L = _csr(qt.liouvillian(H, sc) + qt.liouvillian(None, cops))
    C = [_csr(qt.spre(c) + qt.spost(c.dag())) for c in sc]
    x = rho0.full().reshape(-1, order="F")
    for k in range(1, len(tl)):
        x = euler_steps(L, C, None, x, noise[:, k - 1][None, :], dt, open_=True)
        np.testing.assert_allclose(x, res.states[k].full().reshape(-1, order="F"),
                                   atol=1e-13, rtol=0)


@pytest.mark.parametrize("tlist,dt", [
    (np.linspace(0, 1, 11), 1e-3),
    (np.array([0.0, 0.0004, 0.0011, 0.5, 0.50049, 2.0]), 1e-3),
    (np.linspace(0, 0.3, 4), 0.07),
])
def test_interval_steps_follow_the_reference_integrator(qt, tlist, dt):
    """The map's host count of steps per output interval equals what the reference's
    explicit integrator takes (its time after each interval, sode.py:151-173)."""
    from qutip_gb300.stochastic import interval_steps
    N = 3
    a = qt.destroy(N)
    solver = qt.SSESolver(a.dag() * a, [0.1 * a], heterodyne=False,
                          options={"method": "euler", "dt": dt, "progress_bar": None})
    ig = solver._integrator
    ig.set_state(float(tlist[0]), qt.basis(N, 0).data, np.random.default_rng(0))
    times = []
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        for t in tlist[1:]:
            times.append(ig.integrate(float(t))[0])
    steps = interval_steps(tlist, dt)
    t_cur = float(tlist[0])
    for n, t_ref in zip(steps, times):
        t_cur += dt * n
        assert t_cur == t_ref
