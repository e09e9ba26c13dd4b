"""The QuTiP plugin on the GPU, against the reference QuTiP itself (oracle/_ref) on
the same inputs: ``mesolve`` / ``sesolve`` / ``mcsolve`` with ``method="gpu_vern7"``
unchanged from the user's side, ``map="gpu"`` batched trajectories, and the
GpuDense data-layer operations.

complex128 tolerance: atol 1e-8 / rtol 1e-6 on expectation values and states (the
reference's own solver tolerances).  Jump records: same count and channels, times
inside the reference's bisection window (2 norm_tol target / slope + 2 norm_t_tol,
bounded here by a fixed 1e-3 for these systems)."""
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
    return import_reference()


@pytest.fixture(scope="module")
def plugin(qt):
    from qutip_gb300 import qutip_plugin
    return qutip_plugin


def _jc(qt, N=10):
    a = qt.tensor(qt.destroy(N), qt.qeye(2))
    sm = qt.tensor(qt.qeye(N), qt.sigmam())
    sz = qt.tensor(qt.qeye(N), qt.sigmaz())
    w = 2 * np.pi
    g = 2 * np.pi * 0.05
    H = w * a.dag() * a + w * sz / 2 + g * (a * sm.dag() + a.dag() * sm)
    c_ops = [np.sqrt(0.005) * a, np.sqrt(0.05) * sm]
    psi0 = qt.tensor(qt.basis(N, 0), qt.basis(2, 0))
    return H, c_ops, psi0, [a.dag() * a, sz]


def _ising(qt, L=4, omega=1.3, seed=1234):
    h = np.random.default_rng(seed).uniform(0.5, 1.5, L)
    op = lambda o, i: qt.tensor(*[o if k == i else qt.qeye(2) for k in range(L)])  # noqa: E731
    H0 = sum(-1.0 * op(qt.sigmaz(), i) * op(qt.sigmaz(), i + 1) for i in range(L - 1))
    H1 = sum(-h[i] * op(qt.sigmax(), i) for i in range(L))
    H = qt.QobjEvo([H0, [H1, "cos(w*t)"]], args={"w": omega})
    c_ops = [np.sqrt(0.05) * op(qt.sigmam(), i) for i in range(L)] + \
            [np.sqrt(0.02) * op(qt.sigmaz(), i) for i in range(L)]
    psi0 = qt.tensor(*[qt.basis(2, 0)] * L)
    return H, c_ops, psi0, [op(qt.sigmaz(), i) for i in range(L)]


def _assert_expect(got, want):
    for g, w in zip(got, want):
        np.testing.assert_allclose(np.asarray(g), np.asarray(w), rtol=1e-6, atol=1e-8)


def test_mesolve_jaynes_cummings_drop_in(qt, plugin):
    H, c_ops, psi0, e_ops = _jc(qt)
    rho0 = qt.ket2dm(psi0)
    tl = np.linspace(0, 20, 201)
    ref = qt.mesolve(H, rho0, tl, c_ops, e_ops=e_ops, options={"method": "vern7"})
    got = qt.mesolve(H, rho0, tl, c_ops, e_ops=e_ops,
                     options={"method": "gpu_vern7", "store_final_state": True})
    _assert_expect(got.expect, ref.expect)
    fs = got.final_state
    assert isinstance(fs.data, plugin.GpuDense)
    ref_fs = qt.mesolve(H, rho0, tl, c_ops, options={"method": "vern7",
                                                      "store_final_state": True}).final_state
    np.testing.assert_allclose(fs.full(), ref_fs.full(), rtol=1e-6, atol=1e-8)


def test_mesolve_time_dependent_ising(qt, plugin):
    H, c_ops, psi0, e_ops = _ising(qt, L=4)
    rho0 = qt.ket2dm(psi0)
    tl = np.linspace(0, 10, 101)
    ref = qt.mesolve(H, rho0, tl, c_ops, e_ops=e_ops, options={"method": "vern7"})
    got = qt.mesolve(H, rho0, tl, c_ops, e_ops=e_ops, options={"method": "gpu_vern7"})
    _assert_expect(got.expect, ref.expect)


def test_mesolve_device_built_liouvillian(qt, plugin):
    """L = 5 (1024-row Liouvillian): the integrator merges and lays out QuTiP's Liouvillian
    on the device (dictionary with the real/imaginary split in complex128); results equal
    the reference's, through MESolver.run with a device-resident initial state, a second
    run on the same solver, and the batched expectation values."""
    H, c_ops, psi0, e_ops = _ising(qt, L=5)
    rho0 = qt.ket2dm(psi0)
    tl = np.linspace(0, 4, 41)
    ref = qt.mesolve(H, rho0, tl, c_ops, e_ops=e_ops, options={"method": "vern7"})
    solver = qt.MESolver(H, c_ops, options={"method": "gpu_vern7"})
    op = solver._integrator._op
    assert op.fmt == "dict" and op.dict_split and op.n_rows == 1024
    for state in (rho0, rho0.to("gpu")):
        got = solver.run(state, tl, e_ops=e_ops)
        _assert_expect(got.expect, ref.expect)
    # e_ops asked for in another order, and a single e_op, against the cached batch
    got = solver.run(rho0, tl, e_ops=e_ops[::-1])
    _assert_expect(got.expect, ref.expect[::-1])
    got = solver.run(rho0, tl, e_ops=[e_ops[2]])
    _assert_expect(got.expect, [ref.expect[2]])


def test_expect_batch_never_reuses_a_changed_state(qt, plugin):
    """The batched expectation values of one state are not reused once the state's
    buffer changed in place or a kernel of the library ran."""
    d = 16
    rng = np.random.default_rng(3)
    ops = [qt.rand_herm(d, seed=i).to("csr") for i in range(3)]
    m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    rho = qt.Qobj(m @ m.conj().T).unit().to("gpu")
    want = [qt.expect(o, rho.to("dense")) for o in ops]
    for _ in range(2):
        np.testing.assert_allclose([qt.expect(o, rho) for o in ops], want, rtol=1e-12)
    rho.data.buf.mul_(2.0)                      # in place: torch bumps the version
    np.testing.assert_allclose([qt.expect(o, rho) for o in ops], [2 * w for w in want], rtol=1e-12)
    # a library kernel writing the state through a raw pointer (torch sees no change):
    # rho <- I rho + rho
    plugin.matmul_csr_gpu(qt.qeye(d).to("csr").data, rho.data, scale=1.0, out=rho.data)
    np.testing.assert_allclose([qt.expect(o, rho) for o in ops], [4 * w for w in want], rtol=1e-12)


def test_mesolve_mixed_precision_error_stated(qt, plugin):
    H, c_ops, psi0, e_ops = _ising(qt, L=4)
    rho0 = qt.ket2dm(psi0)
    tl = np.linspace(0, 10, 101)
    ref = qt.mesolve(H, rho0, tl, c_ops, e_ops=e_ops, options={"method": "vern7"})
    got = qt.mesolve(H, rho0, tl, c_ops, e_ops=e_ops,
                     options={"method": "gpu_vern7", "precision": "mixed"})
    err = max(float(np.max(np.abs(np.asarray(g) - np.asarray(w))))
              for g, w in zip(got.expect, ref.expect))
    print(f"\nmixed form vs reference complex128: max |<e_op>| difference {err:.2e}")
    assert err < 1e-6


def test_sesolve_drop_in(qt, plugin):
    H, _, psi0, e_ops = _ising(qt, L=5)
    tl = np.linspace(0, 5, 51)
    ref = qt.sesolve(H, psi0, tl, e_ops=e_ops, options={"method": "vern7"})
    got = qt.sesolve(H, psi0, tl, e_ops=e_ops, options={"method": "gpu_vern7"})
    _assert_expect(got.expect, ref.expect)


def _records(res):
    return [(np.array([t for t, _ in c]), [w for _, w in c]) for c in res.collapse]


def _same_jumps(got, want, tol=1e-3):
    assert len(got) == len(want)
    for (gt, gw), (wt, ww) in zip(got, want):
        assert gw == ww
        assert np.all(np.abs(gt - wt) <= tol)


def test_mcsolve_per_trajectory_integrator(qt, plugin):
    H, c_ops, psi0, e_ops = _jc(qt, N=6)
    tl = np.linspace(0, 20, 101)
    opts = {"method": "vern7", "map": "serial", "keep_runs_results": True}
    ref = qt.mcsolve(H, psi0, tl, c_ops, e_ops=e_ops, ntraj=4, seeds=11, options=opts)
    got = qt.mcsolve(H, psi0, tl, c_ops, e_ops=e_ops, ntraj=4, seeds=11,
                     options={**opts, "method": "gpu_vern7"})
    _same_jumps(_records(got), _records(ref))
    _assert_expect(got.expect, ref.expect)


def test_mcsolve_gpu_map_batched(qt, plugin):
    H, c_ops, psi0, e_ops = _jc(qt, N=6)
    tl = np.linspace(0, 20, 101)
    opts = {"method": "vern7", "map": "serial", "keep_runs_results": True}
    ref = qt.mcsolve(H, psi0, tl, c_ops, e_ops=e_ops, ntraj=32, seeds=5, options=opts)
    got = qt.mcsolve(H, psi0, tl, c_ops, e_ops=e_ops, ntraj=32, seeds=5,
                     options={**opts, "method": "gpu_vern7", "map": "gpu"})
    _same_jumps(_records(got), _records(ref))
    for g, w in zip(got.expect, ref.expect):
        np.testing.assert_allclose(np.asarray(g), np.asarray(w), atol=2e-6)


def test_mcsolve_gpu_map_time_dependent_collapse(qt, plugin):
    """A collapse operator f(t) C with a string coefficient and one with a complex phase
    (mcsolve.py:168-170): the device evaluates |f(t)|^2 ||C psi||^2 for the jump choice
    and f(t) C psi for the jump; jump records and averages match the reference's own
    serial run with the same seeds."""
    H, c_ops, psi0, e_ops = _jc(qt, N=6)
    a = qt.tensor(qt.destroy(6), qt.qeye(2))
    sm = qt.tensor(qt.qeye(6), qt.sigmam())
    c_td = [[np.sqrt(0.1) * a, "exp(-0.05*t)"], [np.sqrt(0.05) * sm, "exp(1j*t)*(1+0.5*sin(t))"]]
    tl = np.linspace(0, 20, 101)
    opts = {"method": "vern7", "map": "serial", "keep_runs_results": True}
    ref = qt.mcsolve(H, psi0, tl, c_td, e_ops=e_ops, ntraj=24, seeds=11, options=opts)
    got = qt.mcsolve(H, psi0, tl, c_td, e_ops=e_ops, ntraj=24, seeds=11,
                     options={**opts, "method": "gpu_vern7", "map": "gpu"})
    _same_jumps(_records(got), _records(ref))
    for g, w in zip(got.expect, ref.expect):
        np.testing.assert_allclose(np.asarray(g), np.asarray(w), atol=2e-6)


def test_gpudense_data_layer(qt, plugin):
    from qutip.core import data as D
    rng = np.random.default_rng(7)
    d = 12
    m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    op = qt.rand_herm(d, density=0.3, seed=3).data
    g = plugin.GpuDense(m)
    np.testing.assert_allclose(g.to_array(), m)
    np.testing.assert_allclose(D.to(D.Dense, g).to_array(), m)
    vec = D.column_stack(g)
    assert vec.shape == (d * d, 1)
    np.testing.assert_allclose(vec.to_array()[:, 0], m.ravel(order="F"))
    back = D.column_unstack(vec, d)
    np.testing.assert_allclose(back.to_array(), m)
    np.testing.assert_allclose(D.matmul(op, g).to_array(), op.to_array() @ m, atol=1e-12)
    np.testing.assert_allclose(D.expect(op, g), np.trace(op.to_array() @ m), rtol=1e-12)
    ket = plugin.GpuDense(m[:, :1])
    want = np.vdot(m[:, 0], op.to_array() @ m[:, 0])
    np.testing.assert_allclose(D.expect(op, ket), want, rtol=1e-12)
    np.testing.assert_allclose(D.trace(g), np.trace(m), rtol=1e-13)
    np.testing.assert_allclose(D.norm.l2(ket), np.linalg.norm(m[:, 0]), rtol=1e-13)
    np.testing.assert_allclose(D.add(g, g, 0.5j).to_array(), m + 0.5j * m)
    np.testing.assert_allclose(D.mul(g, 2 - 1j).to_array(), (2 - 1j) * m)
    np.testing.assert_allclose(g.adjoint().to_array(), m.conj().T)
    np.testing.assert_allclose(g.transpose().to_array(), m.T)
    assert isinstance(D.zeros["gpu"](3, 4), plugin.GpuDense)


def test_mesolve_interpolated_drive(qt, plugin):
    """A pulse given as an array on a time grid (QuTiP's InterCoefficient) drives the
    device solve; same result as the reference."""
    H, c_ops, psi0, e_ops = _jc(qt, N=6)
    a = qt.tensor(qt.destroy(6), qt.qeye(2))
    tp = np.linspace(0, 10, 41)
    pulse = 0.3 * np.exp(-((tp - 4.0) / 1.5) ** 2)
    Ht = [H, [a + a.dag(), qt.coefficient(pulse, tlist=tp, order=3)]]
    rho0 = qt.ket2dm(psi0)
    tl = np.linspace(0, 10, 101)
    ref = qt.mesolve(Ht, rho0, tl, c_ops, e_ops=e_ops, options={"method": "vern7"})
    got = qt.mesolve(Ht, rho0, tl, c_ops, e_ops=e_ops, options={"method": "gpu_vern7"})
    _assert_expect(got.expect, ref.expect)


def test_dia_operators_on_gpudense(qt, plugin):
    """Dia operators (the reference's diagonal format) multiply and take expectation
    values of GpuDense states on the device."""
    from qutip.core import data as D
    a = qt.destroy(12).to("dia")
    H = (a.dag() * a + 0.3 * (a + a.dag())).to("dia")
    assert isinstance(H.data, D.Dia)
    rng = np.random.default_rng(2)
    psi = rng.normal(size=(12, 1)) + 1j * rng.normal(size=(12, 1))
    g = plugin.GpuDense(psi)
    got = D.matmul(H.data, g, 0.5 - 1j)
    np.testing.assert_allclose(got.to_array(), (0.5 - 1j) * (H.full() @ psi), atol=1e-12)
    np.testing.assert_allclose(D.expect(H.data, g), (psi.conj().T @ H.full() @ psi)[0, 0],
                               rtol=1e-12)
    res = qt.sesolve(H, qt.basis(12, 0), np.linspace(0, 3, 31), e_ops=[a.dag() * a],
                     options={"method": "gpu_vern7"})
    ref = qt.sesolve(H, qt.basis(12, 0), np.linspace(0, 3, 31), e_ops=[a.dag() * a],
                     options={"method": "vern7"})
    _assert_expect(res.expect, ref.expect)


def test_mcsolve_gpu_map_mixed_initial_states(qt, plugin):
    """A mixed initial ensemble (MultiTrajSolver._run_mixed): per-trajectory states,
    seeds and correction weights as in the reference."""
    H, c_ops, psi0, e_ops = _jc(qt, N=6)
    psi1 = qt.tensor(qt.basis(6, 1), qt.basis(2, 1))
    ics = [(psi0, 0.3), (psi1, 0.7)]
    tl = np.linspace(0, 10, 51)
    opts = {"method": "vern7", "map": "serial", "keep_runs_results": True}
    ref = qt.MCSolver(H, c_ops, options=opts).run(ics, tl, [8, 12], e_ops=e_ops, seeds=9)
    got = qt.MCSolver(H, c_ops, options={**opts, "method": "gpu_vern7", "map": "gpu"}).run(
        ics, tl, [8, 12], e_ops=e_ops, seeds=9)
    _same_jumps(_records(got), _records(ref))
    for g, w in zip(got.expect, ref.expect):
        np.testing.assert_allclose(np.asarray(g), np.asarray(w), atol=2e-6)


def test_mcsolve_gpu_map_improved_sampling(qt, plugin):
    """Improved sampling (mcsolve.py:716-747): the no-jump run goes through the
    gpu_vern7 integrator, every other trajectory through one batched launch whose
    first jump target sits above the no-jump probability."""
    H, c_ops, psi0, e_ops = _jc(qt, N=6)
    tl = np.linspace(0, 10, 51)
    opts = {"method": "vern7", "map": "serial", "keep_runs_results": True,
            "improved_sampling": True}
    ref = qt.mcsolve(H, psi0, tl, c_ops, e_ops=e_ops, ntraj=16, seeds=21, options=opts)
    got = qt.mcsolve(H, psi0, tl, c_ops, e_ops=e_ops, ntraj=16, seeds=21,
                     options={**opts, "method": "gpu_vern7", "map": "gpu"})
    _same_jumps(_records(got), _records(ref))
    recs = _records(got)
    assert len(recs) == 16 and all(len(w) >= 1 for _, w in recs)  # every sampled run jumps
    for g, w in zip(got.expect, ref.expect):
        np.testing.assert_allclose(np.asarray(g), np.asarray(w), atol=2e-6)


def test_mcsolve_gpu_map_improved_sampling_mixed_dark(qt, plugin):
    """Improved sampling over a mixed ensemble with a dark member (mcsolve.py:749-790,
    544-558): the dark state's trajectories are the zero trajectory of weight 0."""
    H, c_ops, psi0, e_ops = _jc(qt, N=6)
    dark = qt.tensor(qt.basis(6, 0), qt.basis(2, 1))
    ics = [(psi0, 0.45), (dark, 0.55)]
    tl = np.linspace(0, 10, 51)
    opts = {"method": "vern7", "map": "serial", "keep_runs_results": True,
            "improved_sampling": True}
    ref = qt.MCSolver(H, c_ops, options=opts).run(ics, tl, [10, 4], e_ops=e_ops, seeds=4)
    got = qt.MCSolver(H, c_ops, options={**opts, "method": "gpu_vern7", "map": "gpu"}).run(
        ics, tl, [10, 4], e_ops=e_ops, seeds=4)
    _same_jumps(_records(got), _records(ref))
    for g, w in zip(got.expect, ref.expect):
        np.testing.assert_allclose(np.asarray(g), np.asarray(w), atol=2e-6)


def test_propagator_open_and_unitary(qt, plugin):
    """``propagator`` (qutip/solver/propagator.py:183-213) evolves the identity as an
    operator-valued state: the superoperator with collapse operators, and the unitary
    (sesolve) without; the ``Propagator`` class steps it through solver.start/step."""
    N = 4
    a = qt.tensor(qt.destroy(N), qt.qeye(2))
    sm = qt.tensor(qt.qeye(N), qt.sigmam())
    H = [2 * np.pi * a.dag() * a + np.pi * sm.dag() * sm + 0.3 * (a.dag() * sm + a * sm.dag()),
         [a + a.dag(), "0.2*cos(t)"]]
    c_ops = [np.sqrt(0.1) * a, np.sqrt(0.05) * sm]
    ts = [0.0, 0.5, 1.5]
    for cops in (c_ops, None):
        ref = qt.propagator(H, ts, cops, options={"method": "vern7"})
        got = qt.propagator(H, ts, cops, options={"method": "gpu_vern7"})
        assert len(got) == len(ref)
        for g, r in zip(got, ref):
            assert g.dims == r.dims
            np.testing.assert_allclose(g.full(), r.full(), atol=1e-7)
    Hevo = qt.QobjEvo(H)
    P = qt.Propagator(Hevo, c_ops=c_ops, options={"method": "gpu_vern7"})
    Pr = qt.Propagator(Hevo, c_ops=c_ops, options={"method": "vern7"})
    for t in (1.2, 0.4):
        np.testing.assert_allclose(P(t).full(), Pr(t).full(), atol=1e-7)
    # sesolve from an operator initial state: the columns evolve independently
    U = qt.sesolve(H, qt.qeye_like(a), [0, 1.0], options={"method": "gpu_vern7"}).states[-1]
    psi0 = qt.tensor(qt.basis(N, 1), qt.basis(2, 0))
    psi = qt.sesolve(H, psi0, [0, 1.0], options={"method": "gpu_vern7"}).states[-1]
    np.testing.assert_allclose((U * psi0).full(), psi.full(), atol=1e-7)


def test_brmesolve_constant_tensor(qt, plugin):
    """brmesolve (qutip/solver/brmesolve.py:199-333) with ``method="gpu_vern7"``: the
    Bloch-Redfield tensor of constant spectra runs as the device generator."""
    N = 6
    a = qt.destroy(N)
    H = a.dag() * a + 0.25 * (a + a.dag())
    a_ops = [[a + a.dag(), qt.coefficient("0.05 * (w > 0)", args={"w": 0})]]
    c_ops = [np.sqrt(0.01) * a]
    rho0 = qt.ket2dm(qt.basis(N, 3))
    tl = np.linspace(0, 10, 41)
    e_ops = [a.dag() * a, a + a.dag()]
    ref = qt.brmesolve(H, rho0, tl, a_ops=a_ops, c_ops=c_ops, e_ops=e_ops,
                       options={"method": "vern7", "progress_bar": None})
    got = qt.brmesolve(H, rho0, tl, a_ops=a_ops, c_ops=c_ops, e_ops=e_ops,
                       options={"method": "gpu_vern7", "progress_bar": None})
    for g, r in zip(got.expect, ref.expect):
        np.testing.assert_allclose(g, r, atol=1e-8, rtol=1e-6)


def test_mcsolve_gpu_map_target_tol(qt, plugin):
    """``target_tol`` (multitrajresult.py:320-361): the reference's reduce step estimates
    the trajectories still needed and stops the map; the batched launch hands its
    trajectories over in seed order and stops at the same count."""
    N = 6
    a = qt.tensor(qt.destroy(N), qt.qeye(2))
    sm = qt.tensor(qt.qeye(N), qt.sigmam())
    sz = qt.tensor(qt.qeye(N), qt.sigmaz())
    H = 2 * np.pi * (a.dag() * a + sz / 2) + 2 * np.pi * 0.05 * (a * sm.dag() + a.dag() * sm)
    c_ops = [np.sqrt(0.05) * a, np.sqrt(0.2) * sm]
    psi0 = qt.tensor(qt.basis(N, 2), qt.basis(2, 0))
    tl = np.linspace(0, 10, 51)
    opts = {"method": "vern7", "map": "serial", "progress_bar": None}
    kw = dict(e_ops=[a.dag() * a, sz], ntraj=300, seeds=3, target_tol=0.12)
    ref = qt.mcsolve(H, psi0, tl, c_ops, options=opts, **kw)
    got = qt.mcsolve(H, psi0, tl, c_ops, options={**opts, "method": "gpu_vern7", "map": "gpu"},
                     **kw)
    assert got.num_trajectories == ref.num_trajectories < 300
    for g, w in zip(got.expect, ref.expect):
        np.testing.assert_allclose(np.asarray(g), np.asarray(w), atol=2e-6)
    # trajectories are admitted in chunks sized by the reference's own estimate: no more
    # are integrated than a first chunk (256) or the estimate's last chunk needs
    launched = plugin.gpu_map.launched_items
    print(f"\ntarget_tol: {got.num_trajectories} trajectories used, {launched} integrated")
    assert got.num_trajectories <= launched <= max(256, got.num_trajectories + 64)


def test_new_args_reach_the_device_coefficients(qt, plugin):
    """Solver.run(..., args=...) updates the rhs arguments and resets the integrator
    (solver_base.py:457-460); the device coefficients follow the new args."""
    N = 6
    a = qt.destroy(N)
    H = [a.dag() * a, [a + a.dag(), "amp * cos(2 * t)"]]
    c_ops = [np.sqrt(0.1) * a]
    rho0 = qt.ket2dm(qt.basis(N, 0))
    tl = np.linspace(0, 3, 13)
    e_ops = [a.dag() * a]
    ref = qt.MESolver(qt.QobjEvo(H, args={"amp": 0.2}), c_ops, options={"method": "vern7"})
    got = qt.MESolver(qt.QobjEvo(H, args={"amp": 0.2}), c_ops,
                      options={"method": "gpu_vern7"})
    op0 = got._integrator._op
    for amp in (0.2, 0.7, 0.0):
        r = ref.run(rho0, tl, args={"amp": amp}, e_ops=e_ops)
        g = got.run(rho0, tl, args={"amp": amp}, e_ops=e_ops)
        np.testing.assert_allclose(g.expect[0], r.expect[0], atol=1e-8, rtol=1e-6)
        assert got._integrator._op is op0     # new programs, the same operator storage


def test_gpu_map_refuses_other_methods(qt, plugin):
    """map='gpu' integrates with Vern7 on the device; another method is an error, not a
    silent change of integrator."""
    H, c_ops, psi0, e_ops = _jc(qt, N=4)
    for method in ("adams", "dop853"):
        with pytest.raises(TypeError, match="map='gpu'"):
            qt.mcsolve(H, psi0, np.linspace(0, 1, 5), c_ops, e_ops=e_ops, ntraj=2, seeds=1,
                       options={"method": method, "map": "gpu"})


def _bh(qt, cutoff=8, J=1.0, U=0.5, F=0.3, kappa=0.1):
    a = [qt.tensor(*[qt.destroy(cutoff) if k == i else qt.qeye(cutoff) for k in range(3)])
         for i in range(3)]
    n = [x.dag() * x for x in a]
    H = 0
    for i, j in [(0, 1), (1, 2), (2, 0)]:
        H += -J * (a[i].dag() * a[j] + a[j].dag() * a[i])
    for i in range(3):
        H += U / 2 * n[i] * (n[i] - 1)
    H += F * (a[0] + a[0].dag())
    return H, [np.sqrt(kappa) * x for x in a], qt.tensor(*[qt.basis(cutoff, 0)] * 3), n


@pytest.mark.parametrize("prec", ["double", "mixed"])
def test_bh_trimer_4096_trajectories_match_the_reference(qt, plugin, prec):
    """The batched mcsolve workload at full size through qutip.mcsolve with map='gpu':
    4096 trajectories of the Bose-Hubbard trimer (dim 512) over t in [0, 50], seeded as the
    reference's own map='parallel' run in tests/golden/bh_full_mcsolve.npz.

    Jump records (count, channels, each time inside the reference's own bisection
    window, recorded per jump in the fixture): all 4096 identical in complex128; the
    mixed form may let a trajectory cross a window edge, so at most 1 in 200 may differ.
    Averages: in complex128 within 1e-6 of the reference's; in the mixed form within 5
    standard errors of the reference's mean plus the form's 1e-6 bound."""
    import os
    from conftest import GOLDEN, golden
    path = os.path.join(GOLDEN, "bh_full_mcsolve.npz")
    if not os.path.exists(path):
        pytest.skip("full-size mcsolve golden not generated")
    g = golden("bh_full_mcsolve.npz")
    ntraj = int(g["ntraj"])
    H, c_ops, psi0, n = _bh(qt)
    seeds = np.random.SeedSequence(int(g["seed"])).spawn(ntraj)
    res = qt.mcsolve(H, psi0, g["tlist"], c_ops, e_ops=n, ntraj=ntraj, seeds=seeds,
                     options={"method": "gpu_vern7", "map": "gpu", "precision": prec,
                              "progress_bar": False})
    same = 0
    for tr in range(ntraj):
        o0, o1 = int(g["col_off"][tr]), int(g["col_off"][tr + 1])
        wt, ww = g["col_times"][o0:o1], g["col_which"][o0:o1]
        win = g["col_window"][o0:o1]
        gt, gw = np.asarray(res.col_times[tr]), np.asarray(res.col_which[tr])
        if len(gt) == len(wt) and np.all(gw == ww) and np.all(np.abs(gt - wt) <= win):
            same += 1
    sem = g["std_expect"] / np.sqrt(ntraj)
    diff = np.abs(np.array([np.asarray(e) for e in res.expect]).real - g["avg_expect"])
    print(f"\nBH 4096 {prec}: {same}/{ntraj} identical jump records, max |avg diff| "
          f"{diff.max():.2e}, max diff/SEM {np.max(diff / np.maximum(sem, 1e-300)):.2f}")
    if prec == "double":
        assert same == ntraj
        assert diff.max() <= 1e-6
    else:
        assert same >= ntraj - ntraj // 200
        assert np.all(diff <= 5 * sem + 1e-6)
