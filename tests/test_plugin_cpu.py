"""Host-side checks of the QuTiP plugin: coefficient programs decoded from QuTiP's
own coefficient objects, QobjEvo term extraction, and the registrations
(data type alias, specialisations, integrator, map).  Uses the reference QuTiP
built under oracle/_ref; skipped when it is not built."""
import numpy as np
import pytest

from oracle.ref_workloads import reference_available


@pytest.fixture(scope="module")
def qt():
    if not reference_available():
        pytest.skip("reference QuTiP not built (oracle/build_ref.py)")
    from oracle.ref_workloads import import_reference
    return import_reference()


@pytest.fixture(scope="module")
def plugin(qt):
    from qutip_gb300 import qutip_plugin
    return qutip_plugin


TIMES = np.linspace(0.0, 7.0, 29)


def _close(prog, c):
    got = np.array([prog(t) for t in TIMES])
    want = np.array([complex(c(t)) for t in TIMES])
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("expr,args", [
    ("cos(w*t)", {"w": 1.3}),
    ("a*exp(-t/tau) + 1j*b", {"a": 2.0, "tau": 3.0, "b": 0.5}),
    ("t**2", {}),
    ("sin(w*t)**2 - 0.5*cos(2*t)", {"w": 0.7}),
    ("sqrt(1 + t) * exp(1j*w*t)", {"w": 2.0}),
    ("amp * cos(2 * t)", {"amp": 0.0}),          # a zero factor (no 0 ** b on the host)
])
def test_string_coefficients(qt, plugin, expr, args):
    c = qt.coefficient(expr, args=args)
    _close(plugin.device_coefficient(c), c)


def test_coefficient_algebra(qt, plugin):
    a = qt.coefficient("cos(w*t)", args={"w": 1.3})
    b = qt.coefficient("exp(-g*t)", args={"g": 0.2})
    for c in (a.conj(), a + b, a * b, a * qt.coefficient(2.0 - 1j), qt.coefficient(3.0 + 0.5j),
              (a + b.conj()) * b):
        _close(plugin.device_coefficient(c), c)


def test_norm_coefficient(qt, plugin):
    from qutip.core.coefficient import norm
    c = norm(qt.coefficient("exp(1j*w*t) + 0.3", args={"w": 0.9}))
    _close(plugin.device_coefficient(c), c)


def test_python_function_coefficient_is_rejected(qt, plugin):
    c = qt.coefficient(lambda t: np.cos(t) ** 3)
    with pytest.raises(TypeError):
        plugin.device_coefficient(c)


def test_qobjevo_terms_reproduce_the_operator(qt, plugin):
    H = qt.QobjEvo([qt.sigmaz(), [qt.sigmax(), "cos(w*t)"], [qt.sigmay(), "exp(-t)"]],
                   args={"w": 1.3})
    L = qt.liouvillian(H, [0.3 * qt.destroy(2)])
    terms = plugin.qobjevo_terms(L)
    for t in (0.0, 0.4, 2.5):
        got = sum((c(t) if c is not None else 1.0) * m.toarray() for m, c in terms)
        np.testing.assert_allclose(got, L(t).full(), atol=1e-14)


def test_registrations(qt, plugin):
    from qutip.core import data as D
    from qutip.solver import parallel
    from qutip.solver.mcsolve import MCSolver
    from qutip.solver.mesolve import MESolver
    from qutip.solver.sesolve import SESolver
    assert D.to.parse("gpu") is plugin.GpuDense
    for s in (MESolver, SESolver, MCSolver):
        assert s.avail_integrators()["gpu_vern7"] is plugin.IntegratorGpuVern7
    assert parallel._maps["gpu"] is plugin.gpu_map
    assert (D.CSR, plugin.GpuDense) in D.expect._specialisations or \
        D.expect[D.CSR, plugin.GpuDense] is not None
    opts = plugin.IntegratorGpuVern7.integrator_options
    assert opts["atol"] == 1e-8 and opts["rtol"] == 1e-6 and opts["nsteps"] == 1000


@pytest.mark.parametrize("order", [0, 1, 3])
def test_interpolated_coefficients(qt, plugin, order):
    tl = np.linspace(0.0, 6.0, 25)
    vals = np.exp(-((tl - 3.0) ** 2)) * np.exp(0.4j * tl)
    c = qt.coefficient(vals, tlist=tl, order=order)
    prog = plugin.device_coefficient(c)
    ts = np.concatenate([np.linspace(-1.0, 7.0, 57), tl])
    np.testing.assert_allclose([prog(t) for t in ts], [complex(c(t)) for t in ts],
                               rtol=1e-13, atol=1e-14)
    tn = np.sort(np.random.default_rng(1).uniform(0, 6, 20))
    c2 = qt.coefficient(np.sin(tn) + 0j, tlist=tn, order=order)
    prog2 = plugin.device_coefficient(c2)
    np.testing.assert_allclose([prog2(t) for t in ts], [complex(c2(t)) for t in ts],
                               rtol=1e-13, atol=1e-14)


def _jc_dark(qt, N=4):
    a = qt.tensor(qt.destroy(N), qt.qeye(2))
    sm = qt.tensor(qt.qeye(N), qt.sigmam())
    H = 2 * np.pi * (a.dag() * a + 0.05 * (a * sm.dag() + a.dag() * sm))
    c_ops = [np.sqrt(0.05) * a, np.sqrt(0.1) * sm]
    bright = qt.tensor(qt.basis(N, 1), qt.basis(2, 0))
    dark = qt.tensor(qt.basis(N, 0), qt.basis(2, 1))   # H|dark> = 0, no collapse acts on it
    return H, c_ops, bright, dark, [a.dag() * a]


@pytest.mark.parametrize("mixed", [False, True])
def test_map_task_decoding_under_improved_sampling(qt, plugin, mixed):
    """The trajectory tasks the reference's MCSolver hands its map (plain, mixed
    initial states, improved sampling) decode to the seeds, initial states, weights
    and jump-probability floors that the reference's own trajectories use."""
    from qutip.solver import parallel
    H, c_ops, bright, dark, e_ops = _jc_dark(qt)
    calls = []

    def recording_map(task, values, task_args=None, task_kwargs=None, reduce_func=None,
                      **kw):
        if getattr(task, "__name__", "") != "_no_jump_simulation":
            calls.append(plugin._mc_map_items(task, values, task_args or (), task_kwargs))
        return parallel.serial_map(task, values, task_args, task_kwargs, reduce_func, **kw)

    parallel._maps["recording"] = recording_map
    try:
        state = [(bright, 0.4), (dark, 0.6)] if mixed else bright
        ntraj = [3, 2] if mixed else 4
        opts = {"map": "recording", "improved_sampling": True, "keep_runs_results": True}
        res = qt.MCSolver(H, c_ops, options=opts).run(state, np.linspace(0, 2, 5), ntraj,
                                                      e_ops=e_ops, seeds=3)
    finally:
        del parallel._maps["recording"]
    assert len(calls) == 1
    solver, seeds, starts, floors, tlist, _ = calls[0]
    assert isinstance(solver, qt.MCSolver)
    assert len(seeds) == len(starts) == len(floors) == sum(np.atleast_1d(ntraj))
    assert len(tlist) == 5
    for f in floors:
        assert 0.0 < f <= 1.0
    if mixed:
        # the dark state's no-jump probability is one: the floor the reference passes
        # marks those trajectories as the zero trajectory of weight 0
        # correction weights: the state's weight over its share of the trajectories
        np.testing.assert_allclose([w for _, w in starts], [0.4 * 5 / 3] * 3 + [0.6 * 5 / 2] * 2)
        assert all(f >= 1 - 1e-9 for f in floors[3:])
        assert all(f < 0.99 for f in floors[:3])
    else:
        assert len(set(floors)) == 1 and floors[0] < 0.99
    assert res.num_trajectories == sum(np.atleast_1d(ntraj))


def test_map_rejects_other_tasks(qt, plugin):
    with pytest.raises(TypeError):
        plugin.gpu_map(lambda x: x, [1, 2])


def test_map_task_decoding_rejects_what_it_cannot_batch(qt, plugin):
    """The batched map refuses, with TypeError, the no-jump run as a map task, trajectory
    options it does not know, and tasks that are not an MCSolver's trajectories."""
    H, c_ops, bright, dark, e_ops = _jc_dark(qt)
    solver = qt.MCSolver(H, c_ops, options={"map": "serial"})
    tl = np.linspace(0, 1, 3)
    with pytest.raises(TypeError):
        plugin._mc_map_items(solver._run_one_traj, [1], (bright, tl, e_ops), {"no_jump": True})
    with pytest.raises(TypeError):
        plugin._mc_map_items(solver._run_one_traj, [1], (bright, tl, e_ops), {"unknown": 1})
    with pytest.raises(TypeError):
        plugin._mc_map_items(solver._no_jump_simulation, [bright], (tl, e_ops), None)
    me = qt.MESolver(H, c_ops, options={})
    with pytest.raises(TypeError):
        plugin._mc_map_items(me.run, [bright], (tl,), None)
    seeds, starts, floors = plugin._mc_map_items(
        solver._run_one_traj, [4, 5], (bright, tl, e_ops),
        {"no_jump": False, "jump_prob_floor": 0.25})[1:4]
    assert seeds == [4, 5] and floors == [0.25, 0.25] and [w for _, w in starts] == [1.0, 1.0]


def test_map_refuses_integration_methods_it_does_not_run(qt, plugin):
    """map='gpu' runs Vern7 on the device: an MCSolver set to another method is refused
    with TypeError before anything reaches the device."""
    H, c_ops, bright, dark, e_ops = _jc_dark(qt)
    tl = np.linspace(0, 1, 3)
    for method in ("adams", "dop853", "lsoda"):
        solver = qt.MCSolver(H, c_ops, options={"map": "serial", "method": method})
        with pytest.raises(TypeError, match="map='gpu'"):
            plugin.gpu_map(solver._run_one_traj, [1, 2], (bright, tl, e_ops), {})
