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
