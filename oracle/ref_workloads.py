"""The benchmark workloads run through the reference QuTiP (the CPU baseline arm).

TEST INFRASTRUCTURE ONLY: used by ``bench.py``'s CPU-baseline leg and its
``--impl reference`` arm, never by the product.

``reference_available()`` imports the reference compiled by
``oracle/build_ref.py`` from ``oracle/_ref``; when it is missing (for example on a
host without Python headers) the callers fall back to the numpy restatement in
``oracle.solvers`` and report ``kind = "port"``.
"""
from __future__ import annotations

import os
import sys
import time
import warnings

import numpy as np

_REF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")


def reference_available() -> bool:
    try:
        import_reference()
        return True
    except Exception:  # noqa: BLE001 - any import failure means "not available"
        return False


def import_reference():
    if _REF not in sys.path:
        sys.path.insert(0, _REF)
    warnings.filterwarnings("ignore", message="matplotlib not found")
    import qutip  # noqa: F401
    return qutip


def ising_qobjs(L, seed=1234, J=1.0, omega=1.3):
    """The transverse-field Ising workload with the reference's own constructors."""
    qutip = import_reference()
    h = np.random.default_rng(seed).uniform(0.5, 1.5, L)

    def op(o, i):
        return qutip.tensor(*[o if k == i else qutip.qeye(2) for k in range(L)])
    H0 = sum(-J * op(qutip.sigmaz(), i) * op(qutip.sigmaz(), i + 1) for i in range(L - 1))
    H1 = sum(-h[i] * op(qutip.sigmax(), i) for i in range(L))
    H = qutip.QobjEvo([H0, [H1, "cos(w*t)"]], args={"w": omega})
    c_ops = ([np.sqrt(0.05) * op(qutip.sigmam(), i) for i in range(L)]
             + [np.sqrt(0.02) * op(qutip.sigmaz(), i) for i in range(L)])
    psi0 = qutip.tensor(*[qutip.basis(2, 0) for _ in range(L)])
    e_ops = [op(qutip.sigmaz(), i) for i in range(L)]
    return H, c_ops, qutip.ket2dm(psi0), e_ops


def reference_mesolve_sample(L, t_end, n_out, t_sample):
    """Time the reference's vern7 ``mesolve`` on the first ``t_sample`` of ``[0, t_end]``.

    Returns ``(seconds, fraction_of_the_solve)``.  Setup (operator construction,
    first-call string-coefficient compilation) is excluded by a short untimed
    call first.
    """
    qutip = import_reference()
    H, c_ops, rho0, e_ops = ising_qobjs(L)
    opts = {"method": "vern7", "atol": 1e-8, "rtol": 1e-6, "progress_bar": False}
    full = np.linspace(0.0, t_end, n_out)
    tl = full[full <= t_sample + 1e-12]
    solver = qutip.MESolver(H, c_ops, options=opts)
    solver.run(rho0, tl[:2], e_ops=e_ops)
    t0 = time.perf_counter()
    solver.run(rho0, tl, e_ops=e_ops)
    return time.perf_counter() - t0, (tl[-1] - tl[0]) / (t_end - full[0])


def port_mesolve_sample(terms, state0, e_ops, t_end, n_out, t_sample):
    """Same sample through the numpy restatement (``oracle.solvers.mesolve``)."""
    from .solvers import mesolve
    full = np.linspace(0.0, t_end, n_out)
    tl = full[full <= t_sample + 1e-12]
    t0 = time.perf_counter()
    mesolve(terms, state0, tl, e_ops)
    return time.perf_counter() - t0, (tl[-1] - tl[0]) / (t_end - full[0])


def bh_trimer_qobjs(cutoff=8, J=1.0, U=0.5, F=0.3, kappa=0.1):
    """The Bose-Hubbard trimer (ring) with the reference's own constructors."""
    qutip = import_reference()
    a = [qutip.tensor(*[qutip.destroy(cutoff) if k == i else qutip.qeye(cutoff)
                        for k in range(3)]) for i in range(3)]
    n = [x.dag() * x for x in a]
    H = sum(-J * (a[i].dag() * a[j] + a[j].dag() * a[i]) for i, j in ((0, 1), (1, 2), (2, 0)))
    H = H + sum(U / 2 * n[i] * (n[i] - 1) for i in range(3)) + F * (a[0] + a[0].dag())
    c_ops = [np.sqrt(kappa) * x for x in a]
    psi0 = qutip.tensor(*[qutip.basis(cutoff, 0)] * 3)
    return H, c_ops, psi0, n


def reference_mcsolve_sample(ntraj_serial=16, ntraj_parallel=64, t_end=50.0, n_out=501):
    """Time the reference's vern7 ``mcsolve`` of the Bose-Hubbard trimer: ``map="serial"``
    on one core and ``map="parallel"`` on every host core.  Run it in a fresh process
    (``python -m oracle.ref_workloads mcsolve``): the parallel map forks workers.
    Returns trajectories per second for each and the core count."""
    import os
    qutip = import_reference()
    H, c_ops, psi0, e_ops = bh_trimer_qobjs()
    tl = np.linspace(0.0, t_end, n_out)
    base = {"method": "vern7", "atol": 1e-8, "rtol": 1e-6, "progress_bar": False}
    qutip.mcsolve(H, psi0, tl[:3], c_ops, e_ops=e_ops, ntraj=2, seeds=1,
                  options={**base, "map": "serial"})
    t0 = time.perf_counter()
    qutip.mcsolve(H, psi0, tl, c_ops, e_ops=e_ops, ntraj=ntraj_serial, seeds=2,
                  options={**base, "map": "serial"})
    serial = ntraj_serial / (time.perf_counter() - t0)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    qutip.mcsolve(H, psi0, tl, c_ops, e_ops=e_ops, ntraj=ntraj_parallel, seeds=3,
                  options={**base, "map": "parallel", "num_cpus": cores})
    parallel = ntraj_parallel / (time.perf_counter() - t0)
    return {"serial_traj_per_sec": serial, "serial_sample": ntraj_serial,
            "parallel_traj_per_sec": parallel, "parallel_sample": ntraj_parallel,
            "cores": cores}


if __name__ == "__main__":
    import json
    if sys.argv[1:2] == ["mcsolve"]:
        print(json.dumps(reference_mcsolve_sample()))
