"""Generate the golden fixtures in this directory from the reference QuTiP itself.

Run in a checkout that has the compiled reference (``python oracle/build_ref.py all``)::

    python tests/golden/make_golden.py            # small fixtures (about a minute)
    python tests/golden/make_golden.py --large    # + Ising L=10 complex128 mesolve (minutes)
    python tests/golden/make_golden.py --only bh4096   # 4096-trajectory BH mcsolve (minutes)

Every number stored here comes from the reference's own public API
(``qutip.mesolve``, ``qutip.MCSolver``, ``qutip.core.data``) on seeded inputs;
operators are stored as CSR arrays so that the GPU tests can rebuild them without
QuTiP.  The fixtures pin the CPU oracle (``oracle/``) and are the parity targets
of the GPU tests.
"""
from __future__ import annotations

import argparse
import os
import sys
import time
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, ROOT)
warnings.filterwarnings("ignore")

import qutip  # noqa: E402
from qutip import data as _data  # noqa: E402
from qutip.core.data.ode import wrmn_error  # noqa: E402

ME_OPTS = {"method": "vern7", "atol": 1e-8, "rtol": 1e-6, "progress_bar": False}


def _csr_arrays(prefix, q):
    m = _data.to(_data.CSR, q.data).as_scipy() if isinstance(q, qutip.Qobj) else q
    m = m.tocsr()
    m.sort_indices()
    return {f"{prefix}_data": m.data.astype(np.complex128), f"{prefix}_indices": m.indices.astype(np.int32),
            f"{prefix}_indptr": m.indptr.astype(np.int32), f"{prefix}_shape": np.array(m.shape)}


def tableau():
    from qutip.solver.integrator.verner7efficient import vern7_coeff as V
    np.savez(os.path.join(HERE, "vern7_tableau.npz"), a=V["a"], b=V["b"], c=V["c"], e=V["e"],
             bi=V["bi"], order=V["order"])


def kernels():
    rng = np.random.default_rng(7)
    out = {}
    for i, (n, dens) in enumerate([(37, 0.2), (200, 0.05), (513, 0.01)]):
        m = (rng.random((n, n)) < dens) * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
        if i > 0:  # banded, so that the Dia form stays small
            m = np.triu(np.tril(m, 4), -7)
        csr = _data.to(_data.CSR, _data.Dense(m))
        x = rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1))
        out_pre = rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1))
        res = _data.matmul(csr, _data.Dense(x), scale=0.5j, out=_data.Dense(out_pre.copy()))
        sc = csr.as_scipy()
        out.update({f"spmv{i}_data": sc.data, f"spmv{i}_indices": sc.indices.astype(np.int32),
                    f"spmv{i}_indptr": sc.indptr.astype(np.int32), f"spmv{i}_x": x.ravel(),
                    f"spmv{i}_out0": out_pre.ravel(), f"spmv{i}_res": res.to_array().ravel()})
        dia = _data.to(_data.Dia, csr)
        resd = _data.matmul(dia, _data.Dense(x))
        dsc = dia.as_scipy()
        out.update({f"dia{i}_data": dsc.data, f"dia{i}_offsets": dsc.offsets.astype(np.int32),
                    f"dia{i}_res": resd.to_array().ravel()})
        # expect: operator on a density matrix (F order) and on a ket
        if i < 2:
            rho = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
            out[f"exp{i}_rho"] = rho.reshape(-1, order="F")
            out[f"exp{i}_dm"] = np.array(_data.expect(csr, _data.Dense(np.asfortranarray(rho))))
        out[f"exp{i}_ket"] = np.array(_data.expect(csr, _data.Dense(x)))
        y = rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1))
        out[f"wrmn{i}_y"] = y.ravel()
        out[f"wrmn{i}"] = np.array(wrmn_error(_data.Dense(x * 1e-7), _data.Dense(y), 1e-8, 1e-6))
    # expect_super on a small Liouvillian-shaped operator
    d = 6
    m = (rng.random((d * d, d * d)) < 0.3) * (rng.normal(size=(d * d, d * d)) + 0j)
    sup = _data.to(_data.CSR, _data.Dense(m))
    vec = rng.normal(size=(d * d, 1)) + 1j * rng.normal(size=(d * d, 1))
    out["super_data"] = sup.as_scipy().data
    out["super_indices"] = sup.as_scipy().indices.astype(np.int32)
    out["super_indptr"] = sup.as_scipy().indptr.astype(np.int32)
    out["super_vec"] = vec.ravel()
    out["super_res"] = np.array(_data.expect_super(sup, _data.Dense(vec)))
    np.savez(os.path.join(HERE, "kernels.npz"), **out)


def _jc_qobjs(N, wc, wa, g, kappa, gamma):
    a = qutip.tensor(qutip.destroy(N), qutip.qeye(2))
    sm = qutip.tensor(qutip.qeye(N), qutip.sigmam())
    sz = qutip.tensor(qutip.qeye(N), qutip.sigmaz())
    H = wc * a.dag() * a + wa * sz / 2 + g * (a * sm.dag() + a.dag() * sm)
    c_ops = [np.sqrt(kappa) * a, np.sqrt(gamma) * sm]
    psi0 = qutip.tensor(qutip.basis(N, 0), qutip.basis(2, 0))
    return H, c_ops, psi0, [a.dag() * a, sz]


def jc_mesolve():
    H, c_ops, psi0, e_ops = _jc_qobjs(10, 2 * np.pi, 2 * np.pi, 2 * np.pi * 0.05, 0.005, 0.05)
    rho0 = qutip.ket2dm(psi0)
    tlist = np.linspace(0, 20, 201)
    t0 = time.time()
    res = qutip.mesolve(H, rho0, tlist, c_ops, e_ops=e_ops,
                        options={**ME_OPTS, "store_final_state": True})
    wall = time.time() - t0
    solver = qutip.MESolver(qutip.QobjEvo(H), [qutip.QobjEvo(c) for c in c_ops], options=ME_OPTS)
    L = solver.rhs(0)
    ig = solver._integrator
    ig.set_state(0.0, qutip.stack_columns(rho0.data))
    ends = []
    ode = ig._ode_solver
    while ode.t_front < 20.0 and len(ends) < 10000:
        ode.integrate(20.0, step=True)
        ends.append(ode.t_front)
    np.savez(os.path.join(HERE, "jc_mesolve.npz"), tlist=tlist,
             expect=np.array([np.asarray(e) for e in res.expect]),
             final=res.final_state.full().reshape(-1, order="F"), step_ends=np.array(ends),
             rho0=rho0.full().reshape(-1, order="F"), wall=wall,
             **_csr_arrays("L", L), **_csr_arrays("e0", e_ops[0]), **_csr_arrays("e1", e_ops[1]))


def _ising_qobjs(L, seed=1234):
    h = np.random.default_rng(seed).uniform(0.5, 1.5, L)

    def op(o, i):
        return qutip.tensor(*[o if k == i else qutip.qeye(2) for k in range(L)])
    H0 = sum(-1.0 * op(qutip.sigmaz(), i) * op(qutip.sigmaz(), i + 1) for i in range(L - 1))
    H1 = sum(-h[i] * op(qutip.sigmax(), i) for i in range(L))
    H = qutip.QobjEvo([H0, [H1, "cos(w*t)"]], args={"w": 1.3})
    c_ops = ([np.sqrt(0.05) * op(qutip.sigmam(), i) for i in range(L)]
             + [np.sqrt(0.02) * op(qutip.sigmaz(), i) for i in range(L)])
    psi0 = qutip.tensor(*[qutip.basis(2, 0) for _ in range(L)])
    e_ops = [op(qutip.sigmaz(), i) for i in range(L)]
    return H, c_ops, psi0, e_ops, h


def ising(L, tmax=10.0, npts=101, name=None):
    H, c_ops, psi0, e_ops, h = _ising_qobjs(L)
    tlist = np.linspace(0, tmax, npts)
    t0 = time.time()
    res = qutip.mesolve(H, qutip.ket2dm(psi0), tlist, c_ops, e_ops=e_ops,
                        options={**ME_OPTS, "store_final_state": L <= 6})
    wall = time.time() - t0
    extra = {}
    if L <= 6:
        extra["final"] = res.final_state.full().reshape(-1, order="F")
    if L <= 3:
        solver = qutip.MESolver(H, [qutip.QobjEvo(c) for c in c_ops], options=ME_OPTS)
        for tt in (0.0, 0.37, 2.1):
            extra[f"L_at_{tt}"] = solver.rhs(tt).full()
    np.savez(os.path.join(HERE, name or f"ising_L{L}_mesolve.npz"), tlist=tlist, h=h,
             expect=np.array([np.asarray(e) for e in res.expect]), wall=wall, **extra)
    return wall


def _bh_qobjs(cutoff, J=1.0, U=0.5, F=0.3, kappa=0.1):
    a = [qutip.tensor(*[qutip.destroy(cutoff) if k == i else qutip.qeye(cutoff) for k in range(3)])
         for i in range(3)]
    n = [x.dag() * x for x in a]
    H = 0
    for i, j in [(0, 1), (1, 2), (2, 0)]:
        H += -J * (a[i].dag() * a[j] + a[j].dag() * a[i])
    for i in range(3):
        H += U / 2 * n[i] * (n[i] - 1)
    H += F * (a[0] + a[0].dag())
    c_ops = [np.sqrt(kappa) * x for x in a]
    psi0 = qutip.tensor(*[qutip.basis(cutoff, 0) for _ in range(3)])
    return H, c_ops, psi0, n


def _hook_collapse_windows():
    """Record, per recorded jump, the time window the reference's own bisection
    tolerance allows: |norm^2(t) - target| < norm_tol * target around the jump,
    with the slope of norm^2 taken from the initial bracket of the search
    (qutip/solver/mcsolve.py:321-369)."""
    import importlib
    M = importlib.import_module("qutip.solver.mcsolve")
    windows = []
    find0, do0 = M.MCIntegrator._find_collapse_time, M.MCIntegrator._do_collapse

    def find(self, norm_old, norm, t_prev, t_final):
        slope = abs(norm_old - norm) / max(t_final - t_prev, 1e-300)
        self._gold_window = (2 * self.options["norm_tol"] * self.target_norm / max(slope, 1e-300)
                             + 2 * self.options["norm_t_tol"])
        return find0(self, norm_old, norm, t_prev, t_final)

    def do(self, t, state):
        n0 = len(self.collapses)
        do0(self, t, state)
        if len(self.collapses) > n0:
            windows.append(self._gold_window)

    M.MCIntegrator._find_collapse_time = find
    M.MCIntegrator._do_collapse = do
    return windows, (M, find0, do0)


def _mc_fixture(fname, H, c_ops, psi0, e_ops, tlist, ntraj, seed):
    windows, undo = _hook_collapse_windows()
    ss = np.random.SeedSequence(seed)
    seeds = ss.spawn(ntraj)
    states = []
    for s in seeds:
        st = np.random.default_rng(s).bit_generator.state["state"]
        states.append([st["state"] >> 64, st["state"] & (2**64 - 1), st["inc"] >> 64,
                       st["inc"] & (2**64 - 1)])
    t0 = time.time()
    res = qutip.mcsolve(H, psi0, tlist, c_ops, e_ops=e_ops, ntraj=ntraj, seeds=seeds,
                        options={"method": "vern7", "keep_runs_results": True,
                                 "progress_bar": False, "map": "serial"})
    wall = time.time() - t0
    M, find0, do0 = undo
    M.MCIntegrator._find_collapse_time, M.MCIntegrator._do_collapse = find0, do0
    col_t, col_w, col_off = [], [], [0]
    for tr in range(ntraj):
        col_t += list(res.col_times[tr])
        col_w += list(res.col_which[tr])
        col_off.append(len(col_t))
    runs = np.array([np.asarray(e) for e in res.runs_expect])  # (n_e, ntraj, nt)
    Hd = _data.to(_data.CSR, H.data).as_scipy().tocsr()
    out = dict(tlist=tlist, seed=seed, ntraj=ntraj, pcg_state=np.array(states, dtype=np.uint64),
               col_times=np.array(col_t), col_which=np.array(col_w, dtype=np.int32),
               col_off=np.array(col_off, dtype=np.int32), col_window=np.array(windows),
               runs_expect=runs,
               avg_expect=np.array([np.asarray(e) for e in res.expect]), wall=wall,
               psi0=psi0.full().ravel(), **_csr_arrays("H", Hd))
    for i, c in enumerate(c_ops):
        out.update(_csr_arrays(f"c{i}", c))
    for i, e in enumerate(e_ops):
        out.update(_csr_arrays(f"e{i}", e))
    np.savez(os.path.join(HERE, fname), **out)


def mc_fixtures():
    H, c_ops, psi0, n = _bh_qobjs(8)
    _mc_fixture("bh_mcsolve.npz", H, c_ops, psi0, n, np.linspace(0, 50, 501), 24, 20261203)
    H, c_ops, psi0, e_ops = _jc_qobjs(5, 2 * np.pi, 2 * np.pi, 2 * np.pi * 0.08, 0.3, 0.2)
    _mc_fixture("jc_mcsolve.npz", H, c_ops, psi0, e_ops, np.linspace(0, 20, 101), 32, 4242)
    # a strongly driven, strongly damped trimer: several jumps per trajectory
    H, c_ops, psi0, n = _bh_qobjs(4, F=1.0, kappa=0.5)
    _mc_fixture("bh_jumpy_mcsolve.npz", H, c_ops, psi0, n, np.linspace(0, 10, 101), 32, 777)


def bh_full_mcsolve(ntraj=4096, seed=20261203):
    """The Bose-Hubbard trimer (cutoff 8, ring) mcsolve at full size: 4096 trajectories
    over tlist linspace(0, 50, 501), seeds SeedSequence(seed).spawn(4096), the
    reference's vern7 with map="serial" (so that the bisection window of every jump is
    recorded, as for the small fixtures).  Stored: the averaged expectation values, their
    spread over the trajectories (for the statistical error of the mean) and every
    trajectory's jump record with its windows -- not the per-trajectory runs."""
    H, c_ops, psi0, n = _bh_qobjs(8)
    tlist = np.linspace(0, 50, 501)
    seeds = np.random.SeedSequence(seed).spawn(ntraj)
    windows, undo = _hook_collapse_windows()
    t0 = time.time()
    res = qutip.mcsolve(H, psi0, tlist, c_ops, e_ops=n, ntraj=ntraj, seeds=seeds,
                        options={"method": "vern7", "progress_bar": False, "map": "serial"})
    wall = time.time() - t0
    M, find0, do0 = undo
    M.MCIntegrator._find_collapse_time, M.MCIntegrator._do_collapse = find0, do0
    col_t, col_w, col_off = [], [], [0]
    for tr in range(ntraj):
        col_t += list(res.col_times[tr])
        col_w += list(res.col_which[tr])
        col_off.append(len(col_t))
    np.savez_compressed(os.path.join(HERE, "bh_full_mcsolve.npz"), tlist=tlist, seed=seed,
                        ntraj=ntraj, avg_expect=np.array([np.asarray(e) for e in res.expect]),
                        std_expect=np.array([np.asarray(e) for e in res.std_expect]),
                        col_times=np.array(col_t), col_which=np.array(col_w, dtype=np.int8),
                        col_off=np.array(col_off, dtype=np.int32),
                        col_window=np.array(windows), wall=wall, cores=1)


def pcg64():
    out = {}
    for i, seed in enumerate([0, 1, 12345, 2**63 + 7]):
        g = np.random.default_rng(seed)
        st = g.bit_generator.state["state"]
        out[f"s{i}"] = np.array([st["state"] >> 64, st["state"] & (2**64 - 1), st["inc"] >> 64,
                                 st["inc"] & (2**64 - 1)], dtype=np.uint64)
        g2 = np.random.default_rng(seed)
        out[f"raw{i}"] = np.array([g2.bit_generator.random_raw() for _ in range(16)], dtype=np.uint64)
        out[f"dbl{i}"] = np.array([g.random() for _ in range(16)])
    np.savez(os.path.join(HERE, "pcg64.npz"), **out)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--large", action="store_true")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    jobs = {"tableau": tableau, "kernels": kernels, "jc": jc_mesolve,
            "ising3": lambda: ising(3), "ising4": lambda: ising(4), "mc": mc_fixtures, "pcg": pcg64}
    if a.only and "bh4096" in a.only.split(","):
        jobs["bh4096"] = bh_full_mcsolve
    for name, fn in jobs.items():
        if a.only and name not in a.only.split(","):
            continue
        t0 = time.time()
        fn()
        print(f"{name}: {time.time() - t0:.1f}s", flush=True)
    if a.large:
        t0 = time.time()
        ising(10, name="ising_L10_expect.npz")
        print(f"ising10: {time.time() - t0:.1f}s", flush=True)
