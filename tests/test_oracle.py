"""The CPU oracle against golden vectors produced by the reference QuTiP itself."""
import numpy as np
import pytest

from conftest import csr_from, golden, jump_records_match, jump_times_close, pcg_state

from oracle import kernels as K
from oracle.pcg64 import PCG64
from oracle.solvers import mc_trajectory, mesolve
from qutip_gb300 import systems as S
from qutip_gb300 import vern7_tableau as T


def test_tableau_bits_match_reference():
    g = golden("vern7_tableau.npz")
    a = np.zeros((16, 16))
    for i, row in enumerate(T.A):
        a[i, :len(row)] = row
    assert np.array_equal(a, g["a"])
    assert np.array_equal(np.array(T.B), g["b"])
    assert np.array_equal(np.array(T.C), g["c"])
    assert np.array_equal(np.array(T.E), g["e"])
    assert np.array_equal(np.array(T.BI), g["bi"])
    assert T.ORDER == int(g["order"])


@pytest.mark.parametrize("i", [0, 1, 2])
def test_spmv_csr_dia_expect_wrmn(i):
    g = golden("kernels.npz")
    d, c, p = g[f"spmv{i}_data"], g[f"spmv{i}_indices"], g[f"spmv{i}_indptr"]
    x = g[f"spmv{i}_x"]
    out = K.spmv_csr(d, c, p, x, scale=0.5j, out=g[f"spmv{i}_out0"].copy())
    np.testing.assert_allclose(out, g[f"spmv{i}_res"], rtol=1e-13, atol=1e-13)
    n = len(x)
    outd = K.spmv_dia(g[f"dia{i}_data"], g[f"dia{i}_offsets"], n, n, x)
    np.testing.assert_allclose(outd, g[f"dia{i}_res"], rtol=1e-13, atol=1e-13)
    import scipy.sparse as sp
    op = sp.csr_matrix((d, c, p), shape=(n, n))
    if f"exp{i}_rho" in g:
        np.testing.assert_allclose(K.expect_csr_dm(op, g[f"exp{i}_rho"]), g[f"exp{i}_dm"], rtol=1e-12)
    np.testing.assert_allclose(K.expect_csr_ket(op, x), g[f"exp{i}_ket"], rtol=1e-12)
    np.testing.assert_allclose(K.wrmn_error(x * 1e-7, g[f"wrmn{i}_y"], 1e-8, 1e-6), g[f"wrmn{i}"],
                               rtol=1e-13)


def test_expect_super():
    import scipy.sparse as sp
    g = golden("kernels.npz")
    op = sp.csr_matrix((g["super_data"], g["super_indices"], g["super_indptr"]), shape=(36, 36))
    np.testing.assert_allclose(K.expect_super_csr(op, g["super_vec"]), g["super_res"], rtol=1e-12)


def test_pcg64_matches_numpy_draws():
    g = golden("pcg64.npz")
    for i in range(4):
        s = [int(v) for v in g[f"s{i}"]]
        r = PCG64((s[0] << 64) | s[1], (s[2] << 64) | s[3])
        assert [r.next_u64() for _ in range(16)] == [int(v) for v in g[f"raw{i}"]]
        r = PCG64((s[0] << 64) | s[1], (s[2] << 64) | s[3])
        assert [r.random() for _ in range(16)] == list(g[f"dbl{i}"])


def test_jc_mesolve_oracle_matches_reference():
    g = golden("jc_mesolve.npz")
    L = csr_from(g, "L")
    sysm = S.jaynes_cummings()
    L2 = sysm.terms[0][0]
    assert abs(L - L2).max() < 1e-13
    ex, ig = mesolve([(L, None)], g["rho0"], g["tlist"], [csr_from(g, "e0"), csr_from(g, "e1")])
    np.testing.assert_allclose(ex.real, g["expect"], atol=1e-10, rtol=0)
    # the adaptive step sequence is the reference's
    from oracle.vern7 import Vern7
    from oracle.solvers import make_deriv
    v = Vern7(make_deriv([(L, None)]))
    v.set_initial_value(g["rho0"], 0.0)
    ends = []
    while v.t_front < 20.0:
        v.integrate(20.0, step=True)
        ends.append(v.t_front)
    assert len(ends) == len(g["step_ends"])
    np.testing.assert_allclose(ends, g["step_ends"], rtol=1e-8)


@pytest.mark.parametrize("L", [3, 4])
def test_ising_mesolve_oracle_matches_reference(L):
    g = golden(f"ising_L{L}_mesolve.npz")
    sysm = S.ising_chain(L)
    np.testing.assert_array_equal(sysm.meta["h"], g["h"])
    if L == 3:
        for tt in (0.0, 0.37, 2.1):
            Lt = sum(op * (1 if c is None else c(tt)) for op, c in sysm.terms).toarray()
            np.testing.assert_allclose(Lt, g[f"L_at_{tt}"], atol=1e-14)
    ex, _ = mesolve(sysm.terms, sysm.state0, g["tlist"], sysm.e_ops)
    np.testing.assert_allclose(ex.real, g["expect"], atol=1e-9, rtol=0)


def _mc_check(name, build, ntraj, bh_params=None):
    g = golden(name)
    H = csr_from(g, "H")
    c_ops = [csr_from(g, f"c{i}") for i in range(8) if f"c{i}_data" in g]
    e_ops = [csr_from(g, f"e{i}") for i in range(8) if f"e{i}_data" in g]
    heff = [(-1j * H + sum(-0.5 * (c.conj().T @ c) for c in c_ops), None)]
    sysm = build()
    assert abs(sysm.terms[0][0] - heff[0][0]).max() < 1e-13
    for tr in range(ntraj):
        rng = pcg_state(g["pcg_state"][tr])
        ex, cols = mc_trajectory(heff, c_ops, g["psi0"], g["tlist"], e_ops, rng)
        got_t, got_w = [t for t, _ in cols], [w for _, w in cols]
        assert jump_records_match(got_t, got_w, g, tr), (tr, cols)
        if jump_times_close(got_t, g, tr):
            np.testing.assert_allclose(ex.real, g["runs_expect"][:, tr, :], atol=1e-6)


def test_bh_mcsolve_oracle_matches_reference_jump_records():
    _mc_check("bh_mcsolve.npz", lambda: S.bose_hubbard_trimer(8), 24)


def test_bh_jumpy_mcsolve_oracle_matches_reference_jump_records():
    _mc_check("bh_jumpy_mcsolve.npz", lambda: S.bose_hubbard_trimer(4, F=1.0, kappa=0.5, kind="mc"),
              16)


def test_jc_mcsolve_oracle_matches_reference_jump_records():
    _mc_check("jc_mcsolve.npz",
              lambda: S.jaynes_cummings(5, g=2 * np.pi * 0.08, kappa=0.3, gamma=0.2, kind="mc"), 16)
