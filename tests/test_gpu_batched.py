"""Batched persistent solves (one launch, many systems / trajectories) against the
reference's golden results and against the single-system GPU path."""
import numpy as np
import pytest

from conftest import csr_from, golden, jump_records_match, jump_times_close, pcg_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _close(got, want, atol=1e-8, rtol=1e-6):
    got, want = np.asarray(got), np.asarray(want)
    assert np.all(np.abs(got - want) <= atol + rtol * np.abs(want)), np.abs(got - want).max()


@pytest.mark.parametrize("precision,atol", [("double", 1e-8), ("mixed", 2e-6)])
def test_batched_jc_config1_matches_reference(precision, atol):
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import mesolve_batch
    g = golden("jc_mesolve.npz")
    s = S.jaynes_cummings()
    ex, res = mesolve_batch([s, s, s], g["tlist"], precision=precision)
    for e in ex:
        for k in range(2):
            _close(e[k].real, g["expect"][k], atol=atol)
    assert res[0]["steps"] >= len(g["step_ends"])


def test_cta_shape_with_staged_vectors_near_the_default_limit():
    """A CTA-shape launch whose staged vectors (46.6 KB for a 2916-entry mixed-form state)
    plus the kernel's static shared memory exceed the 48 KB default: the launch is opted in
    and its result equals the same system solved in the warp-free cluster shape."""
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem, check_status
    s = S.jaynes_cummings(27, kind="me")
    tl = np.linspace(0, 2, 11)

    def run(group):
        bp = BatchProblem("c64")
        bp.add_item(bp.add_system(s.terms, s.e_ops, tl, "me"), s.state0)
        bp.build(group=group)
        bp.launch()
        r = bp.results()
        check_status(r)
        return r[0]["expect"]
    a, b = run("cta"), run("cluster")
    np.testing.assert_allclose(a, b, atol=2e-6, rtol=0)


def test_mixed_sizes_alone_equals_in_the_mix():
    """Each system of a mixed-size batch gives the result it gives when solved alone."""
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import mesolve_batch
    tl = np.linspace(0, 4, 21)
    systems = [S.jaynes_cummings(n_cav=n, g=2 * np.pi * (0.02 + 0.01 * n), kappa=0.01 * n,
                                 gamma=0.02) for n in (3, 7, 12, 5)] + [S.ising_chain(3),
                                                                      S.ising_chain(4)]
    for prec in ("double", "mixed"):
        mix, _ = mesolve_batch(systems, tl, precision=prec)
        for i, s in enumerate(systems):
            alone, _ = mesolve_batch([s], tl, precision=prec)
            for k in range(len(s.e_ops)):
                np.testing.assert_array_equal(mix[i][k], alone[0][k])


def test_batched_ising_td_matches_reference():
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import mesolve_batch
    g = golden("ising_L4_mesolve.npz")
    ex, _ = mesolve_batch([S.ising_chain(4)], g["tlist"], precision="double")
    for k in range(4):
        _close(ex[0][k].real, g["expect"][k])


def _mc_golden(name, build, precision, group="auto"):
    from qutip_gb300.batched import mcsolve_batch
    g = golden(name)
    s = build()
    ntraj = int(g["ntraj"])
    seeds = []
    for tr in range(ntraj):
        row = [int(v) for v in g["pcg_state"][tr]]
        seeds.append(((row[0] << 64) | row[1], (row[2] << 64) | row[3]))
    r = mcsolve_batch(s, g["tlist"], ntraj, seeds=seeds, precision=precision, group=group)
    same = sum(jump_records_match(r.col_times[tr], r.col_which[tr], g, tr) for tr in range(ntraj))
    for tr in range(ntraj):
        if jump_times_close(r.col_times[tr], g, tr):
            _close(r.runs_expect[:, tr, :].real, g["runs_expect"][:, tr, :], atol=1e-5, rtol=1e-5)
    return g, r, same, ntraj


MC_CASES = {
    "bh_mcsolve.npz": lambda S: S.bose_hubbard_trimer(8),
    "bh_jumpy_mcsolve.npz": lambda S: S.bose_hubbard_trimer(4, F=1.0, kappa=0.5, kind="mc"),
    "jc_mcsolve.npz": lambda S: S.jaynes_cummings(5, g=2 * np.pi * 0.08, kappa=0.3, gamma=0.2,
                                                  kind="mc"),
}


@pytest.mark.parametrize("name", sorted(MC_CASES))
def test_mc_jump_records_identical_double(name):
    """complex128: every trajectory has the reference's jump count and channels, each
    jump time inside the reference's own bisection window."""
    from qutip_gb300 import systems as S
    g, r, same, ntraj = _mc_golden(name, lambda: MC_CASES[name](S), "double")
    assert same == ntraj


@pytest.mark.parametrize("name", sorted(MC_CASES))
def test_mc_mixed_precision_jump_records(name):
    """complex64 stages: jump records match the reference's (observed: every trajectory
    of every fixture).  The slack is one trajectory per fixture: a complex64 trajectory
    may legitimately end its jump-time bisection across the edge of the reference's
    window.  The averaged expectations agree within statistical error."""
    from qutip_gb300 import systems as S
    g, r, same, ntraj = _mc_golden(name, lambda: MC_CASES[name](S), "mixed")
    print(f"\n{name} mixed: {same}/{ntraj} identical jump records")
    assert same >= ntraj - 1
    sem = g["runs_expect"].std(axis=1) / np.sqrt(ntraj)
    diff = np.abs(r.runs_expect.real.mean(axis=1) - g["runs_expect"].mean(axis=1))
    assert np.all(diff <= 5 * sem + 1e-3)


@pytest.mark.parametrize("group", ["cta", "cta128", "cluster"])
@pytest.mark.parametrize("name", sorted(MC_CASES))
def test_mc_other_groups_match_reference(name, group):
    """The same trajectories with one 256-thread CTA, or one 8-CTA thread-block
    cluster, per item instead of a warp."""
    from qutip_gb300 import systems as S
    g, r, same, ntraj = _mc_golden(name, lambda: MC_CASES[name](S), "double", group=group)
    assert same == ntraj


@pytest.mark.parametrize("group", ["cta", "cta128", "cluster"])
def test_batched_me_groups_match_reference(group):
    """Master equations (Jaynes-Cummings N=10, Ising L=4) with CTA and cluster groups."""
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem, check_status
    g = golden("ising_L4_mesolve.npz")
    s = S.ising_chain(4)
    bp = BatchProblem("c128")
    sid = bp.add_system(s.terms, s.e_ops, g["tlist"], "me")
    bp.add_item(sid, s.state0)
    bp.build(group=group)
    bp.launch()
    res = bp.results()
    check_status(res)
    for k in range(4):
        _close(res[0]["expect"][:, k].real, g["expect"][k])


def _jc_problem(n_items, seeds, dtype="c64"):
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem
    s = S.jaynes_cummings(6, g=2 * np.pi * 0.08, kappa=0.3, gamma=0.2, kind="mc")
    bp = BatchProblem(dtype)
    sid = bp.add_system(s.terms, s.e_ops, np.linspace(0, 10, 51), "mc", c_ops=s.c_ops)
    for sd in seeds[:n_items]:
        bp.add_item(sid, s.state0, seed=sd)
    return bp


def test_graph_replay_matches_plain_launches():
    """A captured launch replayed with new seeds gives what a fresh launch with those
    seeds gives, bit for bit."""
    seeds_a = np.random.SeedSequence(1).spawn(96)
    seeds_b = np.random.SeedSequence(2).spawn(96)
    plain_a = _jc_problem(96, seeds_a)
    plain_a.build(max_jumps=64)
    plain_a.launch()
    ra = plain_a.results()
    plain_b = _jc_problem(96, seeds_b)
    plain_b.build(max_jumps=64)
    plain_b.launch()
    rb = plain_b.results()
    bp = _jc_problem(96, seeds_a)
    bp.build(max_jumps=64)
    bp.capture()
    bp.replay()
    torch.cuda.synchronize()
    for x, y in zip(bp.results(), ra):
        np.testing.assert_array_equal(x["expect"], y["expect"])
        np.testing.assert_array_equal(x["col_times"], y["col_times"])
    bp.replay(seeds=seeds_b)
    torch.cuda.synchronize()
    for x, y in zip(bp.results(), rb):
        np.testing.assert_array_equal(x["expect"], y["expect"])
        np.testing.assert_array_equal(x["col_which"], y["col_which"])


def test_tune_batch_picks_a_valid_shape():
    from qutip_gb300.batched import tune_batch
    seeds = np.random.SeedSequence(3).spawn(64)
    best = tune_batch(lambda n: _jc_problem(n, seeds), sample_items=64, reps=1)
    assert best["group"] in ("warp", "cta") and 0 < best["slot_fraction"] <= 1
    assert best["ms"] > 0 and len(best["timings"]) >= 2


@pytest.mark.parametrize("group", ["warp", "cta"])
def test_staged_operator_matches_global_reads(group):
    """The generator copied into shared memory (bulk async copies, mbarrier) gives
    bit-identical trajectories to reading it from global memory."""
    seeds = np.random.SeedSequence(9).spawn(64)
    res = []
    for stage in (False, True):
        bp = _jc_problem(64, seeds)
        bp.build(max_jumps=64, group=group, stage_operator=stage)
        assert bp.staged_operator == stage
        bp.launch()
        res.append(bp.results())
    for x, y in zip(*res):
        np.testing.assert_array_equal(x["expect"], y["expect"])
        np.testing.assert_array_equal(x["col_times"], y["col_times"])


def test_many_collapse_operators_match_oracle():
    """Ising chain L=9 trajectories have 18 collapse operators (sigma-_i, sigma^z_i):
    the device walks all of them in the reference's order (mcsolve.py:384-391)."""
    from oracle.solvers import mc_trajectory
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import mcsolve_batch
    s = S.ising_chain(9, gamma_minus=0.5, gamma_z=0.3, kind="mc")
    assert len(s.c_ops) == 18
    tl = np.linspace(0.0, 2.0, 21)
    seeds = np.random.SeedSequence(12).spawn(3)
    r = mcsolve_batch(s, tl, 3, seeds=seeds, precision="double", max_jumps=64)
    total = 0
    for tr in range(3):
        ex, cols = mc_trajectory(s.terms, s.c_ops, s.state0, tl, s.e_ops, seeds[tr])
        assert [w for _, w in cols] == [int(w) for w in r.col_which[tr]]
        np.testing.assert_allclose(r.col_times[tr], [t for t, _ in cols], atol=1e-3)
        total += len(cols)
    assert total > 0


def test_bad_items_are_rejected_without_touching_memory():
    """A launch whose max_n is smaller than an item's state reports QG_BAD_ITEM for
    that item instead of running it."""
    seeds = np.random.SeedSequence(4).spawn(8)
    bp = _jc_problem(8, seeds)
    bp.build(max_jumps=16)
    bp.struct.max_n = 4          # the JC states have 12 entries
    bp.launch()
    torch.cuda.synchronize()
    st = bp.status.cpu().numpy().reshape(-1, 4)[:, 0]
    assert np.all(st == -8)


def test_single_time_point_and_empty_e_ops():
    """A tlist of one point records only the initial state; a system without e_ops still
    reports the trace."""
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem, check_status
    s = S.jaynes_cummings(5, kind="me")
    bp = BatchProblem("c128")
    a = bp.add_system(s.terms, s.e_ops, np.array([0.0]), "me")
    b = bp.add_system(s.terms, [], np.linspace(0, 1, 5), "me")
    bp.add_item(a, s.state0)
    bp.add_item(b, s.state0)
    bp.build()
    bp.launch()
    res = bp.results()
    check_status(res)
    assert res[0]["expect"].shape == (1, 2)
    np.testing.assert_allclose(res[0]["expect"][0].real, [0.0, 1.0], atol=1e-14)
    assert res[1]["expect"].shape == (5, 0)
    np.testing.assert_allclose(res[1]["norm"].real, 1.0, atol=1e-7)


def test_jump_overflow_is_reported():
    """More jumps than max_jumps stops the trajectory with QG_JUMP_OVERFLOW; the host
    raises with the reference-style message and keeps the recorded jumps."""
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem, check_status
    s = S.bose_hubbard_trimer(4, F=1.0, kappa=0.5, kind="mc")
    bp = BatchProblem("c128")
    sid = bp.add_system(s.terms, s.e_ops, np.linspace(0, 20, 41), "mc", c_ops=s.c_ops)
    for sd in np.random.SeedSequence(3).spawn(8):
        bp.add_item(sid, s.state0, seed=sd)
    bp.build(max_jumps=1)
    bp.launch()
    res = bp.results()
    assert any(r["status"] == -7 for r in res)
    for r in res:
        if r["status"] == -7:
            assert len(r["col_times"]) == 1
    with pytest.raises(RuntimeError, match="max_jumps"):
        check_status(res)


@pytest.mark.parametrize("kind", ["me", "mc"])
def test_many_eops_in_every_group_shape(kind):
    """Outputs with more e_ops than one barrier pair gathers (18 e_ops plus the trace or
    norm: three chunks of sums in the CTA and cluster shapes) equal the warp shape's,
    which sums each e_op on its own; the first four are also the reference's (Ising L=4)."""
    import scipy.sparse as sp
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem, check_status
    g = golden("ising_L4_mesolve.npz")
    s = S.ising_chain(4, kind=kind, gamma_minus=0.05 if kind == "me" else 1e-9,
                      gamma_z=0.02 if kind == "me" else 1e-9)
    eye = sp.identity(2, format="csr", dtype=np.complex128)
    paulis = [sp.csr_matrix(np.array(m, dtype=np.complex128))
              for m in ([[0, 1], [1, 0]], [[0, -1j], [1j, 0]], [[1, 0], [0, -1]])]

    def site(o, i):
        m = sp.identity(1, format="csr", dtype=np.complex128)
        for k in range(4):
            m = sp.kron(m, o if k == i else eye, format="csr")
        return m
    e_ops = list(s.e_ops) + [site(p, i) for p in paulis[:2] for i in range(4)] + \
        [site(paulis[0], i) @ site(paulis[0], i + 1) for i in range(3)] + \
        [site(paulis[2], 0) @ site(paulis[2], 3), site(paulis[1], 1) @ site(paulis[1], 2),
         sp.identity(16, format="csr", dtype=np.complex128)]
    assert len(e_ops) == 18
    tl = g["tlist"] if kind == "me" else np.linspace(0.0, 2.0, 21)
    out = {}
    for group in ("warp", "cta", "cta128", "cluster"):
        bp = BatchProblem("c128")
        sid = bp.add_system(s.terms, e_ops, tl, kind,
                            c_ops=s.c_ops if kind == "mc" else ())
        for k in range(3):
            bp.add_item(sid, s.state0, seed=np.random.SeedSequence(40 + k) if kind == "mc" else None)
        bp.build(group=group, max_jumps=8 if kind == "mc" else 0)
        bp.launch()
        res = bp.results()
        check_status(res)
        out[group] = res
    for group in ("cta", "cta128", "cluster"):
        for a, b in zip(out[group], out["warp"]):
            assert a["jumps"] == b["jumps"] == 0 or kind == "me"
            np.testing.assert_allclose(a["expect"], b["expect"], atol=1e-11, rtol=0)
            np.testing.assert_allclose(a["norm"], b["norm"], atol=1e-11, rtol=0)
    if kind == "me":
        for k in range(4):
            _close(out["cluster"][0]["expect"][:, k].real, g["expect"][k])
