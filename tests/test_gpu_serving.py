"""Continuous-batching server: every job's result in the served mix is the result the
same job gets alone, and the mixed-precision results stay within the stated error of
the plain complex128 per-request solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _jobs(n=40, rate=400.0):
    from qutip_gb300.serving import build_job, jc_request_stream
    specs = jc_request_stream(n, rate=rate, ntraj=6, seed=5, n_min=3, n_max=12)
    tl = np.linspace(0, 5, 26)
    return [build_job(s, tl) for s in specs]


def test_served_results_equal_alone_results():
    from qutip_gb300.serving import Server, percentiles
    jobs = _jobs()
    srv = Server("mixed", n_streams=3, max_jobs_per_launch=7, group="auto")
    jobs, wall = srv.serve(jobs, realtime=True)
    assert srv.stats["launches"] >= 3 and srv.stats["max_concurrent"] >= 1
    assert all(j.done is not None for j in jobs)
    p = percentiles([j.latency for j in jobs])
    assert p["p99_ms"] >= p["p50_ms"] > 0
    alone_srv = Server("mixed", n_streams=1, max_jobs_per_launch=1, group="auto")
    for j in jobs[:12]:
        ref = _jobs()[j.spec.id]
        alone_srv.serve([ref], realtime=False)
        for a, b in zip(j.result, ref.result):
            np.testing.assert_array_equal(a, b)


def test_served_mixed_precision_error_vs_plain_double():
    """Served mesolve requests (mixed form) against the plain complex128 drop-in served in
    real time: relative error <= 1e-6 (max over times and e_ops of the difference over the
    largest |<e_op>|); the real-time plain server returns what solve_plain returns and
    completes every request after its arrival."""
    from qutip_gb300.serving import Server, serve_plain, solve_plain
    jobs = [j for j in _jobs() if j.spec.kind == "me"][:8]
    Server("mixed").serve(jobs, realtime=False)
    plain = [j for j in _jobs() if j.spec.kind == "me"][:8]
    serve_plain(plain, "double")
    worst = 0.0
    for j, p in zip(jobs, plain):
        assert p.done is not None and p.latency > 0
        d = max(float(np.max(np.abs(np.real(a) - np.real(b)))) for a, b in zip(j.result, p.result))
        worst = max(worst, d / max(float(np.max(np.abs(np.real(b)))) for b in p.result))
    for a, b in zip(plain[0].result, solve_plain(plain[0], "double")):
        np.testing.assert_array_equal(a, b)
    print(f"\nserved mixed vs plain complex128: max relative difference {worst:.2e}")
    assert worst < 1e-6


def test_load_policy_results_match_fixed_shape():
    """With the load-dependent group shape, master-equation results equal those of a
    fixed shape to rounding (only the order of the FP64 reductions differs)."""
    from qutip_gb300.serving import Server
    jobs_a = [j for j in _jobs() if j.spec.kind == "me"][:10]
    jobs_b = [j for j in _jobs() if j.spec.kind == "me"][:10]
    Server("mixed", group="load").serve(jobs_a, realtime=False)
    Server("mixed", group="auto", max_jobs_per_launch=512).serve(jobs_b, realtime=False)
    for a, b in zip(jobs_a, jobs_b):
        for x, y in zip(a.result, b.result):
            np.testing.assert_allclose(x, y, rtol=1e-9, atol=1e-12)
