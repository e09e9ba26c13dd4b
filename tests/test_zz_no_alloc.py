"""The allocation-free batched solver (qg_batch_vern7_noalloc) against the regular one.

Some callers cannot allocate device memory -- a host framework that owns the
device memory pool and only lends this library pointers, or a latency-critical
serving loop that must not synchronise on cudaMalloc/cudaFree.  They call the
variant whose workspace is a static device array.  This test calls it through
the C ABI twice in a row (the static array and its queue words keep the last
call's contents, so the second call checks that nothing stale leaks in) and
compares both outputs with qg_batch_vern7 on caller-owned memory.  The file is
collected last so that a failure here cannot hide failures elsewhere.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _problem(dtype):
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem
    bp = BatchProblem(dtype)
    tl = np.linspace(0, 3, 16)
    for n_cav in (3, 6, 9):
        s = S.jaynes_cummings(n_cav=n_cav, kappa=0.05, gamma=0.1)
        bp.add_item(bp.add_system(s.terms, s.e_ops, tl, "me"), s.state0)
    mc = S.bose_hubbard_trimer(3, F=1.0, kappa=0.5, kind="mc")
    sid = bp.add_system(mc.terms, mc.e_ops, np.linspace(0, 5, 26), "mc", c_ops=mc.c_ops)
    for seed in np.random.SeedSequence(11).spawn(12):
        bp.add_item(sid, mc.state0, seed=seed)
    return bp.build(max_jumps=64)


def _snapshot(bp):
    torch.cuda.synchronize()
    return (bp.out.cpu().numpy().copy(), bp.status.cpu().numpy().copy(),
            bp.jump_t.cpu().numpy().copy(), bp.jump_which.cpu().numpy().copy())


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_noalloc_matches_allocating_entry_point_twice(dtype):
    from qutip_gb300 import _lib
    from qutip_gb300.operator import stream_ptr
    lib = _lib.load()
    bp = _problem(dtype)
    bp.launch()
    want = _snapshot(bp)
    assert np.all(want[1].reshape(-1, 4)[:, 0] == 0)
    for _ in range(2):
        bp.out.zero_()
        bp.status.zero_()
        bp.jump_t.zero_()
        bp.jump_which.zero_()
        rc = lib.qg_batch_vern7_noalloc(C.byref(bp.struct), stream_ptr())
        _lib.check(rc, "qg_batch_vern7_noalloc")
        # the staging-timeout flag of this call, read before the next call clears it
        assert lib.qg_batch_noalloc_staging_fault(stream_ptr()) == 0
        got = _snapshot(bp)
        np.testing.assert_allclose(got[0], want[0], rtol=1e-12, atol=1e-14)
        np.testing.assert_array_equal(got[1].reshape(-1, 4)[:, [0, 3]],
                                      want[1].reshape(-1, 4)[:, [0, 3]])
        np.testing.assert_allclose(got[2], want[2], rtol=1e-12, atol=1e-14)
        np.testing.assert_array_equal(got[3], want[3])


def test_noalloc_rejects_oversized_slots():
    from qutip_gb300 import _lib
    from qutip_gb300.operator import stream_ptr
    bp = _problem("c128")
    big = bp.struct.max_n
    bp.struct.max_n = 1 << 20  # one slot of this size exceeds the 16 MiB static workspace
    rc = _lib.load().qg_batch_vern7_noalloc(C.byref(bp.struct), stream_ptr())
    bp.struct.max_n = big
    assert rc == _lib.QG_ERR_ARG
    assert b"static workspace" in _lib.load().qg_last_error()
