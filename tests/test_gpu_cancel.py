"""Failure handling of the persistent batched solver without any GPU fault: a
host-visible cancel flag stops a long launch, every unfinished item reports the
timeout status, and the context stays usable."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_cancel_flag_stops_a_long_launch():
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem
    mc = S.bose_hubbard_trimer(6, F=1.0, kappa=0.05, kind="mc")
    bp = BatchProblem("c64")
    sid = bp.add_system(mc.terms, mc.e_ops, np.linspace(0, 2000, 2001), "mc", c_ops=mc.c_ops)
    for seed in np.random.SeedSequence(3).spawn(2000):
        bp.add_item(sid, mc.state0, seed=seed)
    bp.build(max_jumps=4096)
    flag = torch.zeros(1, dtype=torch.int32).pin_memory()
    bp.set_cancel(flag)
    progress = torch.zeros(bp.n_slots, dtype=torch.int64, device="cuda")
    bp.struct.progress = progress.data_ptr()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        bp.launch()
        ev = torch.cuda.Event()
        ev.record(side)
    time.sleep(0.5)
    assert not ev.query(), "the launch should still be running"
    flag[0] = 1
    t0 = time.time()
    while not ev.query() and time.time() - t0 < 20:
        time.sleep(0.01)
    assert ev.query(), "cancel flag not honoured"
    stopped = time.time() - t0
    st = bp.status.cpu().numpy().reshape(-1, 4)[:, 0]
    assert np.any(st == -6)
    assert set(np.unique(st)) <= {0, -6}
    print(f"\ncancelled {np.sum(st == -6)} of {len(st)} items in {stopped * 1e3:.0f} ms")
    # the context is still usable
    x = torch.ones(4, device="cuda")
    assert float(x.sum()) == 4.0
