"""The bench's multi-rank path on CPU: two gloo ranks on 127.0.0.1 meet at barriers,
take the max of their per-rank times, and the reference arm runs on rank 0 only."""
import contextlib
import io
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world, backend="gloo")
    d.init()
    d.barrier()
    m = d.max(float(rank + 1) * 1.5)
    d.barrier()
    out.put((rank, d.world, m))
    d.close()


def test_two_gloo_ranks_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2, 3.0), (1, 2, 3.0)]


def _ref_rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    called = []
    want = np.load(bench.GOLDEN)["expect"]
    bench.reference_solve = lambda steps, warmup: called.append(steps) or {
        "times": [0.5] * steps, "expect": want, "rhs_s": 0.1, "coefficient": {}}
    d = bench.Dist(world, backend="gloo")

    class A:
        steps, warmup, gpus = 2, 0, world
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(A, d)
    out.put((rank, len(called), buf.getvalue().count('"impl": "reference"')))


def test_reference_arm_runs_on_rank0_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ref_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 1, 1), (1, 0, 0)]
