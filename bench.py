#!/usr/bin/env python
"""Benchmark: time-dependent Lindblad solve of the dissipative transverse-field
Ising chain, L = 10 spins (Hilbert dim 1024, Liouvillian dim 1,048,576,
24.6 M stored entries), Vern7 atol 1e-8 / rtol 1e-6, tlist = linspace(0, 10, 101),
10 e_ops, through QuTiP's own solver API with the GPU integrator plugged in.

One step = one complete solve in complex128, the reference's own arithmetic:
``MESolver(H, c_ops, options={"method": "gpu_vern7"}).run(rho0, tlist, e_ops)``
with QuTiP's Liouvillian already on the device (the solver built once, the initial
state resident).  ``e2e`` is the whole user call ``qutip.mesolve(H, rho0, tlist,
c_ops, e_ops, options={"method": "gpu_vern7"})`` from host Qobjs: QuTiP's Liouvillian
construction, the integrator's device build from host memory, the solve and the
expectation values read back.  The mixed form (complex64 stages, FP64 state and
step control) is reported beside it with its relative error against the
reference's FP64 result.  ``roofline`` is that of the complex128 fused Vern7 stage
kernel, timed with CUDA events on its stream.  Also reported: the served
mixed-size Jaynes-Cummings stream, the batched 4096-trajectory Bose-Hubbard
mcsolve, the matrix-free form and the L = 12 chain.

``--impl reference`` times one complete solve of the same workload with the
reference QuTiP (compiled from its sources into oracle/_ref) on the host cores,
split into ``--steps`` chunks of output times; nothing is extrapolated.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SITES = 10
T_END, N_OUT = 10.0, 101
METRIC = "solves_per_sec"
UNIT = "solves/s"
WORKLOAD = f"ising_chain_L{N_SITES}_mesolve_vern7"
CONFIG = {"workload": WORKLOAD, "n_sites": N_SITES, "hilbert_dim": 2 ** N_SITES,
          "liouvillian_dim": 4 ** N_SITES, "tlist": f"linspace(0,{T_END:g},{N_OUT})",
          "atol": 1e-8, "rtol": 1e-6, "e_ops": N_SITES, "h_seed": 1234,
          "api": "qutip MESolver / mesolve (QuTiP's Liouvillian, vern7 step control)",
          "l2": "per-step working set larger than L2 (129 MB): complex128 operator and 16 "
                "complex128 stage vectors of 16.8 MB each; no flush"}
GOLDEN = os.path.join(ROOT, "tests", "golden", "ising_L10_expect.npz")


def log(msg):
    """Progress to stderr (the JSON result line goes to stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=10,
                    help="output intervals of the CPU-baseline sample (of 100)")
    ap.add_argument("--e2e-reps", type=int, default=2,
                    help="whole mesolve calls timed for e2e (at most --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="headline workload only")
    ap.add_argument("--sections", default="served,mc,matrix,dense,sde,large",
                    help="extra sections after the headline (comma list of served, mc, "
                         "matrix, dense, sde, large)")
    ap.add_argument("--matrix-sites", type=int, default=13,
                    help="spins of the short matrix-form solve in the matrix section (0: skip)")
    ap.add_argument("--served-jobs", type=int, default=10000)
    ap.add_argument("--served-ntraj", type=int, default=100)
    ap.add_argument("--served-plain-sample", type=int, default=60)
    ap.add_argument("--mc-ntraj", type=int, default=4096)
    ap.add_argument("--large-sites", type=int, default=12,
                    help="Ising chain length of the large mixed-precision section (0: skip)")
    ap.add_argument("--profile", default=None,
                    choices=["stage", "batch", "matrix", "dense", "sde", "served-large"],
                    help="run the ncu profiling case only (fused stage kernel, untuned); "
                         "prints nothing to parse")
    ap.add_argument("--profile-sites", type=int, default=10)
    ap.add_argument("--profile-fmt", default="auto", choices=["auto", "sliced", "dict", "csr"],
                    help="operator storage of the stage profiling case")
    ap.add_argument("--profile-dtype", default="c64", choices=["c64", "c128"],
                    help="operator dtype of the stage profiling case")
    ap.add_argument("--profile-ntraj", type=int, default=256)
    ap.add_argument("--profile-branch", default="full", choices=["full", "hermitian"],
                    help="matrix profile: the full form or the Hermitian branch")
    ap.add_argument("--profile-tend", type=float, default=5.0)
    ap.add_argument("--profile-group", default="auto",
                    choices=["auto", "warp", "cta", "cta128", "cluster"])
    return ap.parse_args()


def host_qutip():
    """QuTiP, the host framework the plugin registers into, and the workload's Qobjs.

    On machines without an installed QuTiP this is the build of the reference's own
    sources in oracle/_ref; both arms build their inputs with the same constructors
    (``oracle.ref_workloads.ising_qobjs``).  QuTiP contributes the solver shell (option
    handling, Liouvillian construction, the output loop); in our arm every kernel of
    the integration runs from ``libqutip_gb300.so``."""
    from oracle import ref_workloads as RW
    qt = RW.import_reference()
    return qt, RW


def rel_err(got, want):
    """max over e_ops of max_t |got - want| / max_t |want| (norm-wise relative error of
    each expectation-value trajectory), and whether every point is within the
    reference's own tolerance atol 1e-8 + rtol 1e-6 |want|."""
    got = np.real(np.asarray(got, dtype=np.complex128))
    want = np.asarray(want, dtype=np.float64)
    rel = max(float(np.max(np.abs(g - w)) / max(np.max(np.abs(w)), 1e-300))
              for g, w in zip(got, want))
    absmax = float(np.max(np.abs(got - want)))
    within = bool(np.all(np.abs(got - want) <= 1e-8 + 1e-6 * np.abs(want)))
    return rel, absmax, within


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(self.index), "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- dist ------
class Dist:
    """Replicas over ranks: one process per GPU (NCCL), or CPU processes (gloo) for
    host-side tests.  Each rank solves its own copy of the workload; ranks only
    meet at barriers and in the max of the per-rank times."""

    def __init__(self, n_gpus, backend=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        self.n_gpus = n_gpus
        self.backend = backend

    def _cuda(self):
        import torch
        return self.backend != "gloo" and torch.cuda.is_available()

    def init(self):
        import torch
        if self.backend is None:
            self.backend = "nccl" if torch.cuda.is_available() else "gloo"
        if self._cuda():
            torch.cuda.set_device(self.local)
        if self.world > 1:
            import torch.distributed as dist
            if self.backend == "nccl":
                dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
            else:
                dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        import torch
        if self._cuda():
            torch.cuda.synchronize()
        if self.pg:
            self.pg.barrier()
        if self._cuda():
            torch.cuda.synchronize()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if self._cuda() else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------- cpu baseline --
def coefficient_path(qt, solver, rhs_s):
    """How the reference evaluates the string coefficient ``cos(w*t)``: compiled by
    Cython (``StrCoefficient``) or through Python ``eval`` (``StrFunctionCoefficient``,
    the fallback when Cython, setuptools or filelock is missing), with its measured cost
    per evaluation against one right-hand-side call (two evaluations per call)."""
    coeffs = [el[1] for el in solver.rhs.to_list() if isinstance(el, list)]
    if not coeffs:
        return {"path": "none"}
    c = coeffs[0]
    name = type(c).__name__
    path = ("eval (StrFunctionCoefficient)" if name == "StrFunctionCoefficient"
            else "compiled (StrCoefficient)" if name == "StrCoefficient" else name)
    reps = 2000
    t0 = time.perf_counter()
    for i in range(reps):
        c(0.001 * i)
    us = 1e6 * (time.perf_counter() - t0) / reps
    return {"path": path, "us_per_eval": us, "evals_per_rhs": len(coeffs),
            "share_of_rhs": len(coeffs) * us * 1e-6 / rhs_s}


def reference_rhs_seconds(qt, solver, rho0, reps=2):
    """Seconds per right-hand-side call of the reference (``QobjEvo.matmul_data`` of the
    Liouvillian on vec(rho0))."""
    from qutip.core import data as _data
    y = _data.to(_data.Dense, qt.operator_to_vector(rho0).data)
    solver.rhs.matmul_data(0.1, y)
    t0 = time.perf_counter()
    for _ in range(reps):
        solver.rhs.matmul_data(0.1, y)
    return (time.perf_counter() - t0) / reps


def cpu_baseline(n_sample: int, rhs_sample: int, rhs_full: int):
    """Reference vern7 mesolve (oracle/_ref) on the host over the first ``n_sample`` output
    intervals, scaled to one solve by right-hand-side calls: the reference and the
    complex128 GPU integrator take the same step sequence (tested), so the GPU solve's
    RHS counts of the window (``rhs_sample``) and of the whole solve (``rhs_full``) scale
    the window's time."""
    qt, RW = host_qutip()
    cores = os.cpu_count() or 1
    H, c_ops, rho0, e_ops = RW.ising_qobjs(N_SITES)
    tlist = np.linspace(0.0, T_END, N_OUT)
    opts = {"method": "vern7", "atol": 1e-8, "rtol": 1e-6, "progress_bar": False}
    solver = qt.MESolver(H, c_ops, options=opts)
    solver.run(rho0, tlist[:2], e_ops=e_ops)          # first-call setup out of the timing
    t0 = time.perf_counter()
    solver.run(rho0, tlist[:n_sample + 1], e_ops=e_ops)
    secs = time.perf_counter() - t0
    rhs_s = reference_rhs_seconds(qt, solver, rho0)
    full_s = secs * rhs_full / max(rhs_sample, 1)
    return {"value": 1.0 / full_s, "unit": UNIT, "cores": cores, "kind": "reference",
            "sample": (f"QuTiP reference (oracle/_ref) MESolver.run vern7, CSR complex128 "
                       f"(single-thread matvec, OpenBLAS vector ops on {cores} threads); "
                       f"outputs 0..{n_sample} of {N_OUT - 1} in {secs:.2f} s = {rhs_sample} "
                       f"RHS calls, scaled to the {rhs_full} RHS calls of the whole solve "
                       f"(counts from the complex128 GPU solve, which takes the reference's "
                       f"step sequence); {1e3 * rhs_s:.1f} ms per reference RHS call"),
            "rhs_sample": rhs_sample, "rhs_full": rhs_full, "sample_s": secs,
            "coefficient": coefficient_path(qt, solver, rhs_s)}


def reference_solve(steps: int, warmup: int) -> dict:
    """One complete reference solve of the workload, timed in ``steps`` chunks.

    The solver is built inside the first chunk, as ``qutip.mesolve`` builds it
    (QuTiP's Liouvillian construction included); the chunks then step through the output
    times with ``MESolver.step`` and evaluate the e_ops with ``qutip.expect`` at every
    output, the work ``MESolver.run`` does.  Warm-up steps are short solves of the first
    output interval.  Returns the chunk times, the expectation values, the seconds per
    right-hand-side call and the coefficient path."""
    qt, RW = host_qutip()
    H, c_ops, rho0, e_ops = RW.ising_qobjs(N_SITES)
    tlist = np.linspace(0.0, T_END, N_OUT)
    opts = {"method": "vern7", "atol": 1e-8, "rtol": 1e-6, "progress_bar": False}
    warm = qt.MESolver(H, c_ops, options=opts)
    for _ in range(warmup):
        warm.run(rho0, tlist[:2], e_ops=e_ops)
    K = max(1, min(steps, N_OUT - 1))
    chunks = np.array_split(np.arange(1, N_OUT), K)
    times = []
    expect = np.zeros((len(e_ops), N_OUT))
    solver = None
    for ci, chunk in enumerate(chunks):
        t0 = time.perf_counter()
        if ci == 0:
            solver = qt.MESolver(H, c_ops, options=opts)
            solver.start(rho0, tlist[0])
            expect[:, 0] = [qt.expect(e, rho0) for e in e_ops]
        for i in chunk:
            st = solver.step(tlist[i], copy=False)
            expect[:, i] = [qt.expect(e, st) for e in e_ops]
        times.append(time.perf_counter() - t0)
    rhs_s = reference_rhs_seconds(qt, solver, rho0)
    return {"times": times, "expect": expect, "rhs_s": rhs_s,
            "coefficient": coefficient_path(qt, solver, rhs_s)}


def run_reference(args, dist):
    """``--impl reference``: rank 0 times one complete reference solve (``value`` = 1 /
    the sum of its chunk times); other ranks exit without work."""
    if dist.rank != 0:
        return
    cores = os.cpu_count() or 1
    r = reference_solve(args.steps, args.warmup)
    times = r["times"]
    K = len(times)
    total = float(sum(times))
    v = 1.0 / total
    want = np.load(GOLDEN)["expect"]
    sample = (f"one complete QuTiP reference mesolve (oracle/_ref, vern7, CSR complex128, "
              f"single-thread matvec, OpenBLAS vector ops on {cores} threads) of the workload, "
              f"Liouvillian construction included, timed in {K} chunks of output times "
              f"({total:.1f} s); nothing extrapolated")
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": K, "warmup": args.warmup, "ms_per_step": 1e3 * total / K,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
           "data": "synthetic (seeded h_i ~ U[0.5,1.5], default_rng(1234))", "config": CONFIG,
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "reference",
                            "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "chunk_s": [round(x, 3) for x in times],
           "rhs_call_s": r["rhs_s"], "coefficient": r["coefficient"],
           "max_abs_diff_vs_golden": float(np.max(np.abs(r["expect"] - want)))}
    print(json.dumps(out))


# ------------------------------------------------------------------ ours ----
def stage_bytes(op, n, stage, mixed):
    """Algorithmic HBM bytes of one fused Vern7 stage launch: the operator (superoperator
    entries and row structure, or the matrix-free generator's small operators and its
    constant diagonal factor), the input read once, k_s written, and the vectors the
    stage combination reads and writes (earlier k_j, the base state, the next input)."""
    from qutip_gb300 import vern7_tableau as T
    sk = op.value_bytes()                       # stage dtype (k, ytmp, x)
    base = 8 if mixed else 16                   # y_prev_s (mixed) or y_prev
    b = op.operator_bytes()                     # operator stream (entries, codes, tables)
    b += n * sk                                 # x, read once
    b += n * sk                                 # k_s written
    if stage == T.RK_STEP - 1:
        used = [j for j in range(stage) if T.B[j] != 0 or T.E[j] != 0]
        b += len(used) * n * sk + 16 * n + 16 * n + (8 * n if mixed else 0)  # k_j, y_prev, y_front(+s)
    elif stage != T.RK_EXTRA_STEP - 1:
        row = T.A[stage + 1]
        b += sum(n * sk for j in range(stage) if row[j] != 0) + n * base + n * sk  # k_j, base, next x
    return b


def stage_fp64_fmas(op, n, stage):
    """Algorithmic FP64 fused multiply-adds of one complex128 fused Vern7 stage launch: the
    generator (two per nonzero real or imaginary part of the operator with the real /
    imaginary split dictionary, four per complex entry otherwise; two per row per
    time-dependent group for its coefficient) and the stage combination (two per row per
    nonzero tableau factor; the WRMS error adds four per row at the last stage)."""
    import torch
    from qutip_gb300 import vern7_tableau as T
    if getattr(op, "dict_split", False):
        gen = 2 * int(torch.count_nonzero(op.col).item())
    else:
        gen = 4 * int(op.nnz)
    gen += 2 * n * sum(1 for c in getattr(op, "coeffs", []) if c is not None)
    if stage == T.RK_STEP - 1:
        comb = 2 * n * sum(1 for j in range(T.RK_STEP) if T.B[j] != 0)
        comb += 2 * n * sum(1 for j in range(T.RK_STEP) if T.E[j] != 0) + 4 * n
    else:
        comb = 2 * n * sum(1 for j in range(stage + 1) if T.A[stage + 1][j] != 0)
    return gen + comb


#: FP64 peak of GB300 (nominal): 2 FP64 FMAs per clock per SM x 152 SMs x 2.07 GHz x 2
FP64_PEAK_TFLOPS = 2 * 152 * 2.07e9 * 2 / 1e12

TRAFFIC_PROFILE = "profiles/spmv_dict_c128_ising_L10_stage.md"
SLICED_PROFILE = "profiles/spmv_sliced_ising_L10_stage.md"


def profiled_traffic(path=TRAFFIC_PROFILE):
    """DRAM bytes per fused stage launch from a committed ncu summary, or None."""
    try:
        with open(os.path.join(ROOT, path)) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return int(line.split(":")[1])
    except OSError:
        pass
    return None


def measure_stage_roofline(op, state0, precision, reps=20, fmas=None):
    """Average duration and algorithmic GB/s of the fused stage kernel (events on its stream),
    from the initial state ``state0`` (host vector); ``fmas`` (a list) receives the average
    algorithmic FP64 FMAs per launch."""
    import ctypes as C
    import torch
    from qutip_gb300 import _lib
    from qutip_gb300.operator import stream_ptr
    from qutip_gb300.vern7 import GpuVern7
    ig = GpuVern7(op, precision=precision)
    ig.set_initial_value(torch.from_numpy(np.asarray(state0)).cuda(), 0.0)
    ig.integrate(0.05, step=True)
    total_bytes = sum(stage_bytes(op, ig.n, s, ig.mixed) for s in range(10))
    st = torch.cuda.current_stream()
    for _ in range(2):
        ig._compute_step(ig.dt_safe)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rk = ig._rk()
    sp_ = stream_ptr()
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        for s in range(10):
            op.vern7_stage(rk, s, 0.0, ig.dt_safe, ig.atol, ig.rtol, sp_)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / (reps * 10)
    per_launch = total_bytes / 10
    if fmas is not None:
        fmas.append(sum(stage_fp64_fmas(op, ig.n, s) for s in range(10)) / 10)
    return ms, per_launch, per_launch / (ms * 1e-3) / 1e9


def measure_spmv(op, reps=30):
    import torch
    x = torch.randn(op.n_cols, dtype=op.val.dtype, device="cuda")
    y = torch.empty(op.n_rows, dtype=op.val.dtype, device="cuda")
    op.matvec(0.3, x, y)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        op.matvec(0.3, x, y)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    b = op.spmv_bytes()
    return ms, b, b / (ms * 1e-3) / 1e9


def run_served(args):
    """Served mixed-size Jaynes-Cummings stream: continuous batching (complex64 stages,
    FP64 state) vs the plain complex128 per-request drop-in."""
    import torch
    from qutip_gb300.serving import (Server, build_job, fifo_latencies, jc_request_stream,
                                     percentiles, serve_plain, solve_plain)
    import dataclasses
    from qutip_gb300.serving import Job
    n = args.served_jobs
    specs = jc_request_stream(n, rate=1.0, ntraj=args.served_ntraj, seed=2026)
    jobs = [build_job(sp) for sp in specs]
    log(f"served: {n} jobs built")

    def rearrive(js, new_specs):
        # same requests (the stream's parameters do not depend on the rate), new arrivals
        return [Job(dataclasses.replace(j.spec, arrival=sp.arrival), j.system, j.tlist,
                    j.state_len) for j, sp in zip(js, new_specs)]
    warm = [build_job(sp) for sp in specs[:8]]
    Server("mixed").serve(warm, realtime=False)
    # throughput: every job available at t = 0
    srv = Server("mixed", launch_timeout=60.0)
    _, wall = srv.serve(jobs, realtime=False)
    thr = n / wall
    log(f"served: throughput {thr:.1f} solves/s")
    # latency at a Poisson rate of half the measured throughput
    rate = 0.5 * thr
    specs_r = jc_request_stream(n, rate=rate, ntraj=args.served_ntraj, seed=2026)
    assert all(a.n_cav == b.n_cav and a.seed == b.seed for a, b in zip(specs, specs_r))
    jobs_r = rearrive(jobs, specs_r)
    srv_r = Server("mixed", launch_timeout=60.0)
    _, wall_r = srv_r.serve(jobs_r, realtime=True)
    lat = percentiles([j.latency for j in jobs_r])
    log(f"served: latency {lat}")
    # plain complex128 per-request drop-in: measured service times on a sample
    k = min(args.served_plain_sample, n)
    service = []
    for j in jobs[:k]:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solve_plain(j, "double")
        torch.cuda.synchronize()
        service.append(time.perf_counter() - t0)
    plain_thr = 1.0 / float(np.mean(service))
    svc = [service[i % k] for i in range(n)]
    plain_lat = percentiles(fifo_latencies([sp.arrival for sp in specs_r], svc))
    # a load the plain arm sustains: half its throughput, the first 400 requests
    low_rate = 0.5 * (1.0 / float(np.mean(service)))
    m = min(400, n)
    specs_l = jc_request_stream(n, rate=low_rate, ntraj=args.served_ntraj, seed=2026)[:m]
    jobs_l = rearrive(jobs[:m], specs_l)
    Server("mixed", launch_timeout=60.0).serve(jobs_l, realtime=True)
    lat_low = percentiles([j.latency for j in jobs_l])
    # the plain arm served in real time on the same arrivals (measured, not modelled)
    jobs_lp = rearrive(jobs[:m], specs_l)
    wall_lp = serve_plain(jobs_lp, "double")
    plain_low = percentiles([j.latency for j in jobs_lp])
    plain_low_model = percentiles(fifo_latencies([sp.arrival for sp in specs_l],
                                                 [service[i % k] for i in range(m)]))
    log(f"served: at {low_rate:.1f} req/s served {lat_low}, plain {plain_low}")
    slow = sorted(jobs_l, key=lambda j: -(j.latency or 0))[:6]
    log("served: slowest at that rate: " + "; ".join(
        f"{j.spec.kind} N={j.spec.n_cav} {1e3 * j.latency:.0f} ms launch={j.extra.get('launch')} "
        f"(wait {j.extra.get('wait_ms', 0):.1f}, host {j.extra.get('host_ms', 0):.1f}, "
        f"gpu {j.extra.get('gpu_ms', 0):.1f}, collect {j.extra.get('collect_ms', 0):.1f} ms)"
        for j in slow))
    slowest = [{"kind": j.spec.kind, "n_cav": j.spec.n_cav, "latency_ms": 1e3 * j.latency,
                "launch": list(j.extra.get("launch", ())),
                **{k: j.extra.get(k) for k in ("wait_ms", "host_ms", "gpu_ms", "collect_ms")}}
               for j in slow]
    # error of the served mixed form vs the plain complex128 solve (same requests, same
    # trajectory seeds), relative to the largest |<e_op>| of each request, per kind, over
    # every request of the low-rate stream (both arms solved them)
    errs = {"me": [], "mc": []}
    abs_err = 0.0
    for js, jp in zip(jobs_l, jobs_lp):
        d = max(float(np.max(np.abs(np.real(a) - np.real(b)))) for a, b in zip(js.result, jp.result))
        scale = max(float(np.max(np.abs(np.real(b)))) for b in jp.result)
        errs[js.spec.kind].append(d / scale)
        abs_err = max(abs_err, d)
    # the same comparison at three quarters of the plain arm's throughput (a load it still
    # sustains, with more queueing): both arms served in real time on the same arrivals
    hi_rate = 0.75 * (1.0 / float(np.mean(service)))
    specs_h = jc_request_stream(n, rate=hi_rate, ntraj=args.served_ntraj, seed=2026)[:m]
    jobs_h = rearrive(jobs[:m], specs_h)
    Server("mixed", launch_timeout=60.0).serve(jobs_h, realtime=True)
    lat_h = percentiles([j.latency for j in jobs_h])
    jobs_hp = rearrive(jobs[:m], specs_h)
    wall_hp = serve_plain(jobs_hp, "double")
    plain_h = percentiles([j.latency for j in jobs_hp])
    log(f"served: at {hi_rate:.1f} req/s served {lat_h}, plain {plain_h}")
    n_me = sum(sp.kind == "me" for sp in specs)
    return {
        "workload": f"{n} Jaynes-Cummings jobs, N~U{{5..60}}, {n_me} mesolve / {n - n_me} mcsolve "
                    f"(ntraj={args.served_ntraj}), tlist linspace(0,20,101), seed 2026",
        "served_mixed": {"solves_per_sec": thr, "wall_s": wall, "launches": srv.stats["launches"],
                         "shape_retries": {k: v.stats.get("shape_retries", 0)
                                           for k, v in (("throughput", srv), ("high_rate", srv_r))},
                         "last_shape_error": srv_r.stats.get("last_shape_error",
                                                             srv.stats.get("last_shape_error")),
                         "latency_at_rate": {**lat, "rate_per_s": rate, "wall_s": wall_r,
                                             "max_concurrent_launches": srv_r.stats["max_concurrent"]}},
        "plain_c128": {"solves_per_sec": plain_thr, "service_sample_jobs": k,
                       "latency_at_rate": {**plain_lat, "rate_per_s": rate,
                                           "method": "measured service times, FIFO queue on the "
                                                     "same arrivals"}},
        "speedup_solves_per_sec": thr / plain_thr,
        "speedup_p99": plain_lat["p99_ms"] / lat["p99_ms"],
        "at_plain_sustainable_rate": {"rate_per_s": low_rate, "requests": m,
                                      "served_mixed": lat_low,
                                      "plain_c128": {**plain_low, "wall_s": wall_lp,
                                                     "method": "served in real time, one request "
                                                               "at a time in arrival order"},
                                      "plain_c128_fifo_model": plain_low_model,
                                      "slowest_requests": slowest,
                                      "speedup_p99": plain_low["p99_ms"] / lat_low["p99_ms"]},
        "at_three_quarters_of_plain_throughput": {
            "rate_per_s": hi_rate, "requests": m, "served_mixed": lat_h,
            "plain_c128": {**plain_h, "wall_s": wall_hp,
                           "method": "served in real time, one request at a time in arrival order"},
            "speedup_p99": plain_h["p99_ms"] / lat_h["p99_ms"]},
        "accuracy_vs_c128": {
            "requests": m, "mesolve": len(errs["me"]), "mcsolve": len(errs["mc"]),
            "max_rel_err_mesolve": max(errs["me"], default=None),
            "max_rel_err_mcsolve": max(errs["mc"], default=None),
            "max_abs_err": abs_err,
            "definition": "per request max_t,e |served - plain complex128| / max_t,e |plain|; "
                          "mcsolve with the same trajectory seeds"},
    }


def run_mc_batch(args):
    """Batched mcsolve of the dissipative Bose-Hubbard trimer, 4096 trajectories: the
    launch shape picked by the autotuner, the launch captured in a CUDA graph and
    replayed with fresh seeds each timed step."""
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem, check_status, tune_batch
    from qutip_gb300 import _lib
    s = S.bose_hubbard_trimer(8)
    tl = np.linspace(0.0, 50.0, 501)
    n = args.mc_ntraj

    def make(ntraj, dt, tlist, seeds):
        bp = BatchProblem(dt)
        sid = bp.add_system(s.terms, s.e_ops, tlist, "mc", c_ops=s.c_ops)
        for sd in seeds[:ntraj]:
            bp.add_item(sid, s.state0, seed=sd)
        return bp

    out = {}
    lib = _lib.load()
    for prec, dt in (("mixed", "c64"), ("double", "c128")):
        log(f"mc batch {prec}: tuning")
        tune_seeds = np.random.SeedSequence(7).spawn(2432)
        best = tune_batch(lambda k: make(k, dt, tl[:51], tune_seeds), sample_items=2432, reps=1)
        qdt = _lib.QG_C64 if dt == "c64" else _lib.QG_C128
        full = lib.qg_batch_group_slots(512, qdt, {"warp": 1, "cta": 2, "cluster": 3, "cta128": 4}[best["group"]])
        seeds0 = np.random.SeedSequence(20261203).spawn(n)
        bp = make(n, dt, tl, seeds0)
        bp.build(max_jumps=512, group=best["group"], n_slots=max(1, int(full * best["slot_fraction"])))
        bp.capture()
        bp.replay()                      # warm-up replay
        torch.cuda.synchronize()
        times = []
        for step in range(2):
            seeds = np.random.SeedSequence(20261204 + step).spawn(n)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            bp.replay(seeds=seeds)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        res = bp.results()
        check_status(res)
        runs = np.stack([r["expect"].T for r in res], axis=1)
        dt_s = float(np.median(times))
        out[prec] = {"trajectories_per_sec": n / dt_s, "wall_s": dt_s,
                     "jumps": int(sum(r["jumps"] for r in res)),
                     "n_mean_final": [float(runs[k, :, -1].real.mean()) for k in range(runs.shape[0])],
                     "launch": {"group": best["group"], "slot_fraction": best["slot_fraction"],
                                "n_slots": int(bp.n_slots), "tuned_ms": best["timings"]
                                and {f"{g}@{f}": round(ms, 2) for (g, f), ms in best["timings"].items()},
                                "graph": "captured once, replayed with new seeds (in-place item table)"}}
    out["workload"] = (f"Bose-Hubbard trimer cutoff 8 (dim 512), {n} trajectories, "
                       "tlist linspace(0,50,501), one persistent launch per step")
    if not args.no_cpu_baseline:
        log("mc batch: reference CPU mcsolve sample")
        try:
            p = subprocess.run([sys.executable, "-m", "oracle.ref_workloads", "mcsolve"],
                               cwd=ROOT, capture_output=True, text=True, timeout=600)
            ref = json.loads(p.stdout.strip().splitlines()[-1])
            out["cpu_baseline"] = {**ref, "kind": "reference",
                                   "sample": "QuTiP reference (oracle/_ref) mcsolve vern7, same "
                                             "system and tlist; map='serial' on 1 core and "
                                             "map='parallel' on every host core, fresh process"}
        except Exception as exc:  # noqa: BLE001
            out["cpu_baseline"] = {"value": None, "error": repr(exc)[:300]}
    return out


def hbm_peak_gbs():
    """Measured copy bandwidth of the GB300s (driver-written), else the fallback."""
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = json.load(open(pk)) if os.path.exists(pk) else {}
    if "hbm_gbs" in peaks:
        return float(peaks["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_large(args):
    """Large mixed-precision mesolve: the Ising chain at L = 12 (Liouvillian
    16,777,216 rows), tlist linspace(0,5,51).  The operator is assembled on the device
    (the host holds only the 4096 x 4096 operators); the complex64 solve is timed,
    its error against the complex128 solve of the same operator on the GPU is stated,
    and the complex64 matvec and fused-stage bandwidths are reported against HBM."""
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.solver import ExpectOps, solve_system
    from qutip_gb300.superop import liouvillian_groups
    L = args.large_sites
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = S.ising_chain(L, build_terms=False)
    groups = liouvillian_groups(s.h_terms, s.c_ops)
    op128 = DeviceOperator.from_device_groups(groups, "c128")
    # complex64 straight from the groups: the dictionary tables are built from the rounded
    # values (complex128 values summed on the device in varying order differ in their last
    # bits and do not deduplicate)
    op64 = DeviceOperator.from_device_groups(groups, "c64")
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    host_groups = None
    if not args.no_cpu_baseline:
        # the generator's CSR groups on the host, for the reference's matvec timing below
        host_groups = [(p.cpu().numpy(), i.to(torch.int32).cpu().numpy(), d.cpu().numpy(), c)
                       for p, i, d, c in groups]
    del groups
    torch.cuda.empty_cache()
    log(f"large: L={L} operator assembled on the device in {build_s:.1f} s, "
        f"{op64.nnz} entries ({op64.launch_desc()})")
    ex = ExpectOps(s.e_ops)
    tl = np.linspace(0.0, 5.0, 51)
    r128 = solve_system(s, tl, {"precision": "double"}, op=op128, ex=ex)
    solve_system(s, tl, {"precision": "mixed"}, op=op64, ex=ex)   # warm-up
    times = []
    for _ in range(2):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r64 = solve_system(s, tl, {"precision": "mixed"}, op=op64, ex=ex)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t1)
    err = max(float(np.max(np.abs(np.real(a) - np.real(b)))) for a, b in zip(r64.expect, r128.expect))
    rel = max(float(np.max(np.abs(np.real(a) - np.real(b))) / np.max(np.abs(np.real(b))))
              for a, b in zip(r64.expect, r128.expect))
    spmv_ms, spmv_b, spmv_gbs = measure_spmv(op64, reps=10)
    stage_ms, stage_b, stage_gbs = measure_stage_roofline(op64, s.state0, "mixed", reps=3)
    peak, _ = hbm_peak_gbs()
    out = {"workload": f"ising_chain_L{L}_mesolve_vern7 mixed, tlist linspace(0,5,51)",
           "liouvillian_rows": op64.n_rows, "entries": int(op64.nnz),
           "device_assembly_s": build_s, "solves_per_sec": 1.0 / float(np.median(times)),
           "s_per_solve": float(np.median(times)), "rhs_calls": int(r64.stats.get("rhs", 0)),
           "max_abs_err_vs_fp64_gpu": err, "rel_err_vs_fp64_gpu": rel,
           "steps_mixed_vs_fp64": [int(r64.stats["steps"]), int(r128.stats["steps"])],
           "spmv_c64": {"gbs": spmv_gbs, "ms": spmv_ms, "bytes": int(spmv_b), "frac": spmv_gbs / peak},
           "stage_c64": {"gbs": stage_gbs, "ms": stage_ms, "bytes": int(stage_b),
                         "frac": stage_gbs / peak},
           "cpu_baseline": None}
    del op64, op128
    torch.cuda.empty_cache()
    if host_groups is not None:
        try:
            out["cpu_baseline"] = large_cpu_baseline(host_groups, s.state0,
                                                     int(r128.stats.get("rhs", 0)))
        except Exception as exc:  # noqa: BLE001
            out["cpu_baseline"] = {"value": None, "error": repr(exc)[:300]}
    return out


def large_cpu_baseline(host_groups, state0, rhs_full, reps=2):
    """The reference's right-hand side at L = 12 on the host: its ``QobjEvo.matmul_data``
    (the compiled CSR matvec of every term, with the term's coefficient) on the same
    generator -- downloaded from the device, because building it with QuTiP's Kronecker
    products takes minutes and tens of GB -- timed over ``reps`` calls and scaled by the
    RHS calls of the whole solve.  The reference's Vern7 vector operations are not
    included, so this bounds the reference's speed from above."""
    qt, _ = host_qutip()
    from qutip.core import data as _data
    n = host_groups[0][0].size - 1
    d = int(round(np.sqrt(n)))
    dims = [[[d], [d]], [[d], [d]]]
    def as_function(c):
        return lambda t: c(t)          # the coefficient's value, evaluated on the host

    elems = []
    for indptr, indices, data, c in host_groups:
        m = _data.CSR((data, indices, indptr.astype(np.int32)), shape=(n, n), copy=False)
        q = qt.Qobj(m, dims=dims, superrep="super", copy=False)
        elems.append(q if c is None else [q, as_function(c)])
    evo = qt.QobjEvo(elems)
    x = _data.Dense(np.asarray(state0, dtype=np.complex128).reshape(-1, 1))
    evo.matmul_data(0.1, x)
    t0 = time.perf_counter()
    for _ in range(reps):
        evo.matmul_data(0.1, x)
    rhs_s = (time.perf_counter() - t0) / reps
    return {"value": 1.0 / (rhs_s * rhs_full), "unit": UNIT, "cores": 1, "kind": "reference",
            "sample": (f"the reference's QobjEvo.matmul_data (compiled single-thread CSR matvec) "
                       f"on the L=12 generator, {rhs_s:.2f} s per call over {reps} calls, scaled "
                       f"by the {rhs_full} RHS calls of the whole solve; Vern7 vector operations "
                       "not included (an upper bound on the reference's solves/s)"),
            "rhs_call_s": rhs_s, "rhs_full": rhs_full}


def run_sde(args):
    """Stochastic solvers through QuTiP's own API: ``ssesolve`` (homodyne) and ``smesolve``
    (with a deterministic collapse operator) of a driven cavity (N = 20), tlist
    linspace(0, 1, 11) at dt = 1e-3 (1000 Platen steps per trajectory).  Three ways with
    the same seeds: the reference's ``platen`` (8 trajectories, serial), the drop-in
    integrator ``gpu_platen`` (8 trajectories, one at a time) and ``map="gpu"`` (256
    trajectories in one launch per output interval); wall time per trajectory and the
    largest difference of the first 8 trajectories' expectation values."""
    qt, _ = host_qutip()
    N = 20
    a = qt.destroy(N)
    H = a.dag() * a + 0.5 * (a + a.dag())
    e_ops = [a.dag() * a, a + a.dag()]
    tl = np.linspace(0, 1, 11)
    out = {}

    def opts(method, **kw):
        return {"method": method, "keep_runs_results": True, "progress_bar": False, **kw}
    cases = {
        "ssesolve": lambda o, nt, s0: qt.ssesolve(
            H, qt.basis(N, 3), tl, [np.sqrt(0.3) * a], e_ops=e_ops, ntraj=nt,
            seeds=list(range(s0, s0 + nt)), options=o),
        "smesolve": lambda o, nt, s0: qt.smesolve(
            H, qt.coherent_dm(N, 1.0), tl, c_ops=[np.sqrt(0.1) * a.dag() * a],
            sc_ops=[np.sqrt(0.2) * a], e_ops=e_ops, ntraj=nt, seeds=list(range(s0, s0 + nt)),
            options=o),
    }
    for name, run in cases.items():
        s0 = 100
        run(opts("gpu_platen"), 1, s0)                   # warm-up (operator build, kernels)
        run(opts("platen", map="gpu"), 4, s0)
        nt, nb = 8, 256
        t0 = time.perf_counter()
        ref = run(opts("platen"), nt, s0)
        t_ref = (time.perf_counter() - t0) / nt
        t0 = time.perf_counter()
        one = run(opts("gpu_platen"), nt, s0)
        t_one = (time.perf_counter() - t0) / nt
        t0 = time.perf_counter()
        bat = run(opts("platen", map="gpu"), nb, s0)
        t_bat = (time.perf_counter() - t0) / nb

        def diff(res):
            return max(float(np.max(np.abs(np.asarray(g)[:nt] - np.asarray(r))))
                       for g, r in zip(res.runs_expect, ref.runs_expect))
        out[name] = {"reference_s_per_traj": t_ref, "gpu_platen_s_per_traj": t_one,
                     "map_gpu_s_per_traj": t_bat, "map_gpu_trajectories": nb,
                     "speedup_map_gpu": t_ref / t_bat, "speedup_gpu_platen": t_ref / t_one,
                     "max_abs_diff_gpu_platen": diff(one), "max_abs_diff_map_gpu": diff(bat),
                     "steps_per_traj": 1000}
        log(f"sde: {name} reference {t_ref * 1e3:.1f} ms per trajectory, gpu_platen "
            f"{t_one * 1e3:.1f} ms, map='gpu' {t_bat * 1e3:.2f} ms ({nb} trajectories); "
            f"max |diff| {max(diff(one), diff(bat)):.1e}")
    out["workload"] = (f"driven cavity N={N}, sc_op sqrt(0.3) a (smesolve: sqrt(0.2) a and "
                       "c_op sqrt(0.1) n), tlist linspace(0,1,11), dt 1e-3, same seeds in every "
                       "arm; the reference single-threaded on the host")
    return out


def run_dense(args):
    """The dense small-dimension bucket (tensor-core Lindblad generator, mixed form) against
    the sparse paths, one request at a time: Jaynes-Cummings mesolve (N = 5..60, d = 2N,
    tlist linspace(0, 20, 101)) and dense random systems (d = 32, 64, 128, t in [0, 2]).
    Sparse paths: the matrix-free kernel (one system, whole GPU) and the batched kernel's
    sparse row loop (the served path, one request in one launch).  Also the generator
    application alone, with the tensor-core rate of the MMAs it issues."""
    import scipy.sparse as sp
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem, check_status
    from qutip_gb300.coefficients import coefficient
    from qutip_gb300.dense import DenseLindbladOperator
    from qutip_gb300.lindblad import LindbladOperator
    from qutip_gb300.solver import ExpectOps, solve_system
    from qutip_gb300.systems import OpenSystem

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return 1e3 * best

    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    tf32_peak = 0.5 * float(peaks.get("bf16_tflops", 1900.0))
    out = {"jc": [], "dense_random": []}
    tl = np.linspace(0.0, 20.0, 101)
    for N in (5, 10, 20, 30, 45, 60):
        s = S.jaynes_cummings(N, kind="me")
        ex = ExpectOps(s.e_ops)
        dop = DenseLindbladOperator.from_hamiltonian(s.h_terms, s.c_ops)
        sop = LindbladOperator.from_hamiltonian(s.h_terms, s.c_ops, dtype="c64")
        ms_dense = timed(lambda: solve_system(s, tl, {"precision": "mixed"}, op=dop, ex=ex))
        ms_mf = timed(lambda: solve_system(s, tl, {"precision": "mixed"}, op=sop, ex=ex))

        def batched():
            bp = BatchProblem("c64")
            bp.add_item(bp.add_system(s.terms, s.e_ops, tl, "me"), s.state0)
            bp.build(group="cta")
            bp.launch()
            check_status(bp.results())
        ms_b = timed(batched)
        out["jc"].append({"N": N, "d": 2 * N, "dense_bucket_ms": ms_dense,
                          "matrix_free_sparse_ms": ms_mf, "batched_sparse_row_loop_ms": ms_b})
        log(f"dense: JC N={N}: tensor cores {ms_dense:.1f} ms, matrix-free {ms_mf:.1f} ms, "
            f"batched row loop {ms_b:.1f} ms")
    rng = np.random.default_rng(11)
    for d in (32, 64, 128):
        def rmat(herm=False):
            m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
            return (m + m.conj().T) / 2 if herm else m
        h_terms = [(sp.csr_matrix(rmat(True) / np.sqrt(d)), None),
                   (sp.csr_matrix(0.3 * rmat(True) / np.sqrt(d)), coefficient("cos(1.1*t)"))]
        c_ops = [sp.csr_matrix(0.1 * rmat() / np.sqrt(d)), sp.csr_matrix(0.05 * rmat() / np.sqrt(d))]
        psi = rng.normal(size=d) + 1j * rng.normal(size=d)
        psi /= np.linalg.norm(psi)
        e_ops = [sp.csr_matrix(rmat(True))]
        s = OpenSystem("dense_random", "me", d, None, np.outer(psi, psi.conj()).reshape(-1, order="F"),
                       e_ops, c_ops, h_terms)
        ex = ExpectOps(e_ops)
        trand = np.linspace(0.0, 2.0, 21)
        dop = DenseLindbladOperator.from_hamiltonian(h_terms, c_ops)
        sop = LindbladOperator.from_hamiltonian(h_terms, c_ops, dtype="c64")
        ms_dense = timed(lambda: solve_system(s, trand, {"precision": "mixed"}, op=dop, ex=ex))
        ms_mf = timed(lambda: solve_system(s, trand, {"precision": "mixed"}, op=sop, ex=ex))
        x = torch.randn(d * d, dtype=torch.complex64, device="cuda")
        y = torch.empty_like(x)
        dop.matvec(0.3, x, y)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 50
        e0.record()
        for _ in range(reps):
            dop.matvec(0.3, x, y)
        e1.record()
        e1.synchronize()
        us = 1e3 * e0.elapsed_time(e1) / reps
        tflops = dop.gemm_flops() / (us * 1e-6) / 1e12
        n_sm = dop.n_ctas
        out["dense_random"].append({"d": d, "dense_bucket_ms": ms_dense, "matrix_free_sparse_ms": ms_mf,
                                    "apply_us": us, "issued_tf32_tflops": tflops, "sms": n_sm,
                                    "frac_of_sms_tf32": tflops / (tf32_peak * n_sm / 152.0)})
        log(f"dense: random d={d}: tensor cores {ms_dense:.1f} ms, matrix-free {ms_mf:.1f} ms, "
            f"apply {us:.1f} us = {tflops:.2f} TFLOP/s issued TF32 on {n_sm} SMs")
    out["note"] = ("one CTA (one SM) per 16 output columns per application; TF32 rate per SM "
                   "taken as half the measured bf16 GEMM rate / 152 SMs")
    return out


def run_matrix_form(args, sysm, tlist, ex, want, hbm_peak):
    """The headline workload through mesolve's matrix form (``matrix_form=True``): the
    Lindblad generator applied to vec(rho) without its superoperator
    (:class:`qutip_gb300.lindblad.LindbladOperator`), mixed precision.  Reported: solves/s,
    the relative error against the reference's FP64 result, the fused stage kernel's time
    and algorithmic bytes, and a short solve at ``--matrix-sites`` spins (default 13,
    67,108,864 vec(rho) entries), a size whose superoperator (about 1.9e9 entries) is
    beyond 32-bit indices."""
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.lindblad import LindbladOperator
    from qutip_gb300.solver import ExpectOps, solve_system
    lop = LindbladOperator.from_hamiltonian(sysm.h_terms, sysm.c_ops, dtype="c64")
    opts = {"precision": "mixed", "matrix_form": True}
    solve_system(sysm, tlist, opts, op=lop, ex=ex)      # warm-up
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = solve_system(sysm, tlist, opts, op=lop, ex=ex)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    rel, absmax, within = rel_err(res.expect, want)
    ms, b, gbs = measure_stage_roofline(lop, sysm.state0, "mixed")
    out = {"workload": f"ising_chain_L{N_SITES} mesolve matrix_form=True, mixed, tlist "
                       f"linspace(0,{T_END:g},{N_OUT})",
           "solves_per_sec": 1.0 / float(np.median(times)),
           "rel_err_vs_reference_fp64": rel, "max_abs_err_vs_reference_fp64": absmax,
           "within_reference_tolerance": within,
           "hermitian_branch": bool(lop.hermitian),
           "stage_kernel": {"kernel": "lindblad_kernel<C64,C128,RK>", "ms": ms,
                            "algorithmic_bytes": int(b), "gbs": gbs, "frac_hbm": gbs / hbm_peak,
                            "bound": "instruction issue (operators L1-resident, state "
                                     "L2-resident; HBM carries only the stage vectors)"},
           "operator_bytes": int(lop.operator_bytes()),
           "solver_stats": {k: res.stats[k] for k in ("steps", "rejected", "rhs")}}
    del lop
    L = args.matrix_sites
    if L:
        s = S.ising_chain(L, build_terms=False)
        tl = np.linspace(0.0, 0.05, 3)
        t0 = time.perf_counter()
        big = LindbladOperator.from_hamiltonian(s.h_terms, s.c_ops, dtype="c64")
        exb = ExpectOps(s.e_ops)
        torch.cuda.synchronize()
        build_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        rb = solve_system(s, tl, opts, op=big, ex=exb)
        torch.cuda.synchronize()
        run_s = time.perf_counter() - t0
        bms, bb, bgbs = measure_stage_roofline(big, s.state0, "mixed", reps=2)
        out["large"] = {"workload": f"ising_chain_L{L} mesolve matrix_form=True, mixed, "
                                    "tlist linspace(0,0.05,3)",
                        "vec_rho_entries": big.n_rows, "build_s": build_s, "solve_s": run_s,
                        "rhs_calls": int(rb.stats["rhs"]), "stage_ms": bms,
                        "stage_gbs": bgbs, "device_gb": torch.cuda.max_memory_allocated() / 1e9,
                        "sz0_at_t_end": float(np.real(rb.expect[0][-1]))}
        del big, exb
        torch.cuda.empty_cache()
    return out


def mesolve_opts(precision):
    return {"method": "gpu_vern7", "atol": 1e-8, "rtol": 1e-6, "progress_bar": False,
            "precision": precision}


def operator_upload_bytes(rhs, rho0) -> int:
    """Host-to-device bytes of one mesolve call: each Liouvillian element's CSR arrays as
    stored (32-bit indices and row pointers, complex128 values) and the initial state."""
    import scipy.sparse as sp
    b = 0
    for el in rhs.to_list():
        q = el[0] if isinstance(el, list) else el
        m = sp.csr_matrix(q.data.as_scipy())
        b += m.data.nbytes + m.indices.nbytes + m.indptr.nbytes
    n = rho0.shape[0]
    return b + 16 * n * n


def run_ours(args, dist):
    import torch
    from qutip_gb300 import _lib
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import ExpectOps

    dist.init()
    hbm_peak, peak_src = hbm_peak_gbs()
    qt, RW = host_qutip()
    from qutip_gb300 import qutip_plugin  # noqa: F401  (registers gpu_vern7, GpuDense)
    H, c_ops, rho0, e_ops = RW.ising_qobjs(N_SITES)
    tlist = np.linspace(0.0, T_END, N_OUT)
    want = np.load(GOLDEN)["expect"]             # the reference's FP64 result

    log("building the complex128 solver (QuTiP's Liouvillian, device operator)")
    t0 = time.perf_counter()
    solver = qt.MESolver(H, c_ops, options=mesolve_opts("double"))
    build_s = time.perf_counter() - t0
    ig = solver._integrator
    op = ig._op
    rho_dev = rho0.to("gpu")

    def solve(s=solver):
        return s.run(rho_dev, tlist, e_ops=e_ops)

    log(f"warm-up ({op.launch_desc()})")
    for _ in range(args.warmup):
        res = solve()
    dist.barrier()
    clocks = ClockSampler(dist.local)
    clocks.start()
    n0 = _lib.LAUNCHES[0]
    rhs0 = ig._ode.stats["rhs"]
    steps0 = ig._ode.stats["steps"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        res = solve()
    e1.record()
    dist.barrier()
    ms = e0.elapsed_time(e1)
    launches = _lib.LAUNCHES[0] - n0
    rhs_full = (ig._ode.stats["rhs"] - rhs0) // args.steps
    steps_full = (ig._ode.stats["steps"] - steps0) // args.steps
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = args.steps * dist.world / (ms_max / 1000.0)
    rel, absmax, within = rel_err(res.expect, want)
    log(f"headline {value:.3f} solves/s complex128, rel err {rel:.2e} vs the reference")

    # end to end: the whole user call from host Qobjs, every step
    n_e2e = max(1, min(args.steps, args.e2e_reps))
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        r_e2e = qt.mesolve(H, rho0, tlist, c_ops, e_ops=e_ops, options=mesolve_opts("double"))
    dist.barrier()
    e2e = n_e2e * dist.world / dist.max(time.perf_counter() - t0)
    rel_e2e, _, within_e2e = rel_err(r_e2e.expect, want)
    h2d = operator_upload_bytes(solver.rhs, rho0)
    d2h = N_OUT * (32 * len(e_ops) + 16) + 8 * steps_full
    # where the end-to-end time goes: QuTiP's host Liouvillian, the device build
    t0 = time.perf_counter()
    ref_solver = qt.MESolver(H, c_ops, options={"method": "vern7"})
    liou_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    qutip_plugin.IntegratorGpuVern7(ref_solver, mesolve_opts("double"))
    torch.cuda.synchronize()
    dev_build_s = time.perf_counter() - t0
    del ref_solver
    log(f"e2e {e2e:.3f} solves/s (Liouvillian {liou_s:.2f} s, device build {dev_build_s:.2f} s)")

    # the mixed form through the same API
    solver_m = qt.MESolver(H, c_ops, options=mesolve_opts("mixed"))
    solve(solver_m)
    nm = max(2, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(nm):
        res_m = solve(solver_m)
    torch.cuda.synchronize()
    mixed_v = nm / (time.perf_counter() - t0)
    rel_m, abs_m, within_m = rel_err(res_m.expect, want)
    op64 = solver_m._integrator._op

    log("roofline measurements")
    state0 = rho0.full().reshape(-1, order="F")
    fmas = []
    stage_ms, stage_b, stage_gbs = measure_stage_roofline(op, state0, "double", fmas=fmas)
    fp64_tflops = 2 * fmas[0] / (stage_ms * 1e-3) / 1e12
    spmv_ms, spmv_b, spmv_gbs = measure_spmv(op)
    st64_ms, st64_b, st64_gbs = measure_stage_roofline(op64, state0, "mixed")
    spmv64_ms, spmv64_b, spmv64_gbs = measure_spmv(op64)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "accuracy": {"rel_err_vs_reference_fp64": rel, "max_abs_err": absmax,
                     "within_reference_tolerance": within,
                     "reference": "the reference QuTiP's own vern7 mesolve of the same inputs "
                                  "(tests/golden/ising_L10_expect.npz); rel = max over e_ops of "
                                  "max_t |d| / max_t |want|; tolerance atol 1e-8 + rtol 1e-6 |want|"},
        "data": "synthetic (seeded h_i ~ U[0.5,1.5], default_rng(1234))",
        "config": CONFIG,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "call": "qutip.mesolve(H, rho0, tlist, c_ops, e_ops, options={'method': "
                        "'gpu_vern7'}) from host Qobjs",
                "reps": n_e2e, "rel_err_vs_reference_fp64": rel_e2e,
                "within_reference_tolerance": within_e2e,
                "breakdown_s": {"qutip_liouvillian_host": liou_s, "device_build": dev_build_s,
                                "solve": 1.0 / value}},
        "gpu_launches": int(launches),
        "solver_stats": {"steps": int(steps_full), "rhs": int(rhs_full),
                         "build_s": build_s, "launch": op.launch_desc()},
        "roofline": {"bound": "hbm", "achieved": stage_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": stage_gbs / hbm_peak, "traffic": profiled_traffic(TRAFFIC_PROFILE),
                     "traffic_source": f"{TRAFFIC_PROFILE} (ncu dram__bytes_read.sum + "
                                       "dram__bytes_write.sum per launch)",
                     "kernel": (f"spmv_dict_kernel<C128,C128,RK,{op.code_bytes}> (fused Vern7 "
                                "stage, complex128, dictionary-coded operator)"
                                if op.fmt == "dict" else
                                "spmv_sliced_kernel<C128,C128,RK> (fused Vern7 stage)"),
                     "bytes_per_launch": stage_b, "ms_per_launch": stage_ms,
                     "peak_source": f"{peak_src} hbm_gbs (of {peak_src})"},
        "roofline_fp64": {"bound": "fp64", "achieved": fp64_tflops, "unit": "TFLOP/s",
                          "peak": FP64_PEAK_TFLOPS, "frac": fp64_tflops / FP64_PEAK_TFLOPS,
                          "fmas_per_launch": fmas[0], "ms_per_launch": stage_ms,
                          "peak_source": "nominal: 2 FP64 FMAs per clock per SM x 152 SMs x "
                                         "2.07 GHz (no measured FP64 peak)",
                          "note": "the complex128 stage kernel is bound by the FP64 pipe "
                                  "(sm__pipe_fp64_cycles_active 85 % of active cycles, "
                                  f"{TRAFFIC_PROFILE}); its HBM fraction is the roofline key"},
        "spmv": {"c128_gbs": spmv_gbs, "c128_ms": spmv_ms, "c128_bytes": spmv_b,
                 "frac_c128": spmv_gbs / hbm_peak, "c64_gbs": spmv64_gbs, "c64_ms": spmv64_ms,
                 "c64_bytes": spmv64_b, "frac_c64": spmv64_gbs / hbm_peak},
        "mixed": {"value": mixed_v, "unit": UNIT, "dtype": "c64 stages / f64 state and step control",
                  "rel_err_vs_reference_fp64": rel_m, "max_abs_err": abs_m,
                  "within_reference_tolerance": within_m, "bound_rel": 1e-6,
                  "stage_kernel": {"kernel": f"spmv_dict_kernel<C64,C128,RK,{op64.code_bytes}>"
                                   if op64.fmt == "dict" else op64.launch_desc(),
                                   "ms": st64_ms, "bytes": st64_b, "gbs": st64_gbs,
                                   "frac_hbm": st64_gbs / hbm_peak}},
        "clocks": clk,
    }
    sections = set() if args.quick else set(args.sections.split(","))
    # stdout carries the one JSON line: anything a library prints goes to stderr meanwhile
    _stdout, sys.stdout = sys.stdout, sys.stderr
    if dist.rank == 0 and "served" in sections:
        log("served stream")
        out["served"] = run_served(args)
    if dist.rank == 0 and "mc" in sections:
        log("batched mcsolve")
        out["mc_batched"] = run_mc_batch(args)
    if dist.rank == 0 and "dense" in sections:
        log("dense small-dimension bucket")
        out["dense_bucket"] = run_dense(args)
    if dist.rank == 0 and "sde" in sections:
        log("stochastic solvers")
        out["sde"] = run_sde(args)
    if dist.rank == 0 and "matrix" in sections:
        log("matrix form")
        sysm = S.ising_chain(N_SITES, build_terms=False)
        out["matrix_form"] = run_matrix_form(args, sysm, tlist, ExpectOps(sysm.e_ops), want,
                                             hbm_peak)
    if dist.rank == 0 and "large" in sections and args.large_sites:
        log(f"large: Ising L={args.large_sites}")
        out["large"] = run_large(args)
    if dist.rank == 0 and not args.no_cpu_baseline:
        log("CPU baseline")
        try:
            k = max(1, min(args.cpu_sample, N_OUT - 1))
            ig._ode.stats["rhs"] = 0
            solver.run(rho_dev, tlist[:k + 1], e_ops=e_ops)
            rhs_sample = int(ig._ode.stats["rhs"])
            out["cpu_baseline"] = cpu_baseline(k, rhs_sample, int(rhs_full))
        except Exception as exc:  # noqa: BLE001
            out["cpu_baseline"] = {"value": None, "error": repr(exc)[:300]}
    sys.stdout = _stdout
    if dist.rank == 0:
        print(json.dumps(out))
    dist.close()


def run_profile_case(args):
    """Case for ncu captures: the headline fused stage kernel on the Ising chain with
    ``--profile-sites`` spins (default 10: 1,048,576 rows, 0.32 GB complex64 operator,
    larger than L2; about 1.5 GB on the device).  First-step estimate (2 matvecs),
    then two Vern7 steps of 10 fused stage launches each, without autotuning."""
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.vern7 import GpuVern7
    torch.cuda.set_device(0)
    s = S.ising_chain(args.profile_sites)
    op = DeviceOperator(s.terms, dtype=args.profile_dtype, fmt=args.profile_fmt)
    ig = GpuVern7(op, precision="mixed" if args.profile_dtype == "c64" else "double")
    ig.set_initial_value(torch.from_numpy(s.state0).cuda(), 0.0)
    for _ in range(2):
        ig.integrate(ig.t_front + 0.05, step=True)
    torch.cuda.synchronize()
    print(f"{args.profile_dtype}: launch {op.launch_desc()}, {op.spmv_bytes() / 1e9:.3f} GB per matvec")


def run_profile_matrix(args):
    """ncu case for the matrix-free Lindblad stage kernel: the Ising chain with
    ``--profile-sites`` spins (default 10: vec(rho) of 1,048,576 entries, stage vectors
    larger than L2 taken together), mixed form; first-step estimate (2 applications),
    then two Vern7 steps of 10 fused stage launches each."""
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.lindblad import LindbladOperator
    from qutip_gb300.vern7 import GpuVern7
    torch.cuda.set_device(0)
    s = S.ising_chain(args.profile_sites, build_terms=False)
    op = LindbladOperator.from_hamiltonian(s.h_terms, s.c_ops, dtype="c64")
    op.hermitian = args.profile_branch == "hermitian"
    ig = GpuVern7(op, precision="mixed")
    ig.set_initial_value(torch.from_numpy(s.state0).cuda(), 0.0)
    for _ in range(2):
        ig.integrate(ig.t_front + 0.05, step=True)
    torch.cuda.synchronize()
    print(f"matrix form: {op.launch_desc()}, {op.operator_bytes() / 1e6:.1f} MB generator")


def run_profile_dense(args):
    """ncu case for the dense tensor-core Lindblad kernel: a dense random system of
    dimension ``--profile-sites`` (default 10 is raised to 128 here: d = 128), ten
    applications of the generator."""
    import scipy.sparse as sp
    import torch
    from qutip_gb300.dense import DenseLindbladOperator
    torch.cuda.set_device(0)
    d = 128
    rng = np.random.default_rng(3)
    m = lambda: rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))  # noqa: E731
    h = m()
    op = DenseLindbladOperator.from_hamiltonian([(sp.csr_matrix((h + h.conj().T) / 2), None)],
                                                [sp.csr_matrix(0.1 * m()), sp.csr_matrix(0.1 * m())])
    x = torch.randn(d * d, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    for _ in range(10):
        op.matvec(0.1, x, y)
    torch.cuda.synchronize()
    print(f"dense: {op.launch_desc()}, {op.gemm_flops() / 1e6:.1f} MFLOP issued per application")


def run_profile_sde(args):
    """ncu case for the stochastic Platen kernel: the smesolve system of the ``sde`` section
    (driven cavity N = 20, vec(rho) of 400 entries), 10 steps for 1, 8, 64 and 256
    trajectories, each shape launched twice (the second one timed with CUDA events)."""
    import torch
    qt, _ = host_qutip()
    from qutip_gb300 import qutip_plugin as P
    torch.cuda.set_device(0)
    N = 20
    a = qt.destroy(N)
    H = a.dag() * a + 0.5 * (a + a.dag())
    sol = qt.SMESolver(H, [np.sqrt(0.2) * a], heterodyne=False,
                       c_ops=[np.sqrt(0.1) * a.dag() * a], options={"method": "platen"})
    op = P.sde_operator(sol.rhs)
    rho = qt.coherent_dm(N, 1.0).full().reshape(-1, order="F")
    steps = 10
    for nt in (1, 8, 64, 256):
        states = torch.from_numpy(np.tile(rho, (nt, 1))).cuda()
        dW = torch.from_numpy(np.random.default_rng(1).normal(0, 0.03, size=(nt, steps, 1))).cuda()
        op.advance(states, dW, steps, 1e-3)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        op.advance(states, dW, steps, 1e-3)
        e1.record()
        e1.synchronize()
        print(f"sde: {nt} trajectories, {1e3 * e0.elapsed_time(e1) / steps:.1f} us per step")


def run_profile_batch(args):
    """ncu case for the batched trajectory kernel: ``--profile-ntraj`` Bose-Hubbard
    trajectories (default 256) over t in [0, ``--profile-tend``] (default 5, 10
    outputs per unit time), mixed form, default launch shape."""
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import mcsolve_batch
    torch.cuda.set_device(0)
    s = S.bose_hubbard_trimer(8)
    te = args.profile_tend
    r = mcsolve_batch(s, np.linspace(0.0, te, int(round(10 * te)) + 1), args.profile_ntraj,
                      seeds=5, precision="mixed", group=args.profile_group)
    torch.cuda.synchronize()
    print(f"batch: {len(r.col_times)} trajectories, {sum(len(c) for c in r.col_times)} jumps")


def run_profile_served_large(args):
    """ncu case for the largest served requests: one Jaynes-Cummings mesolve item
    (N = 57, vec(rho) of 12,996 entries, tlist linspace(0, 20, 101)) in the batched kernel
    with the launch shape ``--profile-group`` (the serving policy's ``cluster``), two
    launches (warm-up, then the captured one)."""
    import torch
    from qutip_gb300 import systems as S
    from qutip_gb300.batched import BatchProblem, check_status
    torch.cuda.set_device(0)
    s = S.jaynes_cummings(57, kind="me")
    tl = np.linspace(0.0, 20.0, 101)
    flag = torch.zeros(1, dtype=torch.int32).pin_memory()
    for _ in range(2):
        bp = BatchProblem("c64")
        bp.add_item(bp.add_system(s.terms, s.e_ops, tl, "me"), s.state0)
        bp.build(group=args.profile_group)
        bp.set_cancel(flag)        # as served launches carry it
        bp.launch()
        res = bp.results()
        check_status(res)
    torch.cuda.synchronize()
    print(f"served-large: {res[0]['steps']} steps, {res[0]['rhs']} stage evaluations")


def main():
    args = parse()
    if args.profile == "stage":
        run_profile_case(args)
        return
    if args.profile == "batch":
        run_profile_batch(args)
        return
    if args.profile == "matrix":
        run_profile_matrix(args)
        return
    if args.profile == "dense":
        run_profile_dense(args)
        return
    if args.profile == "sde":
        run_profile_sde(args)
        return
    if args.profile == "served-large":
        run_profile_served_large(args)
        return
    dist = Dist(args.gpus)
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
