#!/usr/bin/env python
"""Benchmark: time-dependent Lindblad solve of the dissipative transverse-field
Ising chain, L = 10 spins (Hilbert dim 1024, Liouvillian dim 1,048,576,
24.6 M stored entries in two coefficient groups), Vern7 atol 1e-8 / rtol 1e-6,
tlist = linspace(0, 10, 101), 10 e_ops.

One step = one complete solve in the mixed form (complex64 generator and stages
with FP32 accumulation; FP64 state, step control and expectation values), whose
error against the complex128 solve is reported with it.  ``value`` is solves/s
with the operator already resident in HBM (0.3 GB, larger than L2, so no flush
is needed); ``e2e`` repeats the solve through the host API with the operator and
initial state copied from pinned host memory every step and the expectation
values read back.  ``roofline`` is that of the fused Vern7 stage kernel (sliced
ELLPACK matvec + stage combination), timed with CUDA events on its stream.
Also reported: the complex128 form, the served mixed-size Jaynes-Cummings stream
(continuous batching vs the plain complex128 per-request drop-in) and the
batched 4096-trajectory Bose-Hubbard mcsolve.

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
          "l2": "per-step working set larger than L2 (129 MB): operator 0.06 GB (dictionary-coded; 0.3 GB uncompressed) + 16 complex64 stage vectors 0.13 GB + complex128 state 0.03 GB; no flush"}


def log(msg):
    """Progress to stderr (the JSON result line goes to stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=float, default=0.3,
                    help="simulated time of the CPU-baseline sample (of 10.0)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="headline workload only")
    ap.add_argument("--sections", default="served,mc,matrix,large",
                    help="extra sections after the headline (comma list of served, mc, "
                         "matrix, large)")
    ap.add_argument("--matrix-sites", type=int, default=13,
                    help="spins of the short matrix-form solve in the matrix section (0: skip)")
    ap.add_argument("--served-jobs", type=int, default=10000)
    ap.add_argument("--served-ntraj", type=int, default=100)
    ap.add_argument("--served-plain-sample", type=int, default=60)
    ap.add_argument("--mc-ntraj", type=int, default=4096)
    ap.add_argument("--large-sites", type=int, default=12,
                    help="Ising chain length of the large mixed-precision section (0: skip)")
    ap.add_argument("--profile", default=None, choices=["stage", "batch", "matrix"],
                    help="run the ncu profiling case only (fused stage kernel, untuned); "
                         "prints nothing to parse")
    ap.add_argument("--profile-sites", type=int, default=10)
    ap.add_argument("--profile-fmt", default="auto", choices=["auto", "sliced", "dict", "csr"],
                    help="operator storage of the stage profiling case")
    ap.add_argument("--profile-ntraj", type=int, default=256)
    ap.add_argument("--profile-tend", type=float, default=5.0)
    ap.add_argument("--profile-group", default="auto",
                    choices=["auto", "warp", "cta", "cta128", "cluster"])
    return ap.parse_args()


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
def cpu_baseline(sample_t: float):
    """Reference vern7 mesolve (compiled from source into oracle/_ref) on the host,
    over the first ``sample_t`` of simulated time, scaled to solves/s."""
    from oracle import ref_workloads as RW
    cores = os.cpu_count() or 1
    if RW.reference_available():
        secs, frac = RW.reference_mesolve_sample(N_SITES, T_END, N_OUT, sample_t)
        kind = "reference"
        what = "QuTiP reference (oracle/_ref) mesolve vern7, CSR complex128, 1-thread SpMV"
    else:
        from qutip_gb300 import systems as S
        s = S.ising_chain(N_SITES)
        secs, frac = RW.port_mesolve_sample(s.terms, s.state0, s.e_ops, T_END, N_OUT, sample_t)
        kind = "port"
        what = "oracle numpy/scipy restatement of vern7 mesolve, complex128"
    value = frac / secs
    return {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"{what}; integrated t in [0,{sample_t:g}] of [0,{T_END:g}] "
                      f"({secs:.2f} s), scaled by simulated time; BLAS threads = host cores"}


def run_reference(args, dist):
    if dist.rank != 0:
        return
    steps = []
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(args.cpu_sample)
        if i >= args.warmup:
            steps.append(b)
    vals = [s["value"] for s in steps]
    v = float(np.median(vals))
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
           "data": "synthetic (seeded h_i ~ U[0.5,1.5])", "config": CONFIG,
           "cpu_baseline": {**steps[-1], "value": v},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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


TRAFFIC_PROFILE = "profiles/spmv_dict_ising_L10_stage.md"
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


def measure_stage_roofline(op, sysm, precision, reps=20):
    """Average duration and algorithmic GB/s of the fused stage kernel (events on its stream)."""
    import ctypes as C
    import torch
    from qutip_gb300 import _lib
    from qutip_gb300.operator import stream_ptr
    from qutip_gb300.vern7 import GpuVern7
    ig = GpuVern7(op, precision=precision)
    ig.set_initial_value(torch.from_numpy(sysm.state0).cuda(), 0.0)
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
                                     percentiles, solve_plain)
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
    plain_low = percentiles(fifo_latencies([sp.arrival for sp in specs_l],
                                           [service[i % k] for i in range(m)]))
    log(f"served: at {low_rate:.1f} req/s served {lat_low}, plain {plain_low}")
    slow = sorted(jobs_l, key=lambda j: -(j.latency or 0))[:6]
    log("served: slowest at that rate: " + "; ".join(
        f"{j.spec.kind} N={j.spec.n_cav} {1e3 * j.latency:.0f} ms launch={j.extra.get('launch')}"
        for j in slow))
    # error of the served mixed form vs the plain complex128 solve on the sample's mesolve jobs
    err = 0.0
    for j in jobs[:k]:
        if j.spec.kind == "me":
            ref = solve_plain(j, "double")
            err = max(err, max(float(np.max(np.abs(np.real(a) - np.real(b))))
                               for a, b in zip(j.result, ref)))
    n_me = sum(sp.kind == "me" for sp in specs)
    return {
        "workload": f"{n} Jaynes-Cummings jobs, N~U{{5..60}}, {n_me} mesolve / {n - n_me} mcsolve "
                    f"(ntraj={args.served_ntraj}), tlist linspace(0,20,101), seed 2026",
        "served_mixed": {"solves_per_sec": thr, "wall_s": wall, "launches": srv.stats["launches"],
                         "latency_at_rate": {**lat, "rate_per_s": rate, "wall_s": wall_r,
                                             "max_concurrent_launches": srv_r.stats["max_concurrent"]}},
        "plain_c128": {"solves_per_sec": plain_thr, "service_sample_jobs": k,
                       "latency_at_rate": {**plain_lat, "rate_per_s": rate,
                                           "method": "measured service times, FIFO queue on the "
                                                     "same arrivals"}},
        "speedup_solves_per_sec": thr / plain_thr,
        "speedup_p99": plain_lat["p99_ms"] / lat["p99_ms"],
        "at_plain_sustainable_rate": {"rate_per_s": low_rate, "requests": m,
                                      "served_mixed": lat_low, "plain_c128": plain_low,
                                      "speedup_p99": plain_low["p99_ms"] / lat_low["p99_ms"]},
        "max_abs_err_vs_c128_expect": err,
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
    del groups
    torch.cuda.empty_cache()
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
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
    spmv_ms, spmv_b, spmv_gbs = measure_spmv(op64, reps=10)
    stage_ms, stage_b, stage_gbs = measure_stage_roofline(op64, s, "mixed", reps=3)
    peak, _ = hbm_peak_gbs()
    out = {"workload": f"ising_chain_L{L}_mesolve_vern7 mixed, tlist linspace(0,5,51)",
           "liouvillian_rows": op64.n_rows, "entries": int(op64.nnz),
           "device_assembly_s": build_s, "solves_per_sec": 1.0 / float(np.median(times)),
           "s_per_solve": float(np.median(times)), "rhs_calls": int(r64.stats.get("rhs", 0)),
           "max_abs_err_vs_fp64_gpu": err,
           "spmv_c64": {"gbs": spmv_gbs, "ms": spmv_ms, "bytes": int(spmv_b), "frac": spmv_gbs / peak},
           "stage_c64": {"gbs": stage_gbs, "ms": stage_ms, "bytes": int(stage_b),
                         "frac": stage_gbs / peak},
           "cpu_baseline": None,
           "cpu_baseline_note": "not run at this size: the reference's host Liouvillian "
                                "construction alone takes minutes (the CPU baseline of the "
                                "headline line is at L = 10)"}
    del op64, op128
    torch.cuda.empty_cache()
    return out


def run_matrix_form(args, sysm, tlist, ex, ref, hbm_peak):
    """The headline workload through mesolve's matrix form (``matrix_form=True``): the
    Lindblad generator applied to vec(rho) without its superoperator
    (:class:`qutip_gb300.lindblad.LindbladOperator`), mixed precision.  Reported: solves/s,
    the error against the complex128 superoperator solve, the fused stage kernel's time
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
    err = max(float(np.max(np.abs(res.expect[k] - ref.expect[k]))) for k in range(len(ex.ops)))
    ms, b, gbs = measure_stage_roofline(lop, sysm, "mixed")
    out = {"workload": f"ising_chain_L{N_SITES} mesolve matrix_form=True, mixed, tlist "
                       f"linspace(0,{T_END:g},{N_OUT})",
           "solves_per_sec": 1.0 / float(np.median(times)),
           "max_abs_err_vs_fp64_superoperator": err,
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
        bms, bb, bgbs = measure_stage_roofline(big, s, "mixed", reps=2)
        out["large"] = {"workload": f"ising_chain_L{L} mesolve matrix_form=True, mixed, "
                                    "tlist linspace(0,0.05,3)",
                        "vec_rho_entries": big.n_rows, "build_s": build_s, "solve_s": run_s,
                        "rhs_calls": int(rb.stats["rhs"]), "stage_ms": bms,
                        "stage_gbs": bgbs, "device_gb": torch.cuda.max_memory_allocated() / 1e9,
                        "sz0_at_t_end": float(np.real(rb.expect[0][-1]))}
        del big, exb
        torch.cuda.empty_cache()
    return out


def run_ours(args, dist):
    import torch
    from qutip_gb300 import _lib
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.solver import ExpectOps, solve_system

    dist.init()
    hbm_peak, peak_src = hbm_peak_gbs()

    log("building the Ising L=10 Liouvillian")
    sysm = S.ising_chain(N_SITES)
    tlist = np.linspace(0.0, T_END, N_OUT)
    op64 = DeviceOperator(sysm.terms, dtype="c64")
    op64.tune()
    op = DeviceOperator(sysm.terms, dtype="c128")
    op.tune()
    ex = ExpectOps(sysm.e_ops)

    def solve(o=op64, prec="mixed"):
        return solve_system(sysm, tlist, {"precision": prec}, op=o, ex=ex)

    log("FP64 reference solve")
    ref = solve(op, "double")  # FP64 result the mixed form is checked against
    log("warm-up")
    for _ in range(args.warmup):
        solve()
    dist.barrier()
    clocks = ClockSampler(dist.local)
    clocks.start()
    n0 = _lib.LAUNCHES[0]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        res = solve()
    e1.record()
    dist.barrier()
    ms = e0.elapsed_time(e1)
    launches = _lib.LAUNCHES[0] - n0
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = args.steps * dist.world / (ms_max / 1000.0)
    err_m = max(float(np.max(np.abs(res.expect[k] - ref.expect[k]))) for k in range(N_SITES))

    log(f"headline {value:.3f} solves/s; end-to-end")
    # end to end: operator + initial state from pinned host memory every step, expect read back
    host = op64.host_copy()
    h2d = sum(h.numel() * h.element_size() for h in host) + sysm.state0.nbytes
    d2h = N_OUT * 2 * (len(sysm.e_ops) + 1) * 8
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        op64.upload(host)
        solve()
    dist.barrier()
    e2e = args.steps * dist.world / dist.max(time.perf_counter() - t0)

    # complex128 form (the plain drop-in precision)
    nd = max(1, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(nd):
        solve(op, "double")
    torch.cuda.synchronize()
    double_v = nd / (time.perf_counter() - t0)

    log("roofline measurements")
    stage_ms, stage_b, stage_gbs = measure_stage_roofline(op64, sysm, "mixed")
    # the same stage with the uncompressed sliced operator (12 bytes per entry)
    op_sl = DeviceOperator(sysm.terms, dtype="c64", fmt="sliced")
    sl_ms, sl_b, sl_gbs = measure_stage_roofline(op_sl, sysm, "mixed")
    del op_sl
    stage128_ms, stage128_b, stage128_gbs = measure_stage_roofline(op, sysm, "double")
    spmv_ms, spmv_b, spmv_gbs = measure_spmv(op)
    spmv64_ms, spmv64_b, spmv64_gbs = measure_spmv(op64)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 stages / f64 state (mixed)",
        "accuracy": {"max_abs_err_vs_fp64_expect": err_m, "bound": 1e-6,
                     "fp64_reference": "the same solve in complex128 on the GPU, which matches "
                                       "the reference QuTiP within atol 1e-8 / rtol 1e-6"},
        "data": "synthetic (seeded h_i ~ U[0.5,1.5], default_rng(1234))",
        "config": {**CONFIG, "parallelism": "replicas" if dist.world > 1 else "single",
                   "spmv_launch": op64.launch_desc()},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": stage_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": stage_gbs / hbm_peak, "traffic": profiled_traffic(),
                     "traffic_source": f"{TRAFFIC_PROFILE} (ncu dram__bytes_read.sum + "
                                       "dram__bytes_write.sum, mean over the 10 stage launches "
                                       "of a step, same operator)",
                     "kernel": (f"spmv_dict_kernel<C64,C128,RK,{op64.code_bytes}> (fused Vern7 "
                                "stage, mixed, dictionary-coded operator)" if op64.fmt == "dict"
                                else "spmv_sliced_kernel<C64,C128,RK> (fused Vern7 stage, mixed)"),
                     "bytes_per_launch": stage_b, "ms_per_launch": stage_ms,
                     "peak_source": f"{peak_src} hbm_gbs (of {peak_src})",
                     "note": "the dictionary codes cut the operator stream from 12 to 2 bytes "
                             "per entry, so HBM no longer bounds this kernel: shared-memory "
                             "table lookups and L2 gathers of x do; see roofline_uncompressed "
                             "for the same stage with the 12-byte entries"},
        "roofline_uncompressed": {"kernel": "spmv_sliced_kernel<C64,C128,RK>",
                                  "bound": "hbm", "achieved": sl_gbs, "peak": hbm_peak,
                                  "unit": "GB/s", "frac": sl_gbs / hbm_peak,
                                  "bytes_per_launch": sl_b, "ms_per_launch": sl_ms,
                                  "traffic": profiled_traffic(SLICED_PROFILE),
                                  "traffic_source": SLICED_PROFILE},
        "double_precision": {"value": double_v, "unit": UNIT,
                             "stage_kernel_gbs": stage128_gbs, "stage_kernel_ms": stage128_ms,
                             "bound": "FP64 throughput (about 4 DFMA per stored entry)"},
        "spmv": {"c64_gbs": spmv64_gbs, "c64_ms": spmv64_ms, "c64_bytes": spmv64_b,
                 "frac_c64": spmv64_gbs / hbm_peak, "c128_gbs": spmv_gbs, "c128_ms": spmv_ms,
                 "c128_bytes": spmv_b, "frac_c128": spmv_gbs / hbm_peak},
        "solver_stats": {k: res.stats[k] for k in ("steps", "rejected", "rhs")},
        "clocks": clk,
    }
    sections = set() if args.quick else set(args.sections.split(","))
    if dist.rank == 0 and "served" in sections:
        log("served stream")
        out["served"] = run_served(args)
    if dist.rank == 0 and "mc" in sections:
        log("batched mcsolve")
        out["mc_batched"] = run_mc_batch(args)
    if dist.rank == 0 and "matrix" in sections:
        log("matrix form")
        out["matrix_form"] = run_matrix_form(args, sysm, tlist, ex, ref, hbm_peak)
    if dist.rank == 0 and "large" in sections and args.large_sites:
        log(f"large: Ising L={args.large_sites}")
        out["large"] = run_large(args)
    if dist.rank == 0 and not args.no_cpu_baseline:
        log("CPU baseline")
        try:
            out["cpu_baseline"] = cpu_baseline(args.cpu_sample)
        except Exception as exc:  # noqa: BLE001
            out["cpu_baseline"] = {"value": None, "error": repr(exc)[:300]}
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
    op = DeviceOperator(s.terms, dtype="c64", fmt=args.profile_fmt)
    ig = GpuVern7(op, precision="mixed")
    ig.set_initial_value(torch.from_numpy(s.state0).cuda(), 0.0)
    for _ in range(2):
        ig.integrate(ig.t_front + 0.05, step=True)
    torch.cuda.synchronize()
    print(f"c64 mixed: launch {op.launch_desc()}, {op.spmv_bytes() / 1e9:.3f} GB per matvec")


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
    ig = GpuVern7(op, precision="mixed")
    ig.set_initial_value(torch.from_numpy(s.state0).cuda(), 0.0)
    for _ in range(2):
        ig.integrate(ig.t_front + 0.05, step=True)
    torch.cuda.synchronize()
    print(f"matrix form: {op.launch_desc()}, {op.operator_bytes() / 1e6:.1f} MB generator")


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
    dist = Dist(args.gpus)
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
