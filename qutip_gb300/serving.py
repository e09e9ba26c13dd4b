"""Continuous-batching server for mixed-size mesolve / mcsolve request streams.

The reference serves one request at a time: each ``mesolve`` call builds its
solver and integrates on the host (qutip/solver/mesolve.py:24-166), and each
``mcsolve`` maps its trajectories over a serial loop or a process pool
(qutip/solver/multitraj.py:169-258, qutip/solver/parallel.py:49-338).

:class:`Server` instead keeps work resident on the GPU and overlaps requests:

* arriving jobs wait in buckets by state length (the batched kernel's workspace
  slot is sized by the largest state of a launch, so similar sizes share a launch);
* a bucket is admitted as one persistent ``qg_batch_vern7`` launch on its own CUDA
  stream as soon as a stream is free and the launch's HBM footprint (operator
  pools, states, outputs and workspace) fits the budget; jobs arriving while
  earlier launches run are admitted into new launches that overlap them;
* completion is taken from a CUDA event per launch; latency = completion - arrival.

Every job's result is the one it gets alone (items never interact), which the
tests check bitwise.
"""
from __future__ import annotations

import gc
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .batched import BatchProblem, check_status
from .systems import OpenSystem, jaynes_cummings

__all__ = ["JobSpec", "Job", "jc_request_stream", "build_job", "Server", "percentiles",
           "fifo_latencies", "solve_plain"]

BUCKETS = (128, 512, 2048, 8192, 1 << 30)


@dataclass
class JobSpec:
    """One request of the served Jaynes-Cummings stream."""
    id: int
    kind: str          # "me" or "mc"
    n_cav: int
    g: float
    kappa: float
    gamma: float
    arrival: float     # seconds after the stream starts
    ntraj: int = 0
    seed: int = 0


@dataclass
class Job:
    spec: JobSpec
    system: OpenSystem
    tlist: np.ndarray
    state_len: int
    result: list | None = None
    done: float | None = None
    status: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def latency(self):
        return None if self.done is None else self.done - self.spec.arrival


def jc_request_stream(n_jobs=10_000, rate=2000.0, mc_fraction=0.3, ntraj=100, seed=2026,
                      n_min=5, n_max=60):
    """Synthetic stream: cavity cutoff N ~ U{5..60}, g ~ U[0.01,0.1]*2pi,
    kappa, gamma ~ logU[1e-3, 1e-1], Poisson arrivals at ``rate`` per second,
    a ``mc_fraction`` share of mcsolve jobs with ``ntraj`` trajectories each."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n_jobs)
    arrivals = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(n_jobs):
        kind = "mc" if rng.random() < mc_fraction else "me"
        out.append(JobSpec(i, kind, int(rng.integers(n_min, n_max + 1)),
                           float(rng.uniform(0.01, 0.1) * 2 * np.pi),
                           float(10 ** rng.uniform(-3, -1)), float(10 ** rng.uniform(-3, -1)),
                           float(arrivals[i]), ntraj if kind == "mc" else 0,
                           int(rng.integers(0, 2**62))))
    return out


def build_job(spec: JobSpec, tlist=None) -> Job:
    tlist = np.linspace(0.0, 20.0, 101) if tlist is None else tlist
    s = jaynes_cummings(spec.n_cav, g=spec.g, kappa=spec.kappa, gamma=spec.gamma, kind=spec.kind)
    n = s.dim * s.dim if spec.kind == "me" else s.dim
    return Job(spec, s, np.asarray(tlist), n)


def percentiles(lat):
    lat = np.asarray([x for x in lat if x is not None])
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}


def fifo_latencies(arrivals, service):
    """Latencies of a single FIFO server with the given service times."""
    free = 0.0
    out = []
    for a, s in zip(arrivals, service):
        start = max(a, free)
        free = start + s
        out.append(free - a)
    return out


def _footprint(jobs, dtype_bytes, lib, dtype):
    nnz = sum(sum(m.nnz for m, _ in j.system.terms) for j in jobs)
    states = sum(j.state_len for j in jobs)
    n_items = sum(max(j.spec.ntraj, 1) for j in jobs)
    max_n = max(j.state_len for j in jobs)
    slots = min(n_items, 600)
    return (nnz * (dtype_bytes + 4) + states * 16 + slots * int(lib.qg_batch_slot_bytes(max_n, dtype))
            + n_items * 101 * 8 * 16)


class Server:
    """Continuous batching over a fixed number of CUDA streams and an HBM budget."""

    def __init__(self, precision="mixed", n_streams=4, hbm_budget=8 << 30, max_items=8192,
                 max_jobs_per_launch=512, max_jumps=256, launch_timeout=120.0, group="load"):
        """``group``: ``"load"`` gives each item of a launch with few large items a
        thread-block cluster (8 SMs), each item of a launch of at most two items per SM
        a CTA, and packs fuller launches one item per warp; ``"auto"``, ``"warp"``,
        ``"cta"`` or ``"cluster"`` fix the shape for every launch (results then do not
        depend on how requests were grouped into launches)."""
        self.precision = precision
        self.dtype = "c64" if precision == "mixed" else "c128"
        self.qdt = _lib.QG_C64 if self.dtype == "c64" else _lib.QG_C128
        self.streams = [torch.cuda.Stream() for _ in range(n_streams)]
        self.budget = int(hbm_budget)
        self.max_items = int(max_items)
        self.max_jobs = int(max_jobs_per_launch)
        self.max_jumps = int(max_jumps)
        self.launch_timeout = float(launch_timeout)
        if group not in ("load", "auto", "warp", "cta", "cta128", "cluster"):
            raise ValueError("group must be 'load', 'auto', 'warp', 'cta', 'cta128' or 'cluster'")
        self.group = group
        self._cluster_cache = {}
        # items per launch up to which each item gets a CTA: two per SM
        self.cta_items = 2 * torch.cuda.get_device_properties(0).multi_processor_count \
            if torch.cuda.is_available() else 0
        self.stats = {"launches": 0, "items": 0, "max_inflight_bytes": 0, "max_concurrent": 0,
                      "max_launch_s": 0.0}

    def _cluster_slots(self, max_n):
        if max_n not in self._cluster_cache:
            lib = _lib.load()
            self._cluster_cache[max_n] = int(lib.qg_batch_group_slots(max_n, self.qdt,
                                                                      _lib.QG_GROUP_CLUSTER))
        return self._cluster_cache[max_n]

    def _launch(self, jobs, stream):
        bp = BatchProblem(self.dtype)
        for j in jobs:
            s = j.system
            if j.spec.kind == "me":
                sid = bp.add_system(s.terms, s.e_ops, j.tlist, "me")
                bp.add_item(sid, s.state0)
            else:
                sid = bp.add_system(s.terms, s.e_ops, j.tlist, "mc", c_ops=s.c_ops)
                for sd in np.random.SeedSequence(j.spec.seed).spawn(j.spec.ntraj):
                    bp.add_item(sid, s.state0, seed=sd)
        # host-visible cancel flag (pinned, mapped): the kernel polls it at every output time
        cancel = torch.zeros(1, dtype=torch.int32).pin_memory()
        # group shape by load: a launch with few items gives each one a CTA (more
        # threads per item, lower latency); a full launch packs items one per warp
        group = self.group
        if group == "load":
            n_items = len(bp.items)
            max_n = max(j.state_len for j in jobs)
            if max_n >= 1600 and n_items <= self._cluster_slots(max_n):
                group = "cluster"     # few large items: 8 SMs each
            elif n_items <= self.cta_items:
                group = "cta128" if max_n <= 512 else "cta"   # small states: 128 threads
            else:
                group = "auto"
        with torch.cuda.stream(stream):
            cost = [bp.sys_info[it[0]]["nnz"] for it in bp.items]
            max_jumps = self.max_jumps if any(j.spec.kind == "mc" for j in jobs) else 0
            order = np.argsort(cost, kind="stable")[::-1]
            try:
                bp.build(max_jumps=max_jumps, order=order, group=group)
            except _lib.QgError as exc:
                # a shape the load policy picked could not be sized (its occupancy query
                # failed): the launch goes out in the default shape, and the event is kept
                if group == "auto":
                    raise
                self.stats["shape_retries"] = self.stats.get("shape_retries", 0) + 1
                self.stats["last_shape_error"] = f"{group}: {exc}"
                group = "auto"
                bp.build(max_jumps=max_jumps, order=order, group=group)
            bp.set_cancel(cancel)
            bp.cancel_flag = cancel
            bp.ev_start = torch.cuda.Event(enable_timing=True)
            bp.ev_start.record(stream)
            bp.launch()
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(stream)
        self.stats["launches"] += 1
        self.stats["items"] += len(bp.items)
        for j in jobs:
            j.extra["launch"] = (group, len(bp.items), len(jobs))
        return bp, ev

    @staticmethod
    def _collect(bp, jobs):
        res = bp.results()
        check_status(res)
        k = 0
        for j in jobs:
            if j.spec.kind == "me":
                j.result = [res[k]["expect"][:, e] for e in range(res[k]["expect"].shape[1])]
                k += 1
            else:
                runs = np.stack([r["expect"] for r in res[k:k + j.spec.ntraj]])
                j.result = [runs[:, :, e].mean(axis=0) for e in range(runs.shape[2])]
                j.extra["jumps"] = [int(r["jumps"]) for r in res[k:k + j.spec.ntraj]]
                k += j.spec.ntraj

    def serve(self, jobs, realtime=True):
        """Run the stream; returns (jobs with results and completion times, wall seconds).

        Python's cyclic garbage collector is paused while serving: with many
        requests alive a full collection takes long enough to stall admission."""
        gc_was_enabled = gc.isenabled()
        gc.disable()
        try:
            return self._serve(jobs, realtime)
        finally:
            if gc_was_enabled:
                gc.enable()

    def _serve(self, jobs, realtime):
        lib = _lib.load()
        pending = deque(sorted(jobs, key=lambda j: j.spec.arrival))
        waiting = {b: deque() for b in BUCKETS}
        inflight = []   # (bp, event, jobs, stream, bytes)
        free_streams = list(self.streams)
        used = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        while pending or inflight or any(waiting.values()):
            now = time.perf_counter() - t0
            while pending and (not realtime or pending[0].spec.arrival <= now):
                j = pending.popleft()
                b = next(b for b in BUCKETS if j.state_len <= b)
                waiting[b].append(j)
            progressed = False
            # admission: the bucket whose oldest job arrived first
            while free_streams:
                cand = [(q[0].spec.arrival, b) for b, q in waiting.items() if q]
                if not cand:
                    break
                _, b = min(cand)
                q = waiting[b]
                take, items = [], 0
                while q and len(take) < self.max_jobs:
                    n_it = max(q[0].spec.ntraj, 1)
                    if take and items + n_it > self.max_items:
                        break
                    trial = take + [q[0]]
                    fb = _footprint(trial, 8 if self.dtype == "c64" else 16, lib, self.qdt)
                    if take and used + fb > self.budget:
                        break
                    take.append(q.popleft())
                    items += n_it
                if not take:
                    break
                fb = _footprint(take, 8 if self.dtype == "c64" else 16, lib, self.qdt)
                if inflight and used + fb > self.budget:
                    for j in reversed(take):
                        q.appendleft(j)
                    break
                st = free_streams.pop()
                t_admit = time.perf_counter()
                bp, ev = self._launch(take, st)
                bp.t_launch = time.perf_counter()
                for j in take:
                    # where a request's latency goes: waiting for admission, the host
                    # side of its launch, the launch on the GPU, collection
                    j.extra["wait_ms"] = 1e3 * (t_admit - t0 - j.spec.arrival)
                    j.extra["host_ms"] = 1e3 * (bp.t_launch - t_admit)
                used += fb
                inflight.append((bp, ev, take, st, fb))
                self.stats["max_inflight_bytes"] = max(self.stats["max_inflight_bytes"], used)
                self.stats["max_concurrent"] = max(self.stats["max_concurrent"], len(inflight))
                progressed = True
            # completions (and the launch watchdog: a launch in flight too long is
            # cancelled through its flag and reported)
            for rec in list(inflight):
                bp, ev, take, st, fb = rec
                age = time.perf_counter() - bp.t_launch
                if not ev.query() and age > self.launch_timeout and bp.cancel_flag[0] == 0:
                    bp.cancel_flag[0] = 1
                if ev.query():
                    self.stats["max_launch_s"] = max(self.stats["max_launch_s"], age)
                    if bp.cancel_flag[0]:
                        raise TimeoutError(
                            f"launch of jobs {[j.spec.id for j in take][:20]} exceeded "
                            f"{self.launch_timeout:.0f} s and was cancelled")
                    t_seen = time.perf_counter()
                    self._collect(bp, take)
                    done = time.perf_counter() - t0
                    gpu_ms = bp.ev_start.elapsed_time(ev)
                    for j in take:
                        j.done = done
                        j.extra["gpu_ms"] = gpu_ms
                        j.extra["collect_ms"] = 1e3 * (time.perf_counter() - t_seen)
                    inflight.remove(rec)
                    free_streams.append(st)
                    used -= fb
                    progressed = True
            if not progressed:
                time.sleep(50e-6)
        return jobs, time.perf_counter() - t0


def serve_plain(jobs, precision="double"):
    """The plain per-request drop-in served in real time: one request at a time in arrival
    order (a single FIFO server), each solved by :func:`solve_plain` once it has arrived.
    Sets ``result`` and ``done`` of every job; returns the wall time."""
    order = sorted(jobs, key=lambda j: j.spec.arrival)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for j in order:
        wait = j.spec.arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        j.result = solve_plain(j, precision)
        torch.cuda.synchronize()
        j.done = time.perf_counter() - t0
    return time.perf_counter() - t0


def solve_plain(job: Job, precision="double"):
    """The plain per-request drop-in: one job alone, complex128, no batching across
    requests -- ``mesolve`` through the single-system integrator, ``mcsolve`` through
    one launch of that request's trajectories."""
    from .solver import solve_system
    from .batched import mcsolve_batch
    if job.spec.kind == "me":
        r = solve_system(job.system, job.tlist, {"precision": precision})
        return r.expect
    seeds = np.random.SeedSequence(job.spec.seed).spawn(job.spec.ntraj)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    r = mcsolve_batch(job.system, job.tlist, job.spec.ntraj, seeds=seeds,
                      precision="double" if precision == "double" else "mixed",
                      group="cta128" if job.spec.ntraj <= 2 * sms else "auto")
    return r.expect
