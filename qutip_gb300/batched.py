"""Batched, persistent solves: many small systems or trajectories in one launch.

The reference runs one solve per call (``Solver.run``, qutip/solver/solver_base.py:159-226)
and maps trajectories over a Python loop or a process pool
(``MultiTrajSolver.run``, qutip/solver/multitraj.py:169-258; ``parallel_map``,
qutip/solver/parallel.py:267-338).  Here every system's generator, e_ops and
collapse operators are packed into shared device pools; each *item* (a
master-equation solve, or one Monte-Carlo trajectory with its own PCG64 stream)
is an entry of an item table, and ``qg_batch_vern7`` runs all of them in one
persistent launch, one warp (small states) or one CTA (large states) per item at
a time, each with its own adaptive step.  :meth:`BatchProblem.capture` records
the launch in a CUDA graph that :meth:`BatchProblem.replay` re-runs with new
seeds written in place; :func:`tune_batch` picks the group shape and slot count
by timing them on a sample of the items.

Trajectories reuse their system's operators (one copy in HBM however many
trajectories run).  Per-trajectory random streams are numpy's PCG64 states
after seeding, so the device draws the same numbers as
``numpy.random.default_rng(seed)`` (qutip/solver/multitraj.py:382-393).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from .coefficients import pack_programs
from .operator import row_major_layout, stream_ptr
from .systems import OpenSystem, merge_terms

__all__ = ["BatchProblem", "mesolve_batch", "mcsolve_batch", "MCResult", "pcg_state_of"]

SYSTEM_DTYPE = np.dtype([("n", "<i4"), ("d", "<i4"), ("n_groups", "<i4"), ("n_eops", "<i4"),
                         ("rp_off", "<i8"), ("coef_off", "<i8"), ("eop_rp_off", "<i8"),
                         ("cop_rp_off", "<i8"), ("tlist_off", "<i8"), ("n_out", "<i4"),
                         ("kind", "<i4"), ("n_cops", "<i4"), ("nsteps", "<i4"),
                         ("atol", "<f8"), ("rtol", "<f8"), ("cop_coef_off", "<i8")],
                        align=True)
ITEM_DTYPE = np.dtype([("system", "<i4"), ("pad", "<i4"), ("y0_off", "<i8"), ("out_off", "<i8"),
                       ("sh", "<u8"), ("sl", "<u8"), ("ih", "<u8"), ("il", "<u8"),
                       ("floor", "<f8")], align=True)


class BatchStruct(C.Structure):
    _fields_ = [("n_systems", C.c_int32), ("n_items", C.c_int32), ("dtype", C.c_int32),
                ("max_n", C.c_int32), ("systems", C.c_void_p), ("items", C.c_void_p),
                ("op_rp", C.c_void_p), ("op_col", C.c_void_p), ("op_val", C.c_void_p),
                ("coef_code", C.c_void_p), ("coef_start", C.c_void_p),
                ("coef_consts", C.c_void_p), ("eop_rp", C.c_void_p), ("eop_col", C.c_void_p),
                ("eop_val", C.c_void_p), ("cop_rp", C.c_void_p), ("cop_col", C.c_void_p),
                ("cop_val", C.c_void_p), ("tlist", C.c_void_p), ("y0", C.c_void_p),
                ("out", C.c_void_p), ("status", C.c_void_p), ("jump_t", C.c_void_p),
                ("jump_which", C.c_void_p), ("max_jumps", C.c_int32), ("n_slots", C.c_int32),
                ("work", C.c_void_p), ("queue", C.c_void_p), ("cancel", C.c_void_p),
                ("progress", C.c_void_p), ("debug", C.c_void_p),
                ("norm_steps", C.c_int32), ("group", C.c_int32), ("norm_t_tol", C.c_double),
                ("norm_tol", C.c_double), ("norm_min_step", C.c_double),
                ("mc_corr_eps", C.c_double), ("stage_op_entries", C.c_int64),
                ("stage_op_rp", C.c_int32), ("pad2_", C.c_int32)]


MC_DEFAULTS = dict(norm_steps=25, norm_t_tol=1e-6, norm_tol=1e-4, norm_min_step=0.1,
                   mc_corr_eps=1e-10)


def pcg_state_of(seed) -> tuple[int, int]:
    """numpy PCG64 (state, increment) of ``default_rng(seed)`` (which wraps
    ``PCG64(seed)``; the bit generator alone is cheaper to build)."""
    st = np.random.PCG64(seed).state["state"]
    return int(st["state"]), int(st["inc"])


def _split128(v: int):
    return (v >> 64) & (2**64 - 1), v & (2**64 - 1)


def _group_major(ops, d):
    """CSR arrays of several d x d operators, one group each: rp[g*(d+1)+r]."""
    rps, cols, vals, off = [], [], [], 0
    for o in ops:
        m = sp.csr_matrix(o, dtype=np.complex128)
        m.sort_indices()
        rps.append(m.indptr.astype(np.int64) + off)
        cols.append(m.indices.astype(np.int32))
        vals.append(m.data)
        off += m.nnz
    if not ops:
        return np.zeros(0, np.int64), np.zeros(0, np.int32), np.zeros(0, np.complex128)
    return np.concatenate(rps), np.concatenate(cols), np.concatenate(vals)


@dataclass
class MCResult:
    times: np.ndarray
    runs_expect: np.ndarray            # [n_eops, ntraj, n_t] (real parts for Hermitian e_ops)
    expect: list
    col_times: list
    col_which: list
    stats: dict = field(default_factory=dict)


class BatchProblem:
    """Host-side builder of the device pools and item table of one batched launch."""

    def __init__(self, dtype: str = "c64", device="cuda"):
        if dtype not in ("c64", "c128"):
            raise TypeError("dtype must be 'c64' or 'c128'")
        self.dtype = dtype
        self.device = torch.device(device)
        self.systems = []
        self.items = []
        self._op_rp, self._op_col, self._op_val = [], [], []
        self._entries = 0
        self._rp_len = 0
        self._coef_code, self._coef_start, self._coef_consts = [], [], []
        self._code_len = self._start_len = self._const_len = 0
        self._eop_rp, self._eop_col, self._eop_val, self._eop_entries, self._eop_rp_len = [], [], [], 0, 0
        self._cop_rp, self._cop_col, self._cop_val, self._cop_entries, self._cop_rp_len = [], [], [], 0, 0
        self._tlist, self._tlist_len = [], 0
        self._y0, self._y0_len = [], 0
        self._out_len = 0
        self.sys_info = []

    def _add_programs(self, coeffs) -> int:
        """Append the coefficient programs of ``coeffs`` (None: constant 1) to the launch's
        pools; returns the offset of their starts in ``coef_start``, or -1 when all are
        constant."""
        if all(c is None for c in coeffs):
            return -1
        code, starts, consts = pack_programs(coeffs)
        # starts index the global code pool; constants are shifted inside the code
        code = code.copy()
        i = 0
        while i < len(code):
            if code[i] == 1:  # OP_CONST
                code[i + 1] += self._const_len // 2
                i += 1
            i += 1
        self._coef_code.append(code)
        self._coef_start.append(starts + self._code_len)
        self._coef_consts.append(consts)
        off = self._start_len
        self._code_len += len(code)
        self._start_len += len(starts)
        self._const_len += len(consts)
        return off

    def add_system(self, terms, e_ops, tlist, kind="me", c_ops=(), dim=None, atol=1e-8,
                   rtol=1e-6, nsteps=1000) -> int:
        """Register a generator (list of (matrix, coefficient)), its e_ops and tlist.
        ``c_ops`` (trajectories): matrices, or ``(matrix, Coefficient | None)`` pairs for
        collapse operators ``f(t) C``; the generator must then carry their
        ``-1/2 |f|^2 C^dag C`` terms, as the reference's H_nh does."""
        terms = merge_terms(terms)
        if len(terms) > _lib.QG_MAX_GROUPS:
            raise ValueError(f"at most {_lib.QG_MAX_GROUPS} coefficient groups")
        n = terms[0][0].shape[0]
        d = dim if dim is not None else (int(round(np.sqrt(n))) if kind == "me" else n)
        if kind == "me" and d * d != n:
            raise ValueError("master-equation generators act on column-stacked d x d states")
        mats = [m for m, _ in terms]
        rp, col, val = row_major_layout(mats)
        self._op_rp.append((rp + self._entries).astype(np.int64))
        self._op_col.append(col)
        self._op_val.append(val)
        rp_off = self._rp_len
        self._rp_len += len(rp)
        self._entries += len(col)
        coef_off = self._add_programs([c for _, c in terms])
        e_rp, e_col, e_val = _group_major(e_ops, d)
        self._eop_rp.append(e_rp + self._eop_entries)
        self._eop_col.append(e_col)
        self._eop_val.append(e_val)
        eop_rp_off = self._eop_rp_len
        self._eop_rp_len += len(e_rp)
        self._eop_entries += len(e_col)
        c_ops = [c if isinstance(c, tuple) else (c, None) for c in c_ops]
        cop_coef_off = self._add_programs([f for _, f in c_ops])
        c_rp, c_col, c_val = _group_major([m for m, _ in c_ops], d)
        self._cop_rp.append(c_rp + self._cop_entries)
        self._cop_col.append(c_col)
        self._cop_val.append(c_val)
        cop_rp_off = self._cop_rp_len
        self._cop_rp_len += len(c_rp)
        self._cop_entries += len(c_col)
        tl = np.asarray(tlist, dtype=np.float64)
        self._tlist.append(tl)
        tlist_off = self._tlist_len
        self._tlist_len += len(tl)
        self.systems.append((n, d, len(terms), len(e_ops), rp_off, coef_off, eop_rp_off,
                             cop_rp_off, tlist_off, len(tl), 0 if kind == "me" else 1,
                             len(c_ops), int(nsteps), float(atol), float(rtol), cop_coef_off))
        self.sys_info.append(dict(n=n, d=d, kind=kind, n_eops=len(e_ops), n_out=len(tl),
                                  nnz=len(col), tlist=tl, rp_len=len(rp)))
        return len(self.systems) - 1

    def add_item(self, system: int, y0, seed=None, jump_prob_floor: float = 0.0) -> int:
        """Queue one solve (a trajectory for ``"mc"`` systems) from ``y0``.

        ``jump_prob_floor`` is improved sampling's lower bound for the first jump
        target (mcsolve.py:245-279): the no-jump probability of ``y0``."""
        if not 0.0 <= float(jump_prob_floor) < 1.0:
            raise ValueError("jump_prob_floor must lie in [0, 1)")
        info = self.sys_info[system]
        y0 = np.asarray(y0, dtype=np.complex128).reshape(-1)
        if y0.shape[0] != info["n"]:
            raise ValueError(f"initial state of length {y0.shape[0]} for a system of size {info['n']}")
        self._y0.append(y0)
        y0_off = self._y0_len
        self._y0_len += len(y0)
        out_off = self._out_len
        self._out_len += info["n_out"] * (info["n_eops"] + 1)
        sh = sl = ih = il = 0
        if seed is not None:
            state, inc = seed if isinstance(seed, tuple) else pcg_state_of(seed)
            sh, sl = _split128(state)
            ih, il = _split128(inc)
        self.items.append((system, 0, y0_off, out_off, sh, sl, ih, il, float(jump_prob_floor)))
        return len(self.items) - 1

    # -- device upload and launch --------------------------------------------
    @staticmethod
    def _host(arrs, np_dtype, pad=8):
        """Concatenated pool in its device dtype, with ``pad`` zero entries (bulk copies
        of the pool may read up to 16 bytes past the last entry)."""
        a = np.concatenate(arrs).astype(np_dtype) if arrs and sum(len(x) for x in arrs) else \
            np.zeros(0, np_dtype)
        return np.concatenate([a, np.zeros(pad, np_dtype)])

    ALIGN = 256

    def _pack_upload(self, pools):
        """Copy ``[(name, host array, torch dtype)]`` to the device in one transfer and
        bind ``self.<name>`` to 256-byte aligned views of it."""
        offs, total = [], 0
        for _, a, _ in pools:
            offs.append(total)
            total += -(-a.nbytes // self.ALIGN) * self.ALIGN
        host = np.zeros(max(total, self.ALIGN), dtype=np.uint8)
        for (_, a, _), off in zip(pools, offs):
            host[off:off + a.nbytes] = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
        dev = torch.from_numpy(host).to(self.device)
        for (name, a, tdt), off in zip(pools, offs):
            setattr(self, name, dev[off:off + a.nbytes].view(tdt))
        return dev

    def _pack_zeros(self, outs):
        """One zeroed device buffer for ``[(name, count, torch dtype)]``, bound as views."""
        offs, total = [], 0
        for _, count, tdt in outs:
            offs.append(total)
            nb = count * torch.empty(0, dtype=tdt).element_size()
            total += -(-nb // self.ALIGN) * self.ALIGN
        dev = torch.zeros(total, dtype=torch.uint8, device=self.device)
        for (name, count, tdt), off in zip(outs, offs):
            nb = count * torch.empty(0, dtype=tdt).element_size()
            setattr(self, name, dev[off:off + nb].view(tdt))
        return dev

    def build(self, max_jumps=0, mc_options=None, order=None, n_slots=None, group="auto",
              stage_operator="auto"):
        """Upload pools; ``order`` permutes the items (longest first balances the queue).

        ``group`` is ``"auto"``, ``"warp"``, ``"cta"``, ``"cta128"`` or ``"cluster"``
        (threads per item: 32, 256, 128, or 8 x 256 on a thread-block cluster);
        ``n_slots`` caps the resident groups (default: all that fit);
        ``stage_operator``: copy the generator of a single-system launch into shared
        memory once per CTA (``"auto"``: when it takes at most 64 KB)."""
        if not self.items:
            raise ValueError("no items")
        lib = _lib.load()
        cdt = torch.complex64 if self.dtype == "c64" else torch.complex128
        qdt = _lib.QG_C64 if self.dtype == "c64" else _lib.QG_C128
        cnp = np.complex64 if self.dtype == "c64" else np.complex128
        sys_np = np.array(self.systems, dtype=SYSTEM_DTYPE)
        items = list(self.items)
        self.order = np.arange(len(items)) if order is None else np.asarray(order)
        items = [items[i] for i in self.order]
        item_np = np.array(items, dtype=ITEM_DTYPE)
        n_items = len(items)
        self.max_jumps = int(max_jumps)
        # every input pool in one host buffer and one copy; device views by name
        pools = [
            ("op_rp", self._host(self._op_rp, np.int32), torch.int32),
            ("op_col", self._host(self._op_col, np.int32), torch.int32),
            ("op_val", self._host(self._op_val, cnp), cdt),
            ("coef_code", self._host(self._coef_code, np.int32), torch.int32),
            ("coef_start", self._host(self._coef_start, np.int32), torch.int32),
            ("coef_consts", self._host(self._coef_consts, np.float64), torch.float64),
            ("eop_rp", self._host(self._eop_rp, np.int32), torch.int32),
            ("eop_col", self._host(self._eop_col, np.int32), torch.int32),
            ("eop_val", self._host(self._eop_val, np.complex128), torch.complex128),
            ("cop_rp", self._host(self._cop_rp, np.int32), torch.int32),
            ("cop_col", self._host(self._cop_col, np.int32), torch.int32),
            ("cop_val", self._host(self._cop_val, np.complex128), torch.complex128),
            ("tlist_d", self._host(self._tlist, np.float64), torch.float64),
            ("y0_d", self._host(self._y0, np.complex128), torch.complex128),
            ("systems_d", sys_np.view(np.uint8).reshape(-1), torch.uint8),
            ("items_d", item_np.view(np.uint8).reshape(-1), torch.uint8),
        ]
        self.inputs = self._pack_upload(pools)
        # outputs (zeroed): one allocation and one fill
        outs = [("out", max(self._out_len, 1), torch.complex128),
                ("status", 4 * n_items, torch.int32),
                ("jump_t", max(n_items * self.max_jumps, 1), torch.float64),
                ("jump_which", max(n_items * self.max_jumps, 1), torch.int32),
                ("queue", 4, torch.int32)]
        self.outputs = self._pack_zeros(outs)
        self.max_n = max(info["n"] for info in self.sys_info)
        if group not in GROUPS:
            raise ValueError(f"group must be one of {sorted(GROUPS)}")
        self.group = group
        stage_entries = stage_rp = 0
        if len(self.systems) == 1 and group != "cluster" and stage_operator:
            info = self.sys_info[0]
            es = 8 if self.dtype == "c64" else 16
            a16 = lambda b: (b + 15) // 16 * 16  # noqa: E731
            op_bytes = a16(4 * info["rp_len"]) + a16(4 * info["nnz"]) + a16(es * info["nnz"])
            if stage_operator is True or op_bytes <= 64 * 1024:
                stage_entries, stage_rp = info["nnz"], info["rp_len"]
        mc = {**MC_DEFAULTS, **(mc_options or {})}
        p = lambda t: t.data_ptr()  # noqa: E731
        self.struct = BatchStruct(
            len(self.systems), n_items, qdt, self.max_n, p(self.systems_d), p(self.items_d),
            p(self.op_rp), p(self.op_col), p(self.op_val), p(self.coef_code), p(self.coef_start),
            p(self.coef_consts), p(self.eop_rp), p(self.eop_col), p(self.eop_val), p(self.cop_rp),
            p(self.cop_col), p(self.cop_val), p(self.tlist_d), p(self.y0_d), p(self.out),
            p(self.status), p(self.jump_t), p(self.jump_which), self.max_jumps, 1,
            None, p(self.queue), None, None, None, int(mc["norm_steps"]), GROUPS[group],
            float(mc["norm_t_tol"]),
            float(mc["norm_tol"]), float(mc["norm_min_step"]), float(mc["mc_corr_eps"]),
            int(stage_entries), int(stage_rp), 0)
        slots = lib.qg_batch_launch_slots(C.byref(self.struct))
        if slots < 0:
            _lib.check(slots, "qg_batch_launch_slots")
        self.n_slots = int(min(n_items, slots if n_slots is None else n_slots))
        slot_bytes = int(lib.qg_batch_slot_bytes(self.max_n, qdt))
        self.work = torch.empty(self.n_slots * slot_bytes, dtype=torch.uint8, device=self.device)
        self.struct.n_slots = self.n_slots
        self.struct.work = p(self.work)
        self.staged_operator = stage_entries > 0
        return self

    def set_cancel(self, host_flag_tensor):
        """Point the kernel at a host-mapped int32 flag (pinned tensor); None clears it."""
        self.struct.cancel = None if host_flag_tensor is None else host_flag_tensor.data_ptr()

    def launch(self):
        _lib.call("qg_batch_vern7", C.byref(self.struct), stream_ptr())

    # -- CUDA graph --------------------------------------------------------
    def capture(self):
        """Record one launch in a CUDA graph (on a side stream, as torch requires).

        The graph keeps this problem's device pointers; :meth:`replay` re-runs it
        after writing new per-item seeds into the item table in place."""
        self._items_np = np.array([self.items[i] for i in self.order], dtype=ITEM_DTYPE)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.launch()
        torch.cuda.synchronize()
        return self.graph

    def replay(self, seeds=None):
        """Re-run the captured launch; ``seeds`` (one per item, in item order) gives
        every trajectory a new PCG64 stream (SeedSequence / int / (state, inc))."""
        if getattr(self, "graph", None) is None:
            raise RuntimeError("capture() first")
        if seeds is not None:
            seeds = list(seeds)
            if len(seeds) != len(self.items):
                raise ValueError("one seed per item")
            inv = np.empty_like(self.order)
            inv[self.order] = np.arange(len(self.order))
            for i, sd in enumerate(seeds):
                state, inc = sd if isinstance(sd, tuple) else pcg_state_of(sd)
                row = inv[i]
                self._items_np[row]["sh"], self._items_np[row]["sl"] = _split128(state)
                self._items_np[row]["ih"], self._items_np[row]["il"] = _split128(inc)
                it = list(self.items[i])
                it[4:8] = [*_split128(state), *_split128(inc)]
                self.items[i] = tuple(it)
            host = torch.from_numpy(self._items_np.view(np.uint8).copy())
            self.items_d.copy_(host, non_blocking=False)
        self.graph.replay()

    def results(self, normalize=True):
        """Per item (original order): expect [n_out, n_eops], status row, jumps."""
        if int(self.queue[2].item()) != 0:
            raise RuntimeError("an operator-staging wait gave up on the device (the results "
                               "were computed from global memory); the GPU may be unhealthy")
        out = self.out.cpu().numpy()
        status = self.status.cpu().numpy().reshape(-1, 4)
        jt = self.jump_t.cpu().numpy()
        jw = self.jump_which.cpu().numpy()
        inv = np.empty_like(self.order)
        inv[self.order] = np.arange(len(self.order))
        res = []
        for i, it in enumerate(self.items):
            k = inv[i]
            info = self.sys_info[it[0]]
            ne, no = info["n_eops"], info["n_out"]
            raw = out[it[3]:it[3] + no * (ne + 1)].reshape(no, ne + 1)
            vals = raw[:, :ne]
            if normalize:
                # outputs a failed item never reached are zero: they become NaN here
                with np.errstate(divide="ignore", invalid="ignore"):
                    vals = vals / raw[:, ne:ne + 1]
            st = status[k]
            nj = int(st[3])
            res.append(dict(expect=vals, norm=raw[:, ne], status=int(st[0]), steps=int(st[1]),
                            rhs=int(st[2]), jumps=nj,
                            col_times=jt[k * self.max_jumps:k * self.max_jumps + min(nj, self.max_jumps)].copy(),
                            col_which=jw[k * self.max_jumps:k * self.max_jumps + min(nj, self.max_jumps)].copy()))
        return res


GROUPS = {"auto": _lib.QG_GROUP_AUTO, "warp": _lib.QG_GROUP_WARP, "cta": _lib.QG_GROUP_CTA,
          "cluster": _lib.QG_GROUP_CLUSTER, "cta128": _lib.QG_GROUP_CTA128}

_TUNED: dict = {}


def tune_batch(make_problem, sample_items=256, candidates=None, reps=2):
    """Pick the group shape and slot count of a batch by timing them.

    ``make_problem(n_items)`` returns an unbuilt :class:`BatchProblem` with the
    first ``n_items`` items of the real batch.  Each candidate ``(group,
    slot_fraction)`` is built and launched ``reps`` times on that sample (events
    on the current stream); the fastest is returned and cached by (dtype, max_n
    bucket, kind).  Candidates default to warp and CTA groups at full, 3/4 and
    1/2 of the resident slots, and 8-CTA clusters at all resident slots.
    """
    probe = make_problem(sample_items)
    kind = probe.sys_info[0]["kind"] if probe.sys_info else 0
    max_n = max(info["n"] for info in probe.sys_info)
    key = (probe.dtype, int(np.ceil(np.log2(max(max_n, 2)))), kind)
    if key in _TUNED:
        return _TUNED[key]
    candidates = candidates or ([(g, f) for g in ("warp", "cta", "cta128")
                                 for f in (1.0, 0.75, 0.5)] + [("cluster", 1.0)])
    lib = _lib.load()
    qdt = _lib.QG_C64 if probe.dtype == "c64" else _lib.QG_C128
    best = None
    timings = {}
    for group, frac in candidates:
        full = lib.qg_batch_group_slots(max_n, qdt, GROUPS[group])
        if full <= 0:
            continue
        n_slots = max(1, int(full * frac))
        bp = make_problem(sample_items)
        bp.build(max_jumps=probe_max_jumps(bp), n_slots=n_slots, group=group)
        bp.launch()  # warm-up
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for _ in range(reps):
            bp.launch()
        end.record()
        end.synchronize()
        ms = start.elapsed_time(end) / reps
        timings[(group, frac)] = ms
        if best is None or ms < best[2]:
            best = (group, frac, ms)
    _TUNED[key] = {"group": best[0], "slot_fraction": best[1], "ms": best[2],
                   "timings": timings, "sample_items": sample_items}
    return _TUNED[key]


def probe_max_jumps(bp):
    return 4096 if any(info["kind"] == 1 for info in bp.sys_info) else 0


STATUS_TEXT = {
    -1: "Too much work done in one call. Try to increase the nsteps parameter or increasing "
        "the tolerance.",
    -2: "Step size becomes too small. Try increasing tolerance.",
    -3: "Step outside available range.",
    -5: "Could not find the collapse time within desired tolerance. Increase accuracy of the "
        "ODE solver or lower the tolerance with the options 'norm_steps', 'norm_tol', "
        "'norm_t_tol'.",
    -6: "Cancelled.",
    -7: "More jumps than max_jumps.",
    -8: "Item not run: bad system index, state longer than max_n, or a coefficient-group "
        "count outside 1..8.",
}


def check_status(res):
    for r in res:
        if r["status"] < 0:
            if r["status"] == -5:
                raise RuntimeError(STATUS_TEXT[-5])
            raise RuntimeError(STATUS_TEXT.get(r["status"], f"status {r['status']}"))


def mesolve_batch(systems, tlists, precision="mixed", atol=1e-8, rtol=1e-6, nsteps=1000):
    """Solve many master equations in one persistent launch.

    ``systems`` are :class:`~qutip_gb300.systems.OpenSystem` of kind ``"me"``;
    ``precision`` ``"mixed"`` (complex64 generator and stages, FP64 state and
    control) or ``"double"``.  Returns one expect array list per system.
    """
    dt = "c64" if precision == "mixed" else "c128"
    bp = BatchProblem(dt)
    tlists = tlists if isinstance(tlists, (list, tuple)) else [tlists] * len(systems)
    for s, tl in zip(systems, tlists):
        sid = bp.add_system(s.terms, s.e_ops, tl, "me", atol=atol, rtol=rtol, nsteps=nsteps)
        bp.add_item(sid, s.state0)
    cost = [bp.sys_info[it[0]]["nnz"] for it in bp.items]
    bp.build(order=np.argsort(cost)[::-1])
    bp.launch()
    res = bp.results()
    check_status(res)
    return [[r["expect"][:, k] for k in range(r["expect"].shape[1])] for r in res], res


def mcsolve_batch(system: OpenSystem, tlist, ntraj, seeds=None, precision="mixed", atol=1e-8,
                  rtol=1e-6, nsteps=1000, max_jumps=512, mc_options=None, group="auto",
                  n_slots=None) -> MCResult:
    """All ``ntraj`` trajectories of one Monte-Carlo system in one persistent launch.

    ``seeds``: an int / SeedSequence (spawned like the reference's ``_read_seed``,
    qutip/solver/multitraj.py:354-374) or a list of per-trajectory seeds.
    ``group`` / ``n_slots``: launch shape (see :meth:`BatchProblem.build`).
    """
    if system.kind != "mc":
        raise ValueError("mcsolve_batch needs a system built with kind='mc'")
    if seeds is None or not isinstance(seeds, (list, tuple)):
        ss = seeds if isinstance(seeds, np.random.SeedSequence) else np.random.SeedSequence(seeds)
        seeds = ss.spawn(ntraj)
    dt = "c64" if precision == "mixed" else "c128"
    bp = BatchProblem(dt)
    sid = bp.add_system(system.terms, system.e_ops, tlist, "mc", c_ops=system.c_ops,
                        atol=atol, rtol=rtol, nsteps=nsteps)
    for i in range(ntraj):
        bp.add_item(sid, system.state0, seed=seeds[i])
    t0 = time.perf_counter()
    bp.build(max_jumps=max_jumps, mc_options=mc_options, group=group, n_slots=n_slots)
    bp.launch()
    res = bp.results()
    check_status(res)
    runs = np.stack([r["expect"].T for r in res], axis=1)  # [n_eops, ntraj, n_t]
    return MCResult(np.asarray(tlist), runs, [runs[k].mean(axis=0) for k in range(runs.shape[0])],
                    [r["col_times"] for r in res], [r["col_which"] for r in res],
                    {"run time": time.perf_counter() - t0, "steps": sum(r["steps"] for r in res),
                     "rhs": sum(r["rhs"] for r in res)})
