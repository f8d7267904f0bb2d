"""Serving loop: query instances arriving over time against device-resident tables.

The reference answers one query at a time: main.py loads the tables, runs the
plan's operators one after another with a ``torch.cuda.synchronize()`` after
each (main.py:273-274) and frees its memory pools per query
(main.py:293-294).  Here the base columns and the built join directories are
loaded into HBM once (``ResidentTables``) and every request only runs its
query's hot path over them:

* ``filter_groupby``: ship_date <= c, group by (flag, status), the eight
  aggregates of the lineitem summary, in key order;
* ``join``: probe date > c1, build date < c2 (through the resident
  directory's row index), sum(price * (1 - discount)) by build key, top 10;
* ``star``: fact -> A (category == c, through A's row directory) -> B -> C,
  sum and count by C key, top 100;

each over a prefix of the resident fact table (the request's fact size),
with its constants bound at launch (the compiled kernels depend on the query
shape only).  A request's scratch (its group table, top-k scratch and
outputs) comes from ``DeviceArena``, a first-fit allocator over one device
slab sized by the HBM budget less the resident bytes.

``Scheduler`` is the continuous-batching loop: requests that have arrived
wait in FIFO order; a request is admitted as soon as an execution slot (a
CUDA stream) and its scratch memory are free, so requests that arrive while
others are on the GPU start without waiting for them to finish and their
kernels overlap on the device.  Completions are found by polling CUDA
events; a request's latency is its completion time minus its arrival time.
With ``slots=1`` the same loop is the one-at-a-time path.

``Scheduler`` only sees an executor with launch / done / finish, so its
admission logic is tested on the CPU with a simulated executor.
"""
from __future__ import annotations

import bisect
import ctypes as C
import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib as L

SHAPES = ("filter_groupby", "join", "star")


# ---------------------------------------------------------------------------- requests
@dataclass
class Request:
    rid: int
    shape: str
    rows: int                 # fact rows (a prefix of the resident fact table)
    consts: Tuple             # filter constants of this request
    arrival: float            # seconds from the start of the run


def poisson_trace(n: int, rate: float, max_rows: int, min_rows: int = 1_000_000, seed: int = 0,
                  shapes: Sequence[str] = SHAPES) -> List[Request]:
    """n requests with exponential inter-arrival times (mean 1/rate s), shapes uniform
    over `shapes`, fact rows log-uniform in [min_rows, max_rows], constants per request:
    ship_date cut-off U[2000, 2557), probe/build date cut-offs U[800, 1800), category U{1..5}."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n)
    arrivals = np.cumsum(gaps) - gaps[0]
    out = []
    lo, hi = math.log(min(min_rows, max_rows)), math.log(max_rows)
    for i in range(n):
        shape = shapes[int(rng.integers(0, len(shapes)))]
        rows = int(math.exp(rng.uniform(lo, hi)))
        if shape == "filter_groupby":
            consts = (int(rng.integers(2000, 2557)),)
        elif shape == "join":
            consts = (int(rng.integers(800, 1800)), int(rng.integers(800, 1800)))
        else:
            consts = (int(rng.integers(1, 6)),)
        out.append(Request(i, shape, rows, consts, float(arrivals[i])))
    return out


# ---------------------------------------------------------------------------- memory
class FirstFit:
    """First-fit allocator of byte ranges in [0, capacity) with coalescing frees.

    Offsets are aligned to `align`; alloc returns None when no free range fits."""

    def __init__(self, capacity: int, align: int = 256):
        self.capacity, self.align = int(capacity), int(align)
        self.free: List[Tuple[int, int]] = [(0, self.capacity)] if capacity > 0 else []   # sorted (offset, size)
        self.used: Dict[int, int] = {}

    @property
    def used_bytes(self) -> int:
        return sum(self.used.values())

    def alloc(self, nbytes: int) -> Optional[int]:
        size = max(self.align, -(-int(nbytes) // self.align) * self.align)
        for i, (off, sz) in enumerate(self.free):
            if sz >= size:
                if sz == size:
                    self.free.pop(i)
                else:
                    self.free[i] = (off + size, sz - size)
                self.used[off] = size
                return off
        return None

    def release(self, off: int) -> None:
        size = self.used.pop(off)
        i = bisect.bisect_left(self.free, (off, 0))
        self.free.insert(i, (off, size))
        # merge with the right neighbour, then the left one
        if i + 1 < len(self.free) and self.free[i][0] + self.free[i][1] == self.free[i + 1][0]:
            self.free[i] = (off, self.free[i][1] + self.free[i + 1][1])
            self.free.pop(i + 1)
        if i > 0 and self.free[i - 1][0] + self.free[i - 1][1] == self.free[i][0]:
            self.free[i - 1] = (self.free[i - 1][0], self.free[i - 1][1] + self.free[i][1])
            self.free.pop(i)


class DeviceArena:
    """The HBM budget: resident tables are charged once; request scratch is carved
    from one device slab of (budget - resident) bytes, at most `slab_cap`."""

    def __init__(self, budget_bytes: int, resident_bytes: int, device=None, slab_cap: int = 8 << 30):
        self.budget, self.resident = int(budget_bytes), int(resident_bytes)
        if self.resident > self.budget:
            raise MemoryError(f"resident tables ({self.resident} B) exceed the HBM budget ({self.budget} B)")
        self.capacity = min(self.budget - self.resident, int(slab_cap))
        self.ff = FirstFit(self.capacity)
        self.slab = None
        self.base = 0
        if device is not None and self.capacity > 0:
            import torch
            self.slab = torch.empty(self.capacity, dtype=torch.uint8, device=device)
            self.base = self.slab.data_ptr()

    def alloc(self, nbytes: int) -> Optional[int]:
        off = self.ff.alloc(nbytes)
        return None if off is None else self.base + off

    def release(self, ptr: int) -> None:
        self.ff.release(ptr - self.base)


# ---------------------------------------------------------------------------- scheduler
@dataclass
class Completed:
    req: Request
    start: float
    end: float
    result: object

    @property
    def latency(self) -> float:
        return self.end - self.req.arrival


class Scheduler:
    """Continuous-batching loop over an executor.

    executor.scratch_bytes(req) -> bytes of device scratch the request needs;
    executor.launch(req, slot, scratch_ptr) -> handle (enqueues all its work);
    executor.done(handle) -> bool (non-blocking);
    executor.finish(handle) -> result (after done).
    `arena` provides alloc/release of scratch; `clock` returns seconds."""

    def __init__(self, executor, arena, slots: int = 8, clock: Callable[[], float] = time.perf_counter):
        if slots < 1:
            raise ValueError("slots must be >= 1")
        self.ex, self.arena, self.slots, self.clock = executor, arena, int(slots), clock
        self.max_inflight = 0

    def run(self, trace: Sequence[Request], idle: Optional[Callable[[float], None]] = None) -> List[Completed]:
        pending = deque(sorted(trace, key=lambda r: (r.arrival, r.rid)))
        queue: deque = deque()
        inflight: List[tuple] = []          # (handle, req, slot, scratch, start)
        free_slots = list(range(self.slots))[::-1]
        done: List[Completed] = []
        t0 = self.clock()
        while pending or queue or inflight:
            now = self.clock() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            # admit in arrival order while a slot and the scratch are free
            while queue and free_slots:
                req = queue[0]
                need = self.ex.scratch_bytes(req)
                ptr = self.arena.alloc(need)
                if ptr is None:
                    if not inflight:
                        raise MemoryError(f"request {req.rid} needs {need} B, more than the arena can ever free")
                    break
                queue.popleft()
                slot = free_slots.pop()
                inflight.append((self.ex.launch(req, slot, ptr), req, slot, ptr, self.clock() - t0))
                self.max_inflight = max(self.max_inflight, len(inflight))
            # retire finished requests
            still = []
            for item in inflight:
                h, req, slot, ptr, start = item
                if self.ex.done(h):
                    res = self.ex.finish(h)
                    end = self.clock() - t0
                    self.arena.release(ptr)
                    free_slots.append(slot)
                    done.append(Completed(req, start, end, res))
                else:
                    still.append(item)
            inflight = still
            if not inflight and not queue and pending and idle is not None:
                idle(pending[0].arrival - (self.clock() - t0))
        return done


def latency_summary(done: Sequence[Completed]) -> dict:
    lat = np.array([c.latency for c in done]) * 1e3
    span = max(c.end for c in done) - min(c.req.arrival for c in done) if done else 0.0
    rows = sum(c.req.rows for c in done)
    return {"requests": len(done), "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "mean_ms": float(lat.mean()) if len(lat) else None,
            "requests_per_s": len(done) / span if span > 0 else None,
            "rows_per_s": rows / span if span > 0 else None}


# ---------------------------------------------------------------------------- resident tables
class ResidentTables:
    """Max-size tables of the three query shapes, on the device, with their directories.

    lineitem: ship_date, quantity, price, discount, tax, flag, status (fact rows n_fact);
    join: build key/date (n_build), probe fk/date/price/discount (n_fact), build directory
    key -> row; star: fact fkA/fkB/price/discount (n_fact), A key/category (n_a) with its
    row directory, B key -> fkC directory (n_b), C row directory (n_c)."""

    def __init__(self, device, n_fact: int, n_build: int = 1_500_000, n_a: int = 2_000_000, n_b: int = 15_000_000,
                 n_c: int = 1_500_000, seed: int = 0):
        import torch
        from . import datagen
        self.dev, self.n_fact = device, int(n_fact)
        self.lib = L.load()
        t = datagen.lineitem(n_fact, seed=seed + 1)
        self.li = {k: torch.from_numpy(v).to(device) for k, v in t.items()}
        j = datagen.join_tables(n_build, n_fact, seed=seed + 2)
        self.jt = {k: torch.from_numpy(v).to(device) for k, v in j.items()}
        s = datagen.star_tables(n_fact, n_a, n_b, n_c, seed=seed + 3)
        self.st = {k: torch.from_numpy(v).to(device) for k, v in s.items()}
        self.doms = {"join": (1, n_build), "a": (1, n_a), "b": (1, n_b), "c": (1, n_c)}
        self.dirs: Dict[str, "torch.Tensor"] = {}
        err = torch.zeros(4, dtype=torch.int32, device=device)
        stream = torch.cuda.current_stream(device).cuda_stream
        INT_MIN = -(1 << 31)
        specs = [("join", self.jt["b_key"], None, -1, -2, err.data_ptr()),
                 ("a", self.st["a_key"], None, -1, -2, err.data_ptr() + 4),
                 ("b", self.st["b_key"], self.st["b_fkc"], INT_MIN, INT_MIN + 1, err.data_ptr() + 8),
                 ("c", self.st["c_key"], None, -1, -2, err.data_ptr() + 12)]
        from .dtypes import code_of
        for name, keys, payload, empty, fail, e in specs:
            mn, mx = self.doms[name]
            d = torch.empty(mx - mn + 1, dtype=torch.int32, device=device)
            L.check(self.lib.tqpk_directory_build(
                keys.data_ptr(), code_of(keys.dtype), keys.numel(), None,
                payload.data_ptr() if payload is not None else None, code_of(payload.dtype) if payload is not None else 0,
                mn, mx - mn + 1, empty, fail, d.data_ptr(), e, stream), "tqpk_directory_build")
            self.dirs[name] = d
        bad = [int(x) for x in err.cpu().tolist() if x]
        if bad:
            L.check(bad[0], "resident directory build (repeated or out-of-domain key)")

    @property
    def nbytes(self) -> int:
        ts = list(self.li.values()) + list(self.jt.values()) + list(self.st.values()) + list(self.dirs.values())
        return int(sum(t.numel() * t.element_size() for t in ts))


# ---------------------------------------------------------------------------- query shapes
LINEITEM_IDS = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
LINEITEM_AGG = {
    "is partial": False, "keys": ["f#5", "s#6"], "input ids": [1, 2, 3, 4, 5, 6],
    "results": ["f#5", "s#6",
                [[["sum", ["q#1"]], "#", "1"], "AS", "sum_qty#201"],
                [[["sum", ["p#2"]], "#", "2"], "AS", "sum_price#202"],
                [[["sum", [["p#2", "*", ["1", "-", "d#3"]]]], "#", "3"], "AS", "sum_disc_price#203"],
                [[["sum", [[["p#2", "*", ["1", "-", "d#3"]], "*", ["1", "+", "t#4"]]]], "#", "4"], "AS", "sum_charge#204"],
                [[["avg", ["q#1"]], "#", "5"], "AS", "avg_qty#205"],
                [[["avg", ["p#2"]], "#", "6"], "AS", "avg_price#206"],
                [[["avg", ["d#3"]], "#", "7"], "AS", "avg_disc#207"],
                [[["count", ["q#1"]], "#", "8L"], "AS", "count_order#208"]],
    "out agg ids": [201, 202, 203, 204, 205, 206, 207, 208]}
JOIN_VALUE = [["p#23", "*", ["1.0", "-", "d#24"]]]


class GpuExecutor:
    """Runs requests of the three shapes over ResidentTables, one CUDA stream per slot.

    Each shape's kernels are compiled once; a request binds its row count,
    constants and scratch pointers at launch.  Results are copied into pinned
    host buffers on the request's stream before its completion event."""

    JOIN_K, STAR_K = 10, 100

    def __init__(self, tables: ResidentTables, slots: int):
        import torch
        from . import jit
        from .expr import compile_aggregate
        from .predicate import compile_filter
        if not jit.available():
            raise RuntimeError("the serving path needs the runtime-compiled kernels (NVRTC)")
        self.t, self.lib, self.dev = tables, tables.lib, tables.dev
        self.streams = [torch.cuda.Stream(self.dev) for _ in range(slots)]
        self._lits: Dict[tuple, object] = {}
        li, jt, st = tables.li, tables.jt, tables.st
        # filter + group-by: the plan (dense key slots) comes from the whole table once
        cols = {LINEITEM_IDS[k]: v for k, v in li.items()}
        self.gb_cols = cols
        self.gb_prog = compile_aggregate(LINEITEM_AGG, cols)
        self.gb_pred = compile_filter([["sd#7", "<=", "2470"]], {7: cols[7]})
        plan = L.GbPlan()
        scratch = torch.empty(256, dtype=torch.uint8, device=self.dev)
        L.check(self.lib.tqpk_groupby_plan(C.byref(self.gb_prog.spec), None, None, tables.n_fact, C.byref(plan),
                                           scratch.data_ptr(), torch.cuda.current_stream(self.dev).cuda_stream),
                "tqpk_groupby_plan")
        self.gb_plan = plan
        src, name, T, smem = jit.groupby_source(self.gb_prog.spec, self.gb_pred.struct, plan)
        self.gb_kernel, self.gb_T, self.gb_smem = jit.compile_kernel(src, name), T, smem
        self.gb_grid = jit.occupancy_grid(self.gb_kernel, T, smem, (tables.n_fact + 3) // 4)
        self.gb_out_dtypes = [dt for (_, _, _, _, dt) in self.gb_prog.outputs]
        ops = []
        from .dtypes import code_of
        for (_, op, a, b, dt) in self.gb_prog.outputs:
            ops += [op, a, b, code_of(dt)]
        self.gb_ops = (C.c_int32 * len(ops))(*ops)
        # join: probe filter on the probe side, build filter through the resident directory
        pcols = {22: jt["p_date"], 23: jt["p_price"], 24: jt["p_discount"]}
        self.j_prog = compile_aggregate({"keys": None, "results": [[[["sum", JOIN_VALUE], "#", "1"], "AS", "v#1"]]},
                                        pcols)
        self.j_reg = self.j_prog.spec.accs[self.j_prog.outputs[0][2]].reg
        self.j_ppred = compile_filter([["pd#22", ">", "1170"]], {22: jt["p_date"]})
        self.j_bpred = compile_filter([["bd#12", "<", "1170"]], {12: jt["b_date"]})
        src, name = jit.join_probe_source(self.j_prog.spec, self.j_reg, self.j_ppred.struct, self.j_bpred.struct)
        self.j_kernel = jit.compile_kernel(src, name)
        self.j_grid = jit.occupancy_grid(self.j_kernel, 256, 0, jit.probe_units(tables.n_fact))
        # star: A's filter through A's row directory
        fcols = {33: st["f_price"], 34: st["f_discount"]}
        self.s_prog = compile_aggregate(
            {"keys": None, "results": [[[["sum", [["p#33", "*", ["1.0", "-", "d#34"]]]], "#", "1"], "AS", "v#1"]]},
            fcols)
        self.s_reg = self.s_prog.spec.accs[self.s_prog.outputs[0][2]].reg
        self.s_apred = compile_filter([["cat#42", "=", "1"]], {42: st["a_cat"]})
        src, name = jit.star_probe_source(self.s_prog.spec, self.s_reg, None, self.s_apred.struct)
        self.s_kernel = jit.compile_kernel(src, name)
        self.s_grid = jit.occupancy_grid(self.s_kernel, 256, 0, jit.probe_units(tables.n_fact))
        self.topk_ws = {k: self.lib.tqpk_dense_topk_workspace_bytes(k) for k in (self.JOIN_K, self.STAR_K)}

    # -- literals, cached per (shape, constants)
    def _pred_lits(self, key, tree, cols):
        from . import jit
        from .predicate import compile_filter
        v = self._lits.get(key)
        if v is None:
            v = jit.pred_lits(compile_filter(tree, cols).struct)
            self._lits[key] = v
        return v

    # -- scratch layout per shape
    @staticmethod
    def _layout(sizes: Sequence[int]) -> Tuple[List[int], int]:
        offs, off = [], 0
        for s in sizes:
            offs.append(off)
            off += -(-int(s) // 256) * 256
        return offs, off

    def _sizes(self, req: Request) -> List[int]:
        if req.shape == "filter_groupby":
            K = int(self.gb_plan.slots)
            return ([int(self.gb_plan.ws_bytes)] + [K * 8 for _ in range(self.gb_prog.spec.n_keys)]
                    + [K * 8 for _ in self.gb_out_dtypes] + [8])
        if req.shape == "join":
            slots = self.t.doms["join"][1] - self.t.doms["join"][0] + 1
            k = self.JOIN_K
        else:
            slots = self.t.doms["c"][1] - self.t.doms["c"][0] + 1
            k = self.STAR_K
        return [slots * 8, slots * 4, self.topk_ws[k], k * 8, k * 8, k * 8, 8, 8]

    def scratch_bytes(self, req: Request) -> int:
        return self._layout(self._sizes(req))[1]

    def launch(self, req: Request, slot: int, ptr: int):
        import torch
        from . import jit
        stream = self.streams[slot]
        s = stream.cuda_stream
        offs, _ = self._layout(self._sizes(req))
        p = [ptr + o for o in offs]
        n = min(int(req.rows), self.t.n_fact)
        with torch.cuda.stream(stream):
            if req.shape == "filter_groupby":
                outs = self._launch_groupby(req, n, p, s)
            elif req.shape == "join":
                outs = self._launch_join(req, n, p, s)
            else:
                outs = self._launch_star(req, n, p, s)
            host = [torch.empty(o.shape, dtype=o.dtype, pin_memory=True) for o in outs]
            for h, o in zip(host, outs):
                h.copy_(o, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return (req, ev, host)

    def _view(self, ptr: int, n: int, dtype):
        """A device tensor over scratch memory (no allocation)."""
        import torch
        return _device_view(ptr, n, dtype, self.dev)

    def _launch_groupby(self, req, n, p, s):
        import torch
        from . import jit
        spec, plan = self.gb_prog.spec, self.gb_plan
        ws, K = p[0], int(plan.slots)
        nk = spec.n_keys
        keys = [self._view(p[1 + k], K, torch.int64 if spec.key_dtypes[k] == L.I64 else
                           {L.U8: torch.uint8, L.I8: torch.int8, L.I32: torch.int32, L.BOOL: torch.bool}[spec.key_dtypes[k]])
                for k in range(nk)]
        outs = [self._view(p[1 + nk + i], K, dt) for i, dt in enumerate(self.gb_out_dtypes)]
        groups = self._view(p[1 + nk + len(outs)], 1, torch.int64)
        L.check(self.lib.tqpk_groupby_prepare(C.byref(spec), C.byref(plan), ws, int(plan.ws_bytes), s),
                "tqpk_groupby_prepare")
        a = jit._Args()
        P = self.gb_pred.struct
        for c in range(P.n_cols):
            a.ptr(P.cols[c])
        a.blob(self._pred_lits(("gb",) + req.consts, [["sd#7", "<=", str(req.consts[0])]], {7: self.gb_cols[7]}))
        for k in range(nk):
            a.ptr(spec.keys[k])
        for c in range(spec.n_cols):
            a.ptr(spec.cols[c])
        a.i64(n)
        a.ptr(self.lib.tqpk_groupby_table(ws))
        a.i32(1)
        a.i32(1)
        a.i32(1)
        a.ptr(None)             # error word: none (the plan's domains come from the data)
        if n > 0:
            jit.launch(self.gb_kernel, self.gb_grid, self.gb_T, self.gb_smem, a, s, L.KID_GROUPBY)
        kp = (C.c_void_p * max(nk, 1))(*[k.data_ptr() for k in keys])
        oc = (C.c_void_p * len(outs))(*[o.data_ptr() for o in outs])
        L.check(self.lib.tqpk_groupby_emit_async(C.byref(spec), C.byref(plan), ws, kp, len(outs), self.gb_ops, oc,
                                                 groups.data_ptr(), s), "tqpk_groupby_emit_async")
        return keys + outs + [groups]

    def _topk_outputs(self, p, k, s, slots, key_min, counts: bool):
        import torch
        sum_t, cnt_t = self._view(p[0], slots, torch.float64), self._view(p[1], slots, torch.int32)
        okeys, ovals, ocnts = (self._view(p[3], k, torch.int64), self._view(p[4], k, torch.float64),
                               self._view(p[5], k, torch.int64))
        ocount, ogroups = self._view(p[6], 1, torch.int64), self._view(p[7], 1, torch.int64)
        return sum_t, cnt_t, okeys, ovals, ocnts, ocount, ogroups

    def _launch_join(self, req, n, p, s):
        import torch
        from . import jit
        mn, mx = self.t.doms["join"]
        slots = mx - mn + 1
        sum_t, occ_t, okeys, ovals, ocnts, ocount, ogroups = self._topk_outputs(p, self.JOIN_K, s, slots, mn, False)
        sum_t.zero_()
        occ_t.zero_()
        jt = self.t.jt
        pp, bp = self.j_ppred.struct, self.j_bpred.struct
        a = jit._Args()
        for c in range(pp.n_cols):
            a.ptr(pp.cols[c])
        a.blob(self._pred_lits(("jp", req.consts[0]), [["pd#22", ">", str(req.consts[0])]], {22: jt["p_date"]}))
        for c in range(bp.n_cols):
            a.ptr(bp.cols[c])
        a.blob(self._pred_lits(("jb", req.consts[1]), [["bd#12", "<", str(req.consts[1])]], {12: jt["b_date"]}))
        spec = self.j_prog.spec
        for c in range(spec.n_cols):
            a.ptr(spec.cols[c])
        a.ptr(jt["p_fk"].data_ptr())
        a.i32(L.I32)
        a.i64(n)
        a.i64(mn)
        a.i64(slots)
        a.ptr(self.t.dirs["join"].data_ptr())
        a.ptr(sum_t.data_ptr())
        a.ptr(occ_t.data_ptr())
        a.i32(1)
        a.i32(1)
        a.i32(1)
        if n > 0:
            jit.launch(self.j_kernel, self.j_grid, 256, 0, a, s, L.KID_PIPE_PROBE)
        L.check(self.lib.tqpk_dense_topk(sum_t.data_ptr(), occ_t.data_ptr(), slots, mn, self.JOIN_K, 1, p[2],
                                         self.topk_ws[self.JOIN_K], okeys.data_ptr(), ovals.data_ptr(), None,
                                         ocount.data_ptr(), ogroups.data_ptr(), s), "tqpk_dense_topk")
        return [okeys, ovals, ocount, ogroups]

    def _launch_star(self, req, n, p, s):
        import torch
        from . import jit
        st, doms = self.t.st, self.t.doms
        cmn, cmx = doms["c"]
        cs = cmx - cmn + 1
        sum_t, cnt_t, okeys, ovals, ocnts, ocount, ogroups = self._topk_outputs(p, self.STAR_K, s, cs, cmn, True)
        sum_t.zero_()
        cnt_t.zero_()
        ap = self.s_apred.struct
        a = jit._Args()
        a.blob(jit.pred_lits(None))
        for c in range(ap.n_cols):
            a.ptr(ap.cols[c])
        a.blob(self._pred_lits(("sa", req.consts[0]), [["cat#42", "=", str(req.consts[0])]], {42: st["a_cat"]}))
        spec = self.s_prog.spec
        for c in range(spec.n_cols):
            a.ptr(spec.cols[c])
        a.ptr(st["f_fka"].data_ptr())
        a.ptr(st["f_fkb"].data_ptr())
        a.i64(n)
        for name in ("a", "b", "c"):
            mn, mx = doms[name]
            a.i64(mn)
            a.i64(mx - mn + 1)
            a.ptr(self.t.dirs[name].data_ptr())
        a.ptr(sum_t.data_ptr())
        a.ptr(cnt_t.data_ptr())
        a.i32(1)
        a.i32(1)
        a.i32(1)
        if n > 0:
            jit.launch(self.s_kernel, self.s_grid, 256, 0, a, s, L.KID_STAR_PROBE)
        L.check(self.lib.tqpk_dense_topk(sum_t.data_ptr(), cnt_t.data_ptr(), cs, cmn, self.STAR_K, 1, p[2],
                                         self.topk_ws[self.STAR_K], okeys.data_ptr(), ovals.data_ptr(),
                                         ocnts.data_ptr(), ocount.data_ptr(), ogroups.data_ptr(), s),
                "tqpk_dense_topk")
        return [okeys, ovals, ocnts, ocount, ogroups]

    def done(self, handle) -> bool:
        return handle[1].query()

    def finish(self, handle):
        """Host arrays of the request's result (trimmed to the group / top-k count)."""
        req, ev, host = handle
        ev.synchronize()
        h = [x.numpy() for x in host]
        if req.shape == "filter_groupby":
            G = int(h[-1][0])
            if G < 0:
                L.check(G, "filter_groupby emit")
            nk = self.gb_prog.spec.n_keys
            keys = [x[:G].copy() for x in h[:nk]]
            outs = {oid: x[:G].copy() for (oid, *_), x in zip(self.gb_prog.outputs, h[nk:-1])}
            return {"keys": keys, "outs": outs, "groups": G}
        if req.shape == "join":
            m = int(h[2][0])
            return {"keys": h[0][:m].copy(), "vals": h[1][:m].copy(), "groups": int(h[3][0])}
        m = int(h[3][0])
        return {"keys": h[0][:m].copy(), "vals": h[1][:m].copy(), "counts": h[2][:m].copy(), "groups": int(h[4][0])}


class _CudaArray:
    """A raw device byte range exposed through the CUDA array interface."""

    def __init__(self, ptr: int, nbytes: int):
        self.__cuda_array_interface__ = {"shape": (max(int(nbytes), 1),), "typestr": "|u1", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def _device_view(ptr: int, n: int, dtype, device):
    """A torch tensor aliasing n elements of device memory at ptr (the arena owns the memory)."""
    import torch
    itemsize = torch.empty((), dtype=dtype).element_size()
    return torch.as_tensor(_CudaArray(ptr, n * itemsize), device=device).view(dtype)[:n]
