"""Many uneven query instances in one persistent launch (csrc/batch.cu).

An instance is either
* ``JoinInstance``: Filter(build), Filter(probe), inner join on a unique
  build key, sum(expr) by build key, top-k (k <= 32); or
* ``GroupByInstance``: Filter, group by dense keys with the aggregate
  ``results`` of ``tqp_hash_aggregate`` (sum/avg/count/min/max), groups in key
  order.

``Batch`` describes every instance to the library, cuts each phase into work
items whose size the ``Autotuner`` picks per instance, and runs them all in
one ``tqpk_batch_run`` launch.  ``capture()`` records the reset memsets and
the launch in a CUDA graph, ``replay()`` re-runs the whole batch with one
graph launch.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib as L
from .dtypes import code_of, dtype_of
from .expr import compile_aggregate, require_f64_outputs
from .predicate import compile_filter


@dataclass
class JoinInstance:
    build_keys: torch.Tensor
    key_domain: tuple
    probe_fk: torch.Tensor
    build_cols: Dict[int, torch.Tensor]
    build_filter: object
    probe_cols: Dict[int, torch.Tensor]
    probe_filter: object
    value_tree: object
    k: int = 10
    descending: bool = True


@dataclass
class GroupByInstance:
    args: dict                         # tqp_hash_aggregate arguments (keys, results, out agg ids)
    columns: Dict[int, torch.Tensor]
    filter_tree: object
    filter_cols: Dict[int, torch.Tensor]
    key_domains: Sequence[tuple]       # (min, max) per group key: table statistics
    n_rows: int = 0


class Autotuner:
    """Work-item sizes (rows per item) and group-table placement per instance.

    ``calibrate()`` times single-instance batches on the device for each size
    class and candidate item size and keeps the fastest; the table can be
    saved/loaded as JSON.  Until calibrated, items are sized so an instance
    spreads over about two items per SM, within [4096, 1 << 20] rows."""

    CANDIDATES = (4096, 16384, 65536, 262144, 1048576)

    def __init__(self, table: Optional[dict] = None):
        self.table = dict(table or {})
        self.sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count \
            if torch.cuda.is_available() else 152

    @staticmethod
    def size_class(n: int) -> int:
        return max(0, int(math.log2(max(n, 1))))

    def rows_per_item(self, kind: str, n: int) -> int:
        key = f"{kind}:{self.size_class(n)}"
        if key in self.table:
            return int(self.table[key])
        target = max(1, n // (2 * self.sms))
        return int(min(1 << 20, max(4096, 1 << int(math.ceil(math.log2(max(target, 1)))))))

    def prefer_private(self, kind: str, slots: int, n_accs: int) -> bool:
        return self.table.get(f"{kind}:private", True) and slots * n_accs * 8 * 256 <= 96 * 1024

    def save(self, path):
        Path(path).write_text(json.dumps(self.table, indent=1, sort_keys=True))

    @classmethod
    def load(cls, path):
        p = Path(path)
        return cls(json.loads(p.read_text()) if p.exists() else None)

    def calibrate(self, make_instance, kind: str, sizes: Sequence[int], reps: int = 5):
        """make_instance(n) -> instance; records the fastest rows_per_item per size class."""
        for n in sizes:
            best = None
            for rpi in self.CANDIDATES:
                if rpi > max(4096, n):
                    continue
                self.table[f"{kind}:{self.size_class(n)}"] = rpi
                b = Batch([make_instance(n)], self)
                b.capture()
                b.replay()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(reps):
                    b.replay()
                torch.cuda.synchronize()
                dt = (time.perf_counter() - t0) / reps
                if best is None or dt < best[0]:
                    best = (dt, rpi)
            self.table[f"{kind}:{self.size_class(n)}"] = best[1]
        return self.table


class Batch:
    def __init__(self, instances: List[object], tuner: Optional[Autotuner] = None):
        self.lib = L.load()
        self.tuner = tuner or Autotuner()
        self.instances = instances
        self.dev = None
        n = len(instances)
        self.rec_bytes = self.lib.tqpk_batch_record_bytes()
        self.h_recs = (C.c_uint8 * (self.rec_bytes * n))()
        self.keep: list = []
        self.outs: list = []
        for i, inst in enumerate(instances):
            rec = C.addressof(self.h_recs) + i * self.rec_bytes
            if isinstance(inst, JoinInstance):
                self.outs.append(self._describe_join(rec, inst))
            else:
                self.outs.append(self._describe_groupby(rec, inst))
        need = self.lib.tqpk_batch_items(C.addressof(self.h_recs), n, None, 0)
        item_bytes = 24
        h_items = (C.c_uint8 * (item_bytes * need))()
        got = self.lib.tqpk_batch_items(C.addressof(self.h_recs), n, C.addressof(h_items), need)
        assert got == need
        self.n_items = int(need)
        self.h_items = bytes(h_items)
        self.d_recs = torch.frombuffer(bytearray(self.h_recs), dtype=torch.uint8).to(self.dev)
        self.d_items = torch.frombuffer(bytearray(h_items), dtype=torch.uint8).to(self.dev)
        self.ctl = torch.zeros(self.lib.tqpk_batch_ctl_bytes(n), dtype=torch.uint8, device=self.dev)
        self.grid = int(self.lib.tqpk_batch_grid())
        self.graph = None

    # ------------------------------------------------------------------ describe
    def _describe_join(self, rec, inst: JoinInstance):
        dev = inst.build_keys.device
        self.dev = dev
        bk, pk = inst.build_keys.contiguous(), inst.probe_fk.contiguous()
        bpred = compile_filter(inst.build_filter, inst.build_cols) if inst.build_filter is not None else None
        ppred = compile_filter(inst.probe_filter, inst.probe_cols) if inst.probe_filter is not None else None
        prog = compile_aggregate({"keys": None, "results": [[[["sum", inst.value_tree], "#", "1"], "AS", "v#1"]]},
                                 inst.probe_cols)
        require_f64_outputs(prog, "batched join")
        vreg = prog.spec.accs[prog.outputs[0][2]].reg
        kmin, kmax = map(int, inst.key_domain)
        ws = torch.empty(self.lib.tqpk_batch_join_workspace_bytes(kmin, kmax), dtype=torch.uint8, device=dev)
        out_keys = torch.empty(inst.k, dtype=torch.int64, device=dev)
        out_vals = torch.empty(inst.k, dtype=torch.float64, device=dev)
        out_count = torch.zeros(1, dtype=torch.int64, device=dev)
        groups = torch.zeros(1, dtype=torch.int64, device=dev)
        rb = self.tuner.rows_per_item("join_build", bk.numel())
        rp = self.tuner.rows_per_item("join_probe", pk.numel())
        L.check(self.lib.tqpk_batch_describe_join(
            rec, bk.data_ptr() if bk.numel() else None, code_of(bk.dtype), bk.numel(),
            C.byref(bpred.struct) if bpred else None, kmin, kmax, pk.data_ptr() if pk.numel() else None,
            code_of(pk.dtype), pk.numel(), C.byref(ppred.struct) if ppred else None, C.byref(prog.spec), vreg,
            inst.k, int(inst.descending), ws.data_ptr(), ws.numel(), out_keys.data_ptr(), out_vals.data_ptr(),
            out_count.data_ptr(), groups.data_ptr(), rb, rp), "tqpk_batch_describe_join")
        self.keep += [bk, pk, bpred, ppred, prog, ws]
        return {"kind": "join", "keys": out_keys, "vals": out_vals, "count": out_count, "groups": groups}

    def _describe_groupby(self, rec, inst: GroupByInstance):
        cols = inst.columns
        dev = next(iter(cols.values())).device
        self.dev = dev
        prog = compile_aggregate(inst.args, cols)
        require_f64_outputs(prog, "batched group-by")
        pred = compile_filter(inst.filter_tree, inst.filter_cols) if inst.filter_tree is not None else None
        nk = prog.spec.n_keys
        kmin = (C.c_int64 * nk)(*[int(d[0]) for d in inst.key_domains])
        kmax = (C.c_int64 * nk)(*[int(d[1]) for d in inst.key_domains])
        K = int(np.prod([int(d[1]) - int(d[0]) + 1 for d in inst.key_domains]))
        n = int(next(iter(cols.values())).shape[0])
        spi = max(256, min(1 << 16, K))
        ws = torch.empty(self.lib.tqpk_batch_groupby_workspace_bytes(C.byref(prog.spec), kmin, kmax, spi),
                         dtype=torch.uint8, device=dev)
        keys = [torch.empty(K, dtype=dtype_of(prog.spec.key_dtypes[k]), device=dev) for k in range(nk)]
        outs = [torch.empty(K, dtype=dt, device=dev) for (_, _, _, _, dt) in prog.outputs]
        ops = []
        for (_, op, a, b, dt) in prog.outputs:
            ops += [op, a, b, code_of(dt)]
        groups = torch.zeros(1, dtype=torch.int64, device=dev)
        rpi = self.tuner.rows_per_item("groupby", n)
        priv = self.tuner.prefer_private("groupby", K, prog.spec.n_accs)
        kp = (C.c_void_p * max(nk, 1))(*[k.data_ptr() for k in keys])
        op_arr = (C.c_int32 * max(len(ops), 1))(*ops)
        oc = (C.c_void_p * max(len(outs), 1))(*[o.data_ptr() for o in outs])
        L.check(self.lib.tqpk_batch_describe_groupby(
            rec, C.byref(prog.spec), C.byref(pred.struct) if pred else None, n, kmin, kmax, ws.data_ptr(),
            ws.numel(), kp, len(outs), op_arr, oc, groups.data_ptr(), rpi, spi, int(priv)),
            "tqpk_batch_describe_groupby")
        self.keep += [prog, pred, ws]
        return {"kind": "groupby", "keys": keys, "outs": outs, "groups": groups, "prog": prog}

    # ------------------------------------------------------------------ run
    def run(self, stream=None):
        s = (stream or torch.cuda.current_stream(self.dev)).cuda_stream
        L.check(self.lib.tqpk_batch_reset(C.addressof(self.h_recs), self.d_recs.data_ptr(), len(self.instances),
                                          self.ctl.data_ptr(), s), "tqpk_batch_reset")
        L.check(self.lib.tqpk_batch_run(self.d_recs.data_ptr(), len(self.instances), self.d_items.data_ptr(),
                                        self.n_items, self.ctl.data_ptr(), self.grid, s), "tqpk_batch_run")

    def capture(self):
        self.run()                       # sets kernel attributes outside the capture
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.run()
        return self.graph

    def replay(self):
        self.graph.replay()

    def item_timeline(self) -> np.ndarray:
        """Runs the batch once (outside any graph) with the per-item timeline on.

        Returns a structured array, one row per work item: inst, phase, begin, end
        (rows or slots), and dequeue / dependency-met / completion times in
        microseconds from the first dequeue, plus the SM id."""
        tr = torch.zeros(self.n_items * 4, dtype=torch.int64, device=self.dev)
        L.check(self.lib.tqpk_batch_set_trace(tr.data_ptr()), "tqpk_batch_set_trace")
        try:
            self.run()
            torch.cuda.synchronize()
        finally:
            self.lib.tqpk_batch_set_trace(None)
        t = tr.cpu().numpy().reshape(-1, 4)
        it = np.frombuffer(self.h_items, dtype=[("inst", "<i4"), ("phase", "<i4"), ("begin", "<i8"), ("end", "<i8")])
        out = np.zeros(self.n_items, dtype=[("inst", "i4"), ("phase", "i4"), ("begin", "i8"), ("end", "i8"),
                                            ("t_deq", "f8"), ("t_ready", "f8"), ("t_done", "f8"), ("sm", "i4")])
        for f in ("inst", "phase", "begin", "end"):
            out[f] = it[f]
        t0 = t[:, 0].min()
        out["t_deq"], out["t_ready"], out["t_done"] = (t[:, 0] - t0) / 1e3, (t[:, 1] - t0) / 1e3, (t[:, 2] - t0) / 1e3
        out["sm"] = t[:, 3]
        return out

    def check_error(self):
        err = C.c_int(0)
        L.check(self.lib.tqpk_batch_error(self.ctl.data_ptr(), C.byref(err),
                                          torch.cuda.current_stream(self.dev).cuda_stream), "tqpk_batch_error")
        if err.value:
            L.check(err.value, "batched run")

    def results(self):
        """Per instance: join -> (keys, sums, groups); groupby -> ({out id: column}, key columns, groups)."""
        self.check_error()
        res = []
        for o in self.outs:
            if o["kind"] == "join":
                m = int(o["count"].item())
                res.append((o["keys"][:m].cpu().numpy(), o["vals"][:m].cpu().numpy(), int(o["groups"].item())))
            else:
                g = int(o["groups"].item())
                prog = o["prog"]
                outs = {oid: col[:g].cpu().numpy() for (oid, *_), col in zip(prog.outputs, o["outs"])}
                keys = [k[:g].cpu().numpy() for k in o["keys"]]
                res.append((outs, keys, g))
        return res
