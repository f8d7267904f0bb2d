#!/usr/bin/env python3
"""Benchmark of the TQP-Inmem relational hot path on GB300.

The default run (``--workload all``) measures every workload and prints one JSON line: the
headline is the filtered equi-join + aggregate + top-10 query -- build side 1,500,000 rows
(key = permutation of 1..1.5M, date), filter date < 1170; probe side 6,001,215 rows (fk uniform
over the build keys, date, price, discount), filter date > 1170; sum(price * (1 - discount))
grouped by build key; top 10 by the sum, descending -- and ``workloads`` holds one record each
for the filter + group-by query (6,001,215 rows), the star join (59,986,052 fact rows), the 64
uneven instances of the batched form and the serving loop.  ``--workload NAME`` runs one.

Synthetic seeded data with the TPC-H-like distributions of tqpk.datagen (TPC-H itself is not
available).  One step = one run of the whole query over inputs resident in HBM, through the fused
pipeline (one CUDA-graph replay).  ``e2e`` = the same query through the drop-in operators
(tqp_filter, join_vortex, tqp_hash_aggregate, tqp_sort) with the input columns copied from pinned
host memory and the result copied back inside the timed region; ``dropin`` = the drop-in
operators over resident columns.  Metric: rows/s = probe (fact) rows / step time.

Beside them: ``reference_cuda`` = TQP-Inmem's own operators (compiled from its source into
oracle/_ref, run unmodified through their public API, main.py's plan order, a synchronisation
after every operator as main.py:273-274) on torch CUDA on the same GPU, resident and end to end;
``cpu_baseline`` = the same operators on their CPU path (torch CPU, every host core), a bounded
sample.  ``--impl reference`` is that CPU path alone, on the workload's full-size query.
"""
from __future__ import annotations

import argparse
from typing import Optional
import copy
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for p in (str(ROOT), str(ROOT / "tqp-inmem_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

PEAK_FALLBACK_GBS = 6800.0


# ---------------------------------------------------------------------------- workloads
_PINNED = {}


def d2h_all(tensors):
    """Results to pinned host memory: every copy queued, then one synchronisation.  The pinned
    buffers are kept per (column, dtype) and grown as needed (pinning memory costs tens of us a
    call); the returned arrays are copies."""
    import torch
    out = {}
    for c, t in tensors.items():
        buf = _PINNED.get((c, t.dtype))
        if buf is None or buf.numel() < t.numel():
            buf = _PINNED[(c, t.dtype)] = torch.empty(max(t.numel(), 1024), dtype=t.dtype, pin_memory=True)
        h = buf[:t.numel()].view(t.shape)
        h.copy_(t, non_blocking=True)
        out[c] = h
    torch.cuda.current_stream().synchronize()
    return {c: h.clone() for c, h in out.items()}


def plan_args(args):
    """A fresh copy of an operator's argument dict, as a plan executor hands each operator its
    own: the top-level lists and dicts are copied (the operators append to 'input ids' and pop
    from 'mask map'); the parsed trees inside them are only read and stay shared."""
    return {k: (list(v) if isinstance(v, list) else dict(v) if isinstance(v, dict) else v) for k, v in args.items()}


class JoinAggTop10:
    name = "join_agg_top10"
    NB, NP = 1_500_000, 6_001_215

    def __init__(self):
        from tqpk import datagen
        self.dg = datagen
        self.t = datagen.join_tables(self.NB, self.NP, seed=7)
        self.fact_rows = self.NP
        self.config = {
            "workload": "filtered equi-join + sum(price*(1-discount)) group by build key + top-10",
            "build_rows": self.NB, "probe_rows": self.NP,
            "build_filter": f"date < {datagen.BUILD_DATE_LT}", "probe_filter": f"date > {datagen.PROBE_DATE_GT}",
            "k": 10, "key_dtype": "int32", "l2": "flushed between steps (256 MB write)",
        }
        self.set_args()
        self.cols = {11: self.t["b_key"], 12: self.t["b_date"], 21: self.t["p_fk"], 22: self.t["p_date"],
                     23: self.t["p_price"], 24: self.t["p_discount"]}
        self.types = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}

    def set_args(self):
        """The operators' argument dicts of the query."""
        from tqpk import datagen
        self.f1 = {"filter tree": [["bd#12", "<", str(datagen.BUILD_DATE_LT)]], "materialized in": [12],
                   "out mask id": 901}
        self.f2 = {"filter tree": [["pd#22", ">", str(datagen.PROBE_DATE_GT)]], "materialized in": [22],
                   "out mask id": 902}
        self.jargs = {"left group": [11, 12], "right group": [21, 22, 23, 24], "materialized in": [11, 21, 23, 24],
                      "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}
        self.value_tree = [["p#23", "*", ["1.0", "-", "d#24"]]]
        self.aargs = {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
                      "results": ["k#11", [[["sum", self.value_tree], "#", "301"], "AS", "rev#302"]],
                      "out agg ids": [302]}
        self.targs = {"limit": 10, "input ids": [11, 302], "key ids": [302], "key orders": [True]}

    # algorithmic bytes: every input column read once, the outputs written once
    def algorithmic_bytes(self):
        return self.NB * 8 + self.NP * 24

    def dominant(self):
        from tqpk import _lib as L
        from tqpk import jit
        # probe + aggregate: reads fk, date, price, discount of every probe row once
        return L.KID_PIPE_PROBE, "tqpk_q_join_probe" if jit.available() else "k_pl_probe_agg", self.NP * 24

    def setup_device(self, dev):
        import torch
        from tqpk.pipeline import JoinAggTopK
        self.d = {c: torch.from_numpy(a).to(dev) for c, a in self.cols.items()}
        self.key_min, self.key_max = int(self.t["b_key"].min()), int(self.t["b_key"].max())  # table statistic
        self.pipe = JoinAggTopK(self.d[11], self.key_min, self.key_max, self.d[21],
                                {12: self.d[12]}, self.f1["filter tree"],
                                {22: self.d[22], 23: self.d[23], 24: self.d[24]}, self.f2["filter tree"],
                                self.value_tree, k=10, descending=True)
        self.host = {c: torch.from_numpy(a).pin_memory() for c, a in self.cols.items()}
        self.dev = dev

    def step_device(self):
        self.pipe.run()

    def capture(self):
        self.pipe.capture()

    def step_graph(self):
        self.pipe.replay()

    def device_result(self):
        return self.pipe.result()[:2]

    def step_e2e(self):
        """Drop-in operators with host buffers: H2D, the plan, D2H of the top-10."""
        import torch
        from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
        from tqpk.variable import Variable
        if not hasattr(self, "staged"):
            from tqpk.ingress import ColumnStager
            self.staged = ColumnStager(self.dev)
        tg = self.staged.stage(self.host, self.types, (12, 22, 11, 21, 23, 24))
        tqp_filter(True, tg, plan_args(self.f1), None, None, None, "f1")
        tqp_filter(True, tg, plan_args(self.f2), None, None, None, "f2")
        join_vortex(True, tg, plan_args(self.jargs), 11, 21, [], "inner", None, None, "j")
        tqp_hash_aggregate(True, tg, plan_args(self.aargs), None, None, "a")
        tqp_sort(True, tg, plan_args(self.targs), True, "t")
        res = d2h_all({11: tg[11].tensor, 302: tg[302].tensor})
        keys, vals = res[11], res[302]
        h2d = sum(h.numel() * h.element_size() for h in self.host.values())
        d2h = keys.numel() * keys.element_size() + vals.numel() * vals.element_size()
        return (keys.numpy().reshape(-1), vals.numpy()), h2d, d2h

    def ref_plan(self, R, tg, pool, ge, sync):
        """main.py's plan over TQP-Inmem's own operators: Filter, Filter, Join, Aggregate,
        take ordered (main.py:152-253), synchronising after each operator (main.py:273-274)."""
        R.filter.tqp_filter(ge, tg, plan_args(self.f1), None, None, pool, "f1"); sync()
        R.filter.tqp_filter(ge, tg, plan_args(self.f2), None, None, pool, "f2"); sync()
        R.hashjoin.join_vortex(ge, tg, plan_args(self.jargs), 11, 21, [], "inner", None, pool, "j"); sync()
        R.aggregate.tqp_hash_aggregate(ge, tg, plan_args(self.aargs), pool, None, "a"); sync()
        groups = int(tg[11].tensor.shape[0])
        R.sort.tqp_sort(ge, tg, plan_args(self.targs), True, "t"); sync()
        return (tg[11].tensor.cpu().numpy().reshape(-1), tg[302].tensor.cpu().numpy()), groups

    def step_dropin(self, tg):
        """The drop-in operators over resident columns (no copies)."""
        from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
        tqp_filter(True, tg, plan_args(self.f1), None, None, None, "f1")
        tqp_filter(True, tg, plan_args(self.f2), None, None, None, "f2")
        join_vortex(True, tg, plan_args(self.jargs), 11, 21, [], "inner", None, None, "j")
        tqp_hash_aggregate(True, tg, plan_args(self.aargs), None, None, "a")
        tqp_sort(True, tg, plan_args(self.targs), True, "t")
        return tg[302].tensor

    def plan(self):
        """The query as a plan executor holds it (main.py:123-130): the operators in order and
        each one's argument dict, keyed by operator id."""
        ops = [3, 4, 5, 6, 7]
        args = {3: dict(plan_args(self.f1), name="Filter"), 4: dict(plan_args(self.f2), name="Filter"),
                5: dict(plan_args(self.jargs), name="Join", **{"left keys": [11], "right keys": [21],
                                                                "join type": "Inner"}),
                6: dict(plan_args(self.aargs), name="Aggregate"), 7: dict(plan_args(self.targs), name="take ordered")}
        return ops, args

    def step_e2e_fused(self):
        """A plan executor that offers each run of operators to try_fused before dispatching them one
        by one (main.py:123-253 with the loop of tqpk.operators.fused); host buffers as step_e2e."""
        from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort, try_fused
        if not hasattr(self, "staged"):
            from tqpk.ingress import ColumnStager
            self.staged = ColumnStager(self.dev)
        tg = self.staged.stage(self.host, self.types, (12, 22, 11, 21, 23, 24))
        ops, args = self.plan()
        i = 0
        while i < len(ops):
            m = try_fused(True, tg, ops, args, i)
            if m:
                i += m
                continue
            a = args[ops[i]]
            if a["name"] == "Filter":
                tqp_filter(True, tg, a, None, None, None, "f")
            elif a["name"] == "Join":
                join_vortex(True, tg, a, a["left keys"][0], a["right keys"][0], [], "inner", None, None, "j")
            elif a["name"] == "Aggregate":
                tqp_hash_aggregate(True, tg, a, None, None, "a")
            else:
                tqp_sort(True, tg, a, True, "t")
            i += 1
        from tqpk.variable import host_values      # the fused path read the rows with its count
        keys, vals = host_values(tg[11]), host_values(tg[302])
        h2d = sum(h.numel() * h.element_size() for h in self.host.values())
        d2h = keys.nbytes + vals.nbytes
        return (keys.reshape(-1), vals), h2d, d2h

    def oracle(self, cols=None):
        from oracle import tqp_oracle as O
        cols = self.cols if cols is None else cols
        oc = dict(cols)
        oc[901] = O.eval_filter(self.f1["filter tree"], {12: cols[12]})
        oc[902] = O.eval_filter(self.f2["filter tree"], {22: cols[22]})
        res, _ = O.join_vortex(oc, copy.deepcopy(self.jargs), 11, 21, "inner")
        agg = O.tqp_hash_aggregate(res, copy.deepcopy(self.aargs))
        top = O.tqp_sort({11: agg[11], 302: agg[302]}, self.targs, True)
        return top[11].reshape(-1), top[302]


class FilterGroupBy:
    name = "filter_groupby"
    N = 6_001_215

    def __init__(self):
        from tqpk import datagen
        self.t = datagen.lineitem(self.N, seed=42)
        self.fact_rows = self.N
        self.config = {"workload": "filter ship_date <= 2470 + group by (flag, status): 4 sums, 3 avgs, count",
                       "rows": self.N, "l2": "flushed between steps (256 MB write)"}
        ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
        self.cols = {ids[k]: v for k, v in self.t.items()}
        self.types = {1: "float", 2: "float", 3: "float", 4: "float", 5: "int", 6: "int", 7: "date"}
        self.fargs = {"filter tree": [[["isnotnull", ["ship_date#7"]], "AND",
                                       ["ship_date#7", "<=", str(datagen.SHIP_DATE_MAX)]]],
                      "materialized in": [7], "out mask id": 900}
        self.aargs = {"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 3, 4, 5, 6],
                      "results": ["flag#5", "status#6",
                                  [[["sum", ["quantity#1"]], "#", "101"], "AS", "a#201"],
                                  [[["sum", ["price#2"]], "#", "102"], "AS", "b#202"],
                                  [[["sum", [["price#2", "*", ["1.0", "-", "discount#3"]]]], "#", "103"], "AS", "c#203"],
                                  [[["sum", [[["price#2", "*", ["1.0", "-", "discount#3"]], "*", ["1.0", "+", "tax#4"]]]],
                                    "#", "104"], "AS", "d#204"],
                                  [[["avg", ["quantity#1"]], "#", "105"], "AS", "e#205"],
                                  [[["avg", ["price#2"]], "#", "106"], "AS", "f#206"],
                                  [[["avg", ["discount#3"]], "#", "107"], "AS", "g#207"],
                                  [[["count", ["1"]], "#", "108L"], "AS", "h#208"]],
                      "out agg ids": [201, 202, 203, 204, 205, 206, 207, 208],
                      "mask map": {1: 900, 2: 900, 3: 900, 4: 900, 5: 900, 6: 900}}
        self.sargs = {"input ids": [5, 6, 201, 202, 203, 204, 205, 206, 207, 208], "key ids": [5, 6],
                      "key orders": [False, False]}

    def algorithmic_bytes(self):
        return self.N * 38

    def fp64_ops(self):
        """FP64 work per launch of the accumulation kernel, for every row that passes the filter:
        (operations, operations per row, instructions per row).  Operations: the float arithmetic
        of the expression program and one add per float sum accumulator.  Instructions: what the
        generated kernel issues, where a product read only by a sum accumulates as one fused
        multiply-add and x * (1 - y) is one fused multiply-add."""
        from tqpk import _lib as L
        from tqpk import jit
        S = self.prog.spec
        arith = sum(1 for i in range(S.n_expr) if S.expr[i].type == L.F64 and S.expr[i].op in
                    (L.X_ADD, L.X_SUB, L.X_MUL, L.X_DIV))
        sums = sum(1 for a in range(S.n_accs) if S.accs[a].kind == L.ACC_SUM and S.accs[a].type == L.F64)
        instr = arith + sums - len(jit._fusable_products(S)) - len(jit._contractions(S, S.n_expr))
        passing = int((self.t["ship_date"] <= 2470).sum())
        return (arith + sums) * passing, arith + sums, instr

    def dominant(self):
        from tqpk import _lib as L
        from tqpk import jit
        # filter + group-by: ship_date (4 B), quantity/price/discount/tax (4 x 8 B), flag, status (1 B each)
        return L.KID_GROUPBY, "tqpk_q_groupby" if jit.available() else "k_groupby_dense", self.N * 38

    def setup_device(self, dev):
        import torch
        from tqpk.expr import compile_aggregate
        from tqpk.predicate import compile_filter
        self.d = {c: torch.from_numpy(a).to(dev) for c, a in self.cols.items()}
        self.pred = compile_filter(self.fargs["filter tree"], {7: self.d[7]})
        a = copy.deepcopy(self.aargs)
        a.pop("mask map")
        self.prog = compile_aggregate(a, self.d)
        self.host = {c: torch.from_numpy(a).pin_memory() for c, a in self.cols.items()}
        self.dev = dev
        self.last = None
        from tqpk import jit
        self.pipe = None
        if jit.available():
            from tqpk.pipeline import GroupByPipeline
            doms = [(int(self.cols[c].min()), int(self.cols[c].max())) for c in (5, 6)]   # table statistics
            self.pipe = GroupByPipeline(self.aargs, {c: self.d[c] for c in range(1, 7)}, self.fargs["filter tree"],
                                        {7: self.d[7]}, doms)

    def step_device(self):
        if self.pipe is not None:
            self.pipe.run()
            return
        from tqpk.ops import groupby
        self.last = groupby(self.prog, self.N, self.dev, pred=self.pred)

    def capture(self):
        if self.pipe is None:
            raise AttributeError("no graph without the runtime compiler")
        self.pipe.capture()

    def step_graph(self):
        self.pipe.replay()

    def device_result(self):
        keys, outs, G = self.pipe.result() if self.pipe is not None else self.last[:3]
        return [k.cpu().numpy() for k in keys], {o: v.cpu().numpy() for o, v in outs.items()}

    def step_e2e(self):
        from tqpk.operators import tqp_filter, tqp_hash_aggregate, tqp_sort
        from tqpk.variable import Variable
        if not hasattr(self, "staged"):
            from tqpk.ingress import ColumnStager
            self.staged = ColumnStager(self.dev)
        tg = self.staged.stage(self.host, self.types, (7, 5, 6, 1, 2, 3, 4))
        tqp_filter(True, tg, plan_args(self.fargs), None, None, None, "f")
        tqp_hash_aggregate(True, tg, plan_args(self.aargs), None, None, "a")
        tqp_sort(True, tg, plan_args(self.sargs), False, "s")
        out = {c: v.numpy() for c, v in d2h_all({c: tg[c].tensor for c in self.sargs["input ids"]}).items()}
        h2d = sum(h.numel() * h.element_size() for h in self.host.values())
        d2h = sum(v.nbytes for v in out.values())
        return out, h2d, d2h

    def ref_plan(self, R, tg, pool, ge, sync):
        """main.py's plan over TQP-Inmem's own operators: Filter, Aggregate, Sort."""
        R.filter.tqp_filter(ge, tg, plan_args(self.fargs), None, None, pool, "f"); sync()
        R.aggregate.tqp_hash_aggregate(ge, tg, plan_args(self.aargs), pool, None, "a"); sync()
        R.sort.tqp_sort(ge, tg, plan_args(self.sargs), False, "s"); sync()
        out = {c: tg[c].tensor.cpu().numpy() for c in self.sargs["input ids"]}
        return out, int(out[5].shape[0])          # the oracle's form: column id -> array

    def step_dropin(self, tg):
        from tqpk.operators import tqp_filter, tqp_hash_aggregate, tqp_sort
        tqp_filter(True, tg, plan_args(self.fargs), None, None, None, "f")
        tqp_hash_aggregate(True, tg, plan_args(self.aargs), None, None, "a")
        tqp_sort(True, tg, plan_args(self.sargs), False, "s")
        return tg[201].tensor

    def oracle(self, cols=None):
        from oracle import tqp_oracle as O
        cols = dict(self.cols if cols is None else cols)
        cols[900] = O.eval_filter(self.fargs["filter tree"], {7: cols[7]})
        agg = O.tqp_hash_aggregate(cols, copy.deepcopy(self.aargs))
        return O.tqp_sort(agg, self.sargs, False)


class StarJoin:
    name = "star_join"
    NF, NA, NB, NC = 59_986_052, 2_000_000, 15_000_000, 1_500_000

    def __init__(self, scale: float = 1.0):
        from tqpk import datagen
        nf, na, nb, nc = (max(1000, int(x * scale)) for x in (self.NF, self.NA, self.NB, self.NC))
        self.n = (nf, na, nb, nc)
        self.t = datagen.star_tables(nf, na, nb, nc, seed=11)
        self.fact_rows = nf
        self.config = {"workload": "star join fact x A(category = 1) x B x C, sum(price*(1-discount)) and count "
                                   "group by C key, top-100", "fact_rows": nf, "a_rows": na, "b_rows": nb,
                       "c_rows": nc, "l2": "inputs (1.4 GB) larger than L2"}
        t = self.t
        self.cols = {31: t["a_key"], 32: t["a_cat"], 41: t["f_fka"], 42: t["f_fkb"], 43: t["f_price"],
                     44: t["f_discount"], 51: t["b_key"], 52: t["b_fkc"], 61: t["c_key"]}
        self.types = {31: "int", 32: "int", 41: "int", 42: "int", 43: "float", 44: "float", 51: "int", 52: "int",
                      61: "int"}
        self.fa = {"filter tree": [["cat#32", "=", str(datagen.STAR_CATEGORY)]], "materialized in": [32],
                   "out mask id": 901}
        # join keys are always part of 'materialized in' (parsing.py:408-410 adds 'join in')
        self.j1 = ({"left group": [31, 32], "right group": [41, 42, 43, 44], "materialized in": [31, 41, 42, 43, 44],
                    "mask map": {31: 901}}, 31, 41)
        self.j2 = ({"left group": [51, 52], "right group": [31, 41, 42, 43, 44],
                    "materialized in": [51, 52, 42, 43, 44]}, 51, 42)
        self.j3 = ({"left group": [61], "right group": [51, 52, 42, 43, 44], "materialized in": [61, 52, 43, 44]},
                   61, 52)
        self.value_tree = [["p#43", "*", ["1.0", "-", "d#44"]]]
        self.aargs = {"is partial": False, "keys": ["c#61"], "input ids": [61, 43, 44],
                      "results": ["c#61", [[["sum", self.value_tree], "#", "71"], "AS", "rev#72"],
                                  [[["count", ["1"]], "#", "73L"], "AS", "cnt#74"]],
                      "out agg ids": [72, 74]}
        self.targs = {"limit": 100, "input ids": [61, 72, 74], "key ids": [72], "key orders": [True]}

    def algorithmic_bytes(self):
        nf, na, nb, nc = self.n
        return nf * 24 + na * 5 + nb * 8 + nc * 4

    def dominant(self):
        from tqpk import _lib as L
        from tqpk import jit
        # fact fkA, fkB (4 B each), price, discount (8 B each)
        return L.KID_STAR_PROBE, "tqpk_q_star_probe" if jit.available() else "k_star_probe", self.n[0] * 24

    def setup_device(self, dev):
        import torch
        from tqpk.pipeline import StarAggTopK
        d = {c: torch.from_numpy(a).to(dev) for c, a in self.cols.items()}
        self.d = d
        dom = lambda a: (int(a.min()), int(a.max()))  # noqa: E731  (table statistics)
        self.pipe = StarAggTopK(d[41], d[42], {43: d[43], 44: d[44]}, None, self.value_tree,
                                d[31], {32: d[32]}, self.fa["filter tree"], dom(self.cols[31]),
                                d[51], d[52], dom(self.cols[51]), d[61], dom(self.cols[61]), k=100)
        self.host = {c: torch.from_numpy(a).pin_memory() for c, a in self.cols.items()}
        self.dev = dev

    def step_device(self):
        self.pipe.run()

    def capture(self):
        self.pipe.capture()

    def step_graph(self):
        self.pipe.replay()

    def device_result(self):
        k, v, c, _ = self.pipe.result()
        return k, v, c

    def _plan(self, tg, ops):
        f, j, a, s = ops
        f(tg, plan_args(self.fa))
        for args, lk, rk in (self.j1, self.j2, self.j3):
            tg = j(tg, plan_args(args), lk, rk)
        tg = a(tg, plan_args(self.aargs))
        return s(tg, plan_args(self.targs))

    def step_e2e(self):
        from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
        from tqpk.variable import Variable
        if not hasattr(self, "staged"):
            from tqpk.ingress import ColumnStager
            self.staged = ColumnStager(self.dev)
        # keys and dimension tables first, the fact value columns last: the joins run while they copy
        tg = self.staged.stage(self.host, self.types, (32, 31, 41, 42, 51, 52, 61, 43, 44))

        def f(tg, a):
            tqp_filter(True, tg, a, None, None, None, "f")

        def j(tg, a, lk, rk):
            join_vortex(True, tg, a, lk, rk, [], "inner", None, None, "j")
            return tg

        def ag(tg, a):
            tqp_hash_aggregate(True, tg, a, None, None, "a")
            return tg

        def so(tg, a):
            tqp_sort(True, tg, a, True, "t")
            return tg
        tg = self._plan(tg, (f, j, ag, so))
        res = d2h_all({c: tg[c].tensor for c in (61, 72, 74)})
        out = [res[c].numpy().reshape(-1) for c in (61, 72, 74)]
        h2d = sum(h.numel() * h.element_size() for h in self.host.values())
        return tuple(out), h2d, sum(o.nbytes for o in out)

    def plan(self):
        """The star query as a plan executor holds it: Filter(A), three Joins, Aggregate, take ordered,
        each operator's argument dict keyed by operator id."""
        ops = [3, 4, 5, 6, 7, 8]
        args = {3: dict(plan_args(self.fa), name="Filter")}
        for u, (ja, lk, rk) in zip((4, 5, 6), (self.j1, self.j2, self.j3)):
            args[u] = dict(plan_args(ja), name="Join", **{"left keys": [lk], "right keys": [rk], "join type": "Inner"})
        args[7] = dict(plan_args(self.aargs), name="Aggregate")
        args[8] = dict(plan_args(self.targs), name="take ordered")
        return ops, args

    def step_e2e_fused(self):
        """A plan executor that offers each run of operators to try_fused (the star shape runs as one
        fused pipeline) before dispatching them one by one; dimension columns copied first."""
        from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort, try_fused
        from tqpk.variable import host_values
        if not hasattr(self, "staged"):
            from tqpk.ingress import ColumnStager
            self.staged = ColumnStager(self.dev)
        tg = self.staged.stage(self.host, self.types, (32, 31, 51, 52, 61, 41, 42, 43, 44))
        ops, args = self.plan()
        i = 0
        while i < len(ops):
            m = try_fused(True, tg, ops, args, i)
            if m:
                i += m
                continue
            a = args[ops[i]]
            if a["name"] == "Filter":
                tqp_filter(True, tg, a, None, None, None, "f")
            elif a["name"] == "Join":
                join_vortex(True, tg, a, a["left keys"][0], a["right keys"][0], [], "inner", None, None, "j")
            elif a["name"] == "Aggregate":
                tqp_hash_aggregate(True, tg, a, None, None, "a")
            else:
                tqp_sort(True, tg, a, True, "t")
            i += 1
        out = [host_values(tg[c]).reshape(-1) for c in (61, 72, 74)]
        h2d = sum(h.numel() * h.element_size() for h in self.host.values())
        return tuple(out), h2d, sum(o.nbytes for o in out)

    def cpu_sample(self):
        """The bounded CPU sample: the same star at a tenth of the size."""
        return StarJoin(scale=0.1)

    def ref_plan(self, R, tg, pool, ge, sync):
        """main.py's plan over TQP-Inmem's own operators: Filter(A), three Joins, Aggregate,
        take ordered."""
        groups = []

        def f(tg, a):
            R.filter.tqp_filter(ge, tg, a, None, None, pool, "f"); sync()

        def j(tg, a, lk, rk):
            R.hashjoin.join_vortex(ge, tg, a, lk, rk, [], "inner", None, pool, "j"); sync()
            return tg

        def ag(tg, a):
            R.aggregate.tqp_hash_aggregate(ge, tg, a, pool, None, "a"); sync()
            groups.append(int(tg[61].tensor.shape[0]))
            return tg

        def so(tg, a):
            R.sort.tqp_sort(ge, tg, a, True, "t"); sync()
            return tg
        tg = self._plan(tg, (f, j, ag, so))
        return tuple(tg[c].tensor.cpu().numpy().reshape(-1) for c in (61, 72, 74)), groups[0]

    def step_dropin(self, tg):
        from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort

        def f(tg, a):
            tqp_filter(True, tg, a, None, None, None, "f")

        def j(tg, a, lk, rk):
            join_vortex(True, tg, a, lk, rk, [], "inner", None, None, "j")
            return tg

        def ag(tg, a):
            tqp_hash_aggregate(True, tg, a, None, None, "a")
            return tg

        def so(tg, a):
            tqp_sort(True, tg, a, True, "t")
            return tg
        return self._plan(tg, (f, j, ag, so))[72].tensor

    def oracle(self, cols=None):
        from oracle import tqp_oracle as O
        cols = dict(self.cols if cols is None else cols)

        def f(tg, a):
            tg[a["out mask id"]] = O.eval_filter(a["filter tree"], {c: tg[c] for c in a["materialized in"]})

        def j(tg, a, lk, rk):
            return O.join_vortex(tg, a, lk, rk, "inner")[0]

        def ag(tg, a):
            out = dict(tg)
            out.update(O.tqp_hash_aggregate(tg, a))
            return out

        def so(tg, a):
            return O.tqp_sort(tg, a, True)
        r = self._plan(cols, (f, j, ag, so))
        return r[61].reshape(-1), r[72], r[74]


class Batched:
    """64 uneven instances (half filter+group-by, half join+aggregate+top-10; rows log-uniform in
    [1e4, 1e7], group cardinality log-uniform in [4, 1e6]) as one persistent launch replayed from a
    CUDA graph, against the same instances run one at a time through the drop-in operators."""
    name = "batched"
    AGG = ["flag#5", "status#6",
           [[["sum", ["quantity#1"]], "#", "101"], "AS", "a#201"],
           [[["sum", ["price#2"]], "#", "102"], "AS", "b#202"],
           [[["sum", [["price#2", "*", ["1.0", "-", "discount#3"]]]], "#", "103"], "AS", "c#203"],
           [[["sum", [[["price#2", "*", ["1.0", "-", "discount#3"]], "*", ["1.0", "+", "tax#4"]]]], "#", "104"],
            "AS", "d#204"],
           [[["avg", ["quantity#1"]], "#", "105"], "AS", "e#205"],
           [[["avg", ["price#2"]], "#", "106"], "AS", "f#206"],
           [[["avg", ["discount#3"]], "#", "107"], "AS", "g#207"],
           [[["count", ["1"]], "#", "108L"], "AS", "h#208"]]
    AGG_IDS = [201, 202, 203, 204, 205, 206, 207, 208]

    def __init__(self, n_instances=64, scale: float = 1.0):
        from tqpk import datagen
        self.dg = datagen
        self.specs = datagen.batch_specs(n_instances, seed=3)
        if scale != 1.0:          # every instance's rows x scale, the same group counts (profiler captures)
            for sp in self.specs:
                sp["rows"] = max(1000, int(sp["rows"] * scale))
        self.fact_rows = sum(s["rows"] for s in self.specs)
        self.config = {"workload": "64 uneven instances: filter+group-by and join+aggregate+top-10, one persistent "
                                   "launch (CUDA graph) vs per-instance drop-in operators",
                       "instances": n_instances, "total_rows": self.fact_rows,
                       "rows_range": [10_000, 10_000_000], "group_range": [4, 1_000_000]}
        if scale != 1.0:
            self.config["scale"] = scale

    def setup_device(self, dev):
        import torch
        from tqpk.batch import Autotuner, Batch, GroupByInstance, JoinInstance
        self.dev = dev
        self.insts, self.plain_args = [], []
        for sp in self.specs:
            if sp["kind"] == "groupby":
                t, (a, b) = self.dg.groupby_instance_tables(sp["rows"], sp["groups"], sp["seed"])
                ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
                d = {ids[k]: torch.from_numpy(v).to(dev) for k, v in t.items()}
                args = {"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 3, 4, 5, 6],
                        "results": self.AGG, "out agg ids": self.AGG_IDS}
                self.insts.append(GroupByInstance(args=args, columns={c: d[c] for c in range(1, 7)},
                                                  filter_tree=[["ship_date#7", "<=", "2470"]], filter_cols={7: d[7]},
                                                  key_domains=[(0, a - 1), (0, b - 1)]))
                self.plain_args.append(("groupby", d))
            else:
                t = self.dg.join_tables(sp["groups"], sp["rows"], sp["seed"])
                d = {k: torch.from_numpy(v).to(dev) for k, v in t.items()}
                self.insts.append(JoinInstance(d["b_key"], (1, sp["groups"]), d["p_fk"], {12: d["b_date"]},
                                               [["bd#12", "<", "1170"]],
                                               {22: d["p_date"], 23: d["p_price"], 24: d["p_discount"]},
                                               [["pd#22", ">", "1170"]], [["p#23", "*", ["1.0", "-", "d#24"]]], k=10))
                self.plain_args.append(("join", d))
        # every instance's input columns, each read once by the batch
        self.input_bytes = sum(t.numel() * t.element_size() for _, d in self.plain_args for t in d.values())
        from tqpk import jit
        if jit.available():
            from tqpk.jitbatch import QueryBatch
            self.batch = QueryBatch(self.insts, Autotuner())      # the generated persistent kernel
        else:
            self.batch = Batch(self.insts, Autotuner())
        self.batch.capture()

    def run_batched(self):
        self.batch.replay()

    def cpu_baseline(self, budget_s: float):
        """TQP-Inmem's operators on their CPU path (torch CPU, every host core) over the instances
        in order until budget_s is spent, as rows/s of that sample, turned into queries/s of the
        64-instance mix (its total rows at that rate).  None with the reason when the reference is
        not available."""
        import torch
        R, why = reference_modules()
        if R is None:
            return {"unavailable": why}
        from oracle import reference
        torch.set_num_threads(os.cpu_count() or 1)
        pool = reference.CpuPool()
        done_rows, spent, done = 0, 0.0, 0
        with reference.cpu_mode():
            for sp, (kind, d) in zip(self.specs, self.plain_args):
                if spent >= budget_s:
                    break
                cols = {c: t.cpu().numpy() for c, t in d.items()}
                t0 = time.perf_counter()
                if kind == "groupby":
                    types = {c: "float" if c <= 4 else ("date" if c == 7 else "int") for c in cols}
                    tg = _ref_tensor_group(R, cols, types)
                    R.filter.tqp_filter(False, tg, {"filter tree": [["ship_date#7", "<=", "2470"]],
                                                    "materialized in": [7], "out mask id": 900}, None, None, pool, "f")
                    R.aggregate.tqp_hash_aggregate(False, tg, {"is partial": False, "keys": ["flag#5", "status#6"],
                                                               "input ids": [1, 2, 3, 4, 5, 6], "results": self.AGG,
                                                               "out agg ids": list(self.AGG_IDS),
                                                               "mask map": {c: 900 for c in range(1, 7)}},
                                                   pool, None, "a")
                    rows = sp["rows"]
                else:
                    j = object.__new__(JoinAggTop10)        # this instance's tables, the query's arguments
                    j.set_args()
                    j.cols = {11: cols["b_key"], 12: cols["b_date"], 21: cols["p_fk"], 22: cols["p_date"],
                              23: cols["p_price"], 24: cols["p_discount"]}
                    j.types = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}
                    tg = _ref_tensor_group(R, j.cols, j.types)
                    torch.manual_seed(0)
                    j.ref_plan(R, tg, pool, False, lambda: None)
                    rows = sp["rows"] + sp["groups"]
                spent += time.perf_counter() - t0
                done_rows += rows
                done += 1
        rate = done_rows / spent
        total = sum(sp["rows"] + (sp["groups"] if sp["kind"] == "join" else 0) for sp in self.specs)
        return {"value": len(self.specs) / (total / rate), "unit": "queries/s", "cores": torch.get_num_threads(),
                "kind": "reference",
                "sample": f"the first {done} of the {len(self.specs)} instances ({done_rows} rows, {spent:.1f} s) through "
                          f"TQP-Inmem's operators (oracle/_ref), gpu_enable=False, torch {torch.__version__} CPU: "
                          f"{rate:.3g} rows/s, scaled to the mix's {total} rows"}

    def run_plain(self):
        """Every instance alone through the drop-in operators (the reference's per-operator path)."""
        import torch
        from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
        from tqpk.variable import Variable
        out = []
        for kind, d in self.plain_args:
            if kind == "groupby":
                tg = {c: Variable(d[c], "float" if c <= 4 else ("date" if c == 7 else "int")) for c in d}
                tqp_filter(True, tg, {"filter tree": [["ship_date#7", "<=", "2470"]], "materialized in": [7],
                                      "out mask id": 900}, None, None, None, "f")
                tqp_hash_aggregate(True, tg, {"is partial": False, "keys": ["flag#5", "status#6"],
                                              "input ids": [1, 2, 3, 4, 5, 6], "results": self.AGG,
                                              "out agg ids": self.AGG_IDS,
                                              "mask map": {c: 900 for c in range(1, 7)}}, None, None, "a")
                out.append(({o: tg[o].tensor for o in self.AGG_IDS}, [tg[5].tensor, tg[6].tensor]))
            else:
                tg = {11: Variable(d["b_key"], "int"), 12: Variable(d["b_date"], "date"),
                      21: Variable(d["p_fk"], "int"), 22: Variable(d["p_date"], "date"),
                      23: Variable(d["p_price"], "float"), 24: Variable(d["p_discount"], "float")}
                tqp_filter(True, tg, {"filter tree": [["bd#12", "<", "1170"]], "materialized in": [12],
                                      "out mask id": 901}, None, None, None, "f")
                tqp_filter(True, tg, {"filter tree": [["pd#22", ">", "1170"]], "materialized in": [22],
                                      "out mask id": 902}, None, None, None, "f")
                join_vortex(True, tg, {"left group": [11, 12], "right group": [21, 22, 23, 24],
                                       "materialized in": [11, 21, 23, 24],
                                       "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}, 11, 21, [], "inner",
                            None, None, "j")
                tqp_hash_aggregate(True, tg, {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
                                              "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]],
                                                                    "#", "1"], "AS", "r#302"]],
                                              "out agg ids": [302]}, None, None, "a")
                tqp_sort(True, tg, {"limit": 10, "input ids": [11, 302], "key ids": [302], "key orders": [True]},
                         True, "t")
                out.append((tg[11].tensor, tg[302].tensor))
        torch.cuda.synchronize()
        return out

    def compare(self, plain, batched):
        for (kind, _), p, b in zip(self.plain_args, plain, batched):
            if kind == "join":
                assert np.array_equal(p[0].cpu().numpy().reshape(-1), b[0])
                pv = p[1].cpu().numpy()
                assert np.all(np.abs(pv - b[1]) <= 1e-12 * np.abs(pv))
            else:
                outs, keys, g = b
                assert np.array_equal(p[1][0].cpu().numpy().reshape(-1), keys[0])
                assert np.array_equal(p[1][1].cpu().numpy().reshape(-1), keys[1])
                for o in self.AGG_IDS:
                    pv = p[0][o].cpu().numpy()
                    if pv.dtype == np.float64:
                        assert np.all(np.abs(pv - outs[o]) <= 1e-12 * np.abs(pv)), o
                    else:
                        assert np.array_equal(pv, outs[o]), o


def run_batched_bench(args):
    import torch
    from tqpk import _lib as L
    import __graft_entry__ as G
    G.build()
    lib = L.load()
    dev = torch.device("cuda", 0)
    w = Batched(scale=args.scale)
    w.setup_device(dev)
    w.run_batched()
    torch.cuda.synchronize()
    batched_res = w.batch.results()
    plain_res = w.run_plain()
    w.compare(plain_res, batched_res)
    for _ in range(args.warmup):
        w.run_batched()
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s, e in evs:
        s.record()
        w.run_batched()          # one CUDA graph: control reset, table reset kernel, persistent kernel
        e.record()
    torch.cuda.synchronize()
    launches = 2 * args.steps    # our kernels inside each replayed graph
    batched_ms = statistics.median([s.elapsed_time(e) for s, e in evs])
    clocks = sampler.stop()
    # the persistent kernel alone (direct launches, CUDA events around it)
    import ctypes as C
    L.check(lib.tqpk_timing_begin(L.KID_BATCH), "tqpk_timing_begin")
    for _ in range(3):
        w.batch.run()
    kms, kn = C.c_double(0), C.c_int32(0)
    L.check(lib.tqpk_timing_end(C.byref(kms), C.byref(kn)), "tqpk_timing_end")
    plain_times = []
    for _ in range(max(2, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w.run_plain()
        plain_times.append(time.perf_counter() - t0)
    plain_s = statistics.median(plain_times)
    n = len(w.specs)
    # end to end: the replay and every instance's result rows read back (two device-to-host reads);
    # the tables stay resident, as in the serving loop
    e2e, d2h = None, 0
    if hasattr(w.batch, "results_host"):
        ts = []
        for _ in range(max(3, min(args.steps, 10))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            w.run_batched()
            res, d2h = w.batch.results_host()
            ts.append(time.perf_counter() - t0)
        w.compare(plain_res, res)
        e2e_s = statistics.median(ts)
        e2e = {"value": n / e2e_s, "unit": "queries/s", "ms_per_step": e2e_s * 1e3, "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": d2h,
               "path": "graph replay + every instance's result rows to pinned host memory; tables resident"}
    kernel_s = kms.value / max(kn.value, 1) / 1000.0
    peak, peak_src = peak_gbs()
    achieved = w.input_bytes / kernel_s / 1e9
    cpu = w.cpu_baseline(budget_s=12.0)
    line = {"metric": "queries/s", "value": n / (batched_ms / 1000.0), "unit": "queries/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": batched_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": dict(w.config, plain_queries_per_s=n / plain_s, speedup_vs_plain=(n / (batched_ms / 1000.0)) /
                           (n / plain_s), batched_rows_per_s=w.fact_rows / (batched_ms / 1000.0),
                           kernel_ms=kernel_s * 1e3),
            "roofline": {"bound": "hbm", "kernel": "tqpk_qb_run", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "algorithmic_bytes_per_launch": w.input_bytes,
                         "launches": kn.value, "avg_launch_us": kernel_s * 1e6,
                         "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                         else "fallback 6.8 TB/s",
                         "note": "every instance's input columns read once per launch"},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "gpu_launches": launches}
    return line


def run_serving_bench(args):
    """The three query shapes over resident 60M-row tables, HBM budget 150 GB, continuous batching
    (8 slots) beside one-at-a-time.  `value` is the closed-loop rate (all requests queued at t=0:
    the capacity) of continuous batching, with one-at-a-time's beside it; latencies (p50/p99) come
    from Poisson arrivals at 1500/s, below both schedulers' capacity, so neither queue grows
    without bound and the percentiles are per-request latency."""
    import dataclasses
    import torch
    import __graft_entry__ as G
    G.build()
    from tqpk import _lib as L
    from tqpk.serve import DeviceArena, GpuExecutor, ResidentTables, Scheduler, latency_summary, poisson_trace
    lib = L.load()
    dev = torch.device("cuda", 0)
    n_fact, rate, slots, budget = 60_000_000, 1500.0, 8, 150 << 30
    t_setup = time.perf_counter()
    tables = ResidentTables(dev, n_fact=n_fact)
    ex = GpuExecutor(tables, slots)
    arena = DeviceArena(budget, tables.nbytes, dev, slab_cap=8 << 30)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    warm = poisson_trace(max(30, 10 * args.warmup), rate, n_fact, seed=100)
    Scheduler(ex, arena, slots).run(warm)
    Scheduler(ex, arena, 1).run(warm[:10])
    n_req = max(400, 100 * args.steps)
    trace = poisson_trace(n_req, rate, n_fact, seed=1)
    sampler = ClockSampler(0)
    sampler.start()
    launches0 = lib.tqpk_launch_count()
    sched = Scheduler(ex, arena, slots)
    cont = sched.run(trace)
    launches = lib.tqpk_launch_count() - launches0
    serial = Scheduler(ex, arena, 1).run(trace)
    burst = [dataclasses.replace(r, arrival=0.0) for r in trace[: max(200, n_req // 4)]]
    cont_sat = Scheduler(ex, arena, slots).run(burst)
    serial_sat = Scheduler(ex, arena, 1).run(burst)
    clocks = sampler.stop()
    sc, ss = latency_summary(cont), latency_summary(serial)
    cap_c, cap_s = latency_summary(cont_sat)["requests_per_s"], latency_summary(serial_sat)["requests_per_s"]
    by_shape = {}
    for shape in ("filter_groupby", "join", "star"):
        sub = [c for c in cont if c.req.shape == shape]
        if sub:
            lat = np.array([c.latency for c in sub]) * 1e3
            by_shape[shape] = {"requests": len(sub), "p50_ms": float(np.percentile(lat, 50)),
                               "p99_ms": float(np.percentile(lat, 99))}
    def result_bytes(r):
        parts = []
        for v in r.values():
            parts += list(v.values()) if isinstance(v, dict) else (v if isinstance(v, list) else [v])
        return sum(np.asarray(x).nbytes for x in parts)
    d2h = sum(result_bytes(c.result) for c in cont)
    line = {"metric": "requests/s", "value": cap_c, "unit": "requests/s", "n_gpus": 1,
            "steps": len(burst), "warmup": len(warm), "ms_per_step": 1e3 / cap_c, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded), Poisson arrivals",
            "config": {"workload": "serving: Poisson arrivals of filter+group-by / join+agg+top-10 / star join+top-100 "
                                   "over resident tables, continuous batching vs one-at-a-time",
                       "value": "closed-loop requests/s of continuous batching (capacity)",
                       "one_at_a_time_closed_loop_requests_per_s": cap_s, "speedup_vs_one_at_a_time": cap_c / cap_s,
                       "arrival_rate_per_s": rate, "requests": n_req, "fact_rows_range": [1_000_000, n_fact],
                       "slots": slots, "hbm_budget_bytes": budget, "resident_bytes": tables.nbytes,
                       "setup_s": setup_s, "l2": "inputs (GBs per shape) larger than L2"},
            "serving": {"continuous": sc, "one_at_a_time": ss, "continuous_by_shape": by_shape,
                        "closed_loop_requests_per_s": {"continuous": cap_c, "one_at_a_time": cap_s,
                                                       "requests": len(burst)},
                        "max_inflight": sched.max_inflight},
            "e2e": {"value": cap_c, "unit": "requests/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": d2h / max(len(cont), 1),
                    "path": "closed loop, each request from the host queue to its result in pinned host memory; "
                            "tables resident"},
            "clocks": clocks, "gpu_launches": launches}
    return line


WORKLOADS = {c.name: c for c in (JoinAggTop10, FilterGroupBy, StarJoin)}


def make_workload(args):
    if args.workload == "star_join":
        return StarJoin(scale=args.scale)
    return WORKLOADS[args.workload]()


# ---------------------------------------------------------------------------- helpers
def peak_gbs():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return PEAK_FALLBACK_GBS, "fallback"


def fp64_peak_gops() -> Optional[float]:
    """Measured FP64 add throughput of this GPU (Gop/s): four independent __dadd_rn chains
    per thread over a full grid, timed with CUDA events."""
    import torch
    from tqpk import jit
    if not jit.available():
        return None
    src = r"""
extern "C" __global__ void fp64_add_rate(double* out, int iters) {
  double a = threadIdx.x * 1e-3, b = blockIdx.x * 1e-6, c = 0.5, d = 0.25;
  const double x = 1.0000001, y = 0.9999999;
  for (int i = 0; i < iters; ++i) {
    a = __dadd_rn(a, x); b = __dadd_rn(b, y); c = __dadd_rn(c, x); d = __dadd_rn(d, y);
  }
  if (a + b + c + d == 12345.678) out[0] = a;
}"""
    h = jit.compile_kernel(src, "fp64_add_rate")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    sms, blocks, iters = torch.cuda.get_device_properties(0).multi_processor_count, 8, 4096
    a = jit._Args()
    a.ptr(out.data_ptr())
    a.i32(iters)
    s = torch.cuda.current_stream().cuda_stream
    jit.launch(h, sms * blocks, 256, 0, a, s)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        jit.launch(h, sms * blocks, 256, 0, a, s)
    e1.record()
    torch.cuda.synchronize()
    ops = 5 * sms * blocks * 256 * iters * 4
    return ops / (e0.elapsed_time(e1) / 1e3) / 1e9


def traffic_per_launch(kernel: str, workload: str):
    """DRAM bytes per launch from the committed ncu summary (profiles/traffic.json)."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return d.get(workload, {}).get(kernel)
    except Exception:
        return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = [r.split(",") for r in out.strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip().lower() == "active"})
        loaded = [x for x in sm if smax and x > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def compare(workload, got, exp):
    if isinstance(workload, StarJoin):
        gk, gv, gc = got
        ek, ev, ec = exp
        assert np.array_equal(np.asarray(gk).reshape(-1), ek), (gk[:5], ek[:5])
        assert np.all(np.abs(np.asarray(gv) - ev) <= 1e-12 * np.abs(ev)), (gv[:5], ev[:5])
        assert np.array_equal(np.asarray(gc).reshape(-1), ec)
    elif isinstance(workload, JoinAggTop10):
        gk, gv = got
        ek, ev = exp
        assert np.array_equal(np.asarray(gk).reshape(-1), np.asarray(ek).reshape(-1)), (gk, ek)
        assert np.all(np.abs(np.asarray(gv) - ev) <= 1e-12 * np.abs(ev)), (gv, ev)
    else:
        keys, outs = got
        ex = exp
        assert np.array_equal(keys[0], ex[5].reshape(-1)) and np.array_equal(keys[1], ex[6].reshape(-1))
        for oid, v in outs.items():
            e = ex[oid]
            if e.dtype == np.float64:
                assert np.all(np.abs(v - e) <= 1e-12 * np.abs(e)), (oid, v, e)
            else:
                assert np.array_equal(v, e), (oid, v, e)


# ---------------------------------------------------------------------------- the reference's operators
def reference_modules():
    """TQP-Inmem's own operator modules (oracle/_ref), or (None, why) when they are unavailable."""
    try:
        from oracle import reference
        return reference.load(), ""
    except Exception as e:                    # missing build, other Python, import failure
        return None, f"{type(e).__name__}: {e}"


def _ref_tensor_group(R, cols, types, device=None):
    import torch
    V = R.variable.Variable
    tg = {}
    for c, a in cols.items():
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
        if device is not None:
            t = t.to(device, non_blocking=True)
        tg[c] = V(t, types[c])
    return tg


def reference_cpu(w, budget_s: float, max_runs: int = 3):
    """TQP-Inmem's operators on their CPU path (gpu_enable=False, torch CPU on every host core)
    over the workload's full-size tables, bounded: runs until max_runs or budget_s; returns
    (cpu_baseline record, last result) or (None, why)."""
    import torch
    R, why = reference_modules()
    if R is None:
        return None, why
    from oracle import reference
    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    pool = reference.CpuPool()
    ts, res = [], None
    t_end = time.perf_counter() + budget_s
    with reference.cpu_mode():
        while len(ts) < max_runs and (not ts or time.perf_counter() + statistics.median(ts) < t_end):
            tg = _ref_tensor_group(R, w.cols, w.types)
            torch.manual_seed(0)
            t0 = time.perf_counter()
            res = w.ref_plan(R, tg, pool, False, lambda: None)
            ts.append(time.perf_counter() - t0)
    med = statistics.median(ts)
    rec = {"value": w.fact_rows / med, "unit": "rows/s", "cores": torch.get_num_threads(), "kind": "reference",
           "sample": f"{type(w).__name__} full-size query ({w.fact_rows} fact rows) x{len(ts)}, median {med:.3f} s: "
                     f"TQP-Inmem's operators (oracle/_ref), gpu_enable=False, torch {torch.__version__} CPU"}
    return rec, res


def reference_cuda(w, dev, steps: int, warmup: int = 2):
    """TQP-Inmem's operators on torch CUDA on this GPU, through main.py's plan with a
    synchronisation after every operator and the reference's own device pool
    (IO/pinned_mem.GPUMemory(40 GB, 40 MB blocks), main.py:56, freed per query, main.py:293-294).
    Resident: the input columns already on the device; e2e: copied from pinned host memory inside
    the timed region and the result read back.  Returns (record, result) or (None, why)."""
    import torch
    R, why = reference_modules()
    if R is None:
        return None, why
    pool = R.pinned_mem.GPUMemory(capacity_gb=40, block_size_mb=40)
    dcols = {c: torch.from_numpy(np.ascontiguousarray(a)).to(dev) for c, a in w.cols.items()}
    hcols = {c: torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for c, a in w.cols.items()}
    sync = torch.cuda.synchronize

    def one(cols, copy_in):
        tg = _ref_tensor_group(R, cols, w.types, device=dev if copy_in else None)
        out = w.ref_plan(R, tg, pool, True, sync)
        pool.free_all()
        return out

    res = None
    for _ in range(warmup):
        res = one(dcols, False)
    sync()
    ts = []
    for _ in range(steps):
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        one(dcols, False)
        s1.record()
        sync()
        ts.append(s0.elapsed_time(s1))
    e2e = []
    for _ in range(max(2, steps // 2)):
        sync()
        t0 = time.perf_counter()
        one(hcols, True)
        sync()
        e2e.append(time.perf_counter() - t0)
    ms, e2e_s = statistics.median(ts), statistics.median(e2e)
    h2d = sum(h.numel() * h.element_size() for h in hcols.values())
    rec = {"value": w.fact_rows / (ms / 1e3), "unit": "rows/s", "ms_per_step": ms, "steps": steps,
           "e2e": {"value": w.fact_rows / e2e_s, "unit": "rows/s", "ms_per_step": e2e_s * 1e3, "h2d_bytes_per_step": h2d},
           "path": f"TQP-Inmem's operators (oracle/_ref) on torch {torch.__version__} CUDA, main.py's plan order"}
    del dcols, hcols, pool
    torch.cuda.empty_cache()
    return rec, res


def run_reference(args, rank, world):
    """The reference arm: TQP-Inmem's own operators on their CPU path (torch CPU, every host
    core), each step one full-size query of the workload.  Falls back to the numpy
    restatement of the same algorithm (oracle/tqp_oracle.py) when the compiled reference is
    unavailable, and says so."""
    if rank != 0:
        return
    import torch
    name = args.workload if args.workload in WORKLOADS else JoinAggTop10.name
    w = make_workload(argparse.Namespace(workload=name, scale=args.scale))
    R, why = reference_modules()
    cores = os.cpu_count() or 1
    if R is not None:
        from oracle import reference
        torch.set_num_threads(cores)
        pool = reference.CpuPool()

        def step():
            tg = _ref_tensor_group(R, w.cols, w.types)
            torch.manual_seed(0)
            w.ref_plan(R, tg, pool, False, lambda: None)
        kind, how = "reference", (f"TQP-Inmem's operators (oracle/_ref), gpu_enable=False, torch {torch.__version__} "
                                  f"CPU, {torch.get_num_threads()} threads")
        ctx = reference.cpu_mode()
    else:
        def step():
            w.oracle()
        kind, how = "port", f"numpy restatement (oracle/tqp_oracle.py), 1 thread; the compiled reference: {why}"
        import contextlib
        ctx = contextlib.nullcontext()
    with ctx:
        for _ in range(args.warmup):
            step()
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            step()
            times.append(time.perf_counter() - t0)
    wall = sum(times)
    value = args.steps * w.fact_rows / wall
    threads = torch.get_num_threads() if R is not None else 1
    line = {
        "impl": "reference", "metric": "rows/s", "value": value, "unit": "rows/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(w.config, parallelism=f"host CPU, {threads} threads"),
        "cpu_baseline": {"value": value, "unit": "rows/s", "cores": threads, "kind": kind,
                         "sample": f"{args.steps} full-size queries, one after another (median "
                                   f"{statistics.median(times):.3f} s): {how}"},
        "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------- our arm
def measure_ours(args, w, rank, world, dev, cpu_budget_s=20.0, with_reference=True):
    """One workload on this GPU: correctness gate, the fused step (CUDA-graph replay) timed with
    CUDA events, the dominant kernel's own launches, the drop-in operators resident and end to end,
    the reference's operators on torch CUDA and on the CPU.  Returns the JSON record."""
    import torch
    from tqpk import _lib as L
    lib = L.load()
    w.setup_device(dev)

    # correctness gate (outside the timed region): the fused step against the oracle
    exp = w.oracle()
    w.step_device()
    torch.cuda.synchronize()
    compare(w, w.device_result(), exp)

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    # keep the GPU loaded ~1 s so clocks settle and are sampled around the timed steps
    t_end = time.perf_counter() + 1.0
    while time.perf_counter() < t_end:
        for _ in range(args.warmup):
            w.step_device()
        torch.cuda.synchronize()
    kid, kname, kbytes = w.dominant()
    # a fused pipeline runs as one CUDA graph per step (its launches and memsets recorded once)
    graph = hasattr(w, "capture") and getattr(w, "pipe", True) is not None
    if graph:
        launches0 = lib.tqpk_launch_count()
        w.capture()
        launches_per_step = (lib.tqpk_launch_count() - launches0) // 2    # capture() runs once eagerly, once recorded
        for _ in range(args.warmup):
            w.step_graph()
        torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    if not graph:
        L.check(lib.tqpk_timing_begin(kid), "tqpk_timing_begin")
    launches0 = lib.tqpk_launch_count()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s0, e0 in evs:
        flush.zero_()
        s0.record()
        w.step_graph() if graph else w.step_device()
        e0.record()
    torch.cuda.synchronize()
    launches = launches_per_step * args.steps if graph else lib.tqpk_launch_count() - launches0
    barrier(world)
    import ctypes as C
    kms, kn = C.c_double(0), C.c_int32(0)
    if graph:
        # the dominant kernel's own duration: direct launches bracketed by CUDA events
        L.check(lib.tqpk_timing_begin(kid), "tqpk_timing_begin")
        for _ in range(args.steps):
            flush.zero_()
            w.step_device()
        torch.cuda.synchronize()
    L.check(lib.tqpk_timing_end(C.byref(kms), C.byref(kn)), "tqpk_timing_end")
    step_ms = [s0.elapsed_time(e0) for s0, e0 in evs]
    total_ms = max_over_ranks(sum(step_ms), world)
    clocks = sampler.stop()

    # the drop-in operators over resident columns (the reference-facing path, no copies)
    from tqpk.variable import Variable
    dropin = []
    for i in range(2 + max(3, min(args.steps, 10))):
        tg = {c: Variable(w.d[c], w.types[c]) for c in w.cols}
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w.step_dropin(tg)
        torch.cuda.synchronize()
        if i >= 2:
            dropin.append(time.perf_counter() - t0)
    dropin_s = statistics.median(dropin)

    # end to end with host buffers: the drop-in operators one by one, and (where the workload has
    # one) the executor that hands the whole run to try_fused
    def timed_e2e(step):
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        ts, out = [], None
        for _ in range(max(3, min(args.steps, 10))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = step()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return max_over_ranks(statistics.median(ts), world), out

    ops_s, (res, h2d, d2h) = timed_e2e(w.step_e2e)
    got_e2e = res if not isinstance(w, FilterGroupBy) else \
        ([res[5].reshape(-1), res[6].reshape(-1)], {o: res[o] for o in w.aargs["out agg ids"]})
    compare(w, got_e2e, exp)
    e2e_s, e2e_path = ops_s, "drop-in operators, pinned host inputs"
    if hasattr(w, "step_e2e_fused"):
        e2e_s, (res_f, h2d, d2h) = timed_e2e(w.step_e2e_fused)
        compare(w, res_f, exp)
        e2e_path = ("plan executor with try_fused (one fused pipeline for the filter-join(s)-aggregate-top-k run), "
                    "pinned host inputs")

    # TQP-Inmem's own operators on torch CUDA on this GPU, and their result against ours
    ref_cuda = None
    if with_reference and rank == 0:
        rec, out = reference_cuda(w, dev, steps=max(3, min(args.steps, 10)))
        if rec is None:
            ref_cuda = {"unavailable": out}
        else:
            (ref_res, ref_groups) = out
            compare(w, got_e2e, ref_res)
            rec["result_matches_ours"] = True
            rec["groups"] = ref_groups
            ref_cuda = rec

    # CPU baseline: the reference's CPU path on the host cores (rank 0, N=1 only), bounded sample
    cpu = None
    if rank == 0 and world == 1:
        sample_w = w.cpu_sample() if hasattr(w, "cpu_sample") else w
        cpu, why = reference_cpu(sample_w, cpu_budget_s) if with_reference else (None, "not run")
        if cpu is None:
            ts = []
            t_budget = time.perf_counter() + cpu_budget_s
            while len(ts) < 3 and (not ts or time.perf_counter() < t_budget):
                t0 = time.perf_counter()
                sample_w.oracle()
                ts.append(time.perf_counter() - t0)
            cpu = {"value": sample_w.fact_rows / statistics.median(ts), "unit": "rows/s", "cores": 1, "kind": "port",
                   "sample": f"full-size query x{len(ts)} (median {statistics.median(ts):.3f} s), numpy restatement "
                             f"(oracle/tqp_oracle.py), 1 thread; the compiled reference: {why}"}

    peak, peak_src = peak_gbs()
    k_avg_s = (kms.value / max(kn.value, 1)) / 1000.0
    achieved = kbytes / k_avg_s / 1e9 if kn.value else None
    traffic = traffic_per_launch(kname, w.name)
    value = world * args.steps * w.fact_rows / (total_ms / 1000.0)
    line = {
        "metric": "rows/s", "value": value, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, TPC-H-like distributions)",
        "config": dict(w.config, parallelism="replicas" if world > 1 else "single GPU",
                       step="one CUDA-graph replay of the fused pipeline" if graph else "direct launches",
                       pipeline_GBps=w.algorithmic_bytes() / (total_ms / args.steps / 1000.0) / 1e9),
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "algorithmic_bytes_per_launch": kbytes, "launches": kn.value,
                     "avg_launch_us": k_avg_s * 1e6, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"
                     if peak_src == "measured" else "fallback 6.8 TB/s"},
        "cpu_baseline": cpu,
        "e2e": {"value": world * w.fact_rows / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3, "path": e2e_path},
        "e2e_operators": {"value": world * w.fact_rows / ops_s, "unit": "rows/s", "ms_per_step": ops_s * 1e3,
                          "path": "drop-in operators one by one, pinned host inputs"},
        "dropin": {"value": w.fact_rows / dropin_s, "unit": "rows/s", "ms_per_step": dropin_s * 1e3,
                   "path": "drop-in operators over resident columns (host time included: synchronisations and "
                           "Python)"},
        "reference_cuda": ref_cuda,
        "clocks": clocks,
        "gpu_launches": launches,
    }
    if hasattr(w, "fp64_ops") and kn.value:
        # the accumulation kernel is bound by the FP64 pipe (1/64 rate on this part), not by HBM
        ops, per_row, instr = w.fp64_ops()
        fpk = fp64_peak_gops()
        got = ops / k_avg_s / 1e9
        issued = ops / per_row * instr / k_avg_s / 1e9
        line["roofline"]["fp64"] = {"ops_per_launch": ops, "ops_per_passing_row": per_row, "achieved": got,
                                    "instructions_per_passing_row": instr, "issued": issued,
                                    "peak": fpk, "unit": "Gop/s", "frac": issued / fpk if fpk else None,
                                    "peak_source": "measured in this run (four independent __dadd_rn chains per thread, "
                                                   "full grid); frac = issued FP64 instructions / that rate"}
    return line


def run_ours(args, rank, world):
    import torch
    import __graft_entry__ as G

    G.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    names = [args.workload] if args.workload != "all" else [JoinAggTop10.name, FilterGroupBy.name, StarJoin.name,
                                                            "batched", "serving"]
    lines = {}
    for name in names:
        if name == "batched":
            rec = run_batched_bench(args) if rank == 0 else None
        elif name == "serving":
            rec = run_serving_bench(args) if rank == 0 else None
        else:
            w = make_workload(argparse.Namespace(workload=name, scale=args.scale))
            rec = measure_ours(args, w, rank, world, dev)
            del w
        lines[name] = rec
        import gc
        gc.collect()
        torch.cuda.empty_cache()
    if rank != 0:
        return
    head = lines[names[0]]
    if len(names) > 1:
        head = dict(head)
        head["workloads"] = {n: lines[n] for n in names[1:]}
    print(json.dumps(head))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["all"] + sorted(WORKLOADS) + ["batched", "serving"], default="all",
                    help="all (default): the join query as the headline, every other workload as a sub-record")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="star_join and batched only: table sizes x scale (a small case for profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world = dist_setup(args.gpus)
    if args.impl == "reference":
        if args.workload in ("batched", "serving"):
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "TQP-Inmem answers one query at a time: the "
                                  "batched and served forms have no reference counterpart"}))
            return
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
