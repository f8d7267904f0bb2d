#!/usr/bin/env python3
"""Benchmark of the TQP-Inmem relational hot path on GB300.

Default workload (``--workload join_agg_top10``): the filtered equi-join +
aggregate + top-10 query -- build side 1,500,000 rows (key = permutation of
1..1.5M, date), filter date < 1170; probe side 6,001,215 rows (fk uniform
over the build keys, date, price, discount), filter date > 1170;
sum(price * (1 - discount)) grouped by build key; top 10 by the sum,
descending.  Synthetic seeded data with the TPC-H-like distributions of
tqpk.datagen (TPC-H itself is not available).

One step = one run of the whole query over inputs resident in HBM, through
the fused pipeline (tqpk_pipeline_join_agg_topk: build, probe+aggregate,
top-k).  ``e2e`` = the same query through the drop-in operators
(tqp_filter x2, join_vortex, tqp_hash_aggregate, tqp_sort with limit) with
the input columns copied from pinned host memory and the result copied back
inside the timed region.  Metric: rows/s = probe (fact) rows / step time.

``--impl reference`` times the reference algorithm's CPU implementation (the
numpy restatement in oracle/) on the host cores, one process per core.
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
def d2h_all(tensors):
    """Results to pinned host memory: every copy queued, then one synchronisation."""
    import torch
    out = {}
    for c, t in tensors.items():
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        out[c] = h
    torch.cuda.current_stream().synchronize()
    return out


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
        self.cols = {11: self.t["b_key"], 12: self.t["b_date"], 21: self.t["p_fk"], 22: self.t["p_date"],
                     23: self.t["p_price"], 24: self.t["p_discount"]}
        self.types = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}

    # algorithmic bytes: every input column read once (SURVEY 8d convention)
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
        """FP64 operations per launch of the accumulation kernel: the float arithmetic of the
        expression program and one add per float sum accumulator, for every row that
        passes the filter."""
        from tqpk import _lib as L
        S = self.prog.spec
        arith = sum(1 for i in range(S.n_expr) if S.expr[i].type == L.F64 and S.expr[i].op in
                    (L.X_ADD, L.X_SUB, L.X_MUL, L.X_DIV))
        sums = sum(1 for a in range(S.n_accs) if S.accs[a].kind == L.ACC_SUM and S.accs[a].type == L.F64)
        passing = int((self.t["ship_date"] <= 2470).sum())
        return (arith + sums) * passing, arith + sums

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

    def __init__(self, n_instances=64):
        from tqpk import datagen
        self.dg = datagen
        self.specs = datagen.batch_specs(n_instances, seed=3)
        self.fact_rows = sum(s["rows"] for s in self.specs)
        self.config = {"workload": "64 uneven instances: filter+group-by and join+aggregate+top-10, one persistent "
                                   "launch (CUDA graph) vs per-instance drop-in operators",
                       "instances": n_instances, "total_rows": self.fact_rows,
                       "rows_range": [10_000, 10_000_000], "group_range": [4, 1_000_000]}

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
        from tqpk import jit
        if jit.available():
            from tqpk.jitbatch import QueryBatch
            self.batch = QueryBatch(self.insts, Autotuner())      # the generated persistent kernel
        else:
            self.batch = Batch(self.insts, Autotuner())
        self.batch.capture()

    def run_batched(self):
        self.batch.replay()

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
    w = Batched()
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
    line = {"metric": "queries/s", "value": n / (batched_ms / 1000.0), "unit": "queries/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": batched_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": dict(w.config, plain_queries_per_s=n / plain_s, speedup_vs_plain=(n / (batched_ms / 1000.0)) /
                           (n / plain_s), batched_rows_per_s=w.fact_rows / (batched_ms / 1000.0),
                           kernel_ms=kms.value / max(kn.value, 1)),
            "clocks": clocks, "gpu_launches": launches}
    print(json.dumps(line))


def run_serving_bench(args):
    """Poisson arrivals (2000/s) of the three query shapes over resident 60M-row tables, HBM budget
    150 GB: continuous batching (8 slots) beside one-at-a-time on the same trace, plus the
    closed-loop (all requests queued at t=0) throughput of both."""
    import dataclasses
    import torch
    import __graft_entry__ as G
    G.build()
    from tqpk import _lib as L
    from tqpk.serve import DeviceArena, GpuExecutor, ResidentTables, Scheduler, latency_summary, poisson_trace
    lib = L.load()
    dev = torch.device("cuda", 0)
    n_fact, rate, slots, budget = 60_000_000, 2000.0, 8, 150 << 30
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
    line = {"metric": "requests/s", "value": sc["requests_per_s"], "unit": "requests/s", "n_gpus": 1,
            "steps": n_req, "warmup": len(warm), "ms_per_step": 1e3 / sc["requests_per_s"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded), Poisson arrivals",
            "config": {"workload": "serving: Poisson arrivals of filter+group-by / join+agg+top-10 / star join+top-100 "
                                   "over resident tables, continuous batching vs one-at-a-time",
                       "arrival_rate_per_s": rate, "requests": n_req, "fact_rows_range": [1_000_000, n_fact],
                       "slots": slots, "hbm_budget_bytes": budget, "resident_bytes": tables.nbytes,
                       "setup_s": setup_s, "l2": "inputs (GBs per shape) larger than L2"},
            "serving": {"continuous": sc, "one_at_a_time": ss, "continuous_by_shape": by_shape,
                        "closed_loop_requests_per_s": {"continuous": latency_summary(cont_sat)["requests_per_s"],
                                                       "one_at_a_time": latency_summary(serial_sat)["requests_per_s"],
                                                       "requests": len(burst)},
                        "max_inflight": sched.max_inflight},
            "e2e": {"value": sc["requests_per_s"], "unit": "requests/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": d2h / max(len(cont), 1),
                    "path": "arrival on the host to result in pinned host memory; tables resident"},
            "clocks": clocks, "gpu_launches": launches}
    print(json.dumps(line))


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


# ---------------------------------------------------------------------------- reference arm
def _ref_worker_init(name):
    global _REF_W
    _REF_W = WORKLOADS[name]()


def _ref_worker_step(_):
    t0 = time.perf_counter()
    _REF_W.oracle()
    return time.perf_counter() - t0


def run_reference(args, rank, world):
    if rank != 0:
        return
    import multiprocessing as mp
    w = make_workload(args)
    cores = os.cpu_count() or 1
    procs = max(1, min(cores, args.steps))
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs, initializer=_ref_worker_init, initargs=(args.workload,)) as pool:
        pool.map(_ref_worker_step, range(min(args.warmup, procs)))
        t0 = time.perf_counter()
        times = pool.map(_ref_worker_step, range(args.steps))
        wall = time.perf_counter() - t0
    value = args.steps * w.fact_rows / wall
    line = {
        "impl": "reference", "metric": "rows/s", "value": value, "unit": "rows/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(w.config, parallelism=f"{procs} host processes"),
        "cpu_baseline": {"value": value, "unit": "rows/s", "cores": procs, "kind": "port",
                         "sample": f"{args.steps} full-size queries on {procs} processes "
                                   f"(median single-query {statistics.median(times):.3f} s)"},
        "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------- our arm
def run_ours(args, rank, world):
    import torch
    from tqpk import _lib as L
    import __graft_entry__ as G

    G.build()
    lib = L.load()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = make_workload(args)
    w.setup_device(dev)

    # correctness gate (outside the timed region)
    exp = w.oracle()
    w.step_device()
    torch.cuda.synchronize()
    compare(w, w.device_result(), exp)

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    sampler = ClockSampler(local)
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
    for s, e in evs:
        flush.zero_()
        s.record()
        w.step_graph() if graph else w.step_device()
        e.record()
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
    step_ms = [s.elapsed_time(e) for s, e in evs]
    total_ms = max_over_ranks(sum(step_ms), world)
    clocks = sampler.stop()

    # end to end through the drop-in operators with host buffers
    for _ in range(2):
        w.step_e2e()
    torch.cuda.synchronize()
    e2e_times, h2d, d2h = [], 0, 0
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res, h2d, d2h = w.step_e2e()
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    compare(w, res if not isinstance(w, FilterGroupBy) else
            ([res[5].reshape(-1), res[6].reshape(-1)], {o: res[o] for o in w.aargs["out agg ids"]}), exp)
    e2e_s = max_over_ranks(statistics.median(e2e_times), world)

    # CPU baseline: the oracle on the host cores (rank 0, N=1 only), bounded sample
    cpu = None
    if rank == 0 and world == 1:
        ts = []
        t_budget = time.perf_counter() + 20.0
        while len(ts) < 3 and (not ts or time.perf_counter() < t_budget):
            t0 = time.perf_counter()
            w.oracle()
            ts.append(time.perf_counter() - t0)
        cpu = {"value": w.fact_rows / statistics.median(ts), "unit": "rows/s", "cores": 1, "kind": "port",
               "sample": f"full-size query x{len(ts)} (median {statistics.median(ts):.3f} s), numpy oracle, 1 thread"}

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
                "d2h_bytes_per_step": d2h, "path": "drop-in operators, pinned host inputs"},
        "clocks": clocks,
        "gpu_launches": launches,
    }
    if hasattr(w, "fp64_ops") and kn.value:
        # the accumulation kernel is bound by the FP64 pipe (1/64 rate on this part), not by HBM
        ops, per_row = w.fp64_ops()
        fpk = fp64_peak_gops()
        got = ops / k_avg_s / 1e9
        line["roofline"]["fp64"] = {"ops_per_launch": ops, "ops_per_passing_row": per_row, "achieved": got,
                                    "peak": fpk, "unit": "Gop/s", "frac": got / fpk if fpk else None,
                                    "peak_source": "measured in this run (four independent __dadd_rn chains per thread, full grid)"}
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batched", "serving"], default="join_agg_top10")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="star_join only: table sizes x scale (a small case for profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world = dist_setup(args.gpus)
    if args.workload == "serving":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference answers one query at a time; its "
                              "per-query CPU time is the other workloads' reference lines"}))
        elif rank == 0:
            run_serving_bench(args)
        return
    if args.workload == "batched":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batched form has no reference counterpart"}))
        elif rank == 0:
            run_batched_bench(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
