"""Generate golden input/output vectors by running TQP-Inmem's own operators.

Run by hand after the reference's operator path has been compiled into oracle/_ref/ (the
recipe ``python oracle/build_ref.py SOURCE_TREE``; __graft_entry__.build() runs it where the
TQP-Inmem source tree is present).  The operators are called unmodified, through their public
API, on their CPU path (``gpu_enable=False``, CPU torch):

* ``operators/filter.py``    ``tqp_filter``
* ``operators/hashjoin.py``  ``join_vortex`` / ``join_kernel_new``
* ``operators/aggregate.py`` ``tqp_hash_aggregate``
* ``operators/sort.py``      ``tqp_sort``
* ``operators/project.py``   ``tqp_project``

oracle/reference.py lists the adaptations that make them import without pandas, pyspark and
pyparsing (none touches the operators' arithmetic); oracle.reference.cpu_mode() maps their
hard-coded ``device='cuda'`` arguments to the CPU.

Each case is written to ``tests/golden/<case>.npz`` with its inputs, the operator arguments
(JSON) and the outputs.  The fixtures are small (a few thousand to ~150k rows) so the tests that
read them run in seconds.
"""
from __future__ import annotations

import copy
import json
import sys
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent


def load_reference():
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    from oracle import reference
    R = reference.load()            # raises ReferenceUnavailable when oracle/_ref was not built
    return R.filter, R.hashjoin, R.aggregate, R.sort, R.variable


class _Pool:
    """Stands in for IO/pinned_mem.GPUMemory: plain allocations, no slab."""

    def malloc_like(self, t):
        return 0, torch.empty_like(t)


# --------------------------------------------------------------------------
# Synthetic inputs (same distributions as the benchmark generators)
# --------------------------------------------------------------------------
def lineitem_like(rng, n):
    return {
        "quantity": rng.integers(1, 51, n).astype(np.float64),
        "price": rng.integers(90000, 10495001, n).astype(np.float64) / 100.0,
        "discount": rng.integers(0, 11, n).astype(np.float64) / 100.0,
        "tax": rng.integers(0, 9, n).astype(np.float64) / 100.0,
        "flag": rng.integers(0, 3, n).astype(np.uint8),
        "status": rng.integers(0, 2, n).astype(np.uint8),
        "ship_date": rng.integers(0, 2557, n).astype(np.int32),
    }


CASES = {}


def case(fn):
    CASES[fn.__name__] = fn
    return fn


def _save(name, inputs: dict, args: dict, outputs: dict):
    arrays = {f"in_{k}": np.ascontiguousarray(v) for k, v in inputs.items()}
    arrays.update({f"out_{k}": np.ascontiguousarray(v) for k, v in outputs.items()})
    arrays["args"] = np.array(json.dumps(args))
    np.savez_compressed(OUT / f"{name}.npz", **arrays)
    sizes = {k: v.shape for k, v in outputs.items()}
    print(f"{name}: {len(inputs)} inputs, outputs {sizes}")


def _tg(V, cols: dict, types_: dict):
    return {cid: V(torch.from_numpy(np.ascontiguousarray(a)), types_[cid]) for cid, a in cols.items()}


# --------------------------------------------------------------------------
# Cases
# --------------------------------------------------------------------------
@case
def filter_agg_sort_lineitem(ref):
    """Filter (ship_date <= 2470) -> 2-key group-by with 8 aggregates -> sort."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(11)
    n = 20000
    t = lineitem_like(rng, n)
    ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
    types_ = {1: "float", 2: "float", 3: "float", 4: "float", 5: "int", 6: "int", 7: "date"}
    cols = {ids[k]: v for k, v in t.items()}
    tg = _tg(V.Variable, cols, types_)
    fargs = {"name": "Filter", "filter tree": [[["isnotnull", ["ship_date#7"]], "AND", ["ship_date#7", "<=", "2470"]]],
             "materialized in": [7], "out mask id": 900}
    f.tqp_filter(False, tg, copy.deepcopy(fargs), None, None, _Pool(), "f")
    mask = tg[900].tensor.numpy().copy()
    results = [
        "flag#5", "status#6",
        [[["sum", ["quantity#1"]], "#", "101"], "AS", "sum_qty#201"],
        [[["sum", ["price#2"]], "#", "102"], "AS", "sum_base_price#202"],
        [[["sum", [["price#2", "*", ["1.0", "-", "discount#3"]]]], "#", "103"], "AS", "sum_disc_price#203"],
        [[["sum", [[["price#2", "*", ["1.0", "-", "discount#3"]], "*", ["1.0", "+", "tax#4"]]]], "#", "104"], "AS", "sum_charge#204"],
        [[["avg", ["quantity#1"]], "#", "105"], "AS", "avg_qty#205"],
        [[["avg", ["price#2"]], "#", "106"], "AS", "avg_price#206"],
        [[["avg", ["discount#3"]], "#", "107"], "AS", "avg_disc#207"],
        [[["count", ["1"]], "#", "108L"], "AS", "count_order#208"],
    ]
    aargs = {"name": "Aggregate", "is partial": False, "keys": ["flag#5", "status#6"],
             "input ids": [1, 2, 3, 4, 5, 6], "results": results,
             "out agg ids": [201, 202, 203, 204, 205, 206, 207, 208],
             "mask map": {1: 900, 2: 900, 3: 900, 4: 900, 5: 900, 6: 900}}
    torch.manual_seed(0)
    ag.tqp_hash_aggregate(False, tg, copy.deepcopy(aargs), _Pool(), None, "a")
    sargs = {"name": "Sort", "input ids": [5, 6, 201, 202, 203, 204, 205, 206, 207, 208],
             "key ids": [5, 6], "key orders": [False, False]}
    so.tqp_sort(False, tg, copy.deepcopy(sargs), False, "s")
    outs = {"mask": mask}
    for cid in sargs["input ids"]:
        outs[str(cid)] = tg[cid].tensor.numpy()
    _save("filter_agg_sort_lineitem", {str(k): v for k, v in cols.items()},
          {"filter": fargs, "aggregate": _jsonable(aargs), "sort": sargs, "types": types_}, outs)


def _jsonable(d):
    d = copy.deepcopy(d)
    if "mask map" in d:
        d["mask map"] = {str(k): v for k, v in d["mask map"].items()}
    return d


@case
def filter_predicates(ref):
    """One table, many predicate trees through tqp_filter (int, date, float+eps, isclose, IN, NOT, char)."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(12)
    n = 5003
    cols = {
        1: rng.integers(0, 2557, n).astype(np.int32),                      # date
        2: (rng.integers(0, 11, n) / 100.0).astype(np.float64),            # float (0.00..0.10)
        3: rng.integers(-50, 50, n).astype(np.int64),                      # int
        4: rng.integers(65, 70, n).astype(np.uint8),                       # 1-char flags 'A'..'E'
        5: rng.normal(0, 1000, n).astype(np.float64),                      # float, signed
    }
    cols[2][:7] = [0.05, 0.05 + 1e-6, 0.05 - 1e-6, 0.05 + 2e-5, 0.06, 0.07 - 1e-9, 0.0]
    cols[5][:4] = [0.0, -0.0, 100.5, 100.5 + 2e-5]
    types_ = {1: "date", 2: "float", 3: "int", 4: "int", 5: "float"}
    trees = [
        ["d#1", "<=", "2470"],
        ["d#1", "<", "1170"],
        ["d#1", ">", "1170"],
        ["d#1", ">=", "100"],
        ["d#1", "=", "42"],
        [[["d#1", ">=", "100"], "AND", ["d#1", "<", "500"]], "OR", ["d#1", ">", "2500"]],
        ["x#2", "<=", "0.05"],
        ["x#2", ">=", "0.05"],
        ["x#2", "<", "0.05"],
        ["x#2", ">", "0.07"],
        ["x#2", "=", "0.06"],
        [["x#2", ">=", "0.02"], "AND", ["x#2", "<=", "0.04"]],
        ["NOT", [["x#2", ">", "0.08"]]],
        ["k#3", "IN", ["1", "5", "-7", "49"]],
        [["isnotnull", ["k#3"]], "AND", ["k#3", "<", "0"]],
        ["c#4", "=", "B"],
        [["c#4", "=", "A"], "OR", ["c#4", "=", "E"]],
        ["y#5", "<=", "100.5"],
        ["y#5", ">=", "-3.25"],
        ["y#5", "=", "100.5"],
        ["y#5", "<=", "0"],
        ["d#1", "<=", "100.5"],
        [["NOT", [["d#1", "<", "1000"]]], "AND", [["y#5", ">", "0.0"], "OR", ["k#3", "=", "3"]]],
        # date literals: days since 1990-01-01 (conversion.py:26-29), one before the epoch
        ["d#1", "<", "1993-03-15"],
        [["d#1", ">=", "1994-01-01"], "AND", ["d#1", "<", "1995-01-01"]],
        ["d#1", "=", "1992-02-29"],
        ["d#1", ">", "1989-12-31"],
    ]
    outs = {}
    for i, tree in enumerate(trees):
        used = sorted({int(s.split("#")[1]) for s in _leaves(tree) if "#" in s})
        tg = _tg(V.Variable, {c: cols[c] for c in used}, types_)
        fa = {"name": "Filter", "filter tree": [tree], "materialized in": used, "out mask id": 999}
        f.tqp_filter(False, tg, fa, None, None, _Pool(), "f")
        outs[f"mask{i}"] = tg[999].tensor.numpy().astype(np.bool_)
    _save("filter_predicates", {str(k): v for k, v in cols.items()},
          {"trees": trees, "types": types_}, outs)


@case
def filter_strings(ref):
    """String predicates on int8 [N, w] columns through tqp_filter: StartsWith, Contains,
    EndsWith (the reference treats it as Contains), LIKE '%a%b%', multi-character =, IN,
    combined with NOT/AND/OR and numeric comparisons."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(31)
    n = 4099
    words1 = ["STANDARD", "SMALL", "MEDIUM", "LARGE", "ECONOMY", "PROMO"]
    words2 = ["ANODIZED", "BURNISHED", "PLATED", "POLISHED", "BRUSHED"]
    words3 = ["TIN", "NICKEL", "BRASS", "STEEL", "COPPER"]
    w = 25
    types_col = np.zeros((n, w), np.int8)
    for i in range(n):
        s = " ".join([words1[rng.integers(0, 6)], words2[rng.integers(0, 5)], words3[rng.integers(0, 5)]])
        types_col[i, :len(s)] = np.frombuffer(s.encode(), np.uint8).astype(np.int8)
    cont = np.zeros((n, 10), np.int8)
    conts = ["SM CASE", "SM BOX", "MED BAG", "LG PKG", "WRAP JAR", "JUMBO DRUM"]
    for i in range(n):
        s = conts[rng.integers(0, len(conts))]
        cont[i, :len(s)] = np.frombuffer(s.encode(), np.uint8).astype(np.int8)
    cols = {1: types_col, 2: cont, 3: rng.integers(0, 50, n).astype(np.int64)}
    types_ = {1: "string", 2: "string", 3: "int"}
    trees = [
        ["StartsWith", ["t#1", "MEDIUM POLISHED"]],
        ["StartsWith", ["t#1", "PROMO"]],
        ["Contains", ["t#1", "BRASS"]],
        ["EndsWith", ["t#1", "STEEL"]],
        ["NOT", [["Contains", ["t#1", "NICKEL"]]]],
        ["t#1", "LIKE", "%BURNISHED%COPPER%"],
        ["t#1", "LIKE", "%SMALL%TIN%"],
        ["c#2", "=", "SM BOX"],
        ["c#2", "IN", ["SM CASE", "LG PKG", "JUMBO DRUM"]],
        [["StartsWith", ["t#1", "LARGE"]], "AND", ["k#3", "<", "20"]],
        [["c#2", "IN", ["MED BAG", "WRAP JAR"]], "OR", ["Contains", ["t#1", "PLATED"]]],
    ]
    outs = {}
    for i, tree in enumerate(trees):
        used = sorted({int(s.split("#")[1]) for s in _leaves(tree) if "#" in s})
        tg = _tg(V.Variable, {c: cols[c] for c in used}, types_)
        fa = {"name": "Filter", "filter tree": [tree], "materialized in": used, "out mask id": 999}
        f.tqp_filter(False, tg, fa, None, None, _Pool(), "f")
        outs[f"mask{i}"] = tg[999].tensor.numpy().astype(np.bool_)
    _save("filter_strings", {str(k): v for k, v in cols.items()}, {"trees": trees, "types": types_}, outs)


@case
def filter_substring(ref):
    """substring(col, start, width) in filters (filter.py:71-76): IN over a 2-byte prefix (the
    customer phone country code), = on a leading slice, a slice clipped at the row's end, and a
    multi-character literal under '>' (the reference compares for equality whatever the
    operator, filter.py:151-158)."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(37)
    n = 5003
    phone = np.zeros((n, 15), np.int8)
    for i in range(n):
        s = f"{rng.integers(10, 35)}-{rng.integers(100, 1000)}-{rng.integers(100, 1000)}-{rng.integers(1000, 10000)}"
        phone[i, :len(s)] = np.frombuffer(s.encode(), np.uint8).astype(np.int8)
    nation = _strings(rng, ["CANADA", "BRAZIL", "PERU", "CHINA"], n, 25)
    cols = {1: phone, 2: nation, 3: rng.normal(4000.0, 3000.0, n)}
    types_ = {1: "string", 2: "string", 3: "float"}
    trees = [
        [["substring", ["p#1", "1", "2"]], "IN", ["13", "31", "23", "29", "30", "18", "17"]],
        [[["isnotnull", ["b#3"]], "AND", [["substring", ["p#1", "1", "2"]], "IN", ["13", "31", "23", "29", "30"]]],
         "AND", ["b#3", ">", "0.0"]],
        [["substring", ["n#2", "1", "3"]], "=", "CAN"],
        [["substring", ["p#1", "14", "5"]], "IN", ["12", "34", "56"]],
        ["n#2", ">", "CANADA"],
        ["NOT", [[["substring", ["n#2", "2", "3"]], "=", "ERU"]]],
    ]
    outs = {}
    for i, tree in enumerate(trees):
        used = sorted({int(s.split("#")[1]) for s in _leaves(tree) if "#" in s})
        tg = _tg(V.Variable, {c: cols[c] for c in used}, types_)
        fa = {"name": "Filter", "filter tree": [tree], "materialized in": used, "out mask id": 999}
        f.tqp_filter(False, tg, fa, None, None, _Pool(), "f")
        outs[f"mask{i}"] = tg[999].tensor.numpy().astype(np.bool_)
    _save("filter_substring", {str(k): v for k, v in cols.items()}, {"trees": trees, "types": types_}, outs)


def _leaves(t):
    if isinstance(t, str):
        yield t
    else:
        for e in t:
            yield from _leaves(e)


def _join_case(ref, name, rng, nb, npb, key_gen, jtype):
    f, hj, ag, so, V = ref
    bkey = key_gen(rng, nb)
    cols = {
        11: bkey,
        12: rng.integers(0, 2557, nb).astype(np.int32),
        21: rng.integers(1, max(2, nb) + 1, npb).astype(np.int32),
        22: rng.integers(0, 2557, npb).astype(np.int32),
        23: rng.integers(90000, 10495001, npb).astype(np.float64) / 100.0,
        24: rng.integers(0, 11, npb).astype(np.float64) / 100.0,
    }
    types_ = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}
    tg = _tg(V.Variable, cols, types_)
    f1 = {"name": "Filter", "filter tree": [["bd#12", "<", "1170"]], "materialized in": [12], "out mask id": 901}
    f2 = {"name": "Filter", "filter tree": [["pd#22", ">", "1170"]], "materialized in": [22], "out mask id": 902}
    f.tqp_filter(False, tg, copy.deepcopy(f1), None, None, _Pool(), "f1")
    f.tqp_filter(False, tg, copy.deepcopy(f2), None, None, _Pool(), "f2")
    jargs = {"name": "Join", "left group": [11, 12], "right group": [21, 22, 23, 24],
             "materialized in": [11, 21, 23, 24], "mask map": {11: 901, 21: 902, 23: 902, 24: 902},
             "left keys": [11], "right keys": [21], "join type": jtype}
    jt = {"Inner": "inner", "LeftSemi": "right-semi", "LeftOuter": "right-outer", "LeftAnti": "right-anti"}[jtype]
    rows = hj.join_vortex(False, tg, copy.deepcopy(jargs), 11, 21, [], jt, None, _Pool(), "j")
    outs = {"rows": np.array(rows), "mask901": tg[901].tensor.numpy(), "mask902": tg[902].tensor.numpy()}
    for k in [11, 21, 23, 24]:
        outs[str(k)] = tg[k].tensor.numpy()
    args = {"filters": [f1, f2], "join": _jsonable(jargs), "type": jt, "types": types_}
    if jtype == "Inner":
        aargs = {"name": "Aggregate", "is partial": False, "keys": ["bkey#11"], "input ids": [11, 23, 24],
                 "results": ["bkey#11", [[["sum", [["price#23", "*", ["1.0", "-", "disc#24"]]]], "#", "301"], "AS", "revenue#302"]],
                 "out agg ids": [302]}
        torch.manual_seed(1)
        ag.tqp_hash_aggregate(False, tg, copy.deepcopy(aargs), _Pool(), None, "a")
        outs["agg_key"] = tg[11].tensor.numpy()
        outs["agg_revenue"] = tg[302].tensor.numpy()
        targs = {"name": "take ordered", "limit": 10, "input ids": [11, 302], "key ids": [302], "key orders": [True]}
        so.tqp_sort(False, tg, copy.deepcopy(targs), True, "t")
        outs["top_key"] = tg[11].tensor.numpy()
        outs["top_revenue"] = tg[302].tensor.numpy()
        args.update({"aggregate": aargs, "topk": targs})
    _save(name, {str(k): v for k, v in cols.items()}, args, outs)


@case
def join_agg_topk_unique(ref):
    """Filtered build (unique keys) x filtered probe -> inner join -> group-by build key -> top-10."""
    _join_case(ref, "join_agg_topk_unique", np.random.default_rng(13), 6000, 24000,
               lambda rng, n: (rng.permutation(n) + 1).astype(np.int32), "Inner")


@case
def join_duplicates(ref):
    """Build keys with duplicates (lmax > 1), inner join."""
    _join_case(ref, "join_duplicates", np.random.default_rng(14), 3000, 9000,
               lambda rng, n: rng.integers(1, n // 3 + 1, n).astype(np.int32), "Inner")


@case
def join_semi(ref):
    _join_case(ref, "join_semi", np.random.default_rng(15), 2000, 7000,
               lambda rng, n: rng.integers(1, n // 2 + 1, n).astype(np.int32), "LeftSemi")


@case
def join_anti(ref):
    _join_case(ref, "join_anti", np.random.default_rng(16), 2000, 7000,
               lambda rng, n: rng.integers(1, n // 2 + 1, n).astype(np.int32), "LeftAnti")


@case
def join_outer(ref):
    _join_case(ref, "join_outer", np.random.default_rng(17), 2000, 7000,
               lambda rng, n: rng.integers(1, n // 2 + 1, n).astype(np.int32), "LeftOuter")


@case
def join_kernel_direct(ref):
    """join_kernel_new called directly: int64 keys, negative keys, empty-match and no-duplicate edge cases."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(18)
    outs, inputs = {}, {}
    specs = [
        ("neg", rng.integers(-1000, 1000, 1500).astype(np.int64), rng.integers(-1200, 1200, 4000).astype(np.int64)),
        ("nomatch", np.arange(0, 500, dtype=np.int64), np.arange(1000, 1400, dtype=np.int64)),
        ("big", (rng.integers(0, 2**40, 800) * 3).astype(np.int64), None),
        ("single", np.array([7], dtype=np.int64), np.array([7, 7, 1, 7], dtype=np.int64)),
    ]
    for name, lk, rk in specs:
        if rk is None:
            rk = np.concatenate([lk[rng.integers(0, lk.size, 1500)], rng.integers(0, 2**40, 500).astype(np.int64)])
        L = {1: V.Variable(torch.from_numpy(lk), "int"), 2: V.Variable(torch.arange(lk.size, dtype=torch.int64), "int")}
        R = {3: V.Variable(torch.from_numpy(rk), "int"), 4: V.Variable(torch.arange(rk.size, dtype=torch.int64), "int")}
        res = hj.join_kernel_new(False, L, R, 1, 3, [], [2, 4], False, "inner", None, None)
        inputs[f"{name}_left"], inputs[f"{name}_right"] = lk, rk
        outs[f"{name}_lidx"] = res[0].numpy()
        outs[f"{name}_ridx"] = res[1].numpy()
    _save("join_kernel_direct", inputs, {"specs": [s[0] for s in specs]}, outs)


@case
def aggregate_ops(ref):
    """Group-by over int32+int64 keys with sum/avg/count/min/max on int and float values; global aggregate."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(19)
    n = 30000
    cols = {
        1: rng.integers(-3, 4, n).astype(np.int32),
        2: rng.integers(0, 200, n).astype(np.int64),
        3: rng.normal(10.0, 50.0, n).astype(np.float64),
        4: rng.integers(0, 1000, n).astype(np.int64),
    }
    types_ = {1: "int", 2: "int", 3: "float", 4: "int"}
    results = [
        "k1#1", "k2#2",
        [[["sum", ["v#3"]], "#", "401"], "AS", "s#501"],
        [[["avg", ["v#3"]], "#", "402"], "AS", "a#502"],
        [[["min", ["v#3"]], "#", "403"], "AS", "mn#503"],
        [[["max", ["w#4"]], "#", "404"], "AS", "mx#504"],
        [[["sum", ["w#4"]], "#", "405"], "AS", "si#505"],
        [[["count", ["w#4"]], "#", "406L"], "AS", "c#506"],
        [[["sum", [["v#3", "*", "2.5"]]], "#", "407"], "AS", "e#507"],
        [[["min", ["w#4"]], "#", "408"], "AS", "mni#508"],
    ]
    aargs = {"name": "Aggregate", "is partial": False, "keys": ["k1#1", "k2#2"], "input ids": [1, 2, 3, 4],
             "results": results, "out agg ids": [501, 502, 503, 504, 505, 506, 507, 508]}
    tg = _tg(V.Variable, cols, types_)
    torch.manual_seed(2)
    ag.tqp_hash_aggregate(False, tg, copy.deepcopy(aargs), _Pool(), None, "a")
    outs = {str(c): tg[c].tensor.numpy() for c in [1, 2, 501, 502, 503, 504, 505, 506, 507, 508]}
    # global (no keys) aggregate over the same table
    gres = [[[["sum", ["v#3"]], "#", "411"], "AS", "gs#511"],
            [[["count", ["1"]], "#", "412L"], "AS", "gc#512"],
            [[["max", ["v#3"]], "#", "413"], "AS", "gm#513"],
            [[["avg", ["w#4"]], "#", "414"], "AS", "ga#514"]]
    gargs = {"name": "Aggregate", "is partial": False, "keys": None, "input ids": [3, 4],
             "results": gres, "out agg ids": [511, 512, 513, 514]}
    tg2 = _tg(V.Variable, {3: cols[3], 4: cols[4]}, types_)
    ag.tqp_hash_aggregate(False, tg2, copy.deepcopy(gargs), _Pool(), None, "g")
    for c in [511, 512, 513, 514]:
        outs[str(c)] = tg2[c].tensor.numpy()
    _save("aggregate_ops", {str(k): v for k, v in cols.items()},
          {"aggregate": aargs, "global": gargs, "types": types_}, outs)


def _strings(rng, words, n, w):
    """An int8 [n, w] string column of the given words (conversion.py:36-37 layout)."""
    pick = rng.integers(0, len(words), n)
    out = np.zeros((n, w), np.int8)
    for i, wd in enumerate(words):
        b = np.frombuffer(wd.encode(), np.uint8).astype(np.int8)
        out[pick == i, :len(b)] = b
    return out


@case
def aggregate_expressions(ref):
    """tqp_project (year(), CASE WHEN over a string condition, arithmetic, a comparison as a
    value) feeding tqp_hash_aggregate with CASE WHEN conditions (string equality with the
    split '1-URGENT' literal, OR/AND/NOT, StartsWith, numeric comparisons without the
    filter's eps), year(), and arithmetic over aggregates (100 * sum / sum, sum / sum)."""
    f, hj, ag, so, V = ref
    from operators import project as pj
    rng = np.random.default_rng(23)
    n = 20000
    cols = {
        1: rng.integers(1, 51, n).astype(np.float64),
        2: rng.integers(90000, 10495001, n).astype(np.float64) / 100.0,
        3: rng.integers(0, 11, n).astype(np.float64) / 100.0,
        6: _strings(rng, ["1-URGENT", "2-HIGH", "3-MEDIUM", "4-NOT SPECIFIED", "5-LOW"], n, 15),
        7: rng.integers(0, 3652, n).astype(np.int32),
        8: _strings(rng, ["PROMO BRUSHED COPPER", "STANDARD POLISHED TIN", "PROMO ANODIZED STEEL",
                          "ECONOMY BURNISHED NICKEL", "MEDIUM PLATED BRASS"], n, 25),
        9: _strings(rng, ["BRAZIL", "CANADA", "PERU", "ARGENTINA", "BRAZILIA"], n, 25),
        10: rng.integers(0, 3, n).astype(np.uint8),
    }
    types_ = {1: "float", 2: "float", 3: "float", 6: "string", 7: "date", 8: "string", 9: "string", 10: "int"}
    tg = _tg(V.Variable, cols, types_)
    pargs = {"name": "Project", "rename map": {}, "materialized in": [1, 2, 3, 7, 9],
             "used expr": [[["year", ["ship_date#7"]], "AS", "y#20"],
                           [["CASE", "WHEN", ["nation#9", "=", "BRAZIL"], "THEN", "price#2", "ELSE", "0.0", "END"],
                            "AS", "v#21"],
                           [[["price#2", "*", ["1.0", "-", "discount#3"]]], "AS", "w#22"],
                           [["quantity#1", "<", "10"], "AS", "b#23"]],
             "materialized out": [20, 21, 22, 23]}
    pj.tqp_project(False, tg, copy.deepcopy(pargs), None, _Pool(), "p")
    proj = {str(c): tg[c].tensor.numpy().copy() for c in (20, 21, 22, 23)}
    disc_price = [["price#2", "*", ["1.0", "-", "discount#3"]]]
    urgent = [[["prio#6", "=", ["1", "-", "URGENT"]]], "OR", [["prio#6", "=", ["2", "-", "HIGH"]]]]
    not_urgent = [["NOT", [["prio#6", "=", ["1", "-", "URGENT"]]]], "AND", ["NOT", [["prio#6", "=", ["2", "-", "HIGH"]]]]]
    results = [
        "flag#10", "y#20",
        [[["sum", ["CASE", "WHEN", urgent, "THEN", "1", "ELSE", "0", "END"]], "#", "301L"], "AS", "high#401L"],
        [[["sum", ["CASE", "WHEN", not_urgent, "THEN", "1", "ELSE", "0", "END"]], "#", "302L"], "AS", "low#402L"],
        [[["100.0", "*", [["sum", ["CASE", "WHEN", ["StartsWith", ["p_type#8", "PROMO"]], "THEN", disc_price,
                                   "ELSE", "0.0", "END"]], "#", "303"]], "/", [["sum", disc_price], "#", "304"]],
         "AS", "promo#403"],
        [[[["sum", ["CASE", "WHEN", ["nation#9", "=", "BRAZIL"], "THEN", "price#2", "ELSE", "0.0", "END"]], "#", "305"],
          "/", [["sum", "price#2"], "#", "306"]], "AS", "share#404"],
        [[["sum", ["CASE", "WHEN", ["quantity#1", "<", "10"], "THEN", "price#2", "ELSE", "0.0", "END"]], "#", "307"],
         "AS", "small#405"],
        [[["avg", ["CASE", "WHEN", ["discount#3", ">=", "0.05"], "THEN", "quantity#1", "ELSE", "0.0", "END"]], "#",
          "308"], "AS", "avgq#406"],
        [[["max", ["CASE", "WHEN", ["quantity#1", "<>", "25.0"], "THEN", "ship_date#7", "ELSE", "0", "END"]], "#",
          "309"], "AS", "mx#407"],
        [[["min", [["year", ["ship_date#7"]]]], "#", "310"], "AS", "miny#408"],
        [[["count", ["CASE", "WHEN", ["price#2", ">", "50000.5"], "THEN", "quantity#1", "ELSE", "-64.0", "END"]],
          "#", "311L"], "AS", "cnt#409L"],
        [[["sum", [["year", ["ship_date#7"]]]], "#", "312L"], "AS", "sumy#410L"],
    ]
    aargs = {"name": "Aggregate", "is partial": False, "keys": ["flag#10", "y#20"],
             "input ids": [1, 2, 3, 6, 7, 8, 9, 10, 20], "results": results,
             "out agg ids": [401, 402, 403, 404, 405, 406, 407, 408, 409, 410]}
    torch.manual_seed(5)
    ag.tqp_hash_aggregate(False, tg, copy.deepcopy(aargs), _Pool(), None, "a")
    outs = {str(c): tg[c].tensor.numpy() for c in [10, 20] + aargs["out agg ids"]}
    outs.update({f"p{k}": v for k, v in proj.items()})
    _save("aggregate_expressions", {str(k): v for k, v in cols.items()},
          {"project": pargs, "aggregate": aargs, "types": types_}, outs)


@case
def aggregate_string_keys(ref):
    """Group keys the reference stacks as 2-D (aggregate.py:291-311): a string key alone, five
    keys mixing int, string, float and uint8 (more than four), and a float key with -0.0 and
    +0.0 rows; under a late-materialisation mask."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(41)
    n = 30011
    cust = rng.integers(0, 60, n).astype(np.int64)
    phone = np.zeros((n, 15), np.int8)
    for c in range(60):
        s_ = f"{10 + c % 25}-{100 + c}-{200 + 3 * c}-{1000 + 7 * c}"
        phone[cust == c, :len(s_)] = np.frombuffer(s_.encode(), np.uint8).astype(np.int8)
    acct = (cust - 10).astype(np.float64) * 1.5
    acct[rng.integers(0, n, 500)] = -0.0
    cols = {
        1: _strings(rng, ["MAIL", "SHIP", "AIR", "REG AIR", "TRUCK", "RAIL", "FOB"], n, 10),
        2: _strings(rng, ["BRAZIL", "CANADA", "PERU", "CHINA"], n, 25),
        3: cust, 4: acct,
        5: rng.integers(90000, 10495001, n).astype(np.float64) / 100.0,
        6: rng.integers(0, 3, n).astype(np.uint8),
        7: phone,
        8: rng.integers(0, 2570, n).astype(np.int32),
    }
    types_ = {1: "string", 2: "string", 3: "int", 4: "float", 5: "float", 6: "int", 7: "string", 8: "date"}
    fargs = {"name": "Filter", "filter tree": [["d#8", "<", "2400"]], "materialized in": [8], "out mask id": 900}
    tg = _tg(V.Variable, cols, types_)
    f.tqp_filter(False, tg, copy.deepcopy(fargs), None, None, _Pool(), "f")
    mask = tg[900].tensor.numpy().copy()
    sets = {
        "a": {"keys": ["mode#1"], "input ids": [1, 5],
              "results": ["mode#1", [[["sum", ["p#5"]], "#", "11"], "AS", "s#111"],
                          [[["count", ["1"]], "#", "12L"], "AS", "c#112L"], [[["min", ["p#5"]], "#", "13"], "AS", "m#113"]],
              "out agg ids": [111, 112, 113]},
        "b": {"keys": ["ck#3", "nat#2", "bal#4", "ph#7", "fl#6"], "input ids": [2, 3, 4, 5, 6, 7],
              "results": ["ck#3", "nat#2", "bal#4", "ph#7", "fl#6", [[["sum", ["p#5"]], "#", "21"], "AS", "s#121"],
                          [[["avg", ["p#5"]], "#", "22"], "AS", "a#122"]],
              "out agg ids": [121, 122]},
        "c": {"keys": ["bal#4"], "input ids": [4, 5],
              "results": ["bal#4", [[["count", ["1"]], "#", "31L"], "AS", "c#131L"],
                          [[["max", ["p#5"]], "#", "32"], "AS", "x#132"]],
              "out agg ids": [131, 132]},
    }
    outs = {"mask": mask}
    for name, a_ in sets.items():
        aargs = dict(a_, **{"name": "Aggregate", "is partial": False,
                            "mask map": {c: 900 for c in a_["input ids"]}})
        tgi = _tg(V.Variable, cols, types_)
        tgi[900] = tg[900]
        torch.manual_seed(7)
        ag.tqp_hash_aggregate(False, tgi, copy.deepcopy(aargs), _Pool(), None, "a")
        key_ids = [int(k.split("#")[-1]) for k in a_["keys"]]
        for c in key_ids + a_["out agg ids"]:
            outs[f"{name}_{c}"] = tgi[c].tensor.numpy()
        sets[name] = _jsonable(aargs)
    _save("aggregate_string_keys", {str(k): v for k, v in cols.items()},
          {"filter": fargs, "sets": sets, "types": types_}, outs)


@case
def aggregate_two_step(ref):
    """rows/groups >= 2^16 selects the reference's 2-step scatter_reduce path."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(20)
    n = 140000
    cols = {1: rng.integers(0, 2, n).astype(np.int64),
            2: (rng.integers(90000, 10495001, n) / 100.0).astype(np.float64),
            3: rng.integers(1, 51, n).astype(np.int64)}
    types_ = {1: "int", 2: "float", 3: "int"}
    results = ["g#1",
               [[["sum", ["p#2"]], "#", "601"], "AS", "s#701"],
               [[["avg", ["p#2"]], "#", "602"], "AS", "a#702"],
               [[["min", ["p#2"]], "#", "603"], "AS", "mn#703"],
               [[["max", ["q#3"]], "#", "604"], "AS", "mx#704"],
               [[["count", ["1"]], "#", "605L"], "AS", "c#705"],
               [[["sum", ["q#3"]], "#", "606"], "AS", "sq#706"]]
    aargs = {"name": "Aggregate", "is partial": False, "keys": ["g#1"], "input ids": [1, 2, 3],
             "results": results, "out agg ids": [701, 702, 703, 704, 705, 706]}
    tg = _tg(V.Variable, cols, types_)
    torch.manual_seed(3)
    ag.tqp_hash_aggregate(False, tg, copy.deepcopy(aargs), _Pool(), None, "a")
    outs = {str(c): tg[c].tensor.numpy() for c in [1, 701, 702, 703, 704, 705, 706]}
    _save("aggregate_two_step", {str(k): v for k, v in cols.items()}, {"aggregate": aargs, "types": types_}, outs)


@case
def aggregate_float32(ref):
    """torch's float32 results: an integer column with a Python float, integer true division and a
    CASE mixing a float literal with integers (aggregate.py:76-87, :203-233), under sum, avg, min,
    max and count; float32 meeting a float64 column widens to float64.  Two aggregates: 4 groups
    (the 1-step path: float32 bincount sums) and 2 groups of 70,000 rows (the 2-step path, whose avg
    is float64, :170)."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(29)
    ins, outs, args = {}, {}, {}
    for tag, n, g in (("one", 30000, 4), ("two", 140000, 2)):
        cols = {1: rng.integers(0, g, n).astype(np.int64),
                2: rng.integers(1, 51, n).astype(np.int64),
                3: rng.integers(1, 10, n).astype(np.int64),
                4: (rng.integers(90000, 10495001, n) / 100.0).astype(np.float64)}
        types_ = {1: "int", 2: "int", 3: "int", 4: "float"}
        results = ["g#1",
                   [[["sum", [["q#2", "*", "1.5"]]], "#", "801"], "AS", "a#901"],
                   [[["avg", [["q#2", "*", "0.1"]]], "#", "802"], "AS", "b#902"],
                   [[["sum", [["q#2", "/", "d#3"]]], "#", "803"], "AS", "c#903"],
                   [[["min", [["q#2", "*", "1.5"]]], "#", "804"], "AS", "d#904"],
                   [[["max", [["d#3", "/", "q#2"]]], "#", "805"], "AS", "e#905"],
                   [[["sum", ["CASE", "WHEN", ["q#2", ">", "25"], "THEN", "1.0", "ELSE", "0", "END"]], "#", "806"],
                    "AS", "f#906"],
                   [[["count", [["q#2", "*", "0.5"]]], "#", "807L"], "AS", "h#907L"],
                   [[["sum", [["p#4", "*", ["q#2", "*", "0.5"]]]], "#", "808"], "AS", "i#908"],
                   [[["sum", [[["q#2", "*", "0.25"], "+", "d#3"]]], "#", "809"], "AS", "j#909"]]
        aargs = {"name": "Aggregate", "is partial": False, "keys": ["g#1"], "input ids": [1, 2, 3, 4],
                 "results": results, "out agg ids": [901, 902, 903, 904, 905, 906, 907, 908, 909]}
        tg = _tg(V.Variable, cols, types_)
        torch.manual_seed(7)
        ag.tqp_hash_aggregate(False, tg, copy.deepcopy(aargs), _Pool(), None, "a")
        for c in [1] + aargs["out agg ids"]:
            outs[f"{tag}_{c}"] = tg[c].tensor.numpy()
            outs[f"{tag}_{c}_type"] = np.array(tg[c].tensor_type)
        for c, v in cols.items():
            ins[f"{tag}_{c}"] = v
        args[tag] = {"aggregate": aargs, "types": types_}
        if tag == "one":                 # the same expressions as a projection (project.py:20-67)
            from operators import project as pj
            pargs = {"name": "Project", "rename map": {}, "materialized in": [2, 3, 4],
                     "used expr": [[[["q#2", "*", "1.5"]], "AS", "x#41"], [[["q#2", "/", "d#3"]], "AS", "y#42"],
                                   [[["p#4", "*", ["q#2", "*", "0.5"]]], "AS", "z#43"]],
                     "materialized out": [41, 42, 43]}
            tg = _tg(V.Variable, cols, types_)
            pj.tqp_project(False, tg, copy.deepcopy(pargs), None, _Pool(), "p")
            for c in pargs["materialized out"]:
                outs[f"proj_{c}"] = tg[c].tensor.numpy().copy()
                outs[f"proj_{c}_type"] = np.array([tg[c].tensor_type])
            args["project"] = pargs
    _save("aggregate_float32", ins, args, outs)


@case
def aggregate_substring(ref):
    """substring(col, l, 1) as an aggregate value (aggregate.py:114-119): sum and count of the
    one-byte slice (squeezed to [N], :179-182), alone and times a Python int."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(37)
    n = 12000
    cols = {1: rng.integers(0, 5, n).astype(np.int64),
            2: _strings(rng, ["BRAZIL", "CANADA", "PERU", "ARGENTINA", "CHINA", "EGYPT"], n, 25)}
    types_ = {1: "int", 2: "string"}
    results = ["g#1",
               [[["sum", [["substring", ["c#2", "1", "1"]]]], "#", "501"], "AS", "a#601"],
               [[["count", [["substring", ["c#2", "2", "1"]]]], "#", "502L"], "AS", "b#602L"],
               [[["sum", [[["substring", ["c#2", "3", "1"]], "*", "2"]]], "#", "503"], "AS", "c#603"]]
    aargs = {"name": "Aggregate", "is partial": False, "keys": ["g#1"], "input ids": [1, 2],
             "results": results, "out agg ids": [601, 602, 603]}
    tg = _tg(V.Variable, cols, types_)
    torch.manual_seed(11)
    ag.tqp_hash_aggregate(False, tg, copy.deepcopy(aargs), _Pool(), None, "a")
    outs = {str(c): tg[c].tensor.numpy() for c in [1, 601, 602, 603]}
    _save("aggregate_substring", {str(k): v for k, v in cols.items()}, {"aggregate": aargs, "types": types_}, outs)


@case
def sort_multikey(ref):
    """tqp_sort: multi-key (desc float, asc int, desc int), ties, limit; plus [G,1] 2-D keys."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(21)
    n = 4000
    cols = {1: rng.integers(0, 5, n).astype(np.float64) * 0.5,
            2: rng.integers(-20, 20, n).astype(np.int64),
            3: rng.integers(0, 3, n).astype(np.int32),
            4: np.arange(n, dtype=np.int64),
            5: rng.integers(0, 4, (n, 1)).astype(np.uint8)}
    cols[1][:3] = [-0.0, 0.0, -1.5]
    types_ = {1: "float", 2: "int", 3: "date", 4: "int", 5: "int"}
    outs = {}
    specs = [
        ({"input ids": [1, 2, 3, 4], "key ids": [1, 2, 3], "key orders": [True, False, True]}, False),
        ({"input ids": [1, 2, 3, 4], "key ids": [2], "key orders": [True], "limit": 25}, True),
        ({"input ids": [1, 2, 4], "key ids": [1], "key orders": [False], "limit": 100}, True),
        ({"input ids": [5, 4], "key ids": [5, 2], "key orders": [False, True]}, False),
    ]
    for i, (sa, lim) in enumerate(specs):
        used = sorted(set(sa["input ids"]) | set(sa["key ids"]))
        tg = _tg(V.Variable, {c: cols[c] for c in used}, types_)
        so.tqp_sort(False, tg, copy.deepcopy(sa), lim, "s")
        for c in sa["input ids"]:
            outs[f"s{i}_{c}"] = tg[c].tensor.numpy()
    _save("sort_multikey", {str(k): v for k, v in cols.items()},
          {"specs": [[s, l] for s, l in specs], "types": types_}, outs)


@case
def late_materialisation_masks(ref):
    """Operators whose inputs do not share one mask (vortex_pipeline.py:54-58 compacts each
    masked input by its own mask): an aggregate over masked columns beside an already compacted
    one, an aggregate over two different masks with equal counts, and a join whose probe side
    mixes masked and compacted columns."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(53)
    n = 20011
    m900 = rng.random(n) < 0.6
    kept = int(m900.sum())
    m901 = np.roll(m900, 7)                                # another mask with the same count
    cols = {1: rng.integers(0, 40, n).astype(np.int64), 3: rng.normal(100.0, 30.0, n),
            6: rng.normal(5.0, 2.0, kept), 7: rng.integers(-50, 50, n).astype(np.int64),
            900: m900, 901: m901}
    types_ = {1: "int", 3: "float", 6: "float", 7: "int", 900: "bool", 901: "bool"}
    res = ["k#1", [[["sum", ["v#3"]], "#", "601"], "AS", "s#611"], [[["sum", ["w#6"]], "#", "602"], "AS", "t#612"],
           [[["count", ["1"]], "#", "603L"], "AS", "c#613"], [[["max", ["v#3"]], "#", "604"], "AS", "m#614"]]
    mixed = {"name": "Aggregate", "is partial": False, "keys": ["k#1"], "input ids": [1, 3, 6], "results": res,
             "out agg ids": [611, 612, 613, 614], "mask map": {1: 900, 3: 900}}
    tg = _tg(V.Variable, {c: cols[c] for c in (1, 3, 6, 900)}, types_)
    torch.manual_seed(3)
    ag.tqp_hash_aggregate(False, tg, copy.deepcopy(mixed), _Pool(), None, "a")
    outs = {f"mixed_{c}": tg[c].tensor.numpy() for c in (1, 611, 612, 613, 614)}
    res2 = ["k#1", [[["sum", ["v#3"]], "#", "621"], "AS", "s#631"], [[["sum", ["x#7"]], "#", "622"], "AS", "t#632"]]
    two = {"name": "Aggregate", "is partial": False, "keys": ["k#1"], "input ids": [1, 3, 7], "results": res2,
           "out agg ids": [631, 632], "mask map": {1: 900, 3: 900, 7: 901}}
    tg = _tg(V.Variable, {c: cols[c] for c in (1, 3, 7, 900, 901)}, types_)
    torch.manual_seed(4)
    ag.tqp_hash_aggregate(False, tg, copy.deepcopy(two), _Pool(), None, "a")
    outs.update({f"two_{c}": tg[c].tensor.numpy() for c in (1, 631, 632)})
    # join: build side filtered (mask 911), probe side = key and value masked by 912 beside a
    # column already compacted by that filter
    nb, npr = 3001, 12007
    b_key = (rng.permutation(nb) + 1).astype(np.int32)
    m911 = rng.random(nb) < 0.5
    p_key = rng.integers(1, nb + 1, npr).astype(np.int32)
    m912 = rng.random(npr) < 0.55
    jcols = {11: b_key, 21: p_key, 23: rng.normal(10.0, 3.0, npr), 26: rng.integers(0, 9, int(m912.sum())).astype(np.int64),
             911: m911, 912: m912}
    jtypes = {11: "int", 21: "int", 23: "float", 26: "int", 911: "bool", 912: "bool"}
    jargs = {"name": "Join", "left group": [11], "right group": [21, 23, 26], "materialized in": [11, 21, 23, 26],
             "mask map": {11: 911, 21: 912, 23: 912}}
    tg = _tg(V.Variable, jcols, jtypes)
    hj.join_vortex(False, tg, copy.deepcopy(jargs), 11, 21, [], "inner", None, _Pool(), "j")
    outs.update({f"join_{c}": tg[c].tensor.numpy() for c in (11, 21, 23, 26)})
    ins = {str(k): v for k, v in cols.items()}
    ins.update({f"j{k}": v for k, v in jcols.items()})
    _save("late_materialisation_masks", ins, {"mixed": _jsonable(mixed), "two": _jsonable(two), "join": _jsonable(jargs),
                                              "types": types_, "jtypes": jtypes}, outs)


@case
def join_outer_string_payload(ref):
    """A right-outer join that must null-fill an int8 [N, w] build-side payload: the reference's
    index_with_null (conversion.py:52-57) masks [M, w] rows with an [M] mask, which torch does
    not broadcast, so the operator raises; the fixture records the error class."""
    f, hj, ag, so, V = ref
    rng = np.random.default_rng(59)
    nb, npr = 400, 1500
    cols = {11: (rng.permutation(nb) + 1).astype(np.int32), 13: _strings(rng, ["RED", "GREEN", "BLUE"], nb, 10),
            21: rng.integers(1, 2 * nb, npr).astype(np.int32)}
    types_ = {11: "int", 13: "string", 21: "int"}
    jargs = {"name": "Join", "left group": [11, 13], "right group": [21], "materialized in": [11, 13, 21]}
    tg = _tg(V.Variable, cols, types_)
    try:
        hj.join_vortex(False, tg, copy.deepcopy(jargs), 11, 21, [], "right-outer", None, _Pool(), "j")
        err = ""
    except Exception as e:                     # noqa: BLE001  (recorded, not hidden)
        err = type(e).__name__
    _save("join_outer_string_payload", {str(k): v for k, v in cols.items()},
          {"join": jargs, "types": types_, "error": err}, {"raised": np.array(err)})


def main(argv):
    ref = load_reference()
    from oracle import reference
    with reference.cpu_mode():
        for name, fn in CASES.items():
            if len(argv) > 1 and name not in argv[1:]:
                continue
            fn(ref)


if __name__ == "__main__":
    main(sys.argv)
