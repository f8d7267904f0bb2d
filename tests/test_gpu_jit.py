"""Query-specialised (runtime-compiled) kernels against the interpreting kernels and the oracle."""
import copy

import numpy as np
import pytest
import torch

from golden_io import assert_f64_close, load
from oracle import tqp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    from tqpk import build, _lib
    build.build()
    return _lib.load()


def test_nvrtc_available_on_the_gpu_box():
    from tqpk import jit
    assert jit.available(), "NVRTC could not be opened; the hot loops would run interpreted"


@pytest.mark.parametrize("jit_on", ["1", "0"])
def test_lineitem_groupby_both_paths(monkeypatch, jit_on):
    monkeypatch.setenv("TQPK_JIT", jit_on)
    from tqpk import datagen
    from tqpk.operators import tqp_filter, tqp_hash_aggregate
    from tqpk.variable import Variable
    _, _, args = load("filter_agg_sort_lineitem")
    t = datagen.lineitem(1_000_003, seed=4)
    ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
    cols = {ids[k]: v for k, v in t.items()}
    tg = {c: Variable(torch.from_numpy(a).cuda(), args["types"][str(c)]) for c, a in cols.items()}
    tqp_filter(True, tg, copy.deepcopy(args["filter"]), None, None, None, "f")
    aargs = copy.deepcopy(args["aggregate"])
    aargs["mask map"] = {int(k): v for k, v in aargs["mask map"].items()}
    tqp_hash_aggregate(True, tg, copy.deepcopy(aargs), None, None, "a")
    oc = dict(cols)
    oc[900] = cols[7] <= 2470
    ref = O.tqp_hash_aggregate(oc, aargs)
    for c in (5, 6):
        np.testing.assert_array_equal(tg[c].tensor.cpu().numpy(), ref[c])
    for a in aargs["out agg ids"]:
        got = tg[a].tensor.cpu().numpy()
        (assert_f64_close if ref[a].dtype == np.float64 else np.testing.assert_array_equal)(got, ref[a])


@pytest.mark.parametrize("jit_on", ["1", "0"])
def test_groupby_predicate_fused_both_paths(monkeypatch, jit_on):
    """The fused predicate form (no mask) with min/max/count-not-null and int sums."""
    monkeypatch.setenv("TQPK_JIT", jit_on)
    from tqpk.expr import compile_aggregate
    from tqpk.ops import groupby
    from tqpk.predicate import compile_filter
    rng = np.random.default_rng(17)
    n = 500_001
    cols = {1: rng.integers(-3, 4, n).astype(np.int32), 2: rng.integers(0, 300, n).astype(np.int64),
            3: rng.normal(10, 50, n), 4: rng.integers(-100, 1000, n).astype(np.int64),
            5: rng.integers(0, 2557, n).astype(np.int32)}
    d = {c: torch.from_numpy(a).cuda() for c, a in cols.items()}
    results = ["k1#1", "k2#2",
               [[["sum", ["v#3"]], "#", "1"], "AS", "s#501"], [[["min", ["v#3"]], "#", "2"], "AS", "a#502"],
               [[["max", ["w#4"]], "#", "3"], "AS", "b#503"], [[["sum", ["w#4"]], "#", "4"], "AS", "c#504"],
               [[["count", ["w#4"]], "#", "5L"], "AS", "d#505"], [[["avg", [["v#3", "*", "2.5"]]], "#", "6"], "AS", "e#506"]]
    args = {"is partial": False, "keys": ["k1#1", "k2#2"], "input ids": [1, 2, 3, 4], "results": results,
            "out agg ids": [501, 502, 503, 504, 505, 506]}
    tree = [[["d#5", ">=", "300"], "AND", ["d#5", "<", "2000"]], "OR", ["v#3", "<=", "0.5"]]
    prog = compile_aggregate(args, d)
    pred = compile_filter(tree, {5: d[5], 3: d[3]})
    keys, outs, G, _ = groupby(prog, n, d[1].device, pred=pred)
    mask = O.eval_filter(tree, cols)
    oc = dict(cols)
    oc[99] = mask
    ref = O.tqp_hash_aggregate(oc, dict(args, **{"mask map": {1: 99, 2: 99, 3: 99, 4: 99}}))
    np.testing.assert_array_equal(keys[0].cpu().numpy(), ref[1].reshape(-1))
    np.testing.assert_array_equal(keys[1].cpu().numpy(), ref[2].reshape(-1))
    # v#3 has both signs: its sums cancel, so their tolerance scales with sum(|v|) per group
    gid = (cols[1][mask].astype(np.int64) + 3) * 300 + cols[2][mask]
    _, inv = np.unique(gid, return_inverse=True)
    absum = np.bincount(inv, weights=np.abs(cols[3][mask]))
    cnt = np.bincount(inv)
    mag = {501: absum, 506: absum * 2.5 / cnt}
    for a in args["out agg ids"]:
        got = outs[a].cpu().numpy()
        if ref[a].dtype == np.float64:
            assert_f64_close(got, ref[a], magnitude=mag.get(a))
        else:
            np.testing.assert_array_equal(got, ref[a])


@pytest.mark.parametrize("jit_on", ["1", "0"])
def test_join_pipeline_both_paths(monkeypatch, jit_on):
    monkeypatch.setenv("TQPK_JIT", jit_on)
    from tqpk import datagen
    from tqpk.pipeline import JoinAggTopK
    t = datagen.join_tables(200_000, 900_001, seed=21)
    d = {k: torch.from_numpy(v).cuda() for k, v in t.items()}
    p = JoinAggTopK(d["b_key"], 1, 200_000, d["p_fk"], {12: d["b_date"]}, [["bd#12", "<", "1170"]],
                    {22: d["p_date"], 23: d["p_price"], 24: d["p_discount"]}, [["pd#22", ">", "1170"]],
                    [["p#23", "*", ["1.0", "-", "d#24"]]], k=10)
    p.run()
    keys, vals, groups = p.result()
    cols = {11: t["b_key"], 12: t["b_date"], 21: t["p_fk"], 22: t["p_date"], 23: t["p_price"], 24: t["p_discount"]}
    oc = dict(cols)
    oc[901] = cols[12] < 1170
    oc[902] = cols[22] > 1170
    res, _ = O.join_vortex(oc, {"left group": [11, 12], "right group": [21, 22, 23, 24],
                                "materialized in": [11, 21, 23, 24],
                                "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}, 11, 21, "inner")
    agg = O.tqp_hash_aggregate(res, {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
                                     "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "1"],
                                                          "AS", "r#302"]], "out agg ids": [302]})
    top = O.tqp_sort({11: agg[11], 302: agg[302]}, {"limit": 10, "input ids": [11, 302], "key ids": [302],
                                                    "key orders": [True]}, True)
    assert groups == agg[11].shape[0]
    np.testing.assert_array_equal(keys, top[11].reshape(-1))
    assert_f64_close(vals, top[302])


@pytest.mark.parametrize("jit_on", ["1", "0"])
def test_shared_table_sums_stay_accurate(monkeypatch, jit_on):
    """Mid-cardinality keys (one table per CTA) with 16k repeated small values per group:
    every sum within 1e-13 of the exactly rounded sum (math.fsum)."""
    monkeypatch.setenv("TQPK_JIT", jit_on)
    import math
    from tqpk import _lib as L
    from tqpk.expr import compile_aggregate
    from tqpk.ops import groupby
    rng = np.random.default_rng(5)
    n, G = 8_000_000, 500
    key = rng.integers(0, G, n).astype(np.int32)
    disc = rng.integers(0, 11, n).astype(np.float64) / 100.0
    d = {1: torch.from_numpy(key).cuda(), 2: torch.from_numpy(disc).cuda()}
    args = {"is partial": False, "keys": ["k#1"], "input ids": [1, 2],
            "results": ["k#1", [[["sum", ["d#2"]], "#", "1"], "AS", "s#601"],
                        [[["avg", ["d#2"]], "#", "2"], "AS", "a#602"]], "out agg ids": [601, 602]}
    prog = compile_aggregate(args, d)
    keys, outs, Gout, plan = groupby(prog, n, d[1].device)
    assert plan.mode == L.GB_DENSE_SHARED
    order = np.argsort(key, kind="stable")
    bounds = np.searchsorted(key[order], np.arange(G + 1))
    exact = np.array([math.fsum(disc[order[bounds[g]:bounds[g + 1]]]) for g in range(G)])
    np.testing.assert_array_equal(keys[0].cpu().numpy(), np.arange(G))
    s = outs[601].cpu().numpy()
    assert np.max(np.abs(s - exact) / np.abs(exact)) <= 1e-13


@pytest.mark.parametrize("n,spec", [
    (1_000_003, "wide"),        # one key over [0, 1e12): far more slots than rows
    (800_000, "q3"),            # three keys: order key x date x priority
    (50_000, "neg"),            # negative keys, int8 + int64
    (0, "wide"),
])
def test_sparse_key_space_groups_through_the_hash_table(n, spec):
    from tqpk import _lib as L
    from tqpk.expr import compile_aggregate
    from tqpk.ops import groupby
    from tqpk.predicate import compile_filter
    rng = np.random.default_rng(n + len(spec))
    if spec == "wide":
        keys = {1: rng.integers(0, 10**12, n).astype(np.int64) // 997 * 997}
    elif spec == "q3":
        keys = {1: rng.integers(1, 6_000_000, n).astype(np.int64), 2: rng.integers(0, 2557, n).astype(np.int32),
                3: np.zeros(n, np.int32)}
    else:
        keys = {1: rng.integers(-120, 120, n).astype(np.int8), 2: rng.integers(-10**10, 10**10, n).astype(np.int64)}
    cols = dict(keys)
    cols[8] = rng.integers(90000, 10495001, n) / 100.0
    cols[9] = rng.integers(0, 11, n) / 100.0
    cols[10] = rng.integers(0, 2557, n).astype(np.int32)
    d = {c: torch.from_numpy(a).cuda() for c, a in cols.items()}
    kn = [f"k{c}#{c}" for c in keys]
    results = kn + [[[["sum", [["p#8", "*", ["1", "-", "d#9"]]]], "#", "1"], "AS", "r#501"],
                    [[["count", ["p#8"]], "#", "2L"], "AS", "c#502"], [[["max", ["d#9"]], "#", "3"], "AS", "m#503"],
                    [[["avg", ["p#8"]], "#", "4"], "AS", "a#504"]]
    args = {"is partial": False, "keys": kn, "input ids": list(keys) + [8, 9], "results": results,
            "out agg ids": [501, 502, 503, 504]}
    tree = [["dt#10", "<", "2000"]]
    prog = compile_aggregate(args, {c: d[c] for c in list(keys) + [8, 9]})
    pred = compile_filter(tree, {10: d[10]})
    out_keys, outs, G, plan = groupby(prog, n, d[8].device, pred=pred)
    if n:
        assert plan.mode == L.GB_HASH
    oc = dict(cols)
    oc[99] = O.eval_filter(tree, cols) if n else np.zeros(0, bool)
    ref = O.tqp_hash_aggregate(oc, dict(args, **{"mask map": {c: 99 for c in list(keys) + [8, 9]}}))
    assert G == (ref[501].shape[0] if n else 0)
    for i, c in enumerate(keys):
        np.testing.assert_array_equal(out_keys[i].cpu().numpy(), ref[c].reshape(-1))
    for a in args["out agg ids"]:
        got = outs[a].cpu().numpy()
        (assert_f64_close if ref[a].dtype == np.float64 else np.testing.assert_array_equal)(got, ref[a])


def test_key_space_beyond_62_bits_raises():
    from tqpk.expr import compile_aggregate
    from tqpk.ops import groupby
    n = 1000
    rng = np.random.default_rng(3)
    cols = {c: rng.integers(-2**40, 2**40, n).astype(np.int64) for c in (1, 2)}
    cols[8] = rng.random(n)
    d = {c: torch.from_numpy(a).cuda() for c, a in cols.items()}
    args = {"is partial": False, "keys": ["a#1", "b#2"], "input ids": [1, 2, 8],
            "results": ["a#1", "b#2", [[["sum", ["v#8"]], "#", "1"], "AS", "s#501"]], "out agg ids": [501]}
    prog = compile_aggregate(args, d)
    with pytest.raises(NotImplementedError):
        groupby(prog, n, d[8].device)


def test_projection_operator_matches_the_oracle():
    """Drop-in tqp_project: renames, float and integer expressions, int32/int64 promotion."""
    from tqpk.operators import tqp_project
    from tqpk.variable import Variable
    rng = np.random.default_rng(12)
    n = 300_007
    cols = {1: rng.integers(90000, 10495001, n) / 100.0, 2: rng.integers(0, 11, n) / 100.0,
            3: rng.integers(-50, 50, n).astype(np.int32), 4: rng.integers(0, 10**9, n).astype(np.int64),
            5: rng.integers(0, 2557, n).astype(np.int32)}
    args = {"rename map": {5: 55},
            "used expr": ["p#1", [["p#1", "AS", "pp#11"]], [[["p#1", "*", ["1", "-", "d#2"]], "AS", "dp#12"]],
                          [[["q#3", "+", "q#3"], "AS", "qq#13"]], [[["w#4", "*", "q#3"], "AS", "wq#14"]],
                          [[["w#4", "-", "3"], "AS", "w3#15"]], [[["p#1", "/", ["q#3", "+", "100"]], "AS", "r#16"]]],
            "materialized in": [1, 2, 3, 4], "materialized out": [12, 13, 14, 15, 16]}
    tg = {c: Variable(torch.from_numpy(a).cuda(), "float" if a.dtype == np.float64 else "int") for c, a in cols.items()}
    assert tqp_project(True, tg, args, None, None) == -1
    ref = O.tqp_project(cols, args)
    assert tg[55] is tg[5]
    for oid in args["materialized out"]:
        got = tg[oid].tensor.cpu().numpy()
        assert got.dtype == ref[oid].dtype, (oid, got.dtype, ref[oid].dtype)
        (assert_f64_close if ref[oid].dtype == np.float64 else np.testing.assert_array_equal)(got, ref[oid])
