"""GPU parity: the CUDA path (through the drop-in operators and the C ABI)
against golden vectors from the reference and against the oracle.

Tolerances: masks, keys, counts, join pairs, sort orders bit-exact; float64
sums and averages within 1e-12 relative (and within 1e-12 of math.fsum)."""
import copy

import numpy as np
import pytest
import torch

from golden_io import assert_f64_close, load, rows_sorted
from oracle import tqp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need CUDA")
    from tqpk import build, _lib
    build.build()
    return _lib.load()


def V(a, t="int"):
    from tqpk.variable import Variable
    return Variable(torch.from_numpy(np.ascontiguousarray(a)).cuda(), t)


def tg_from(ins, types):
    return {int(k): V(v, types[str(k)]) for k, v in ins.items() if isinstance(k, int)}


def np_(t):
    return t.detach().cpu().numpy()


# ------------------------------------------------------------------ filter
def test_filter_predicates_golden():
    from tqpk.operators import tqp_filter
    ins, outs, args = load("filter_predicates")
    for i, tree in enumerate(args["trees"]):
        used = sorted({int(s.split("#")[1]) for s in _leaves(tree) if "#" in s})
        tg = {c: V(ins[c], args["types"][str(c)]) for c in used}
        tqp_filter(True, tg, {"filter tree": [tree], "materialized in": used, "out mask id": 999},
                   None, None, None, "f")
        np.testing.assert_array_equal(np_(tg[999].tensor), outs[f"mask{i}"], err_msg=str(tree))


def test_filter_strings_golden():
    """StartsWith / Contains / EndsWith / LIKE / multi-character = / IN on int8 [N, w] columns."""
    from tqpk.operators import tqp_filter
    ins, outs, args = load("filter_strings")
    for i, tree in enumerate(args["trees"]):
        used = sorted({int(s.split("#")[1]) for s in _leaves(tree) if "#" in s})
        tg = {c: V(ins[c], args["types"][str(c)]) for c in used}
        tqp_filter(True, tg, {"filter tree": [tree], "materialized in": used, "out mask id": 999},
                   None, None, None, "f")
        np.testing.assert_array_equal(np_(tg[999].tensor), outs[f"mask{i}"], err_msg=str(tree))


def test_filter_substring_golden():
    """substring(col, start, width) views: IN over a prefix, = on a slice, a slice clipped at
    the row's end, NOT; a multi-character literal under '>' compares for equality."""
    from tqpk.operators import tqp_filter
    ins, outs, args = load("filter_substring")
    for i, tree in enumerate(args["trees"]):
        used = sorted({int(s.split("#")[1]) for s in _leaves(tree) if "#" in s})
        tg = {c: V(ins[c], args["types"][str(c)]) for c in used}
        tqp_filter(True, tg, {"filter tree": [tree], "materialized in": used, "out mask id": 999},
                   None, None, None, "f")
        np.testing.assert_array_equal(np_(tg[999].tensor), outs[f"mask{i}"], err_msg=str(tree))


@pytest.mark.parametrize("n", [1, 4097, 500_001])
def test_string_predicates_in_group_by_and_join_build(n):
    """String filters fused into the group-by (library evaluator) and the join build side."""
    from tqpk.expr import compile_aggregate
    from tqpk.ops import groupby
    from tqpk.pipeline import JoinAggTopK
    from tqpk.predicate import compile_filter
    ins, _, args = load("filter_strings")
    rng = np.random.default_rng(n)
    pick = rng.integers(0, ins[1].shape[0], n)
    words = ins[1][pick]
    key = rng.integers(0, 7, n).astype(np.int32)
    val = rng.integers(100, 100000, n) / 100.0
    d = {1: torch.from_numpy(words).cuda(), 2: torch.from_numpy(key).cuda(), 3: torch.from_numpy(val).cuda()}
    tree = [["Contains", ["t#1", "BRASS"]], "OR", ["t#1", "LIKE", "%SMALL%TIN%"]]
    aargs = {"is partial": False, "keys": ["k#2"], "input ids": [2, 3],
             "results": ["k#2", [[["sum", ["v#3"]], "#", "1"], "AS", "s#501"], [[["count", ["v#3"]], "#", "2L"], "AS", "c#502"]],
             "out agg ids": [501, 502]}
    prog = compile_aggregate(aargs, {2: d[2], 3: d[3]})
    keys, outs, G, _ = groupby(prog, n, d[2].device, pred=compile_filter(tree, {1: d[1]}))
    oc = {1: words, 2: key, 3: val}
    oc[99] = O.eval_filter(tree, {1: words})
    ref = O.tqp_hash_aggregate(oc, dict(aargs, **{"mask map": {2: 99, 3: 99}}))
    np.testing.assert_array_equal(np_(keys[0]), ref[2].reshape(-1))
    assert_f64_close(np_(outs[501]), ref[501])
    np.testing.assert_array_equal(np_(outs[502]), ref[502])
    # the same filter on the build side of the fused join
    bkey = torch.arange(1, n + 1, dtype=torch.int32, device="cuda")
    fk = torch.from_numpy(rng.integers(1, n + 1, 3 * n).astype(np.int32)).cuda()
    pv = torch.from_numpy(rng.integers(100, 100000, 3 * n) / 100.0).cuda()
    p = JoinAggTopK(bkey, 1, n, fk, {1: d[1]}, tree, {23: pv}, None, ["p#23"], k=5)
    p.run()
    got_keys, got_vals, groups = p.result()
    ok = O.eval_filter(tree, {1: words})
    fkn = np_(fk)
    sums = np.bincount(fkn - 1, weights=np_(pv) * ok[fkn - 1], minlength=n)
    present = np.bincount(fkn - 1, weights=ok[fkn - 1].astype(np.float64), minlength=n) > 0
    assert groups == int(present.sum())
    order = O._stable_order(np.where(present, sums, -np.inf), True)[:min(5, int(present.sum()))]
    np.testing.assert_array_equal(got_keys, order + 1)


def _leaves(t):
    if isinstance(t, str):
        yield t
    else:
        for e in t:
            yield from _leaves(e)


@pytest.mark.parametrize("n,offset", [(1, 0), (3, 0), (4097, 0), (1_000_003, 0), (100_003, 1), (100_003, 3)])
def test_filter_matches_oracle_sizes_and_alignment(n, offset):
    from tqpk.operators import tqp_filter
    _, _, args = load("filter_predicates")
    rng = np.random.default_rng(n + offset)
    base = {1: rng.integers(0, 2557, n + offset).astype(np.int32),
            2: (rng.integers(0, 11, n + offset) / 100.0),
            3: rng.integers(-50, 50, n + offset).astype(np.int64),
            4: rng.integers(65, 70, n + offset).astype(np.uint8),
            5: rng.normal(0, 1000, n + offset)}
    dev = {c: torch.from_numpy(a).cuda()[offset:] for c, a in base.items()}   # unaligned views when offset > 0
    host = {c: a[offset:] for c, a in base.items()}
    for tree in args["trees"]:
        used = sorted({int(s.split("#")[1]) for s in _leaves(tree) if "#" in s})
        from tqpk.variable import Variable
        tg = {c: Variable(dev[c], args["types"][str(c)]) for c in used}
        tqp_filter(True, tg, {"filter tree": [tree], "materialized in": used, "out mask id": 999}, None, None, None, "f")
        np.testing.assert_array_equal(np_(tg[999].tensor), O.eval_filter([tree], host), err_msg=str(tree))


@pytest.mark.parametrize("n", [0, 1, 5, 4096, 4097, 333_333])
@pytest.mark.parametrize("density", [0.0, 0.03, 0.5, 1.0])
def test_compact_stable(n, density):
    from tqpk.ops import compact
    rng = np.random.default_rng(n)
    m = rng.random(n) < density
    a = rng.integers(-2**40, 2**40, n)
    b = rng.integers(0, 255, n).astype(np.uint8)
    c = rng.random(n)
    d = rng.integers(0, 1 << 30, n).astype(np.int32)
    cols = [torch.from_numpy(x).cuda() for x in (a, b, c, d)]
    out, cnt = compact(cols, mask=torch.from_numpy(m).cuda(), with_row_ids=True)
    assert cnt == int(m.sum())
    for got, exp in zip(out, (a[m], b[m], c[m], d[m], np.nonzero(m)[0])):
        np.testing.assert_array_equal(np_(got), exp)


# ------------------------------------------------------------------ filter + aggregate + sort (lineitem)
def test_filter_agg_sort_lineitem_golden():
    from tqpk.operators import tqp_filter, tqp_hash_aggregate, tqp_sort
    ins, outs, args = load("filter_agg_sort_lineitem")
    tg = tg_from(ins, args["types"])
    tqp_filter(True, tg, copy.deepcopy(args["filter"]), None, None, None, "f")
    np.testing.assert_array_equal(np_(tg[900].tensor), outs["mask"])
    aargs = copy.deepcopy(args["aggregate"])
    aargs["mask map"] = {int(k): v for k, v in aargs["mask map"].items()}
    tqp_hash_aggregate(True, tg, aargs, None, None, "a")
    tqp_sort(True, tg, copy.deepcopy(args["sort"]), False, "s")
    for cid in args["sort"]["input ids"]:
        g, o = outs[str(cid)], np_(tg[cid].tensor)
        assert g.dtype == o.dtype and g.shape == o.shape, (cid, g.dtype, o.dtype, g.shape, o.shape)
        if g.dtype == np.float64:
            assert_f64_close(o, g)
        else:
            np.testing.assert_array_equal(o, g)


def test_lineitem_scaled_vs_oracle_and_fsum():
    from tqpk import datagen
    from tqpk.operators import tqp_filter, tqp_hash_aggregate
    _, _, args = load("filter_agg_sort_lineitem")
    t = datagen.lineitem(2_000_003, seed=3)
    ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
    cols = {ids[k]: v for k, v in t.items()}
    tg = {c: V(a, args["types"][str(c)]) for c, a in cols.items()}
    tqp_filter(True, tg, copy.deepcopy(args["filter"]), None, None, None, "f")
    aargs = copy.deepcopy(args["aggregate"])
    aargs["mask map"] = {int(k): v for k, v in aargs["mask map"].items()}
    tqp_hash_aggregate(True, tg, aargs, None, None, "a")
    mask = cols[7] <= datagen.SHIP_DATE_MAX
    ocols = dict(cols)
    ocols[900] = mask
    ref = O.tqp_hash_aggregate(ocols, copy.deepcopy(aargs))
    np.testing.assert_array_equal(np_(tg[5].tensor), ref[5])
    np.testing.assert_array_equal(np_(tg[6].tensor), ref[6])
    for a in aargs["out agg ids"]:
        if ref[a].dtype == np.float64:
            assert_f64_close(np_(tg[a].tensor), ref[a])
        else:
            np.testing.assert_array_equal(np_(tg[a].tensor), ref[a])
    # accuracy against the correctly rounded sum
    flag, status = cols[5][mask], cols[6][mask]
    _, inv = O.group_rows([flag, status])
    G = int(inv.max()) + 1
    truth = O.fsum_groups(cols[2][mask] * (1.0 - cols[3][mask]), inv, G)
    assert_f64_close(np_(tg[203].tensor), truth)


# ------------------------------------------------------------------ joins
@pytest.mark.parametrize("name", ["join_agg_topk_unique", "join_duplicates", "join_semi", "join_anti", "join_outer"])
def test_join_golden(name):
    from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
    ins, outs, args = load(name)
    tg = tg_from(ins, args["types"])
    for fa in args["filters"]:
        tqp_filter(True, tg, copy.deepcopy(fa), None, None, None, "f")
    np.testing.assert_array_equal(np_(tg[901].tensor), outs["mask901"])
    jargs = copy.deepcopy(args["join"])
    jargs["mask map"] = {int(k): v for k, v in jargs["mask map"].items()}
    rows = join_vortex(True, tg, jargs, 11, 21, [], args["type"], None, None, "j")
    assert rows == int(outs["rows"].reshape(-1)[0])
    ids = (11, 21, 23, 24) if outs["11"].size else (21, 23, 24)
    if not outs["11"].size:
        assert tg[11].tensor.numel() == 0
    np.testing.assert_array_equal(rows_sorted(*[np_(tg[c].tensor) for c in ids]),
                                  rows_sorted(*[outs[str(c)] for c in ids]))
    if "aggregate" in args:
        if name == "join_agg_topk_unique":   # unique build keys: the reference's exact row order
            for c in ids:
                np.testing.assert_array_equal(np_(tg[c].tensor), outs[str(c)])
        tqp_hash_aggregate(True, tg, copy.deepcopy(args["aggregate"]), None, None, "a")
        order = np.argsort(outs["agg_key"].reshape(-1), kind="stable")
        np.testing.assert_array_equal(np_(tg[11].tensor), outs["agg_key"][order])
        assert_f64_close(np_(tg[302].tensor), outs["agg_revenue"][order])
        tqp_sort(True, tg, copy.deepcopy(args["topk"]), True, "t")
        np.testing.assert_array_equal(np_(tg[11].tensor), outs["top_key"])
        assert_f64_close(np_(tg[302].tensor), outs["top_revenue"])


def test_join_kernel_direct_golden():
    from tqpk.operators import join_kernel_new
    from tqpk.variable import Variable
    ins, outs, args = load("join_kernel_direct")
    for name in args["specs"]:
        lk, rk = ins[f"{name}_left"], ins[f"{name}_right"]
        Lt = {1: V(lk), 2: Variable(torch.arange(lk.size, device="cuda"), "int")}
        Rt = {3: V(rk), 4: Variable(torch.arange(rk.size, device="cuda"), "int")}
        li, ri = join_kernel_new(True, Lt, Rt, 1, 3, [], [2, 4], False, "inner", None, None)
        np.testing.assert_array_equal(rows_sorted(np_(li), np_(ri)),
                                      rows_sorted(outs[f"{name}_lidx"], outs[f"{name}_ridx"]))
        np.testing.assert_array_equal(np_(ri), outs[f"{name}_ridx"])


@pytest.mark.parametrize("nb,np_rows,dups,sparse", [(200_000, 800_000, False, False), (50_000, 300_000, True, False),
                                                    (40_000, 100_000, False, True), (30_000, 90_000, True, True),
                                                    (1, 10, False, False), (0, 100, False, False)])
def test_join_scaled_vs_oracle(nb, np_rows, dups, sparse):
    from tqpk.ops import join_build, join_probe
    rng = np.random.default_rng(nb + np_rows)
    if dups:
        bk = rng.integers(1, max(2, nb // 3), nb)
    else:
        bk = rng.permutation(nb) + 1
    if sparse:
        bk = bk * 1_000_003 + 17
    pk = bk[rng.integers(0, max(nb, 1), np_rows)] if nb else rng.integers(0, 5, np_rows)
    pk = np.where(rng.random(np_rows) < 0.3, pk + 1, pk)
    bm = rng.random(nb) < 0.6
    pm = rng.random(np_rows) < 0.7
    for dt in (np.int32, np.int64) if not sparse else (np.int64,):
        b = join_build(torch.from_numpy(bk.astype(dt)).cuda(), torch.from_numpy(bm).cuda())
        for jt in ("inner", "right-semi", "right-anti", "right-outer"):
            bi, pi = join_probe(b, torch.from_numpy(pk.astype(dt)).cuda(), torch.from_numpy(pm).cuda(), jt)
            bsel, psel = np.nonzero(bm)[0], np.nonzero(pm)[0]
            li, ri = O.join_indices(bk[bm], pk[pm], jt)
            exp_b = np.where(li == O.NULL, O.NULL, bsel[np.where(li == O.NULL, 0, li)]) if li.size else li
            exp_p = psel[ri]
            if jt in ("right-semi", "right-anti"):
                np.testing.assert_array_equal(np_(pi), exp_p)
            else:
                if jt == "right-outer" and li.size == 0:
                    exp_b = np.full(exp_p.size, O.NULL)
                np.testing.assert_array_equal(np_(pi), exp_p)            # probe order is the reference's
                np.testing.assert_array_equal(np_(bi), exp_b)            # stable bucket order


# ------------------------------------------------------------------ aggregates
def test_aggregate_ops_golden():
    from tqpk.operators import tqp_hash_aggregate
    ins, outs, args = load("aggregate_ops")
    tg = tg_from(ins, args["types"])
    tqp_hash_aggregate(True, tg, copy.deepcopy(args["aggregate"]), None, None, "a")
    ids = args["aggregate"]["out agg ids"]
    order = np.lexsort([outs["2"].reshape(-1), outs["1"].reshape(-1)])
    np.testing.assert_array_equal(np_(tg[1].tensor), outs["1"][order])
    np.testing.assert_array_equal(np_(tg[2].tensor), outs["2"][order])
    for i in ids:
        g = outs[str(i)][order]
        o = np_(tg[i].tensor)
        assert o.dtype == g.dtype, (i, o.dtype, g.dtype)
        assert_f64_close(o, g) if g.dtype == np.float64 else np.testing.assert_array_equal(o, g)
    tg2 = tg_from({3: ins[3], 4: ins[4]}, args["types"])
    tqp_hash_aggregate(True, tg2, copy.deepcopy(args["global"]), None, None, "g")
    for i in args["global"]["out agg ids"]:
        g, o = outs[str(i)], np_(tg2[i].tensor)
        assert o.dtype == g.dtype and o.shape == g.shape
        assert_f64_close(o, g) if g.dtype == np.float64 else np.testing.assert_array_equal(o, g)


def test_aggregate_expressions_golden():
    """tqp_project (year, CASE over a string condition, a comparison as a value) then
    tqp_hash_aggregate with CASE conditions, year() and arithmetic over aggregates."""
    from tqpk.operators import tqp_hash_aggregate, tqp_project
    ins, outs, args = load("aggregate_expressions")
    tg = tg_from(ins, args["types"])
    tqp_project(True, tg, copy.deepcopy(args["project"]), None, None, "p")
    for c in args["project"]["materialized out"]:
        o, g = np_(tg[c].tensor), outs[f"p{c}"]
        assert o.dtype == g.dtype, (c, o.dtype, g.dtype)
        np.testing.assert_array_equal(o, g)
    tqp_hash_aggregate(True, tg, copy.deepcopy(args["aggregate"]), None, None, "a")
    order = np.lexsort([outs["20"].reshape(-1), outs["10"].reshape(-1)])
    np.testing.assert_array_equal(np_(tg[10].tensor), outs["10"][order])
    np.testing.assert_array_equal(np_(tg[20].tensor), outs["20"][order])
    for i in args["aggregate"]["out agg ids"]:
        g, o = outs[str(i)][order], np_(tg[i].tensor)
        assert o.dtype == g.dtype, (i, o.dtype, g.dtype)
        assert_f64_close(o, g) if g.dtype == np.float64 else np.testing.assert_array_equal(o, g)


def test_case_conditions_vs_oracle_at_size():
    """CASE WHEN at 3M rows (generated accumulation kernel, shared-table mode) against the oracle."""
    from tqpk.operators import tqp_hash_aggregate
    rng = np.random.default_rng(31)
    n = 3_000_000
    cols = {1: rng.integers(1, 51, n).astype(np.float64), 2: rng.integers(90000, 10495001, n) / 100.0,
            3: rng.integers(0, 11, n) / 100.0, 4: rng.integers(0, 3652, n).astype(np.int32),
            5: rng.integers(0, 700, n).astype(np.int32)}
    res = ["k#5",
           [[["sum", ["CASE", "WHEN", [["q#1", "<", "24"], "AND", ["d#3", ">=", "0.05"]], "THEN",
                      [["p#2", "*", ["1.0", "-", "d#3"]]], "ELSE", "0.0", "END"]], "#", "1"], "AS", "a#11"],
           [[["sum", ["CASE", "WHEN", ["NOT", ["q#1", "=", "1"]], "THEN", "1", "ELSE", "0", "END"]], "#", "2L"], "AS",
            "b#12L"],
           [[[["sum", ["CASE", "WHEN", ["y#4", ">", "1000"], "THEN", "p#2", "ELSE", "0.0", "END"]], "#", "3"], "/",
             [["sum", "p#2"], "#", "4"]], "AS", "c#13"],
           [[["max", [["year", ["y#4"]]]], "#", "5"], "AS", "d#14"]]
    args = {"is partial": False, "keys": ["k#5"], "input ids": [1, 2, 3, 4, 5], "results": res,
            "out agg ids": [11, 12, 13, 14]}
    tg = {1: V(cols[1], "float"), 2: V(cols[2], "float"), 3: V(cols[3], "float"), 4: V(cols[4], "date"), 5: V(cols[5])}
    tqp_hash_aggregate(True, tg, copy.deepcopy(args), None, None, "a")
    ref = O.tqp_hash_aggregate(cols, copy.deepcopy(args))
    np.testing.assert_array_equal(np_(tg[5].tensor), ref[5])
    for i in (11, 13):
        assert_f64_close(np_(tg[i].tensor), ref[i])
    for i in (12, 14):
        np.testing.assert_array_equal(np_(tg[i].tensor), ref[i])


def test_aggregate_string_keys_golden():
    """String (2-D) keys, five mixed keys (int, string, float, uint8), a float key with -0.0
    and +0.0 rows, under a late-materialisation mask: numbered by the key-encoding pass,
    grouped by code, key outputs gathered as [G, w] / [G, 1]."""
    from golden_io import key_tuple_order
    from tqpk.operators import tqp_filter, tqp_hash_aggregate
    ins, outs, args = load("aggregate_string_keys")
    for name, a in args["sets"].items():
        tg = tg_from(ins, args["types"])
        tqp_filter(True, tg, copy.deepcopy(args["filter"]), None, None, None, "f")
        a = copy.deepcopy(a)
        a["mask map"] = {int(k): v for k, v in a["mask map"].items()}
        tqp_hash_aggregate(True, tg, a, None, None, "a")
        kids = [O.get_id(k) for k in a["keys"]]
        order = key_tuple_order([outs[f"{name}_{k}"] for k in kids])
        for k in kids:
            g, o = outs[f"{name}_{k}"][order], np_(tg[k].tensor)
            assert o.dtype == g.dtype and o.shape == g.shape, (name, k, o.dtype, o.shape, g.shape)
            np.testing.assert_array_equal(o, g)
        for i in a["out agg ids"]:
            g, o = outs[f"{name}_{i}"][order], np_(tg[i].tensor)
            assert o.dtype == g.dtype, (name, i)
            assert_f64_close(o, g) if g.dtype == np.float64 else np.testing.assert_array_equal(o, g)


@pytest.mark.parametrize("n", [1, 1000, 2_000_003])
def test_key_encode_vs_oracle_at_size(n):
    """Key encoding at size: a 10-byte string key and an int key, ~n/3 groups at the top size."""
    from tqpk.ops import encode_keys
    rng = np.random.default_rng(n)
    s = rng.integers(65, 70, (n, 10)).astype(np.int8)
    s[:, 6:] = 0
    k = rng.integers(0, max(1, n // 1000), n).astype(np.int32)
    codes, reps, G = encode_keys([torch.from_numpy(s).cuda(), torch.from_numpy(k).cuda()])
    ukeys, inverse = O.group_rows([s, k])
    assert G == ukeys[0].shape[0]
    np.testing.assert_array_equal(np_(codes), inverse)
    r = np_(reps)
    np.testing.assert_array_equal(s[r], ukeys[0])
    np.testing.assert_array_equal(k[r], ukeys[1].reshape(-1))


def test_join_gathers_string_payloads():
    """join_vortex materialises a 2-D string column of each side (row gather)."""
    from tqpk.operators import join_vortex
    from tqpk.variable import Variable
    rng = np.random.default_rng(3)
    nb, npr = 5000, 40_000
    bk = rng.permutation(nb).astype(np.int64)
    bs = rng.integers(65, 91, (nb, 25)).astype(np.int8)
    pk = rng.integers(0, nb + 500, npr).astype(np.int64)
    ps = rng.integers(65, 91, (npr, 15)).astype(np.int8)
    tg = {1: V(bk), 2: Variable(torch.from_numpy(bs).cuda(), "string"), 3: V(pk),
          4: Variable(torch.from_numpy(ps).cuda(), "string")}
    join_vortex(True, tg, {"left group": [1, 2], "right group": [3, 4], "materialized in": [1, 2, 3, 4]},
                1, 3, [], "inner", None, None, "j")
    bi, pi = O.join_indices(bk, pk, "inner")
    np.testing.assert_array_equal(np_(tg[2].tensor), bs[bi])
    np.testing.assert_array_equal(np_(tg[4].tensor), ps[pi])


@pytest.mark.parametrize("desc,limit", [(False, None), (True, None), (True, 7), (False, 100)])
def test_sort_string_keys_vs_oracle(desc, limit):
    """tqp_sort on a 19-byte string key (three word passes) then an int key, with and
    without a limit; string payloads gathered row by row."""
    from tqpk.operators import tqp_sort
    from tqpk.variable import Variable
    rng = np.random.default_rng(17)
    n = 50_003
    sk = rng.integers(60, 68, (n, 19)).astype(np.int8)
    sk[:, 3:] = 0
    sk[rng.integers(0, n, 300), 10] = -5          # a negative byte deep in the row
    ik = rng.integers(0, 50, n).astype(np.int32)
    pay = rng.integers(65, 91, (n, 11)).astype(np.int8)
    tg = {1: Variable(torch.from_numpy(sk).cuda(), "string"), 2: V(ik),
          3: Variable(torch.from_numpy(pay).cuda(), "string")}
    args = {"input ids": [1, 2, 3], "key ids": [1, 2], "key orders": [desc, False]}
    if limit is not None:
        args["limit"] = limit
    tqp_sort(True, tg, copy.deepcopy(args), limit is not None, "s")
    ref = O.tqp_sort({1: sk, 2: ik, 3: pay}, args, limit is not None)
    for c in (1, 2, 3):
        np.testing.assert_array_equal(np_(tg[c].tensor), ref[c], err_msg=str(c))


def test_aggregate_two_step_golden():
    from tqpk.operators import tqp_hash_aggregate
    ins, outs, args = load("aggregate_two_step")
    tg = tg_from(ins, args["types"])
    tqp_hash_aggregate(True, tg, copy.deepcopy(args["aggregate"]), None, None, "a")
    order = np.argsort(outs["1"].reshape(-1), kind="stable")
    np.testing.assert_array_equal(np_(tg[1].tensor), outs["1"][order])
    for i in args["aggregate"]["out agg ids"]:
        g, o = outs[str(i)][order], np_(tg[i].tensor)
        assert o.dtype == g.dtype
        assert_f64_close(o, g) if g.dtype == np.float64 else np.testing.assert_array_equal(o, g)


@pytest.mark.parametrize("tag", ["one", "two"])
def test_aggregate_float32_golden(tag):
    """torch's float32 results (an integer column with a Python float, integer true division,
    CASE mixing a float literal with integers) against the reference's own outputs: dtypes and
    column types as the reference gives them (float32, typed "string" by its torch_to_type; the
    2-step path's avg float64), min / max / count exact; sums are accumulated in float64 here and
    rounded once, the reference adds in float32 row by row, so they agree within that rounding
    (2e-4 relative for 7,500-70,000 rows per group)."""
    from tqpk.operators import tqp_hash_aggregate
    ins, outs, args = load("aggregate_float32")
    a = args[tag]
    cols = {int(k.split("_")[1]): v for k, v in ins.items() if isinstance(k, str) and k.startswith(tag + "_")}
    tg = {c: V(v, a["types"][str(c)]) for c, v in cols.items()}
    tqp_hash_aggregate(True, tg, copy.deepcopy(a["aggregate"]), None, None, "a")
    g1 = outs[f"{tag}_1"].reshape(-1)
    order = np.argsort(g1, kind="stable")
    np.testing.assert_array_equal(np_(tg[1].tensor).reshape(-1), g1[order])
    for i in a["aggregate"]["out agg ids"]:
        g, o = outs[f"{tag}_{i}"][order], np_(tg[i].tensor)
        assert o.dtype == g.dtype, (i, o.dtype, g.dtype)
        assert tg[i].tensor_type == str(outs[f"{tag}_{i}_type"].reshape(-1)[0]), i
        if i in (904, 905, 907):                            # min, max, count: exact
            np.testing.assert_array_equal(o, g)
        elif g.dtype == np.float32 or i == 902:
            np.testing.assert_allclose(o, g, rtol=2e-4, atol=0)
        else:
            assert_f64_close(o, g)


def test_project_float32_golden():
    """Float32 projections (an integer column times a Python float, integer true division) are the
    reference's values bit for bit, typed as it types them."""
    from tqpk.operators import tqp_project
    ins, outs, args = load("aggregate_float32")
    a = args["one"]
    cols = {int(k.split("_")[1]): v for k, v in ins.items() if isinstance(k, str) and k.startswith("one_")}
    tg = {c: V(v, a["types"][str(c)]) for c, v in cols.items()}
    tqp_project(True, tg, copy.deepcopy(args["project"]), None, None, "p")
    for c in args["project"]["materialized out"]:
        g, o = outs[f"proj_{c}"], np_(tg[c].tensor)
        assert o.dtype == g.dtype, (c, o.dtype, g.dtype)
        assert tg[c].tensor_type == str(outs[f"proj_{c}_type"].reshape(-1)[0]), c
        np.testing.assert_array_equal(o, g)


def test_aggregate_substring_golden():
    """sum / count of a one-byte substring of a string column (the reference squeezes the [N, 1]
    slice), and the slice times 2, which wraps in int8 as torch's int8 arithmetic does."""
    from tqpk.operators import tqp_hash_aggregate
    ins, outs, args = load("aggregate_substring")
    tg = tg_from(ins, args["types"])
    tqp_hash_aggregate(True, tg, copy.deepcopy(args["aggregate"]), None, None, "a")
    order = np.argsort(outs["1"].reshape(-1), kind="stable")
    np.testing.assert_array_equal(np_(tg[1].tensor), outs["1"][order])
    for i in args["aggregate"]["out agg ids"]:
        g, o = outs[str(i)][order], np_(tg[i].tensor)
        assert o.dtype == g.dtype
        np.testing.assert_array_equal(o, g)


def test_aggregate_high_cardinality_vs_oracle():
    from tqpk.operators import tqp_hash_aggregate
    rng = np.random.default_rng(9)
    n = 1_500_000
    cols = {1: rng.integers(1, 600_000, n).astype(np.int32), 2: rng.integers(90000, 10495001, n) / 100.0,
            3: rng.integers(0, 11, n) / 100.0}
    args = {"is partial": False, "keys": ["k#1"], "input ids": [1, 2, 3],
            "results": ["k#1", [[["sum", [["p#2", "*", ["1.0", "-", "d#3"]]]], "#", "9"], "AS", "r#10"],
                        [[["count", ["1"]], "#", "8L"], "AS", "c#11"], [[["max", ["p#2"]], "#", "7"], "AS", "m#12"]],
            "out agg ids": [10, 11, 12]}
    tg = {1: V(cols[1]), 2: V(cols[2], "float"), 3: V(cols[3], "float")}
    tqp_hash_aggregate(True, tg, copy.deepcopy(args), None, None, "a")
    ref = O.tqp_hash_aggregate(cols, copy.deepcopy(args))
    np.testing.assert_array_equal(np_(tg[1].tensor), ref[1])
    assert_f64_close(np_(tg[10].tensor), ref[10])
    np.testing.assert_array_equal(np_(tg[11].tensor), ref[11])
    np.testing.assert_array_equal(np_(tg[12].tensor), ref[12])


def test_aggregate_empty_and_all_filtered():
    from tqpk.operators import tqp_filter, tqp_hash_aggregate
    n = 1000
    cols = {1: np.zeros(n, np.int32), 2: np.ones(n), 7: np.arange(n, dtype=np.int32)}
    tg = {1: V(cols[1]), 2: V(cols[2], "float"), 7: V(cols[7], "date")}
    tqp_filter(True, tg, {"filter tree": [["d#7", "<", "0"]], "materialized in": [7], "out mask id": 99},
               None, None, None, "f")
    args = {"is partial": False, "keys": ["k#1"], "input ids": [1, 2],
            "results": ["k#1", [[["sum", ["p#2"]], "#", "9"], "AS", "r#10"]], "out agg ids": [10],
            "mask map": {1: 99, 2: 99}}
    tqp_hash_aggregate(True, tg, args, None, None, "a")
    assert tg[10].tensor.numel() == 0 and tuple(tg[1].tensor.shape) == (0, 1)


# ------------------------------------------------------------------ sort / top-k
def test_sort_multikey_golden():
    from tqpk.operators import tqp_sort
    ins, outs, args = load("sort_multikey")
    for i, (spec, lim) in enumerate(args["specs"]):
        used = sorted(set(spec["input ids"]) | set(spec["key ids"]))
        tg = {c: V(ins[c], args["types"][str(c)]) for c in used}
        tqp_sort(True, tg, copy.deepcopy(spec), lim, "s")
        for c in spec["input ids"]:
            np.testing.assert_array_equal(np_(tg[c].tensor), outs[f"s{i}_{c}"], err_msg=f"spec {i} col {c}")


@pytest.mark.parametrize("n", [1, 6, 1000, 2048, 2049])
@pytest.mark.parametrize("desc", [False, True])
def test_argsort_small_single_cta_path(n, desc):
    """n <= 2048 sorts in one CTA (bitonic on key, position); 2049 takes the radix path."""
    from tqpk.ops import argsort_stable
    rng = np.random.default_rng(n)
    for dtype in (np.int32, np.float64, np.uint8):
        k = (rng.integers(-5, 5, n) * 0.5).astype(dtype) if dtype == np.float64 else rng.integers(0, 7, n).astype(dtype)
        if dtype == np.float64 and n > 3:
            k[:3] = [-0.0, 0.0, np.nan]
        perm_in = rng.permutation(n)
        got = np_(argsort_stable(torch.from_numpy(k).cuda(), desc, torch.from_numpy(perm_in).cuda()))
        np.testing.assert_array_equal(got, perm_in[O._stable_order(k[perm_in], desc)])
        got = np_(argsort_stable(torch.from_numpy(k).cuda(), desc))
        np.testing.assert_array_equal(got, O._stable_order(k, desc))


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.float64, np.uint8, np.int8])
@pytest.mark.parametrize("desc", [False, True])
def test_argsort_stable_vs_numpy(dtype, desc):
    from tqpk.ops import argsort_stable, topk_stable
    rng = np.random.default_rng(3)
    n = 1_000_003
    if dtype == np.float64:
        k = rng.integers(-500, 500, n) * 0.25
        k[:4] = [-0.0, 0.0, np.inf, -np.inf]
    elif dtype in (np.uint8, np.int8):
        k = rng.integers(np.iinfo(dtype).min, np.iinfo(dtype).max, n).astype(dtype)
    else:
        k = rng.integers(np.iinfo(dtype).min // 2, np.iinfo(dtype).max // 2, n).astype(dtype)
        k[rng.integers(0, n, n // 2)] = 7     # heavy ties
    k = k.astype(dtype)
    perm_in = rng.permutation(n)
    got = np_(argsort_stable(torch.from_numpy(k).cuda(), desc, torch.from_numpy(perm_in).cuda()))
    exp = perm_in[O._stable_order(k[perm_in], desc)]
    np.testing.assert_array_equal(got, exp)
    for kk in (1, 10, 100, 5000):
        top = np_(topk_stable(torch.from_numpy(k).cuda(), kk, desc, torch.from_numpy(perm_in).cuda()))
        np.testing.assert_array_equal(top, exp[:kk])


# ------------------------------------------------------------------ loud failures
def test_cpu_tensors_and_unsupported_shapes_raise():
    from tqpk.ops import argsort_stable
    from tqpk.operators import tqp_filter, tqp_hash_aggregate
    with pytest.raises(ValueError):
        argsort_stable(torch.zeros(10, dtype=torch.int32))
    tg = {1: V(np.zeros(10, np.int8).reshape(5, 2))}
    with pytest.raises(NotImplementedError):       # a numeric literal against a string slice
        tqp_filter(True, tg, {"filter tree": [[["substring", ["s#1", "1", "2"]], "=", "12"]], "materialized in": [1],
                              "out mask id": 2}, None, None, None, "f")
    with pytest.raises(NotImplementedError):
        tqp_filter(False, tg, {"filter tree": [["s#1", "=", "A"]], "materialized in": [1], "out mask id": 2},
                   None, None, None, "f")


@pytest.mark.parametrize("jtype", ["inner", "right-semi", "right-anti", "right-outer"])
def test_join_conditions_every_join_type(jtype):
    """Extra join conditions (a second key and a <> condition, hashjoin.py:100-108) with the
    semi / anti / outer forms derived from the pairs they keep (hashjoin.py:110-151)."""
    from tqpk.operators import join_vortex
    from tqpk.variable import Variable
    rng = np.random.default_rng(hash(jtype) % 1000)
    nb, npr = 20_000, 90_001
    cols = {11: rng.integers(0, 4000, nb).astype(np.int64), 12: rng.integers(0, 5, nb).astype(np.int32),
            13: rng.integers(0, 100, nb).astype(np.int64),
            21: rng.integers(0, 4500, npr).astype(np.int64), 22: rng.integers(0, 5, npr).astype(np.int32),
            23: rng.integers(0, 100, npr).astype(np.int64), 24: rng.integers(0, 2557, npr).astype(np.int32)}
    cols[902] = cols[24] > 1000
    conds = [["#12", "=", "#22"], ["s#13", "<", "t#23"]]
    args = {"left group": [11, 12, 13], "right group": [21, 22, 23, 24], "materialized in": [11, 12, 13, 21, 22, 23],
            "mask map": {21: 902, 22: 902, 23: 902}}
    tg = {c: Variable(torch.from_numpy(a).cuda(), "int") for c, a in cols.items() if c != 902}
    tg[902] = Variable(torch.from_numpy(cols[902]).cuda(), "bool")
    rows = join_vortex(True, tg, copy.deepcopy(args), 11, 21, copy.deepcopy(conds), jtype, None, None, "j")
    ref, ref_rows = O.join_vortex(cols, copy.deepcopy(args), 11, 21, jtype, conds)
    assert rows == ref_rows
    for c in (11, 12, 13, 21, 22, 23):
        got = np_(tg[c].tensor).reshape(-1)
        np.testing.assert_array_equal(got, np.asarray(ref[c]).reshape(-1), err_msg=str(c))


def test_operators_wait_for_columns_still_copying():
    """Columns copied from pinned host memory on a side stream, each Variable carrying the
    copy's event: every operator waits for a column right before its first kernel reads it,
    and the chained filter -> join -> aggregate -> top-10 matches the oracle."""
    from tqpk import datagen
    from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
    from tqpk.variable import Variable
    t = datagen.join_tables(300_000, 2_000_003, seed=5)
    cols = {11: t["b_key"], 12: t["b_date"], 21: t["p_fk"], 22: t["p_date"], 23: t["p_price"], 24: t["p_discount"]}
    types = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}
    host = {c: torch.from_numpy(a).pin_memory() for c, a in cols.items()}
    side = torch.cuda.Stream()
    main = torch.cuda.current_stream()
    dst = {c: torch.empty(h.shape, dtype=h.dtype, device="cuda") for c, h in host.items()}
    side.wait_stream(main)
    tg = {}
    with torch.cuda.stream(side):
        for c in (12, 22, 11, 21, 23, 24):
            dst[c].copy_(host[c], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(side)
            tg[c] = Variable(dst[c], types[c], ready=ev)
    f1 = {"filter tree": [["bd#12", "<", "1170"]], "materialized in": [12], "out mask id": 901}
    f2 = {"filter tree": [["pd#22", ">", "1170"]], "materialized in": [22], "out mask id": 902}
    jargs = {"left group": [11, 12], "right group": [21, 22, 23, 24], "materialized in": [11, 21, 23, 24],
             "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}
    aargs = {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
             "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "301"], "AS", "rev#302"]],
             "out agg ids": [302]}
    targs = {"limit": 10, "input ids": [11, 302], "key ids": [302], "key orders": [True]}
    tqp_filter(True, tg, copy.deepcopy(f1), None, None, None, "f1")
    tqp_filter(True, tg, copy.deepcopy(f2), None, None, None, "f2")
    join_vortex(True, tg, copy.deepcopy(jargs), 11, 21, [], "inner", None, None, "j")
    tqp_hash_aggregate(True, tg, copy.deepcopy(aargs), None, None, "a")
    tqp_sort(True, tg, copy.deepcopy(targs), True, "t")
    got_k, got_v = np_(tg[11].tensor).reshape(-1), np_(tg[302].tensor)
    oc = dict(cols)
    oc[901] = O.eval_filter(f1["filter tree"], {12: cols[12]})
    oc[902] = O.eval_filter(f2["filter tree"], {22: cols[22]})
    j = O.join_vortex(oc, copy.deepcopy(jargs), 11, 21, "inner")[0]
    agg = O.tqp_hash_aggregate(j, copy.deepcopy(aargs))
    top = O.tqp_sort(agg, targs, True)
    np.testing.assert_array_equal(got_k, top[11].reshape(-1))
    assert_f64_close(got_v, top[302])


def test_key_encode_edge_cases():
    """Every row masked out (no groups), one row, a float key with -0.0 / +0.0, and string keys
    with bytes >= 128 as uint8 (unsigned order) and as int8 (signed order)."""
    from tqpk.ops import encode_keys
    s = np.array([[1, 2], [3, 4], [1, 2]], np.int8)
    codes, reps, G = encode_keys([torch.from_numpy(s).cuda()], torch.zeros(3, dtype=torch.bool, device="cuda"))
    assert G == 0 and reps.numel() == 0
    codes, reps, G = encode_keys([torch.from_numpy(s[:1]).cuda()])
    assert G == 1 and np_(codes).tolist() == [0] and np_(reps).tolist() == [0]
    f = np.array([0.0, -0.0, 1.5, -2.0, 1.5, 0.0], np.float64)
    codes, reps, G = encode_keys([torch.from_numpy(f).cuda()])
    assert G == 3 and np_(codes).tolist() == [1, 1, 2, 0, 2, 1]
    u = np.array([[200, 1], [5, 1], [200, 0], [5, 1]], np.uint8)
    codes, reps, G = encode_keys([torch.from_numpy(u).cuda()])
    _, inv = O.group_rows([u])                       # uint8 bytes order unsigned, int8 bytes signed
    np.testing.assert_array_equal(np_(codes), inv)
    codes, reps, G = encode_keys([torch.from_numpy(u.view(np.int8)).cuda()])
    _, inv = O.group_rows([u.view(np.int8)])
    np.testing.assert_array_equal(np_(codes), inv)


def test_project_case_over_a_string_condition_and_year_edges():
    """tqp_project: CASE WHEN on a string equality, year() at the first and last day the
    reference's table covers, and a comparison as a bool output."""
    from tqpk.operators import tqp_project
    from tqpk.variable import Variable
    rng = np.random.default_rng(2)
    n = 10_001
    nat = np.zeros((n, 25), np.int8)
    names = ["BRAZIL", "PERU"]
    pick = rng.integers(0, 2, n)
    for i, nm in enumerate(names):
        nat[pick == i, :len(nm)] = np.frombuffer(nm.encode(), np.uint8).astype(np.int8)
    days = rng.integers(0, 3652, n).astype(np.int32)
    days[:4] = [0, 364, 365, 3651]
    price = rng.integers(100, 10000, n) / 100.0
    cols = {1: nat, 2: days, 3: price}
    args = {"rename map": {}, "materialized in": [1, 2, 3],
            "used expr": [[["CASE", "WHEN", ["n#1", "=", "BRAZIL"], "THEN", "p#3", "ELSE", "0.0", "END"], "AS", "v#10"],
                          [["year", ["d#2"]], "AS", "y#11"], [["p#3", ">=", "50.0"], "AS", "b#12"]],
            "materialized out": [10, 11, 12]}
    tg = {1: Variable(torch.from_numpy(nat).cuda(), "string"), 2: V(days, "date"), 3: V(price, "float")}
    tqp_project(True, tg, copy.deepcopy(args), None, None, "p")
    ref = O.tqp_project(cols, args)
    for c in (10, 11, 12):
        o = np_(tg[c].tensor)
        assert o.dtype == ref[c].dtype, c
        np.testing.assert_array_equal(o, ref[c])
    assert np_(tg[11].tensor)[:4].tolist() == [1990, 1990, 1991, 1999]


def test_scan_staged_and_synchronous_paths_feed_the_operators(tmp_path):
    """tqp_scan places the columns on the device synchronously (the reference's behaviour, in a
    pool with malloc_like) or queues them on a ColumnStager; a filter and an aggregate over the
    staged columns match the oracle."""
    import torch.nn as nn
    from tqpk.ingress import ColumnStager
    from tqpk.operators import tqp_filter, tqp_hash_aggregate, tqp_scan

    class Holder(nn.Module):
        def __init__(self, t):
            super().__init__()
            self.p = nn.Parameter(t, requires_grad=False)

        def forward(self):
            return self.p

    class Pool:
        def __init__(self):
            self.n = 0

        def malloc_like(self, t):
            self.n += 1
            return self.n, torch.empty_like(t)

    rng = np.random.default_rng(6)
    n = 2_000_003
    data = {"K": rng.integers(0, 7, n).astype(np.int32), "V": rng.integers(90000, 10495001, n) / 100.0,
            "D": rng.integers(0, 2557, n).astype(np.int32)}
    for name, a in data.items():
        torch.jit.script(Holder(torch.from_numpy(a))).save(str(tmp_path / f"SF1-tensor-{name}.pth"))
    schema = {"K": "integer", "V": "decimal", "D": "date"}
    args = {"output names": ["k", "v", "d"], "output ids": [1, 2, 3]}
    for stager, pool in ((None, Pool()), (ColumnStager(), None), (ColumnStager(), Pool())):
        tg = {}
        assert tqp_scan(True, tg, args, {"tensors path": str(tmp_path)}, schema, 1, pool, stager=stager) == n
        assert (getattr(tg[2], "ready", None) is not None) == (stager is not None)
        tqp_filter(True, tg, {"filter tree": [["d#3", "<=", "2000"]], "materialized in": [3], "out mask id": 900},
                   None, None, None, "f")
        aargs = {"is partial": False, "keys": ["k#1"], "input ids": [1, 2],
                 "results": ["k#1", [[["sum", ["v#2"]], "#", "1"], "AS", "s#10"]], "out agg ids": [10],
                 "mask map": {1: 900, 2: 900}}
        tqp_hash_aggregate(True, tg, copy.deepcopy(aargs), None, None, "a")
        oc = {1: data["K"].astype(np.int64), 2: data["V"], 900: data["D"] <= 2000}
        ref = O.tqp_hash_aggregate(oc, copy.deepcopy(aargs))
        np.testing.assert_array_equal(np_(tg[1].tensor), ref[1])
        assert_f64_close(np_(tg[10].tensor), ref[10])


@pytest.mark.parametrize("spread", [1, 1_000_003])
def test_join_key_range_feeds_the_groupby_plan(spread):
    """An inner join's key outputs carry the filtered build-key range; the group-by that
    follows plans from it (dense keys) or falls back to reading the keys (a range too
    sparse for a slot table), and both give the oracle's groups."""
    import copy
    from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate
    from tqpk.variable import Variable
    rng = np.random.default_rng(spread)
    nb, np_ = 20_000, 90_001
    bkey = (rng.permutation(nb).astype(np.int64) * spread + 5).astype(np.int64)
    cols = {11: bkey, 12: rng.integers(0, 2557, nb).astype(np.int32),
            21: bkey[rng.integers(0, nb, np_)], 22: rng.integers(0, 2557, np_).astype(np.int32),
            23: rng.integers(90000, 10495001, np_) / 100.0, 24: rng.integers(0, 11, np_) / 100.0}
    types = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}
    tg = {c: Variable(torch.from_numpy(a).cuda(), types[c]) for c, a in cols.items()}
    f1 = {"filter tree": [["bd#12", "<", "1170"]], "materialized in": [12], "out mask id": 901}
    f2 = {"filter tree": [["pd#22", ">", "1170"]], "materialized in": [22], "out mask id": 902}
    jargs = {"left group": [11, 12], "right group": [21, 22, 23, 24], "materialized in": [11, 21, 23, 24],
             "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}
    aargs = {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
             "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "301"], "AS", "rev#302"],
                         [[["count", ["1"]], "#", "303L"], "AS", "c#304"]],
             "out agg ids": [302, 304]}
    tqp_filter(True, tg, copy.deepcopy(f1), None, None, None, "f1")
    tqp_filter(True, tg, copy.deepcopy(f2), None, None, None, "f2")
    join_vortex(True, tg, copy.deepcopy(jargs), 11, 21, [], "inner", None, None, "j")
    kr = tg[11]._key_range
    passing = cols[11][cols[12] < 1170]
    assert kr == (int(passing.min()), int(passing.max()))
    tqp_hash_aggregate(True, tg, copy.deepcopy(aargs), None, None, "a")
    oc = dict(cols)
    oc[901] = O.eval_filter(f1["filter tree"], {12: cols[12]})
    oc[902] = O.eval_filter(f2["filter tree"], {22: cols[22]})
    res, _ = O.join_vortex(oc, copy.deepcopy(jargs), 11, 21, "inner")
    agg = O.tqp_hash_aggregate(res, copy.deepcopy(aargs))
    np.testing.assert_array_equal(tg[11].tensor.cpu().numpy().reshape(-1), agg[11].reshape(-1))
    np.testing.assert_array_equal(tg[304].tensor.cpu().numpy().reshape(-1), agg[304].reshape(-1))
    assert_f64_close(tg[302].tensor.cpu().numpy().reshape(-1), agg[302].reshape(-1))


@pytest.mark.parametrize("keys,orders,limit", [([5, 6], [False, False], None), ([5], [False], 3),
                                               ([6, 5], [False, False], None), ([5, 6], [True, False], None),
                                               ([5, 6], [False, False], 4)])
def test_sort_after_groupby_on_its_keys(keys, orders, limit):
    """A sort on an ascending prefix of the group keys returns the group-by's own order (the
    sort is elided); other key lists and orders sort; all match the oracle."""
    import copy
    from tqpk import datagen
    from tqpk.operators import tqp_hash_aggregate, tqp_sort
    from tqpk.variable import Variable
    t = datagen.lineitem(200_003, seed=12)
    ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
    cols = {ids[k]: v for k, v in t.items()}
    types = {1: "float", 2: "float", 3: "float", 4: "float", 5: "int", 6: "int", 7: "date"}
    tg = {c: Variable(torch.from_numpy(a).cuda(), types[c]) for c, a in cols.items()}
    aargs = {"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 5, 6],
             "results": ["flag#5", "status#6", [[["sum", ["quantity#1"]], "#", "101"], "AS", "a#201"],
                         [[["count", ["1"]], "#", "108L"], "AS", "h#208"]],
             "out agg ids": [201, 208]}
    sargs = {"input ids": [5, 6, 201, 208], "key ids": keys, "key orders": orders}
    if limit is not None:
        sargs["limit"] = limit
    tqp_hash_aggregate(True, tg, copy.deepcopy(aargs), None, None, "a")
    elided = orders == [False] * len(orders) and keys == [5, 6][:len(keys)]
    assert all(getattr(tg[c], "_row_order", None) is tg[5]._row_order for c in sargs["input ids"])
    tqp_sort(True, tg, copy.deepcopy(sargs), limit is not None, "s")
    agg = O.tqp_hash_aggregate(dict(cols), copy.deepcopy(aargs))
    ref = O.tqp_sort({c: agg[c] for c in sargs["input ids"]}, sargs, limit is not None)
    for c in sargs["input ids"]:
        got = tg[c].tensor.cpu().numpy()
        assert got.shape == np.asarray(ref[c]).shape, (c, got.shape, np.asarray(ref[c]).shape)
        if got.dtype == np.float64:
            assert_f64_close(got.reshape(-1), np.asarray(ref[c]).reshape(-1))
        else:
            np.testing.assert_array_equal(got, ref[c])
    # an elided sort without a limit leaves the group-by's columns in place (still tagged);
    # a sort that ran, or a limit, makes new columns
    assert (getattr(tg[201], "_row_order", None) is not None) == (elided and limit is None)


@pytest.mark.parametrize("nb,np_", [(20_000, 400_003), (3_000, 2_000_001)])
def test_staged_join_aggregate_topk_counts_groups_before_the_values(nb, np_):
    """Columns copied from pinned host memory on a side stream, value columns last: the join
    gathers them late, the aggregate counts its groups from the keys while they are still in
    flight, and the result equals the oracle's."""
    import copy
    from tqpk import datagen
    from tqpk.ingress import ColumnStager
    from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
    t = datagen.join_tables(nb, np_, seed=nb)
    cols = {11: t["b_key"], 12: t["b_date"], 21: t["p_fk"], 22: t["p_date"], 23: t["p_price"], 24: t["p_discount"]}
    types = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}
    host = {c: torch.from_numpy(a).pin_memory() for c, a in cols.items()}
    f1 = {"filter tree": [["bd#12", "<", "1170"]], "materialized in": [12], "out mask id": 901}
    f2 = {"filter tree": [["pd#22", ">", "1170"]], "materialized in": [22], "out mask id": 902}
    jargs = {"left group": [11, 12], "right group": [21, 22, 23, 24], "materialized in": [11, 21, 23, 24],
             "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}
    aargs = {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
             "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "301"], "AS", "rev#302"]],
             "out agg ids": [302]}
    targs = {"limit": 10, "input ids": [11, 302], "key ids": [302], "key orders": [True]}
    stager = ColumnStager()
    for _ in range(2):
        tg = stager.stage(host, types, (12, 22, 11, 21, 23, 24))
        tqp_filter(True, tg, copy.deepcopy(f1), None, None, None, "f1")
        tqp_filter(True, tg, copy.deepcopy(f2), None, None, None, "f2")
        join_vortex(True, tg, copy.deepcopy(jargs), 11, 21, [], "inner", None, None, "j")
        tqp_hash_aggregate(True, tg, copy.deepcopy(aargs), None, None, "a")
        tqp_sort(True, tg, copy.deepcopy(targs), True, "t")
        got_k = tg[11].tensor.cpu().numpy().reshape(-1)
        got_v = tg[302].tensor.cpu().numpy().reshape(-1)
        oc = dict(cols)
        oc[901] = O.eval_filter(f1["filter tree"], {12: cols[12]})
        oc[902] = O.eval_filter(f2["filter tree"], {22: cols[22]})
        res, _ = O.join_vortex(oc, copy.deepcopy(jargs), 11, 21, "inner")
        agg = O.tqp_hash_aggregate(res, copy.deepcopy(aargs))
        top = O.tqp_sort({11: agg[11], 302: agg[302]}, targs, True)
        np.testing.assert_array_equal(got_k, top[11].reshape(-1))
        assert_f64_close(got_v, top[302].reshape(-1))


def test_sort_after_groupby_sorts_a_replaced_column():
    """A group-by output column whose tensor was replaced afterwards is no longer known to be in
    key order: the sort runs (and matches the oracle on the replaced data)."""
    import copy
    from tqpk import datagen
    from tqpk.operators import tqp_hash_aggregate, tqp_sort
    from tqpk.variable import Variable
    t = datagen.lineitem(50_001, seed=13)
    cols = {1: t["quantity"], 5: t["flag"], 6: t["status"]}
    types = {1: "float", 5: "int", 6: "int"}
    tg = {c: Variable(torch.from_numpy(a).cuda(), types[c]) for c, a in cols.items()}
    aargs = {"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 5, 6],
             "results": ["flag#5", "status#6", [[["sum", ["quantity#1"]], "#", "101"], "AS", "a#201"]],
             "out agg ids": [201]}
    tqp_hash_aggregate(True, tg, copy.deepcopy(aargs), None, None, "a")
    flipped = torch.flip(tg[5].tensor, dims=[0]).contiguous()
    tg[5].tensor = flipped                           # same Variable, other rows
    sargs = {"input ids": [5, 6, 201], "key ids": [5, 6], "key orders": [False, False]}
    host = {c: tg[c].tensor.cpu().numpy() for c in sargs["input ids"]}
    tqp_sort(True, tg, copy.deepcopy(sargs), False, "s")
    ref = O.tqp_sort(host, sargs, False)
    for c in sargs["input ids"]:
        np.testing.assert_array_equal(tg[c].tensor.cpu().numpy(), ref[c])


def test_project_substring_then_group_by_it():
    """tqp_project of substring(phone, 1, 2) gives the int8 [N, 2] slice the reference's
    evaluate returns (aggregate.py:114-119); a group-by over that string key (with a numeric
    projection beside it) matches the oracle."""
    import copy
    from tqpk.operators import tqp_hash_aggregate, tqp_project
    from tqpk.variable import Variable
    rng = np.random.default_rng(22)
    n = 100_003
    code = rng.integers(10, 35, n)
    phone = rng.integers(ord("0"), ord("9") + 1, (n, 15)).astype(np.int8)
    phone[:, 0] = ord("0") + code // 10
    phone[:, 1] = ord("0") + code % 10
    phone[:, 2] = ord("-")
    bal = rng.integers(-99999, 999999, n) / 100.0
    cols = {317: phone, 318: bal}
    tg = {317: Variable(torch.from_numpy(phone).cuda(), "string"), 318: Variable(torch.from_numpy(bal).cuda(), "float")}
    pargs = {"rename map": {}, "materialized in": [317, 318],
             "used expr": [[["substring", ["c_phone#317", "1", "2"]], "AS", "cntrycode#400"],
                           [["c_acctbal#318", "*", "2.0"], "AS", "dbl#401"]],
             "materialized out": [400, 401]}
    tqp_project(True, tg, copy.deepcopy(pargs), None, None, "p")
    ref = O.tqp_project(dict(cols), copy.deepcopy(pargs))
    got = tg[400].tensor.cpu().numpy()
    assert got.dtype == np.int8 and got.shape == (n, 2) and tg[400].tensor_type == "string"
    np.testing.assert_array_equal(got, ref[400])
    np.testing.assert_array_equal(tg[401].tensor.cpu().numpy(), ref[401])
    aargs = {"is partial": False, "keys": ["cntrycode#400"], "input ids": [400, 401],
             "results": ["cntrycode#400", [[["count", ["1"]], "#", "500L"], "AS", "n#501"],
                         [[["sum", ["dbl#401"]], "#", "502"], "AS", "s#503"]],
             "out agg ids": [501, 503]}
    tqp_hash_aggregate(True, tg, copy.deepcopy(aargs), None, None, "a")
    agg = O.tqp_hash_aggregate({400: ref[400], 401: ref[401]}, copy.deepcopy(aargs))
    np.testing.assert_array_equal(tg[400].tensor.cpu().numpy(), agg[400])
    np.testing.assert_array_equal(tg[501].tensor.cpu().numpy().reshape(-1), agg[501].reshape(-1))
    assert_f64_close(tg[503].tensor.cpu().numpy().reshape(-1), agg[503].reshape(-1),
                     magnitude=np.abs(ref[401]).sum())


def test_late_materialisation_masks_golden():
    """Inputs that do not share one mask: each masked column is compacted by its own mask first,
    as the reference's pipeline does (vortex_pipeline.py:54-58)."""
    from tqpk.operators import join_vortex, tqp_hash_aggregate
    ins, outs, args = load("late_materialisation_masks")
    types = args["types"]
    cols = {k: v for k, v in ins.items() if isinstance(k, int)}

    def tg_of(ids, types_):
        return {c: V(cols[c] if c in cols else None, types_[str(c)]) for c in ids}
    for name, ids, out_ids in (("mixed", (1, 3, 6, 900), (611, 612, 613, 614)), ("two", (1, 3, 7, 900, 901), (631, 632))):
        a = copy.deepcopy(args[name])
        a["mask map"] = {int(k): v for k, v in a["mask map"].items()}
        tg = tg_of(ids, types)
        tqp_hash_aggregate(True, tg, a, None, None, "a")
        order = np.argsort(outs[f"{name}_1"].reshape(-1), kind="stable")
        np.testing.assert_array_equal(np_(tg[1].tensor).reshape(-1), outs[f"{name}_1"].reshape(-1)[order])
        for c in out_ids:
            g, o = outs[f"{name}_{c}"][order], np_(tg[c].tensor)
            assert o.dtype == g.dtype, (c, o.dtype, g.dtype)
            assert_f64_close(o, g) if g.dtype == np.float64 else np.testing.assert_array_equal(o, g)
    jcols = {int(k[1:]): v for k, v in ins.items() if isinstance(k, str) and k.startswith("j")}
    tg = {c: V(v, args["jtypes"][str(c)]) for c, v in jcols.items()}
    j = copy.deepcopy(args["join"])
    j["mask map"] = {int(k): v for k, v in j["mask map"].items()}
    join_vortex(True, tg, j, 11, 21, [], "inner", None, None, "j")
    for c in (11, 21, 23, 26):
        np.testing.assert_array_equal(np_(tg[c].tensor).reshape(-1), outs[f"join_{c}"].reshape(-1))


def test_join_outer_string_payload_raises_like_the_reference():
    """The reference's null fill of an [N, w] payload does not broadcast and raises RuntimeError
    (conversion.py:52-57); the drop-in raises the same class."""
    from tqpk.operators import join_vortex
    ins, outs, args = load("join_outer_string_payload")
    assert args["error"] == "RuntimeError"
    tg = tg_from(ins, args["types"])
    with pytest.raises(RuntimeError):
        join_vortex(True, tg, copy.deepcopy(args["join"]), 11, 21, [], "right-outer", None, None, "j")
