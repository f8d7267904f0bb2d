"""Pins the oracle against golden vectors produced by the reference's own
operators (tests/golden/make_golden.py).  CPU only."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import tqp_oracle as O

GOLD = Path(__file__).resolve().parent / "golden"


def load(name):
    z = np.load(GOLD / f"{name}.npz", allow_pickle=False)
    ins = {int(k[3:]) if k[3:].isdigit() else k[3:]: z[k] for k in z.files if k.startswith("in_")}
    outs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return ins, outs, json.loads(str(z["args"]))


def _by_key(keys, *vals):
    order = np.lexsort([k.reshape(-1) for k in reversed(keys)])
    return [k.reshape(-1)[order] for k in keys], [v[order] for v in vals]


def assert_f64_close(a, b, rel=1e-12):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape
    scale = np.maximum(np.abs(a), np.abs(b))
    assert np.all(np.abs(a - b) <= rel * scale + 1e-300), (a, b)


def test_filter_predicates():
    ins, outs, args = load("filter_predicates")
    for i, tree in enumerate(args["trees"]):
        got = O.eval_filter([tree], ins)
        np.testing.assert_array_equal(got.reshape(-1), outs[f"mask{i}"], err_msg=str(tree))


def test_filter_strings():
    ins, outs, args = load("filter_strings")
    for i, tree in enumerate(args["trees"]):
        got = O.eval_filter([tree], ins)
        np.testing.assert_array_equal(got.reshape(-1), outs[f"mask{i}"], err_msg=str(tree))


def test_filter_substring():
    ins, outs, args = load("filter_substring")
    for i, tree in enumerate(args["trees"]):
        got = O.eval_filter([tree], ins)
        np.testing.assert_array_equal(got.reshape(-1), outs[f"mask{i}"], err_msg=str(tree))


def test_filter_agg_sort_lineitem():
    ins, outs, args = load("filter_agg_sort_lineitem")
    mask = O.eval_filter(args["filter"]["filter tree"], {7: ins[7]})
    np.testing.assert_array_equal(mask, outs["mask"])
    cols = dict(ins)
    cols[900] = mask
    agg = O.tqp_hash_aggregate(cols, args["aggregate"])
    srt = O.tqp_sort(agg, args["sort"], False)
    for cid in args["sort"]["input ids"]:
        g, o = outs[str(cid)], srt[cid]
        assert g.dtype == o.dtype and g.shape == o.shape, cid
        if g.dtype == np.float64:
            assert_f64_close(o, g)
        else:
            np.testing.assert_array_equal(o, g)


@pytest.mark.parametrize("name", ["join_agg_topk_unique", "join_duplicates", "join_semi", "join_anti", "join_outer"])
def test_join_cases(name):
    ins, outs, args = load(name)
    cols = dict(ins)
    for fa in args["filters"]:
        used = fa["materialized in"]
        cols[fa["out mask id"]] = O.eval_filter(fa["filter tree"], {c: ins[c] for c in used})
    np.testing.assert_array_equal(cols[901], outs["mask901"])
    np.testing.assert_array_equal(cols[902], outs["mask902"])
    res, rows = O.join_vortex(cols, args["join"], 11, 21, args["type"])
    assert rows == int(outs["rows"].reshape(-1)[0])
    # pairs are compared as sorted sets of output rows
    ids = (11, 21, 23, 24)
    if outs["11"].size == 0:          # semi / anti joins output no build-side rows
        assert res[11].size == 0
        ids = (21, 23, 24)
    got = np.stack([res[c].astype(np.float64) for c in ids], 1)
    exp = np.stack([outs[str(c)].astype(np.float64) for c in ids], 1)
    np.testing.assert_array_equal(got[np.lexsort(got.T[::-1])], exp[np.lexsort(exp.T[::-1])])
    if "aggregate" in args:
        agg = O.tqp_hash_aggregate(res, args["aggregate"])
        (gk,), (gv,) = _by_key([outs["agg_key"]], outs["agg_revenue"])
        np.testing.assert_array_equal(agg[11].reshape(-1), gk)
        assert_f64_close(agg[302], gv)
        top = O.tqp_sort({11: agg[11], 302: agg[302]}, args["topk"], True)
        np.testing.assert_array_equal(top[11], outs["top_key"])
        assert_f64_close(top[302], outs["top_revenue"])


def test_join_kernel_direct():
    ins, outs, args = load("join_kernel_direct")
    for name in args["specs"]:
        li, ri = O.join_indices(ins[f"{name}_left"], ins[f"{name}_right"], "inner")
        got = np.stack([li, ri], 1)
        exp = np.stack([outs[f"{name}_lidx"], outs[f"{name}_ridx"]], 1)
        np.testing.assert_array_equal(got[np.lexsort(got.T[::-1])], exp[np.lexsort(exp.T[::-1])])
        # probe-row order is the reference's (ascending matched right row)
        np.testing.assert_array_equal(ri, outs[f"{name}_ridx"])


def test_aggregate_ops():
    ins, outs, args = load("aggregate_ops")
    agg = O.tqp_hash_aggregate(dict(ins), args["aggregate"])
    ids = args["aggregate"]["out agg ids"]
    keys_g, vals_g = _by_key([outs["1"], outs["2"]], *[outs[str(i)] for i in ids])
    np.testing.assert_array_equal(agg[1].reshape(-1), keys_g[0])
    np.testing.assert_array_equal(agg[2].reshape(-1), keys_g[1])
    for i, g in zip(ids, vals_g):
        assert agg[i].dtype == g.dtype, i
        if g.dtype == np.float64:
            assert_f64_close(agg[i], g)
        else:
            np.testing.assert_array_equal(agg[i], g)
    glob = O.tqp_hash_aggregate({3: ins[3], 4: ins[4]}, args["global"])
    for i in args["global"]["out agg ids"]:
        g = outs[str(i)]
        assert glob[i].dtype == g.dtype
        assert_f64_close(glob[i], g) if g.dtype == np.float64 else np.testing.assert_array_equal(glob[i], g)


def test_aggregate_two_step():
    ins, outs, args = load("aggregate_two_step")
    agg = O.tqp_hash_aggregate(dict(ins), args["aggregate"])
    ids = args["aggregate"]["out agg ids"]
    (k,), vals = _by_key([outs["1"]], *[outs[str(i)] for i in ids])
    np.testing.assert_array_equal(agg[1].reshape(-1), k)
    for i, g in zip(ids, vals):
        assert agg[i].dtype == g.dtype
        assert_f64_close(agg[i], g) if g.dtype == np.float64 else np.testing.assert_array_equal(agg[i], g)


def test_aggregate_expressions():
    """CASE WHEN / conditions / year() / arithmetic over aggregates, after a projection."""
    ins, outs, args = load("aggregate_expressions")
    proj = O.tqp_project(dict(ins), args["project"])
    for c in args["project"]["materialized out"]:
        g = outs[f"p{c}"]
        assert proj[c].dtype == g.dtype, c
        np.testing.assert_array_equal(proj[c], g)
    agg = O.tqp_hash_aggregate(proj, args["aggregate"])
    ids = args["aggregate"]["out agg ids"]
    keys_g, vals_g = _by_key([outs["10"], outs["20"]], *[outs[str(i)] for i in ids])
    np.testing.assert_array_equal(agg[10].reshape(-1), keys_g[0])
    np.testing.assert_array_equal(agg[20].reshape(-1), keys_g[1])
    for i, g in zip(ids, vals_g):
        assert agg[i].dtype == g.dtype, i
        assert_f64_close(agg[i], g) if g.dtype == np.float64 else np.testing.assert_array_equal(agg[i], g)


def test_aggregate_string_keys():
    """String keys, five mixed keys, a float key with -0.0 / +0.0, under a mask."""
    from golden_io import key_tuple_order
    ins, outs, args = load("aggregate_string_keys")
    mask = O.eval_filter(args["filter"]["filter tree"], {8: ins[8]})
    np.testing.assert_array_equal(mask, outs["mask"])
    cols = dict(ins)
    cols[900] = mask
    for name, a in args["sets"].items():
        agg = O.tqp_hash_aggregate(cols, a)
        kids = [O.get_id(k) for k in a["keys"]]
        order = key_tuple_order([outs[f"{name}_{k}"] for k in kids])
        for k in kids:
            g = outs[f"{name}_{k}"][order]
            assert agg[k].dtype == g.dtype and agg[k].shape == g.shape, (name, k)
            np.testing.assert_array_equal(agg[k], g)
        for i in a["out agg ids"]:
            g = outs[f"{name}_{i}"][order]
            assert agg[i].dtype == g.dtype, (name, i)
            assert_f64_close(agg[i], g) if g.dtype == np.float64 else np.testing.assert_array_equal(agg[i], g)


def test_oracle_year_past_the_table_raises():
    with pytest.raises(IndexError):
        O.eval_agg_expr(["year", ["d#1"]], {1: np.array([3651, 3652], np.int32)})


def test_sort_multikey():
    ins, outs, args = load("sort_multikey")
    for i, (spec, lim) in enumerate(args["specs"]):
        res = O.tqp_sort(ins, spec, lim)
        for c in spec["input ids"]:
            np.testing.assert_array_equal(res[c], outs[f"s{i}_{c}"], err_msg=f"spec {i} col {c}")


def test_fsum_truth_close_to_bincount():
    rng = np.random.default_rng(5)
    v = rng.integers(90000, 10495001, 200000) / 100.0
    inv = rng.integers(0, 4, v.size)
    assert_f64_close(O.fsum_groups(v, inv, 4), np.bincount(inv, weights=v, minlength=4), rel=1e-13)


def test_oracle_projection_dtypes_follow_torch():
    import numpy as np
    from oracle import tqp_oracle as O
    cols = {1: np.array([1.5, 2.5]), 3: np.array([1, 2], np.int32), 4: np.array([10, 20], np.int64)}
    args = {"rename map": {}, "used expr": [[[["q#3", "+", "q#3"], "AS", "a#13"]], [[["w#4", "*", "q#3"], "AS", "b#14"]],
                                             [[["p#1", "*", "2"], "AS", "c#15"]]],
            "materialized in": [1, 3, 4], "materialized out": [13, 14, 15]}
    out = O.tqp_project(cols, args)
    assert out[13].dtype == np.int32 and out[14].dtype == np.int64 and out[15].dtype == np.float64
    np.testing.assert_array_equal(out[14], [10, 40])


def test_late_materialisation_masks():
    ins, outs, args = load("late_materialisation_masks")
    cols = {k: v for k, v in ins.items() if isinstance(k, int)}
    mixed = dict(args["mixed"], **{"mask map": {int(k): v for k, v in args["mixed"]["mask map"].items()}})
    got = O.tqp_hash_aggregate(cols, mixed)
    (k,), vals = _by_key([outs["mixed_1"]], *[outs[f"mixed_{c}"] for c in (611, 612, 613, 614)])
    (gk,), gvals = _by_key([got[1]], *[got[c] for c in (611, 612, 613, 614)])
    np.testing.assert_array_equal(gk, k)
    for a, b in zip(gvals, vals):
        assert_f64_close(a, b) if b.dtype == np.float64 else np.testing.assert_array_equal(a, b)
    two = dict(args["two"], **{"mask map": {int(k): v for k, v in args["two"]["mask map"].items()}})
    got = O.tqp_hash_aggregate(cols, two)
    (k,), vals = _by_key([outs["two_1"]], outs["two_631"], outs["two_632"])
    (gk,), gvals = _by_key([got[1]], got[631], got[632])
    np.testing.assert_array_equal(gk, k)
    for a, b in zip(gvals, vals):
        assert_f64_close(a, b) if b.dtype == np.float64 else np.testing.assert_array_equal(a, b)
    jcols = {int(k[1:]): v for k, v in ins.items() if isinstance(k, str) and k.startswith("j")}
    j = dict(args["join"], **{"mask map": {int(k): v for k, v in args["join"]["mask map"].items()}})
    res, _ = O.join_vortex(jcols, j, 11, 21, "inner")
    for c in (11, 21, 23, 26):
        np.testing.assert_array_equal(res[c].reshape(-1), outs[f"join_{c}"].reshape(-1))


def f32_tag(ins, outs, tag):
    """One aggregate of the float32 fixture: its inputs, its outputs ordered by key."""
    cols = {int(k.split("_")[1]): v for k, v in ins.items() if isinstance(k, str) and k.startswith(tag + "_")}
    return cols, {k[len(tag) + 1:]: v for k, v in outs.items() if k.startswith(tag + "_")}


@pytest.mark.parametrize("tag", ["one", "two"])
def test_aggregate_float32(tag):
    """torch's float32 results (an integer column with a Python float, integer true division, a
    CASE mixing a float literal with integers): the 1-step path's float32 sums are the
    reference's row-order float32 additions, bit for bit; the 2-step path's per-group sum of
    float32 sub-slots may differ in its last bits (summation order)."""
    ins, outs, args = load("aggregate_float32")
    cols, out = f32_tag(ins, outs, tag)
    a = args[tag]["aggregate"]
    agg = O.tqp_hash_aggregate(cols, a)
    ids = a["out agg ids"]
    (k,), vals = _by_key([out["1"]], *[out[str(i)] for i in ids])
    np.testing.assert_array_equal(agg[1].reshape(-1), k)
    for i, g in zip(ids, vals):
        assert agg[i].dtype == g.dtype, (i, agg[i].dtype, g.dtype)
        if tag == "two" and (g.dtype == np.float32 or i == 902):    # 902: float64 avg of a float32 sum
            np.testing.assert_allclose(agg[i], g, rtol=2e-6, atol=0)
        elif g.dtype == np.float64:
            assert_f64_close(agg[i], g)
        else:
            np.testing.assert_array_equal(agg[i], g, err_msg=str(i))


def test_project_float32():
    """The same float32 expressions as a projection: the oracle's float32 arithmetic is the
    reference's bit for bit (and float64 where a float64 column takes part)."""
    ins, outs, args = load("aggregate_float32")
    cols, _ = f32_tag(ins, outs, "one")
    proj = O.tqp_project(cols, args["project"])
    for c in args["project"]["materialized out"]:
        g = outs[f"proj_{c}"]
        assert proj[c].dtype == g.dtype, c
        np.testing.assert_array_equal(proj[c], g)


def test_aggregate_substring():
    """sum / count of a one-byte substring (alone and times 2, which wraps in int8 as torch's does)."""
    ins, outs, args = load("aggregate_substring")
    agg = O.tqp_hash_aggregate(dict(ins), args["aggregate"])
    ids = args["aggregate"]["out agg ids"]
    (k,), vals = _by_key([outs["1"]], *[outs[str(i)] for i in ids])
    np.testing.assert_array_equal(agg[1].reshape(-1), k)
    for i, g in zip(ids, vals):
        assert agg[i].dtype == g.dtype, i
        np.testing.assert_array_equal(agg[i], g)


def test_join_outer_string_payload_raises():
    """The reference's right-outer join raised RuntimeError on this fixture: the null fill of an
    [N, w] build-side column broadcasts its [K] mask over the [K, w] rows (conversion.py:52-57)."""
    ins, outs, args = load("join_outer_string_payload")
    assert str(outs["raised"].reshape(-1)[0]) == args["error"] == "RuntimeError"
    with pytest.raises(RuntimeError):
        O.join_vortex(dict(ins), args["join"], 11, 21, "right-outer")
