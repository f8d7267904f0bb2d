"""GPU parity on random inputs: the generators of tests/test_oracle_vs_reference.py (whose oracle runs
there beside the reference's own operators) through the CUDA path, against the oracle; and the
right-outer null fill of 2-D build-side columns.  The file is named so pytest collects it after the
other GPU tests: under -x, a failure here leaves their results standing.

Masks bit-exact; float64 sums and averages within 1e-12 relative, or 1e-12 of the group's sum of
|terms| where they cancel (over its count for an average); float32 results within 2e-4 of the same
scale (their row-by-row float32 summation); integers exact.  Float64 minima and maxima are
within the same bound: the generated group-by evaluates x * (1 - y) as one fused multiply-add.
"""
import copy

import numpy as np
import pytest
import torch

from golden_io import assert_f64_close
from oracle import tqp_oracle as O
from test_oracle_vs_reference import AGGS, KEYS, SUBQUERY, TYPES, col, columns, num_expr, tree, _has_col, _key_order

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need CUDA")
    from tqpk import build, _lib
    build.build()
    return _lib.load()


def _v(a, t="int"):
    from tqpk.variable import Variable
    return Variable(torch.from_numpy(np.ascontiguousarray(a)).cuda(), t)


def np_(t):
    return t.detach().cpu().numpy()


def _vars(cols):
    from tqpk.variable import Variable
    return {c: Variable(torch.from_numpy(np.ascontiguousarray(a)).cuda(), TYPES.get(c, "bool")) for c, a in cols.items()}


@pytest.mark.parametrize("seed", range(6))
def test_filter_random_trees_vs_oracle(seed):
    """Random numeric and string predicate trees through tqp_filter."""
    from tqpk.operators import tqp_filter
    rng = np.random.default_rng(2100 + seed)
    cols = columns(rng, 40_003)
    ran = 0
    for i in range(12):
        t = tree(rng)
        used = sorted({c for c in (1, 2, 3, 4, 5, 7) if col(c) in repr(t)})
        args = {"name": "Filter", "filter tree": [t], "materialized in": used, "out mask id": 900}
        try:
            expect = np.asarray(O.eval_filter([t], {c: cols[c] for c in used}, 40_003, SUBQUERY)).reshape(-1)
        except (TypeError, ValueError) as e:        # the reference rejects these too
            with pytest.raises(type(e)):
                tqp_filter(True, _vars({c: cols[c] for c in used}), copy.deepcopy(args), SUBQUERY, None, None, "f")
            continue
        tg = _vars({c: cols[c] for c in used})
        try:
            tqp_filter(True, tg, copy.deepcopy(args), SUBQUERY, None, None, "f")
        except NotImplementedError as e:            # a program longer than the kernel's 32 instructions
            assert "longer than" in str(e), e
            continue
        np.testing.assert_array_equal(tg[900].tensor.cpu().numpy().reshape(-1), expect, err_msg=repr(t))
        ran += 1
    assert ran >= 6


def _check(got, exp, magnitude, what):
    assert got.dtype == exp.dtype and got.shape == exp.shape, (what, got.dtype, exp.dtype)
    if exp.dtype == np.float32:
        # the reference adds float32 values row by row; the kernels add their float64 images and
        # round once: within 2e-4 of the larger of the result and the group's sum of |terms|
        scale = np.abs(exp.astype(np.float64))
        if magnitude is not None:
            scale = np.maximum(scale, magnitude)
        ok = (np.abs(got.astype(np.float64) - exp.astype(np.float64)) <= 2e-4 * scale) | (got == exp)
        assert np.all(ok), (what, got[~ok][:5], exp[~ok][:5])
    elif exp.dtype.kind == "f":
        assert_f64_close(got, exp, magnitude=magnitude)
    else:
        np.testing.assert_array_equal(got, exp, err_msg=what)


@pytest.mark.parametrize("seed", range(16))
def test_group_by_random_expressions_vs_oracle(seed):
    """Random arithmetic / CASE expressions over float64, int64, int32 and uint8 columns, and the
    fixed expression set, under sum / avg / min / max / count, grouped by int32, uint8, int64 and
    string keys, some behind a filter's mask, through tqp_hash_aggregate."""
    from tqpk.operators import tqp_hash_aggregate
    rng = np.random.default_rng(2200 + seed)
    n = int(rng.integers(50, 30_000))
    cols = columns(rng, n)
    keys = KEYS[seed % len(KEYS)]
    results, args_of = list(keys), {}
    for i in range(4):
        if i < 2:
            e = num_expr(rng)
            while not _has_col(e):
                e = num_expr(rng)
            fn = str(rng.choice(["sum", "avg", "min", "max", "count"]))
            arg = e if isinstance(e, list) and e and e[0] == "CASE" else [e]
            call = [fn, arg]
        else:
            call = AGGS[int(rng.integers(0, len(AGGS)))]
        results.append([[call, "#", f"{400 + i}" + ("L" if call[0] == "count" else "")], "AS", f"r#{500 + i}"])
        args_of[500 + i] = call[1]
    used = sorted({c for c in cols if col(c) in repr(results)} | {3})
    args = {"name": "Aggregate", "is partial": False, "keys": keys or None, "input ids": used, "results": results,
            "out agg ids": [500 + i for i in range(4)]}
    cols_in = {c: cols[c] for c in used}
    if seed % 3 == 1:
        cols_in[900] = cols[1] > 1000
        args["mask map"] = {c: 900 for c in used}
    exp = O.tqp_hash_aggregate(cols_in, copy.deepcopy(args))
    tg = _vars(cols_in)
    try:
        tqp_hash_aggregate(True, tg, copy.deepcopy(args), None, None, "a")
    except NotImplementedError as e:                # a program beyond the kernel's limits
        assert "exceed" in str(e) or "more than" in str(e), e
        pytest.skip(str(e))
    key_ids = [int(k.split("#")[1]) for k in keys]
    eo = _key_order([exp[k] for k in key_ids])
    go = _key_order([tg[k].tensor.cpu().numpy() for k in key_ids])
    for k in key_ids:
        np.testing.assert_array_equal(tg[k].tensor.cpu().numpy()[go], exp[k][eo])
    masked = {c: (a[cols_in[900]] if 900 in cols_in else a) for c, a in cols_in.items() if c != 900}
    rows = next(iter(masked.values())).shape[0]
    if key_ids:
        _, inverse = O.group_rows([masked[k] for k in key_ids])          # the oracle's (ascending) groups
        G = int(inverse.max()) + 1 if inverse.size else 0
    else:
        inverse, G = np.zeros(rows, np.int64), 1
    for oid in args["out agg ids"]:
        # float64 sums: within 1e-12 of the group's sum of |terms| (any two summation orders are);
        # averages: that over the group's count
        magnitude = None
        try:
            v = O.eval_agg_expr(args_of[oid], masked)
            if isinstance(v, np.ndarray) and v.ndim == 1 and v.size == rows:
                a = np.abs(np.where(np.isfinite(v.astype(np.float64)), v.astype(np.float64), 0.0))
                magnitude = np.bincount(inverse, weights=a, minlength=G)
                if results[len(keys) + oid - 500][0][0][0] == "avg":
                    magnitude = magnitude / np.maximum(np.bincount(inverse, minlength=G), 1)
                magnitude = magnitude[eo] if key_ids else magnitude
        except Exception:                           # noqa: BLE001  a bound only, where it evaluates
            magnitude = None
        g = tg[oid].tensor.cpu().numpy()
        e = exp[oid]
        if key_ids:
            g, e = g[go], e[eo]
        _check(g, e, magnitude, f"{oid}: {results[len(keys) + oid - 500]}")


JOIN_TYPES = ["inner", "right-semi", "right-anti", "right-outer"]


@pytest.mark.parametrize("seed", range(16))
def test_join_random_key_dtypes_vs_oracle(seed):
    """Random joins of every type whose build and probe keys have different integer dtypes (the
    reference joins them, hashjoin.py:39-65), dense and sparse key domains, with masks, through
    join_vortex: the probe side in the reference's order, the build rows as a multiset per probe row
    (the reference's build-key sort is unstable)."""
    from tqpk.operators import join_vortex
    from tqpk.variable import Variable
    rng = np.random.default_rng(2300 + seed)
    jtype = JOIN_TYPES[seed % 4]
    bdt, pdt = [(np.int32, np.int64), (np.int64, np.int32), (np.int64, np.int64), (np.int32, np.uint8)][(seed // 4) % 4]
    nb, npr = int(rng.integers(50, 5000)), int(rng.integers(100, 40_000))
    hi = 250 if pdt == np.uint8 else nb + 40
    bkey = rng.permutation(min(nb, hi - 1)) + 1 if seed % 3 else rng.integers(1, max(2, min(nb, hi) // 3), nb)
    pkey = rng.integers(1, hi, npr)
    if seed % 2 and bdt == np.int64 and pdt == np.int64:       # a sparse key domain (the sorted directory)
        bkey, pkey = bkey * 1_000_003 + 17, pkey * 1_000_003 + 17
    cols = {11: bkey.astype(bdt), 12: rng.integers(0, 5, bkey.size).astype(np.int32),
            21: pkey.astype(pdt), 22: rng.integers(0, 5, npr).astype(np.int32),
            23: rng.integers(90000, 10495001, npr).astype(np.float64) / 100.0}
    cols[901] = rng.random(bkey.size) < 0.8
    cols[902] = rng.random(npr) < 0.7
    args = {"name": "Join", "left group": [11, 12], "right group": [21, 22, 23], "materialized in": [11, 12, 21, 22, 23]}
    if seed % 5 != 0:
        args["mask map"] = {11: 901, 12: 901, 21: 902, 22: 902, 23: 902}
    types_ = {11: "int", 12: "int", 21: "int", 22: "int", 23: "float", 901: "bool", 902: "bool"}
    exp, exp_rows = O.join_vortex(cols, copy.deepcopy(args), 11, 21, jtype)
    tg = {c: Variable(torch.from_numpy(np.ascontiguousarray(a)).cuda(), types_[c]) for c, a in cols.items()}
    rows = join_vortex(True, tg, copy.deepcopy(args), 11, 21, [], jtype, None, None, "j")
    assert rows == exp_rows
    for c in (21, 22, 23):
        np.testing.assert_array_equal(tg[c].tensor.cpu().numpy(), np.asarray(exp[c]), err_msg=f"{c} {jtype}")
    left = [c for c in (11, 12) if np.asarray(exp[c]).size]
    for c in (11, 12):
        assert tuple(tg[c].tensor.shape) == np.asarray(exp[c]).shape, (c, jtype)
    if left:
        e = np.stack([np.asarray(exp[c]).astype(np.float64) for c in left + [21, 22, 23]], 1)
        g = np.stack([tg[c].tensor.cpu().numpy().astype(np.float64) for c in left + [21, 22, 23]], 1)
        np.testing.assert_array_equal(g[np.lexsort(g.T[::-1])], e[np.lexsort(e.T[::-1])], err_msg=jtype)


@pytest.mark.parametrize("shape", ["k_equals_w", "one_row", "column_n1"])
def test_join_outer_two_dimensional_build_columns(shape):
    """A right-outer join's 2-D build-side columns are null-filled by the reference's broadcast
    rule (conversion.py:52-57): K == w output rows fill column j of every row whose build index j
    is null, K == 1 is a plain gather, and an [N, 1] column with K > 1 raises RuntimeError.  The
    oracle follows the rule and is checked against the reference's own function on the CPU."""
    from tqpk.operators import join_vortex
    left_keys = np.arange(10, dtype=np.int32)
    right_keys = {"k_equals_w": [1, 100, 3, 200], "one_row": [7], "column_n1": [1, 100, 3]}[shape]
    right_keys = np.asarray(right_keys, dtype=np.int32)
    payload = (np.arange(40, dtype=np.int64).reshape(10, 4) % 91 + 33).astype(np.int8)   # [10, 4] rows
    if shape == "column_n1":
        payload = np.arange(100, 110, dtype=np.int64).reshape(10, 1)
    cols = {11: left_keys, 12: payload, 21: right_keys}
    args = {"left group": [11, 12], "right group": [21], "materialized in": [11, 12, 21]}
    tg = {11: _v(left_keys), 12: _v(payload, "string" if payload.dtype == np.int8 else "int"), 21: _v(right_keys)}
    if shape == "column_n1":
        with pytest.raises(RuntimeError):
            O.join_vortex(cols, copy.deepcopy(args), 11, 21, "right-outer")
        with pytest.raises(RuntimeError):
            join_vortex(True, tg, copy.deepcopy(args), 11, 21, [], "right-outer", None, None, "j")
        return
    ref, ref_rows = O.join_vortex(cols, copy.deepcopy(args), 11, 21, "right-outer")
    rows = join_vortex(True, tg, copy.deepcopy(args), 11, 21, [], "right-outer", None, None, "j")
    assert rows == ref_rows
    for c in (11, 12, 21):
        got = np_(tg[c].tensor)
        assert got.shape == np.asarray(ref[c]).shape, c
        np.testing.assert_array_equal(got, ref[c], err_msg=str(c))


@pytest.mark.parametrize("seed", range(12))
def test_project_random_expressions_vs_oracle(seed):
    """Random arithmetic / CASE trees and the fixed projection set (year(), string conditions,
    float32 and uint8 results, a substring slice) through tqp_project: row-wise results, so equal
    to the oracle's bit for bit, with the same dtypes."""
    from test_oracle_vs_reference import PROJ
    from tqpk.operators import tqp_project
    rng = np.random.default_rng(2400 + seed)
    n = int(rng.integers(1, 50_000))
    cols = columns(rng, n)
    picks = sorted(rng.choice(len(PROJ), 4, replace=False))
    exprs = [PROJ[p] for p in picks]
    outs = [41 + int(p) for p in picks]
    for j in range(3):
        e = num_expr(rng)
        while not (isinstance(e, list) and _has_col(e)):
            e = num_expr(rng)
        exprs.append([e if e[0] == "CASE" else [e], "AS", f"q#{60 + j}"])
        outs.append(60 + j)
    used = sorted({c for c in cols if col(c) in repr(exprs)})
    args = {"name": "Project", "rename map": {}, "materialized in": used, "used expr": exprs, "materialized out": outs}
    exp = O.tqp_project({c: cols[c] for c in used}, copy.deepcopy(args))
    tg = _vars({c: cols[c] for c in used})
    tqp_project(True, tg, copy.deepcopy(args), None, None, "p")
    for c in outs:
        got = tg[c].tensor.cpu().numpy()
        assert got.dtype == exp[c].dtype and got.shape == exp[c].shape, (c, got.dtype, exp[c].dtype)
        np.testing.assert_array_equal(got, exp[c], err_msg=str(exprs[outs.index(c)]))


@pytest.mark.parametrize("seed", range(12))
def test_sort_random_keys_vs_oracle(seed):
    """Random multi-key sorts through tqp_sort: int, date, uint8, float keys with ties (and both
    zeros), string keys, either direction, with and without a limit (the stable top-k)."""
    from tqpk.operators import tqp_sort
    rng = np.random.default_rng(2500 + seed)
    n = int(rng.integers(1, 60_000))
    cols = columns(rng, n)
    cols[5] = np.round(cols[5] / 20) * 20                     # ties, and -0.0 beside 0.0
    nk = int(rng.integers(1, 4))
    key_ids = [int(c) for c in rng.choice([1, 3, 4, 5, 6, 7], nk, replace=False)]
    inputs = sorted(set(key_ids) | {int(c) for c in rng.choice([2, 3, 8], 2, replace=False)})
    args = {"input ids": inputs, "key ids": key_ids, "key orders": [bool(b) for b in rng.integers(0, 2, nk)]}
    with_limit = bool(seed % 2)
    if with_limit:
        args["limit"] = int(rng.integers(1, min(n, 300) + 1))
    exp = O.tqp_sort({c: cols[c] for c in inputs}, args, with_limit)
    tg = _vars({c: cols[c] for c in inputs})
    tqp_sort(True, tg, copy.deepcopy(args), with_limit, "s")
    for c in inputs:
        got = tg[c].tensor.cpu().numpy()
        assert got.dtype == exp[c].dtype and got.shape == exp[c].shape, (c, args)
        np.testing.assert_array_equal(got, exp[c], err_msg=f"column {c} of {args}")
