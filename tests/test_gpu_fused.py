"""try_fused on the GPU: the fused run of Filter, Filter, Join, Aggregate, take ordered leaves the
same take-ordered outputs in tensor_group as the drop-in operators run one by one (keys
bit-exact, float64 sums within 1e-12 relative), from resident or still-copying columns; a
repeated build key runs nothing."""
import copy

import numpy as np
import pytest
import torch

from golden_io import assert_f64_close

pytestmark = pytest.mark.gpu


def _plan(limit=10, desc=True):
    ops = [3, 4, 5, 6, 7]
    args = {
        3: {"name": "Filter", "filter tree": [["bd#12", "<", "1170"]], "materialized in": [12], "out mask id": 901},
        4: {"name": "Filter", "filter tree": [["pd#22", ">", "1170"]], "materialized in": [22], "out mask id": 902},
        5: {"name": "Join", "left keys": [11], "right keys": [21], "join type": "Inner",
            "left group": [11, 12], "right group": [21, 22, 23, 24], "materialized in": [11, 21, 23, 24],
            "mask map": {11: 901, 21: 902, 23: 902, 24: 902}},
        6: {"name": "Aggregate", "is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
            "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "301"], "AS", "rev#302"]],
            "out agg ids": [302]},
        7: {"name": "take ordered", "limit": limit, "input ids": [11, 302], "key ids": [302], "key orders": [desc]},
    }
    return ops, args


TYPES = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}


def _tables(nb, np_, seed, dup=False):
    from tqpk import datagen
    t = datagen.join_tables(nb, np_, seed)
    if dup:
        t["b_key"][nb // 2] = t["b_key"][nb // 3]
    return {11: t["b_key"], 12: t["b_date"], 21: t["p_fk"], 22: t["p_date"], 23: t["p_price"], 24: t["p_discount"]}


def _operators(cols, ops, args):
    from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
    from tqpk.variable import Variable
    tg = {c: Variable(torch.from_numpy(a).cuda(), TYPES[c]) for c, a in cols.items()}
    a = copy.deepcopy(args)
    tqp_filter(True, tg, a[3], None, None, None, "f1")
    tqp_filter(True, tg, a[4], None, None, None, "f2")
    join_vortex(True, tg, a[5], 11, 21, [], "inner", None, None, "j")
    tqp_hash_aggregate(True, tg, a[6], None, None, "a")
    tqp_sort(True, tg, a[7], True, "t")
    return tg


@pytest.mark.parametrize("nb,np_,limit,desc", [(200_000, 800_003, 10, True), (1_500_000, 6_001_215, 10, True),
                                               (5_000, 20_000, 100, False), (300, 500, 256, True)])
def test_fused_run_matches_the_operators(nb, np_, limit, desc):
    from tqpk.operators import try_fused
    from tqpk.variable import Variable
    cols = _tables(nb, np_, 41)
    ops, args = _plan(limit, desc)
    exp = _operators(cols, ops, args)
    tg = {c: Variable(torch.from_numpy(a).cuda(), TYPES[c]) for c, a in cols.items()}
    assert try_fused(True, tg, ops, copy.deepcopy(args), 0) == 5
    got_k, exp_k = tg[11].tensor, exp[11].tensor
    assert got_k.shape == exp_k.shape and got_k.dtype == exp_k.dtype and tg[11].tensor_type == "int"
    np.testing.assert_array_equal(got_k.cpu().numpy(), exp_k.cpu().numpy())
    assert tg[302].tensor.dtype == torch.float64 and tg[302].tensor_type == "float"
    assert_f64_close(tg[302].tensor.cpu().numpy(), exp[302].tensor.cpu().numpy())
    # the rows read back with the count equal the device columns bit for bit
    from tqpk.variable import host_values
    np.testing.assert_array_equal(host_values(tg[11]), got_k.cpu().numpy())
    np.testing.assert_array_equal(host_values(tg[302]).view(np.uint64), tg[302].tensor.cpu().numpy().view(np.uint64))


def test_fused_run_from_columns_still_copying():
    from tqpk.ingress import ColumnStager
    from tqpk.operators import try_fused
    cols = _tables(400_000, 1_600_001, 43)
    ops, args = _plan()
    exp = _operators(cols, ops, args)
    host = {c: torch.from_numpy(a).pin_memory() for c, a in cols.items()}
    for _ in range(2):
        tg = ColumnStager(torch.device("cuda")).stage(host, TYPES, (12, 11, 22, 21, 23, 24))
        assert try_fused(True, tg, ops, copy.deepcopy(args), 0) == 5
        np.testing.assert_array_equal(tg[11].tensor.cpu().numpy(), exp[11].tensor.cpu().numpy())
        assert_f64_close(tg[302].tensor.cpu().numpy(), exp[302].tensor.cpu().numpy())


def test_repeated_build_key_runs_nothing():
    from tqpk.operators import try_fused
    from tqpk.variable import Variable
    cols = _tables(50_000, 200_000, 47, dup=True)
    ops, args = _plan()
    tg = {c: Variable(torch.from_numpy(a).cuda(), TYPES[c]) for c, a in cols.items()}
    before = {c: v.tensor for c, v in tg.items()}
    assert try_fused(True, tg, ops, copy.deepcopy(args), 0) == 0
    assert set(tg) == set(before) and all(tg[c].tensor is before[c] for c in tg)
    # the operators then run the same plan (duplicates allowed there)
    exp = _operators(cols, ops, args)
    assert exp[11].tensor.shape == (10, 1)


# ---------------------------------------------------------------------------- the star plan
STAR_TYPES = {31: "int", 32: "int", 41: "int", 42: "int", 43: "float", 44: "float", 51: "int", 52: "int", 61: "int"}


def _star_plan(limit=100, with_count=True):
    ops = [3, 4, 5, 6, 7, 8]
    results = ["c#61", [[["sum", [["p#43", "*", ["1.0", "-", "d#44"]]]], "#", "71"], "AS", "rev#72"]]
    if with_count:
        results.append([[["count", ["1"]], "#", "73L"], "AS", "cnt#74"])
    args = {
        3: {"name": "Filter", "filter tree": [["cat#32", "=", "1"]], "materialized in": [32], "out mask id": 901},
        4: {"name": "Join", "left keys": [31], "right keys": [41], "join type": "Inner", "left group": [31, 32],
            "right group": [41, 42, 43, 44], "materialized in": [31, 41, 42, 43, 44], "mask map": {31: 901}},
        5: {"name": "Join", "left keys": [51], "right keys": [42], "join type": "Inner", "left group": [51, 52],
            "right group": [31, 41, 42, 43, 44], "materialized in": [51, 52, 42, 43, 44]},
        6: {"name": "Join", "left keys": [61], "right keys": [52], "join type": "Inner", "left group": [61],
            "right group": [51, 52, 42, 43, 44], "materialized in": [61, 52, 43, 44]},
        7: {"name": "Aggregate", "is partial": False, "keys": ["c#61"], "input ids": [61, 43, 44],
            "results": results, "out agg ids": [72, 74] if with_count else [72]},
        8: {"name": "take ordered", "limit": limit, "input ids": [61, 72, 74] if with_count else [61, 72],
            "key ids": [72], "key orders": [True]},
    }
    return ops, args


def _star_tables(nf, na, nb, nc, seed, dup=False):
    from tqpk import datagen
    t = datagen.star_tables(nf, na, nb, nc, seed)
    if dup:
        t["b_key"][nb // 2] = t["b_key"][nb // 3]
    return {31: t["a_key"], 32: t["a_cat"], 41: t["f_fka"], 42: t["f_fkb"], 43: t["f_price"], 44: t["f_discount"],
            51: t["b_key"], 52: t["b_fkc"], 61: t["c_key"]}


def _star_operators(cols, ops, args):
    from tqpk.operators import join_vortex, tqp_filter, tqp_hash_aggregate, tqp_sort
    from tqpk.variable import Variable
    tg = {c: Variable(torch.from_numpy(a).cuda(), STAR_TYPES[c]) for c, a in cols.items()}
    a = copy.deepcopy(args)
    tqp_filter(True, tg, a[3], None, None, None, "f")
    for u, lk, rk in ((4, 31, 41), (5, 51, 42), (6, 61, 52)):
        join_vortex(True, tg, a[u], lk, rk, [], "inner", None, None, "j")
    tqp_hash_aggregate(True, tg, a[7], None, None, "a")
    tqp_sort(True, tg, a[8], True, "t")
    return tg


@pytest.mark.parametrize("sizes,limit,with_count", [((400_000, 20_000, 100_000, 10_000), 100, True),
                                                     ((2_000_000, 200_000, 500_000, 150_000), 10, True),
                                                     ((50_000, 3_000, 8_000, 500), 256, False)])
def test_fused_star_matches_the_operators(sizes, limit, with_count):
    from tqpk.operators import try_fused
    from tqpk.variable import Variable, host_values
    cols = _star_tables(*sizes, seed=61)
    ops, args = _star_plan(limit, with_count)
    exp = _star_operators(cols, ops, args)
    tg = {c: Variable(torch.from_numpy(a).cuda(), STAR_TYPES[c]) for c, a in cols.items()}
    assert try_fused(True, tg, ops, copy.deepcopy(args), 0) == 6
    got_k, exp_k = tg[61].tensor, exp[61].tensor
    assert got_k.shape == exp_k.shape and got_k.dtype == exp_k.dtype and tg[61].tensor_type == "int"
    np.testing.assert_array_equal(got_k.cpu().numpy(), exp_k.cpu().numpy())
    assert_f64_close(tg[72].tensor.cpu().numpy(), exp[72].tensor.cpu().numpy())
    np.testing.assert_array_equal(host_values(tg[61]), got_k.cpu().numpy())
    np.testing.assert_array_equal(host_values(tg[72]).view(np.uint64), tg[72].tensor.cpu().numpy().view(np.uint64))
    if with_count:
        assert tg[74].tensor.dtype == exp[74].tensor.dtype and tg[74].tensor_type == "int"
        np.testing.assert_array_equal(tg[74].tensor.cpu().numpy().reshape(-1), exp[74].tensor.cpu().numpy().reshape(-1))
        np.testing.assert_array_equal(host_values(tg[74]), tg[74].tensor.cpu().numpy())


def test_fused_star_with_a_repeated_dimension_key_runs_nothing():
    from tqpk.operators import try_fused
    from tqpk.variable import Variable
    cols = _star_tables(100_000, 5_000, 20_000, 2_000, seed=62, dup=True)
    ops, args = _star_plan()
    tg = {c: Variable(torch.from_numpy(a).cuda(), STAR_TYPES[c]) for c, a in cols.items()}
    before = {c: v.tensor for c, v in tg.items()}
    assert try_fused(True, tg, ops, copy.deepcopy(args), 0) == 0
    assert set(tg) == set(before) and all(tg[c].tensor is before[c] for c in tg)
