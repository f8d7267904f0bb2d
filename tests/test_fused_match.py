"""try_fused's plan-shape matcher on the CPU: the filtered join + aggregate + top-k run of
operators is recognised, and variants it does not cover are left to the operators."""
import copy

import numpy as np
import pytest
import torch

from tqpk.operators.fused import _match_join_agg_topk, try_fused
from tqpk.variable import Variable


def plan():
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
        7: {"name": "take ordered", "limit": 10, "input ids": [11, 302], "key ids": [302], "key orders": [True]},
    }
    tg = {11: Variable(torch.arange(1, 9, dtype=torch.int32), "int"), 12: Variable(torch.zeros(8, dtype=torch.int32), "date"),
          21: Variable(torch.ones(20, dtype=torch.int32), "int"), 22: Variable(torch.zeros(20, dtype=torch.int32), "date"),
          23: Variable(torch.ones(20, dtype=torch.float64), "float"), 24: Variable(torch.zeros(20, dtype=torch.float64), "float")}
    return tg, ops, args


def test_recognises_the_filtered_join_aggregate_topk_run():
    tg, ops, args = plan()
    m = _match_join_agg_topk(tg, ops, args, 0)
    assert m is not None and m["n_ops"] == 5
    assert (m["bk"], m["pk"], m["k"], m["desc"], m["key_out"], m["agg_out"]) == (11, 21, 10, True, 11, 302)
    assert set(m["filters"]) == {"b", "p"} and m["vcols"] == [23, 24]


def test_recognises_it_without_filters_and_from_a_later_position():
    tg, ops, args = plan()
    a = copy.deepcopy(args)
    a[5]["mask map"] = {}
    m = _match_join_agg_topk(tg, [5, 6, 7], a, 0)
    assert m is not None and m["n_ops"] == 3 and m["filters"] == {}
    with_scan = dict(args)
    with_scan[1] = {"name": "Scan"}
    assert _match_join_agg_topk(tg, [1] + ops, with_scan, 1)["n_ops"] == 5


@pytest.mark.parametrize("change", [
    lambda a: a[5].update({"join type": "LeftSemi"}),
    lambda a: a[5].update({"join condition": ["x"]}),
    lambda a: a[5].update({"left keys": [11, 12], "right keys": [21, 22]}),
    lambda a: a[6].update({"keys": ["k#11", "d#12"]}),
    lambda a: a[6]["results"].append([[["count", ["1"]], "#", "9"], "AS", "c#303"]),
    lambda a: a[6]["results"].__setitem__(1, [[["max", [["p#23"]]], "#", "301"], "AS", "rev#302"]),
    lambda a: a[7].update({"limit": 300}),
    lambda a: a[7].update({"key ids": [11]}),
    lambda a: a[5]["mask map"].update({23: 999}),
    lambda a: a[3].update({"materialized in": [22]}),
    lambda a: a[6].update({"mask map": {23: 902}}),
])
def test_other_shapes_are_left_to_the_operators(change):
    tg, ops, args = plan()
    a = copy.deepcopy(args)
    change(a)
    assert _match_join_agg_topk(tg, ops, a, 0) is None


def test_float_build_keys_and_cpu_columns_run_nothing():
    tg, ops, args = plan()
    tg[11] = Variable(tg[11].tensor.double(), "float")
    assert _match_join_agg_topk(tg, ops, args, 0) is None
    tg, ops, args = plan()
    assert try_fused(True, tg, ops, args, 0) == 0          # CPU tensors: the operators run
    assert try_fused(False, tg, ops, args, 0) == 0


def star_plan():
    """The star query as the plan executor holds it: Filter(A), three joins, Aggregate by the C
    key (sum and count), take ordered."""
    ops = [3, 4, 5, 6, 7, 8]
    args = {
        3: {"name": "Filter", "filter tree": [["cat#32", "=", "1"]], "materialized in": [32], "out mask id": 901},
        4: {"name": "Join", "left keys": [31], "right keys": [41], "join type": "Inner", "left group": [31, 32],
            "right group": [41, 42, 43, 44], "materialized in": [31, 41, 42, 43, 44], "mask map": {31: 901}},
        5: {"name": "Join", "left keys": [51], "right keys": [42], "join type": "Inner", "left group": [51, 52],
            "right group": [31, 41, 42, 43, 44], "materialized in": [51, 52, 42, 43, 44]},
        6: {"name": "Join", "left keys": [61], "right keys": [52], "join type": "Inner", "left group": [61],
            "right group": [51, 52, 42, 43, 44], "materialized in": [61, 52, 43, 44]},
        7: {"name": "Aggregate", "is partial": False, "keys": ["c#61"], "input ids": [61, 43, 44],
            "results": ["c#61", [[["sum", [["p#43", "*", ["1.0", "-", "d#44"]]]], "#", "71"], "AS", "rev#72"],
                        [[["count", ["1"]], "#", "73L"], "AS", "cnt#74"]], "out agg ids": [72, 74]},
        8: {"name": "take ordered", "limit": 100, "input ids": [61, 72, 74], "key ids": [72], "key orders": [True]},
    }
    i32 = lambda n: Variable(torch.arange(1, n + 1, dtype=torch.int32), "int")  # noqa: E731
    tg = {31: i32(8), 32: Variable(torch.ones(8, dtype=torch.uint8), "int"), 41: i32(20), 42: i32(20),
          43: Variable(torch.ones(20, dtype=torch.float64), "float"),
          44: Variable(torch.zeros(20, dtype=torch.float64), "float"), 51: i32(10), 52: i32(10), 61: i32(5)}
    return tg, ops, args


def test_recognises_the_star_plan():
    from tqpk.operators.fused import _match_star_agg_topk
    tg, ops, args = star_plan()
    assert _match_join_agg_topk(tg, ops, args, 0) is None
    m = _match_star_agg_topk(tg, ops, args, 0)
    assert m is not None and m["n_ops"] == 6
    assert m["keys"] == (31, 41, 51, 42, 61, 52) and set(m["filters"]) == {"a"}
    assert (m["k"], m["desc"], m["key_out"], m["agg_out"], m["cnt_out"], m["vcols"]) == (100, True, 61, 72, 74, [43, 44])
    a = copy.deepcopy(args)                       # without the count
    a[7]["results"].pop()
    a[7]["out agg ids"] = [72]
    a[8]["input ids"] = [61, 72]
    m = _match_star_agg_topk(tg, ops, a, 0)
    assert m is not None and m["cnt_out"] is None


@pytest.mark.parametrize("change", [
    lambda a: a[5].update({"right keys": [31]}),          # B joined on A's key, not a fact column
    lambda a: a[6].update({"right keys": [42]}),          # C joined on a fact column, not B's
    lambda a: a[6].update({"join type": "LeftOuter"}),
    lambda a: a[5].update({"mask map": {51: 901}}),
    lambda a: a[7].update({"keys": ["b#51"]}),
    lambda a: a[7]["results"].append([[["sum", ["p#43"]], "#", "75"], "AS", "s#76"]),
    lambda a: a[7]["results"].__setitem__(1, [[["sum", ["b#52"]], "#", "71"], "AS", "rev#72"]),
    lambda a: a[8].update({"input ids": [61, 72]}),
    lambda a: a[8].update({"limit": 1000}),
    lambda a: a[3].update({"materialized in": [43]}),
])
def test_other_star_shapes_are_left_to_the_operators(change):
    from tqpk.operators.fused import _match_star_agg_topk
    tg, ops, args = star_plan()
    a = copy.deepcopy(args)
    change(a)
    assert _match_star_agg_topk(tg, ops, a, 0) is None
