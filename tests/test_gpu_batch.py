"""Batched persistent-launch execution of uneven instances against the oracle."""
import copy

import numpy as np
import pytest
import torch

from golden_io import assert_f64_close
from oracle import tqp_oracle as O

pytestmark = pytest.mark.gpu

AGG_RESULTS = [
    "flag#5", "status#6",
    [[["sum", ["quantity#1"]], "#", "101"], "AS", "a#201"],
    [[["sum", [["price#2", "*", ["1.0", "-", "discount#3"]]]], "#", "103"], "AS", "c#203"],
    [[["sum", [[["price#2", "*", ["1.0", "-", "discount#3"]], "*", ["1.0", "+", "tax#4"]]]], "#", "104"], "AS", "d#204"],
    [[["avg", ["discount#3"]], "#", "107"], "AS", "g#207"],
    [[["min", ["price#2"]], "#", "109"], "AS", "m#209"],
    [[["count", ["1"]], "#", "108L"], "AS", "h#208"]]
AGG_IDS = [201, 203, 204, 207, 209, 208]
FILTER = [["ship_date#7", "<=", "2470"]]


@pytest.fixture(scope="module", autouse=True)
def lib():
    from tqpk import build, _lib
    build.build()
    return _lib.load()


def make_groupby(rows, groups, seed):
    from tqpk import datagen
    from tqpk.batch import GroupByInstance
    t, (a, b) = datagen.groupby_instance_tables(rows, groups, seed)
    ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
    cols = {ids[k]: v for k, v in t.items()}
    d = {c: torch.from_numpy(x).cuda() for c, x in cols.items()}
    args = {"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 3, 4, 5, 6],
            "results": AGG_RESULTS, "out agg ids": AGG_IDS}
    inst = GroupByInstance(args=args, columns={c: d[c] for c in (1, 2, 3, 4, 5, 6)}, filter_tree=FILTER,
                           filter_cols={7: d[7]}, key_domains=[(0, a - 1), (0, b - 1)])
    oc = dict(cols)
    oc[900] = O.eval_filter(FILTER, {7: cols[7]})
    oargs = dict(copy.deepcopy(args), **{"mask map": {c: 900 for c in (1, 2, 3, 4, 5, 6)}})
    return inst, O.tqp_hash_aggregate(oc, oargs)


def make_join(rows, groups, seed, k=10):
    from tqpk import datagen
    from tqpk.batch import JoinInstance
    t = datagen.join_tables(groups, rows, seed)
    d = {c: torch.from_numpy(x).cuda() for c, x in t.items()}
    inst = JoinInstance(d["b_key"], (1, groups), d["p_fk"], {12: d["b_date"]}, [["bd#12", "<", "1170"]],
                        {22: d["p_date"], 23: d["p_price"], 24: d["p_discount"]}, [["pd#22", ">", "1170"]],
                        [["p#23", "*", ["1.0", "-", "d#24"]]], k=k)
    cols = {11: t["b_key"], 12: t["b_date"], 21: t["p_fk"], 22: t["p_date"], 23: t["p_price"], 24: t["p_discount"]}
    oc = dict(cols)
    oc[901] = O.eval_filter([["bd#12", "<", "1170"]], {12: cols[12]})
    oc[902] = O.eval_filter([["pd#22", ">", "1170"]], {22: cols[22]})
    jargs = {"left group": [11, 12], "right group": [21, 22, 23, 24], "materialized in": [11, 21, 23, 24],
             "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}
    res, _ = O.join_vortex(oc, jargs, 11, 21, "inner")
    agg = O.tqp_hash_aggregate(res, {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
                                     "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "1"],
                                                          "AS", "r#302"]], "out agg ids": [302]})
    top = O.tqp_sort({11: agg[11], 302: agg[302]}, {"limit": k, "input ids": [11, 302], "key ids": [302],
                                                    "key orders": [True]}, True)
    return inst, (top[11].reshape(-1), top[302], agg[11].shape[0])


def check(results, expected):
    for (kind, exp), got in zip(expected, results):
        if kind == "join":
            keys, vals, groups = got
            ek, ev, eg = exp
            np.testing.assert_array_equal(keys, ek)
            assert_f64_close(vals, ev)
            assert groups == eg
        else:
            outs, keys, g = got
            np.testing.assert_array_equal(keys[0], exp[5].reshape(-1))
            np.testing.assert_array_equal(keys[1], exp[6].reshape(-1))
            for oid in AGG_IDS:
                e = exp[oid]
                (assert_f64_close if e.dtype == np.float64 else np.testing.assert_array_equal)(outs[oid], e)


def batch_class(impl):
    if impl == "library":
        from tqpk.batch import Batch
        return Batch
    from tqpk.jitbatch import QueryBatch
    return QueryBatch


@pytest.mark.parametrize("impl", ["library", "generated"])
def test_batch_uneven_instances_vs_oracle(impl):
    Batch = batch_class(impl)
    shapes = [("groupby", 1000, 4), ("join", 5000, 300), ("groupby", 250_000, 5000), ("join", 300_000, 20_000),
              ("groupby", 40_000, 60), ("join", 1000, 7), ("groupby", 3, 2), ("join", 120_000, 100_000),
              ("groupby", 700_001, 1), ("join", 64, 1000), ("groupby", 90_000, 40_000), ("join", 2_000_000, 500)]
    insts, expected = [], []
    for i, (kind, rows, g) in enumerate(shapes):
        inst, exp = (make_groupby if kind == "groupby" else make_join)(rows, g, 100 + i)
        insts.append(inst)
        expected.append((kind, exp))
    b = Batch(insts)
    b.run()
    check(b.results(), expected)
    b.capture()
    for _ in range(2):                          # graph replays give the same results
        b.replay()
        check(b.results(), expected)
    if hasattr(b, "results_host"):              # the two-read form returns the same rows
        res, nbytes = b.results_host()
        check(res, expected)
        assert nbytes > 0


@pytest.mark.parametrize("impl", ["library", "generated"])
def test_batch_item_sizes_do_not_change_results(impl):
    from tqpk.batch import Autotuner
    Batch = batch_class(impl)
    insts, expected = [], []
    for i, (kind, rows, g) in enumerate([("groupby", 300_000, 12), ("join", 400_000, 50_000)]):
        inst, exp = (make_groupby if kind == "groupby" else make_join)(rows, g, 7 + i)
        insts.append(inst)
        expected.append((kind, exp))
    for rpi in (4096, 65536, 1 << 20):
        tuner = Autotuner({f"{k}:{c}": rpi for k in ("groupby", "join_build", "join_probe") for c in range(30)})
        b = Batch(insts, tuner)
        b.run()
        check(b.results(), expected)


def test_generated_batch_table_modes_and_empty_instances():
    """Group tables of every placement (per thread, several shared copies, one per CTA, global), join
    sums of every placement (per thread, shared copies, global) and instances with no rows, in one
    generated batch."""
    from tqpk.jitbatch import QueryBatch, _mode
    shapes = [("groupby", 200_000, 2), ("groupby", 200_000, 150), ("groupby", 200_000, 500),
              ("groupby", 200_000, 30_000), ("groupby", 0, 9), ("join", 0, 100), ("join", 50_000, 1),
              ("join", 300_000, 40), ("join", 300_000, 500), ("join", 100_000, 60_000)]
    insts, expected = [], []
    for i, (kind, rows, g) in enumerate(shapes):
        inst, exp = (make_groupby if kind == "groupby" else make_join)(rows, g, 300 + i)
        insts.append(inst)
        expected.append((kind, exp))
    b = QueryBatch(insts)
    placements = {(int(b.recs[i].mode), int(b.recs[i].copies)) for i, (kind, _, _) in enumerate(shapes)
                  if kind == "groupby"}
    assert (1, 256) in placements and (2, 1) in placements and (4, 1) in placements
    assert any(m == 2 and 1 < c < 256 for m, c in placements)
    join_modes = {int(b.recs[i].mode) for i, (kind, rows, _) in enumerate(shapes) if kind == "join" and rows}
    assert join_modes == {0, 1, 2}
    b.run()
    check(b.results(), expected)


def test_generated_batch_dependency_wait_times_out():
    """A phase whose predecessor count can never be reached (one phase-0 item more than
    the queue holds): the bounded wait gives up, the kernel still finishes every item and
    the host reads TQPK_ETIMEOUT from the control block."""
    from tqpk.jitbatch import QueryBatch
    inst, _ = make_groupby(50_000, 12, 901)
    b = QueryBatch([inst])
    b.recs[0].ni[0] += 1
    b.d_recs.copy_(torch.frombuffer(bytearray(bytes(b.recs)), dtype=torch.uint8))
    b.run()
    torch.cuda.synchronize()
    with pytest.raises(TimeoutError):
        b.check_error()


def test_generated_batch_key_outside_its_domain_is_reported():
    """A group key outside the instance's declared key domain: the row is skipped (no table write
    past the domain) and the batch reports TQPK_EINVAL (ValueError)."""
    from tqpk.batch import GroupByInstance
    from tqpk.jitbatch import QueryBatch
    inst, _ = make_groupby(50_000, 150, 401)
    (a0, a1), (b0, b1) = inst.key_domains
    narrow = GroupByInstance(args=inst.args, columns=inst.columns, filter_tree=inst.filter_tree,
                             filter_cols=inst.filter_cols, key_domains=[(a0, a1 - 1), (b0, b1)])
    b = QueryBatch([narrow])
    b.run()
    with pytest.raises(ValueError):
        b.results()
