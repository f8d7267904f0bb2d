"""Serving loop on the GPU: every request's result is the same alone and in the mix,
and matches the oracle on the same resident tables."""
import copy
import dataclasses

import numpy as np
import pytest
import torch

from golden_io import assert_f64_close
from oracle import tqp_oracle as O

pytestmark = pytest.mark.gpu

SIZES = dict(n_fact=1_200_000, n_build=150_000, n_a=200_000, n_b=900_000, n_c=120_000, seed=4)


@pytest.fixture(scope="module")
def served():
    from tqpk import build
    build.build()
    from tqpk.serve import DeviceArena, GpuExecutor, ResidentTables
    tables = ResidentTables(torch.device("cuda", 0), **SIZES)
    ex = GpuExecutor(tables, slots=6)
    arena = DeviceArena(150 << 30, tables.nbytes, torch.device("cuda", 0), slab_cap=1 << 30)
    return tables, ex, arena


def _same(a, b, shape):
    if shape == "filter_groupby":
        assert a["groups"] == b["groups"]
        for x, y in zip(a["keys"], b["keys"]):
            np.testing.assert_array_equal(x, y)
        for o in a["outs"]:
            if a["outs"][o].dtype == np.float64:
                assert_f64_close(a["outs"][o], b["outs"][o])
            else:
                np.testing.assert_array_equal(a["outs"][o], b["outs"][o])
    else:
        assert a["groups"] == b["groups"]
        np.testing.assert_array_equal(a["keys"], b["keys"])
        assert_f64_close(a["vals"], b["vals"])
        if shape == "star":
            np.testing.assert_array_equal(a["counts"], b["counts"])


def test_results_alone_equal_results_in_the_mix(served):
    from tqpk.serve import Scheduler, poisson_trace
    tables, ex, arena = served
    trace = poisson_trace(36, 20_000.0, SIZES["n_fact"], min_rows=50_000, seed=9)   # arrivals 50 us apart
    sched = Scheduler(ex, arena, slots=6)
    mixed = {c.req.rid: c for c in sched.run(trace)}
    assert sched.max_inflight > 1, "requests never overlapped"
    assert arena.ff.used_bytes == 0
    for req in trace:
        alone = Scheduler(ex, arena, slots=1).run([dataclasses.replace(req, arrival=0.0)])[0]
        _same(alone.result, mixed[req.rid].result, req.shape)


def _np_tables():
    from tqpk import datagen
    s = SIZES["seed"]
    li = datagen.lineitem(SIZES["n_fact"], seed=s + 1)
    jt = datagen.join_tables(SIZES["n_build"], SIZES["n_fact"], seed=s + 2)
    st = datagen.star_tables(SIZES["n_fact"], SIZES["n_a"], SIZES["n_b"], SIZES["n_c"], seed=s + 3)
    return li, jt, st


def test_served_results_match_the_oracle(served):
    from tqpk.serve import LINEITEM_AGG, LINEITEM_IDS, Request, Scheduler
    import bench
    tables, ex, arena = served
    li, jt, st = _np_tables()
    reqs = [Request(0, "filter_groupby", 700_001, (2300,), 0.0), Request(1, "join", 900_003, (1000, 1500), 0.0),
            Request(2, "star", 1_100_000, (3,), 0.0)]
    got = {c.req.rid: c.result for c in Scheduler(ex, arena, slots=3).run(reqs)}
    # filter + group-by over the first 700,001 rows
    n = 700_001
    cols = {LINEITEM_IDS[k]: v[:n] for k, v in li.items()}
    cols[900] = cols[7] <= 2300
    args = dict(copy.deepcopy(LINEITEM_AGG), **{"mask map": {c: 900 for c in range(1, 7)}})
    ref = O.tqp_hash_aggregate(cols, args)
    g = got[0]
    np.testing.assert_array_equal(g["keys"][0], ref[5].reshape(-1))
    np.testing.assert_array_equal(g["keys"][1], ref[6].reshape(-1))
    for a in LINEITEM_AGG["out agg ids"]:
        (assert_f64_close if ref[a].dtype == np.float64 else np.testing.assert_array_equal)(g["outs"][a], ref[a])
    # join: probe prefix of 900,003 rows, probe date > 1000, build date < 1500, top 10
    n = 900_003
    oc = {11: jt["b_key"], 12: jt["b_date"], 21: jt["p_fk"][:n], 22: jt["p_date"][:n], 23: jt["p_price"][:n],
          24: jt["p_discount"][:n]}
    oc[901] = oc[12] < 1500
    oc[902] = oc[22] > 1000
    res, _ = O.join_vortex(oc, {"left group": [11, 12], "right group": [21, 22, 23, 24],
                                "materialized in": [11, 21, 23, 24],
                                "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}, 11, 21, "inner")
    agg = O.tqp_hash_aggregate(res, {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
                                     "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "1"],
                                                          "AS", "r#302"]], "out agg ids": [302]})
    top = O.tqp_sort({11: agg[11], 302: agg[302]}, {"limit": 10, "input ids": [11, 302], "key ids": [302],
                                                    "key orders": [True]}, True)
    assert got[1]["groups"] == agg[11].shape[0]
    np.testing.assert_array_equal(got[1]["keys"], top[11].reshape(-1))
    assert_f64_close(got[1]["vals"], top[302])
    # star: fact prefix of 1,100,000 rows, A category == 3, top 100
    n = 1_100_000
    w = bench.StarJoin(scale=0.0001)
    w.fa = dict(w.fa, **{"filter tree": [["cat#32", "=", "3"]]})
    cols = {31: st["a_key"], 32: st["a_cat"], 41: st["f_fka"][:n], 42: st["f_fkb"][:n], 43: st["f_price"][:n],
            44: st["f_discount"][:n], 51: st["b_key"], 52: st["b_fkc"], 61: st["c_key"]}
    ek, ev, ec = w.oracle(cols)
    np.testing.assert_array_equal(got[2]["keys"], ek)
    assert_f64_close(got[2]["vals"], ev)
    np.testing.assert_array_equal(got[2]["counts"], ec)


def test_empty_prefix_requests(served):
    from tqpk.serve import Request, Scheduler
    tables, ex, arena = served
    reqs = [Request(0, "filter_groupby", 0, (2300,), 0.0), Request(1, "join", 0, (1000, 1500), 0.0),
            Request(2, "star", 0, (3,), 0.0)]
    got = {c.req.rid: c.result for c in Scheduler(ex, arena, slots=3).run(reqs)}
    assert got[0]["groups"] == 0 and got[1]["groups"] == 0 and got[2]["groups"] == 0
    assert len(got[1]["keys"]) == 0 and len(got[2]["keys"]) == 0
