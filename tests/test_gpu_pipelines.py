"""GPU parity of the fused pipelines against the oracle's operator sequence.

Keys and order bit-exact, float64 sums within 1e-12 relative."""
import copy

import numpy as np
import pytest
import torch

from golden_io import assert_f64_close
from oracle import tqp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    from tqpk import build, _lib
    build.build()
    return _lib.load()


def _oracle_join(cols, f1, f2, k):
    jargs = {"left group": [11, 12], "right group": [21, 22, 23, 24], "materialized in": [11, 21, 23, 24],
             "mask map": {11: 901, 21: 902, 23: 902, 24: 902}}
    aargs = {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
             "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "1"], "AS", "r#302"]],
             "out agg ids": [302]}
    oc = dict(cols)
    oc[901] = O.eval_filter(f1, {12: cols[12]}) if f1 else np.ones(cols[11].size, bool)
    oc[902] = O.eval_filter(f2, {22: cols[22]}) if f2 else np.ones(cols[21].size, bool)
    res, _ = O.join_vortex(oc, jargs, 11, 21, "inner")
    agg = O.tqp_hash_aggregate(res, aargs)
    top = O.tqp_sort({11: agg[11], 302: agg[302]}, {"limit": k, "input ids": [11, 302], "key ids": [302],
                                                    "key orders": [True]}, True)
    return top[11].reshape(-1), top[302], agg[11].shape[0]


@pytest.mark.parametrize("nb,np_rows,k,offset,dtype,filters", [
    (100_000, 400_000, 10, 0, np.int32, True),
    (3_000, 20_000, 200, 1_000_000, np.int64, True),
    (50, 300, 256, -20, np.int32, False),
    (1, 10, 10, 5, np.int64, True),
    (20_000, 0, 10, 0, np.int32, True),
])
def test_join_pipeline_vs_oracle(nb, np_rows, k, offset, dtype, filters):
    from tqpk.pipeline import JoinAggTopK
    rng = np.random.default_rng(nb + np_rows)
    cols = {11: (rng.permutation(nb) + 1 + offset).astype(dtype), 12: rng.integers(0, 2557, nb).astype(np.int32),
            21: (rng.integers(1, nb + 3, np_rows) + offset).astype(dtype), 22: rng.integers(0, 2557, np_rows).astype(np.int32),
            23: rng.integers(90000, 10495001, np_rows) / 100.0, 24: rng.integers(0, 11, np_rows) / 100.0}
    f1 = [["bd#12", "<", "1170"]] if filters else None
    f2 = [["pd#22", ">", "1170"]] if filters else None
    d = {c: torch.from_numpy(a).cuda() for c, a in cols.items()}
    p = JoinAggTopK(d[11], int(cols[11].min()), int(cols[11].max()), d[21], {12: d[12]}, f1,
                    {22: d[22], 23: d[23], 24: d[24]}, f2, [["p#23", "*", ["1.0", "-", "d#24"]]], k=k)
    for _ in range(2):              # reruns reuse the workspace
        p.run()
        keys, vals, groups = p.result()
    ek, ev, eg = _oracle_join(cols, f1, f2, k)
    assert groups == eg
    np.testing.assert_array_equal(keys, ek)
    assert_f64_close(vals, ev)


@pytest.mark.parametrize("tma", ["1", "0"])
@pytest.mark.parametrize("nb,np_rows,dtype", [(100_000, 1_000_003, np.int32), (5_000, 2048, np.int32),
                                              (70_000, 1_048_575, np.int64), (2_000, 1024, np.int64),
                                              (9_000, 1023, np.int32), (300, 128, np.int32), (300, 127, np.int32),
                                              (40_000, 9_000_001, np.int32)])
def test_join_probe_staged_and_plain_paths(monkeypatch, tma, nb, np_rows, dtype):
    """The TMA-staged probe (full 128-row chunks + a plain-load tail) and the register
    probe give the oracle's result, with and without a whole number of chunks."""
    monkeypatch.setenv("TQPK_TMA", tma)
    from tqpk.pipeline import JoinAggTopK
    rng = np.random.default_rng(nb ^ np_rows)
    cols = {11: (rng.permutation(nb) + 1).astype(dtype), 12: rng.integers(0, 2557, nb).astype(np.int32),
            21: rng.integers(1, nb + 3, np_rows).astype(dtype), 22: rng.integers(0, 2557, np_rows).astype(np.int32),
            23: rng.integers(90000, 10495001, np_rows) / 100.0, 24: rng.integers(0, 11, np_rows) / 100.0}
    f1, f2 = [["bd#12", "<", "1170"]], [["pd#22", ">", "1170"]]
    d = {c: torch.from_numpy(a).cuda() for c, a in cols.items()}
    p = JoinAggTopK(d[11], 1, nb, d[21], {12: d[12]}, f1, {22: d[22], 23: d[23], 24: d[24]}, f2,
                    [["p#23", "*", ["1.0", "-", "d#24"]]], k=10)
    p.run()
    keys, vals, groups = p.result()
    from tqpk import jit
    assert bool(getattr(p, "_probe_smem", 0)) == (tma == "1" and np_rows >= jit.TMA_ROWS)
    ek, ev, eg = _oracle_join(cols, f1, f2, 10)
    assert groups == eg
    np.testing.assert_array_equal(keys, ek)
    assert_f64_close(vals, ev)


@pytest.mark.parametrize("bits", [True, False])
@pytest.mark.parametrize("nb,np_rows", [(1_500_000, 2_000_003), (33, 1000), (100_001, 777)])
def test_join_probe_bitmap_and_row_directory(monkeypatch, bits, nb, np_rows):
    """The generated probe over the build side's membership bitmap (the default while it fits
    256 KB) and over its row directory give the oracle's groups, with build keys missing from
    the key domain and a domain size that is not a multiple of 32."""
    from tqpk import pipeline as P
    monkeypatch.setattr(P, "JOIN_DIR_BITS", bits)
    rng = np.random.default_rng(nb)
    keys = rng.permutation(nb + nb // 3)[:nb] + 7
    cols = {11: keys.astype(np.int32), 12: rng.integers(0, 2557, nb).astype(np.int32),
            21: rng.integers(0, nb + nb // 3 + 20, np_rows).astype(np.int32),
            22: rng.integers(0, 2557, np_rows).astype(np.int32),
            23: rng.integers(90000, 10495001, np_rows) / 100.0, 24: rng.integers(0, 11, np_rows) / 100.0}
    f1, f2 = [["bd#12", "<", "1170"]], [["pd#22", ">", "1170"]]
    d = {c: torch.from_numpy(a).cuda() for c, a in cols.items()}
    p = P.JoinAggTopK(d[11], int(cols[11].min()), int(cols[11].max()), d[21], {12: d[12]}, f1,
                      {22: d[22], 23: d[23], 24: d[24]}, f2, [["p#23", "*", ["1.0", "-", "d#24"]]], k=10)
    p.run()
    keys_, vals, groups = p.result()
    assert p._bits == bits
    ek, ev, eg = _oracle_join(cols, f1, f2, 10)
    assert groups == eg
    np.testing.assert_array_equal(keys_, ek)
    assert_f64_close(vals, ev)


def test_join_pipeline_zero_sums_still_count_as_groups():
    """Every value is +0.0 or -0.0, so every matched group sums to zero: the groups are told
    apart from empty slots by occupancy alone (the sums start at -0.0 in the generated path and
    a -0.0 value is added as +0.0), the count of groups and the top-10 (ties by key) match."""
    from tqpk.pipeline import JoinAggTopK
    rng = np.random.default_rng(8)
    nb, np_rows = 5000, 40_000
    cols = {11: (rng.permutation(nb) + 1).astype(np.int32), 12: rng.integers(0, 2557, nb).astype(np.int32),
            21: rng.integers(1, nb + 3, np_rows).astype(np.int32), 22: rng.integers(0, 2557, np_rows).astype(np.int32),
            23: np.where(rng.random(np_rows) < 0.5, -0.0, 0.0), 24: rng.integers(0, 11, np_rows) / 100.0}
    f1, f2 = [["bd#12", "<", "1170"]], [["pd#22", ">", "1170"]]
    d = {c: torch.from_numpy(a).cuda() for c, a in cols.items()}
    p = JoinAggTopK(d[11], 1, nb, d[21], {12: d[12]}, f1, {22: d[22], 23: d[23], 24: d[24]}, f2,
                    [["p#23", "*", ["1.0", "-", "d#24"]]], k=10)
    p.run()
    keys, vals, groups = p.result()
    ek, ev, eg = _oracle_join(cols, f1, f2, 10)
    assert groups == eg
    np.testing.assert_array_equal(keys, ek)
    np.testing.assert_array_equal(vals, ev)
    assert not np.signbit(vals).any()                 # +0.0 sums, as the reference's bincount gives


def test_join_pipeline_repeated_build_key_raises():
    from tqpk.pipeline import JoinAggTopK
    bk = torch.tensor([1, 2, 2, 3], dtype=torch.int32, device="cuda")
    pk = torch.tensor([1, 2, 3], dtype=torch.int32, device="cuda")
    v = torch.ones(3, dtype=torch.float64, device="cuda")
    p = JoinAggTopK(bk, 1, 3, pk, {}, None, {23: v}, None, ["p#23"], k=2)
    p.run()
    with pytest.raises(NotImplementedError):
        p.result()


@pytest.mark.parametrize("jit_on", ["1", "0"])
@pytest.mark.parametrize("scale,k", [(0.05, 100), (0.01, 7), (0.002, 256)])
def test_star_pipeline_vs_oracle(monkeypatch, jit_on, scale, k):
    monkeypatch.setenv("TQPK_JIT", jit_on)
    import bench
    from tqpk.pipeline import StarAggTopK
    w = bench.StarJoin(scale=scale)
    w.targs = dict(w.targs, limit=k)
    ek, ev, ec = w.oracle()
    d = {c: torch.from_numpy(a).cuda() for c, a in w.cols.items()}
    dom = lambda a: (int(a.min()), int(a.max()))  # noqa: E731
    p = StarAggTopK(d[41], d[42], {43: d[43], 44: d[44]}, None, w.value_tree, d[31], {32: d[32]},
                    w.fa["filter tree"], dom(w.cols[31]), d[51], d[52], dom(w.cols[51]), d[61], dom(w.cols[61]), k=k)
    p.run()
    keys, vals, cnts, groups = p.result()
    np.testing.assert_array_equal(keys, ek)
    assert_f64_close(vals, ev)
    np.testing.assert_array_equal(cnts, ec)


@pytest.mark.parametrize("jit_on", ["1", "0"])
def test_star_pipeline_with_missing_dimension_rows(monkeypatch, jit_on):
    """C holds only a third of the keys B points at, and B misses keys the fact table names:
    the composed B -> C directory (generated path) and the three-hop probe (library path)
    drop the same rows as the oracle's joins."""
    monkeypatch.setenv("TQPK_JIT", jit_on)
    import bench
    from tqpk.pipeline import StarAggTopK
    w = bench.StarJoin(scale=0.02)
    rng = np.random.default_rng(3)
    c_keys = w.cols[61]
    w.cols[61] = c_keys[rng.random(c_keys.size) < 0.33]
    b_keep = rng.random(w.cols[51].size) < 0.8
    w.cols[51], w.cols[52] = w.cols[51][b_keep], w.cols[52][b_keep]
    ek, ev, ec = w.oracle()
    d = {c: torch.from_numpy(a).cuda() for c, a in w.cols.items()}
    dom = lambda a: (int(a.min()), int(a.max()))  # noqa: E731
    p = StarAggTopK(d[41], d[42], {43: d[43], 44: d[44]}, None, w.value_tree, d[31], {32: d[32]},
                    w.fa["filter tree"], dom(w.cols[31]), d[51], d[52], dom(w.cols[51]), d[61], dom(w.cols[61]), k=100)
    p.run()
    keys, vals, cnts, groups = p.result()
    np.testing.assert_array_equal(keys, ek)
    assert_f64_close(vals, ev)
    np.testing.assert_array_equal(cnts, ec)


@pytest.mark.parametrize("slots", [1, 31, 32, 33, 1000, 2_000_003])
def test_directory_bits(slots):
    """Bit s of the membership bitmap is set exactly where the directory names a row."""
    from tqpk import _lib as L
    rng = np.random.default_rng(slots)
    d = rng.integers(-2, 50, slots).astype(np.int32)
    d[rng.random(slots) < 0.5] = -1
    dd = torch.from_numpy(d).cuda()
    words = (slots + 31) // 32
    bits = torch.full((words + 1,), -7, dtype=torch.int32, device="cuda")      # one guard word
    L.check(L.load().tqpk_directory_bits(dd.data_ptr(), slots, bits.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream), "tqpk_directory_bits")
    got = bits.cpu().numpy().view(np.uint32)
    assert got[words] == np.uint32(0xFFFFFFF9)                                  # untouched
    want = np.packbits(np.concatenate([d >= 0, np.zeros(words * 32 - slots, bool)]).reshape(-1, 8)[:, ::-1]
                       ).view(np.uint32)
    np.testing.assert_array_equal(got[:words], want)


@pytest.mark.parametrize("a_bits", ["1", "0"])
def test_star_pipeline_a_bitmap_and_row_directory_agree(monkeypatch, a_bits):
    """The generated star probe gives the oracle's result with A's membership bitmap and
    with A's row directory, A having keys missing from its domain and a domain size
    that is not a multiple of 32."""
    monkeypatch.setenv("TQPK_JIT", "1")
    monkeypatch.setenv("TQPK_STAR_ABITS", a_bits)
    import bench
    from tqpk.pipeline import StarAggTopK
    w = bench.StarJoin(scale=0.01)
    rng = np.random.default_rng(11)
    keep = rng.random(w.cols[31].size) < 0.7
    w.cols[31], w.cols[32] = w.cols[31][keep], w.cols[32][keep]
    w.cols[31][-1] = int(w.cols[31].max()) + 45                  # the domain's last word half used
    ek, ev, ec = w.oracle()
    d = {c: torch.from_numpy(a).cuda() for c, a in w.cols.items()}
    dom = lambda a: (int(a.min()), int(a.max()))  # noqa: E731
    p = StarAggTopK(d[41], d[42], {43: d[43], 44: d[44]}, None, w.value_tree, d[31], {32: d[32]},
                    w.fa["filter tree"], dom(w.cols[31]), d[51], d[52], dom(w.cols[51]), d[61], dom(w.cols[61]), k=100)
    p.run()
    keys, vals, cnts, groups = p.result()
    assert p._a_bits == (a_bits == "1")
    np.testing.assert_array_equal(keys, ek)
    assert_f64_close(vals, ev)
    np.testing.assert_array_equal(cnts, ec)


@pytest.mark.parametrize("k", [200, 256, 257, 1000])
def test_topk_stable_large_k(k):
    from tqpk.ops import topk_stable
    rng = np.random.default_rng(k)
    x = rng.integers(-1000, 1000, 300_001).astype(np.int64)
    got = topk_stable(torch.from_numpy(x).cuda(), k, True).cpu().numpy()
    np.testing.assert_array_equal(got, O._stable_order(x, True)[:k])


@pytest.mark.parametrize("n,k,hi", [(100_003, 10, 1), (200_000, 100, 3), (5_000_000, 256, 1 << 40),
                                    (3, 10, 5), (0, 10, 5), (4097, 1, 2)])
@pytest.mark.parametrize("desc", [True, False])
def test_topk_threshold_path_and_tie_fallback(n, k, hi, desc):
    """Few distinct values put more items under the cut than the candidate list holds
    (the warp-list fallback runs); many distinct values take the sorted-candidates path."""
    from tqpk.ops import topk_stable
    rng = np.random.default_rng(n + k)
    x = rng.integers(0, hi, n).astype(np.int64)
    got = topk_stable(torch.from_numpy(x).cuda(), k, desc).cpu().numpy()
    np.testing.assert_array_equal(got, O._stable_order(x, desc)[:k])


@pytest.mark.parametrize("repeat", [False, True])
@pytest.mark.parametrize("n,slots", [(15_000, 20_011), (1_000_003, 1_000_003), (5, 7)])
def test_directory_build_next_matches_build_then_compose(repeat, n, slots):
    """tqpk_directory_build_next (composition with the next directory while building) writes
    the same directory as tqpk_directory_build + tqpk_directory_compose, and reports a
    repeated key the same way."""
    import ctypes as C
    from tqpk import _lib as L
    from tqpk.predicate import compile_filter
    lib = L.load()
    rng = np.random.default_rng(n + int(repeat))
    keys = (rng.permutation(slots)[:n] + 3).astype(np.int32)
    if repeat and n > 1:
        keys[-1] = keys[0]
    nxt_slots = 997
    payload = rng.integers(-5, nxt_slots + 10, n).astype(np.int32)
    cat = rng.integers(0, 3, n).astype(np.int32)
    nxt = np.where(rng.random(nxt_slots) < 0.6, np.arange(nxt_slots), -1).astype(np.int32)
    d = {k: torch.from_numpy(v).cuda() for k, v in (("k", keys), ("p", payload), ("c", cat), ("x", nxt))}
    pred = compile_filter([["c#1", "<", "2"]], {1: d["c"]})
    s = torch.cuda.current_stream().cuda_stream
    INT_MIN = -(1 << 31)
    a = torch.empty(slots, dtype=torch.int32, device="cuda")
    b = torch.empty(slots, dtype=torch.int32, device="cuda")
    err = torch.zeros(2, dtype=torch.int32, device="cuda")
    L.check(lib.tqpk_directory_build(d["k"].data_ptr(), L.I32, n, C.byref(pred.struct), d["p"].data_ptr(), L.I32, 3,
                                     slots, INT_MIN, INT_MIN + 1, a.data_ptr(), err.data_ptr(), s), "build")
    L.check(lib.tqpk_directory_compose(a.data_ptr(), slots, d["x"].data_ptr(), 0, nxt_slots, INT_MIN, INT_MIN + 1, s),
            "compose")
    L.check(lib.tqpk_directory_build_next(d["k"].data_ptr(), L.I32, n, C.byref(pred.struct), d["p"].data_ptr(), L.I32,
                                          3, slots, INT_MIN, INT_MIN + 1, d["x"].data_ptr(), 0, nxt_slots,
                                          b.data_ptr(), err.data_ptr() + 4, s), "build_next")
    e = err.cpu().numpy()
    assert (e[0] == L.EUNSUPPORTED) == (repeat and n > 1)
    assert e[1] == e[0]
    if not (repeat and n > 1):
        np.testing.assert_array_equal(b.cpu().numpy(), a.cpu().numpy())


@pytest.mark.parametrize("ties", [1500, 3000, 5000])
@pytest.mark.parametrize("desc", [True, False])
def test_topk_tied_candidates_around_the_sort_capacity(ties, desc):
    """A block of equal best keys puts `ties` items under the cut: up to 2048 the last filter
    CTA sorts them in shared memory, above that it takes the warp lists; both keep the
    stable order (smaller position first among equal keys)."""
    from tqpk.ops import topk_stable
    rng = np.random.default_rng(ties)
    n = 300_007
    x = rng.integers(1000, 1 << 40, n).astype(np.int64)
    x[rng.choice(n, ties, replace=False)] = (1 << 41) if desc else 5
    for k in (10, 100):
        got = topk_stable(torch.from_numpy(x).cuda(), k, desc).cpu().numpy()
        np.testing.assert_array_equal(got, O._stable_order(x, desc)[:k])


@pytest.mark.parametrize("n,groups", [(1_000_003, 6), (200_000, 1400), (50_000, 30_000), (3, 4)])
def test_groupby_pipeline_domains_and_graph_replay(n, groups):
    """Filter + group-by over table-statistic key domains, no host synchronisation inside;
    graph replays give the oracle's groups in key order."""
    from tqpk import datagen
    from tqpk.pipeline import GroupByPipeline
    t, (a, b) = datagen.groupby_instance_tables(n, groups, 17)
    ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
    cols = {ids[k]: v for k, v in t.items()}
    d = {c: torch.from_numpy(x).cuda() for c, x in cols.items()}
    results = ["flag#5", "status#6", [[["sum", [["price#2", "*", ["1.0", "-", "discount#3"]]]], "#", "1"], "AS", "c#203"],
               [[["avg", ["discount#3"]], "#", "2"], "AS", "g#207"], [[["min", ["price#2"]], "#", "3"], "AS", "m#209"],
               [[["count", ["1"]], "#", "4L"], "AS", "h#208"]]
    args = {"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 3, 4, 5, 6], "results": results,
            "out agg ids": [203, 207, 209, 208]}
    tree = [["ship_date#7", "<=", "2000"]]
    p = GroupByPipeline(args, {c: d[c] for c in range(1, 7)}, tree, {7: d[7]}, [(0, a - 1), (0, b - 1)])
    oc = dict(cols)
    oc[900] = O.eval_filter(tree, {7: cols[7]})
    ref = O.tqp_hash_aggregate(oc, dict(copy.deepcopy(args), **{"mask map": {c: 900 for c in range(1, 7)}}))
    p.capture()
    for _ in range(2):
        p.replay()
        keys, outs, G = p.result()
        np.testing.assert_array_equal(keys[0].cpu().numpy(), ref[5].reshape(-1))
        np.testing.assert_array_equal(keys[1].cpu().numpy(), ref[6].reshape(-1))
        for oid in args["out agg ids"]:
            e = ref[oid]
            (assert_f64_close if e.dtype == np.float64 else np.testing.assert_array_equal)(outs[oid].cpu().numpy(), e)


def test_groupby_pipeline_key_outside_declared_domain_raises():
    """GroupByPipeline's key domains are table statistics given by the caller: a key outside them is
    not written past the table; result() raises ValueError (TQPK_EINVAL)."""
    from tqpk import datagen
    from tqpk.pipeline import GroupByPipeline
    t, (a, b) = datagen.groupby_instance_tables(100_000, 40, 5)
    ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
    d = {ids[k]: torch.from_numpy(v).cuda() for k, v in t.items()}
    args = {"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 5, 6],
            "results": ["flag#5", "status#6", [[["sum", ["quantity#1"]], "#", "1"], "AS", "q#101"]],
            "out agg ids": [101]}
    p = GroupByPipeline(args, {c: d[c] for c in (1, 2, 5, 6)}, None, {}, [(0, a - 2), (0, b - 1)])
    p.run()
    with pytest.raises(ValueError):
        p.result()
