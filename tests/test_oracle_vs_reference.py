"""The oracle against the reference's own operators on seeded random inputs (CPU).

The golden fixtures pin the oracle on fixed cases.  Here the compiled reference (oracle/_ref, its
CPU path: gpu_enable=False on CPU tensors) and the oracle run side by side on randomly drawn filter
trees, group-bys, sorts and joins (with masks, duplicate and missing keys, extra join conditions
and every join type), so that the oracle the GPU tests check the kernels against is pinned beyond
the fixtures.  Keys, masks, counts, orders and integer results are compared exactly, float64
results within 1e-12 relative.
"""
import copy
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from golden_io import assert_f64_close  # noqa: E402
from oracle import reference  # noqa: E402
from oracle import tqp_oracle as O  # noqa: E402

TYPES = {1: "date", 2: "float", 3: "int", 4: "int", 5: "float", 6: "int", 7: "string", 8: "float"}
NAMES = {1: "d", 2: "x", 3: "k", 4: "c", 5: "y", 6: "a", 7: "s", 8: "z"}
NULL = O.NULL


class _Pool:
    def malloc_like(self, t):
        return 0, torch.empty_like(t)


@pytest.fixture(scope="module")
def ref():
    ok, why = reference.available()
    if not ok:
        pytest.skip(why)
    R = reference.load()
    with reference.cpu_mode():
        yield R


def columns(rng, n):
    words = [b"RED", b"GREEN", b"BLUE", b"GOLD", b"GREY"]
    pick = rng.integers(0, len(words), n)
    s = np.zeros((n, 6), np.int8)
    for i, w in enumerate(words):
        s[pick == i, :len(w)] = np.frombuffer(w, np.uint8).astype(np.int8)
    return {
        1: rng.integers(0, 2557, n).astype(np.int32),                       # a date (days)
        2: rng.integers(0, 11, n).astype(np.float64) / 100.0,               # a discount
        3: rng.integers(-50, 51, n).astype(np.int64),
        4: rng.integers(ord("A"), ord("G"), n).astype(np.uint8),            # a one-byte flag
        5: np.round(rng.uniform(-10, 200, n), 2),
        6: rng.integers(0, 7, n).astype(np.int32),
        7: s,
        8: rng.integers(90000, 10495001, n).astype(np.float64) / 100.0,     # a price
    }


def tg_of(R, cols):
    V = R.variable.Variable
    return {c: V(torch.from_numpy(np.ascontiguousarray(a)), TYPES.get(c, "int")) for c, a in cols.items()}


def col(c):
    return f"{NAMES[c]}#{c}"


# ------------------------------------------------------------------ filter
WORDS = ["RED", "GREEN", "BLUE", "GOLD", "GREY", "PINK"]


def string_leaf(rng):
    k = int(rng.integers(0, 7))
    if k == 0:
        return [col(7), "=", str(rng.choice(WORDS))]
    if k == 1:
        return ["StartsWith", [col(7), str(rng.choice(["GR", "B", "GO", "RE", "PI"]))]]
    if k == 2:
        return [str(rng.choice(["Contains", "EndsWith"])), [col(7), str(rng.choice(["E", "EE", "LD", "EN", "Y"]))]]
    if k == 3:
        return [col(7), "LIKE", str(rng.choice(["%G%E%", "%R%D%", "%E%N%", "%B%E%"]))]
    if k == 4:
        return [col(7), "IN", [str(w) for w in rng.choice(WORDS, int(rng.integers(1, 4)), replace=False)]]
    # a multi-character literal is compared for equality whatever the operator (filter.py:151-158)
    return [col(7), str(rng.choice(["<", ">=", "<>"])), str(rng.choice(WORDS))]


SUBQUERY = 25.375            # a scalar subquery's result, as the executor passes it (main.py:267)


def leaf(rng):
    c = int(rng.choice([1, 2, 3, 4, 5, 7]))
    if c == 7:
        return string_leaf(rng)
    r = rng.random()
    if r < 0.06 and c in (2, 3, 5):
        return [col(c), str(rng.choice(["<", "<=", ">", ">="])), "Subquery"]
    if r < 0.12 and c in (2, 3, 5):               # cast(column as double) (filter.py:78-83)
        return [["cast", [f"{col(c)} as double"]], str(rng.choice(["<", ">="])), str(rng.choice(["10", "0.5", "-3"]))]
    op = str(rng.choice(["<", "<=", ">", ">=", "=", "<>"], p=[0.19, 0.19, 0.19, 0.19, 0.19, 0.05]))
    if c == 1:
        lit = str(rng.choice(["1170", "2470", "100.5", "1993-03-15", "1995-01-01", "1989-12-31", "42"]))
    elif c == 2:
        lit = str(rng.choice(["0.05", "0.06", "0.0", "0.1", "0.07"]))
    elif c == 3:
        if rng.random() < 0.25:
            return [col(3), "IN", [str(v) for v in rng.integers(-60, 60, int(rng.integers(1, 5)))]]
        lit = str(rng.choice(["0", "-7", "49", "12.5", "-50"]))
    elif c == 4:
        return [col(4), "=", chr(int(rng.integers(ord("A"), ord("H"))))]
    else:
        lit = str(rng.choice(["100.5", "-3.25", "0", "0.0", "150"]))
    return [col(c), op, lit]


def tree(rng, depth=0):
    r = rng.random()
    if depth >= 3 or r < 0.35:
        return leaf(rng)
    if r < 0.45:
        return ["NOT", [tree(rng, depth + 1)]]
    if r < 0.5:
        return [["isnotnull", [col(3)]], "AND", tree(rng, depth + 1)]
    return [tree(rng, depth + 1), str(rng.choice(["AND", "OR"])), tree(rng, depth + 1)]


@pytest.mark.parametrize("seed", range(16))
def test_filter_trees(ref, seed):
    rng = np.random.default_rng(100 + seed)
    cols = columns(rng, 3001)
    for i in range(12):
        t = tree(rng)
        used = sorted({c for c in (1, 2, 3, 4, 5, 7) if col(c) in repr(t)})
        tg = tg_of(ref, {c: cols[c] for c in used})
        args = {"name": "Filter", "filter tree": [t], "materialized in": used, "out mask id": 900}
        try:
            ref.filter.tqp_filter(False, tg, copy.deepcopy(args), SUBQUERY, None, _Pool(), "f")
        except Exception as e:                      # noqa: BLE001  the oracle must raise the same class
            with pytest.raises(type(e)):
                O.eval_filter([t], {c: cols[c] for c in used}, 3001, SUBQUERY)
            continue
        expect = tg[900].tensor.numpy().reshape(-1)
        got = np.asarray(O.eval_filter([t], {c: cols[c] for c in used}, 3001, SUBQUERY)).reshape(-1)
        np.testing.assert_array_equal(got, expect, err_msg=repr(t))


def _model_program(prog, cols):
    """A numpy model of the kernels' predicate interpreter (eval_pred4 and pred_leaf4 in
    csrc/common.cuh) for the numeric instructions: int64 compares, a float32 compare of the
    converted value with the float32 literal, float64 compares and isclose."""
    from tqpk import _lib as L
    cmp = {L.LT: np.less, L.LE: np.less_equal, L.GT: np.greater, L.GE: np.greater_equal, L.EQ: np.equal,
           L.NE: np.not_equal}
    S, st = prog.struct, []
    n = next(iter(cols.values())).shape[0]
    for k in range(S.n_insn):
        I = S.insn[k]
        if I.op == L.P_CMP:
            x = cols[prog.col_ids[I.col]].reshape(-1)
            if I.domain == L.DOM_F64:
                xd = x.astype(np.float64)
                if I.cmp == L.ISCLOSE:
                    err = np.abs(xd - I.lit_f)
                    st.append((xd == I.lit_f) | (np.isfinite(err) & (err <= I.lit_aux)))
                else:
                    st.append(cmp[I.cmp](xd, I.lit_f))
            elif I.domain == L.DOM_F32:
                st.append(cmp[I.cmp](x.astype(np.int64).astype(np.float32), np.float32(I.lit_f)))
            else:
                st.append(cmp[I.cmp](x.astype(np.int64), np.int64(I.lit_i)))
        elif I.op in (L.P_STRCMP, L.P_PREFIX, L.P_CONTAINS, L.P_LIKE2):   # str_leaf4 on int8 [N, w] rows
            a = cols[prog.col_ids[I.col]].astype(np.int64)
            w = S.widths[I.col]
            pool = np.ctypeslib.as_array(S.strpool).astype(np.uint8).astype(np.int8).astype(np.int64)
            code = I.lit_i & 0xFFFFFFFFFFFFFFFF

            def at(off, ln, pos=0):
                return (a[:, pos:pos + ln] == pool[off:off + ln]).all(axis=1)
            if I.op == L.P_STRCMP:
                st.append(cmp[I.cmp](a[:, :w], pool[code & 0xFFFFFFFF:(code & 0xFFFFFFFF) + w]).all(axis=1))
            elif I.op == L.P_PREFIX:
                st.append(at(code & 0xFFFFFFFF, code >> 32))
            elif I.op == L.P_CONTAINS:
                ln = code >> 32
                st.append(np.any([at(code & 0xFFFFFFFF, ln, p) for p in range(w - ln + 1)], axis=0)
                          if w >= ln else np.zeros(n, bool))
            else:
                oa, na, ob, nb = code & 0xFFFF, (code >> 16) & 0xFFFF, (code >> 32) & 0xFFFF, code >> 48
                seen, out = np.zeros(n, bool), np.zeros(n, bool)
                for p in range(w - na - nb + 1):
                    seen |= at(oa, na, p)
                    out |= seen & at(ob, nb, p + na)
                st.append(out)
        elif I.op == L.P_CMPCOL:                      # column against column, the second slot in lit_i
            x = cols[prog.col_ids[I.col]].reshape(-1)
            y = cols[prog.col_ids[int(I.lit_i)]].reshape(-1)
            t = np.float64 if I.domain == L.DOM_F64 else np.int64
            st.append(cmp[I.cmp](x.astype(t), y.astype(t)))
        elif I.op == L.P_MASK:                        # a bool column, nonzero bytes true
            st.append(cols[prog.col_ids[I.col]].reshape(-1).astype(np.uint8) != 0)
        elif I.op == L.P_AND:
            b = st.pop()
            st[-1] = st[-1] & b
        elif I.op == L.P_OR:
            b = st.pop()
            st[-1] = st[-1] | b
        elif I.op == L.P_NOT:
            st[-1] = ~st[-1]
        elif I.op in (L.P_TRUE, L.P_FALSE):
            st.append(np.full(n, I.op == L.P_TRUE))
        else:
            raise NotImplementedError(f"instruction {I.op} is not modelled")
    assert len(st) == 1
    return st[0]


@pytest.mark.parametrize("seed", range(16))
def test_drop_in_filter_compiler_follows_the_reference(ref, seed):
    """tqpk.predicate.compile_filter turns the reference's trees and literals into the kernels'
    instructions on the host: the eps of float literals, isclose for float equality, float32
    for an integer column against a float literal, date and character literals, IN lists and
    isnotnull.  Its programs, run by a numpy model of the kernels' interpreter, give the
    reference's masks; trees the reference rejects are rejected with the same exception class."""
    from tqpk.predicate import compile_filter
    rng = np.random.default_rng(700 + seed)
    cols = columns(rng, 2001)
    for i in range(12):
        t = tree(rng)
        used = sorted({c for c in (1, 2, 3, 4, 5, 7) if col(c) in repr(t)})
        tg = tg_of(ref, {c: cols[c] for c in used})
        args = {"name": "Filter", "filter tree": [t], "materialized in": used, "out mask id": 900}
        tc = {c: torch.from_numpy(cols[c]) for c in used}
        try:
            ref.filter.tqp_filter(False, tg, copy.deepcopy(args), SUBQUERY, None, _Pool(), "f")
        except Exception as e:                      # noqa: BLE001  the compiler must raise the same class
            with pytest.raises(type(e)):
                compile_filter([copy.deepcopy(t)], tc, SUBQUERY)
            continue
        prog = compile_filter([copy.deepcopy(t)], tc, SUBQUERY)
        got = _model_program(prog, {c: cols[c] for c in used})
        np.testing.assert_array_equal(got, tg[900].tensor.numpy().reshape(-1), err_msg=repr(t))


# ------------------------------------------------------------------ aggregate
AGGS = [
    ["sum", [col(5)]], ["avg", [col(2)]], ["min", [col(5)]], ["max", [col(3)]], ["sum", [col(3)]],
    ["count", ["1"]], ["count", [col(3)]], ["avg", [col(3)]], ["min", [col(1)]], ["max", [col(8)]],
    ["sum", [[col(8), "*", ["1.0", "-", col(2)]]]],
    ["sum", [[[col(8), "*", ["1.0", "-", col(2)]], "*", ["1.0", "+", col(2)]]]],
    ["sum", [[col(3), "*", "2"]]], ["max", [[col(5), "+", col(2)]]], ["avg", [col(8)]],
    # torch's float32 results: an integer column with a float literal, integer true division,
    # a CASE mixing a float literal with integers
    ["sum", [[col(3), "*", "0.5"]]], ["avg", [[col(6), "/", [col(6), "+", "1"]]]], ["max", [[col(6), "*", "2.5"]]],
    ["sum", ["CASE", "WHEN", [col(3), ">", "25"], "THEN", "1.0", "ELSE", "0", "END"]],
    # integer arithmetic in the narrower type (uint8 wraps), mixed integer widths
    ["sum", [[col(4), "+", col(4)]]], ["min", [[col(6), "-", col(3)]]],
    # string conditions
    ["sum", ["CASE", "WHEN", [col(7), "=", "GREEN"], "THEN", col(8), "ELSE", "0.0", "END"]],
    ["sum", ["CASE", "WHEN", ["StartsWith", [col(7), "GR"]], "THEN", "1", "ELSE", "0", "END"]],
]
KEYS = [[], [col(6)], [col(6), col(4)], [col(3)], [col(7)], [col(4), col(7)], [col(2)], [col(5), col(6)]]


def _tuple_codes(key_cols, n):
    """Row codes of key tuples in ascending tuple order: each column ranked by value (floats too;
    -0.0 equals 0.0), string columns byte by byte, then the tuples of ranks."""
    ranks = []
    for k in key_cols:
        k = np.asarray(k).reshape(n, -1)
        for j in range(k.shape[1]):
            v = k[:, j]
            v = np.where(v == 0, 0, v) if v.dtype.kind == "f" else v
            ranks.append(np.unique(v, return_inverse=True)[1].reshape(-1))
    return np.stack(ranks, 1) if ranks else np.zeros((n, 0), np.int64)


def _key_order(keys):
    flat = []
    for k in keys:
        k = k.reshape(k.shape[0], -1)
        flat += [k[:, j] for j in range(k.shape[1])]
    return np.lexsort(flat[::-1]) if flat else np.zeros(1, np.int64)


@pytest.mark.parametrize("seed", range(24 + len(KEYS)))
def test_group_by(ref, seed):
    """Seeds below 24 draw 2-5 expressions; the last len(KEYS) seeds run every expression under
    each key set."""
    rng = np.random.default_rng(200 + seed)
    n = int(rng.integers(1, 4000))
    cols = columns(rng, n)
    keys = KEYS[seed % len(KEYS)]
    picks = rng.choice(len(AGGS), int(rng.integers(2, 6)), replace=False) if seed < 24 else np.arange(len(AGGS))
    results = list(keys) + [[[AGGS[p], "#", f"{400 + i}" + ("L" if AGGS[p][0] == "count" else "")], "AS",
                             f"r#{500 + i}"] for i, p in enumerate(picks)]
    key_ids = [int(k.split("#")[1]) for k in keys]
    used = sorted({c for c in cols if col(c) in repr(results)})
    args = {"name": "Aggregate", "is partial": False, "keys": keys or None, "input ids": used, "results": results,
            "out agg ids": [500 + i for i in range(len(picks))]}
    cols_in = {c: cols[c] for c in used}
    if seed % 2:                                     # behind a filter's mask
        cols_in[900] = cols[1] > 1000
        args["mask map"] = {c: 900 for c in used}
    tg = tg_of(ref, cols_in)
    if 900 in cols_in:
        tg[900] = ref.variable.Variable(torch.from_numpy(cols_in[900]), "bool")
    torch.manual_seed(seed)
    ref.aggregate.tqp_hash_aggregate(False, tg, copy.deepcopy(args), _Pool(), None, "a")
    got = O.tqp_hash_aggregate(cols_in, copy.deepcopy(args))
    ek = [tg[k].tensor.numpy() for k in key_ids]
    gk = [got[k] for k in key_ids]
    eo, go = _key_order(ek), _key_order(gk)
    for e, g in zip(ek, gk):
        assert e.shape == g.shape and e.dtype == g.dtype
        np.testing.assert_array_equal(g[go], e[eo])
    for oid in args["out agg ids"]:
        e, g = tg[oid].tensor.numpy(), got[oid]
        assert e.dtype == g.dtype and e.shape == g.shape, (oid, e.dtype, g.dtype, e.shape, g.shape)
        if keys:
            e, g = e[eo], g[go]
        if e.dtype == np.float32:                    # summation order may move the last bits
            np.testing.assert_allclose(g, e, rtol=2e-6, atol=2e-6 * max(1.0, float(np.abs(e).max(initial=0))))
        elif e.dtype.kind == "f":
            assert_f64_close(g, e)
        else:
            np.testing.assert_array_equal(g, e)


# ------------------------------------------------------------------ project
PROJ = [
    [["year", [col(1)]], "AS", "p#41"],
    [["CASE", "WHEN", [col(7), "=", "GREEN"], "THEN", col(8), "ELSE", "0.0", "END"], "AS", "p#42"],
    [[[col(8), "*", ["1.0", "-", col(2)]]], "AS", "p#43"],
    [[col(3), "<", "10"], "AS", "p#44"],
    [[[col(3), "*", "1.5"]], "AS", "p#45"],
    [[[col(6), "/", [col(6), "+", "1"]]], "AS", "p#46"],
    [[[col(4), "+", col(4)]], "AS", "p#47"],
    [[[col(6), "-", col(3)]], "AS", "p#48"],
    [["CASE", "WHEN", [col(3), ">", "25"], "THEN", "1.0", "ELSE", "0", "END"], "AS", "p#49"],
    [[[col(5), "*", col(6)]], "AS", "p#50"],
    [["substring", [col(7), "2", "3"]], "AS", "p#51"],          # the [N, 3] int8 slice of the rows
]


@pytest.mark.parametrize("seed", range(32))
def test_project(ref, seed, monkeypatch):
    """Four of the expressions above and three random trees per projection (more than one
    32-instruction program: the operator splits them)."""
    rng = np.random.default_rng(500 + seed)
    n = int(rng.integers(1, 3000))
    cols = columns(rng, n)
    picks = sorted(rng.choice(len(PROJ), 4, replace=False))
    exprs = [PROJ[p] for p in picks]
    outs = [41 + int(p) for p in picks]
    for j in range(3):                       # random arithmetic / CASE trees (not a bare column)
        e = num_expr(rng)
        while not (isinstance(e, list) and _has_col(e)):
            e = num_expr(rng)
        exprs.append([e if e[0] == "CASE" else [e], "AS", f"q#{60 + j}"])
        outs.append(60 + j)
    used = sorted({c for c in cols if col(c) in repr(exprs)})
    args = {"name": "Project", "rename map": {}, "materialized in": used, "used expr": exprs, "materialized out": outs}
    tg = tg_of(ref, {c: cols[c] for c in used})
    ref.project.tqp_project(False, tg, copy.deepcopy(args), None, _Pool(), "p")
    got = O.tqp_project({c: cols[c] for c in used}, copy.deepcopy(args))
    # the drop-in operator, its projection programs run by the interpreter model instead of the kernel
    from tqpk.operators import project as P
    from tqpk.variable import Variable

    def model_project(prog, rows, device):
        for pred, t in prog.masks:
            t.numpy()[:] = _model_program(pred, cols)
        regs = _model_registers(prog.spec, list(prog.tensors) + [t for _, t in prog.masks], rows)
        return [torch.from_numpy(np.ascontiguousarray(regs[r])).to(dt) for r, dt in prog.outputs]
    monkeypatch.setattr(P, "project", model_project)
    mine = {c: Variable(torch.from_numpy(np.ascontiguousarray(cols[c])), TYPES[c]) for c in used}
    P.tqp_project(True, mine, copy.deepcopy(args), None, None, "p")
    for c in outs:
        e = tg[c].tensor.numpy()
        assert mine[c].tensor_type == tg[c].tensor_type, (c, mine[c].tensor_type, tg[c].tensor_type)
        for name, g in (("oracle", got[c]), ("drop-in", mine[c].tensor.numpy())):
            assert g.dtype == e.dtype and g.shape == e.shape, (name, c, g.dtype, e.dtype)
            np.testing.assert_array_equal(g, e, err_msg=f"{name}: {c}")


# ------------------------------------------------------------------ sort
@pytest.mark.parametrize("seed", range(16))
def test_sort(ref, seed):
    rng = np.random.default_rng(300 + seed)
    n = int(rng.integers(1, 3000))
    cols = columns(rng, n)
    cols[5] = np.round(cols[5] / 20) * 20                                   # ties in the float key
    nk = int(rng.integers(1, 4))
    key_ids = [int(c) for c in rng.choice([1, 3, 4, 5, 6, 7], nk, replace=False)]
    inputs = sorted(set(key_ids) | {int(c) for c in rng.choice([2, 3, 8], 2, replace=False)})
    args = {"input ids": inputs, "key ids": key_ids, "key orders": [bool(b) for b in rng.integers(0, 2, nk)]}
    with_limit = bool(seed % 2)
    if with_limit:
        args["limit"] = int(rng.integers(1, n + 1))
    tg = tg_of(ref, {c: cols[c] for c in inputs})
    ref.sort.tqp_sort(False, tg, copy.deepcopy(args), with_limit, "s")
    got = O.tqp_sort({c: cols[c] for c in inputs}, args, with_limit)
    for c in inputs:
        np.testing.assert_array_equal(got[c], tg[c].tensor.numpy(), err_msg=f"column {c} of {args}")


# ------------------------------------------------------------------ join
JOIN_TYPES = ["inner", "right-semi", "right-anti", "right-outer"]


@pytest.mark.parametrize("seed", range(24))
def test_join(ref, seed):
    rng = np.random.default_rng(400 + seed)
    jtype = JOIN_TYPES[seed % 4]
    nb, npr = int(rng.integers(1, 800)), int(rng.integers(1, 2500))
    unique = seed % 3 != 0
    bkey = (rng.permutation(nb) + 1) if unique else rng.integers(1, max(2, nb // 3), nb)
    cols = {11: bkey.astype(np.int32), 12: rng.integers(0, 5, nb).astype(np.int32),
            13: rng.integers(0, 2557, nb).astype(np.int32),
            21: rng.integers(1, nb + 40, npr).astype(np.int32), 22: rng.integers(0, 5, npr).astype(np.int32),
            23: rng.integers(90000, 10495001, npr).astype(np.float64) / 100.0,
            24: rng.integers(0, 2557, npr).astype(np.int32)}
    types_ = {11: "int", 12: "int", 13: "date", 21: "int", 22: "int", 23: "float", 24: "date"}
    masked = seed % 2 == 0
    cols[901] = cols[13] < 1700
    cols[902] = cols[24] > 900
    args = {"name": "Join", "left group": [11, 12, 13], "right group": [21, 22, 23, 24],
            "materialized in": [11, 12, 21, 22, 23]}
    if masked:
        args["mask map"] = {11: 901, 12: 901, 21: 902, 22: 902, 23: 902}
    conds = [["#12", "=", "#22"]] if seed % 3 == 1 else []
    V = ref.variable.Variable
    tg = {c: V(torch.from_numpy(a), types_.get(c, "bool")) for c, a in cols.items()}
    try:
        rows = ref.hashjoin.join_vortex(False, tg, copy.deepcopy(args), 11, 21, copy.deepcopy(conds), jtype, None,
                                        _Pool(), "j")
    except RuntimeError:
        with pytest.raises(RuntimeError):
            O.join_vortex(cols, copy.deepcopy(args), 11, 21, jtype, conds)
        return
    got, got_rows = O.join_vortex(cols, copy.deepcopy(args), 11, 21, jtype, conds)
    assert got_rows == rows
    # the probe side comes in the reference's order (its matched probe rows ascending, hashjoin.py:65,93)
    for c in (21, 22, 23):
        np.testing.assert_array_equal(np.asarray(got[c]), tg[c].tensor.numpy(), err_msg=f"column {c}, {jtype}")
    # the build rows that match one probe row come in the order of the reference's torch.sort of the
    # build keys (hashjoin.py:43), which is not a stable sort: compared as a multiset of whole rows
    left = [c for c in (11, 12) if tg[c].tensor.numel()]
    for c in (11, 12):
        assert np.asarray(got[c]).shape == tuple(tg[c].tensor.shape), (c, jtype)
    if left:
        e = np.stack([tg[c].tensor.numpy().astype(np.float64) for c in left + [21, 22, 23]], 1)
        g = np.stack([np.asarray(got[c]).astype(np.float64) for c in left + [21, 22, 23]], 1)
        np.testing.assert_array_equal(g[np.lexsort(g.T[::-1])], e[np.lexsort(e.T[::-1])], err_msg=jtype)


# ------------------------------------------------------------------ the drop-in's compilers
def _tensors(cols):
    return {c: torch.from_numpy(np.ascontiguousarray(a)) for c, a in cols.items()}


@pytest.mark.parametrize("keys", KEYS, ids=[",".join(k) or "global" for k in KEYS])
def test_drop_in_aggregate_dtypes_follow_the_reference(ref, keys):
    """tqpk.expr.compile_aggregate decides each output's dtype on the host (the kernels write what
    it says; float32 results are rounded from float64 by its `casts`).  Those decisions, and the
    type names the drop-in gives the outputs, equal the reference's for every expression above."""
    from tqpk.expr import compile_aggregate, needs_key_codes
    from tqpk.variable import torch_to_type
    rng = np.random.default_rng(600)
    cols = columns(rng, 300)
    key_ids = [int(k.split("#")[1]) for k in keys]
    for i, agg in enumerate(AGGS):
        results = list(keys) + [[[agg, "#", "400" + ("L" if agg[0] == "count" else "")], "AS", "r#500"]]
        # at least one input column (with none, both return empty float32 columns before compiling)
        used = sorted({c for c in cols if col(c) in repr(results)} | {3})
        args = {"name": "Aggregate", "is partial": False, "keys": keys or None, "input ids": used,
                "results": results, "out agg ids": [500]}
        tg = tg_of(ref, {c: cols[c] for c in used})
        torch.manual_seed(i)
        ref.aggregate.tqp_hash_aggregate(False, tg, copy.deepcopy(args), _Pool(), None, "a")
        tc = _tensors({c: cols[c] for c in used})
        # string keys are numbered first (tqpk.ops.encode_keys) and the kernel groups by the code
        codes = torch.zeros(300, dtype=torch.int32) if needs_key_codes(args, tc) else None
        prog = compile_aggregate(copy.deepcopy(args), tc, derived=True, key_codes=codes)
        dt = {o[0]: o[4] for o in prog.outputs}[500]
        if 500 in prog.casts:                        # the 2-step path (>= 2^16 rows per group) is not reached here
            dt = prog.casts[500][0]
        e = tg[500]
        assert dt == e.tensor.dtype, (agg, dt, e.tensor.dtype)
        assert torch_to_type(dt) == e.tensor_type, (agg, torch_to_type(dt), e.tensor_type)
        for k in key_ids:
            assert tg[k].tensor.dtype == torch.from_numpy(cols[k][:1]).dtype


def test_drop_in_projection_dtypes_follow_the_reference(ref):
    """tqpk.expr.compile_projection's output dtypes and the drop-in's type names against the
    reference's tqp_project, for every projection expression above."""
    from tqpk.expr import compile_projection
    from tqpk.variable import torch_to_type
    rng = np.random.default_rng(601)
    cols = columns(rng, 300)
    from tqpk.operators.project import _substring_of
    for p, expr in enumerate(PROJ):
        if _substring_of(expr) is not None:          # a slice of the rows, not a compiled expression
            continue
        used = sorted({c for c in cols if col(c) in repr(expr)})
        out = 41 + p
        args = {"name": "Project", "rename map": {}, "materialized in": used, "used expr": [expr],
                "materialized out": [out]}
        tg = tg_of(ref, {c: cols[c] for c in used})
        ref.project.tqp_project(False, tg, copy.deepcopy(args), None, _Pool(), "p")
        prog = compile_projection([copy.deepcopy(expr)], _tensors({c: cols[c] for c in used}), derived=True)
        (dt,) = [d for (_, d) in prog.outputs]
        assert dt == tg[out].tensor.dtype, (expr, dt, tg[out].tensor.dtype)
        assert torch_to_type(dt) == tg[out].tensor_type, (expr, torch_to_type(dt), tg[out].tensor_type)


# ------------------------------------------------------------------ expression programs
def _year(d):
    """The kernels' expr_year: days since 1990-01-01 to the proleptic Gregorian year (days before
    1990 in 1990), H. Hinnant's civil_from_days."""
    d = np.asarray(d, np.int64)
    z = d + 7305 + 719468
    era = z // 146097
    doe = z - era * 146097
    yoe = (doe - doe // 1460 + doe // 36524 - doe // 146096) // 365
    doy = doe - (365 * yoe + yoe // 4 - yoe // 100)
    mp = (5 * doy + 2) // 153
    return np.where(d < 0, 1990, yoe + era * 400 + (mp >= 10))


def _model_registers(spec, tensors, n):
    """A numpy model of the kernels' expression interpreter (expr_apply, expr_apply_f32 and
    int_wrap in csrc/common.cuh): int64, float64 and float32 registers, round-to-nearest float32
    arithmetic, integer results wrapped to int8 / uint8 / int32 where torch's dtype is narrower."""
    from tqpk import _lib as L
    by_ptr = {t.data_ptr(): t for t in tensors}
    wrap = {L.I8: np.int8, L.U8: np.uint8, L.I32: np.int32}
    regs = []
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        for i in range(spec.n_expr):
            X = spec.expr[i]
            a = regs[X.a] if 0 <= X.a < i else None
            b = regs[X.b] if 0 <= X.b < i else None
            arith = {L.X_ADD: np.add, L.X_SUB: np.subtract, L.X_MUL: np.multiply, L.X_DIV: np.divide}
            if X.type == L.F32 and X.op != L.X_SELECT:
                if X.op == L.X_CONST:
                    r = np.full(n, np.float32(X.cf))
                elif X.op == L.X_TOF32:
                    r = a.astype(np.int64).astype(np.float32)
                else:
                    r = arith[X.op](a.astype(np.float32), b.astype(np.float32)).astype(np.float32)
            elif X.wrap and X.type == L.I64 and X.op in (L.X_ADD, L.X_SUB, L.X_MUL):
                r = arith[X.op](a.astype(np.int64), b.astype(np.int64)).astype(wrap[X.wrap]).astype(np.int64)
            elif X.op == L.X_F32TOF64:
                r = a.astype(np.float32).astype(np.float64)
            elif X.op == L.X_SELECT:
                r = np.where(a != 0, b, regs[X.col])
            elif X.op == L.X_YEAR:
                r = _year(a)
            elif X.op == L.X_COL:
                t = by_ptr[spec.cols[X.col]]
                c = t.reshape(-1).numpy() if t.dim() == 2 and t.shape[1] == 1 else t.numpy()
                r = c.astype(np.float64) if X.type == L.F64 else c.astype(np.int64)
            elif X.op == L.X_CONST:
                r = np.full(n, X.cf if X.type == L.F64 else X.ci, np.float64 if X.type == L.F64 else np.int64)
            elif X.op == L.X_TOF64:
                r = a.astype(np.int64).astype(np.float64)
            elif X.op == L.X_DIV:
                r = np.divide(a.astype(np.float64), b.astype(np.float64))
            elif X.type == L.F64:
                r = arith[X.op](a.astype(np.float64), b.astype(np.float64))
            else:
                r = arith[X.op](a.astype(np.int64), b.astype(np.int64))
            regs.append(r)
    return regs


def _fill_conditions(prog):
    """The bool columns of the program's conditions, from their predicates (filled by the filter
    kernel before the program runs)."""
    for pred, t in prog.masks:
        t.numpy()[:] = _model_program(pred, {cid: x.numpy() for cid, x in zip(pred.col_ids, pred.tensors)})


def _model_outputs(prog, regs, inv, G):
    """The accumulators per group, the outputs as the emission writes them (csrc/groupby.cu: avg =
    float64 sum / count, counts as integers), the float32 casts, then the arithmetic over
    aggregates as a projection over the groups."""
    from tqpk import _lib as L
    from tqpk.expr import _HIDDEN_ID, compile_projection
    accs = []
    for a in range(prog.spec.n_accs):
        A = prog.spec.accs[a]
        if A.kind == L.ACC_COUNT_ROWS:
            accs.append((np.bincount(inv, minlength=G).astype(np.int64), False, True))
            continue
        f = A.type == L.F64
        r = regs[A.reg].astype(np.float64 if f else np.int64)
        if A.kind == L.ACC_COUNT_NOTNULL:                # values equal to the null marker are not counted
            accs.append((np.bincount(inv, weights=(r != L.NULL_INDEX), minlength=G).astype(np.int64), False, True))
            continue
        if A.kind == L.ACC_SUM:
            v = np.zeros(G, r.dtype)
            np.add.at(v, inv, r)
        else:                                             # min / max start from the record's initial value
            v = np.full(G, A.init_f if f else A.init_i, r.dtype)
            (np.minimum if A.kind == L.ACC_MIN else np.maximum).at(v, inv, r)
        accs.append((v, f, False))
    res = {}
    for oid, op, ia, ib, dt in prog.outputs:
        v, f, is_count = accs[ia]
        if op == L.OUT_AVG:
            v = v.astype(np.float64) / accs[ib][0].astype(np.float64)
        res[oid] = torch.from_numpy(np.ascontiguousarray(v)).to(dt)
    for oid, (dt, is_avg) in prog.casts.items():      # rows per group stay below the 2-step path here
        if oid in res:
            res[oid] = res[oid].to(dt)
    if prog.post:
        hidden = {oid: res.pop(oid) for oid in list(res) if oid >= _HIDDEN_ID}
        for oid, tree, dt in prog.post:
            pp = compile_projection([tree], hidden)
            (reg, pdt), = pp.outputs
            res[oid] = torch.from_numpy(np.ascontiguousarray(_model_registers(pp.spec, pp.tensors, G)[reg])).to(pdt)
    return res


def _model_aggregate(prog, cols, key_ids, n):
    """A compiled AggregateProgram under the model above, grouped by the input key columns
    (keys ascending)."""
    _fill_conditions(prog)
    regs = _model_registers(prog.spec, list(prog.tensors) + [t for _, t in prog.masks], n)
    if key_ids:
        _, inv = np.unique(_tuple_codes([cols[k] for k in key_ids], n), axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        G = int(inv.max()) + 1
    else:
        inv, G = np.zeros(n, np.int64), 1
    return _model_outputs(prog, regs, inv, G)


def _model_groupby(prog, n, device=None, mask=None, before_values=None, key_ranges=None, values_late=False):
    """tqpk.ops.groupby under the model: the rows passing the filter mask grouped by the program's
    own key columns (or its key code), keys ascending; (key columns, outputs, groups, plan)."""
    from tqpk.dtypes import dtype_of
    if before_values is not None:
        before_values()
    _fill_conditions(prog)
    tensors = list(prog.tensors) + [t for _, t in prog.masks]
    by_ptr = {t.data_ptr(): t for t in tensors}
    sel = np.ones(n, bool) if mask is None else mask.reshape(-1).numpy().astype(bool)
    regs = [r[sel] for r in _model_registers(prog.spec, tensors, n)]
    S = prog.spec
    keys = [by_ptr[S.keys[k]].reshape(-1).numpy()[sel].astype(np.int64) for k in range(S.n_keys)]
    if keys:
        uniq, inv = np.unique(np.stack(keys, 1), axis=0, return_inverse=True)
        inv, G = inv.reshape(-1), uniq.shape[0]
    else:
        uniq, inv, G = np.zeros((1, 0), np.int64), np.zeros(int(sel.sum()), np.int64), 1
    res = _model_outputs(prog, regs, inv, G)
    key_cols = [torch.from_numpy(np.ascontiguousarray(uniq[:, k])).to(dtype_of(S.key_dtypes[k]))
                for k in range(S.n_keys)]
    return key_cols, res, G, None


def _model_encode_keys(key_cols, mask):
    """tqpk.ops.encode_keys under the model: int32 codes in key-tuple order for the rows passing
    the mask, a representative row per code, the number of codes."""
    n = key_cols[0].shape[0]
    sel = np.ones(n, bool) if mask is None else mask.reshape(-1).numpy().astype(bool)
    rows = np.nonzero(sel)[0]
    stacked = _tuple_codes([k.numpy() for k in key_cols], n)[rows]
    uniq, first, inv = np.unique(stacked, axis=0, return_index=True, return_inverse=True)
    codes = np.zeros(n, np.int32)
    codes[rows] = inv.reshape(-1)
    return torch.from_numpy(codes), torch.from_numpy(rows[first].astype(np.int64)), int(uniq.shape[0])


ARITH_COLS = [5, 2, 8, 3, 6, 4]           # float64, float64, float64, int64, int32, uint8
LITS = ["1.0", "2", "0.5", "1", "3", "0.25"]


def num_expr(rng, depth=0):
    r = rng.random()
    if depth >= 2 or r < 0.3:
        if rng.random() < 0.1:                   # two literals: a 0-dim tensor in torch
            return [str(rng.choice(LITS)), str(rng.choice(["+", "-", "*", "/"])), str(rng.choice(LITS))]
        return col(int(rng.choice(ARITH_COLS))) if rng.random() < 0.75 else str(rng.choice(LITS))
    if r < 0.38:
        cond = [col(int(rng.choice([3, 5, 6]))), str(rng.choice(["<", ">", "<=", ">="])), str(rng.choice(["0", "3", "25"]))]
        if rng.random() < 0.3:
            cond = [col(7), "=", str(rng.choice(WORDS))]
        return ["CASE", "WHEN", cond, "THEN", num_expr(rng, depth + 1), "ELSE", num_expr(rng, depth + 1), "END"]
    op = str(rng.choice(["+", "-", "*", "/"], p=[0.3, 0.3, 0.3, 0.1]))
    if op == "/":                            # divisors that are never zero
        return [num_expr(rng, depth + 1), "/", [[col(6), "+", "1"], col(8), "2", "0.5"][int(rng.integers(0, 4))]]
    return [num_expr(rng, depth + 1), op, num_expr(rng, depth + 1)]


def _has_col(t):
    return "#" in repr(t)


@pytest.mark.parametrize("seed", range(64))
def test_drop_in_expression_programs_follow_the_reference(ref, seed):
    """Random arithmetic / CASE expressions over float64, int64, int32 and uint8 columns under sum,
    avg, min, max and count, grouped by a key: the drop-in's compiled program, run by the numpy
    model of the kernels' interpreter, against the reference's values and dtypes (and the oracle
    against the reference).  Float64 within 1e-12 relative, float32 within its summation rounding,
    integers exact."""
    from tqpk.expr import compile_aggregate, needs_key_codes
    rng = np.random.default_rng(800 + seed)
    n = int(rng.integers(1, 2000))
    cols = columns(rng, n)
    keys = [KEYS[1], KEYS[2], KEYS[3], KEYS[4]][seed % 4]
    key_ids = [int(k.split("#")[1]) for k in keys]
    results, fns = list(keys), []
    for i in range(4):
        e = num_expr(rng)
        while not _has_col(e):
            e = num_expr(rng)
        fn = str(rng.choice(["sum", "avg", "min", "max", "count"]))
        arg = e if isinstance(e, list) and e and e[0] == "CASE" else [e]
        results.append([[[fn, arg], "#", f"{400 + i}" + ("L" if fn == "count" else "")], "AS", f"r#{500 + i}"])
        fns.append(fn)
    used = sorted({c for c in cols if col(c) in repr(results)})
    args = {"name": "Aggregate", "is partial": False, "keys": keys, "input ids": used, "results": results,
            "out agg ids": [500 + i for i in range(4)]}
    tg = tg_of(ref, {c: cols[c] for c in used})
    torch.manual_seed(seed)
    tc = {c: torch.from_numpy(np.ascontiguousarray(cols[c])) for c in used}
    codes = torch.zeros(n, dtype=torch.int32) if needs_key_codes(args, tc) else None
    try:
        ref.aggregate.tqp_hash_aggregate(False, tg, copy.deepcopy(args), _Pool(), None, "a")
    except Exception as e:                              # noqa: BLE001  both must raise the same class
        with pytest.raises(type(e)):
            O.tqp_hash_aggregate({c: cols[c] for c in used}, copy.deepcopy(args))
        with pytest.raises(type(e)):
            compile_aggregate(copy.deepcopy(args), tc, derived=True, key_codes=codes)
        return
    oracle = O.tqp_hash_aggregate({c: cols[c] for c in used}, copy.deepcopy(args))
    try:
        prog = compile_aggregate(copy.deepcopy(args), tc, derived=True, key_codes=codes)
    except NotImplementedError as e:                    # the program's size limits raise, never truncate
        assert "exceed" in str(e), e
        prog = None
    model = _model_aggregate(prog, {c: cols[c] for c in used}, key_ids, n) if prog is not None else {}
    eo = _key_order([tg[k].tensor.numpy() for k in key_ids])
    go = _key_order([oracle[k] for k in key_ids])
    for i in range(4):
        oid = 500 + i
        e = tg[oid].tensor.numpy()[eo]
        checks = [("oracle", oracle[oid][go])] + ([("drop-in", model[oid].numpy())] if model else [])
        for name, g in checks:
            assert g.dtype == e.dtype, (name, results[len(keys) + i], g.dtype, e.dtype)
            if e.dtype == np.float32:
                np.testing.assert_allclose(g, e, rtol=2e-6, atol=2e-6 * max(1.0, float(np.abs(e).max(initial=0))),
                                           err_msg=f"{name}: {results[len(keys) + i]}")
            elif e.dtype.kind == "f":
                assert_f64_close(g, e)
            else:
                np.testing.assert_array_equal(g, e, err_msg=f"{name}: {results[len(keys) + i]}")


@pytest.mark.parametrize("fn", ["sum", "avg", "min", "max", "count"])
def test_aggregate_of_literals(ref, fn):
    """An aggregate of two combined literals fails in the reference (torch gives a 0-dim tensor its
    reductions reject); the oracle and the drop-in's compiler raise the same class.  A bare literal
    is expanded to one value per row (aggregate.py:149-152) by all three."""
    from tqpk.expr import compile_aggregate
    rng = np.random.default_rng(900)
    cols = columns(rng, 200)
    for arg, fails in ((["2", "+", "0.25"], True), (["3", "*", "2"], True), ("2", False), ("0.5", False)):
        res = [[[fn, [arg]], "#", "400" + ("L" if fn == "count" else "")], "AS", "r#500"]
        args = {"name": "Aggregate", "is partial": False, "keys": [col(6)], "input ids": [3, 6],
                "results": [col(6), res], "out agg ids": [500]}
        tg = tg_of(ref, {3: cols[3], 6: cols[6]})
        tc = {c: torch.from_numpy(cols[c]) for c in (3, 6)}
        try:
            ref.aggregate.tqp_hash_aggregate(False, tg, copy.deepcopy(args), _Pool(), None, "a")
            raised = None
        except Exception as e:                          # noqa: BLE001
            raised = type(e)
        assert (raised is not None) == fails, (fn, arg, raised)
        if raised is not None:
            with pytest.raises(raised):
                O.tqp_hash_aggregate({3: cols[3], 6: cols[6]}, copy.deepcopy(args))
            with pytest.raises(raised):
                compile_aggregate(copy.deepcopy(args), tc, derived=True)
            continue
        prog = compile_aggregate(copy.deepcopy(args), tc, derived=True)
        model = _model_aggregate(prog, {3: cols[3], 6: cols[6]}, [6], 200)[500].numpy()
        oracle = O.tqp_hash_aggregate({3: cols[3], 6: cols[6]}, copy.deepcopy(args))[500]
        e = tg[500].tensor.numpy()[_key_order([tg[6].tensor.numpy()])]
        for g in (model, oracle):
            assert g.dtype == e.dtype, (fn, arg, g.dtype, e.dtype)
            np.testing.assert_allclose(g, e, rtol=1e-6)


# ------------------------------------------------------------------ the drop-in join operator
@pytest.fixture()
def cpu_join_kernels(monkeypatch):
    """tqpk.operators.hashjoin with the library calls it makes replaced by numpy models of their
    documented results: the directory build and probe (the oracle's index join, pinned above, on the
    rows passing each side's mask, original row ids out; an outer probe without any pair still
    gives every unmatched row a null build index), the predicate mask (the interpreter model),
    compaction, row marking and the gathers."""
    from types import SimpleNamespace
    from tqpk import ops
    from tqpk.operators import hashjoin as H

    def join_build(keys, mask=None):
        k = keys.reshape(-1).numpy()
        m = np.ones(k.size, bool) if mask is None else mask.numpy().astype(bool)
        sel = k[m]
        plan = SimpleNamespace(key_min=int(sel.min()) if sel.size else 0, key_max=int(sel.max()) if sel.size else -1,
                               nb_rows=int(m.sum()))
        return SimpleNamespace(keys=k, mask=m, plan=plan)

    def join_probe(b, probe_keys, probe_mask=None, join_type="inner"):
        pk = probe_keys.reshape(-1).numpy()
        pm = np.ones(pk.size, bool) if probe_mask is None else probe_mask.numpy().astype(bool)
        bsel, psel = np.nonzero(b.mask)[0], np.nonzero(pm)[0]
        li, ri = O.join_indices(b.keys[b.mask], pk[pm], join_type)
        pi = psel[ri]
        if join_type in ("right-semi", "right-anti"):
            bi = np.zeros(0, np.int64)
        elif join_type == "right-outer" and li.size == 0:
            bi = np.full(pi.size, NULL, np.int64)
        else:
            bi = np.where(li == NULL, NULL, bsel[np.where(li == NULL, 0, li)]) if li.size else li
        return torch.from_numpy(bi.astype(np.int64)), torch.from_numpy(pi.astype(np.int64))

    def filter_mask(pred, n, device, with_count=False):
        cols = {cid: t.numpy() for cid, t in zip(pred.col_ids, pred.tensors)}
        m = torch.from_numpy(np.asarray(_model_program(pred, cols), bool).reshape(-1)) if n else torch.zeros(0, dtype=torch.bool)
        return m, (torch.tensor([int(m.sum())]) if with_count else None)

    def compact(cols, mask=None, pred=None, with_row_ids=False):
        m = mask.reshape(-1)
        outs = [c.reshape(-1)[m] for c in cols] + ([torch.nonzero(m).reshape(-1)] if with_row_ids else [])
        return outs, int(m.sum())

    def mark_rows(idx, n):
        f = torch.zeros(n, dtype=torch.bool)
        f[idx] = True
        return f

    def gather_1d(cols, idx, null_aware):
        outs = []
        for c in cols:
            c = c.reshape(-1)
            nul = idx == NULL
            o = c[idx.masked_fill(nul, 0)].clone()
            if null_aware:
                o[nul] = NULL
            outs.append(o)
        return outs

    for name, f in (("join_build", join_build), ("join_probe", join_probe), ("filter_mask", filter_mask),
                    ("compact", compact), ("mark_rows", mark_rows)):
        monkeypatch.setattr(H, name, f)
    monkeypatch.setattr(ops, "_gather_1d", gather_1d)
    monkeypatch.setattr(ops, "gather_rows", lambda col, idx: col[idx])
    return H


@pytest.mark.parametrize("seed", range(24))
def test_drop_in_join_operator_follows_the_reference(ref, cpu_join_kernels, seed):
    """The drop-in join_vortex (masks popped from `mask map`, pairs, extra conditions on the
    gathered pair columns, semi / anti / outer derived from the kept pairs, gathered outputs)
    against the reference's on the random joins above."""
    from tqpk.variable import Variable
    rng = np.random.default_rng(400 + seed)
    jtype = JOIN_TYPES[seed % 4]
    nb, npr = int(rng.integers(1, 800)), int(rng.integers(1, 2500))
    unique = seed % 3 != 0
    bkey = (rng.permutation(nb) + 1) if unique else rng.integers(1, max(2, nb // 3), nb)
    cols = {11: bkey.astype(np.int32), 12: rng.integers(0, 5, nb).astype(np.int32),
            13: rng.integers(0, 2557, nb).astype(np.int32),
            21: rng.integers(1, nb + 40, npr).astype(np.int32), 22: rng.integers(0, 5, npr).astype(np.int32),
            23: rng.integers(90000, 10495001, npr).astype(np.float64) / 100.0,
            24: rng.integers(0, 2557, npr).astype(np.int32)}
    types_ = {11: "int", 12: "int", 13: "date", 21: "int", 22: "int", 23: "float", 24: "date"}
    cols[901] = cols[13] < 1700
    cols[902] = cols[24] > 900
    args = {"name": "Join", "left group": [11, 12, 13], "right group": [21, 22, 23, 24],
            "materialized in": [11, 12, 21, 22, 23]}
    if seed % 2 == 0:
        args["mask map"] = {11: 901, 12: 901, 21: 902, 22: 902, 23: 902}
    conds = [["#12", "=", "#22"]] if seed % 3 == 1 else []
    V = ref.variable.Variable
    tg = {c: V(torch.from_numpy(a), types_.get(c, "bool")) for c, a in cols.items()}
    rows = ref.hashjoin.join_vortex(False, tg, copy.deepcopy(args), 11, 21, copy.deepcopy(conds), jtype, None,
                                    _Pool(), "j")
    mine = {c: Variable(torch.from_numpy(a.copy()), types_.get(c, "bool")) for c, a in cols.items()}
    got_rows = cpu_join_kernels.join_vortex(True, mine, copy.deepcopy(args), 11, 21, copy.deepcopy(conds), jtype,
                                            None, None, "j")
    assert got_rows == rows
    for c in (21, 22, 23):
        np.testing.assert_array_equal(mine[c].tensor.numpy(), tg[c].tensor.numpy(), err_msg=f"column {c}, {jtype}")
    left = [c for c in (11, 12) if tg[c].tensor.numel()]
    for c in (11, 12):
        assert tuple(mine[c].tensor.shape) == tuple(tg[c].tensor.shape), (c, jtype)
        assert mine[c].tensor.dtype == tg[c].tensor.dtype, (c, jtype)
    if left:
        e = np.stack([tg[c].tensor.numpy().astype(np.float64) for c in left + [21, 22, 23]], 1)
        g = np.stack([mine[c].tensor.numpy().astype(np.float64) for c in left + [21, 22, 23]], 1)
        np.testing.assert_array_equal(g[np.lexsort(g.T[::-1])], e[np.lexsort(e.T[::-1])], err_msg=jtype)


# ------------------------------------------------------------------ the drop-in aggregate operator
@pytest.mark.parametrize("seed", range(24))
def test_drop_in_aggregate_operator_follows_the_reference(ref, monkeypatch, seed):
    """The drop-in tqp_hash_aggregate (`mask map` handling, key codes for string keys, outputs
    written as [G, 1] keys and typed aggregates) against the reference, with its library calls
    (the group-by, the key numbering, the gathers) replaced by the models above."""
    from tqpk import ops
    from tqpk.operators import aggregate as A
    from tqpk.variable import Variable
    monkeypatch.setattr(A, "groupby", _model_groupby)
    monkeypatch.setattr(A, "encode_keys", _model_encode_keys)
    monkeypatch.setattr(ops, "_gather_1d", lambda cols, idx, null_aware: [c.reshape(-1)[idx] for c in cols])
    monkeypatch.setattr(ops, "gather_rows", lambda col, idx: col[idx])
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(1, 3000))
    cols = columns(rng, n)
    keys = KEYS[seed % len(KEYS)]
    picks = rng.choice(len(AGGS), int(rng.integers(2, 7)), replace=False)
    results = list(keys) + [[[AGGS[p], "#", f"{400 + i}" + ("L" if AGGS[p][0] == "count" else "")], "AS",
                             f"r#{500 + i}"] for i, p in enumerate(picks)]
    key_ids = [int(k.split("#")[1]) for k in keys]
    used = sorted({c for c in cols if col(c) in repr(results)} | {3})
    args = {"name": "Aggregate", "is partial": False, "keys": keys or None, "input ids": used, "results": results,
            "out agg ids": [500 + i for i in range(len(picks))]}
    cols_in = {c: cols[c] for c in used}
    if (seed // len(KEYS)) % 2:                      # behind a filter's mask
        cols_in[900] = cols[1] > 1000
        args["mask map"] = {c: 900 for c in used}
    tg = tg_of(ref, cols_in)
    mine = {c: Variable(torch.from_numpy(np.ascontiguousarray(a).copy()), TYPES.get(c, "int")) for c, a in cols_in.items()}
    if 900 in cols_in:
        tg[900] = ref.variable.Variable(torch.from_numpy(cols_in[900]), "bool")
        mine[900] = Variable(torch.from_numpy(cols_in[900].copy()), "bool")
    torch.manual_seed(seed)
    rows = ref.aggregate.tqp_hash_aggregate(False, tg, copy.deepcopy(args), _Pool(), None, "a")
    got_rows = A.tqp_hash_aggregate(True, mine, copy.deepcopy(args), None, None, "a")
    assert got_rows == rows
    eo = _key_order([tg[k].tensor.numpy() for k in key_ids])
    go = _key_order([mine[k].tensor.numpy() for k in key_ids])
    for k in key_ids:
        e, g = tg[k], mine[k]
        assert (g.tensor_type, g.tensor.dtype, tuple(g.tensor.shape)) == (e.tensor_type, e.tensor.dtype,
                                                                          tuple(e.tensor.shape)), k
        np.testing.assert_array_equal(g.tensor.numpy()[go], e.tensor.numpy()[eo])
    for oid in args["out agg ids"]:
        e, g = tg[oid], mine[oid]
        assert (g.tensor_type, g.tensor.dtype, tuple(g.tensor.shape)) == (e.tensor_type, e.tensor.dtype,
                                                                          tuple(e.tensor.shape)), oid
        ev, gv = e.tensor.numpy(), g.tensor.numpy()
        if keys:
            ev, gv = ev[eo], gv[go]
        if ev.dtype == np.float32:
            np.testing.assert_allclose(gv, ev, rtol=2e-6, atol=2e-6 * max(1.0, float(np.abs(ev).max(initial=0))))
        elif ev.dtype.kind == "f":
            assert_f64_close(gv, ev)
        else:
            np.testing.assert_array_equal(gv, ev)


# ------------------------------------------------------------------ the drop-in filter and sort operators
@pytest.mark.parametrize("seed", range(8))
def test_drop_in_filter_operator_follows_the_reference(ref, monkeypatch, seed):
    """tqp_filter with its mask kernel replaced by the interpreter model: the mask column it writes
    (id, dtype, type name, values) against the reference's, for random numeric and string trees."""
    from tqpk.operators import filter as F
    from tqpk.variable import Variable

    def filter_mask(pred, n, device, with_count=False):
        m = np.asarray(_model_program(pred, {cid: t.numpy() for cid, t in zip(pred.col_ids, pred.tensors)}), bool)
        return torch.from_numpy(m.reshape(-1).copy()), None
    monkeypatch.setattr(F, "filter_mask", filter_mask)
    rng = np.random.default_rng(1100 + seed)
    cols = columns(rng, 1500)
    for i in range(10):
        t = tree(rng)
        used = sorted({c for c in (1, 2, 3, 4, 5, 7) if col(c) in repr(t)})
        args = {"name": "Filter", "filter tree": [t], "materialized in": used, "out mask id": 900}
        tg = tg_of(ref, {c: cols[c] for c in used})
        mine = {c: Variable(torch.from_numpy(cols[c].copy()), TYPES[c]) for c in used}
        try:
            ref.filter.tqp_filter(False, tg, copy.deepcopy(args), SUBQUERY, None, _Pool(), "f")
        except Exception as e:                      # noqa: BLE001  the same class from the operator
            with pytest.raises(type(e)):
                F.tqp_filter(True, mine, copy.deepcopy(args), SUBQUERY, None, None, "f")
            continue
        F.tqp_filter(True, mine, copy.deepcopy(args), SUBQUERY, None, None, "f")
        e, g = tg[900], mine[900]
        assert (g.tensor_type, g.tensor.dtype) == (e.tensor_type, e.tensor.dtype), repr(t)
        np.testing.assert_array_equal(g.tensor.numpy().reshape(-1), e.tensor.numpy().reshape(-1), err_msg=repr(t))


@pytest.mark.parametrize("seed", range(16))
def test_drop_in_sort_operator_follows_the_reference(ref, monkeypatch, seed):
    """tqp_sort with its kernels replaced by models (a stable sort of keys[perm] per pass, the
    oracle's pinned order; the string rows' 8-byte words as order-preserving integers): the LSD
    passes over keys and string words, the stable top-k for the limit and the gathers against the
    reference's sorted columns."""
    from tqpk import ops
    from tqpk.operators import sort as S
    from tqpk.variable import Variable

    def argsort_stable(keys, descending=False, perm_in=None):
        k = keys.reshape(-1).numpy()
        p = np.arange(k.size) if perm_in is None else perm_in.numpy()
        return torch.from_numpy(p[O._stable_order(k[p], bool(descending))].astype(np.int64))

    def topk_stable(keys, k, descending=False, perm_in=None):
        return argsort_stable(keys, descending, perm_in)[:k]

    def string_words(col, word):
        b = col.numpy()[:, 8 * word:8 * word + 8].astype(np.int64)
        b = np.pad(b, ((0, 0), (0, 8 - b.shape[1])))
        b = (b + 128 if col.dtype == torch.int8 else b).astype(np.uint64)   # bytes in the column type's order
        out = np.zeros(b.shape[0], np.uint64)
        for j in range(8):                                      # big-endian unsigned word
            out = (out << np.uint64(8)) | b[:, j]
        return torch.from_numpy((out ^ np.uint64(1 << 63)).view(np.int64))   # the same order as int64
    for name, f in (("argsort_stable", argsort_stable), ("topk_stable", topk_stable), ("string_words", string_words),
                    ("gather_rows", lambda col, idx: col[idx])):
        monkeypatch.setattr(S, name, f)
    monkeypatch.setattr(ops, "_gather_1d", lambda cols, idx, null_aware: [c.reshape(-1)[idx] for c in cols])
    monkeypatch.setattr(ops, "gather_rows", lambda col, idx: col[idx])
    rng = np.random.default_rng(1200 + seed)
    n = int(rng.integers(1, 3000))
    cols = columns(rng, n)
    cols[5] = np.round(cols[5] / 20) * 20
    nk = int(rng.integers(1, 4))
    key_ids = [int(c) for c in rng.choice([1, 3, 4, 5, 6, 7], nk, replace=False)]
    inputs = sorted(set(key_ids) | {int(c) for c in rng.choice([2, 3, 8], 2, replace=False)})
    args = {"input ids": inputs, "key ids": key_ids, "key orders": [bool(b) for b in rng.integers(0, 2, nk)]}
    with_limit = bool(seed % 2)
    if with_limit:
        args["limit"] = int(rng.integers(1, n + 1))
    tg = tg_of(ref, {c: cols[c] for c in inputs})
    mine = {c: Variable(torch.from_numpy(cols[c].copy()), TYPES[c]) for c in inputs}
    rows = ref.sort.tqp_sort(False, tg, copy.deepcopy(args), with_limit, "s")
    got_rows = S.tqp_sort(True, mine, copy.deepcopy(args), with_limit, "s")
    assert got_rows == rows
    for c in inputs:
        e, g = tg[c], mine[c]
        assert (g.tensor_type, g.tensor.dtype, tuple(g.tensor.shape)) == (e.tensor_type, e.tensor.dtype,
                                                                          tuple(e.tensor.shape)), c
        np.testing.assert_array_equal(g.tensor.numpy(), e.tensor.numpy(), err_msg=f"column {c} of {args}")


# ------------------------------------------------------------------ whole plans through the drop-in operators
def _install_models(monkeypatch):
    """Every library call of the drop-in operators replaced by the models above."""
    from types import SimpleNamespace  # noqa: F401
    from tqpk import ops
    from tqpk.operators import aggregate as A, filter as F, hashjoin as H, sort as S

    def filter_mask(pred, n, device, with_count=False):
        m = np.asarray(_model_program(pred, {cid: t.numpy() for cid, t in zip(pred.col_ids, pred.tensors)}), bool)
        m = torch.from_numpy(m.reshape(-1).copy()) if n else torch.zeros(0, dtype=torch.bool)
        return m, (torch.tensor([int(m.sum())]) if with_count else None)

    def argsort_stable(keys, descending=False, perm_in=None):
        k = keys.reshape(-1).numpy()
        p = np.arange(k.size) if perm_in is None else perm_in.numpy()
        return torch.from_numpy(p[O._stable_order(k[p], bool(descending))].astype(np.int64))

    monkeypatch.setattr(F, "filter_mask", filter_mask)
    monkeypatch.setattr(A, "groupby", _model_groupby)
    monkeypatch.setattr(A, "encode_keys", _model_encode_keys)
    monkeypatch.setattr(S, "argsort_stable", argsort_stable)
    monkeypatch.setattr(S, "topk_stable", lambda keys, k, descending=False, perm_in=None:
                        argsort_stable(keys, descending, perm_in)[:k])
    monkeypatch.setattr(S, "gather_rows", lambda col, idx: col[idx])
    monkeypatch.setattr(ops, "gather_rows", lambda col, idx: col[idx])
    return A, F, H, S


@pytest.mark.parametrize("seed", range(12))
def test_drop_in_plans_follow_the_reference(ref, monkeypatch, cpu_join_kernels, seed):
    """Filter (build) -> Filter (probe) -> Join -> Aggregate by the build key -> Sort, run by the
    reference's operators and by the drop-in's (library calls modelled) in the order main.py's
    executor runs them: the final columns, their dtypes and type names."""
    from tqpk.variable import Variable
    A, F, H, S = _install_models(monkeypatch)
    rng = np.random.default_rng(1300 + seed)
    nb, npr = int(rng.integers(50, 1500)), int(rng.integers(100, 5000))
    bkey = (rng.permutation(nb) + 1) if seed % 3 else rng.integers(1, nb // 2 + 2, nb)
    cols = {11: bkey.astype(np.int32), 12: rng.integers(0, 2557, nb).astype(np.int32),
            21: rng.integers(1, nb + 40, npr).astype(np.int32), 22: rng.integers(0, 2557, npr).astype(np.int32),
            23: rng.integers(90000, 10495001, npr).astype(np.float64) / 100.0,
            24: rng.integers(0, 11, npr).astype(np.float64) / 100.0}
    types_ = {11: "int", 12: "date", 21: "int", 22: "date", 23: "float", 24: "float"}
    f1 = {"name": "Filter", "filter tree": [["bd#12", "<", str(int(rng.integers(500, 2000)))]], "materialized in": [12],
          "out mask id": 901}
    f2 = {"name": "Filter", "filter tree": [["pd#22", ">", str(int(rng.integers(300, 1500)))]], "materialized in": [22],
          "out mask id": 902}
    jargs = {"name": "Join", "left group": [11, 12], "right group": [21, 22, 23, 24], "materialized in": [11, 21, 23, 24],
             "mask map": {11: 901, 21: 902, 23: 902, 24: 902}, "left keys": [11], "right keys": [21],
             "join type": "Inner"}
    value = [["price#23", "*", ["1.0", "-", "disc#24"]]] if seed % 2 else [["price#23", "*", "disc#24"]]
    aargs = {"name": "Aggregate", "is partial": False, "keys": ["bkey#11"], "input ids": [11, 23, 24],
             "results": ["bkey#11", [[["sum", value], "#", "301"], "AS", "revenue#302"],
                         [[["count", ["1"]], "#", "303L"], "AS", "n#304"]], "out agg ids": [302, 304]}
    if seed % 4 < 2:
        sargs = {"name": "take ordered", "limit": int(rng.integers(1, 30)), "input ids": [11, 302, 304],
                 "key ids": [302, 11], "key orders": [True, False]}
    else:                                                # by the group key, ascending: the sort is the identity
        sargs = {"name": "Sort", "input ids": [11, 302, 304], "key ids": [11], "key orders": [False]}
    limit = "limit" in sargs

    def run(filter_, join, aggregate, sort, V, gpu, pool):
        tg = {c: V(torch.from_numpy(a.copy()), types_[c]) for c, a in cols.items()}
        filter_(gpu, tg, copy.deepcopy(f1), None, None, pool, "f1")
        filter_(gpu, tg, copy.deepcopy(f2), None, None, pool, "f2")
        join(gpu, tg, copy.deepcopy(jargs), 11, 21, [], "inner", None, pool, "j")
        torch.manual_seed(seed)
        aggregate(gpu, tg, copy.deepcopy(aargs), pool, None, "a")
        sort(gpu, tg, copy.deepcopy(sargs), limit, "s")
        return tg

    e = run(ref.filter.tqp_filter, ref.hashjoin.join_vortex, ref.aggregate.tqp_hash_aggregate, ref.sort.tqp_sort,
            ref.variable.Variable, False, _Pool())
    g = run(F.tqp_filter, H.join_vortex, A.tqp_hash_aggregate, S.tqp_sort, Variable, True, None)
    # the reference's group order is a random hash's, so only a sort on keys it can tell apart
    # fixes its rows; ties in the sum are ordered by the key here (the second sort key)
    for c in sargs["input ids"]:
        ev, gv = e[c].tensor.numpy(), g[c].tensor.numpy()
        assert (g[c].tensor_type, gv.dtype, gv.shape) == (e[c].tensor_type, ev.dtype, ev.shape), c
        if ev.dtype.kind == "f":
            assert_f64_close(gv, ev)
        else:
            np.testing.assert_array_equal(gv, ev, err_msg=str(c))


def _full_results(o):
    """Whole result expressions with output id o: arithmetic over aggregates, year(), a CASE counted
    against the null marker, one-byte substrings under sum and count (aggregate.py:100-101,
    :114-119, :179-182, :197-233)."""
    disc = [[col(8), "*", ["1.0", "-", col(2)]]]
    return [
        [[["100.0", "*", [["sum", ["CASE", "WHEN", ["StartsWith", [col(7), "GR"]], "THEN", disc, "ELSE", "0.0", "END"]],
                          "#", "7001"]], "/", [["sum", disc], "#", "7002"]], "AS", f"p#{o}"],
        [[[["sum", ["CASE", "WHEN", [col(7), "=", "GREEN"], "THEN", col(8), "ELSE", "0.0", "END"]], "#", "7003"], "/",
          [["sum", col(8)], "#", "7004"]], "AS", f"q#{o}"],
        [[["min", [["year", [col(1)]]]], "#", "7005"], "AS", f"y#{o}"],
        [[["sum", [["year", [col(1)]]]], "#", "7006L"], "AS", f"v#{o}L"],
        [[["count", ["CASE", "WHEN", [col(8), ">", "50000.5"], "THEN", col(5), "ELSE", "-64.0", "END"]], "#", "7007L"],
         "AS", f"c#{o}L"],
        [[["sum", [["substring", [col(7), "1", "1"]]]], "#", "7008"], "AS", f"s#{o}"],
        [[["count", [["substring", [col(7), "2", "1"]]]], "#", "7009L"], "AS", f"t#{o}L"],
        [[["sum", [[["substring", [col(7), "3", "1"]], "*", "2"]]], "#", "7010"], "AS", f"u#{o}"],
    ]


@pytest.mark.parametrize("seed", range(16))
def test_drop_in_aggregate_operator_whole_expressions(ref, monkeypatch, seed):
    """As above, with arithmetic over aggregates, year(), a CASE counted against the null marker
    and one-byte substrings among the results."""
    from tqpk import ops
    from tqpk.operators import aggregate as A
    from tqpk.variable import Variable
    monkeypatch.setattr(A, "groupby", _model_groupby)
    monkeypatch.setattr(A, "encode_keys", _model_encode_keys)
    monkeypatch.setattr(ops, "_gather_1d", lambda cols, idx, null_aware: [c.reshape(-1)[idx] for c in cols])
    monkeypatch.setattr(ops, "gather_rows", lambda col, idx: col[idx])
    rng = np.random.default_rng(1400 + seed)
    n = int(rng.integers(1, 3000))
    cols = columns(rng, n)
    keys = [KEYS[0], KEYS[1], KEYS[2], KEYS[3]][seed % 4]
    whole = _full_results(0)
    picks = rng.choice(len(whole), int(rng.integers(2, 4)), replace=False)
    results = list(keys) + [_full_results(600 + i)[p] for i, p in enumerate(picks)]
    out_ids = [600 + i for i in range(len(picks))]
    extra = int(rng.integers(0, len(AGGS)))
    results.append([[AGGS[extra], "#", "7100" + ("L" if AGGS[extra][0] == "count" else "")], "AS", "r#700"])
    out_ids.append(700)
    key_ids = [int(k.split("#")[1]) for k in keys]
    used = sorted({c for c in cols if col(c) in repr(results)} | {3})
    args = {"name": "Aggregate", "is partial": False, "keys": keys or None, "input ids": used, "results": results,
            "out agg ids": out_ids}
    cols_in = {c: cols[c] for c in used}
    tg = tg_of(ref, cols_in)
    mine = {c: Variable(torch.from_numpy(np.ascontiguousarray(a).copy()), TYPES.get(c, "int")) for c, a in cols_in.items()}
    torch.manual_seed(seed)
    rows = ref.aggregate.tqp_hash_aggregate(False, tg, copy.deepcopy(args), _Pool(), None, "a")
    got_rows = A.tqp_hash_aggregate(True, mine, copy.deepcopy(args), None, None, "a")
    assert got_rows == rows
    eo = _key_order([tg[k].tensor.numpy() for k in key_ids])
    go = _key_order([mine[k].tensor.numpy() for k in key_ids])
    for oid in out_ids:
        e, g = tg[oid], mine[oid]
        assert (g.tensor_type, g.tensor.dtype, tuple(g.tensor.shape)) == (e.tensor_type, e.tensor.dtype,
                                                                          tuple(e.tensor.shape)), (oid, results)
        ev, gv = e.tensor.numpy(), g.tensor.numpy()
        if keys:
            ev, gv = ev[eo], gv[go]
        if ev.dtype == np.float32:
            np.testing.assert_allclose(gv, ev, rtol=2e-6, atol=2e-6 * max(1.0, float(np.abs(ev).max(initial=0))))
        elif ev.dtype.kind == "f":
            assert_f64_close(gv, ev)
        else:
            np.testing.assert_array_equal(gv, ev, err_msg=str(oid))


@pytest.mark.parametrize("seed", range(4))
def test_drop_in_star_plan_follows_the_reference(ref, monkeypatch, cpu_join_kernels, seed):
    """The star plan (Filter A; fact ⋈ A; ⋈ B; ⋈ C; sum and count by the C key; take ordered),
    each join's outputs the next one's inputs, through the reference's operators and the
    drop-in's (library calls modelled)."""
    from tqpk import datagen
    from tqpk.variable import Variable
    A, F, H, S = _install_models(monkeypatch)
    t = datagen.star_tables(20_000, 2_000, 3_000, 400, 70 + seed)
    cols = {31: t["a_key"], 32: t["a_cat"], 41: t["f_fka"], 42: t["f_fkb"], 43: t["f_price"], 44: t["f_discount"],
            51: t["b_key"], 52: t["b_fkc"], 61: t["c_key"]}
    types_ = {31: "int", 32: "int", 41: "int", 42: "int", 43: "float", 44: "float", 51: "int", 52: "int", 61: "int"}
    results = ["c#61", [[["sum", [["p#43", "*", ["1.0", "-", "d#44"]]]], "#", "71"], "AS", "rev#72"],
               [[["count", ["1"]], "#", "73L"], "AS", "cnt#74"]]
    plan = [
        ("f", {"name": "Filter", "filter tree": [["cat#32", "=", "1"]], "materialized in": [32], "out mask id": 901}),
        ("j", {"name": "Join", "left group": [31, 32], "right group": [41, 42, 43, 44],
               "materialized in": [31, 41, 42, 43, 44], "mask map": {31: 901}}, 31, 41),
        ("j", {"name": "Join", "left group": [51, 52], "right group": [31, 41, 42, 43, 44],
               "materialized in": [51, 52, 42, 43, 44]}, 51, 42),
        ("j", {"name": "Join", "left group": [61], "right group": [51, 52, 42, 43, 44],
               "materialized in": [61, 52, 43, 44]}, 61, 52),
        ("a", {"name": "Aggregate", "is partial": False, "keys": ["c#61"], "input ids": [61, 43, 44],
               "results": results, "out agg ids": [72, 74]}),
        ("t", {"name": "take ordered", "limit": 25, "input ids": [61, 72, 74], "key ids": [72], "key orders": [True]}),
    ]

    def run(filter_, join, aggregate, sort, V, gpu, pool):
        tg = {c: V(torch.from_numpy(a.copy()), types_[c]) for c, a in cols.items()}
        for step in plan:
            kind, a = step[0], copy.deepcopy(step[1])
            if kind == "f":
                filter_(gpu, tg, a, None, None, pool, "f")
            elif kind == "j":
                join(gpu, tg, a, step[2], step[3], [], "inner", None, pool, "j")
            elif kind == "a":
                torch.manual_seed(seed)
                aggregate(gpu, tg, a, pool, None, "a")
            else:
                sort(gpu, tg, a, True, "t")
        return tg

    e = run(ref.filter.tqp_filter, ref.hashjoin.join_vortex, ref.aggregate.tqp_hash_aggregate, ref.sort.tqp_sort,
            ref.variable.Variable, False, _Pool())
    g = run(F.tqp_filter, H.join_vortex, A.tqp_hash_aggregate, S.tqp_sort, Variable, True, None)
    for c in (61, 72, 74):
        ev, gv = e[c].tensor.numpy(), g[c].tensor.numpy()
        assert (g[c].tensor_type, gv.dtype, gv.shape) == (e[c].tensor_type, ev.dtype, ev.shape), c
        if ev.dtype.kind == "f":
            assert_f64_close(gv, ev)
        else:
            np.testing.assert_array_equal(gv, ev, err_msg=str(c))
