"""Host-side compilers (filter trees, aggregate trees) on CPU tensors: no GPU."""
import numpy as np
import pytest
import torch

from tqpk import _lib as L
from tqpk.expr import compile_aggregate
from tqpk.predicate import EPS, compile_filter


def cols():
    return {1: torch.zeros(8, dtype=torch.int32), 2: torch.zeros(8, dtype=torch.float64),
            3: torch.zeros(8, dtype=torch.int64), 4: torch.zeros(8, dtype=torch.uint8)}


def insns(p):
    return [(i.op, i.col, i.cmp, i.domain, i.lit_i, i.lit_f, i.lit_aux) for i in p.struct.insn[:p.struct.n_insn]]


def test_int_compare_and_isnotnull():
    p = compile_filter([[["isnotnull", ["d#1"]], "AND", ["d#1", "<=", "2470"]]], cols())
    assert insns(p) == [(L.P_TRUE, 0, 0, 0, 0, 0.0, 0.0), (L.P_CMP, 0, L.LE, L.DOM_I64, 2470, 0.0, 0.0),
                        (L.P_AND, 0, 0, 0, 0, 0.0, 0.0)]


def test_float_literal_gets_eps_like_reference():
    p = compile_filter(["x#2", "<=", "0.05"], cols())
    assert insns(p)[0][5] == 0.05 + EPS
    p = compile_filter(["x#2", ">=", "0.05"], cols())
    assert insns(p)[0][5] == 0.05 - EPS
    p = compile_filter(["x#2", "<", "0.05"], cols())
    assert insns(p)[0][5] == 0.05


def test_float_equality_is_isclose():
    (op, col, cmp, dom, li, lf, la), = insns(compile_filter(["x#2", "=", "0.06"], cols()))
    assert cmp == L.ISCLOSE and lf == 0.06 and la == EPS + abs(1e-5 * 0.06)


def test_int_column_vs_float_literal_is_float32():
    (op, col, cmp, dom, li, lf, la), = insns(compile_filter(["d#1", "<=", "100.5"], cols()))
    assert dom == L.DOM_F32 and lf == float(np.float32(100.5 + EPS))


def test_date_literal_and_char_literal():
    (i,) = insns(compile_filter(["d#1", "<", "1993-03-15"], cols()))
    assert i[4] == (np.datetime64("1993-03-15") - np.datetime64("1990-01-01")).astype(int)
    (i,) = insns(compile_filter(["c#4", "=", "B"], cols()))
    assert i[4] == ord("B")


def test_in_list_and_not():
    p = compile_filter(["NOT", [["k#3", "IN", ["1", "5"]]]], cols())
    ops = [x[0] for x in insns(p)]
    assert ops == [L.P_CMP, L.P_CMP, L.P_OR, L.P_NOT]


def test_unsupported_raise_loudly():
    with pytest.raises(NotImplementedError):
        compile_filter(["StartsWith", ["c#4", "AB"]], cols())
    with pytest.raises(ValueError):
        compile_filter(["d#1", "<>", "3"], cols())
    with pytest.raises(TypeError):
        compile_filter(["x#2", "=", "3"], cols())


def test_aggregate_program_shares_subexpressions():
    t = {i: torch.zeros(4, dtype=torch.float64) for i in (1, 2, 3, 4)}
    t[5] = torch.zeros(4, dtype=torch.uint8)
    t[6] = torch.zeros(4, dtype=torch.uint8)
    res = ["f#5", "s#6",
           [[["sum", [["p#2", "*", ["1.0", "-", "d#3"]]]], "#", "1"], "AS", "a#201"],
           [[["sum", [[["p#2", "*", ["1.0", "-", "d#3"]], "*", ["1.0", "+", "t#4"]]]], "#", "2"], "AS", "b#202"],
           [[["avg", ["q#1"]], "#", "3"], "AS", "c#203"],
           [[["sum", ["q#1"]], "#", "4"], "AS", "e#204"],
           [[["count", ["1"]], "#", "5L"], "AS", "g#205"]]
    prog = compile_aggregate({"keys": ["f#5", "s#6"], "results": res}, t)
    s = prog.spec
    ops = [s.expr[i].op for i in range(s.n_expr)]
    # p, 1.0, d, (1-d), p*(1-d), t, (1+t), *, q : 4 arithmetic instructions only
    assert sum(o in (L.X_ADD, L.X_SUB, L.X_MUL) for o in ops) == 4
    # accumulators: rows, sum(p*(1-d)), sum(charge), sum(q)   (avg(q) and sum(q) share one)
    assert s.n_accs == 4
    assert [o[1] for o in prog.outputs] == [L.OUT_ACC, L.OUT_ACC, L.OUT_AVG, L.OUT_ACC, L.OUT_ACC]
    assert prog.outputs[-1][2] == 0  # count(1) reads the row count


def test_aggregate_dtypes_follow_torch():
    t = {1: torch.zeros(4, dtype=torch.int32), 2: torch.zeros(4, dtype=torch.float64)}
    res = [[[["min", ["d#1"]], "#", "1"], "AS", "a#11"], [[["sum", ["d#1"]], "#", "2"], "AS", "b#12"],
           [[["max", ["x#2"]], "#", "3"], "AS", "c#13"]]
    prog = compile_aggregate({"keys": None, "results": res}, t)
    assert [o[4] for o in prog.outputs] == [torch.int32, torch.int64, torch.float64]
    # an integer column with a Python float is float32 in torch: float32 registers, the sum
    # accumulated in float64 and returned as float32
    p32 = compile_aggregate({"keys": None, "results": [[[["sum", [["d#1", "*", "0.5"]]], "#", "1"], "AS", "a#1"],
                                                       [[["avg", [["d#1", "/", "d#1"]]], "#", "2"], "AS", "b#2"]]}, t)
    types = [p32.spec.expr[i].type for i in range(p32.spec.n_expr)]
    assert L.F32 in types and p32.casts == {1: (torch.float32, False), 2: (torch.float32, True)}
    assert all(p32.spec.expr[p32.spec.accs[a].reg].type != L.F32 for a in range(1, p32.spec.n_accs))
    with pytest.raises(NotImplementedError):      # arithmetic over such an aggregate stays off the kernels
        compile_aggregate({"keys": None, "results": [[["2", "*", [[["sum", [["d#1", "*", "0.5"]]], "#", "1"]]],
                                                      "AS", "a#1"]]}, t, derived=True)
