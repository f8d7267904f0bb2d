"""Compiles TQP-Inmem aggregate ``results`` trees into one device program.

Input: the ``args['results']`` list of ``tqp_hash_aggregate``
(``operators/aggregate.py:236-393``), e.g.
``[[['sum', [['price#2', '*', ['1.0', '-', 'disc#3']]]], '#', '103'], 'AS', 'rev#203']``.

Output: a ``tqpk_groupby_spec`` with
* one straight-line expression program shared by every aggregate (common
  subexpressions such as ``price * (1 - disc)`` are computed once per row),
* a deduplicated accumulator list (``avg(x)`` reuses ``sum(x)``; every
  ``avg`` divides by accumulator 0, the group's row count),
* output ops that reproduce the reference's result dtypes: float sums and
  averages in float64, integer sums and counts in int64 (``:184-193``),
  ``min``/``max`` in the expression's own dtype (``:154-167``).

Arithmetic follows torch's promotion (``aggregate.py:203-233`` applies
torch.add/sub/mul/div to tensors and Python numbers): float64 wins; integer
tensors with Python ints stay integer.  An integer tensor combined with a
Python float, or an integer true division, is float32 in torch; those are
rejected with NotImplementedError rather than computed differently.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Dict, List, Tuple

import torch

from . import _lib as L
from .dtypes import code_of
from .predicate import get_id, _is_float

_AGG_FNS = ("sum", "avg", "count", "min", "max")
_INT_ORDER = {torch.bool: 0, torch.uint8: 1, torch.int8: 1, torch.int32: 3, torch.int64: 4}


def _strip(t):
    while isinstance(t, list) and len(t) == 1:
        t = t[0]
    return t


def right_most(tree):
    """parsing.py:42-45"""
    return right_most(tree[-1]) if isinstance(tree, list) else tree


def is_key_result(tree) -> bool:
    """aggregate.py:268 / parsing.py:94"""
    return isinstance(tree, str) or (len(tree) == 3 and tree[1] == "AS" and isinstance(tree[0], str))


@dataclass
class _Node:
    reg: int
    f64: bool
    dtype: torch.dtype


@dataclass
class AggregateProgram:
    spec: Any
    tensors: List[torch.Tensor] = field(default_factory=list)
    key_ids: List[int] = field(default_factory=list)        # grouping columns (args['keys'])
    key_outputs: List[Tuple[int, int]] = field(default_factory=list)   # (out id, input key id)
    outputs: List[Tuple[int, int, int, int, torch.dtype]] = field(default_factory=list)  # (out id, op, a, b, dtype)


class _Builder:
    def __init__(self, columns: Dict[int, torch.Tensor]):
        self.columns = columns
        self.expr: List[tuple] = []
        self.memo: Dict[tuple, int] = {}
        self.col_slot: Dict[int, int] = {}
        self.col_tensors: List[torch.Tensor] = []
        self.accs: List[tuple] = [(L.ACC_COUNT_ROWS, L.I64, 0, 0, 0.0)]
        self.acc_memo: Dict[tuple, int] = {}

    def _insn(self, key, op, f64, a=0, b=0, col=0, ci=0, cf=0.0) -> int:
        if key in self.memo:
            return self.memo[key]
        if len(self.expr) >= L.MAX_EXPR:
            raise NotImplementedError(f"aggregate expressions exceed {L.MAX_EXPR} instructions")
        self.expr.append((op, L.F64 if f64 else L.I64, a, b, col, ci, cf))
        self.memo[key] = len(self.expr) - 1
        return self.memo[key]

    def column(self, cid: int) -> _Node:
        t = self.columns[cid]
        if t.dim() == 2 and t.shape[1] == 1:
            t = t.reshape(-1)
        if t.dim() != 1:
            raise NotImplementedError("string (2-D) columns in aggregate expressions are not on the kernel path")
        if t.dtype not in (torch.float64, *_INT_ORDER):
            raise TypeError(f"aggregate column dtype {t.dtype} is not handled")
        if cid not in self.col_slot:
            if len(self.col_slot) >= L.MAX_COLS:
                raise NotImplementedError(f"aggregate reads more than {L.MAX_COLS} columns")
            t = t.contiguous()
            self.col_slot[cid] = len(self.col_tensors)
            self.col_tensors.append(t)
        f64 = t.dtype == torch.float64
        reg = self._insn(("col", cid), L.X_COL, f64, col=self.col_slot[cid])
        return _Node(reg, f64, t.dtype)

    def const(self, v) -> _Node:
        if isinstance(v, float):
            return _Node(self._insn(("cf", v), L.X_CONST, True, cf=v), True, torch.float64)
        return _Node(self._insn(("ci", v), L.X_CONST, False, ci=int(v)), False, torch.int64)

    def to_f64(self, n: _Node) -> int:
        return n.reg if n.f64 else self._insn(("tof64", n.reg), L.X_TOF64, True, a=n.reg)

    def value(self, tree):
        """aggregate.py:58-233 arithmetic: returns a _Node or a Python number."""
        if isinstance(tree, str):
            if tree.isdigit():
                return int(tree)
            if _is_float(tree):
                return float(tree)
            if "#" in tree and tree.split("#")[-1].replace("L", "").isdigit():
                return self.column(get_id(tree))
            raise NotImplementedError(f"aggregate operand {tree!r}")
        tree = _strip(tree)
        if isinstance(tree, str):
            return self.value(tree)
        if len(tree) == 3 and tree[1] in ("#", "AS"):
            return self.value(tree[0])
        if len(tree) == 3 and tree[1] in "+-*/":
            return self.binary(tree[1], self.value(tree[0]), self.value(tree[2]))
        if len(tree) == 2 and tree[0] == "cast":
            literal, _, cast_type = tree[1][0].split(" ")
            if cast_type == "double":
                return self.value(literal)
        raise NotImplementedError(f"aggregate expression {tree!r} is not on the kernel path")

    def binary(self, op: str, a, b):
        op_code = {"+": L.X_ADD, "-": L.X_SUB, "*": L.X_MUL, "/": L.X_DIV}[op]
        if not isinstance(a, _Node) and not isinstance(b, _Node):
            return {"+": a + b, "-": a - b, "*": a * b, "/": a / b}[op]
        # torch promotion of the pair
        def kind(x):
            if isinstance(x, _Node):
                return "f" if x.f64 else "i"
            return "pf" if isinstance(x, float) else "pi"
        ka, kb = kind(a), kind(b)
        if "f" in (ka, kb):
            f64, dtype = True, torch.float64
        elif "pf" in (ka, kb) or op == "/":
            raise NotImplementedError("integer tensor with a float literal (or integer division) is float32 in torch")
        else:
            ints = [x.dtype for x in (a, b) if isinstance(x, _Node)]
            dtype = max(ints, key=lambda d: _INT_ORDER[d])
            if len(ints) == 2 and {ints[0], ints[1]} == {torch.uint8, torch.int8}:
                raise NotImplementedError("uint8 with int8 promotes to int16 in torch")
            if dtype == torch.bool:
                dtype = torch.int64
            f64 = False
        na = a if isinstance(a, _Node) else self.const(float(a) if f64 else int(a))
        nb = b if isinstance(b, _Node) else self.const(float(b) if f64 else int(b))
        ra = self.to_f64(na) if f64 else na.reg
        rb = self.to_f64(nb) if f64 else nb.reg
        reg = self._insn((op, ra, rb, f64), op_code, f64, a=ra, b=rb)
        return _Node(reg, f64, dtype)

    def acc(self, kind: int, node: _Node, init_i=0, init_f=0.0) -> int:
        key = (kind, node.reg, node.f64, init_i, init_f)
        if key not in self.acc_memo:
            if len(self.accs) >= L.MAX_ACCS:
                raise NotImplementedError(f"more than {L.MAX_ACCS} accumulators")
            self.accs.append((kind, L.F64 if node.f64 else L.I64, node.reg, init_i, init_f))
            self.acc_memo[key] = len(self.accs) - 1
        return self.acc_memo[key]


def _agg_call(tree):
    """Walks [[fn, arg], '#', id] / [.., 'AS', name] down to (fn, arg)."""
    t = _strip(tree)
    while isinstance(t, list) and len(t) == 3 and t[1] in ("#", "AS"):
        t = _strip(t[0])
    if isinstance(t, list) and len(t) == 2 and t[0] in _AGG_FNS:
        return t[0], t[1]
    raise NotImplementedError(f"aggregate result {tree!r}: only plain sum/avg/count/min/max calls run on the kernels")


def compile_aggregate(args: dict, columns: Dict[int, torch.Tensor]) -> AggregateProgram:
    b = _Builder(columns)
    prog = AggregateProgram(spec=None)
    prog.key_ids = [get_id(k) for k in (args.get("keys") or [])]
    if len(prog.key_ids) > L.MAX_KEYS:
        raise NotImplementedError(f"more than {L.MAX_KEYS} group keys")
    for tree in args["results"]:
        tree = _strip(tree)
        oid = get_id(right_most(tree))
        if is_key_result(tree):
            prog.key_outputs.append((oid, get_id(tree if isinstance(tree, str) else tree[0])))
            continue
        fn, arg = _agg_call(tree)
        v = b.value(arg)
        scalar = not isinstance(v, _Node)
        if fn == "count" and scalar and v != L.NULL_INDEX:  # count(1): every row counts
            prog.outputs.append((oid, L.OUT_ACC, 0, 0, torch.int64))
            continue
        if scalar:                                          # aggregate.py:149-152: full(cnt_rows, v)
            v = b.const(v)
        if fn == "sum":
            a = b.acc(L.ACC_SUM, v)
            prog.outputs.append((oid, L.OUT_ACC, a, 0, torch.float64 if v.f64 else torch.int64))
        elif fn == "avg":
            a = b.acc(L.ACC_SUM, v)
            prog.outputs.append((oid, L.OUT_AVG, a, 0, torch.float64))
        elif fn == "count":
            a = b.acc(L.ACC_COUNT_NOTNULL, v)
            prog.outputs.append((oid, L.OUT_ACC, a, 0, torch.int64))
        elif fn == "min":
            if v.f64:
                a = b.acc(L.ACC_MIN, v, init_f=float(torch.finfo(torch.float64).max))
            else:
                a = b.acc(L.ACC_MIN, v, init_i=int(torch.iinfo(v.dtype if v.dtype != torch.bool else torch.int64).max))
            prog.outputs.append((oid, L.OUT_ACC, a, 0, v.dtype))
        else:  # max starts from zero, as the reference's zeros() initial tensor
            a = b.acc(L.ACC_MAX, v)
            prog.outputs.append((oid, L.OUT_ACC, a, 0, v.dtype))
    if len(prog.outputs) > L.MAX_ACCS:
        raise NotImplementedError(f"more than {L.MAX_ACCS} aggregate outputs")
    s = L.GroupbySpec()
    s.n_keys = len(prog.key_ids)
    for k, kid in enumerate(prog.key_ids):
        t = columns[kid]
        if t.dim() == 2 and t.shape[1] == 1:
            t = t.reshape(-1)
        if t.dim() != 1 or t.dtype not in _INT_ORDER:
            raise NotImplementedError(f"group key {kid} ({t.dtype}, {tuple(t.shape)}) is not an integer column")
        t = t.contiguous()
        prog.tensors.append(t)
        s.keys[k] = t.data_ptr()
        s.key_dtypes[k] = code_of(t.dtype)
    s.n_cols = len(b.col_tensors)
    for i, t in enumerate(b.col_tensors):
        s.cols[i] = t.data_ptr()
        s.col_dtypes[i] = code_of(t.dtype)
    prog.tensors.extend(b.col_tensors)
    s.n_expr = len(b.expr)
    for i, (op, ty, a, bb, col, ci, cf) in enumerate(b.expr):
        s.expr[i] = L.ExprInsn(op, ty, a, bb, col, 0, ci, cf)
    s.n_accs = len(b.accs)
    for i, (kind, ty, reg, ii, ff) in enumerate(b.accs):
        s.accs[i] = L.Acc(kind, ty, reg, 0, ii, ff)
    prog.spec = s
    return prog


@dataclass
class ProjectionProgram:
    spec: Any                                   # expression program (no keys; accumulator 0 only)
    tensors: List[torch.Tensor] = field(default_factory=list)
    outputs: List[Tuple[int, torch.dtype]] = field(default_factory=list)   # (register, result dtype)


def is_trivial_projection(tree) -> bool:
    """A bare column or `column AS name` (project.py:27-31): renamed, not computed."""
    while isinstance(tree, list) and len(tree) == 1:
        tree = tree[0]
    return isinstance(tree, str) or (tree[1] == "AS" and isinstance(tree[0], str))


def compile_projection(trees, columns: Dict[int, torch.Tensor]) -> ProjectionProgram:
    """The computed expressions of a projection (project.py:20-40) as one SSA program: each
    output is a register with the dtype torch gives the expression (aggregate.py:203-233)."""
    b = _Builder(columns)
    outs = []
    for tree in trees:
        while isinstance(tree, list) and len(tree) == 1:
            tree = tree[0]
        if is_trivial_projection(tree):
            continue
        expr = tree[0] if len(tree) > 1 and tree[1] == "AS" else tree
        v = b.value(expr)
        if not isinstance(v, _Node):
            raise NotImplementedError(f"projection of a literal {expr!r}")
        outs.append((v.reg, v.dtype))
    spec = L.GroupbySpec()
    spec.n_keys = 0
    spec.n_cols = len(b.col_tensors)
    for i, t in enumerate(b.col_tensors):
        spec.cols[i] = t.data_ptr()
        spec.col_dtypes[i] = code_of(t.dtype)
    spec.n_expr = len(b.expr)
    for i, (op, ty, a, bb, col, ci, cf) in enumerate(b.expr):
        X = spec.expr[i]
        X.op, X.type, X.a, X.b, X.col, X.ci, X.cf = op, ty, a, bb, col, ci, cf
    spec.n_accs = 1
    spec.accs[0].kind, spec.accs[0].type = L.ACC_COUNT_ROWS, L.I64
    return ProjectionProgram(spec=spec, tensors=list(b.col_tensors), outputs=outs)
