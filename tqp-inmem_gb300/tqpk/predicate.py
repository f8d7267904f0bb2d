"""Compiles TQP-Inmem filter trees into the device predicate program.

The input is the parsed tree the reference's ``operators/filter.py:evaluate``
walks (``filter.py:14-162``): nested lists of strings such as
``[['isnotnull', ['d#7']], 'AND', ['d#7', '<=', '1998-09-02']]``.  The output
is a postfix ``tqpk_predicate`` (include/tqpk.h) whose comparisons carry the
reference's exact semantics:

* float literals with ``<=``/``>=`` get the reference's ``+-eps``
  (``filter.py:145-149``), computed here in Python double arithmetic exactly
  as the reference does;
* ``=`` on a float64 column is ``torch.isclose(atol=eps)`` (``:160-161``); the
  allowed error ``atol + |rtol * lit|`` is precomputed the same way;
* an integer column against a Python float compares in float32, the dtype
  torch promotes that pair to;
* ``isnotnull`` is all-true (``:67-69``), ``IN`` is an OR of equalities
  (``:90-119``), a one-character string literal compares with ``ord``.

String columns are int8 ``[N, w]`` tensors (zero padded, conversion.py:36-37):
``StartsWith`` (``:48-55``), ``Contains`` / ``EndsWith`` (``:56-62``, the
reference treats both as a substring search), ``LIKE '%a%b%'`` (``:121-127``),
a multi-character literal compared byte-wise against the literal padded to w
(``:151-158``) and ``IN`` lists of such literals compile to the string
instructions; their literal bytes go to the predicate's string pool.
``substring(col, start, width)`` is a view of a string column (pointer offset,
its own width, the column's row stride), usable wherever a string column is.
"""
from __future__ import annotations

import datetime as _dt
from dataclasses import dataclass, field
from typing import Any, Dict, List

import numpy as np

from . import _lib as L
from .dtypes import code_of

EPS = 1e-5        # constants.py:8
RTOL = 1e-5       # torch.isclose default rtol
_EPOCH = _dt.date(1990, 1, 1)   # conversion.py:11

_CMP = {"<": L.LT, "<=": L.LE, ">": L.GT, ">=": L.GE, "=": L.EQ, "<>": L.NE}
_FLIP = {"<": ">", "<=": ">=", ">": "<", ">=": "<=", "=": "=", "<>": "<>"}


def get_id(name: str) -> int:
    """parsing.py:15-16"""
    return int(name.split("#")[-1].replace("L", ""))


def _is_date(s: str) -> bool:
    return len(s) == 10 and s.count("-") == 2 and s.replace("-", "").isdigit()


def _is_float(s: str) -> bool:
    return s.replace(".", "").replace("-", "").replace("E", "").isdigit()


@dataclass
class _Col:
    cid: int


@dataclass
class _Sub:
    """substring(col, start, width): the byte columns [start-1, start-1+width) of a string
    column (filter.py:71-76, a strided view; Python slicing clips at the row's end)."""
    cid: int
    start: int
    width: int

    @property
    def key(self):
        return ("sub", self.cid, self.start, self.width)


@dataclass
class CompiledPredicate:
    """A predicate program plus the column tensors it reads (kept alive)."""
    struct: Any
    tensors: List[Any] = field(default_factory=list)
    col_ids: List[int] = field(default_factory=list)

    def bind(self):
        return self.struct


class _Compiler:
    def __init__(self, columns: Dict[int, Any], subquery=None, agg: bool = False):
        self.columns = columns
        self.subquery = subquery
        self.agg = agg          # the comparison rules of aggregate.py:203-233 instead of filter.py's
        self.insn: List[tuple] = []
        self.slots: Dict[int, int] = {}
        self.str_cols = set()
        self.pool = b""

    # -- values -------------------------------------------------------------
    def value(self, tree):
        if self.agg:
            return self._agg_value(tree)
        if isinstance(tree, str):
            if tree == "Subquery":
                if self.subquery is None:
                    raise ValueError("filter references a subquery result but none was given")
                return self.subquery
            if _is_date(tree):
                return (_dt.date.fromisoformat(tree) - _EPOCH).days
            if _is_float(tree):
                return float(tree) if "." in tree else int(tree)
            if "#" in tree and not tree.startswith("Brand#"):
                return _Col(get_id(tree))
            return tree
        if len(tree) == 1:
            return self.value(tree[0])
        if len(tree) == 3 and tree[1] == "#":
            return _Col(int(tree[-1]))
        if len(tree) == 2 and tree[0] == "cast":
            literal, _, cast_type = tree[1][0].split(" ")
            if cast_type == "double":
                return self.value(literal)
        if len(tree) == 2 and tree[0] == "substring":
            assert len(tree[1]) == 3
            col, start, width = tree[1]
            base = self.value(col)
            if not isinstance(base, _Col):
                raise NotImplementedError("substring of a non-column operand")
            W = self.str_tensor(base.cid).shape[-1]
            l0, w = int(start) - 1, int(width)
            if l0 < 0 or w <= 0 or l0 >= W:
                raise NotImplementedError(f"substring({start}, {width}) of a {W}-byte column")
            return _Sub(base.cid, l0, min(W, l0 + w) - l0)
        return None  # a boolean sub-expression

    def _agg_value(self, tree):
        """Operands as aggregate.py:58-67 and :203-233 read them: digits are ints, other
        numbers floats, `1 - URGENT` (a literal the plan parser split at '-') joins back
        into the string '1-URGENT' (:224-227)."""
        if isinstance(tree, str):
            if tree.isdigit():
                return int(tree)
            if _is_float(tree):
                return float(tree)               # a date literal raises here, as float() does there
            if "#" in tree and tree.split("#")[-1].replace("L", "").isdigit():
                return _Col(get_id(tree))
            return tree
        if len(tree) == 1:
            return self._agg_value(tree[0])
        if len(tree) == 3 and tree[1] == "#":
            return self._agg_value(tree[0])
        if len(tree) == 2 and tree[0] == "cast":
            literal, _, cast_type = tree[1][0].split(" ")
            if cast_type == "double":
                return self._agg_value(literal)
        if len(tree) == 3 and tree[1] == "-":
            lv, rv = self._agg_value(tree[0]), self._agg_value(tree[2])
            if isinstance(lv, int) and isinstance(rv, str):
                return "".join(tree)
        return None

    def slot(self, cid) -> int:
        """Slot of a column id, or of a substring view key ('sub', id, start, width)."""
        if cid not in self.slots:
            if (cid[1] if isinstance(cid, tuple) else cid) not in self.columns:
                raise KeyError(f"filter column {cid} is not among the operator's inputs")
            if len(self.slots) >= L.MAX_COLS:
                raise NotImplementedError(f"predicate reads more than {L.MAX_COLS} columns")
            self.slots[cid] = len(self.slots)
        return self.slots[cid]

    def col_tensor(self, cid: int):
        t = self.columns[cid]
        if t.dim() == 2 and t.shape[1] == 1:
            t = t.reshape(-1)
        if t.dim() != 1:
            raise NotImplementedError("a string (2-D) column is compared only by the string predicates")
        return t

    def str_tensor(self, cid: int):
        t = self.columns[cid]
        if t.dim() != 2 or t.dtype not in (torch_int8(), torch_uint8()):
            raise NotImplementedError("string predicates take int8 [N, w] columns")
        return t

    def pool_add(self, data: bytes) -> int:
        off = len(self.pool)
        if off + len(data) > L.MAX_STRPOOL:
            raise NotImplementedError(f"string literals exceed {L.MAX_STRPOOL} bytes")
        self.pool += data
        return off

    def emit_str(self, op: int, cid: int, cmp: int, lit: int):
        self.str_cols.add(cid)
        self.insn.append((op, self.slot(cid), cmp, 0, lit, 0.0, 0.0))

    @staticmethod
    def _bytes(s: str, w: int) -> bytes:
        """conversion.py:36-37: character codes padded with zeros to w (np.pad raises past w)."""
        codes = [ord(c) for c in s]
        if len(codes) > w:
            raise ValueError(f"string literal {s!r} is longer than the column ({w} bytes)")
        if any(c > 255 for c in codes):
            raise NotImplementedError("non-byte characters in a string literal")
        return bytes(codes) + bytes(w - len(codes))

    def dtype(self, cid: int) -> int:
        return code_of(self.col_tensor(cid).dtype)

    # -- emission -------------------------------------------------------------
    def emit_cmp(self, col: _Col, op: str, lit):
        dt = self.dtype(col.cid)
        s = self.slot(col.cid)
        if dt == L.F64:
            self.insn.append((L.P_CMP, s, _CMP[op], L.DOM_F64, 0, float(lit), 0.0))
        elif isinstance(lit, float):
            self.insn.append((L.P_CMP, s, _CMP[op], L.DOM_F32, 0, float(np.float32(lit)), 0.0))
        else:
            self.insn.append((L.P_CMP, s, _CMP[op], L.DOM_I64, int(lit), 0.0, 0.0))

    def emit(self, tree):
        """Emits code that pushes a bool mask for `tree`."""
        if isinstance(tree, list) and len(tree) == 1:
            return self.emit(tree[0])
        if isinstance(tree, str) or (len(tree) == 3 and tree[1] == "#"):
            v = self.value(tree)
            if isinstance(v, _Col) and self.col_tensor(v.cid).dtype.is_floating_point is False \
                    and self.dtype(v.cid) in (L.BOOL,):
                self.insn.append((L.P_MASK, self.slot(v.cid), 0, 0, 0, 0.0, 0.0))
                return
            raise NotImplementedError(f"filter leaf {tree!r} is not a boolean")
        if len(tree) == 2:
            head = tree[0]
            if head == "NOT":
                self.emit(tree[1])
                self.insn.append((L.P_NOT, 0, 0, 0, 0, 0.0, 0.0))
                return
            if self.agg and head not in ("StartsWith",):        # aggregate.py:89-122
                raise ValueError(f"Unsupported aggregation function: {head}")
            if head == "isnotnull":
                self.insn.append((L.P_TRUE, 0, 0, 0, 0, 0.0, 0.0))
                return
            if head in ("StartsWith", "EndsWith", "Contains"):
                cid, name = get_id(tree[1][0]), tree[1][1]
                t = self.str_tensor(cid)
                if head == "StartsWith":
                    assert t.shape[-1] >= len(name)                       # filter.py:51
                data = self._bytes(name, len(name))
                off = self.pool_add(data)
                self.emit_str(L.P_PREFIX if head == "StartsWith" else L.P_CONTAINS, cid, 0, off | (len(data) << 32))
                return
            if head == "substring":
                raise NotImplementedError(f"filter leaf {tree!r} is not a boolean")
            raise ValueError(f"Unsupported Function: {head}")
        op = tree[-2]
        if self.agg and op in ("IN", "LIKE"):                  # aggregate.py:206-222
            raise ValueError(f"Unsupported Operation: {op}")
        if op == "IN":
            L_ = self.value(tree[0])
            if isinstance(L_, _Sub):                             # filter.py:110-113 on a [N, w] slice
                if not tree[-1]:
                    self.insn.append((L.P_FALSE, 0, 0, 0, 0, 0.0, 0.0))
                    return
                for i, r in enumerate(tree[-1]):
                    assert len(r) != 1, "single characters against a string column (filter.py:111)"
                    self.emit_str(L.P_STRCMP, L_.key, L.EQ, self.pool_add(self._bytes(r, L_.width)))
                    if i:
                        self.insn.append((L.P_OR, 0, 0, 0, 0, 0.0, 0.0))
                return
            if not isinstance(L_, _Col):
                raise NotImplementedError("IN on a non-column operand")
            if self.columns[L_.cid].dim() == 2 and self.columns[L_.cid].shape[1] != 1:   # filter.py:110-113
                w = self.str_tensor(L_.cid).shape[-1]
                if not tree[-1]:
                    self.insn.append((L.P_FALSE, 0, 0, 0, 0, 0.0, 0.0))
                    return
                for i, r in enumerate(tree[-1]):
                    assert len(r) != 1, "single characters against a string column (filter.py:111)"
                    self.emit_str(L.P_STRCMP, L_.cid, L.EQ, self.pool_add(self._bytes(r, w)))
                    if i:
                        self.insn.append((L.P_OR, 0, 0, 0, 0, 0.0, 0.0))
                return
            dt = self.dtype(L_.cid)
            if dt in (L.I64, L.I32):
                vals = [int(r) for r in tree[-1]]
            elif dt == L.F64:
                vals = [float(r) for r in tree[-1]]
            else:
                raise AssertionError("IN supports int/date/float columns only (filter.py:96-102)")
            if not vals:
                self.insn.append((L.P_FALSE, 0, 0, 0, 0, 0.0, 0.0))
                return
            for i, r in enumerate(vals):
                self.emit_cmp(L_, "=", r) if dt != L.F64 else self.insn.append(
                    (L.P_CMP, self.slot(L_.cid), L.EQ, L.DOM_F64, 0, r, 0.0))
                if i:
                    self.insn.append((L.P_OR, 0, 0, 0, 0, 0.0, 0.0))
            return
        if op == "LIKE":                                   # filter.py:121-127
            L_ = self.value(tree[0])
            if not isinstance(L_, _Col):
                raise NotImplementedError("LIKE on a non-column operand")
            self.str_tensor(L_.cid)
            assert tree[-1].count("%") == 3
            _, w1, w2, _ = tree[-1].split("%")
            a, b = self._bytes(w1, len(w1)), self._bytes(w2, len(w2))
            oa, ob = self.pool_add(a), self.pool_add(b)
            self.emit_str(L.P_LIKE2, L_.cid, 0, oa | (len(a) << 16) | (ob << 32) | (len(b) << 48))
            return
        if op in ("AND", "OR"):
            self.emit(tree[0])
            self.emit(tree[-1])
            self.insn.append((L.P_AND if op == "AND" else L.P_OR, 0, 0, 0, 0, 0.0, 0.0))
            return
        if op not in ("<=", ">=", "<", ">", "=") + (("<>",) if self.agg else ()):
            raise ValueError(f"Unsupported Operation: {op}")
        Lv = self.value(tree[0])
        Rv = self.value(tree[-1])
        if self.agg:
            return self._agg_cmp(tree, op, Lv, Rv)
        if isinstance(Lv, _Col) and isinstance(Rv, _Col):
            da, db = self.dtype(Lv.cid), self.dtype(Rv.cid)
            dom = L.DOM_F64 if L.F64 in (da, db) else L.DOM_I64
            self.insn.append((L.P_CMPCOL, self.slot(Lv.cid), _CMP[op], dom, self.slot(Rv.cid), 0.0, 0.0))
            return
        if isinstance(Lv, _Sub) and isinstance(Rv, str) and len(Rv) > 1:      # filter.py:151-158 on a slice
            return self.emit_str(L.P_STRCMP, Lv.key, L.EQ, self.pool_add(self._bytes(Rv, Lv.width)))
        if not isinstance(Lv, _Col):
            if isinstance(Rv, _Col):      # literal <op> column: same comparison mirrored
                Lv, Rv, op = Rv, Lv, _FLIP[op]
            else:
                raise NotImplementedError(f"comparison without a column operand: {tree!r}")
        if isinstance(Rv, float):                          # filter.py:145-149
            if op == "<=":
                return self.emit_cmp(Lv, "<=", Rv + EPS)
            if op == ">=":
                return self.emit_cmp(Lv, ">=", Rv - EPS)
        if isinstance(Rv, str):                            # filter.py:151-158
            if len(Rv) == 1:
                return self.emit_cmp(Lv, op, ord(Rv))
            t = self.columns[Lv.cid]
            if t.dim() != 2:
                raise NotImplementedError("multi-character literal against a one-dimensional column")
            w = self.str_tensor(Lv.cid).shape[-1]
            # (L == R).all(dim=1) whatever the operator (filter.py:158)
            return self.emit_str(L.P_STRCMP, Lv.cid, L.EQ, self.pool_add(self._bytes(Rv, w)))
        if op == "=" and self.dtype(Lv.cid) == L.F64:     # filter.py:160-161
            if not isinstance(Rv, float):
                raise TypeError("isclose against a non-float literal (the reference raises here too)")
            allowed = EPS + abs(RTOL * Rv)
            self.insn.append((L.P_CMP, self.slot(Lv.cid), L.ISCLOSE, L.DOM_F64, 0, Rv, allowed))
            return
        return self.emit_cmp(Lv, op, Rv)

    def _agg_cmp(self, tree, op, Lv, Rv):
        """aggregate.py:224-233: ops[op](L, R) on tensors and Python numbers."""
        if isinstance(Lv, _Col) and isinstance(Rv, _Col):
            da, db = self.dtype(Lv.cid), self.dtype(Rv.cid)
            dom = L.DOM_F64 if L.F64 in (da, db) else L.DOM_I64
            self.insn.append((L.P_CMPCOL, self.slot(Lv.cid), _CMP[op], dom, self.slot(Rv.cid), 0.0, 0.0))
            return
        if isinstance(Rv, str):
            if not isinstance(Lv, _Col):
                raise NotImplementedError(f"string comparison without a column operand: {tree!r}")
            if len(Rv) == 1:
                return self.emit_cmp(Lv, op, ord(Rv))
            w = self.str_tensor(Lv.cid).shape[-1]
            return self.emit_str(L.P_STRCMP, Lv.cid, L.EQ, self.pool_add(self._bytes(Rv, w)))
        if not isinstance(Lv, _Col):
            if isinstance(Rv, _Col) and isinstance(Lv, (int, float)):
                Lv, Rv, op = Rv, Lv, _FLIP[op]
            else:
                raise NotImplementedError(f"comparison without a column operand: {tree!r}")
        if not isinstance(Rv, (int, float)):
            raise NotImplementedError(f"comparison operand {tree[-1]!r} is not on the kernel path")
        return self.emit_cmp(Lv, op, Rv)


def compile_filter(tree, columns: Dict[int, Any], subquery=None, agg: bool = False) -> CompiledPredicate:
    """Compiles a filter tree over ``columns`` (id -> 1-D device tensor).  With agg the
    tree is a condition inside an aggregate or projection expression and compares as
    aggregate.py:203-233 does: torch.le/ge/eq/ne without the filter's eps and isclose,
    `<>` allowed, a multi-character string literal tested for equality whatever the
    operator (:229-231), IN/LIKE and functions other than NOT/StartsWith rejected."""
    c = _Compiler(columns, subquery, agg)
    c.emit(tree)
    if len(c.insn) > L.MAX_PRED:
        raise NotImplementedError(f"predicate longer than {L.MAX_PRED} instructions")
    p = L.Predicate()
    p.n_insn = len(c.insn)
    p.n_cols = len(c.slots)
    tensors = []
    ids = [None] * len(c.slots)
    for cid, s in c.slots.items():
        if isinstance(cid, tuple):                     # substring view: offset pointer, own width, row stride
            _, base_id, start, width = cid
            t = c.str_tensor(base_id).contiguous()
            tensors.append(t)
            ids[s] = base_id
            p.cols[s] = t.data_ptr() + start
            p.widths[s] = width
            p.strides[s] = int(t.shape[1])
            p.dtypes[s] = code_of(t.dtype)
            continue
        if cid in c.str_cols:
            t = c.str_tensor(cid).contiguous()
            p.widths[s] = int(t.shape[1])
        else:
            t = c.col_tensor(cid).contiguous()
        tensors.append(t)
        ids[s] = cid
        p.cols[s] = t.data_ptr()
        p.dtypes[s] = code_of(t.dtype)
    for i, (op, col, cmp, dom, li, lf, la) in enumerate(c.insn):
        p.insn[i] = L.PredInsn(op, col, cmp, dom, li, lf, la)
    for i, b in enumerate(c.pool):
        p.strpool[i] = b
    return CompiledPredicate(p, tensors, ids)


def has_strings(P) -> bool:
    """The predicate uses string instructions (only the library's evaluator runs them)."""
    return P is not None and any(P.insn[k].op in (L.P_STRCMP, L.P_PREFIX, L.P_CONTAINS, L.P_LIKE2)
                                 for k in range(P.n_insn))


def torch_int8():
    import torch
    return torch.int8


def torch_uint8():
    import torch
    return torch.uint8
