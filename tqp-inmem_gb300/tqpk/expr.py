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
Python float, an integer true division, or a CASE mixing a float literal with
integers is float32 in torch (its default float dtype): those registers are
float32 (TQPK_F32), computed in float32 with round-to-nearest as torch does,
and widened exactly to float64 where they meet a float64 tensor.  An
aggregate of a float32 expression accumulates in float64 and its output is
rounded to float32 (``casts``), the dtype the reference returns (its own
float32 sums round at every row).

With ``derived=True`` (the operator path) the rest of the reference's
expression language compiles too:

* a condition (comparisons, AND/OR, NOT, StartsWith, string equality,
  ``aggregate.py:89-99, 203-233``) becomes a bool column: the condition is a
  predicate program (aggregate comparison rules, no eps) that the filter
  kernel evaluates into a 1-byte mask before the accumulation kernel reads it;
* ``CASE WHEN c THEN x ELSE y END`` (``:76-87``) is a SELECT instruction with
  torch.where's promotion;
* ``year(d)`` (``:100-101``) is a YEAR instruction;
* a result that combines aggregates arithmetically (``sum(a) / sum(b)``,
  ``100.0 * sum(..) / sum(..)``; ``:197-233`` evaluates each call, then the
  arithmetic on the per-group tensors) computes its calls as hidden
  accumulator outputs and the arithmetic as a projection over the groups.
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
_COND_OPS = ("<=", ">=", "<", ">", "=", "<>", "AND", "OR")
_HIDDEN_ID = 1 << 40          # ids of hidden per-group columns (aggregate calls inside a result expression)


class _Literal0Int(int):
    """Two integer literals combined by + - *: torch returns a 0-dim int64 tensor, which promotes
    like a Python int."""


class _Literal0F32(float):
    """Two literals combined with a float among them, or divided: torch returns a 0-dim float32
    tensor (its default float dtype), computed in float32.  It promotes like a Python float, with
    the float32 value: 2 + 0.1 is 2.0999999046325684 when it meets a float64 column."""


def _fold_literals(op: str, a, b):
    """torch.add / sub / mul / div of two Python numbers (aggregate.py:233)."""
    if isinstance(a, float) or isinstance(b, float) or op == "/":
        import numpy as np
        fa, fb = np.float32(a), np.float32(b)
        with np.errstate(all="ignore"):
            return _Literal0F32({"+": fa + fb, "-": fa - fb, "*": fa * fb, "/": fa / fb}[op])
    return _Literal0Int({"+": a + b, "-": a - b, "*": a * b}[op])


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
    wide: bool = False        # a one-byte substring: the reference's [N, 1] slice (aggregate.py:114-119)

    @property
    def f32(self) -> bool:
        return self.dtype == torch.float32


@dataclass
class AggregateProgram:
    spec: Any
    tensors: List[torch.Tensor] = field(default_factory=list)
    key_ids: List[int] = field(default_factory=list)        # grouping columns (args['keys'])
    key_outputs: List[Tuple[int, int]] = field(default_factory=list)   # (out id, input key id)
    outputs: List[Tuple[int, int, int, int, torch.dtype]] = field(default_factory=list)  # (out id, op, a, b, dtype)
    masks: List[Tuple[Any, torch.Tensor]] = field(default_factory=list)   # (condition predicate, its bool column)
    post: List[Tuple[int, Any, torch.dtype]] = field(default_factory=list)  # (out id, arithmetic over hidden ids, dtype)
    # outputs computed in float64 whose reference dtype is float32: out id -> (dtype, avg result id of the
    # reference's 2-step path, which stays float64 there: aggregate.py:170)
    casts: Dict[int, Tuple[torch.dtype, bool]] = field(default_factory=dict)
    encoded: bool = False     # the kernel groups by one int32 code column standing for the key tuple


def needs_key_codes(args: dict, columns: Dict[int, torch.Tensor]) -> bool:
    """Key tuples the dense / packed-hash slots cannot take: a 2-D (string) key, a float
    key, or more than TQPK_MAX_KEYS keys (aggregate.py:291-311 stacks any of these)."""
    keys = [get_id(k) for k in (args.get("keys") or [])]
    if len(keys) > L.MAX_KEYS:
        return True
    for kid in keys:
        t = columns[kid]
        if (t.dim() == 2 and t.shape[1] != 1) or t.dtype not in _INT_ORDER:
            return True
    return False


class _Builder:
    def __init__(self, columns: Dict[int, torch.Tensor], derived: bool = False):
        self.columns = dict(columns)
        self.derived = derived
        self.masks: List[Tuple[Any, torch.Tensor]] = []
        self.mask_memo: Dict[str, int] = {}
        self.expr: List[tuple] = []
        self.memo: Dict[tuple, int] = {}
        self.col_slot: Dict[int, int] = {}
        self.col_tensors: List[torch.Tensor] = []
        self.accs: List[tuple] = [(L.ACC_COUNT_ROWS, L.I64, 0, 0, 0.0)]
        self.acc_memo: Dict[tuple, int] = {}

    def _insn(self, key, op, f64, a=0, b=0, col=0, ci=0, cf=0.0, f32=False, wrap=0) -> int:
        if key in self.memo:
            return self.memo[key]
        if len(self.expr) >= L.MAX_EXPR:
            raise NotImplementedError(f"aggregate expressions exceed {L.MAX_EXPR} instructions")
        self.expr.append((op, L.F32 if f32 else L.F64 if f64 else L.I64, a, b, col, ci, cf, wrap))
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

    def const32(self, v) -> _Node:
        """A Python number taken into a float32 operation (torch casts it to float32)."""
        return _Node(self._insn(("cf32", float(v)), L.X_CONST, False, cf=float(v), f32=True), False, torch.float32)

    def to_f64(self, n: _Node) -> int:
        if n.f64:
            return n.reg
        if n.f32:
            return self._insn(("f32tof64", n.reg), L.X_F32TOF64, True, a=n.reg)
        return self._insn(("tof64", n.reg), L.X_TOF64, True, a=n.reg)

    def to_f32(self, x) -> int:
        """An integer node or a Python number as a float32 register."""
        if not isinstance(x, _Node):
            return self.const32(x).reg
        if x.f32:
            return x.reg
        assert not x.f64
        return self._insn(("tof32", x.reg), L.X_TOF32, False, a=x.reg, f32=True)

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
        if len(tree) == 3 and tree[1] in ("+", "-", "*", "/"):
            return self.binary(tree[1], self.value(tree[0]), self.value(tree[2]))
        if len(tree) == 2 and tree[0] == "cast":
            literal, _, cast_type = tree[1][0].split(" ")
            if cast_type == "double":
                return self.value(literal)
        if len(tree) == 2 and tree[0] == "substring":
            return self.substring(tree[1])
        if self.derived:
            if len(tree) == 8 and tree[0] == "CASE":
                assert tree[1] == "WHEN" and tree[3] == "THEN" and tree[5] == "ELSE" and tree[7] == "END"
                return self.select(self.value(tree[2]), self.value(tree[4]), self.value(tree[6]))
            if len(tree) == 2 and tree[0] == "year":
                d = self.value(tree[1])
                if not isinstance(d, _Node) or d.f64:
                    raise NotImplementedError("year() of a non-integer operand is not on the kernel path")
                return _Node(self._insn(("year", d.reg), L.X_YEAR, False, a=d.reg), False, torch.int64)
            if (len(tree) == 2 and tree[0] in ("NOT", "StartsWith")) or (len(tree) == 3 and tree[1] in _COND_OPS):
                return self.condition(tree)
        raise NotImplementedError(f"aggregate expression {tree!r} is not on the kernel path")

    def substring(self, arg) -> _Node:
        """substring(col, l, w) as a value (aggregate.py:114-119): the reference slices the [N, w]
        string rows; only a one-byte slice gives weights its sum / count accept (squeezed to [N],
        :179-182), so w = 1 is a column of those bytes (copied out of the rows), and anything wider
        fails in the reference and raises here."""
        sub, l, w = arg
        cid, l, w = get_id(sub), int(l) - 1, int(w)
        col = self.columns[cid]
        if col.dim() != 2 or col.dtype not in (torch.int8, torch.uint8) or not 0 <= l < col.shape[1]:
            raise NotImplementedError(f"substring of a {tuple(col.shape)} {col.dtype} column")
        if w != 1:
            raise NotImplementedError("a substring wider than one byte as an aggregate value (the reference's "
                                      "bincount rejects [N, w] weights)")
        key = ("substr", cid, l)
        if key not in self.mask_memo:
            hid = _HIDDEN_ID * 3 + len(self.mask_memo)
            self.columns[hid] = col[:, l].contiguous()
            self.mask_memo[key] = hid
        n = self.column(self.mask_memo[key])
        return _Node(n.reg, n.f64, n.dtype, wide=True)

    def condition(self, tree) -> _Node:
        """A boolean sub-expression as a bool column, filled by the filter kernel before the
        program runs (aggregate comparison rules)."""
        from .predicate import compile_filter
        key = repr(tree)
        if key not in self.mask_memo:
            pred = compile_filter(tree, {c: t for c, t in self.columns.items() if c < _HIDDEN_ID}, agg=True)
            t0 = pred.tensors[0]
            mask = torch.empty(t0.shape[0], dtype=torch.bool, device=t0.device)
            cid = _HIDDEN_ID * 2 + len(self.masks)
            self.columns[cid] = mask
            self.masks.append((pred, mask))
            self.mask_memo[key] = cid
        return self.column(self.mask_memo[key])

    def select(self, c, t, e) -> _Node:
        """torch.where(c, t, e) with torch's promotion of the two branches."""
        if not isinstance(c, _Node) or c.dtype != torch.bool:
            raise NotImplementedError("CASE WHEN needs a boolean condition")
        if any(isinstance(x, _Node) and x.wide for x in (c, t, e)):
            raise NotImplementedError("a one-byte substring inside CASE WHEN")
        nodes = [x for x in (t, e) if isinstance(x, _Node)]
        pys = [x for x in (t, e) if not isinstance(x, _Node)]
        if any(n.f64 for n in nodes):
            f64, dtype = True, torch.float64
        elif any(n.f32 for n in nodes) or any(isinstance(x, float) for x in pys):
            # torch.where with a float32 branch, or a float literal beside integers: float32
            rt, re_ = self.to_f32(t), self.to_f32(e)
            reg = self._insn(("sel32", c.reg, rt, re_), L.X_SELECT, False, a=c.reg, b=rt, col=re_, f32=True)
            return _Node(reg, False, torch.float32)
        elif not nodes:
            f64, dtype = False, torch.int64
        else:
            ints = [n.dtype for n in nodes]
            if len(ints) == 2 and {ints[0], ints[1]} == {torch.uint8, torch.int8}:
                raise NotImplementedError("uint8 with int8 promotes to int16 in torch")
            dtype = max(ints, key=lambda d: _INT_ORDER[d])
            if dtype == torch.bool and pys:
                dtype = torch.int64
            f64 = False
        regs = []
        narrow = {torch.int8: "int8", torch.uint8: "uint8", torch.int32: "int32"}.get(dtype) if not f64 else None
        for x in (t, e):
            if not isinstance(x, _Node) and narrow:       # a Python int taken into an int8/uint8/int32 where
                import numpy as np                          # torch casts it to that dtype (wrapping)
                x = int(np.array(int(x) & ((1 << 64) - 1), dtype=np.uint64).astype(narrow))
            n = x if isinstance(x, _Node) else self.const(float(x) if f64 else int(x))
            regs.append(self.to_f64(n) if f64 else n.reg)
        reg = self._insn(("sel", c.reg, regs[0], regs[1], f64), L.X_SELECT, f64, a=c.reg, b=regs[0], col=regs[1])
        return _Node(reg, f64, dtype)

    def binary(self, op: str, a, b):
        op_code = {"+": L.X_ADD, "-": L.X_SUB, "*": L.X_MUL, "/": L.X_DIV}[op]
        if not isinstance(a, _Node) and not isinstance(b, _Node):
            return _fold_literals(op, a, b)
        wides = [x.wide for x in (a, b) if isinstance(x, _Node)]
        if any(wides) and not all(wides):
            raise NotImplementedError("a one-byte substring with a column: the reference broadcasts [N, 1] "
                                      "against [N]")
        wide = any(wides)
        # torch promotion of the pair
        def kind(x):
            if isinstance(x, _Node):
                return "f" if x.f64 else "g" if x.f32 else "i"
            return "pf" if isinstance(x, float) else "pi"
        ka, kb = kind(a), kind(b)
        if "f" in (ka, kb):
            f64, dtype = True, torch.float64
        elif "g" in (ka, kb) or "pf" in (ka, kb) or op == "/":
            # float32 (torch's default float dtype): a float32 tensor with integers or Python numbers,
            # an integer tensor with a Python float, or an integer true division
            ra, rb = self.to_f32(a), self.to_f32(b)
            reg = self._insn((op, ra, rb, "f32"), op_code, False, a=ra, b=rb, f32=True)
            return _Node(reg, False, torch.float32, wide=wide)
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
        # torch's int8 / uint8 / int32 arithmetic wraps at its own width
        wrap = 0 if f64 else {torch.int8: L.I8, torch.uint8: L.U8, torch.int32: L.I32}.get(dtype, 0)
        reg = self._insn((op, ra, rb, f64, wrap), op_code, f64, a=ra, b=rb, wrap=wrap)
        return _Node(reg, f64, dtype, wide=wide)

    def acc(self, kind: int, node: _Node, init_i=0, init_f=0.0) -> int:
        key = (kind, node.reg, node.f64, init_i, init_f)
        if key not in self.acc_memo:
            if len(self.accs) >= L.MAX_ACCS:
                raise NotImplementedError(f"more than {L.MAX_ACCS} accumulators")
            self.accs.append((kind, L.F64 if node.f64 else L.I64, node.reg, init_i, init_f))
            self.acc_memo[key] = len(self.accs) - 1
        return self.acc_memo[key]


def require_f64_outputs(prog: "AggregateProgram", what: str) -> None:
    """The fused and batched paths write float64 / int64 results only: an aggregate of a float32
    expression (torch's float32 result) is left to the operator path."""
    if prog.casts:
        raise NotImplementedError(f"{what}: an aggregate of a float32 expression runs on the operator path")


def _call_of(t):
    """(fn, arg) when t is an aggregate call, possibly wrapped as [[fn, arg], '#', id]."""
    t = _strip(t)
    while isinstance(t, list) and len(t) == 3 and t[1] == "#":
        t = _strip(t[0])
    if isinstance(t, list) and len(t) == 2 and isinstance(t[0], str) and t[0] in _AGG_FNS:
        return t[0], t[1]
    return None


def _agg_call(tree):
    """Walks [[fn, arg], '#', id] / [.., 'AS', name] down to (fn, arg)."""
    t = _strip(tree)
    while isinstance(t, list) and len(t) == 3 and t[1] in ("#", "AS"):
        t = _strip(t[0])
    if isinstance(t, list) and len(t) == 2 and t[0] in _AGG_FNS:
        return t[0], t[1]
    raise NotImplementedError(f"aggregate result {tree!r}: only plain sum/avg/count/min/max calls run on the kernels")


def _lift_calls(t, calls: list, base: int):
    """Replaces each aggregate call inside a result expression by a hidden column name
    (ids base, base + 1, ...)."""
    c = _call_of(t)
    if c is not None:
        hid = base + len(calls)
        calls.append((hid, c[0], c[1]))
        return f"agg#{hid}"
    if isinstance(t, list):
        return [_lift_calls(x, calls, base) for x in t]
    return t


def _add_output(b: _Builder, prog: AggregateProgram, oid: int, fn: str, arg):
    v = b.value(arg)
    if isinstance(v, (_Literal0Int, _Literal0F32)):
        # the reference's reductions take a 0-dim tensor as their values and fail (bincount /
        # scatter_reduce want one value per row); a bare literal is expanded instead (:149-152)
        raise RuntimeError(f"{fn} of two combined literals: the reference's reductions reject the 0-dim "
                           "tensor they give")
    scalar = not isinstance(v, _Node)
    if fn == "count" and scalar and v != L.NULL_INDEX:      # count(1): every row counts
        prog.outputs.append((oid, L.OUT_ACC, 0, 0, torch.int64))
        return
    if scalar:                                              # aggregate.py:149-152: full(cnt_rows, v)
        v = b.const(v)
    if v.wide and fn not in ("sum", "count"):
        # min/max scatter [N, 1] values by an [N] index and avg's bincount takes 1-D weights only: the
        # reference fails on these (only sum and count squeeze their values first, :179-182)
        raise NotImplementedError(f"{fn} of a substring: the reference fails on its [N, 1] values")
    if v.f32:
        # a float32 expression: accumulated from its exact float64 value; the output is rounded to
        # float32 (sum, min, max, and avg of the 1-step path; the 2-step avg is float64, :170)
        v = _Node(b.to_f64(v), True, torch.float64)
        if fn != "count":
            prog.casts[oid] = (torch.float32, fn == "avg")
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


# Compiled aggregate programs by query shape (result trees, keys, the columns' dtypes and
# widths): a repeated query re-binds the column pointers of the cached program instead of
# parsing its trees again (tens of microseconds of host time per call).
_AGG_MEMO: Dict[tuple, Tuple[AggregateProgram, List[int]]] = {}
_AGG_MEMO_MAX = 256


def _as_1d(t: torch.Tensor) -> torch.Tensor:
    return (t.reshape(-1) if t.dim() == 2 and t.shape[1] == 1 else t).contiguous()


def compile_aggregate(args: dict, columns: Dict[int, torch.Tensor], derived: bool = False,
                      key_codes: torch.Tensor = None) -> AggregateProgram:
    """derived=False keeps to plain calls over arithmetic (every fused pipeline);
    derived=True adds conditions, CASE, year() and arithmetic over aggregates.
    key_codes (int32 [n], from ops.encode_keys) replaces the key tuple in the kernel."""
    sig = None
    if key_codes is None:
        sig = (repr(args["results"]), repr(args.get("keys")), derived,
               tuple(sorted((c, t.dtype, t.dim(), t.shape[1] if t.dim() == 2 else 0) for c, t in columns.items())))
        hit = _AGG_MEMO.get(sig)
        if hit is not None:
            return _rebind(hit[0], hit[1], columns)
    prog, col_ids = _compile_aggregate(args, columns, derived, key_codes)
    if sig is not None and not prog.masks and all(c < _HIDDEN_ID for c in col_ids):   # no derived columns
        if len(_AGG_MEMO) >= _AGG_MEMO_MAX:
            _AGG_MEMO.clear()
        _AGG_MEMO[sig] = (prog, col_ids)
    return prog


def _rebind(proto: AggregateProgram, col_ids: List[int], columns: Dict[int, torch.Tensor]) -> AggregateProgram:
    """A copy of a cached program reading these columns (same dtypes and widths)."""
    s = L.GroupbySpec.from_buffer_copy(proto.spec)
    tensors = []
    for k, kid in enumerate(proto.key_ids):
        t = _as_1d(columns[kid])
        tensors.append(t)
        s.keys[k] = t.data_ptr()
    for i, cid in enumerate(col_ids):
        t = _as_1d(columns[cid])
        tensors.append(t)
        s.cols[i] = t.data_ptr()
    return AggregateProgram(spec=s, tensors=tensors, key_ids=list(proto.key_ids),
                            key_outputs=list(proto.key_outputs), outputs=list(proto.outputs), masks=[],
                            post=list(proto.post), encoded=False, casts=dict(proto.casts))


def _compile_aggregate(args: dict, columns: Dict[int, torch.Tensor], derived: bool,
                       key_codes: torch.Tensor) -> Tuple[AggregateProgram, List[int]]:
    b = _Builder(columns, derived)
    prog = AggregateProgram(spec=None)
    prog.key_ids = [get_id(k) for k in (args.get("keys") or [])]
    prog.encoded = key_codes is not None
    if len(prog.key_ids) > L.MAX_KEYS and not prog.encoded:
        raise NotImplementedError(f"more than {L.MAX_KEYS} group keys")
    for tree in args["results"]:
        tree = _strip(tree)
        oid = get_id(right_most(tree))
        if is_key_result(tree):
            prog.key_outputs.append((oid, get_id(tree if isinstance(tree, str) else tree[0])))
            continue
        body = tree[0] if isinstance(tree, list) and len(tree) == 3 and tree[1] == "AS" else tree
        call = _call_of(body)
        if call is not None:
            _add_output(b, prog, oid, *call)
            continue
        if not derived:
            _agg_call(tree)                                 # raises NotImplementedError
        calls: list = []
        lifted = _lift_calls(body, calls, _HIDDEN_ID + sum(1 for o in prog.outputs if o[0] >= _HIDDEN_ID))
        if not calls:
            raise NotImplementedError(f"aggregate result {tree!r} has no aggregate call")
        for hid, fn, arg in calls:
            _add_output(b, prog, hid, fn, arg)
            if hid in prog.casts:
                raise NotImplementedError("arithmetic over an aggregate of a float32 expression")
        dts = {hid: dt for (hid, _, _, _, dt) in prog.outputs if hid in {c[0] for c in calls}}
        trial = compile_projection([lifted], {h: torch.empty(0, dtype=dt) for h, dt in dts.items()})
        prog.post.append((oid, lifted, trial.outputs[0][1]))
    if len(prog.outputs) > L.MAX_ACCS:
        raise NotImplementedError(f"more than {L.MAX_ACCS} aggregate outputs")
    s = L.GroupbySpec()
    if prog.encoded:
        t = key_codes.contiguous()
        s.n_keys = 1
        prog.tensors.append(t)
        s.keys[0] = t.data_ptr()
        s.key_dtypes[0] = code_of(t.dtype)
    else:
        s.n_keys = len(prog.key_ids)
    for k, kid in enumerate([] if prog.encoded else prog.key_ids):
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
    for i, (op, ty, a, bb, col, ci, cf, wrap) in enumerate(b.expr):
        s.expr[i] = L.ExprInsn(op, ty, a, bb, col, wrap, ci, cf)
    s.n_accs = len(b.accs)
    for i, (kind, ty, reg, ii, ff) in enumerate(b.accs):
        s.accs[i] = L.Acc(kind, ty, reg, 0, ii, ff)
    prog.spec = s
    prog.masks = b.masks
    return prog, [cid for cid, _ in sorted(b.col_slot.items(), key=lambda kv: kv[1])]


@dataclass
class ProjectionProgram:
    spec: Any                                   # expression program (no keys; accumulator 0 only)
    tensors: List[torch.Tensor] = field(default_factory=list)
    outputs: List[Tuple[int, torch.dtype]] = field(default_factory=list)   # (register, result dtype)
    masks: List[Tuple[Any, torch.Tensor]] = field(default_factory=list)   # (condition predicate, its bool column)


def is_trivial_projection(tree) -> bool:
    """A bare column or `column AS name` (project.py:27-31): renamed, not computed."""
    while isinstance(tree, list) and len(tree) == 1:
        tree = tree[0]
    return isinstance(tree, str) or (tree[1] == "AS" and isinstance(tree[0], str))


def compile_projection(trees, columns: Dict[int, torch.Tensor], derived: bool = False) -> ProjectionProgram:
    """The computed expressions of a projection (project.py:20-40) as one SSA program: each
    output is a register with the dtype torch gives the expression (aggregate.py:203-233).
    derived=True adds conditions, CASE and year() (bool columns filled before the launch)."""
    b = _Builder(columns, derived)
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
        # a float32 result is written through its exact float64 value and narrowed afterwards
        outs.append((b.to_f64(v) if v.f32 else v.reg, v.dtype))
    spec = L.GroupbySpec()
    spec.n_keys = 0
    spec.n_cols = len(b.col_tensors)
    for i, t in enumerate(b.col_tensors):
        spec.cols[i] = t.data_ptr()
        spec.col_dtypes[i] = code_of(t.dtype)
    spec.n_expr = len(b.expr)
    for i, (op, ty, a, bb, col, ci, cf, wrap) in enumerate(b.expr):
        X = spec.expr[i]
        X.op, X.type, X.a, X.b, X.col, X.ci, X.cf, X.wrap = op, ty, a, bb, col, ci, cf, wrap
    spec.n_accs = 1
    spec.accs[0].kind, spec.accs[0].type = L.ACC_COUNT_ROWS, L.I64
    return ProjectionProgram(spec=spec, tensors=list(b.col_tensors), outputs=outs, masks=b.masks)
