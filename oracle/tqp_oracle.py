"""Parity oracle: a CPU (numpy) restatement of TQP-Inmem's relational operators.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module.  It
is used by ``tests/`` (as the checker), by ``__graft_entry__.smoke()`` (to
check one small GPU invocation) and by ``bench.py`` (the timed CPU baseline,
and the ``--impl reference`` arm).  It never produces a product result.

The oracle is pinned against golden vectors produced by running the
reference's own operators (``tests/golden/make_golden.py`` ->
``tests/golden/*.npz``; checked by ``tests/test_oracle_golden.py``).

Each function cites the reference code it restates (paths are relative to
the TQP-Inmem source tree).  Where the reference is non-deterministic, the
oracle picks one deterministic answer that the reference can also produce:

* group order: the reference orders groups by a random linear hash of the key
  tuple (``operators/aggregate.py:320-327``); the oracle orders them by key
  tuple, ascending.  For one non-negative key the two orders coincide.
* pairs inside one build-key bucket: the reference sorts build keys with an
  unstable sort (``operators/hashjoin.py:43``); the oracle uses a stable one
  (ascending build row inside a bucket).
"""
from __future__ import annotations

import datetime as _dt
from typing import Dict, List, Sequence, Tuple

import numpy as np

# constants.py:3-9
EPS = 1e-5
NULL = -64

_EPOCH = _dt.date(1990, 1, 1)  # conversion.py:11 (YEAR_START = 1990)


# ---------------------------------------------------------------------------
# Literals (conversion.py:20-33, parsing.py:15-16)
# ---------------------------------------------------------------------------
def get_id(name: str) -> int:
    """parsing.py:15-16"""
    return int(name.split("#")[-1].replace("L", ""))


def is_date(s: str) -> bool:
    """conversion.py:20-21"""
    return len(s) == 10 and s.count("-") == 2 and s.replace("-", "").isdigit()


def is_float(s: str) -> bool:
    """conversion.py:23-24"""
    return s.replace(".", "").replace("-", "").replace("E", "").isdigit()


def date_to_days(s: str) -> int:
    """conversion.py:26-29: days between the date and 1990-01-01."""
    return (_dt.date.fromisoformat(s) - _EPOCH).days


# ---------------------------------------------------------------------------
# Filter: operators/filter.py:14-162
# ---------------------------------------------------------------------------
def _cmp(op: str, a, b):
    return {"<=": np.less_equal, ">=": np.greater_equal, "<": np.less, ">": np.greater,
            "=": np.equal, "<>": np.not_equal}[op](a, b)


def _is_int(a: np.ndarray) -> bool:
    return a.dtype.kind in "iu"


def _torch_compare(op: str, col: np.ndarray, lit):
    """A column compared with a Python scalar, with torch's type promotion.

    An integer column against a Python float is compared in float32 (torch's
    default dtype); every other combination compares exactly.
    """
    if _is_int(col) and isinstance(lit, float):
        return _cmp(op, col.astype(np.float32), np.float32(lit))
    if _is_int(col):
        return _cmp(op, col.astype(np.int64), np.int64(lit))
    return _cmp(op, col, np.float64(lit))


def _isclose(a: np.ndarray, b: float, rtol=1e-5, atol=EPS) -> np.ndarray:
    """torch.isclose(a, full(b), atol=eps) as used at filter.py:160-161."""
    err = np.abs(a - b)
    allowed = atol + np.abs(rtol * b)
    return (a == b) | (np.isfinite(err) & (err <= allowed))


def _str_bytes(s: str, w: int) -> np.ndarray:
    """conversion.py:36-37 (str_to_np): the characters' codes padded with zeros to w, as int8."""
    return np.pad(np.array([ord(c) for c in s], np.int64), (0, w - len(s))).astype(np.int8)


def _like_contains(a: np.ndarray, p: np.ndarray) -> np.ndarray:
    """like.py:3-11: p occurs at some position of each row."""
    n1, m = p.shape[0], a.shape[1]
    out = np.zeros(a.shape[0], bool)
    for pos in range(m - n1 + 1):
        out |= (a[:, pos:pos + n1] == p).all(axis=1)
    return out


def _like_mask(a: np.ndarray, p1: np.ndarray, p2: np.ndarray) -> np.ndarray:
    """like.py:13-22: p2 starts at or after the end of an earlier occurrence of p1."""
    n1, n2, m = p1.shape[0], p2.shape[0], a.shape[1]
    appear = np.zeros(a.shape[0], bool)
    out = np.zeros(a.shape[0], bool)
    for pos in range(m - n1 - n2 + 1):
        appear |= (a[:, pos:pos + n1] == p1).all(axis=1)
        out |= appear & (a[:, pos + n1:pos + n1 + n2] == p2).all(axis=1)
    return out


def eval_filter(tree, cols: Dict[int, np.ndarray], rows: int | None = None, subquery=None):
    """Evaluate a parsed filter tree into a bool mask (filter.py:14-162).

    String columns are int8 [N, w] tensors, zero padded (conversion.py:36-37):
    StartsWith compares the first len(name) bytes (:48-55), Contains and
    EndsWith search every position (:56-62, like.py:3-11), LIKE '%a%b%' finds
    b after an occurrence of a (:121-127, like.py:13-22), and a multi-character
    literal compares byte-wise against the literal padded to w (:151-158).
    """
    if rows is None:
        rows = next(iter(cols.values())).shape[0]
    if isinstance(tree, str):                                      # :18-35
        if tree == "Subquery":
            return subquery
        if is_date(tree):
            return date_to_days(tree)
        if is_float(tree):
            return float(tree) if "." in tree else int(tree)
        if "#" in tree and not tree.startswith("Brand#"):
            return cols[get_id(tree)].reshape(-1) if cols[get_id(tree)].ndim == 2 and cols[get_id(tree)].shape[1] == 1 else cols[get_id(tree)]
        return tree
    if len(tree) == 1:                                             # :37-38
        return eval_filter(tree[0], cols, rows, subquery)
    if len(tree) == 3 and tree[1] == "#":                          # :40-44
        return cols[int(tree[-1])]
    if len(tree) == 2:                                             # :46-86
        if tree[0] == "StartsWith":                                # :48-55
            t = cols[get_id(tree[1][0])]
            p = _str_bytes(tree[1][1], len(tree[1][1]))
            assert t.shape[-1] >= len(p)
            return (t[:, :len(p)] == p).all(axis=1)
        if tree[0] in ("EndsWith", "Contains"):                    # :56-62
            return _like_contains(cols[get_id(tree[1][0])], _str_bytes(tree[1][1], len(tree[1][1])))
        if tree[0] == "NOT":
            return ~eval_filter(tree[1], cols, rows, subquery)
        if tree[0] == "isnotnull":
            return np.ones(rows, dtype=bool)
        if tree[0] == "substring":                                 # :71-76: a column slice [:, l-1:l-1+w]
            assert len(tree[1]) == 3
            sub, l, w = tree[1]
            l, w = int(l) - 1, int(w)
            return eval_filter(sub, cols, rows, subquery)[:, l:l + w]
        if tree[0] == "cast":
            literal, _, cast_type = tree[1][0].split(" ")
            if cast_type == "double":
                return eval_filter(literal, cols, rows, subquery)
        raise ValueError(f"Unsupported Function: {tree[0]}")            # :87, the reference's error
    op = tree[-2]
    if op == "LIKE":                                               # :121-127
        L = eval_filter(tree[0], cols, rows, subquery)
        assert tree[-1].count("%") == 3
        _, w1, w2, _ = tree[-1].split("%")
        return _like_mask(L, _str_bytes(w1, len(w1)), _str_bytes(w2, len(w2)))
    if op == "IN":                                                 # :90-119
        L = eval_filter(tree[0], cols, rows, subquery)
        mask = np.zeros(rows, dtype=bool)
        for r in tree[-1]:
            if L.ndim == 2:                                        # :110-113
                assert len(r) > 1
                mask |= (L == _str_bytes(r, L.shape[-1])).all(axis=1)
            elif _is_int(L):
                if len(r) == 1 and not r.lstrip("-").isdigit():
                    mask |= L == ord(r)
                else:
                    mask |= L.astype(np.int64) == int(r)
            else:
                mask |= L == float(r)
        return mask
    if op not in ("<=", ">=", "<", ">", "=", "AND", "OR"):         # :129-140
        raise ValueError(f"Unsupported Operation: {op}")             # the reference's error class
    L = eval_filter(tree[0], cols, rows, subquery)
    R = eval_filter(tree[-1], cols, rows, subquery)
    if op == "AND":
        return np.logical_and(L, R)
    if op == "OR":
        return np.logical_or(L, R)
    if isinstance(R, float):                                       # :145-149
        if op == "<=":
            return _torch_compare("<=", L, R + EPS)
        if op == ">=":
            return _torch_compare(">=", L, R - EPS)
    if isinstance(R, str):                                         # :151-158
        if len(R) == 1:
            return _torch_compare(op, L, ord(R))
        if L.ndim != 2:
            raise NotImplementedError("multi-character literal against a one-dimensional column")
        return (L == _str_bytes(R, L.shape[-1])).all(axis=1)       # equality whatever the operator
    if op == "=" and L.dtype == np.float64:                        # :160-161
        if not isinstance(R, float):
            raise TypeError("isclose against a non-float literal (the reference raises here too)")
        return _isclose(L, R)
    if isinstance(R, np.ndarray):
        return _cmp(op, L, R)
    return _torch_compare(op, L, R)                                # :162


# ---------------------------------------------------------------------------
# Late materialisation: IO/vortex_pipeline.py:51-66
# ---------------------------------------------------------------------------
def apply_mask_map(cols: Dict[int, np.ndarray], mask_map: Dict[int, int]) -> Dict[int, np.ndarray]:
    """Compacts every column that has a mask (``tensor[mask]``, :58) and drops
    the mask columns themselves (:61-64)."""
    masks = set(mask_map.values())
    out = {}
    for cid, a in cols.items():
        if cid in masks:
            continue
        out[cid] = a[cols[mask_map[cid]]] if cid in mask_map else a
    return out


# ---------------------------------------------------------------------------
# Join: operators/hashjoin.py:24-177
# ---------------------------------------------------------------------------
def join_indices(left: np.ndarray, right: np.ndarray, jtype: str = "inner", keep=None):
    """Sort-based equi-join of two key columns (hashjoin.py:24-151).

    Returns (left_idx, right_idx) as int64; for ``right-outer`` unmatched right
    rows are appended with left index ``NULL`` (:135-158).  ``keep(cs, cr)``,
    when given, is the extra join conditions' mask over the key-equal pairs
    (:100-108); every join type is derived from the pairs it keeps.
    """
    left = left.reshape(-1)
    right = right.reshape(-1)
    perm = np.argsort(left, kind="stable")                         # :41-44
    sorted_keys = left[perm]
    uniq, starts, counts = np.unique(sorted_keys, return_index=True, return_counts=True)  # :48-52
    pos = np.searchsorted(uniq, right)                             # :57
    in_range = pos < uniq.size                                     # :59
    eq = np.zeros(right.size, dtype=bool)
    eq[in_range] = uniq[pos[in_range]] == right[in_range]          # :60-61
    mr = np.nonzero(eq)[0]                                         # :65
    if mr.size:
        b = pos[mr]
        lens = counts[b]
        cr = np.repeat(mr, lens)                                   # :93
        offs = np.arange(cr.size) - np.repeat(np.cumsum(lens) - lens, lens)
        cs = perm[np.repeat(starts[b], lens) + offs]               # :77-86
    else:
        cs = np.zeros(0, np.int64)
        cr = np.zeros(0, np.int64)
    cs = cs.astype(np.int64)
    cr = cr.astype(np.int64)
    if keep is not None and cs.size:                               # :100-108
        k = np.asarray(keep(cs, cr), bool).reshape(-1)
        cs, cr = cs[k], cr[k]
    if jtype == "inner":                                           # :118-120
        return cs, cr
    matched = np.unique(cr)
    if jtype == "right-semi":                                      # :121-124
        return np.zeros(0, np.int64), matched
    unmatched = np.setdiff1d(np.arange(right.size, dtype=np.int64), matched)
    if jtype == "right-anti":                                      # :125-134
        return np.zeros(0, np.int64), unmatched
    if jtype == "right-outer":                                     # :135-158
        if cs.size == 0:
            # :154 only pads the left index when there was at least one match
            return cs, np.concatenate([cr, unmatched])
        return (np.concatenate([cs, np.full(unmatched.size, NULL, np.int64)]),
                np.concatenate([cr, unmatched]))
    raise ValueError(jtype)


def _cond_ids(tree, out):
    if isinstance(tree, str):
        if "#" in tree and not tree.startswith("Brand#"):
            out[get_id(tree)] = True
    elif isinstance(tree, list):
        if len(tree) == 3 and tree[1] == "#":
            out[int(tree[-1])] = True
            return
        for e in tree:
            _cond_ids(e, out)


def index_with_null(data: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """conversion.py:52-57: data[idx] with NULL rows where idx is NULL.

    The reference fills with ``masked_fill_(mask, null)``, which broadcasts the [K] mask against
    the gathered rows from the right.  For a 2-D [K, w] result that works only for K == 1 (the
    row) or K == w (column j of every row where idx[j] is NULL); any other K raises RuntimeError,
    and so does this restatement."""
    m = idx == NULL
    out = data[np.where(m, 0, idx)].copy()
    if out.ndim == 2:
        K, w = out.shape
        if K == w:
            out[:, m] = NULL
        elif K == 1:
            out[m] = NULL
        else:
            raise RuntimeError(f"the [{K}] null mask does not broadcast over [{K}, {w}] rows")
        return out
    out[m] = NULL
    return out


def join_vortex(cols: Dict[int, np.ndarray], args: dict, leftcol: int, rightcol: int, jtype: str,
                conditions=()):
    """hashjoin.py:179-248: late-materialised inputs, join, gathered outputs.

    ``cols`` maps column id -> array (masks included).  Returns a new dict
    with the output columns replaced and the operator's row count.
    ``conditions`` are filter trees over both sides' columns, evaluated on the
    key-equal pairs (evaluate_join, :15-22, applied at :100-108).
    """
    mask_map = {int(k): v for k, v in args.get("mask map", {}).items()}
    groups = [args["left group"], args["right group"]]
    out_ids, inp = [], {}
    for side in (0, 1):
        for c in args["materialized in"]:
            if c in groups[side]:
                inp[c] = cols[c]
                out_ids.append(c)
                if c in mask_map:
                    inp[mask_map[c]] = cols[mask_map[c]]
    used_masks = {c: mask_map[c] for c in out_ids if c in mask_map}
    m = apply_mask_map(inp, used_masks)
    left_ids = {c for c in out_ids if c in groups[0]}

    def keep(cs, cr):
        mask = np.ones(cs.size, bool)
        for cond in conditions:
            leaves = {}
            _cond_ids(cond, leaves)
            pair_cols = {c: (m[c][cs] if c in left_ids else m[c][cr]) for c in leaves}
            mask &= np.asarray(eval_filter(cond, pair_cols, cs.size), bool).reshape(-1)
        return mask
    li, ri = join_indices(m[leftcol], m[rightcol], jtype, keep if conditions else None)
    sel = index_with_null if (jtype == "right-outer" and li.size > 0) else (lambda x, i: x[i])
    res = dict(cols)
    for c in out_ids:
        a = m[c]
        if c in groups[0]:
            res[c] = sel(a, li) if a.shape[0] > 0 else a[:0]
        else:
            res[c] = a[ri] if a.shape[0] > 0 else a[:0]
    rows = next(iter(res.values())).shape[0]
    return res, rows


# ---------------------------------------------------------------------------
# Aggregate: operators/aggregate.py:58-393
# ---------------------------------------------------------------------------
class _V:
    """A value during expression evaluation: an array or a Python scalar."""


def _promote(a, b):
    """torch result type of a binary op between arrays/Python scalars.

    f64 with anything -> f64; a float32 array with integers or Python numbers, or an integer
    array with a Python float -> float32 (torch's default float dtype); integers with integers
    -> the wider integer dtype.
    """
    def kind(x):
        if isinstance(x, np.ndarray) and x.ndim == 0:                # a 0-dim tensor: a scalar of its kind
            return "pf" if x.dtype.kind == "f" else "pi"
        if isinstance(x, np.ndarray):
            if x.dtype == np.float32:
                return "g"
            return "f" if x.dtype.kind == "f" else ("b" if x.dtype == bool else "i")
        return "pf" if isinstance(x, float) else "pi"
    ka, kb = kind(a), kind(b)
    if "f" in (ka, kb):
        return np.float64
    if "g" in (ka, kb) or "pf" in (ka, kb):
        return np.float32
    # integer tensors: the wider tensor dtype (a Python int does not widen it); bool counts as int64
    order = [np.int8, np.uint8, np.int16, np.int32, np.int64]
    ints = [x.dtype.type for x in (a, b) if isinstance(x, np.ndarray) and x.ndim > 0 and x.dtype != bool]
    if not ints:
        return np.int64
    if len(ints) == 2 and {ints[0], ints[1]} == {np.int8, np.uint8}:
        return np.int16
    return max(ints, key=order.index)


_YEAR_RANGE = np.arange(1990, 2000, dtype=np.int64)                            # conversion.py:14
_YEAR_EDGES = np.cumsum([365 if y % 4 else 366 for y in range(1990, 2000)])     # conversion.py:15
_AGG_CALLS = ("sum", "avg", "count", "min", "max")


def _is_float_scalar(x) -> bool:
    return isinstance(x, float) or (isinstance(x, np.ndarray) and x.ndim == 0 and x.dtype.kind == "f")


def _scalar(x):
    """A 0-dim result (two literals combined) as the Python number torch compares it as."""
    return x.item() if isinstance(x, np.ndarray) and x.ndim == 0 else x


def _where(mask, a, b):
    """torch.where(mask, a, b) with torch's promotion of arrays and Python scalars
    (aggregate.py:87).  A float literal with integers (or two float literals), or a float32
    branch without a float64 one, is float32 in torch (its default float dtype)."""
    arrs = [x for x in (a, b) if isinstance(x, np.ndarray) and x.ndim > 0]
    pys = [x for x in (a, b) if not (isinstance(x, np.ndarray) and x.ndim > 0)]     # 0-dim tensors too
    if any(x.dtype == np.float64 for x in arrs):
        dt = np.float64
    elif any(x.dtype == np.float32 for x in arrs) or any(_is_float_scalar(x) for x in pys):
        f32 = [x.astype(np.float32) if isinstance(x, np.ndarray) else np.float32(x) for x in (a, b)]
        return np.where(mask, f32[0], f32[1]).astype(np.float32)
    elif not arrs:
        dt = np.int64
    else:
        order = [np.bool_, np.int8, np.uint8, np.int16, np.int32, np.int64]
        kinds = [x.dtype.type for x in arrs]
        if len(kinds) == 2 and {kinds[0], kinds[1]} == {np.int8, np.uint8}:
            raise NotImplementedError("uint8 with int8 promotes to int16 in torch")
        dt = max(kinds, key=order.index)
        if dt == np.bool_ and pys:
            dt = np.int64
    return np.where(mask, a, b).astype(dt)


def _agg_compare(op: str, L, R):
    """ops[op](L, R) of aggregate.py:224-233 for arrays and Python numbers."""
    L, R = _scalar(L), _scalar(R)
    if isinstance(L, np.ndarray) and isinstance(R, np.ndarray):
        return _cmp(op, L, R)
    if isinstance(L, np.ndarray):
        return _torch_compare(op, L, R)
    if isinstance(R, np.ndarray):
        flip = {"<": ">", "<=": ">=", ">": "<", ">=": "<=", "=": "=", "<>": "<>"}[op]
        return _torch_compare(flip, R, L)
    return _cmp(op, L, R)


def eval_agg_expr(tree, cols: Dict[int, np.ndarray], ctx=None):
    """evaluate() of aggregate.py:58-233.  Row-wise expressions give arrays over the
    rows; an aggregate call (only with ctx = (inverse, G, n)) gives an array over
    the groups, so arithmetic around calls is per-group (:197-233)."""
    if isinstance(tree, str):                                      # :59-67
        if tree.isdigit():
            return int(tree)
        if is_float(tree):
            return float(tree)
        if "#" in tree and tree.split("#")[-1].replace("L", "").isdigit():
            return cols[get_id(tree)]
        return tree
    if len(tree) == 1:                                             # :69-70
        return eval_agg_expr(tree[0], cols, ctx)
    if len(tree) == 3 and tree[1] == "#":                          # :72-74
        return eval_agg_expr(tree[0], cols, ctx)
    if len(tree) == 8:                                             # :76-87 CASE WHEN c THEN a ELSE b END
        assert tree[0] == "CASE" and tree[1] == "WHEN" and tree[3] == "THEN" and tree[5] == "ELSE" and tree[7] == "END"
        mask = eval_agg_expr(tree[2], cols, ctx)
        return _where(mask, eval_agg_expr(tree[4], cols, ctx), eval_agg_expr(tree[6], cols, ctx))
    if len(tree) == 2:
        head = tree[0]
        if head == "StartsWith":                                   # :89-99
            t = cols[get_id(tree[1][0])]
            name = tree[1][1]
            assert t.shape[-1] >= len(name)
            return (t[:, :len(name)] == _str_bytes(name, len(name))).all(axis=1)
        if head == "year":                                         # :100-101
            R = eval_agg_expr(tree[1], cols, ctx)
            idx = np.searchsorted(_YEAR_EDGES, R, side="right")
            if np.any(idx >= _YEAR_RANGE.size):
                raise IndexError("year() of a day past the reference's 1990-1999 table")
            return _YEAR_RANGE[idx]
        if head == "NOT":                                          # :103-104
            return ~eval_agg_expr(tree[1], cols, ctx)
        if head == "cast":                                         # :106-113
            literal, _, cast_type = tree[1][0].split(" ")
            if cast_type == "double":
                return eval_agg_expr(literal, cols, ctx)
            raise ValueError(f"Unsupported cast type: {cast_type}")
        if head == "substring":                                    # :114-119: a slice of the string rows
            sub, l, w = tree[1]
            l, w = int(l) - 1, int(w)
            return np.asarray(eval_agg_expr(sub, cols, ctx))[:, l:l + w]
        if head not in _AGG_CALLS:                                 # :122-123
            raise ValueError(f"Unsupported aggregation function: {head}")
        if ctx is None:
            raise ValueError("aggregate call outside an aggregation")
        inverse, G, n = ctx
        return reduce_groups(head, eval_agg_expr(tree[1], cols, ctx), inverse, G, n)
    op = tree[-2]
    if op == "AS":                                                 # :199-200
        return eval_agg_expr(tree[0], cols, ctx)
    if op not in ("+", "-", "*", "/", "<=", ">=", "<", ">", "=", "<>", "AND", "OR"):
        raise ValueError(f"Unsupported Operation: {op}")
    L = eval_agg_expr(tree[0], cols, ctx)
    R = eval_agg_expr(tree[-1], cols, ctx)
    if isinstance(R, str):                                         # :224-231
        if isinstance(L, int):
            assert op == "-"
            return "".join(tree)
        if len(R) == 1:
            return _agg_compare(op, L, ord(R))
        return (L == _str_bytes(R, L.shape[-1])).all(axis=1)
    if op in ("AND", "OR"):
        return (np.logical_and if op == "AND" else np.logical_or)(L, R)
    if op not in ("+", "-", "*", "/"):
        return _agg_compare(op, L, R)
    t = _promote(L, R)
    if op == "/" and t != np.float64:
        t = np.float32                                             # integer true division: float32
    La = np.asarray(L, dtype=t) if not isinstance(L, np.ndarray) else L.astype(t, copy=False)
    Ra = np.asarray(R, dtype=t) if not isinstance(R, np.ndarray) else R.astype(t, copy=False)
    with np.errstate(all="ignore"):
        # two literals give a 0-dim tensor in torch (int64, or float32 with its rounding), kept as
        # a 0-d array: it promotes like a scalar but keeps the float32 value
        return np.asarray({"+": np.add, "-": np.subtract, "*": np.multiply, "/": np.true_divide}[op](La, Ra))


def group_rows(key_cols: Sequence[np.ndarray]) -> Tuple[List[np.ndarray], np.ndarray]:
    """Group ids of key tuples (aggregate.py:298-333), ordered by key tuple."""
    n = key_cols[0].shape[0]
    if n == 0:
        return [k.reshape(0, k.shape[1] if k.ndim == 2 else 1) for k in key_cols], np.zeros(0, np.int64)
    flat = [k.reshape(n, -1) for k in key_cols]
    order = np.lexsort([f[:, j] for f in reversed(flat) for j in reversed(range(f.shape[1]))])
    stacked = [f[order] for f in flat]
    change = np.zeros(n, dtype=bool)
    change[0] = True
    for s in stacked:
        change[1:] |= np.any(s[1:] != s[:-1], axis=1)
    gid_sorted = np.cumsum(change) - 1
    inverse = np.empty(n, np.int64)
    inverse[order] = gid_sorted
    firsts = order[change]
    return [f[firsts] for f in flat], inverse


def _sum_2steps(inverse: np.ndarray, v: np.ndarray, G: int, S: int) -> np.ndarray:
    """scatter_reduce_2steps 'sum' (aggregate.py:133-147): row i goes to sub-slot
    i % S of its group, sub-slots are accumulated in row order, then each
    group's S sub-slots are summed (pairwise, as a torch/numpy row sum)."""
    flat = inverse * S + (np.arange(inverse.size) % S)
    part = np.bincount(flat, weights=v, minlength=G * S)
    return part.reshape(G, S).sum(axis=1)


def reduce_groups(fn: str, v, inverse: np.ndarray, G: int, n: int) -> np.ndarray:
    """The reductions of aggregate.py:122-195, including the 2-step
    sub-slot form the reference switches to when rows/groups >= 2^16
    (:127-131); the two forms differ only in float summation order."""
    if isinstance(v, int):                                          # :149-152
        v = np.full(n, v, np.int64)
    elif isinstance(v, float):
        v = np.full(n, v, np.float64)
    elif isinstance(v, np.ndarray) and v.ndim == 0:
        raise RuntimeError("an aggregate of a 0-dim tensor (two literals) fails in the reference")
    if v.ndim == 2:                                                 # string slices (substring)
        # sum and count squeeze their values (:179-182); min/max scatter them by a 1-D index and
        # avg's bincount takes 1-D weights only, which the reference fails on
        if fn not in ("sum", "count"):
            raise RuntimeError(f"{fn} of [N, w] values fails in the reference")
        v = np.squeeze(v) if v.size >= 2 else v.reshape(-1)
        if v.ndim != 1:
            raise RuntimeError("bincount of [N, w] weights fails in the reference")
    two_step = G > 0 and n / G >= (1 << 16)                         # :127-131
    S = max(1, n // (G << 6)) if two_step else 1
    is_int = v.dtype.kind in "iub"
    if v.dtype == np.float32 and fn in ("sum", "avg"):
        # float32 values: torch accumulates in float32, in row order (bincount / scatter_reduce on
        # the CPU), the 2-step sub-slots then summed per group; the 2-step avg is float64 (:170)
        if two_step:
            flat = inverse * S + (np.arange(inverse.size) % S)
            part = np.zeros(G * S, np.float32)
            np.add.at(part, flat, v)
            s = part.reshape(G, S).sum(axis=1, dtype=np.float32)
            if fn == "avg":
                with np.errstate(all="ignore"):
                    return s.astype(np.float64) / _sum_2steps(inverse, np.ones(n), G, S)
            return s
        s = np.zeros(G, np.float32)
        np.add.at(s, inverse, v)
        if fn == "avg":
            with np.errstate(all="ignore"):
                return (s / np.bincount(inverse, minlength=G).astype(np.float32)).astype(np.float32)
        return s
    if two_step and fn in ("sum", "avg", "count"):
        vv = (v != NULL).astype(np.float64) if fn == "count" else v.astype(np.float64)
        s = _sum_2steps(inverse, vv, G, S)
        if fn == "avg":
            with np.errstate(all="ignore"):
                return s / _sum_2steps(inverse, np.ones(n), G, S)
        return np.round(s).astype(np.int64) if (is_int or fn == "count") else s
    if fn == "min":                                                 # :154-160 (the value's own dtype)
        init = np.iinfo(v.dtype).max if is_int else np.finfo(v.dtype).max
        out = np.full(G, init, dtype=v.dtype)
        np.minimum.at(out, inverse, v)
        return out
    if fn == "max":                                                 # :161-167 (initial value 0)
        out = np.zeros(G, dtype=v.dtype)
        np.maximum.at(out, inverse, v)
        return out
    if fn == "avg":                                                 # :168-177
        s = np.bincount(inverse, weights=v.astype(np.float64), minlength=G)
        c = np.bincount(inverse, minlength=G)
        with np.errstate(all="ignore"):
            return s / c
    if fn == "count":                                               # :184-185
        v = (v != NULL).astype(np.int64)
        is_int = True
    s = np.bincount(inverse, weights=v.astype(np.float64), minlength=G).astype(np.float64)   # :187-190
    if is_int:                                                      # :192-193
        return np.round(s).astype(np.int64)
    return s


def fsum_groups(v: np.ndarray, inverse: np.ndarray, G: int) -> np.ndarray:
    """Correctly rounded per-group sums (math.fsum), the accuracy reference."""
    import math
    order = np.argsort(inverse, kind="stable")
    bounds = np.searchsorted(inverse[order], np.arange(G + 1))
    vs = v[order]
    return np.array([math.fsum(vs[bounds[g]:bounds[g + 1]]) for g in range(G)], dtype=np.float64)


def _strip(tree):
    while isinstance(tree, list) and len(tree) == 1:
        tree = tree[0]
    return tree


def _is_key(tree) -> bool:
    return isinstance(tree, str) or (len(tree) == 3 and tree[1] == "AS" and isinstance(tree[0], str))


def _right_most(tree):
    """parsing.py:42-45"""
    return _right_most(tree[-1]) if isinstance(tree, list) else tree


def _agg_fn_and_arg(tree):
    """Walks [[fn, arg], '#', id] / [.., 'AS', name] down to (fn, arg)."""
    t = tree
    while True:
        t = _strip(t)
        if isinstance(t, list) and len(t) == 3 and t[1] in ("#", "AS"):
            t = t[0]
            continue
        break
    if not (isinstance(t, list) and len(t) == 2 and t[0] in ("sum", "avg", "count", "min", "max")):
        raise NotImplementedError(f"aggregate result {tree!r} is not a plain aggregate call")
    return t[0], t[1]


def tqp_hash_aggregate(cols: Dict[int, np.ndarray], args: dict):
    """aggregate.py:236-393: returns {out id: array} (keys as [G, 1])."""
    assert not args["is partial"]
    mask_map = {int(k): v for k, v in (args.get("mask map") or {}).items()}
    inp = {c: cols[c] for c in args["input ids"]}
    for k, v in mask_map.items():
        if k in inp:
            inp[v] = cols[v]
    m = apply_mask_map(inp, {k: v for k, v in mask_map.items() if k in args["input ids"]})
    n = next(iter(m.values())).shape[0]
    if args["keys"]:
        key_ids = [get_id(k) for k in args["keys"]]
        ukeys, inverse = group_rows([m[k] for k in key_ids])
        G = ukeys[0].shape[0]
    else:
        key_ids, ukeys, inverse, G = [], [], np.zeros(n, np.int64), 1
    out = {}
    for tree in args["results"]:
        tree = _strip(tree)
        oid = get_id(_right_most(tree))
        if _is_key(tree):
            kid = get_id(tree if isinstance(tree, str) else tree[0])
            uk = ukeys[key_ids.index(kid)]
            out[oid] = uk.reshape(G, uk.shape[1] if uk.ndim == 2 else 1).astype(m[kid].dtype)
        else:
            out[oid] = eval_agg_expr(tree, m, (inverse, G, n))     # :276-281: evaluate(tree)
    return out


# ---------------------------------------------------------------------------
# Sort: operators/sort.py:6-58
# ---------------------------------------------------------------------------
def _stable_order(x: np.ndarray, desc: bool) -> np.ndarray:
    if x.ndim == 2:                                                 # :31-35 (unique ranks of rows)
        _, inv = np.unique(x, axis=0, return_inverse=True)
        x = inv.reshape(-1)
    if not desc:
        return np.argsort(x, kind="stable")                         # NaN sorts last, as torch puts it
    if x.dtype.kind == "f":
        return np.lexsort((-x, ~np.isnan(x)))                       # torch: NaN is the largest, first when descending
    return np.argsort(~x.astype(np.int64), kind="stable")


def sort_perm(key_cols: Sequence[np.ndarray], descs: Sequence[bool]) -> np.ndarray:
    """LSD sequence of stable sorts from the last key to the first (:22-35)."""
    n = key_cols[0].shape[0]
    perm = np.arange(n, dtype=np.int64)
    for k, d in zip(reversed(list(key_cols)), reversed(list(descs))):
        perm = perm[_stable_order(k[perm], d)]
    return perm


def tqp_sort(cols: Dict[int, np.ndarray], args: dict, with_limit: bool):
    """sort.py:6-58: returns {id: reordered array} for every input id."""
    perm = sort_perm([cols[k] for k in args["key ids"]], args["key orders"])
    if with_limit:
        perm = perm[: args["limit"]]
    return {c: cols[c][perm] for c in args["input ids"]}


def tqp_project(cols: Dict[int, np.ndarray], args: dict) -> Dict[int, np.ndarray]:
    """operators/project.py:10-69: renames, then every computed expression of 'used expr'
    (a bare column or `column AS name` is only renamed) evaluated row-wise
    (aggregate.py:203-233 arithmetic), stored as float64 and cast back to the
    expression's dtype, placed at 'materialized out' in order."""
    out = dict(cols)
    for orig, new in args["rename map"].items():           # :13-14
        out[new] = out[orig]
    results = []
    for tree in args["used expr"]:                          # :23-40
        while isinstance(tree, list) and len(tree) == 1:
            tree = tree[0]
        if isinstance(tree, str) or (tree[1] == "AS" and isinstance(tree[0], str)):
            continue
        r = eval_agg_expr(tree[0] if len(tree) > 1 and tree[1] == "AS" else tree,
                          {k: out[k] for k in args["materialized in"]})
        results.append(np.asarray(r).astype(np.float64).astype(np.asarray(r).dtype))   # :38, :58
    for i, oid in enumerate(args["materialized out"]):     # :56-61
        out[oid] = results[i]
    return out
