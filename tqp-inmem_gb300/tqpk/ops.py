"""Tensor-level wrappers of the libtqpk C ABI.

Every function takes device tensors, allocates outputs and workspaces through
torch's caching allocator, launches on the current CUDA stream and raises a
Python exception for a non-zero status.  There is no CPU or torch fallback:
if libtqpk.so is missing or a shape is unsupported the call raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _lib as L
from .dtypes import code_of, dtype_of
from .expr import AggregateProgram
from .predicate import CompiledPredicate


def _ws(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def _stream(device) -> int:
    return L.stream_handle(device)


def _col1d(t: torch.Tensor) -> torch.Tensor:
    if t.dim() == 2 and t.shape[1] == 1:
        t = t.reshape(-1)
    if t.dim() != 1:
        raise NotImplementedError(f"2-D column {tuple(t.shape)} is not on the kernel path")
    return t.contiguous()


def _check_cuda(*ts):
    for t in ts:
        if t is not None and not t.is_cuda:
            raise ValueError("tqpk kernels take CUDA tensors (no CPU fallback)")


def _vp_array(ptrs: Sequence[Optional[int]]):
    arr = (C.c_void_p * max(len(ptrs), 1))()
    for i, p in enumerate(ptrs):
        arr[i] = p
    return arr


def _i32_array(vals: Sequence[int]):
    arr = (C.c_int32 * max(len(vals), 1))()
    for i, v in enumerate(vals):
        arr[i] = v
    return arr


# ---------------------------------------------------------------- (a) filter
def filter_mask(pred: CompiledPredicate, n: int, device, with_count: bool = False):
    """Bool mask of the predicate over n rows and, with_count, a device count of true rows
    (else None)."""
    lib = L.load()
    mask = torch.empty(n, dtype=torch.bool, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device) if with_count else None
    _check_cuda(*pred.tensors)
    L.check(lib.tqpk_filter_mask(C.byref(pred.struct), n, mask.data_ptr() if n else None,
                                 count.data_ptr() if count is not None else None, _stream(device)),
            "tqpk_filter_mask")
    return mask, count


def fill_masks(masks, device) -> None:
    """Evaluates the conditions of a compiled aggregate/projection (CASE WHEN, comparisons
    used as values) into their preallocated bool columns."""
    lib = L.load()
    for pred, out in masks:
        _check_cuda(out, *pred.tensors)
        n = int(out.numel())
        L.check(lib.tqpk_filter_mask(C.byref(pred.struct), n, out.data_ptr() if n else None, None,
                                     _stream(device)), "tqpk_filter_mask")


def compact(cols: Sequence[torch.Tensor], mask: Optional[torch.Tensor] = None,
            pred: Optional[CompiledPredicate] = None, with_row_ids: bool = False) -> Tuple[List[torch.Tensor], int]:
    """Stable compaction of columns by a mask (or a predicate): tensor[mask]."""
    lib = L.load()
    cols = [_col1d(c) for c in cols]
    if mask is None and pred is None:
        raise ValueError("compact needs a mask or a predicate")
    n = int(mask.numel()) if mask is not None else (int(cols[0].numel()) if cols else 0)
    device = (mask if mask is not None else cols[0]).device
    _check_cuda(mask, *cols)
    outs = [torch.empty(n, dtype=c.dtype, device=device) for c in cols]
    dts = [code_of(c.dtype) for c in cols]
    ins = [c.data_ptr() for c in cols]
    optr = [o.data_ptr() for o in outs]
    if with_row_ids:
        rid = torch.empty(n, dtype=torch.int64, device=device)
        outs.append(rid)
        ins.append(None)
        optr.append(rid.data_ptr())
        dts.append(-1)
    if len(ins) > L.MAX_COLS:
        raise NotImplementedError(f"compaction of more than {L.MAX_COLS} columns")
    cnt = torch.zeros(1, dtype=torch.int64, device=device)
    ws = _ws(lib.tqpk_compact_workspace_bytes(n), device)
    dt_arr = _i32_array([d if d >= 0 else L.ROWID for d in dts])
    L.check(lib.tqpk_compact(C.byref(pred.struct) if pred is not None else None,
                             mask.data_ptr() if mask is not None else None, n, len(ins), _vp_array(ins), dt_arr,
                             _vp_array(optr), cnt.data_ptr(), ws.data_ptr(), ws.numel(), _stream(device)),
            "tqpk_compact")
    m = int(cnt.item())
    if m < 0:                                 # a bounded device wait gave up: the count is its status
        L.check(m, "tqpk_compact")
    return [o[:m] for o in outs], m


def key_range(col: torch.Tensor) -> Tuple[int, int]:
    """(min, max) of an integer column over all its rows (one host read); min > max when empty."""
    lib = L.load()
    col = _col1d(col)
    _check_cuda(col)
    lo, hi = C.c_int64(0), C.c_int64(-1)
    if col.numel() == 0:
        return 0, -1
    scratch = _ws(256, col.device)
    L.check(lib.tqpk_key_range(col.data_ptr(), code_of(col.dtype), col.numel(), scratch.data_ptr(), C.byref(lo),
                               C.byref(hi), _stream(col.device)), "tqpk_key_range")
    return int(lo.value), int(hi.value)


# ---------------------------------------------------------------- (d) group-by
def _count_groups_from_keys(prog: AggregateProgram, plan, pred, n: int, device, s: int) -> int:
    """Occupied slots of the group table, from the key columns (and the mask) alone: a
    count-only pass of the generated kernel into a table of its own, then one host read.
    Lets the group count come back while the value columns are still being copied."""
    from . import jit
    lib = L.load()
    cs = L.GroupbySpec.from_buffer_copy(prog.spec)
    cs.n_cols, cs.n_expr, cs.n_accs = 0, 0, 1            # accumulator 0 counts the rows of a group
    cplan = L.GbPlan.from_buffer_copy(plan)
    ws = _ws(cplan.ws_bytes, device)
    L.check(lib.tqpk_groupby_prepare(C.byref(cs), C.byref(cplan), ws.data_ptr(), ws.numel(), s),
            "tqpk_groupby_prepare")
    jit.run_groupby(cs, pred, cplan, ws, n, s, pred.tensors if pred is not None else (),
                    [t for t in prog.tensors[:prog.spec.n_keys]], ())
    g = C.c_int64(0)
    L.check(lib.tqpk_groupby_count(C.byref(cs), C.byref(cplan), ws.data_ptr(), C.byref(g), s), "tqpk_groupby_count")
    return int(g.value)


def groupby(prog: AggregateProgram, n: int, device, mask: Optional[torch.Tensor] = None,
            pred: Optional[CompiledPredicate] = None, before_values=None, key_ranges=None,
            values_late: bool = False):
    """Runs the compiled aggregate; returns (key columns [G], {out id: column}, G).
    before_values, when given, is called after the plan (which reads only the keys and
    the mask) and before the first kernel that reads the value columns.  key_ranges, when
    given, bounds each key column ((min, max) per key, in spec order): the plan is made from
    them without reading the keys (no host synchronisation), unless they call for the hash
    table of sparse key spaces.  values_late: the value columns are still arriving; the group
    count is then taken from the keys first, and the accumulation and emission are queued
    behind the values without another host synchronisation."""
    lib = L.load()
    _check_cuda(mask, *prog.tensors)
    s = _stream(device)
    plan = L.GbPlan()
    pp = C.byref(pred.struct) if pred is not None else None
    mp = mask.data_ptr() if mask is not None else None
    planned = False
    if key_ranges is not None and len(key_ranges) == prog.spec.n_keys and n > 0:
        nk = prog.spec.n_keys
        kmin = (C.c_int64 * max(nk, 1))(*[int(r[0]) for r in key_ranges])
        kmax = (C.c_int64 * max(nk, 1))(*[int(r[1]) for r in key_ranges])
        planned = (lib.tqpk_groupby_plan_domains(C.byref(prog.spec), kmin, kmax, n, C.byref(plan)) == 0
                   and plan.mode != L.GB_HASH)
        if not planned:
            plan = L.GbPlan()
    if not planned:
        scratch = _ws(256, device)
        L.check(lib.tqpk_groupby_plan(C.byref(prog.spec), pp, mp, n, C.byref(plan), scratch.data_ptr(), s),
                "tqpk_groupby_plan")
    ws = _ws(plan.ws_bytes, device)
    groups = C.c_int64(0)
    from . import jit
    from .predicate import has_strings
    use_jit = (jit.available() and plan.mode != L.GB_HASH and plan.n_rows > 0 and n > 0
               and not has_strings(pred.struct if pred is not None else None))
    if use_jit and mask is not None and pred is None:
        pred = _mask_predicate(mask)              # the mask as a one-instruction predicate
    g_early = None
    if use_jit and values_late and not prog.masks:
        g_early = _count_groups_from_keys(prog, plan, pred, n, device, s)
    if before_values is not None:
        before_values()
    fill_masks(prog.masks, device)
    if use_jit and (mask is None or pred is not None):
        # query-specialised accumulation kernel between the library's prepare and count stages
        L.check(lib.tqpk_groupby_prepare(C.byref(prog.spec), C.byref(plan), ws.data_ptr(), ws.numel(), s),
                "tqpk_groupby_prepare")
        jit.run_groupby(prog.spec, pred, plan, ws, n, s, pred.tensors if pred is not None else (),
                        [t for t in prog.tensors[:prog.spec.n_keys]], prog.tensors[prog.spec.n_keys:])
    ops = []
    for (_, op, a, b, dt) in prog.outputs:
        ops += [op, a, b, code_of(dt)]
    if use_jit and (mask is None or pred is not None):
        # count and emit with one host read: outputs sized for every slot, the device count
        # (or a negative status) read once, then views of the first G rows
        K = int(plan.slots)
        keys = [torch.empty(K, dtype=dtype_of(prog.spec.key_dtypes[k]), device=device) for k in range(prog.spec.n_keys)]
        outs = [torch.empty(K, dtype=dt, device=device) for (_, _, _, _, dt) in prog.outputs]
        gdev = torch.empty(1, dtype=torch.int64, device=device)
        L.check(lib.tqpk_groupby_emit_async(C.byref(prog.spec), C.byref(plan), ws.data_ptr(),
                                            _vp_array([k.data_ptr() for k in keys]), len(outs), _i32_array(ops),
                                            _vp_array([o.data_ptr() for o in outs]), gdev.data_ptr(), s),
                "tqpk_groupby_emit_async")
        if g_early is not None:
            G = g_early                      # the emit's own count (or status) is checked once it lands
            _defer_count_check(gdev, G, "tqpk_groupby_emit_async")
        else:
            G = int(gdev.item())
        if G < 0:
            L.check(G, "tqpk_groupby_emit_async")
        keys = [k[:G] for k in keys]
        outs = [o[:G] for o in outs]
    else:
        L.check(lib.tqpk_groupby_run(C.byref(prog.spec), C.byref(plan), pp, mp, n, ws.data_ptr(), ws.numel(),
                                     C.byref(groups), s), "tqpk_groupby_run")
        G = groups.value
        keys = [torch.empty(G, dtype=dtype_of(prog.spec.key_dtypes[k]), device=device)
                for k in range(prog.spec.n_keys)]
        outs = [torch.empty(G, dtype=dt, device=device) for (_, _, _, _, dt) in prog.outputs]
        L.check(lib.tqpk_groupby_emit(C.byref(prog.spec), C.byref(plan), ws.data_ptr(), G,
                                      _vp_array([k.data_ptr() for k in keys]), len(outs), _i32_array(ops),
                                      _vp_array([o.data_ptr() for o in outs]), s), "tqpk_groupby_emit")
    res = {oid: o for (oid, *_), o in zip(prog.outputs, outs)}
    if prog.casts:
        # aggregates of float32 expressions, accumulated in float64, returned as float32 as the
        # reference returns them, except the avg of its 2-step path (rows / groups >= 2^16), which
        # is float64 there (aggregate.py:127-131, :170)
        rows = int(plan.n_rows) if (pred is not None or mask is not None) else n
        two_step = G > 0 and rows / G >= (1 << 16)
        for oid, (dt, is_avg) in prog.casts.items():
            if oid in res and not (is_avg and two_step):
                res[oid] = res[oid].to(dt)
    if prog.post:
        # arithmetic over aggregates (aggregate.py:197-233): a projection over the group columns
        from .expr import _HIDDEN_ID, compile_projection
        hidden = {oid: res.pop(oid) for oid in list(res) if oid >= _HIDDEN_ID}
        for oid, tree, dt in prog.post:
            pp = compile_projection([tree], hidden)
            res[oid] = project(pp, G, device)[0]
            assert res[oid].dtype == dt
    return keys, res, G, plan


# Counts written on the device by calls that did not wait for them (the group count of an emission
# whose size was known beforehand): each is copied to pinned host memory behind its kernel and
# compared with the size used, once its event has completed.  Every drop-in operator checks them
# on entry, so a failure (a negative status, or a count that disagrees) raises at the latest in
# the next operator call after the one that made it; check_deferred(wait=True) waits for them.
_DEFERRED: list = []


def _defer_count_check(d_count: torch.Tensor, expected: int, what: str) -> None:
    h = torch.empty(1, dtype=torch.int64, pin_memory=True)
    h.copy_(d_count, non_blocking=True)
    ev = torch.cuda.Event()
    ev.record()
    _DEFERRED.append((h, ev, int(expected), what))


def check_deferred(wait: bool = False) -> None:
    """Raises for any deferred device count that came back as an error status or differs from
    the size its call used; entries whose kernels have not finished stay queued (unless wait)."""
    pending, failed = [], None
    for h, ev, expected, what in _DEFERRED:
        if wait:
            ev.synchronize()
        elif not ev.query():
            pending.append((h, ev, expected, what))
            continue
        got = int(h[0])
        if failed is None and got != expected:
            failed = (got, expected, what)
    _DEFERRED[:] = pending
    if failed is not None:
        got, expected, what = failed
        if got < 0:
            L.check(got, what)
        raise RuntimeError(f"{what}: the device counted {got} rows where {expected} were sized")


def _mask_predicate(mask: torch.Tensor) -> CompiledPredicate:
    p = L.Predicate()
    p.n_insn, p.n_cols = 1, 1
    m = mask.contiguous()
    p.cols[0] = m.data_ptr()
    p.dtypes[0] = L.BOOL
    p.insn[0] = L.PredInsn(L.P_MASK, 0, 0, 0, 0, 0.0, 0.0)
    return CompiledPredicate(p, [m], [-1])


# ---------------------------------------------------------------- (b) sort / (e) top-k
def argsort_stable(keys: torch.Tensor, descending: bool = False,
                   perm_in: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Stable sort of keys[perm_in] -> permuted perm_in (int64)."""
    lib = L.load()
    keys = _col1d(keys)
    n = int(perm_in.numel()) if perm_in is not None else int(keys.numel())
    _check_cuda(keys, perm_in)
    out = torch.empty(n, dtype=torch.int64, device=keys.device)
    if n == 0:
        return out
    ws = _ws(lib.tqpk_sort_workspace_bytes(n), keys.device) if n > 2048 else None   # small sorts: one CTA
    L.check(lib.tqpk_argsort_stable(keys.data_ptr(), code_of(keys.dtype), int(bool(descending)),
                                    perm_in.data_ptr() if perm_in is not None else None, n, out.data_ptr(),
                                    ws.data_ptr() if ws is not None else None, ws.numel() if ws is not None else 0,
                                    _stream(keys.device)), "tqpk_argsort_stable")
    return out


def topk_stable(keys: torch.Tensor, k: int, descending: bool = False,
                perm_in: Optional[torch.Tensor] = None) -> torch.Tensor:
    """First k of the stable sort of keys[perm_in] (ties in input order)."""
    lib = L.load()
    keys = _col1d(keys)
    n = int(perm_in.numel()) if perm_in is not None else int(keys.numel())
    m = max(0, min(int(k), n))
    _check_cuda(keys, perm_in)
    out = torch.empty(m, dtype=torch.int64, device=keys.device)
    if m == 0:
        return out
    ws = _ws(lib.tqpk_topk_workspace_bytes(n, m), keys.device)
    L.check(lib.tqpk_topk_stable(keys.data_ptr(), code_of(keys.dtype), int(bool(descending)),
                                 perm_in.data_ptr() if perm_in is not None else None, n, m, out.data_ptr(),
                                 ws.data_ptr(), ws.numel(), _stream(keys.device)), "tqpk_topk_stable")
    return out


# ---------------------------------------------------------------- (c) join
JOIN_TYPES = {"inner": L.JT_INNER, "right-semi": L.JT_SEMI, "right-anti": L.JT_ANTI, "right-outer": L.JT_OUTER}


@dataclass
class JoinBuild:
    plan: L.JoinPlan
    ws: torch.Tensor
    keys: torch.Tensor
    device: torch.device


def join_build(keys: torch.Tensor, mask: Optional[torch.Tensor] = None) -> JoinBuild:
    lib = L.load()
    keys = _col1d(keys)
    _check_cuda(keys, mask)
    if keys.dtype == torch.float64:
        raise NotImplementedError("join on a float64 key is not on the kernel path")
    dev = keys.device
    s = _stream(dev)
    plan = L.JoinPlan()
    scratch = _ws(256, dev)
    mp = mask.data_ptr() if mask is not None else None
    n = int(keys.numel())
    L.check(lib.tqpk_join_plan_build(keys.data_ptr() if n else None, code_of(keys.dtype), mp, n, C.byref(plan),
                                     scratch.data_ptr(), s), "tqpk_join_plan_build")
    ws = _ws(plan.ws_bytes, dev)
    L.check(lib.tqpk_join_build(C.byref(plan), keys.data_ptr() if n else None, code_of(keys.dtype), mp, n,
                                ws.data_ptr(), ws.numel(), s), "tqpk_join_build")
    return JoinBuild(plan, ws, keys, dev)


def join_probe(build: JoinBuild, probe_keys: torch.Tensor, probe_mask: Optional[torch.Tensor] = None,
               join_type: str = "inner") -> Tuple[torch.Tensor, torch.Tensor]:
    """(build_idx, probe_idx) int64 row ids of the original inputs."""
    lib = L.load()
    pk = _col1d(probe_keys)
    _check_cuda(pk, probe_mask)
    if pk.dtype == torch.float64:
        raise NotImplementedError("join on a float64 key is not on the kernel path")
    jt = JOIN_TYPES[join_type]
    dev = build.device
    s = _stream(dev)
    n = int(pk.numel())
    pws = _ws(lib.tqpk_join_probe_workspace_bytes(n), dev)
    mp = probe_mask.data_ptr() if probe_mask is not None else None
    # Unique build keys (and semi/anti joins) give at most one output per probe row.
    cap = n if (build.plan.unique or jt in (L.JT_SEMI, L.JT_ANTI)) else 0
    for _ in range(2):
        ob = torch.empty(cap, dtype=torch.int64, device=dev)
        op = torch.empty(cap, dtype=torch.int64, device=dev)
        cnt = C.c_int64(0)
        st = lib.tqpk_join_probe(C.byref(build.plan), build.ws.data_ptr(), pk.data_ptr() if n else None,
                                 code_of(pk.dtype), mp, n, jt, ob.data_ptr() if cap else None,
                                 op.data_ptr() if cap else None, cap, C.byref(cnt), pws.data_ptr(), pws.numel(), s)
        if st == L.ECAPACITY:
            cap = cnt.value
            continue
        L.check(st, "tqpk_join_probe")
        m = cnt.value
        return ob[:m], op[:m]
    raise RuntimeError("tqpk_join_probe: output size changed between calls")


def gather_rows(col: torch.Tensor, idx: torch.Tensor) -> torch.Tensor:
    """col[idx] for a 2-D [N, w] column (string rows of w bytes)."""
    lib = L.load()
    _check_cuda(col, idx)
    c = col.contiguous()
    n = int(idx.numel())
    out = torch.empty((n,) + tuple(c.shape[1:]), dtype=c.dtype, device=c.device)
    if n == 0:
        return out
    rb = c.element_size() * (c[0].numel() if c.shape[0] else 1)
    L.check(lib.tqpk_gather_rows(c.data_ptr(), int(c.shape[0]), rb, idx.contiguous().data_ptr(), n, out.data_ptr(),
                                 _stream(c.device)), "tqpk_gather_rows")
    return out


def string_words(col: torch.Tensor, word: int) -> torch.Tensor:
    """Sort keys (int64) of 8-byte word `word` of an int8/uint8 [N, w] column."""
    lib = L.load()
    _check_cuda(col)
    c = col.contiguous()
    n, w = int(c.shape[0]), int(c.shape[1])
    out = torch.empty(n, dtype=torch.int64, device=c.device)
    L.check(lib.tqpk_string_words(c.data_ptr() if n else None, n, w, word, int(c.dtype == torch.int8),
                                  out.data_ptr() if n else None, _stream(c.device)), "tqpk_string_words")
    return out


def encode_keys(keys: Sequence[torch.Tensor], mask: Optional[torch.Tensor] = None):
    """Dense group codes of key tuples (string, float and any number of keys):
    (codes int32 [n], reps int64 [G] with groups in ascending key-tuple order, G)."""
    lib = L.load()
    ks, dts, ws = [], [], []
    for k in keys:
        if k.dim() == 2 and k.shape[1] == 1:
            k = k.reshape(-1)
        k = k.contiguous()
        if k.dim() == 2:
            if k.dtype not in (torch.int8, torch.uint8):
                raise NotImplementedError(f"2-D group key of dtype {k.dtype}")
            ws.append(int(k.shape[1]))
        else:
            ws.append(0)
        ks.append(k)
        dts.append(code_of(k.dtype))
    _check_cuda(mask, *ks)
    if len(ks) > L.MAX_COLS:
        raise NotImplementedError(f"more than {L.MAX_COLS} group keys")
    n = int(ks[0].shape[0])
    device = ks[0].device
    codes = torch.empty(n, dtype=torch.int32, device=device)
    reps = torch.empty(max(n, 1), dtype=torch.int64, device=device)
    ws_t = _ws(lib.tqpk_key_encode_workspace_bytes(n), device)
    G = C.c_int64(0)
    L.check(lib.tqpk_key_encode(len(ks), _vp_array([k.data_ptr() for k in ks]), _i32_array(dts), _i32_array(ws),
                                mask.data_ptr() if mask is not None else None, n, codes.data_ptr() if n else None,
                                reps.data_ptr(), C.byref(G), ws_t.data_ptr(), ws_t.numel(), _stream(device)),
            "tqpk_key_encode")
    return codes, reps[:G.value], G.value


def gather(cols: Sequence[torch.Tensor], idx: torch.Tensor, null_aware: bool = False) -> List[torch.Tensor]:
    """out_c = col_c[idx], shaped as torch's indexing shapes it: [K] for a 1-D column, [K, w] for a
    2-D [N, w] column (string rows gathered row by row; [N, 1] through the 1-D kernel).  With
    null_aware an index of -64 yields -64, as the reference's index_with_null (conversion.py:52-57);
    a 2-D column follows that function's broadcast rule (_index_with_null_2d)."""
    if any(c.dim() == 2 for c in cols):
        out = [None] * len(cols)
        flat = [i for i, c in enumerate(cols) if c.dim() == 1 or (c.shape[1] == 1 and not null_aware)]
        rows = set(range(len(cols))) - set(flat)
        for i in sorted(rows):
            out[i] = _index_with_null_2d(cols[i], idx) if null_aware else gather_rows(cols[i], idx)
        if flat:
            for i, o in zip(flat, _gather_1d([cols[i].reshape(-1) for i in flat], idx, null_aware)):
                out[i] = o.reshape(-1, 1) if cols[i].dim() == 2 else o
        return out
    return _gather_1d(cols, idx, null_aware)


def _index_with_null_2d(col: torch.Tensor, idx: torch.Tensor) -> torch.Tensor:
    """index_with_null (conversion.py:52-57) of a 2-D [N, w] column.  The reference gathers with
    null indices read as row 0, then calls masked_fill_ with the [K] null mask, which torch
    broadcasts against the [K, w] rows from the right.  K == 1 fills the row, K == w fills column j
    of every row whose index j is null, and any other K is refused with RuntimeError (the
    reference's right-outer join raises there).  The same three outcomes here."""
    K, w = int(idx.numel()), int(col.shape[1])
    if K not in (1, w):
        raise RuntimeError(f"index_with_null: the [{K}] null mask does not broadcast over [{K}, {w}] rows "
                           "(a right-outer join's 2-D build-side column)")
    null = idx == L.NULL_INDEX
    out = gather([col], idx.masked_fill(null, 0))[0]
    out.masked_fill_(null, L.NULL_INDEX)
    return out


def _gather_1d(cols: Sequence[torch.Tensor], idx: torch.Tensor, null_aware: bool) -> List[torch.Tensor]:
    """tqpk_gather of 1-D columns (at most MAX_COLS per launch)."""
    lib = L.load()
    cols = [_col1d(c) for c in cols]
    _check_cuda(idx, *cols)
    n = int(idx.numel())
    outs = [torch.empty(n, dtype=c.dtype, device=idx.device) for c in cols]
    if n == 0 or not cols:
        return outs
    if len(cols) > L.MAX_COLS:
        return _gather_1d(cols[:L.MAX_COLS], idx, null_aware) + _gather_1d(cols[L.MAX_COLS:], idx, null_aware)
    L.check(lib.tqpk_gather(len(cols), _vp_array([c.data_ptr() for c in cols]),
                            _i32_array([code_of(c.dtype) for c in cols]), idx.contiguous().data_ptr(), n,
                            int(bool(null_aware)), _vp_array([o.data_ptr() for o in outs]), _stream(idx.device)),
            "tqpk_gather")
    return outs


def project(prog, n: int, device) -> List[torch.Tensor]:
    """Evaluates a compiled projection over n rows: one output column per computed expression."""
    from . import jit
    from .dtypes import code_of
    _check_cuda(*prog.tensors)
    # float32 results (torch's default float dtype) are written as their exact float64 values,
    # then narrowed: the same float32
    wdt = [torch.float64 if dt == torch.float32 else dt for (_, dt) in prog.outputs]
    outs = [torch.empty(n, dtype=dt, device=device) for dt in wdt]
    if n == 0 or not outs:
        return [o.to(dt) for o, (_, dt) in zip(outs, prog.outputs)]
    fill_masks(prog.masks, device)
    if not jit.available():
        raise NotImplementedError("projection needs the runtime compiler (NVRTC)")
    src, name = jit.project_source(prog.spec, [(r, code_of(dt)) for (r, _), dt in zip(prog.outputs, wdt)])
    h = jit.compile_kernel(src, name)
    a = jit._Args()
    for c in range(prog.spec.n_cols):
        a.ptr(prog.spec.cols[c])
    for o in outs:
        a.ptr(o.data_ptr())
    a.i64(n)
    a.i32(jit._aligned(*prog.tensors))
    jit.launch(h, jit.occupancy_grid(h, 256, 0, (n + 3) // 4), 256, 0, a, _stream(device))
    return [o if o.dtype == dt else o.to(dt) for o, (_, dt) in zip(outs, prog.outputs)]


def mark_rows(idx: torch.Tensor, n: int) -> torch.Tensor:
    """Bool flags over n rows: True at every index in idx."""
    lib = L.load()
    flags = torch.zeros(n, dtype=torch.bool, device=idx.device)
    _check_cuda(idx)
    idx = idx.contiguous()
    L.check(lib.tqpk_mark_rows(idx.data_ptr() if idx.numel() else None, idx.numel(),
                               flags.data_ptr() if n else None, n, _stream(idx.device)), "tqpk_mark_rows")
    return flags
