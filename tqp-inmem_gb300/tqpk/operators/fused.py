"""Plan-shape entry for a plan executor: runs a recognised run of operators as one fused pipeline.

TQP-Inmem's executor (main.py:123-279) calls one operator at a time, so the drop-in operators
materialise every intermediate the reference does: the join's pairs and gathered columns, the
group table, the full sort before the limit.  ``try_fused`` lets the executor hand a run of its
operators to a fused pipeline instead:

    i = 0
    while i < len(ops):
        m = try_fused(gpu_enable, tensor_group, ops, args, i) if gpu_enable else 0
        if m:
            i += m
            continue
        ...                       # the existing per-operator dispatch of ops[i]
        i += 1

Recognised shape (the plan main.py:152-253 runs for a filtered equi-join + aggregate + top-k):

    [Filter (build side)] [Filter (probe side)] Join (inner, one key, no condition)
    Aggregate (grouped by the build key; one sum of an expression over probe columns)
    take ordered (by that sum, limit <= 256)

It runs as tqpk.pipeline.JoinAggTopK: the build side's membership bitmap, one probe pass that
accumulates the sums in a slot table, one top-k pass.  Its outputs are the take-ordered
operator's: the key column ([m, 1], the build key's dtype and type) and the sum column (float64)
in the stable order of the operator path (sum, then ascending key); each output also carries `host`,
its rows as a numpy array, brought back by the same device-to-host read as the row count
(tqpk.variable.host_values reads it).  The intermediate columns of
the run (the filters' masks, the joined columns, the full group table) are not produced; the
plan's later operators only read the take-ordered operator's outputs in this shape.

and the star plan (main.py:152-253 with three joins):

    [Filter (dimension A)] [Filter (fact)] Join (A.key = fact.fkA) Join (B.key = fact.fkB)
    Join (C.key = B.fkC), all inner on one key; Aggregate (grouped by C's key; one sum of an
    expression over fact columns, optionally count(1)); take ordered (by that sum, limit <= 256)

runs as tqpk.pipeline.StarAggTopK: direct-address directories of A (its filter applied), B (composed
with C's) and C, one probe pass over the fact rows, one top-k; its outputs are the take-ordered
operator's (C key [m, 1], sum float64, count int64) in the same order.

Anything else returns 0 and runs nothing, and so does a build or dimension side whose key repeats
(the fused forms need primary keys): the executor then runs the same operators one by one.
"""
from __future__ import annotations

from typing import Dict, List, Optional

import torch

from ..predicate import get_id
from ..variable import make_like, wait_ready


def _tree_ids(t, out):
    if isinstance(t, str):
        if "#" in t:
            try:
                out.add(get_id(t))
            except ValueError:
                pass
    elif isinstance(t, (list, tuple)):
        for e in t:
            _tree_ids(e, out)
    return out


def _unwrap(t):
    while isinstance(t, list) and len(t) == 1:
        t = t[0]
    return t


def _is_key(t) -> bool:
    t = _unwrap(t)
    return isinstance(t, str) or (isinstance(t, list) and len(t) == 3 and t[1] == "AS" and isinstance(t[0], str))


def _sum_result(t):
    """The value tree of [[["sum", tree], "#", id], "AS", "name#out"] and the output id, else None."""
    t = _unwrap(t)
    if not (isinstance(t, list) and len(t) == 3 and t[1] == "AS"):
        return None
    call = _unwrap(t[0])
    if not (isinstance(call, list) and len(call) == 3 and call[1] == "#"):
        return None
    fn = _unwrap(call[0])
    if not (isinstance(fn, list) and len(fn) == 2 and fn[0] == "sum"):
        return None
    return fn[1], get_id(t[2])


def _match_join_agg_topk(tensor_group, ops, args, start) -> Optional[dict]:
    i, filters = start, []
    while i < len(ops) and args[ops[i]].get("name") == "Filter" and len(filters) < 2:
        filters.append(args[ops[i]])
        i += 1
    if i + 3 > len(ops):
        return None
    j, a, t = (args[ops[i]], args[ops[i + 1]], args[ops[i + 2]])
    if (j.get("name"), a.get("name"), t.get("name")) != ("Join", "Aggregate", "take ordered"):
        return None
    if j.get("join type") != "Inner" or "join condition" in j:
        return None
    if len(j.get("left keys", [])) != 1 or len(j.get("right keys", [])) != 1:
        return None
    bk, pk = j["left keys"][0], j["right keys"][0]
    left, right = set(j["left group"]), set(j["right group"])
    if bk not in left or pk not in right or bk not in tensor_group or pk not in tensor_group:
        return None
    # the filters: each one's mask guards one side of the join, computed from that side's columns
    mask_map = j.get("mask map", {})
    side_filter = {}
    for f in filters:
        mid = f.get("out mask id")
        cols = set(f.get("materialized in", []))
        guarded = {c for c, m in mask_map.items() if m == mid}
        if not guarded or "filter tree" not in f:
            return None
        side = "b" if guarded <= left and cols <= left else "p" if guarded <= right and cols <= right else None
        if side is None or side in side_filter:
            return None
        side_filter[side] = f
    for c, m in mask_map.items():          # every masked join input is covered by one of these filters
        if c in left and (side_filter.get("b") is None or side_filter["b"]["out mask id"] != m):
            return None
        if c in right and (side_filter.get("p") is None or side_filter["p"]["out mask id"] != m):
            return None
    # the aggregate: group by the build key, one sum over probe columns
    if a.get("is partial") or "mask map" in a:
        return None
    keys = a.get("keys") or []
    if len(keys) != 1 or get_id(keys[0]) != bk:
        return None
    results = a.get("results", [])
    key_res = [r for r in results if _is_key(r)]
    sums = [r for r in results if not _is_key(r)]
    if len(key_res) != 1 or len(sums) != 1 or len(a.get("out agg ids", [])) != 1:
        return None
    kr = _unwrap(key_res[0])
    key_in = get_id(kr if isinstance(kr, str) else kr[0])
    key_out = get_id(kr if isinstance(kr, str) else kr[-1])
    sr = _sum_result(sums[0])
    if key_in != bk or sr is None:
        return None
    value_tree, agg_out = sr
    if agg_out != a["out agg ids"][0]:
        return None
    vcols = _tree_ids(value_tree, set())
    if not vcols or not vcols <= right or any(c not in tensor_group for c in vcols):
        return None
    # take ordered by that sum
    limit = t.get("limit")
    if not isinstance(limit, int) or not 1 <= limit <= 256:
        return None
    if list(t.get("key ids", [])) != [agg_out] or len(t.get("key orders", [])) != 1:
        return None
    if set(t.get("input ids", [])) != {key_out, agg_out}:
        return None
    bkt = tensor_group[bk].tensor
    pkt = tensor_group[pk].tensor
    if bkt.dtype not in (torch.int32, torch.int64) or pkt.dtype not in (torch.int32, torch.int64):
        return None
    if bkt.dim() != 1 and not (bkt.dim() == 2 and bkt.shape[1] == 1):
        return None
    return {"n_ops": len(filters) + 3, "bk": bk, "pk": pk, "filters": side_filter, "value_tree": [value_tree],
            "vcols": sorted(vcols), "k": limit, "desc": bool(t["key orders"][0]), "key_out": key_out,
            "agg_out": agg_out}


def _fcols(tensor_group, f):
    return {c: tensor_group[c].tensor.reshape(-1) if tensor_group[c].tensor.dim() == 2 and
            tensor_group[c].tensor.shape[1] == 1 else tensor_group[c].tensor for c in f["materialized in"]}


def _run_join_agg_topk(tensor_group, m) -> bool:
    from .. import _lib as L
    from ..ops import key_range
    from ..pipeline import JoinAggTopK
    bv, pv = tensor_group[m["bk"]], tensor_group[m["pk"]]
    if not (bv.tensor.is_cuda and pv.tensor.is_cuda):
        return False
    fb, fp = m["filters"].get("b"), m["filters"].get("p")
    build_vars = [bv] + ([tensor_group[c] for c in fb["materialized in"]] if fb else [])
    probe_vars = [pv] + ([tensor_group[c] for c in fp["materialized in"]] if fp else []) + \
        [tensor_group[c] for c in m["vcols"]]
    wait_ready(bv)
    bk = bv.tensor.reshape(-1)
    if bk.numel() == 0:
        return False
    kmin, kmax = key_range(bk)                       # the build key's domain (one host read)
    if kmax - kmin + 1 > (1 << 31):
        return False
    pcols = {c: tensor_group[c].tensor.reshape(-1) for c in set(m["vcols"]) | (set(fp["materialized in"]) if fp else set())}
    try:
        pipe = JoinAggTopK(bk, kmin, kmax, pv.tensor.reshape(-1), _fcols(tensor_group, fb) if fb else {},
                           fb["filter tree"] if fb else None, pcols, fp["filter tree"] if fp else None,
                           m["value_tree"], k=m["k"], descending=m["desc"])
    except NotImplementedError:                      # e.g. a float32 sum: the operators run instead
        return False
    wait_ready(*build_vars)
    pipe.run(before_probe=lambda: wait_ready(*probe_vars))
    try:
        keys, vals, count = pipe.result_device(key_dtype=bv.tensor.dtype)   # cast queued before the read
    except NotImplementedError:                      # a repeated build key: the operator path runs instead
        return False
    tensor_group[m["key_out"]] = kv = make_like(bv, keys.reshape(count, 1), bv.tensor_type)
    tensor_group[m["agg_out"]] = sv = make_like(bv, vals, "float")
    hk, hs = pipe.result_host                         # read together with the count
    kv.host, sv.host = hk.reshape(count, 1), hs
    return True


def _join_parts(j):
    """(left key, right key, left group, right group) of an inner one-key join without a
    condition, else None."""
    if j.get("name") != "Join" or j.get("join type") != "Inner" or "join condition" in j:
        return None
    if len(j.get("left keys", [])) != 1 or len(j.get("right keys", [])) != 1:
        return None
    return j["left keys"][0], j["right keys"][0], set(j["left group"]), set(j["right group"])


def _int_key(tensor_group, c) -> bool:
    t = tensor_group[c].tensor if c in tensor_group else None
    return (t is not None and t.dtype in (torch.int32, torch.int64)
            and (t.dim() == 1 or (t.dim() == 2 and t.shape[1] == 1)))


def _count_result(t):
    """The output id of [[["count", ["1"]], "#", id], "AS", "name#out"], else None."""
    t = _unwrap(t)
    if not (isinstance(t, list) and len(t) == 3 and t[1] == "AS"):
        return None
    call = _unwrap(t[0])
    if not (isinstance(call, list) and len(call) == 3 and call[1] == "#"):
        return None
    fn = _unwrap(call[0])
    if not (isinstance(fn, list) and len(fn) == 2 and fn[0] == "count" and _unwrap(fn[1]) == "1"):
        return None
    return get_id(t[2])


def _match_star_agg_topk(tensor_group, ops, args, start) -> Optional[dict]:
    """[Filter (A)] [Filter (fact)] Join(A, fact.fkA) Join(B, fact.fkB) Join(C, B.fkC),
    Aggregate by the C key (one sum over fact columns, optionally count(1)), take ordered by
    the sum (main.py:152-253 for the star plan)."""
    i, filters = start, []
    while i < len(ops) and args[ops[i]].get("name") == "Filter" and len(filters) < 2:
        filters.append(args[ops[i]])
        i += 1
    if i + 5 > len(ops):
        return None
    j1, j2, j3, a, t = (args[ops[i + q]] for q in range(5))
    if (a.get("name"), t.get("name")) != ("Aggregate", "take ordered"):
        return None
    parts = [_join_parts(j) for j in (j1, j2, j3)]
    if any(p is None for p in parts):
        return None
    (ak, fka, a_grp, f_grp), (bk, fkb, b_grp, r2), (ck, fkc, c_grp, r3) = parts
    if not (ak in a_grp and fka in f_grp and bk in b_grp and fkb in f_grp and fkb in r2
            and ck in c_grp and fkc in b_grp and fkc in r3):
        return None
    if any(not _int_key(tensor_group, c) for c in (ak, fka, bk, fkb, ck, fkc)):
        return None
    if j2.get("mask map") or j3.get("mask map"):
        return None
    # the filters: each guards A's or the fact table's columns of the first join
    mask_map = j1.get("mask map", {})
    side_filter = {}
    for fl in filters:
        mid = fl.get("out mask id")
        cols = set(fl.get("materialized in", []))
        guarded = {c for c, m in mask_map.items() if m == mid}
        if not guarded or "filter tree" not in fl:
            return None
        side = "a" if guarded <= a_grp and cols <= a_grp else "f" if guarded <= f_grp and cols <= f_grp else None
        if side is None or side in side_filter:
            return None
        side_filter[side] = fl
    for c, m in mask_map.items():
        grp = "a" if c in a_grp else "f" if c in f_grp else None
        if grp is None or side_filter.get(grp) is None or side_filter[grp]["out mask id"] != m:
            return None
    # the aggregate: by the C key, one sum over fact columns, optionally count(1)
    if a.get("is partial") or "mask map" in a:
        return None
    keys = a.get("keys") or []
    if len(keys) != 1 or get_id(keys[0]) != ck:
        return None
    results = a.get("results", [])
    key_res = [r for r in results if _is_key(r)]
    others = [r for r in results if not _is_key(r)]
    if len(key_res) != 1:
        return None
    kr = _unwrap(key_res[0])
    if get_id(kr if isinstance(kr, str) else kr[0]) != ck:
        return None
    key_out = get_id(kr if isinstance(kr, str) else kr[-1])
    sums = [_sum_result(r) for r in others]
    counts = [_count_result(r) for r in others]
    if sum(x is not None for x in sums) != 1 or any(x is None and y is None for x, y in zip(sums, counts)):
        return None
    value_tree, agg_out = next(x for x in sums if x is not None)
    cnt_out = [y for x, y in zip(sums, counts) if x is None]
    if len(cnt_out) > 1:
        return None
    cnt_out = cnt_out[0] if cnt_out else None
    if sorted(a.get("out agg ids", [])) != sorted([agg_out] + ([cnt_out] if cnt_out is not None else [])):
        return None
    vcols = _tree_ids(value_tree, set())
    if not vcols or not vcols <= f_grp or any(c not in tensor_group for c in vcols):
        return None
    limit = t.get("limit")
    if not isinstance(limit, int) or not 1 <= limit <= 256:
        return None
    if list(t.get("key ids", [])) != [agg_out] or len(t.get("key orders", [])) != 1:
        return None
    if set(t.get("input ids", [])) != {key_out, agg_out} | ({cnt_out} if cnt_out is not None else set()):
        return None
    return {"n_ops": len(filters) + 5, "keys": (ak, fka, bk, fkb, ck, fkc), "filters": side_filter,
            "value_tree": [value_tree], "vcols": sorted(vcols), "k": limit, "desc": bool(t["key orders"][0]),
            "key_out": key_out, "agg_out": agg_out, "cnt_out": cnt_out}


def _run_star_agg_topk(tensor_group, m) -> bool:
    from ..ops import key_range
    from ..pipeline import StarAggTopK
    ak, fka, bk, fkb, ck, fkc = m["keys"]
    v = {c: tensor_group[c] for c in (ak, fka, bk, fkb, ck, fkc)}
    if not all(x.tensor.is_cuda for x in v.values()):
        return False
    fa, ff = m["filters"].get("a"), m["filters"].get("f")
    dim_vars = [v[ak], v[bk], v[fkc], v[ck]] + ([tensor_group[c] for c in fa["materialized in"]] if fa else [])
    fact_vars = [v[fka], v[fkb]] + [tensor_group[c] for c in m["vcols"]] + \
        ([tensor_group[c] for c in ff["materialized in"]] if ff else [])
    wait_ready(*dim_vars)
    col = lambda c: tensor_group[c].tensor.reshape(-1)          # noqa: E731
    doms = []
    for c in (ak, bk, ck):                                      # the dimension key domains (host reads)
        if col(c).numel() == 0:
            return False
        lo, hi = key_range(col(c))
        if hi - lo + 1 > (1 << 31):
            return False
        doms.append((lo, hi))
    fact_cols = {c: col(c) for c in set(m["vcols"]) | (set(ff["materialized in"]) if ff else set())}
    a_cols = {c: col(c) for c in fa["materialized in"]} if fa else {}
    try:
        pipe = StarAggTopK(col(fka), col(fkb), fact_cols, ff["filter tree"] if ff else None, m["value_tree"],
                           col(ak), a_cols, fa["filter tree"] if fa else None, doms[0], col(bk), col(fkc), doms[1],
                           col(ck), doms[2], k=m["k"], descending=m["desc"])
        pipe.run(before_probe=lambda: wait_ready(*fact_vars))
        keys, vals, cnts, count = pipe.result_device()
    except NotImplementedError:                   # a repeated dimension key: the operators run instead
        return False
    cv = v[ck]
    kt = cv.tensor.dtype
    tensor_group[m["key_out"]] = kv = make_like(cv, keys.to(kt).reshape(count, 1), cv.tensor_type)
    tensor_group[m["agg_out"]] = sv = make_like(cv, vals, "float")
    hk, hs, hc = pipe.result_host
    kv.host, sv.host = hk.astype(str(kt).replace("torch.", "")).reshape(count, 1), hs
    if m["cnt_out"] is not None:
        tensor_group[m["cnt_out"]] = nv = make_like(cv, cnts, "int")
        nv.host = hc
    return True


def try_fused(gpu_enable, tensor_group: Dict[int, object], ops: List[int], args: Dict[int, dict], start: int = 0) -> int:
    """Runs ops[start:start+m] (their argument dicts in args) as one fused pipeline when they form a
    shape covered here; returns m, or 0 when nothing ran (the executor then runs ops[start])."""
    if not gpu_enable or start >= len(ops):
        return 0
    m = _match_join_agg_topk(tensor_group, ops, args, start)
    if m is not None and _run_join_agg_topk(tensor_group, m):
        return m["n_ops"]
    m = _match_star_agg_topk(tensor_group, ops, args, start)
    if m is not None and _run_star_agg_topk(tensor_group, m):
        return m["n_ops"]
    return 0
