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

Anything else returns 0 and runs nothing, and so does a build side whose key repeats (the
fused form needs a primary key): the executor then runs the same operators one by one.
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
    pipe = JoinAggTopK(bk, kmin, kmax, pv.tensor.reshape(-1), _fcols(tensor_group, fb) if fb else {},
                       fb["filter tree"] if fb else None, pcols, fp["filter tree"] if fp else None,
                       m["value_tree"], k=m["k"], descending=m["desc"])
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


def try_fused(gpu_enable, tensor_group: Dict[int, object], ops: List[int], args: Dict[int, dict], start: int = 0) -> int:
    """Runs ops[start:start+m] (their argument dicts in args) as one fused pipeline when they form a
    shape covered here; returns m, or 0 when nothing ran (the executor then runs ops[start])."""
    if not gpu_enable or start >= len(ops):
        return 0
    m = _match_join_agg_topk(tensor_group, ops, args, start)
    if m is not None and _run_join_agg_topk(tensor_group, m):
        return m["n_ops"]
    return 0
