"""Drop-in ``join_vortex`` / ``join_kernel_new`` (operators/hashjoin.py).

``join_vortex`` keeps the reference's argument handling (hashjoin.py:191-208:
key normalisation, ``materialized in`` per side, masks popped from
``args['mask map']``) and its return value (the row count of the first
``tensor_group`` entry, :248).  The work differs in three places, none of
which changes a result:

* masked inputs are not compacted (vortex_pipeline.py:58); the build and the
  probe skip failing rows in place and emit ids of the original rows;
* the sort / unique_consecutive / searchsorted / padded-matrix expansion
  (:39-97) is one directory build plus one single-pass probe kernel;
* the output columns are gathered by one multi-column gather kernel
  (:153-175, with index_with_null for right-outer, conversion.py:52-57).

Extra join conditions (:100-108, e.g. the second key of a two-key join,
main.py:208-217) are evaluated on the gathered pair columns with the
predicate kernel and the pairs compacted; the semi, anti and outer forms are
then derived from the probe rows that keep a pair (:110-151).
"""
from __future__ import annotations

from typing import Dict, List

import torch

from .. import _lib as L
from ..ops import check_deferred, compact, filter_mask, gather, join_build, join_probe, mark_rows
from ..predicate import compile_filter
from ..variable import make_like, wait_ready
from ._materialize import materialize
from .filter import _require_gpu

LEFT, RIGHT = 0, 1


def _normalize(v):
    if hasattr(v, "normalize"):
        v.normalize()
    elif v.tensor.dim() == 2:
        v.tensor = v.tensor.squeeze()


def _side_mask(tensor_group, cols: List[int], mask_map: Dict[int, int], key: int):
    """The one mask shared by a side's columns (None when the side is unfiltered), or the string
    "mixed" when its columns carry different masks or some carry none."""
    masks = {mask_map.get(c) for c in cols}
    if key not in cols:
        masks.add(mask_map.get(key))
    if len(masks) > 1:
        return "mixed"
    m = masks.pop() if masks else None
    return tensor_group[m].tensor if m is not None else None


def _pairs(tensors_left, tensors_right, left_key, right_key, condition_list, jtype, left_mask, right_mask):
    lk = tensors_left[left_key].tensor
    rk = tensors_right[right_key].tensor
    wait_ready(tensors_left[left_key])
    b = join_build(lk, left_mask)
    wait_ready(tensors_right[right_key])
    # with extra conditions every form starts from the key-equal pairs (hashjoin.py:100-108)
    bi, pi = join_probe(b, rk, right_mask, "inner" if condition_list else jtype)
    for cond in condition_list:                       # hashjoin.py:100-108
        ids = set()
        _collect_ids(cond, ids)
        cols = {}
        for cid in ids:
            if cid in tensors_left:
                wait_ready(tensors_left[cid])
                cols[cid] = gather([tensors_left[cid].tensor], bi)[0]
            else:
                wait_ready(tensors_right[cid])
                cols[cid] = gather([tensors_right[cid].tensor], pi)[0]
        pred = compile_filter(cond, cols)
        keep, _ = filter_mask(pred, int(bi.numel()), bi.device)
        (bi, pi), _ = compact([bi, pi], mask=keep)
    if condition_list and jtype != "inner":
        bi, pi = _non_inner(bi, pi, rk, right_mask, jtype)
    key_range = (int(b.plan.key_min), int(b.plan.key_max)) if b.plan.key_max >= b.plan.key_min else None
    return bi, pi, b.plan.nb_rows, key_range


def _non_inner(bi, pi, rk, right_mask, jtype):
    """hashjoin.py:110-151 from the pairs left after the conditions: semi = probe rows with
    a pair (ascending), anti = probe rows (passing their mask) without one, outer = the
    pairs followed by the anti rows with a null build index."""
    n = int(rk.numel())
    hit = mark_rows(pi, n)
    dev = rk.device
    if jtype == "right-semi":
        (rows,), _ = compact([], mask=hit, with_row_ids=True)
        return torch.empty(0, dtype=torch.int64, device=dev), rows
    tree = ["NOT", ["h#2"]] if right_mask is None else [["m#1"], "AND", ["NOT", ["h#2"]]]
    cols = {2: hit} if right_mask is None else {1: right_mask.to(torch.bool), 2: hit}
    lone, _ = filter_mask(compile_filter(tree, cols), n, dev)
    (rows,), _ = compact([], mask=lone, with_row_ids=True)
    if jtype == "right-anti":
        return torch.empty(0, dtype=torch.int64, device=dev), rows
    nulls = torch.full((rows.numel(),), L.NULL_INDEX, dtype=torch.int64, device=dev)
    return torch.cat([bi, nulls]), torch.cat([pi, rows])


def _collect_ids(tree, out):
    if isinstance(tree, str):
        if "#" in tree and not tree.startswith("Brand#"):
            out.add(int(tree.split("#")[-1].replace("L", "")))
    elif isinstance(tree, list):
        if len(tree) == 3 and tree[1] == "#":
            out.add(int(tree[-1]))
            return
        for e in tree:
            _collect_ids(e, out)


def join_kernel_new(gpu_enable, tensors_left, tensors_right, left_key, right_key, condition_list, join_output_keys,
                    return_global_index, type, left_global_idx, right_global_idx, left_mask=None, right_mask=None):
    """hashjoin.py:24-177 on unmasked (already materialised) inputs."""
    assert type in {"inner", "right-semi", "right-anti", "right-outer"}, "Invalid Join type."
    _normalize(tensors_left[left_key])
    _normalize(tensors_right[right_key])
    bi, pi, _, _ = _pairs(tensors_left, tensors_right, left_key, right_key, condition_list, type, left_mask,
                          right_mask)
    return _outputs(tensors_left, tensors_right, join_output_keys, type, bi, pi, return_global_index,
                    left_global_idx, right_global_idx)


_side = {}


def _pending(v) -> bool:
    """A column whose host copy has not finished yet (its `ready` event is not complete)."""
    ev = getattr(v, "ready", None)
    return ev is not None and not ev.query()


def _gather_when_ready(v, idx, null_aware):
    """col[idx] on a side stream after the column's copy and this stream's work so far (the
    indices); returns the output and the event after the gather."""
    dev = idx.device
    side = _side.get(dev.index)
    if side is None:
        side = _side[dev.index] = torch.cuda.Stream(dev)
    main = torch.cuda.current_stream(dev)
    side.wait_stream(main)
    side.wait_event(v.ready)
    with torch.cuda.stream(side):
        o = gather([v.tensor], idx, null_aware)[0]
        ev = torch.cuda.Event()
        ev.record(side)
    o.record_stream(main)            # read on the caller's stream after the event
    idx.record_stream(side)
    v.tensor.record_stream(side)
    return o, ev


def _outputs(tensors_left, tensors_right, keys, jtype, bi, pi, return_global_index=False, lg=None, rg=None,
             left_rows=None, right_rows=None, ready_out=None):
    null_aware = False
    if jtype == "right-outer":
        n_pairs = int((bi != L.NULL_INDEX).sum().item()) if bi.numel() else 0
        if n_pairs == 0:          # hashjoin.py:154: no null padding without a match
            bi = bi[:0]
        else:
            null_aware = True
    elif jtype in ("right-semi", "right-anti"):
        bi = torch.empty(0, dtype=torch.int64, device=pi.device)
    lcols = [k for k in keys if k in tensors_left]
    rcols = [k for k in keys if k not in tensors_left]
    # columns still arriving are gathered on a side stream once they land; their outputs carry
    # the gather's event, so this join (and whatever the caller queues next) does not wait here
    late_l = [k for k in lcols if _pending(tensors_left[k])]
    late_r = [k for k in rcols if _pending(tensors_right[k])]
    now_l = [k for k in lcols if k not in late_l]
    now_r = [k for k in rcols if k not in late_r]
    wait_ready(*[tensors_left[k] for k in now_l], *[tensors_right[k] for k in now_r])
    out = {}
    if now_l:
        out.update(zip(now_l, gather([tensors_left[k].tensor for k in now_l], bi, null_aware)))
    if now_r:
        out.update(zip(now_r, gather([tensors_right[k].tensor for k in now_r], pi)))
    events = {}
    for k in late_l:
        out[k], events[k] = _gather_when_ready(tensors_left[k], bi, null_aware)
    for k in late_r:
        out[k], events[k] = _gather_when_ready(tensors_right[k], pi, False)
    if ready_out is not None:
        ready_out.update(events)
    lout = [out[k] for k in lcols]
    rout = [out[k] for k in rcols]
    res, li, ri = [], iter(lout), iter(rout)
    for k in keys:                                     # hashjoin.py:161-172
        if k in tensors_left:
            rows = left_rows if left_rows is not None else tensors_left[k].tensor.shape[0]
            res.append(next(li) if rows > 0 else torch.tensor([]))
        else:
            rows = right_rows if right_rows is not None else tensors_right[k].tensor.shape[0]
            res.append(next(ri) if rows > 0 else torch.tensor([]))
    if return_global_index:
        res.extend(gather([lg.tensor], bi, null_aware) + gather([rg.tensor], pi))
    return res


def join_vortex(gpu_enable, tensor_group, args, leftcol, rightcol, condition_list, type, cpu_mem_pool,
                gpu_mem_pool, name):
    _require_gpu(gpu_enable)
    check_deferred()
    join_key_index = [leftcol, rightcol]
    groupings = [args["left group"], args["right group"]]
    join_mask_map, join_output = {}, []
    side_cols = [[], []]
    for side in (LEFT, RIGHT):                         # hashjoin.py:198-208
        _normalize(tensor_group[join_key_index[side]])
        for used_col in args["materialized in"]:
            if used_col in groupings[side]:
                join_output.append(used_col)
                side_cols[side].append(used_col)
                if "mask map" in args and used_col in args["mask map"]:
                    join_mask_map[used_col] = args["mask map"].pop(used_col)
    masks = [_side_mask(tensor_group, side_cols[s] or [join_key_index[s]], join_mask_map, join_key_index[s])
             for s in (LEFT, RIGHT)]
    tl = {k: tensor_group[k] for k in groupings[LEFT] if k in tensor_group}
    tr = {k: tensor_group[k] for k in groupings[RIGHT] if k in tensor_group}
    for s, t in ((LEFT, tl), (RIGHT, tr)):
        if isinstance(masks[s], str):
            # a side whose columns carry different masks (or masked beside compacted ones): each
            # masked column is compacted by its own mask first (vortex_pipeline.py:54-58) and the
            # side joins unmasked
            cols = set(side_cols[s]) | {join_key_index[s]}
            t.update(materialize(tensor_group, cols, join_mask_map))
            lengths = {t[c].tensor.shape[0] for c in cols}
            if len(lengths) > 1:
                raise RuntimeError(f"join inputs have different lengths after their masks: {sorted(lengths)}")
            masks[s] = None
    if leftcol not in tl or rightcol not in tr:
        raise KeyError("join key is not in its side's group")
    bi, pi, nb_rows, key_range = _pairs(tl, tr, leftcol, rightcol, condition_list, type, masks[LEFT],
                                        masks[RIGHT])
    # only "does the probe side have rows" matters (hashjoin.py:161-172); any output row answers it
    if pi.numel() > 0:
        np_rows = int(pi.numel())
    else:
        np_rows = int(masks[RIGHT].sum().item()) if masks[RIGHT] is not None else tr[rightcol].tensor.shape[0]
    late = {}
    outs = _outputs(tl, tr, join_output, type, bi, pi, left_rows=nb_rows, right_rows=np_rows, ready_out=late)
    for i, k in enumerate(join_output):                # hashjoin.py:234-238
        tensor_group[k] = make_like(tensor_group[k], outs[i], tensor_group[k].tensor_type)
        if k in late:                                  # gathered on a side stream after a late input
            tensor_group[k].ready = late[k]
        if type == "inner" and key_range is not None and k in (leftcol, rightcol):
            tensor_group[k]._key_range = key_range     # every output key equals a filtered build key
    return next(iter(tensor_group.values())).tensor.size(0)
