"""Drop-in ``tqp_hash_aggregate`` (operators/aggregate.py:236-393).

Keeps the reference's argument handling (``input ids``/``mask map``/``keys``/
``results``/``out agg ids``), its ``tensor_group`` writes (key columns as
[G, 1] tensors with the input key's type, aggregates typed by their dtype,
:380-390) and its return value (rows of the first ``tensor_group`` entry).

The filter mask is applied inside the aggregation kernel (the reference
compacts every input column first, vortex_pipeline.py:58), every aggregate is
computed in the same pass, and groups come out in ascending key order (the
reference's order is the ascending order of a random linear hash of the key
tuple, :320-327; for one non-negative key the two coincide).  Key tuples with a
string (2-D) key, a float key or more than four keys are first numbered by
ops.encode_keys (codes in key-tuple order) and grouped by that code.
"""
from __future__ import annotations

import torch

from ..expr import compile_aggregate, needs_key_codes
from ..ops import check_deferred, encode_keys, gather, groupby
from ._materialize import materialize
from ..variable import make_like, torch_to_type, wait_ready
from .filter import _require_gpu


def tqp_hash_aggregate(gpu_enable, tensor_group, args, gpu_mem_pool, cpu_mem_pool, name="aggregation"):
    _require_gpu(gpu_enable)
    check_deferred()
    assert not args["is partial"]
    transfer_set = args["input ids"]
    agg_mask_map = {}
    if "mask map" in args:                              # aggregate.py:249-257
        for k, v in args["mask map"].items():
            if k in transfer_set:
                agg_mask_map[k] = v
                if v not in transfer_set:
                    transfer_set.append(v)
    mask_ids = set(agg_mask_map.values())
    data_ids = [c for c in transfer_set if c not in mask_ids]
    tg = tensor_group                                   # the columns read (outputs go to tensor_group)
    if len(mask_ids) > 1 or (mask_ids and any(c not in agg_mask_map for c in data_ids)):
        # columns under different masks, or masked beside already compacted ones: each masked
        # column is compacted by its own mask first, as the reference's pipeline does for every
        # input (vortex_pipeline.py:54-58), and the aggregate runs on the compacted columns
        tg = dict(tensor_group)
        tg.update(materialize(tensor_group, data_ids, agg_mask_map))
        lengths = {tg[c].tensor.shape[0] for c in data_ids}
        if len(lengths) > 1:
            raise RuntimeError(f"aggregate inputs have different lengths after their masks: {sorted(lengths)}")
        mask_ids, agg_mask_map = set(), {}
    mask = tg[next(iter(mask_ids))].tensor if mask_ids else None

    key_ids, key_ids_new, key_types_name = [], [], []
    for tree in args["results"]:                        # aggregate.py:265-275
        t = tree
        while isinstance(t, list) and len(t) == 1:
            t = t[0]
        if isinstance(t, str) or (len(t) == 3 and t[1] == "AS" and isinstance(t[0], str)):
            kid = int((t if isinstance(t, str) else t[0]).split("#")[-1].replace("L", ""))
            key_ids.append(kid)
            key_types_name.append(tg[kid].tensor_type)
    agg_ids = args["out agg ids"]

    cols = {c: tg[c].tensor for c in data_ids}
    key_set = {int(k.split("#")[-1].replace("L", "")) for k in (args.get("keys") or [])}
    wait_ready(*[tg[c] for c in transfer_set if c in key_set or c in mask_ids])   # the plan's inputs

    def values_ready():
        wait_ready(*[tg[c] for c in transfer_set if c not in key_set and c not in mask_ids])

    def _pending(v):
        ev = getattr(v, "ready", None)
        return ev is not None and not ev.query()
    # value columns still in flight (a host copy or a late gather): count the groups from the keys
    values_late = any(_pending(tg[c]) for c in transfer_set if c not in key_set and c not in mask_ids)
    proto = tg[data_ids[0]] if data_ids else None
    n = next(iter(cols.values())).shape[0] if cols else 0
    device = next(iter(cols.values())).device if cols else torch.device("cuda")
    if all(tg[c].tensor.numel() == 0 for c in transfer_set):
        # vortex_pipeline.py:51-52: empty inputs give empty (float32) outputs
        keys_out = {k: torch.tensor([], device=device) for k in range(len(key_ids))}
        vals_out = {a: torch.tensor([], device=device) for a in agg_ids}
        prog = None
    elif needs_key_codes(args, cols):
        # string / float / many keys: number the key tuples first, group by the code
        kids = [int(k.split("#")[-1].replace("L", "")) for k in args["keys"]]
        codes, reps, G0 = encode_keys([cols[k] for k in kids], mask)
        prog = compile_aggregate(args, cols, derived=True, key_codes=codes)
        _, vals_out, G, _ = groupby(prog, n, device, mask=mask, before_values=values_ready)
        assert G == G0, (G, G0)
        keys_out = {}
        for i, (oid, kid) in enumerate(prog.key_outputs):
            k = gather([cols[kid]], reps)[0]
            keys_out[i] = k if k.dim() == 2 else k.reshape(G, 1)     # unique_key_cols[:, pos_l:pos_r]
    else:
        prog = compile_aggregate(args, cols, derived=True)
        ranges = [getattr(tg[kid], "_key_range", None) for kid in prog.key_ids]
        keys, vals_out, G, _ = groupby(prog, n, device, mask=mask, before_values=values_ready,
                                       key_ranges=ranges if ranges and all(r is not None for r in ranges) else None,
                                       values_late=values_late)
        keys_out = {}
        for i, (oid, kid) in enumerate(prog.key_outputs):
            keys_out[i] = keys[prog.key_ids.index(kid)].reshape(G, 1)
    key_out_ids = [oid for (oid, _) in prog.key_outputs] if prog else \
        [int((t if isinstance(t, str) else t[-1]).split("#")[-1].replace("L", "")) for t in _key_trees(args)]
    for a in agg_ids:                                   # aggregate.py:383-390
        v = vals_out[a]
        tensor_group[a] = make_like(proto, v, torch_to_type(v.dtype))
    for i, oid in enumerate(key_out_ids):
        tensor_group[oid] = make_like(proto, keys_out[i], key_types_name[i])
    if prog is not None and not prog.encoded:
        # the groups come out in ascending key-tuple order (mixed-radix slots, or the packed key
        # for sparse spaces): tqp_sort on a prefix of these keys, ascending, keeps this order
        by = []
        for kid in prog.key_ids:
            oid = next((o for (o, k) in prog.key_outputs if k == kid), None)
            if oid is None:
                break
            by.append(oid)
        if by:
            out_ids = list(agg_ids) + list(key_out_ids)
            # the tag holds each column's storage, so a column whose tensor was replaced no longer matches
            order = (object(), tuple(by), {oid: tensor_group[oid].tensor.data_ptr() for oid in out_ids})
            for oid in out_ids:
                tensor_group[oid]._row_order = order
    return list(tensor_group.values())[0].tensor.size(0)


def _key_trees(args):
    out = []
    for tree in args["results"]:
        t = tree
        while isinstance(t, list) and len(t) == 1:
            t = t[0]
        if isinstance(t, str) or (len(t) == 3 and t[1] == "AS" and isinstance(t[0], str)):
            out.append(t)
    return out
