"""Drop-in ``tqp_sort`` (operators/sort.py:6-58).

The reference runs one stable torch.sort per key, last key first, each time
gathering the key through ``perm`` (:26-35), then slices ``perm[:limit]``
(:41-42) and gathers every input column (:44-54).  Here each key is one
tqpk_argsort_stable call that sorts keys[perm] and permutes perm in the same
kernels; with a limit the first key uses the stable top-k, which returns the
same rows as the full sort followed by the slice.  A [N, w] key (the
reference ranks its rows with unique(dim=0)) is sorted as ceil(w/8) stable
passes over 8-byte words of the rows, last word first, which gives the same
lexicographic order and ties; [N, w] columns are gathered row by row.
When every input column comes from one tqp_hash_aggregate call, whose groups are
in ascending key-tuple order, and the sort keys are a prefix of those group keys,
all ascending, the stable sort is the identity: only the limit is applied.
"""
from __future__ import annotations

import torch

from ..ops import argsort_stable, check_deferred, gather, gather_rows, string_words, topk_stable
from ..variable import make_like, wait_ready
from .filter import _require_gpu


def tqp_sort(gpu_enable, tensor_group, args, with_limit, name="sort"):
    _require_gpu(gpu_enable)
    check_deferred()
    limit = args["limit"] if with_limit else None
    input_ids = args["input ids"]
    rows = tensor_group[input_ids[0]].tensor.shape[0]
    key_ids, key_descs = args["key ids"], args["key orders"]
    k0 = tensor_group[key_ids[0]].tensor
    if k0.numel() * k0.element_size() >= 8_000_000_000:   # sort.py:22-23, 38-39
        raise RuntimeError("sort input exceeds in-memory limit")
    device = k0.device
    order = getattr(tensor_group[input_ids[0]], "_row_order", None)
    if (order is not None and not any(key_descs) and tuple(key_ids) == order[1][:len(key_ids)]
            and all(getattr(tensor_group[c], "_row_order", None) is order
                    and order[2].get(c) == tensor_group[c].tensor.data_ptr() for c in {*input_ids, *key_ids})):
        # every input column holds one group-by's output, whose rows are already in ascending
        # order of these keys: the stable sort is the identity, only the limit is left
        if limit is not None:
            for c in input_ids:
                v = tensor_group[c]
                tensor_group[c] = make_like(v, v.tensor[:limit], v.tensor_type)
        return rows
    wait_ready(*[tensor_group[k] for k in key_ids])
    perm = None                                           # identity until the first pass
    steps = []
    for key_id, desc in zip(reversed(key_ids), reversed(key_descs)):
        col = tensor_group[key_id].tensor
        if col.dim() == 2 and col.shape[1] > 1:
            if col.dtype not in (torch.int8, torch.uint8):
                raise NotImplementedError(f"2-D sort key of dtype {col.dtype}")
            steps += [(string_words(col, wd), desc) for wd in reversed(range((col.shape[1] + 7) // 8))]
        else:
            steps.append((col.reshape(-1), desc))
    for i, (key, desc) in enumerate(steps):
        last = i == len(steps) - 1
        if last and limit is not None:
            perm = topk_stable(key, limit, desc, perm)
        else:
            perm = argsort_stable(key, desc, perm)
    if perm is None:                                      # no key columns
        perm = torch.arange(rows, device=device, dtype=torch.int64)
    if limit is not None:
        perm = perm[:limit]
    wait_ready(*[tensor_group[k] for k in input_ids])
    flat, shapes = [], []
    for key_id in input_ids:                              # sort.py:44-54
        t = tensor_group[key_id].tensor
        if not t.is_cuda:
            t = t.to(device)
        flat.append(t)
    # every 1-D (or [N, 1]) column in one multi-column gather launch; [N, w] rows by row gather
    one_d = [i for i, t in enumerate(flat) if t.dim() == 1 or (t.dim() == 2 and t.shape[1] == 1)]
    outs = [None] * len(flat)
    if one_d:
        for i, o in zip(one_d, gather([flat[i].reshape(-1) for i in one_d], perm)):
            outs[i] = o.reshape(-1, 1) if flat[i].dim() == 2 else o
    for i, t in enumerate(flat):
        if outs[i] is None:
            outs[i] = gather_rows(t, perm)
    for key_id, out in zip(input_ids, outs):
        tensor_group[key_id] = make_like(tensor_group[key_id], out, tensor_group[key_id].tensor_type)
    return rows
