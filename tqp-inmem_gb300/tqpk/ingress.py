"""Column ingress: the reference's scan (operators/scan.py:8-54) and an asynchronous stager.

The reference reads each column from a TorchScript file, converts it to the
engine's dtypes (dates int32, decimals float64, text int8 [N, w], the rest
int64), copies it into its device pool (`mem_pool.malloc_like`,
IO/pinned_mem.py) and synchronises.  `tqp_scan` does the same with the same
arguments; with a `ColumnStager` it instead queues every host->device copy on
a side stream in the given column order and returns at once, each column's
Variable carrying the event after its copy (`ready`).  The operators of this
package wait for a column right before their first kernel that reads it
(tqpk.variable.wait_ready), so filters, join builds and probes, and the
aggregate's planning overlap the copies of the columns they do not read yet.
"""
from __future__ import annotations

import os
from typing import Dict, Iterable, Optional

import torch

from .variable import Variable, date_dtype, float_dtype, int_dtype, string_dtype

# operators/scan.py:10-17
TYPE_MAPPING = {
    "identifier": "int",
    "integer": "int",
    "decimal": "float",
    "date": "date",
    "variable text": "string",
    "fixed text": "string",
}


def convert_column(t: torch.Tensor, tensor_type: str) -> torch.Tensor:
    """scan.py:34-42: the dtype each column type is kept in."""
    if tensor_type == "date":
        return t.to(date_dtype)
    if torch.is_floating_point(t):
        return t.to(float_dtype)
    if tensor_type == "string":
        return t.to(string_dtype)
    assert t.dim() == 1
    return t.to(int_dtype)


class ColumnStager:
    """Host -> device copies of columns on one side stream, each followed by an event.

    `stage(host, types, order)` allocates the device columns (from `mem_pool` when it has
    `malloc_like`, else from torch's caching allocator), queues the copies in `order`
    (the order the plan reads the columns; the rest follow) and returns Variables whose
    `ready` event completes when their copy has.  Host tensors should be pinned for the
    copies to be asynchronous; unpinned ones are copied through a pinned staging buffer
    first."""

    def __init__(self, device=None):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.stream = torch.cuda.Stream(self.device)

    def stage(self, host: Dict[int, torch.Tensor], types: Dict[int, str], order: Optional[Iterable[int]] = None,
              mem_pool=None) -> Dict[int, Variable]:
        main = torch.cuda.current_stream(self.device)
        ids = list(order or []) + [c for c in host if c not in set(order or [])]
        pool = mem_pool if mem_pool is not None and hasattr(mem_pool, "malloc_like") else None
        # The side stream waits once for the work queued on `main` so far: memory the allocator
        # hands out below may have been used by it.  Each column is allocated (on `main`) right
        # before its copy is queued, so the first copy starts after one allocation, not all.
        self.stream.wait_stream(main)
        out = {}
        for c in ids:
            h = host[c]
            ptr = None
            if pool is not None:
                ptr, d = pool.malloc_like(torch.empty(h.shape, dtype=h.dtype, device=self.device))
            else:
                d = torch.empty(h.shape, dtype=h.dtype, device=self.device)
            if not h.is_pinned():
                h = h.pin_memory()
            ev = torch.cuda.Event()
            with torch.cuda.stream(self.stream):
                d.copy_(h, non_blocking=True)
                ev.record(self.stream)
            d.record_stream(self.stream)
            v = Variable(d, types[c], ready=ev)
            if ptr is not None:
                v.backing_mem_ptr = ptr
            out[c] = v
        return out


def load_column(path: str) -> torch.Tensor:
    """The column a TorchScript file holds as its first parameter (scan.py:25-26)."""
    return list(torch.jit.load(path, map_location="cpu").parameters())[0].detach()


def tqp_scan(gpu_enable, o_tensor_group, args, config_json, schema_table, SF, mem_pool, name="scan",
             stager: Optional[ColumnStager] = None):
    """operators/scan.py:8-54 with the same arguments and return value (the row count).

    Each column of `args['output names']` is read from
    `<config_json['tensors path']>/SF<SF>-tensor-<NAME>.pth`, typed through the schema
    (`schema_table[NAME]`, TYPE_MAPPING), marked sorted when it is the table's primary key,
    converted as the reference converts it and, with gpu_enable, placed on the device: in
    `mem_pool` when it has `malloc_like` (the reference's pool), else in torch's allocator.
    Without a stager the copies are synchronous, as in the reference; with one they are
    queued on its stream in column order and every Variable carries its copy's `ready`
    event, so the caller can start the plan while the later columns are still in flight."""
    tensor_path = config_json.get("tensors path")
    col_names, col_ids = args["output names"], args["output ids"]
    rows = 0
    host, types, sorted_ids = {}, {}, set()
    for col_name, col_id in zip(col_names, col_ids):
        col_name = col_name.upper()
        t = load_column(os.path.join(tensor_path, f"SF{SF}-tensor-{col_name}.pth"))
        tensor_type = TYPE_MAPPING[schema_table[col_name].split(",")[0]]
        if col_name == schema_table.get("PRIMARY_KEY"):
            sorted_ids.add(col_id)
        rows = t.shape[0]
        host[col_id] = convert_column(t, tensor_type)
        types[col_id] = tensor_type
    if not gpu_enable:
        for c in col_ids:
            o_tensor_group[c] = Variable(host[c], types[c], is_sorted=c in sorted_ids)
        return rows
    if stager is not None:
        staged = stager.stage(host, types, col_ids, mem_pool)
        for c in col_ids:
            staged[c].is_sorted = c in sorted_ids
            o_tensor_group[c] = staged[c]
        return rows
    dev = torch.device("cuda", torch.cuda.current_device())
    for c in col_ids:
        ptr = None
        if mem_pool is not None and hasattr(mem_pool, "malloc_like"):
            ptr, d = mem_pool.malloc_like(torch.empty(host[c].shape, dtype=host[c].dtype, device=dev))
            d.copy_(host[c])
        else:
            d = host[c].to(dev)
        o_tensor_group[c] = Variable(d, types[c], backing_mem_ptr=ptr, is_sorted=c in sorted_ids)
    torch.cuda.synchronize()
    return rows
