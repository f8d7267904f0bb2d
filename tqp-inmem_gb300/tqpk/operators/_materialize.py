"""Compaction of columns that still carry a filter mask (late materialisation).

The reference's pipeline compacts every masked input column by its own mask before an operator
runs (IO/vortex_pipeline.py:54-58: ``tensor[input_tensors[mask]]``).  The drop-in operators
normally read the mask in place instead; when one operator's inputs carry different masks, or
masked columns sit beside columns that are already compacted, they compact the masked ones
first with this helper (one stable compaction per mask, tqpk_compact) and run unmasked.
"""
from __future__ import annotations

from typing import Dict, Iterable

from ..ops import compact, gather_rows
from ..variable import make_like, wait_ready


def materialize(tensor_group, col_ids: Iterable[int], mask_map: Dict[int, int]):
    """{column: Variable} for each column of col_ids that has a mask in mask_map: its rows where
    the mask is set, in row order (tensor[mask]).  Columns under the same mask are compacted in
    one launch."""
    by_mask: Dict[int, list] = {}
    for c in col_ids:
        if c in mask_map:
            by_mask.setdefault(mask_map[c], []).append(c)
    out = {}
    for mid, cols in by_mask.items():
        m = tensor_group[mid]
        wait_ready(m, *[tensor_group[c] for c in cols])
        flat = [c for c in cols if tensor_group[c].tensor.dim() == 1 or tensor_group[c].tensor.shape[-1] == 1]
        rows2d = [c for c in cols if c not in flat]
        mask = m.tensor.reshape(-1)
        res, _ = compact([tensor_group[c].tensor.reshape(-1) for c in flat], mask=mask, with_row_ids=bool(rows2d))
        for c, t in zip(flat, res):
            src = tensor_group[c].tensor
            out[c] = make_like(tensor_group[c], t.reshape(-1, 1) if src.dim() == 2 else t, tensor_group[c].tensor_type)
        for c in rows2d:                                   # [N, w] string rows, by the kept row ids
            out[c] = make_like(tensor_group[c], gather_rows(tensor_group[c].tensor, res[-1]), tensor_group[c].tensor_type)
    return out
