"""Drop-in ``tqp_filter`` (operators/filter.py:164-204).

Evaluates the whole filter tree in one kernel (tqpk_filter_mask) and stores
the bool mask under ``args['out mask id']`` for late materialisation, as the
reference does; the rows are compacted (or skipped) by the consumer.
"""
from __future__ import annotations

from ..ops import check_deferred, filter_mask
from ..predicate import compile_filter
from ..variable import make_like, wait_ready


def _require_gpu(gpu_enable):
    if not gpu_enable:
        raise NotImplementedError("tqpk operators run on the GPU only (gpu_enable=False)")


def tqp_filter(gpu_enable, tensor_group, args, subquery_result, cpu_mem_pool, gpu_mem_pool, name):
    _require_gpu(gpu_enable)
    check_deferred()
    assert "mask map" not in args, "Filter not accepting masks"
    input_columns = {k: tensor_group[k] for k in args["materialized in"]}
    if len(input_columns) == 0:
        return -1
    first = next(iter(input_columns.values()))
    rows = first.tensor.size(0)
    cols = {k: v.tensor for k, v in input_columns.items()}
    pred = compile_filter(args["filter tree"], cols, subquery_result)
    wait_ready(*input_columns.values())
    mask, _ = filter_mask(pred, rows, first.tensor.device)
    tensor_group[args["out mask id"]] = make_like(first, mask, "bool")
    return -1
