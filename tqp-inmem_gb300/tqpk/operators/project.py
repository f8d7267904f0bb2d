"""Drop-in ``tqp_project`` (operators/project.py:10-69).

Renames columns (``args['rename map']``) and evaluates the computed expressions of
``args['used expr']`` in one generated kernel over the ``materialized in`` columns; the
results land at ``args['materialized out']`` with the dtype torch gives each expression
(integer results pass through float64, as the reference stores them).
"""
from __future__ import annotations

from ..expr import compile_projection, is_trivial_projection
from ..ops import project
from ..variable import make_like, torch_to_type, wait_ready
from .filter import _require_gpu


def tqp_project(gpu_enable, tensor_group, args, cpu_mem_pool, gpu_mem_pool, name="project"):
    _require_gpu(gpu_enable)
    for orig, new in args["rename map"].items():
        tensor_group[new] = tensor_group[orig]
    if len(args["used expr"]) > 0:
        assert "mask map" not in args
        inputs = {k: tensor_group[k] for k in args["materialized in"]}
        first = next(iter(inputs.values()))
        rows = first.tensor.size(0)
        prog = compile_projection(args["used expr"], {k: v.tensor for k, v in inputs.items()}, derived=True)
        wait_ready(*inputs.values())
        outs = project(prog, rows, first.tensor.device)
        for i, out_id in enumerate(args["materialized out"]):
            tensor_group[out_id] = make_like(first, outs[i], torch_to_type(outs[i].dtype))
    return -1
