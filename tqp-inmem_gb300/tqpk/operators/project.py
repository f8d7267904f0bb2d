"""Drop-in ``tqp_project`` (operators/project.py:10-69).

Renames columns (``args['rename map']``) and evaluates the computed expressions of
``args['used expr']`` in one generated kernel over the ``materialized in`` columns; the
results land at ``args['materialized out']`` with the dtype torch gives each expression
(integer results pass through float64, as the reference stores them).  A
``substring(col, l, w)`` result is the int8 [N, w] slice of the string rows, as the
reference's evaluate returns it (aggregate.py:114-119).
"""
from __future__ import annotations

import torch

from ..expr import compile_projection, is_trivial_projection
from ..predicate import get_id
from ..ops import check_deferred, project
from ..variable import make_like, torch_to_type, wait_ready
from .filter import _require_gpu


def _substring_of(tree):
    """(column id, start, width) of a `substring(col, l, w)` result (aggregate.py:114-119), else None."""
    while isinstance(tree, list) and len(tree) == 1:
        tree = tree[0]
    if isinstance(tree, list) and len(tree) == 3 and tree[1] == "AS":
        tree = tree[0]
    while isinstance(tree, list) and len(tree) == 1:
        tree = tree[0]
    if isinstance(tree, list) and len(tree) == 2 and tree[0] == "substring":
        sub, l, w = tree[1]
        return get_id(sub), int(l) - 1, int(w)
    return None


def _is_size_limit(e: NotImplementedError) -> bool:
    return "exceed" in str(e) or "more than" in str(e)


def projection_programs(trees, columns):
    """The computed expressions as projection programs: one while they fit the program's limits
    (32 instructions, 16 columns), else consecutive runs of expressions, each one program and one
    launch.  An expression too large for a program of its own still raises."""
    try:
        return [compile_projection(trees, columns, derived=True)]
    except NotImplementedError as e:
        if len(trees) == 1 or not _is_size_limit(e):
            raise
    progs, run, last = [], [], None
    for t in trees:
        try:
            last_try = compile_projection(run + [t], columns, derived=True)
        except NotImplementedError as e:
            if not run or not _is_size_limit(e):
                raise
            progs.append(last)
            run, last_try = [], compile_projection([t], columns, derived=True)
        run.append(t)
        last = last_try
    progs.append(last)
    return progs


def tqp_project(gpu_enable, tensor_group, args, cpu_mem_pool, gpu_mem_pool, name="project"):
    _require_gpu(gpu_enable)
    check_deferred()
    for orig, new in args["rename map"].items():
        tensor_group[new] = tensor_group[orig]
    if len(args["used expr"]) > 0:
        assert "mask map" not in args
        inputs = {k: tensor_group[k] for k in args["materialized in"]}
        first = next(iter(inputs.values()))
        rows = first.tensor.size(0)
        computed = [t for t in args["used expr"] if not is_trivial_projection(t)]
        subs = [_substring_of(t) for t in computed]
        numeric = [t for t, sub in zip(computed, subs) if sub is None]
        wait_ready(*inputs.values())
        nums = iter([])
        if numeric:
            results = []
            for prog in projection_programs(numeric, {k: v.tensor for k, v in inputs.items()}):
                results += project(prog, rows, first.tensor.device)
            nums = iter(results)
        outs = []
        for sub in subs:
            if sub is None:
                outs.append(next(nums))
                continue
            cid, l, w = sub          # the byte columns [l, l + w) of each string row, stored densely
            col = inputs[cid].tensor
            if col.dim() != 2 or col.dtype not in (torch.int8, torch.uint8):
                raise NotImplementedError(f"substring of a {tuple(col.shape)} {col.dtype} column")
            outs.append(col[:, l:l + w].contiguous())
        for i, out_id in enumerate(args["materialized out"]):
            tensor_group[out_id] = make_like(first, outs[i], torch_to_type(outs[i].dtype))
    return -1
