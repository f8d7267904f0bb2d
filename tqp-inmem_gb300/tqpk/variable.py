"""Column container with the same interface as TQP-Inmem's ``variable.py``.

The drop-in operators accept any object with ``.tensor`` and ``.tensor_type``
(normally the reference's own ``variable.Variable``) and build their outputs
with the class of the input they replace, so the plan executor keeps seeing
its own type.  This class is the stand-in for callers without the reference
tree (tests, the benchmark).  Reference: variable.py:9-61, constants.py:3-6.
"""
from __future__ import annotations

import torch

string_dtype = torch.int8
int_dtype = torch.int64
float_dtype = torch.float64
date_dtype = torch.int32


class Variable:
    """variable.py:9-43"""

    def __init__(self, tensor, tensor_type: str, backing_mem_ptr=None, var_state="cpu resident",
                 is_sorted: bool = False, ready=None):
        self.tensor = tensor
        self.tensor_type = tensor_type
        self.state = var_state
        self.backing_mem_ptr = backing_mem_ptr
        self.is_sorted = is_sorted
        self.ready = ready      # CUDA event after which the tensor's data is on the device (None: already)
        # inclusive (min, max) bound on the values, set by join_vortex only (an inner join's key
        # outputs all lie in the filtered build side's key range); a group-by over columns that
        # carry one plans its slot table from it without a key-range pass.  The group-by indexes
        # its table with this bound, so nothing else sets it.
        self._key_range = None

    def __repr__(self):
        return f"Variable (tensor size = {self.tensor.shape} ({self.tensor.dtype}), tensor type = '{self.tensor_type}')"

    def __iter__(self):
        yield self.tensor
        yield self.tensor_type

    def normalize(self):
        if self.tensor.dim() == 2:
            self.tensor = self.tensor.squeeze()
        if self.tensor.dim() == 0:
            self.tensor = self.tensor.unsqueeze(0)
        assert self.tensor.dim() == 1


def wait_ready(*variables) -> None:
    """Orders the current stream after the copies that fill these columns: a column still
    arriving from the host (a Variable with a `ready` event, e.g. one copied on a side
    stream) is waited for right before the first kernel that reads it, so the operators
    before it overlap the copy.  Columns without the attribute (the reference's Variable)
    are ready."""
    for v in variables:
        ev = getattr(v, "ready", None) if v is not None else None
        if ev is not None:
            torch.cuda.current_stream(v.tensor.device).wait_event(ev)


def host_values(v):
    """A column's rows as a numpy array: the copy its producer already brought to the host with
    its own result read (`host`, set by the fused pipelines), else one device-to-host copy."""
    h = getattr(v, "host", None)
    if h is not None and tuple(h.shape) == tuple(v.tensor.shape):
        return h
    return v.tensor.cpu().numpy()


def torch_to_type(dtype) -> str:
    """variable.py:45-52"""
    if dtype == float_dtype:
        return "float"
    if dtype == date_dtype:
        return "date"
    if dtype == int_dtype:
        return "int"
    return "string"


def make_like(proto, tensor, tensor_type: str):
    """A new column of the same class as `proto` (the caller's Variable type)."""
    cls = type(proto) if proto is not None and hasattr(proto, "tensor_type") else Variable
    return cls(tensor, tensor_type)
