"""torch dtype <-> libtqpk dtype codes (constants.py:3-6 plus uint8/bool)."""
from __future__ import annotations

import torch

from . import _lib as L

_TO_CODE = {torch.int8: L.I8, torch.uint8: L.U8, torch.int32: L.I32, torch.int64: L.I64,
            torch.float64: L.F64, torch.bool: L.BOOL}
_FROM_CODE = {v: k for k, v in _TO_CODE.items()}


def code_of(dtype: torch.dtype) -> int:
    try:
        return _TO_CODE[dtype]
    except KeyError:
        raise TypeError(f"dtype {dtype} is not handled by the tqpk kernels") from None


def dtype_of(code: int) -> torch.dtype:
    return _FROM_CODE[code]


def is_int(dtype: torch.dtype) -> bool:
    return dtype in (torch.int8, torch.uint8, torch.int32, torch.int64, torch.bool)
