"""tqpk: GB300 (sm_103a) kernels for TQP-Inmem's relational operator hot path.

Layout:
  _lib.py       ctypes binding of libtqpk.so (include/tqpk.h)
  build.py      in-tree nvcc build of libtqpk.so
  predicate.py  filter tree -> device predicate program
  expr.py       aggregate result trees -> device expression/accumulator program
  ops.py        tensor-level wrappers of the C ABI
  operators/    drop-in tqp_filter / join_vortex / tqp_hash_aggregate / tqp_sort
  pipeline.py   fused filter -> join -> aggregate -> top-k pipelines
"""
from . import _lib  # noqa: F401

__all__ = ["_lib"]
