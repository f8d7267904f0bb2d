"""Drop-in replacements for TQP-Inmem's hot-path operators.

Same names, arguments, return values, ``tensor_group`` mutations and errors
as the reference functions; the work runs in libtqpk.so:

  filter.tqp_filter             operators/filter.py:164-204
  hashjoin.join_vortex          operators/hashjoin.py:179-248
  hashjoin.join_kernel_new      operators/hashjoin.py:24-177
  aggregate.tqp_hash_aggregate  operators/aggregate.py:236-393
  sort.tqp_sort                 operators/sort.py:6-58
  project.tqp_project           operators/project.py:10-69
  ingress.tqp_scan              operators/scan.py:8-54 (device placement; optionally asynchronous)

and, for a plan executor that can hand a run of operators over at once, fused.try_fused (a
filtered join + aggregate + top-k as one fused pipeline; main.py:152-253).
"""
from .filter import tqp_filter
from .hashjoin import join_vortex, join_kernel_new
from .aggregate import tqp_hash_aggregate
from .sort import tqp_sort
from .project import tqp_project
from ..ingress import tqp_scan
from .fused import try_fused

__all__ = ["tqp_filter", "join_vortex", "join_kernel_new", "tqp_hash_aggregate", "tqp_sort", "tqp_project", "tqp_scan", "try_fused"]
