"""ctypes binding of libtqpk.so (declarations in include/tqpk.h).

The structures below mirror the C structs field for field; ``load()`` checks
their sizes against ``tqpk_abi_sizes`` exported by the library, so a layout
drift fails loudly at import instead of corrupting kernel arguments.
Status codes are mapped onto Python exceptions (the reference raises
ValueError / MemoryError / RuntimeError from the same places).
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libtqpk.so"

OK, EINVAL, ENOMEM, ETIMEOUT, EDTYPE, ECUDA, ECAPACITY, EUNSUPPORTED = 0, -1, -2, -3, -4, -5, -6, -7
ROWID, I8, U8, I32, I64, F64, BOOL = 0, 1, 2, 3, 4, 5, 6
MAX_COLS, MAX_PRED, MAX_KEYS, MAX_EXPR, MAX_ACCS = 16, 32, 4, 32, 16
NULL_INDEX = -64

P_CMP, P_AND, P_OR, P_NOT, P_TRUE, P_FALSE, P_MASK, P_CMPCOL = 1, 2, 3, 4, 5, 6, 7, 8
P_STRCMP, P_PREFIX, P_CONTAINS, P_LIKE2 = 9, 10, 11, 12
LT, LE, GT, GE, EQ, NE, ISCLOSE = 0, 1, 2, 3, 4, 5, 6
DOM_I64, DOM_F64, DOM_F32 = 0, 1, 2
X_COL, X_CONST, X_ADD, X_SUB, X_MUL, X_DIV, X_TOF64, X_SELECT, X_YEAR = 1, 2, 3, 4, 5, 6, 7, 8, 9
X_TOF32, X_F32TOF64 = 10, 11
F32 = 7                      # expression register type only: float32 in the low 32 bits
ACC_SUM, ACC_COUNT_NOTNULL, ACC_COUNT_ROWS, ACC_MIN, ACC_MAX = 1, 2, 3, 4, 5
GB_GLOBAL_ONE, GB_DENSE_PRIVATE, GB_DENSE_SHARED, GB_DENSE_GLOBAL, GB_HASH = 0, 1, 2, 3, 4
OUT_ACC, OUT_AVG = 0, 1
JOIN_DIRECT, JOIN_SORTED = 1, 2
JT_INNER, JT_SEMI, JT_ANTI, JT_OUTER = 0, 1, 2, 3


class PredInsn(C.Structure):
    _fields_ = [("op", C.c_int32), ("col", C.c_int32), ("cmp", C.c_int32), ("domain", C.c_int32),
                ("lit_i", C.c_int64), ("lit_f", C.c_double), ("lit_aux", C.c_double)]


MAX_STRPOOL = 512


class Predicate(C.Structure):
    _fields_ = [("n_insn", C.c_int32), ("n_cols", C.c_int32), ("cols", C.c_void_p * MAX_COLS),
                ("dtypes", C.c_int32 * MAX_COLS), ("insn", PredInsn * MAX_PRED),
                ("widths", C.c_int32 * MAX_COLS), ("strpool", C.c_uint8 * MAX_STRPOOL),
                ("strides", C.c_int32 * MAX_COLS)]


class ExprInsn(C.Structure):
    _fields_ = [("op", C.c_int32), ("type", C.c_int32), ("a", C.c_int32), ("b", C.c_int32),
                ("col", C.c_int32), ("wrap", C.c_int32), ("ci", C.c_int64), ("cf", C.c_double)]


class Acc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("type", C.c_int32), ("reg", C.c_int32), ("pad", C.c_int32),
                ("init_i", C.c_int64), ("init_f", C.c_double)]


class GroupbySpec(C.Structure):
    _fields_ = [("n_keys", C.c_int32), ("keys", C.c_void_p * MAX_KEYS), ("key_dtypes", C.c_int32 * MAX_KEYS),
                ("n_cols", C.c_int32), ("cols", C.c_void_p * MAX_COLS), ("col_dtypes", C.c_int32 * MAX_COLS),
                ("n_expr", C.c_int32), ("expr", ExprInsn * MAX_EXPR), ("n_accs", C.c_int32),
                ("accs", Acc * MAX_ACCS)]


class GbPlan(C.Structure):
    _fields_ = [("mode", C.c_int32), ("threads", C.c_int32), ("n_rows", C.c_int64), ("slots", C.c_int64),
                ("key_min", C.c_int64 * MAX_KEYS), ("key_range", C.c_int64 * MAX_KEYS),
                ("key_stride", C.c_int64 * MAX_KEYS), ("ws_bytes", C.c_size_t)]


class JoinPlan(C.Structure):
    _fields_ = [("mode", C.c_int32), ("unique", C.c_int32), ("nb_rows", C.c_int64), ("key_min", C.c_int64),
                ("key_max", C.c_int64), ("slots", C.c_int64), ("n_unique", C.c_int64), ("ws_bytes", C.c_size_t)]


_VP, _I64, _I32, _SZ = C.c_void_p, C.c_int64, C.c_int32, C.c_size_t
_P = C.POINTER

# name -> (restype, argtypes); the order and meaning follow include/tqpk.h
SIGNATURES = {
    "tqpk_version": (C.c_int, []),
    "tqpk_status_string": (C.c_char_p, [C.c_int]),
    "tqpk_launch_count": (_I64, []),
    "tqpk_abi_sizes": (C.c_int, [_P(_I64), C.c_int]),
    "tqpk_filter_mask": (C.c_int, [_P(Predicate), _I64, _VP, _VP, _VP]),
    "tqpk_compact_workspace_bytes": (_SZ, [_I64]),
    "tqpk_compact": (C.c_int, [_P(Predicate), _VP, _I64, _I32, _P(_VP), _P(_I32), _P(_VP), _VP, _VP, _SZ, _VP]),
    "tqpk_groupby_plan": (C.c_int, [_P(GroupbySpec), _P(Predicate), _VP, _I64, _P(GbPlan), _VP, _VP]),
    "tqpk_groupby_run": (C.c_int, [_P(GroupbySpec), _P(GbPlan), _P(Predicate), _VP, _I64, _VP, _SZ, _P(_I64), _VP]),
    "tqpk_groupby_emit": (C.c_int, [_P(GroupbySpec), _P(GbPlan), _VP, _I64, _P(_VP), _I32, _P(_I32), _P(_VP), _VP]),
    "tqpk_sort_workspace_bytes": (_SZ, [_I64]),
    "tqpk_argsort_stable": (C.c_int, [_VP, _I32, _I32, _VP, _I64, _VP, _VP, _SZ, _VP]),
    "tqpk_topk_workspace_bytes": (_SZ, [_I64, _I64]),
    "tqpk_topk_stable": (C.c_int, [_VP, _I32, _I32, _VP, _I64, _I64, _VP, _VP, _SZ, _VP]),
    "tqpk_join_plan_build": (C.c_int, [_VP, _I32, _VP, _I64, _P(JoinPlan), _VP, _VP]),
    "tqpk_join_build": (C.c_int, [_P(JoinPlan), _VP, _I32, _VP, _I64, _VP, _SZ, _VP]),
    "tqpk_join_probe_workspace_bytes": (_SZ, [_I64]),
    "tqpk_join_probe": (C.c_int, [_P(JoinPlan), _VP, _VP, _I32, _VP, _I64, _I32, _VP, _VP, _I64, _P(_I64), _VP,
                                  _SZ, _VP]),
    "tqpk_gather": (C.c_int, [_I32, _P(_VP), _P(_I32), _VP, _I64, _I32, _P(_VP), _VP]),
    "tqpk_mark_rows": (C.c_int, [_VP, _I64, _VP, _I64, _VP]),
    "tqpk_key_encode_workspace_bytes": (_SZ, [_I64]),
    "tqpk_key_encode": (C.c_int, [_I32, _P(_VP), _P(_I32), _P(_I32), _VP, _I64, _VP, _VP, _P(_I64), _VP, _SZ, _VP]),
    "tqpk_gather_rows": (C.c_int, [_VP, _I64, _I64, _VP, _I64, _VP, _VP]),
    "tqpk_string_words": (C.c_int, [_VP, _I64, _I32, _I32, _I32, _VP, _VP]),
    "tqpk_directory_compose": (C.c_int, [_VP, _I64, _VP, _I64, _I64, _I32, _I32, _VP]),
    "tqpk_directory_bits": (C.c_int, [_VP, _I64, _VP, _VP]),
    "tqpk_batch_record_bytes": (_SZ, []),
    "tqpk_batch_join_workspace_bytes": (_SZ, [_I64, _I64]),
    "tqpk_batch_describe_join": (C.c_int, [_VP, _VP, _I32, _I64, _P(Predicate), _I64, _I64, _VP, _I32, _I64,
                                           _P(Predicate), _P(GroupbySpec), _I32, _I32, _I32, _VP, _SZ, _VP, _VP,
                                           _VP, _VP, _I64, _I64]),
    "tqpk_batch_groupby_workspace_bytes": (_SZ, [_P(GroupbySpec), _P(_I64), _P(_I64), _I64]),
    "tqpk_batch_describe_groupby": (C.c_int, [_VP, _P(GroupbySpec), _P(Predicate), _I64, _P(_I64), _P(_I64), _VP,
                                              _SZ, _P(_VP), _I32, _P(_I32), _P(_VP), _VP, _I64, _I64, _I32]),
    "tqpk_batch_items": (_I64, [_VP, _I32, _VP, _I64]),
    "tqpk_batch_ctl_bytes": (_SZ, [_I32]),
    "tqpk_batch_reset": (C.c_int, [_VP, _VP, _I32, _VP, _VP]),
    "tqpk_batch_run": (C.c_int, [_VP, _I32, _VP, _I32, _VP, _I32, _VP]),
    "tqpk_batch_error": (C.c_int, [_VP, _P(C.c_int), _VP]),
    "tqpk_batch_grid": (_I32, []),
    "tqpk_batch_set_trace": (C.c_int, [_VP]),
    "tqpk_jit_available": (C.c_int, []),
    "tqpk_jit_check": (C.c_int, [C.c_char_p, C.c_char_p, _SZ]),
    "tqpk_jit_compile": (C.c_int, [C.c_char_p, C.c_char_p, _P(_VP), C.c_char_p, _SZ]),
    "tqpk_jit_occupancy": (C.c_int, [_VP, _I32, _SZ]),
    "tqpk_jit_launch": (C.c_int, [_VP, _I32, _I32, _SZ, _P(_VP), _I32, _VP]),
    "tqpk_jit_prefer_shared": (C.c_int, [_VP, _I32]),
    "tqpk_num_sms": (_I32, []),
    "tqpk_groupby_prepare": (C.c_int, [_P(GroupbySpec), _P(GbPlan), _VP, _SZ, _VP]),
    "tqpk_groupby_plan_domains": (C.c_int, [_P(GroupbySpec), _P(_I64), _P(_I64), _I64, _P(GbPlan)]),
    "tqpk_groupby_count": (C.c_int, [_P(GroupbySpec), _P(GbPlan), _VP, _P(_I64), _VP]),
    "tqpk_groupby_table": (_VP, [_VP]),
    "tqpk_pipeline_join_agg_topk_stages": (C.c_int, [_I32, _VP, _I32, _I64, _P(Predicate), _I64, _I64, _VP, _I32, _I64,
                                                     _P(Predicate), _P(GroupbySpec), _I32, _I32, _I32, _VP, _SZ, _VP,
                                                     _VP, _VP, _VP, _VP]),
    "tqpk_pipeline_join_tables": (C.c_int, [_VP, _SZ, _I64, _I64, _P(_VP), _P(_VP), _P(_VP)]),
    "tqpk_pipeline_join_words": (C.c_int, [_VP, _SZ, _I64, _I64, _P(_VP), _P(_VP)]),
    "tqpk_directory_build": (C.c_int, [_VP, _I32, _I64, _P(Predicate), _VP, _I32, _I64, _I64, _I32, _I32, _VP, _VP,
                                       _VP]),
    "tqpk_directory_build_next": (C.c_int, [_VP, _I32, _I64, _P(Predicate), _VP, _I32, _I64, _I64, _I32, _I32,
                                            _VP, _I64, _I64, _VP, _VP, _VP]),
    "tqpk_dense_topk_workspace_bytes": (_SZ, [_I32]),
    "tqpk_dense_topk": (C.c_int, [_VP, _VP, _I64, _I64, _I32, _I32, _VP, _SZ, _VP, _VP, _VP, _VP, _VP, _VP]),
    "tqpk_groupby_emit_async": (C.c_int, [_P(GroupbySpec), _P(GbPlan), _VP, _P(_VP), _I32, _P(_I32), _P(_VP), _VP,
                                          _VP]),
    "tqpk_compact_noalloc_max_rows": (_I64, []),
    "tqpk_compact_noalloc": (C.c_int, [_P(Predicate), _VP, _I64, _I32, _P(_VP), _P(_I32), _P(_VP), _VP, _VP]),
    "tqpk_debug_compact_wait": (C.c_int, [_I32, _I64]),
    "tqpk_debug_topk_barrier": (C.c_int, [_I32, _I32]),
    "tqpk_key_range": (C.c_int, [_VP, _I32, _I64, _VP, _P(_I64), _P(_I64), _VP]),
    "tqpk_timing_begin": (C.c_int, [_I32]),
    "tqpk_timing_end": (C.c_int, [_P(C.c_double), _P(_I32)]),
    "tqpk_pipeline_join_agg_topk_workspace_bytes": (_SZ, [_I64, _I64]),
    "tqpk_pipeline_join_agg_topk": (C.c_int, [_VP, _I32, _I64, _P(Predicate), _I64, _I64, _VP, _I32, _I64,
                                              _P(Predicate), _P(GroupbySpec), _I32, _I32, _I32, _VP, _SZ, _VP, _VP,
                                              _VP, _VP, _VP]),
    "tqpk_pipeline_error": (C.c_int, [_VP, _P(C.c_int), _VP]),
    "tqpk_pipeline_star_workspace_bytes": (_SZ, [_I64, _I64, _I64]),
    "tqpk_pipeline_star_agg_topk": (C.c_int, [_VP, _I32, _VP, _I32, _I64, _P(Predicate), _P(GroupbySpec), _I32,
                                              _VP, _I32, _I64, _P(Predicate), _I64, _I64,
                                              _VP, _I32, _VP, _I32, _I64, _I64, _I64,
                                              _VP, _I32, _I64, _I64, _I64, _I32, _I32, _VP, _SZ,
                                              _VP, _VP, _VP, _VP, _VP, _VP]),
}

KID_FILTER_MASK, KID_GROUPBY, KID_JOIN_PROBE, KID_PIPE_PROBE, KID_PIPE_BUILD, KID_PIPE_TOPK = 1, 3, 5, 6, 7, 8
KID_STAR_PROBE, KID_BATCH = 9, 10

_STRUCTS = [PredInsn, Predicate, ExprInsn, Acc, GroupbySpec, GbPlan, JoinPlan]

_lock = threading.Lock()
_lib = None


class TqpkError(RuntimeError):
    pass


def _exc(status: int):
    return {EINVAL: ValueError, ENOMEM: MemoryError, ETIMEOUT: TimeoutError, EDTYPE: TypeError,
            ECUDA: RuntimeError, EUNSUPPORTED: NotImplementedError}.get(status, TqpkError)


def load(path: Path | str | None = None):
    """Loads libtqpk.so (raises if it was not built) and checks the ABI."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(f"{p} is missing: build it with tqpk.build.build() (nvcc, sm_103a)")
        lib = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        sizes = (_I64 * len(_STRUCTS))()
        n = lib.tqpk_abi_sizes(sizes, len(_STRUCTS))
        if n != len(_STRUCTS):
            raise RuntimeError("libtqpk ABI mismatch: struct count")
        for s, got in zip(_STRUCTS, sizes):
            if C.sizeof(s) != got:
                raise RuntimeError(f"libtqpk ABI mismatch: sizeof({s.__name__}) {C.sizeof(s)} != {got}")
        _lib = lib
        return lib


def check(status: int, what: str):
    if status != OK:
        lib = load()
        msg = lib.tqpk_status_string(status).decode()
        raise _exc(status)(f"{what}: {msg} (status {status})")


def ptr(t) -> int | None:
    """Device address of a tensor (None for an absent optional argument)."""
    return None if t is None else t.data_ptr()


def stream_handle(device=None) -> int:
    """cudaStream_t of the current torch stream of `device` (None: the current device).

    torch's raw-stream query skips building a Stream object, about 15 us of host time per
    call on the Grace host, and the operators ask once per library call."""
    import torch
    idx = device.index if isinstance(device, torch.device) else device
    if idx is None:
        idx = torch.cuda.current_device()
    raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    if raw is not None:
        return int(raw(int(idx)))
    return torch.cuda.current_stream(idx).cuda_stream
