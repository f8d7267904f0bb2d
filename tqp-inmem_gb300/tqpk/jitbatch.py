"""Batched query instances as one generated persistent kernel.

``QueryBatch`` takes the same instances as ``tqpk.batch.Batch``
(``GroupByInstance``: filter + dense group-by; ``JoinInstance``: filter both
sides + join on a unique build key + sum by build key + top-k) and runs all of
them in one persistent launch fed by a device work queue, replayable from a
CUDA graph.  Unlike the library's ``k_batch`` (which interprets each
instance's predicate, expression and accumulator programs from its record),
the kernel here is generated from the batch's distinct query programs: every
program becomes straight-line device functions (the code of the generated
single-query kernels, over a work item's row range), and instances that
share a program share its code, reading their columns, constants and tables
from their record.

Work items are (instance, phase, begin, end), ordered phase-major; a CTA takes
the next item with an atomic ticket and, for phase p > 0, waits (bounded) until
every phase p-1 item of the same instance has finished.  Phases:

* group-by: 0 accumulate rows [b, e) into the instance's table (per-thread or
  shared copies of a shared-memory table merged into the global one, or
  reductions straight into the global table, chosen by table size), 1 count
  the occupied slots of [b, e), 2 write the groups of [b, e) at their offset
  (key order);
* join: 0 build the key directory from build rows [b, e), 1 probe rows [b, e)
  (predicate, lookup, value, FP64 sum per build key), 2 per-item top-k of
  slots [b, e), 3 merge the per-item lists (one item).

The result layout and arithmetic are those of the single-query kernels, so
the outputs equal the operators' (sums within FP64 reordering).
"""
from __future__ import annotations

import ctypes as C
import math
import re
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib as L
from . import jit
from .batch import Autotuner, GroupByInstance, JoinInstance
from .dtypes import code_of, dtype_of
from .expr import compile_aggregate, require_f64_outputs
from .predicate import compile_filter

# dynamic shared memory of the persistent kernel (group tables, join sums) and its CTAs per SM:
# 64-instance batch 2.32 ms with 96 KB at 2 CTAs per SM, 2.06 ms with 48 KB at 3, 1.95 ms with 32 KB
# at 4 (more warps to cover the reductions' and loads' latency outweigh the smaller shared tables),
# 2.37 ms at 5 (registers spill)
SMEM = 32 * 1024
MIN_CTAS = 4
T = 256                   # threads per CTA
MAXK = 32                 # join top-k bound (one warp-list row per lane)

# record layout: (name, C type, ctypes type, count); the C struct text and the
# ctypes mirror are both generated from this list
_P = C.c_void_p
_FIELDS = [
    ("kind", "int", C.c_int32, 1), ("prog", "int", C.c_int32, 1), ("mode", "int", C.c_int32, 1),
    ("k", "int", C.c_int32, 1), ("desc", "int", C.c_int32, 1), ("flags", "int", C.c_int32, 1),
    ("copies", "int", C.c_int32, 1), ("pad", "int", C.c_int32, 1),
    ("fk_dt", "int", C.c_int32, 1), ("bk_dt", "int", C.c_int32, 1),
    ("n", "long long", C.c_int64, 1), ("nb", "long long", C.c_int64, 1), ("slots", "long long", C.c_int64, 1),
    ("range_slots", "long long", C.c_int64, 1), ("ni", "long long", C.c_int64, 4),
    ("kmin", "long long", C.c_int64, 4), ("kstride", "long long", C.c_int64, 4), ("krange", "long long", C.c_int64, 4),
    ("pc", "const void*", _P, 16), ("kc", "const void*", _P, 4), ("vc", "const void*", _P, 16),
    ("bc", "const void*", _P, 16),
    ("gacc", "unsigned long long*", _P, 1), ("range_count", "long long*", _P, 1),
    ("cand_key", "unsigned long long*", _P, 1), ("cand_idx", "long long*", _P, 1),
    ("out_key", "void*", _P, 4), ("out_col", "void*", _P, 16), ("out_groups", "long long*", _P, 1),
    ("dir", "int*", _P, 1), ("sum", "double*", _P, 1), ("occ", "unsigned*", _P, 1),
    ("out_keys", "long long*", _P, 1), ("out_vals", "double*", _P, 1), ("out_count", "long long*", _P, 1),
    ("lp", "PL", jit.PredLits, 1), ("lb", "PL", jit.PredLits, 1),
]


class QInst(C.Structure):
    _fields_ = [(n, ct * cnt if cnt > 1 else ct) for (n, _, ct, cnt) in _FIELDS]


def _struct_c() -> str:
    lines = ["struct QInst {"]
    for n, ctype, _, cnt in _FIELDS:
        lines.append(f"  {ctype} {n}{f'[{cnt}]' if cnt > 1 else ''};")
    lines.append("};")
    return "\n".join(lines)


KIND_GB, KIND_JOIN = 0, 1
F_PVEC, F_KVEC, F_VVEC, F_FVEC, F_BVEC = 1, 2, 4, 8, 16

_BATCH_PRELUDE = r"""
struct WorkItem { int inst, phase; long long begin, end; };
__device__ __forceinline__ unsigned long long ld_acq(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void set_err(int* err, int code) { atomicCAS(err, 0, code); }
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t; asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t)); return t;
}
__device__ __forceinline__ double from_ord(u64 u) { return u2d((u >> 63) ? (u & ~(1ull << 63)) : ~u); }
__device__ __forceinline__ u64 sum_key(double v, int desc) {   // integer instructions only
  u64 b = d2u(v);
  if ((b << 1) == 0) b = 0;                                         // -0.0 ranks as +0.0
  else if ((b & 0x7ff0000000000000ull) == 0x7ff0000000000000ull && (b & 0x000fffffffffffffull))
    b = 0x7ff8000000000000ull;                                      // every NaN as one
  const u64 u = (b >> 63) ? ~b : (b | (1ull << 63));
  return desc ? ~u : u;
}
__device__ __forceinline__ bool tk_better(u64 ka, i64 ia, u64 kb, i64 ib) { return ka < kb || (ka == kb && ia < ib); }
// a warp's best k (<= 32) entries, sorted, entry p on lane p
struct WL {
  u64 key; i64 idx;
  __device__ void init() { key = ~0ull; idx = -1; }
  __device__ void insert(int k, u64 ck, i64 ci) {
    const int lane = threadIdx.x & 31;
    const bool b = lane < k && idx >= 0 && tk_better(key, idx, ck, ci);
    const int pos = __popc(__ballot_sync(0xffffffffu, b));
    if (pos >= k) return;
    const u64 uk = __shfl_up_sync(0xffffffffu, key, 1);
    const i64 ui = __shfl_up_sync(0xffffffffu, idx, 1);
    if (lane > pos && lane < k) { key = uk; idx = ui; }
    if (lane == pos) { key = ck; idx = ci; }
  }
  __device__ void offer(int k, u64 ck, i64 ci, bool valid) {
    const u64 tk = __shfl_sync(0xffffffffu, key, k - 1);
    const i64 ti = __shfl_sync(0xffffffffu, idx, k - 1);
    unsigned pending = __ballot_sync(0xffffffffu, valid && (ti < 0 || tk_better(ck, ci, tk, ti)));
    while (pending) {
      const int src = __ffs(pending) - 1;
      pending &= pending - 1;
      insert(k, __shfl_sync(0xffffffffu, ck, src), __shfl_sync(0xffffffffu, ci, src));
    }
  }
};
"""


def _hoist(code: str, rec: str) -> Tuple[List[str], str]:
    """Moves literal reads lp.i[k] / lb.f[k] ... out of the row loop: returns
    (declarations reading them once from the record, code using the locals)."""
    decls, seen = [], set()

    def sub(m):
        nm = f"{m.group(1)}_{m.group(2)}{m.group(3)}"
        if nm not in seen:
            seen.add(nm)
            t = "long long" if m.group(2) == "i" else "double"
            decls.append(f"const {t} {nm} = {rec}.{m.group(1)}.{m.group(2)}[{m.group(3)}];")
        return nm
    return decls, re.sub(r"\b(lp|lb)\.([ifa])\[(\d+)\]", sub, code)


def _ptr_decls(cols: Sequence[int], dtypes, field: str, pfx: str) -> List[str]:
    out = []
    for c in cols:
        t = jit._CTYPE[dtypes[c]]
        out.append(f"const {t}* __restrict__ {pfx}{c} = (const {t}*)I.{field}[{c}];")
    return out


def _ld4(cols, dtypes, tile: str, ptr: str, n: str, vec: str) -> List[str]:
    return [f"const V4<{jit._CTYPE[dtypes[c]]}> {tile}{c} = ld4({ptr}{c}, r0, {n}, {vec});" for c in cols]


# ---------------------------------------------------------------------------- group-by program
def _gb_functions(p: int, spec, pred) -> str:
    S = spec
    A = S.n_accs
    pcols, pexpr = jit._pred_code(pred, "p") if pred is not None else ([], "true")
    lit_decls, pexpr = _hoist(pexpr, "I")
    ecols, elines = jit._expr_code(S, S.n_expr, "c", contract=True)   # sums only: x * (1 - y) as one FMA
    kcols = list(range(S.n_keys))
    src = [f"__device__ void gb_agg_{p}(const QInst& I, i64 b, i64 e, u64* sm, int* err) {{",
           f"  constexpr int A = {A};",
           "  const i64 K = I.slots, n = I.n;",
           "  const int mode = I.mode, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;",
           "  const bool vp = I.flags & 1, vk = I.flags & 2, vc = I.flags & 4;",
           "  u64* __restrict__ gacc = I.gacc;"]
    src += ["  " + d for d in lit_decls]
    if pred is not None:
        src += ["  " + d for d in _ptr_decls(pcols, pred.dtypes, "pc", "pp")]
    src += ["  " + d for d in _ptr_decls(kcols, S.key_dtypes, "kc", "kp")]
    src += ["  " + d for d in _ptr_decls(ecols, S.col_dtypes, "vc", "cp")]
    src += [f"  const i64 km{k} = I.kmin[{k}], ks{k} = I.kstride[{k}], kr{k} = I.krange[{k}];" for k in kcols]
    inits = " : ".join(f"(a == {i}) ? {jit._acc_init(S.accs[i])}" for i in range(A)) + " : 0ull"
    src += ["  // table copies in shared memory: one per thread (mode 1, plain updates), or `copies`",
            "  // (a power of two) shared by threads tid % copies with shared-memory atomics (mode 2);",
            "  // mode 4: reductions into the global table only",
            "  const i64 copies = mode == 1 ? " + str(T) + " : I.copies;",
            "  const i64 me = threadIdx.x & (copies - 1);",
            "  const int lgc = __ffsll(copies) - 1;            // copies is a power of two",
            "  if (mode != 4) {                                  // K * A * copies cells fit in 32 bits",
            f"    for (int i = threadIdx.x; i < (int)(K * A * copies); i += {T}) {{ const int a = (i >> lgc) % A; "
            f"sm[i] = {inits}; }}",
            "    __syncthreads();",
            "  }",
            f"  for (i64 r0 = b + 4 * (i64)threadIdx.x; r0 < e; r0 += 4 * {T}) {{"]
    if pred is not None:
        src += ["    " + l for l in _ld4(pcols, pred.dtypes, "P", "pp", "n", "vp")]
    src += ["    " + l for l in _ld4(kcols, S.key_dtypes, "Kc", "kp", "n", "vk")]
    src += ["    " + l for l in _ld4(ecols, S.col_dtypes, "Cv", "cp", "n", "vc")]
    src += ["#pragma unroll", "    for (int j = 0; j < 4; ++j) {", "      if (r0 + j >= e) break;",
            f"      if (!({jit._rename(pexpr, 'p', 'P')})) continue;"]
    slot = " + ".join(f"((i64)Kc{k}.v[j] - km{k}) * ks{k}" for k in kcols) or "0"
    # a key outside its declared domain would index past the table: the row is skipped and the
    # batch reports TQPK_EINVAL
    if kcols:
        src.append("      if (" + " || ".join(f"(u64)((i64)Kc{k}.v[j] - km{k}) >= (u64)kr{k}" for k in kcols)
                   + ") { set_err(err, -1); continue; }")
    src.append(f"      const i64 slot = {slot};")
    src += ["      " + jit._rename(l, "c", "Cv") for l in elines]
    for a in range(A):
        acc = S.accs[a]
        v = jit._acc_value(acc)
        src.append(f"      {{ const u64 x = {v};")
        src.append(f"        if (mode == 4) {{ {jit._merge_atomic(acc, f'&gacc[{a} * K + slot]', 'x', glob=True)} }}")
        src.append(f"        else if (mode == 1) {{ u64* c = &sm[(slot * A + {a}) * copies + me]; "
                   f"*c = {jit._combine(acc, '*c', 'x')}; }}")
        src.append(f"        else {{ {jit._merge_atomic(acc, f'&sm[(slot * A + {a}) * copies + me]', 'x')} }} }}")
    src += ["    }", "  }", "  if (mode == 4) return;", "  __syncthreads();",
            "  // fold the copies of each cell and merge it into the global table: mode 1 (256 copies of",
            "  // at most 48 cells) one warp per cell, lanes over the copies; mode 2 one thread per cell,",
            "  // its copies in turn (a warp-wide shuffle reduction would spend 5 x 32 FP64 combines on",
            "  // every cell however few copies it has, and FP64 issues at 1/64 rate)",
            "  if (mode == 1) {",
            "  for (int c = wid; c < (int)(K * A); c += " + str(T // 32) + ") {",
            "    const int a = c % A; const int s = c / A;",
            "    switch (a) {"]
    for a in range(A):
        acc = S.accs[a]
        init = jit._acc_init(acc)
        src += [f"    case {a}: {{",
                f"      u64 v = {init};",
                f"      for (int t = lane; t < {T}; t += 32) v = {jit._combine(acc, 'v', f'sm[c * {T} + t]')};",
                "      for (int o = 16; o; o >>= 1) { const u64 w = __shfl_xor_sync(0xffffffffu, v, o); "
                f"v = {jit._combine(acc, 'v', 'w')}; }}",
                f"      if (lane == 0 && v != {init}) {{ {jit._merge_atomic(acc, f'&gacc[{a} * K + s]', 'v', glob=True)} }}",
                "      break; }"]
    src += ["    }", "  }", "  } else {",
            f"  for (int c = threadIdx.x; c < (int)(K * A); c += {T}) {{",
            "    const int a = c % A; const int s = c / A;",
            "    switch (a) {"]
    for a in range(A):
        acc = S.accs[a]
        init = jit._acc_init(acc)
        src += [f"    case {a}: {{",
                f"      u64 v = {init};",
                f"      for (int t = 0; t < (int)copies; ++t) v = {jit._combine(acc, 'v', '(sm[(c << lgc) + t])')};",
                f"      if (v != {init}) {{ {jit._merge_atomic(acc, f'&gacc[{a} * K + s]', 'v', glob=True)} }}",
                "      break; }"]
    src += ["    }", "  }", "  }", "  __syncthreads();", "}"]
    # emit: the groups of slots [b, e) at their output offset
    src += [f"__device__ void gb_emit_{p}(const QInst& I, i64 item, i64 b, i64 e, int* sw) {{",
            "  __shared__ i64 s_base;",
            "  if (threadIdx.x < 32) {            // groups of the items before this one: warp 0's lanes in turn",
            "    i64 base = 0;",
            "    for (i64 r = threadIdx.x; r < item; r += 32) base += __ldcg(&I.range_count[r]);",
            "    for (int o = 16; o; o >>= 1) base += __shfl_xor_sync(0xffffffffu, base, o);",
            "    if (threadIdx.x == 0) {",
            "      s_base = base;",
            "      if (item == I.ni[2] - 1 && I.out_groups) *I.out_groups = base + __ldcg(&I.range_count[item]);",
            "    }",
            "  }",
            "  __syncthreads();",
            "  const i64 K = I.slots;",
            "  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;",
            f"  for (i64 t0 = b; t0 < e; t0 += {T}) {{",
            "    const i64 s = t0 + threadIdx.x;",
            "    const bool occ = s < e && __ldcg(&I.gacc[s]) != 0;",
            "    const unsigned bal = __ballot_sync(0xffffffffu, occ);",
            "    if (lane == 0) sw[wid] = __popc(bal);",
            "    __syncthreads();",
            "    int before = 0, total = 0;",
            f"    for (int w = 0; w < {T // 32}; ++w) {{ if (w < wid) before += sw[w]; total += sw[w]; }}",
            "    if (occ) {",
            "      const i64 pos = s_base + before + __popc(bal & ((1u << lane) - 1));"]
    for k in kcols:
        t = jit._CTYPE[S.key_dtypes[k]]
        src.append(f"      (({t}*)I.out_key[{k}])[pos] = ({t})(I.kmin[{k}] + (s / I.kstride[{k}]) % I.krange[{k}]);")
    return "\n".join(src), (p, S)


def _gb_emit_outputs(p: int, spec, outputs) -> str:
    """The output stores of gb_emit_{p} (depends on the output list too)."""
    S = spec
    lines = []
    for o, (_, op, a, b, dt) in enumerate(outputs):
        acc = S.accs[a]
        ct = jit._CTYPE[code_of(dt)]
        isf = acc.type == L.F64 and acc.kind not in (L.ACC_COUNT_ROWS, L.ACC_COUNT_NOTNULL)
        v = f"__ldcg(&I.gacc[{a} * K + s])"
        if isf and acc.kind in (L.ACC_MIN, L.ACC_MAX):
            val, isf_now = f"from_ord({v})", True
        elif isf:
            val, isf_now = f"u2d({v})", True
        else:
            val, isf_now = f"(long long){v}", False
        if op == L.OUT_AVG:
            den = f"(double)(long long)__ldcg(&I.gacc[{b} * K + s])"
            num = val if isf_now else f"(double){val}"
            val, isf_now = f"__ddiv_rn({num}, {den})", True
        lines.append(f"      (({ct}*)I.out_col[{o}])[pos] = ({ct})({val});")
    lines += ["    }", "    __syncthreads();", "    if (threadIdx.x == 0) s_base += total;", "    __syncthreads();",
              "  }", "}"]
    return "\n".join(lines)


# ---------------------------------------------------------------------------- join program
def _join_functions(p: int, spec, val_reg: int, ppred, bpred) -> str:
    S = spec
    # build: directory of the build rows passing the build predicate
    bcols, bexpr = jit._pred_code(bpred, "p", "lb") if bpred is not None else ([], "true")
    blit, bexpr = _hoist(bexpr, "I")
    src = [f"__device__ void jn_build_{p}(const QInst& I, i64 b, i64 e, int* err) {{",
           "  const i64 n = I.nb, kmin = I.kmin[0], slots = I.slots;",
           "  const bool vb = I.flags & 16;"]
    src += ["  " + d for d in blit]
    if bpred is not None:
        src += ["  " + d for d in _ptr_decls(bcols, bpred.dtypes, "bc", "pp")]
    src += [f"  for (i64 r0 = b + 4 * (i64)threadIdx.x; r0 < e; r0 += 4 * {T}) {{"]
    if bpred is not None:
        src += ["    " + l for l in _ld4(bcols, bpred.dtypes, "P", "pp", "n", "vb")]
    src += ["    const V4<i64> BK = (I.bk_dt == 4) ? ld4((const long long*)I.kc[1], r0, n, false) : "
            "[&]{ V4<int> t = ld4((const int*)I.kc[1], r0, n, false); V4<i64> o; "
            "for (int q = 0; q < 4; ++q) o.v[q] = t.v[q]; return o; }();",
            "    int old[4];       // the four claims in flight together, their results read afterwards",
            "#pragma unroll", "    for (int j = 0; j < 4; ++j) {",
            f"      const bool in = r0 + j < e && ({jit._rename(bexpr, 'p', 'P')});",
            "      const i64 slot = BK.v[j] - kmin;",
            "      const bool put = in && slot >= 0 && slot < slots;",
            "      if (in && !put) set_err(err, -1);",
            "      old[j] = put ? atomicCAS(&I.dir[slot], -1, (int)(r0 + j)) : -1;",
            "    }",
            "#pragma unroll", "    for (int j = 0; j < 4; ++j) if (old[j] != -1) set_err(err, -7);",
            "  }", "}"]
    # probe: predicate, lookup, warp-dense value pass
    pcols, pexpr = jit._pred_code(ppred, "p") if ppred is not None else ([], "true")
    plit, pexpr = _hoist(pexpr, "I")
    ecols, elines = jit._expr_code(S, val_reg + 1, "c")
    src += [f"__device__ void jn_probe_{p}(const QInst& I, i64 b, i64 e, u64* sm) {{",
            "  __shared__ unsigned char q_off[8][256];",
            "  __shared__ int q_slot[8][256];",
            "  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;",
            "  const i64 np = I.n, key_min = I.kmin[0], slots = I.slots;",
            "  const bool vp = I.flags & 1, vf = I.flags & 8;",
            "  const int* __restrict__ dir = I.dir;",
            "  double* __restrict__ sum = I.sum;",
            "  unsigned* __restrict__ occ = I.occ;",
            "  // sums of a small key domain gather in shared memory first (many rows per key: reductions",
            "  // into a few global cells queue at the L2): mode 1 one copy per thread, mode 2 `copies`",
            "  // copies shared by threads tid % copies; cells start at -0.0, the untouched marker",
            "  const int jm = I.mode, copies = jm == 1 ? " + str(T) + " : I.copies;",
            "  const int lgc = __ffs(copies) - 1, me = threadIdx.x & (copies - 1);",
            "  if (jm) {",
            f"    for (int i = threadIdx.x; i < (int)slots * copies; i += {T}) sm[i] = 0x8000000000000000ull;",
            "    __syncthreads();",
            "  }"]
    src += ["  " + d for d in plit]
    if ppred is not None:
        src += ["  " + d for d in _ptr_decls(pcols, ppred.dtypes, "pc", "pp")]
    for c in ecols:
        t = jit._CTYPE[S.col_dtypes[c]]
        src.append(f"  const {t}* __restrict__ cp{c} = (const {t}*)I.vc[{c}];")
    src += ["  // rows [b, e) as groups of 8 per lane (b % 8 == 0); e is a multiple of 8 or the end",
            "  for (i64 w0 = (b >> 3) + (threadIdx.x & ~31); w0 < ((e + 7) >> 3); w0 += " + str(T) + ") {",
            "    const i64 g = w0 + lane, wrow = w0 << 3;",
            "    i64 sl[2][4]; unsigned m[2];",
            "#pragma unroll",
            "    for (int u = 0; u < 2; ++u) {",
            "      const i64 r0 = ((g << 1) + u) << 2;",
            "      m[u] = 0;",
            "      if (r0 >= e) continue;"]
    if ppred is not None:
        src += ["      " + l for l in _ld4(pcols, ppred.dtypes, "P", "pp", "np", "vp")]
    src += ["      const V4<i64> F = (I.fk_dt == 4) ? ld4((const long long*)I.kc[0], r0, np, vf) : "
            "[&]{ V4<int> t = ld4((const int*)I.kc[0], r0, np, vf); V4<i64> o; "
            "for (int q = 0; q < 4; ++q) o.v[q] = t.v[q]; return o; }();",
            "#pragma unroll",
            "      for (int j = 0; j < 4; ++j) {",
            "        sl[u][j] = F.v[j] - key_min;",
            f"        const bool ok = (r0 + j < e) && ({jit._rename(pexpr, 'p', 'P')}) && sl[u][j] >= 0 && sl[u][j] < slots;",
            "        m[u] |= (unsigned)ok << j;",
            "      }",
            "    }",
            "#pragma unroll",
            "    for (int u = 0; u < 2; ++u)",
            "#pragma unroll",
            "      for (int j = 0; j < 4; ++j)",
            "        if (((m[u] >> j) & 1u) && __ldcg(&dir[sl[u][j]]) < 0) m[u] &= ~(1u << j);"]
    sum_stmt = ("if (jm == 0) { gred_add(&sum[slot], vz); occ[slot] = 1u; } else { "
                "const double va = d2u(vz) == 0x8000000000000000ull ? 0.0 : vz; "
                "double* cell = (double*)&sm[((int)slot << lgc) + me]; "
                "if (jm == 1) *cell = __dadd_rn(*cell, va); else atomicAdd(cell, va); }")
    src += jit._dense_tail(S, val_reg, ecols, elines, "np", "sl", [], sum_stmt=sum_stmt)
    src += ["  }",
            "  if (jm) {            // fold each key's copies (untouched ones skipped) into the global sums",
            "    __syncthreads();",
            f"    for (int s = threadIdx.x; s < (int)slots; s += {T}) {{",
            "      double t = 0.0; bool hit = false;",
            "      for (int c = 0; c < copies; ++c) {",
            "        const u64 x = sm[(s << lgc) + ((c + s) & (copies - 1))];   // staggered: fewer bank conflicts",
            "        if (x != 0x8000000000000000ull) { t = __dadd_rn(t, u2d(x)); hit = true; }",
            "      }",
            "      if (hit) { gred_add(&sum[s], t); occ[s] = 1u; }",
            "    }",
            "    __syncthreads();",
            "  }",
            "}"]
    return "\n".join(src)


_GENERIC = r"""
__device__ void gb_count(const QInst& I, i64 item, i64 b, i64 e) {
  unsigned local = 0;
  for (i64 s = b + threadIdx.x; s < e; s += blockDim.x) local += __ldcg(&I.gacc[s]) != 0;   // acc 0 counts rows
  local = __reduce_add_sync(0xffffffffu, local);
  __shared__ unsigned long long s_cnt;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(&s_cnt, (unsigned long long)local);
  __syncthreads();
  if (threadIdx.x == 0) I.range_count[item] = (i64)s_cnt;
}
// per-item top-k of slots [b, e): 8 warp lists merged by warp 0 into cand[item]
__device__ void jn_topk_part(const QInst& I, i64 item, i64 b, i64 e, u64* sk, i64* si) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, k = I.k;
  WL wl; wl.init();
  unsigned valid = 0;
  for (i64 base = b + (i64)wid * 128; base < e; base += 1024) {
    const i64 i0 = base + lane * 4;
    u64 key[4]; unsigned ok = 0;
    if (i0 + 4 <= e) {
      const uint4 cc = __ldcg(reinterpret_cast<const uint4*>(I.occ + i0));
      const double2 x = __ldcg(reinterpret_cast<const double2*>(I.sum + i0));
      const double2 y = __ldcg(reinterpret_cast<const double2*>(I.sum + i0 + 2));
      const unsigned c[4] = {cc.x, cc.y, cc.z, cc.w};
      const double v[4] = {x.x, x.y, y.x, y.y};
      for (int q = 0; q < 4; ++q) { key[q] = sum_key(v[q], I.desc); ok |= (c[q] != 0u ? 1u : 0u) << q; }
    } else {
      for (int q = 0; q < 4; ++q) {
        const bool in = i0 + q < e;
        key[q] = sum_key(in ? __ldcg(&I.sum[i0 + q]) : 0.0, I.desc);
        ok |= ((in && __ldcg(&I.occ[i0 + q]) != 0u) ? 1u : 0u) << q;
      }
    }
    valid += __popc(ok);
    for (int q = 0; q < 4; ++q) wl.offer(k, key[q], i0 + q, (ok >> q) & 1u);
  }
  valid = __reduce_add_sync(0xffffffffu, valid);
  sk[wid * 32 + lane] = wl.key;
  si[wid * 32 + lane] = wl.idx;
  __shared__ unsigned long long s_valid;
  if (threadIdx.x == 0) s_valid = 0;
  __syncthreads();
  if (lane == 0 && valid) atomicAdd(&s_valid, (unsigned long long)valid);
  __syncthreads();
  if (wid == 0) {
    WL m; m.init();
    for (int w = 0; w < 8; ++w) m.offer(k, sk[w * 32 + lane], si[w * 32 + lane], lane < k && si[w * 32 + lane] >= 0);
    if (lane < k) { I.cand_key[item * k + lane] = m.key; I.cand_idx[item * k + lane] = m.idx; }
    if (lane == 0) I.range_count[item] = (i64)s_valid;
  }
  __syncthreads();
}
__device__ void jn_topk_merge(const QInst& I, u64* sk, i64* si) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, k = I.k;
  const i64 parts = I.ni[2], total = parts * k;
  WL wl; wl.init();
  for (i64 base = 0; base < total; base += 256) {
    const i64 g = base + threadIdx.x;
    const i64 ii = g < total ? __ldcg(&I.cand_idx[g]) : -1;
    wl.offer(k, g < total ? __ldcg(&I.cand_key[g]) : ~0ull, ii, ii >= 0);
  }
  sk[wid * 32 + lane] = wl.key;
  si[wid * 32 + lane] = wl.idx;
  __syncthreads();
  if (wid == 0) {
    WL m; m.init();
    for (int w = 0; w < 8; ++w) m.offer(k, sk[w * 32 + lane], si[w * 32 + lane], lane < k && si[w * 32 + lane] >= 0);
    const bool v = lane < k && m.idx >= 0;
    const int cnt = __popc(__ballot_sync(0xffffffffu, v));
    if (v) { I.out_keys[lane] = I.kmin[0] + m.idx; I.out_vals[lane] = __ldcg(&I.sum[m.idx]); }
    i64 groups = 0;
    for (i64 r = lane; r < parts; r += 32) groups += __ldcg(&I.range_count[r]);
    for (int o = 16; o; o >>= 1) groups += __shfl_xor_sync(0xffffffffu, groups, o);
    if (lane == 0) {
      *I.out_count = cnt;
      if (I.out_groups) *I.out_groups = groups;
    }
  }
  __syncthreads();
}
"""


# result packing: span i copies desc[3i+1] bytes from address desc[3i] to out + desc[3i+2]
# (sources 256-byte aligned allocations, offsets multiples of 16: 16-byte pieces, then bytes)
_PACK_SRC = r"""
extern "C" __global__ void tqpk_pack_spans(const long long* __restrict__ desc, int n, unsigned char* __restrict__ out) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x, nt = (long long)gridDim.x * blockDim.x;
  for (int i = 0; i < n; ++i) {
    const unsigned char* src = (const unsigned char*)desc[3 * i];
    const long long nb = desc[3 * i + 1];
    unsigned char* dst = out + desc[3 * i + 2];
    const long long n16 = nb >> 4;
    for (long long j = tid; j < n16; j += nt) ((uint4*)dst)[j] = ((const uint4*)src)[j];
    for (long long j = (n16 << 4) + tid; j < nb; j += nt) dst[j] = src[j];
  }
}
"""


def batch_source(gb_progs, join_progs) -> str:
    """gb_progs: [(spec, pred, outputs)], join_progs: [(spec, val_reg, ppred, bpred)]."""
    parts = [jit.PRELUDE, _BATCH_PRELUDE, _struct_c(), _GENERIC]
    for p, (spec, pred, outputs) in enumerate(gb_progs):
        body, _ = _gb_functions(p, spec, pred)
        parts.append(body + "\n" + _gb_emit_outputs(p, spec, outputs))
    for p, (spec, vreg, ppred, bpred) in enumerate(join_progs):
        parts.append(_join_functions(p, spec, vreg, ppred, bpred))
    gb_agg = "\n".join(f"        case {p}: gb_agg_{p}(I, W.begin, W.end, sm, err); break;" for p in range(len(gb_progs)))
    gb_emit = "\n".join(f"        case {p}: gb_emit_{p}(I, W.begin / I.range_slots, W.begin, W.end, sw); break;"
                        for p in range(len(gb_progs)))
    jb = "\n".join(f"        case {p}: jn_build_{p}(I, W.begin, W.end, err); break;" for p in range(len(join_progs)))
    jp = "\n".join(f"        case {p}: jn_probe_{p}(I, W.begin, W.end, sm); break;" for p in range(len(join_progs)))
    parts.append(f"""
extern "C" __global__ void __launch_bounds__({T}, {MIN_CTAS}) tqpk_qb_run(const QInst* __restrict__ insts,
    const WorkItem* __restrict__ items, int n_items, unsigned* ticket, unsigned long long* done, int* err,
    unsigned long long* trace) {{
  extern __shared__ u64 sm[];
  __shared__ int s_item;
  __shared__ int sw[{T // 32}];
  __shared__ u64 sk[{T}];
  __shared__ i64 si[{T}];
  while (true) {{
    if (threadIdx.x == 0) s_item = (int)atomicAdd(ticket, 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) return;
    const WorkItem W = items[it];
    const QInst& I = insts[W.inst];
    unsigned long long t0 = 0, t1 = 0;
    if (trace && threadIdx.x == 0) t0 = gtimer();
    if (W.phase > 0 && threadIdx.x == 0) {{
      const unsigned long long need = (unsigned long long)I.ni[W.phase - 1];
      const unsigned long long* flag = &done[W.inst * 4 + W.phase - 1];
      int spins = 0;
      while (ld_acq(flag) < need) {{
        if (++spins > (1 << 21)) {{ set_err(err, -3); break; }}
        __nanosleep(128);
      }}
    }}
    __syncthreads();
    if (trace && threadIdx.x == 0) t1 = gtimer();
    if (I.kind == {KIND_GB}) {{
      if (W.phase == 0) {{
        switch (I.prog) {{
{gb_agg}
        }}
      }} else if (W.phase == 1) {{
        gb_count(I, W.begin / I.range_slots, W.begin, W.end);
      }} else {{
        switch (I.prog) {{
{gb_emit}
        }}
      }}
    }} else {{
      if (W.phase == 0) {{
        switch (I.prog) {{
{jb}
        }}
      }} else if (W.phase == 1) {{
        switch (I.prog) {{
{jp}
        }}
      }} else if (W.phase == 2) {{
        jn_topk_part(I, W.begin / I.range_slots, W.begin, W.end, sk, si);
      }} else {{
        jn_topk_merge(I, sk, si);
      }}
    }}
    __syncthreads();
    if (threadIdx.x == 0) {{
      __threadfence();
      atomicAdd(&done[W.inst * 4 + W.phase], 1ull);
      if (trace) {{
        unsigned smid; asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        trace[4 * it] = t0; trace[4 * it + 1] = t1; trace[4 * it + 2] = gtimer(); trace[4 * it + 3] = smid;
      }}
    }}
  }}
}}
""")
    # table reset kernel (group tables to their accumulator initial values; join directories empty)
    inits = []
    for p, (spec, pred, outputs) in enumerate(gb_progs):
        vals = ", ".join(jit._acc_init(spec.accs[a]) for a in range(spec.n_accs))
        inits.append(f"      case {p}: {{ const u64 iv[] = {{{vals}}}; v = iv[j / I.slots]; break; }}")
    init_cases = "\n".join(inits)
    parts.append(f"""
extern "C" __global__ void tqpk_qb_reset(const QInst* __restrict__ insts, int n_inst) {{
  for (int i = blockIdx.y; i < n_inst; i += gridDim.y) {{
    const QInst& I = insts[i];
    const i64 stride = (i64)gridDim.x * blockDim.x;
    if (I.kind == {KIND_GB}) {{
      const i64 total = I.slots * I.ni[3];   // ni[3] holds the accumulator count for group-by
      for (i64 j = blockIdx.x * (i64)blockDim.x + threadIdx.x; j < total; j += stride) {{
        u64 v = 0;
        switch (I.prog) {{
{init_cases}
        }}
        I.gacc[j] = v;
      }}
    }} else {{
      for (i64 j = blockIdx.x * (i64)blockDim.x + threadIdx.x; j < I.slots; j += stride) {{
        I.dir[j] = -1; I.sum[j] = 0.0; I.occ[j] = 0u;
      }}
    }}
  }}
}}
""")
    return "\n".join(parts)


# ---------------------------------------------------------------------------- host side
def _no_strings(pred):
    from .predicate import has_strings
    if pred is not None and has_strings(pred.struct):
        raise NotImplementedError("string predicates run on the operator path, not in the generated batch kernel")


def _mode(K: int, A: int) -> Tuple[int, int]:
    """(mode, copies) of a group table of K slots x A accumulators: as many shared-memory
    copies as fit (a power of two, at most one per thread); with 32 or more, the lanes of a
    warp never update the same copy."""
    fit = SMEM // max(1, K * A * 8)
    if fit >= T:
        return 1, T
    if fit >= 1:
        return 2, 1 << int(math.floor(math.log2(fit)))
    return 4, 1


def _join_mode(slots: int, rows_per_item: int) -> Tuple[int, int]:
    """(mode, copies) of a join probe's sums: a shared-memory table per item when the key domain
    is small next to the item (one copy per thread, mode 1, or the shared copies that fit, mode 2),
    else reductions straight into the global sums (mode 0)."""
    fit = SMEM // max(1, slots * 8)
    if fit >= T:
        return 1, T
    if fit >= 1 and slots * 4 <= rows_per_item:
        return 2, 1 << int(math.floor(math.log2(fit)))
    return 0, 1


def _aligned(*ts) -> bool:
    return all(t.data_ptr() % 16 == 0 for t in ts if t is not None)


class QueryBatch:
    """Instances of tqpk.batch (GroupByInstance / JoinInstance) in one generated persistent launch."""

    def __init__(self, instances: List[object], tuner: Optional[Autotuner] = None):
        if not jit.available():
            raise RuntimeError("QueryBatch needs the runtime compiler (NVRTC)")
        self.lib = L.load()
        self.tuner = tuner or Autotuner()
        self.instances = instances
        n = len(instances)
        self.recs = (QInst * n)()
        self.keep: list = []
        self.outs: list = []
        self.gb_progs, self.join_progs = [], []
        self._gb_index: Dict[str, int] = {}
        self._jn_index: Dict[str, int] = {}
        self.dev = None
        items = []
        for i, inst in enumerate(instances):
            if isinstance(inst, JoinInstance):
                self.outs.append(self._describe_join(self.recs[i], inst))
            else:
                self.outs.append(self._describe_groupby(self.recs[i], inst))
        phases = {KIND_GB: 3, KIND_JOIN: 4}
        for ph in range(4):
            for i, r in enumerate(self.recs):
                if ph >= phases[r.kind]:
                    continue
                if r.kind == KIND_GB:
                    total, step = (r.n, self._rpi[i]) if ph == 0 else (r.slots, r.range_slots)
                else:
                    total, step = [(r.nb, self._rpi[i][0]), (r.n, self._rpi[i][1]), (r.slots, r.range_slots),
                                   (1, 1)][ph]
                for j in range(int(r.ni[ph])):
                    items.append((i, ph, j * step, min(total, (j + 1) * step)))
        self.n_items = len(items)
        arr = np.zeros(self.n_items, dtype=[("inst", "<i4"), ("phase", "<i4"), ("begin", "<i8"), ("end", "<i8")])
        for f, col in zip(arr.dtype.names, zip(*items)):
            arr[f] = col
        self.items_np = arr
        self.d_items = torch.from_numpy(arr.view(np.uint8).copy()).to(self.dev)
        self.d_recs = torch.frombuffer(bytearray(bytes(self.recs)), dtype=torch.uint8).to(self.dev)
        self.ctl = torch.zeros(64 + 32 * n, dtype=torch.uint8, device=self.dev)
        src = batch_source(self.gb_progs, self.join_progs)
        self.source = src
        self.k_run = jit.compile_kernel(src, "tqpk_qb_run")
        self.k_reset = jit.compile_kernel(src, "tqpk_qb_reset")
        self.grid = max(1, jit.occupancy_grid(self.k_run, T, SMEM, 1 << 30))
        self.graph = None
        self._trace = None

    # ------------------------------------------------------------------ describe
    def _program(self, table: Dict[str, int], progs: list, key: str, entry) -> int:
        if key not in table:
            table[key] = len(progs)
            progs.append(entry)
        return table[key]

    def _describe_groupby(self, R: QInst, inst: GroupByInstance):
        cols = inst.columns
        dev = next(iter(cols.values())).device
        self.dev = dev
        prog = compile_aggregate(inst.args, cols)
        require_f64_outputs(prog, "batched group-by")
        pred = compile_filter(inst.filter_tree, inst.filter_cols) if inst.filter_tree is not None else None
        _no_strings(pred)
        S = prog.spec
        nk = S.n_keys
        K = int(np.prod([int(d[1]) - int(d[0]) + 1 for d in inst.key_domains])) if nk else 1
        n = int(next(iter(cols.values())).shape[0])
        code, _ = _gb_functions(0, S, pred.struct if pred else None)
        key = code + _gb_emit_outputs(0, S, prog.outputs)
        p = self._program(self._gb_index, self.gb_progs, key, (S, pred.struct if pred else None, prog.outputs))
        R.kind, R.prog, R.n, R.slots = KIND_GB, p, n, K
        R.mode, R.copies = _mode(K, S.n_accs)
        stride = 1
        for k in range(nk - 1, -1, -1):
            lo, hi = int(inst.key_domains[k][0]), int(inst.key_domains[k][1])
            R.kmin[k], R.krange[k], R.kstride[k] = lo, hi - lo + 1, stride
            stride *= hi - lo + 1
        rpi = self.tuner.rows_per_item("groupby", n)
        R.range_slots = min(4096, -(-K // 256) * 256)
        R.ni[0] = -(-n // rpi) if n else 0
        R.ni[1] = R.ni[2] = -(-K // R.range_slots)
        R.ni[3] = S.n_accs
        if pred is not None:
            for c in range(pred.struct.n_cols):
                R.pc[c] = pred.struct.cols[c]
            R.lp = jit.pred_lits(pred.struct)
        for k in range(nk):
            R.kc[k] = S.keys[k]
        for c in range(S.n_cols):
            R.vc[c] = S.cols[c]
        R.flags = ((F_PVEC if pred is None or _aligned(*pred.tensors) else 0)
                   | (F_KVEC if _aligned(*prog.tensors[:nk]) else 0) | (F_VVEC if _aligned(*prog.tensors[nk:]) else 0))
        gacc = torch.empty(K * S.n_accs, dtype=torch.int64, device=dev)
        rc = torch.zeros(int(R.ni[1]), dtype=torch.int64, device=dev)
        keys = [torch.empty(K, dtype=dtype_of(S.key_dtypes[k]), device=dev) for k in range(nk)]
        outs = [torch.empty(K, dtype=dt, device=dev) for (_, _, _, _, dt) in prog.outputs]
        groups = torch.zeros(1, dtype=torch.int64, device=dev)
        R.gacc, R.range_count, R.out_groups = gacc.data_ptr(), rc.data_ptr(), groups.data_ptr()
        for k in range(nk):
            R.out_key[k] = keys[k].data_ptr()
        for o, t in enumerate(outs):
            R.out_col[o] = t.data_ptr()
        self._rpi = getattr(self, "_rpi", {})
        self._rpi[len(self.outs)] = rpi
        self.keep += [prog, pred, gacc, rc]
        return {"kind": "groupby", "keys": keys, "outs": outs, "groups": groups, "prog": prog}

    def _describe_join(self, R: QInst, inst: JoinInstance):
        dev = inst.build_keys.device
        self.dev = dev
        if not 1 <= inst.k <= MAXK:
            raise NotImplementedError(f"the batched join top-k handles k <= {MAXK}")
        bk, pk = inst.build_keys.contiguous(), inst.probe_fk.contiguous()
        if bk.dtype not in (torch.int32, torch.int64) or pk.dtype not in (torch.int32, torch.int64):
            raise TypeError("join keys must be int32 or int64")
        bpred = compile_filter(inst.build_filter, inst.build_cols) if inst.build_filter is not None else None
        ppred = compile_filter(inst.probe_filter, inst.probe_cols) if inst.probe_filter is not None else None
        _no_strings(bpred)
        _no_strings(ppred)
        prog = compile_aggregate({"keys": None, "results": [[[["sum", inst.value_tree], "#", "1"], "AS", "v#1"]]},
                                 inst.probe_cols)
        require_f64_outputs(prog, "batched join")
        S = prog.spec
        vreg = S.accs[prog.outputs[0][2]].reg
        key = _join_functions(0, S, vreg, ppred.struct if ppred else None, bpred.struct if bpred else None)
        p = self._program(self._jn_index, self.join_progs, key,
                          (S, vreg, ppred.struct if ppred else None, bpred.struct if bpred else None))
        kmin, kmax = map(int, inst.key_domain)
        slots = kmax - kmin + 1
        if slots > (1 << 31):
            raise NotImplementedError("join key domain above 2^31 slots")
        R.kind, R.prog, R.k, R.desc = KIND_JOIN, p, int(inst.k), int(inst.descending)
        R.n, R.nb, R.slots, R.kmin[0] = pk.numel(), bk.numel(), slots, kmin
        R.fk_dt, R.bk_dt = code_of(pk.dtype), code_of(bk.dtype)
        rb = self.tuner.rows_per_item("join_build", bk.numel())
        rp = self.tuner.rows_per_item("join_probe", pk.numel())
        R.mode, R.copies = _join_mode(slots, rp)
        R.range_slots = min(1 << 14, -(-slots // 256) * 256)
        R.ni[0] = -(-bk.numel() // rb) if bk.numel() else 0
        R.ni[1] = -(-pk.numel() // rp) if pk.numel() else 0
        R.ni[2] = -(-slots // R.range_slots)
        R.ni[3] = 1
        R.kc[0], R.kc[1] = pk.data_ptr(), bk.data_ptr()
        if ppred is not None:
            for c in range(ppred.struct.n_cols):
                R.pc[c] = ppred.struct.cols[c]
            R.lp = jit.pred_lits(ppred.struct)
        if bpred is not None:
            for c in range(bpred.struct.n_cols):
                R.bc[c] = bpred.struct.cols[c]
            R.lb = jit.pred_lits(bpred.struct)
        for c in range(S.n_cols):
            R.vc[c] = S.cols[c]
        R.flags = ((F_PVEC if ppred is None or _aligned(*ppred.tensors) else 0)
                   | (F_VVEC if _aligned(*prog.tensors) else 0) | (F_FVEC if _aligned(pk) else 0)
                   | (F_BVEC if bpred is None or _aligned(*bpred.tensors) else 0))
        d = torch.empty(slots, dtype=torch.int32, device=dev)
        sm = torch.empty(slots, dtype=torch.float64, device=dev)
        oc = torch.empty(-(-slots // 4) * 4, dtype=torch.int32, device=dev)
        rc = torch.zeros(int(R.ni[2]), dtype=torch.int64, device=dev)
        ck = torch.empty(int(R.ni[2]) * R.k, dtype=torch.int64, device=dev)
        ci = torch.empty(int(R.ni[2]) * R.k, dtype=torch.int64, device=dev)
        out_keys = torch.empty(inst.k, dtype=torch.int64, device=dev)
        out_vals = torch.empty(inst.k, dtype=torch.float64, device=dev)
        out_count = torch.zeros(1, dtype=torch.int64, device=dev)
        groups = torch.zeros(1, dtype=torch.int64, device=dev)
        R.dir, R.sum, R.occ = d.data_ptr(), sm.data_ptr(), oc.data_ptr()
        R.range_count, R.cand_key, R.cand_idx = rc.data_ptr(), ck.data_ptr(), ci.data_ptr()
        R.out_keys, R.out_vals, R.out_count, R.out_groups = (out_keys.data_ptr(), out_vals.data_ptr(),
                                                            out_count.data_ptr(), groups.data_ptr())
        self._rpi = getattr(self, "_rpi", {})
        self._rpi[len(self.outs)] = (rb, rp)
        self.keep += [bk, pk, bpred, ppred, prog, d, sm, oc, rc, ck, ci]
        return {"kind": "join", "keys": out_keys, "vals": out_vals, "count": out_count, "groups": groups}

    # ------------------------------------------------------------------ run
    def run(self, stream=None):
        st = stream or torch.cuda.current_stream(self.dev)
        s = st.cuda_stream
        n = len(self.instances)
        with torch.cuda.stream(st):
            self.ctl.zero_()
        a = jit._Args()
        a.ptr(self.d_recs.data_ptr())
        a.i32(n)
        jit.launch(self.k_reset, 512, 256, 0, a, s)
        a = jit._Args()
        ctl = self.ctl.data_ptr()
        a.ptr(self.d_recs.data_ptr())
        a.ptr(self.d_items.data_ptr())
        a.i32(self.n_items)
        a.ptr(ctl)
        a.ptr(ctl + 64)
        a.ptr(ctl + 4)
        a.ptr(self._trace.data_ptr() if self._trace is not None else None)
        jit.launch(self.k_run, self.grid, T, SMEM, a, s, L.KID_BATCH)

    def capture(self):
        self.run()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.run()
        return self.graph

    def replay(self):
        self.graph.replay()

    def check_error(self):
        err = int(self.ctl[4:8].view(torch.int32).item())
        if err:
            L.check(err, "batched run")

    def results_host(self):
        """results() with two device-to-host reads in all: every instance's row and group counts
        (and the error word) packed into one copy; then one generated kernel packs every result
        row (each column's first rows, 16-byte aligned spans) and one copy brings them to pinned
        memory.  Returns (results, bytes read); the arrays are views of that pinned buffer, valid
        until the next call (copy what is kept longer)."""
        if not hasattr(self, "_span_cols"):
            self._count_src, self._span_cols = [self.ctl[4:8].view(torch.int32).to(torch.int64)], []
            for o in self.outs:             # (tensor, index of its row count in the packed counts)
                if o["kind"] == "join":
                    at = len(self._count_src)
                    self._count_src += [o["count"], o["groups"]]
                    self._span_cols += [(o["keys"], at), (o["vals"], at)]
                else:
                    at = len(self._count_src)
                    self._count_src.append(o["groups"])
                    self._span_cols += [(t, at) for t in list(o["keys"]) + list(o["outs"])]
            self._span_src = np.array([t.data_ptr() for t, _ in self._span_cols], dtype=np.int64)
            self._span_es = np.array([t.element_size() for t, _ in self._span_cols], dtype=np.int64)
            self._span_at = np.array([at for _, at in self._span_cols], dtype=np.int64)
            self._k_pack = jit.compile_kernel(_PACK_SRC, "tqpk_pack_spans")
        st = torch.cuda.current_stream(self.dev)
        self._count_src[0] = self.ctl[4:8].view(torch.int32).to(torch.int64)   # the error word, this run
        counts = torch.cat(self._count_src)
        hc = self._pinned("counts", counts.numel(), torch.int64)
        hc.copy_(counts, non_blocking=True)
        st.synchronize()
        c = hc.numpy().copy()
        if c[0]:
            L.check(int(c[0]), "batched run")
        rows = c[self._span_at]
        nbytes = rows * self._span_es
        offs = np.zeros(len(nbytes), dtype=np.int64)
        if len(nbytes) > 1:
            offs[1:] = np.cumsum((nbytes + 15) // 16 * 16)[:-1]
        total = int(offs[-1] + nbytes[-1]) if len(nbytes) else 0
        desc = self._pinned("desc", 3 * len(nbytes), torch.int64)
        dn = desc.numpy().reshape(-1, 3)
        dn[:, 0], dn[:, 1], dn[:, 2] = self._span_src, nbytes, offs
        ddesc = self._device_buf("desc", desc.numel() * 8).view(torch.int64)
        ddesc.copy_(desc, non_blocking=True)
        packed = self._device_buf("rows", max(total, 16))
        a = jit._Args()
        a.ptr(ddesc.data_ptr())
        a.i32(len(nbytes))
        a.ptr(packed.data_ptr())
        jit.launch(self._k_pack, max(1, min(4 * 152, (total // 16 + 255) // 256)), 256, 0, a, st.cuda_stream)
        hp = self._pinned("rows", total, torch.uint8)
        hp.copy_(packed[:total], non_blocking=True)
        st.synchronize()
        buf = hp.numpy()
        arrays = [buf[o:o + n].view(np.dtype(str(t.dtype).replace("torch.", "")))
                  for (t, _), o, n in zip(self._span_cols, offs.tolist(), nbytes.tolist())]
        res, i, pos = [], 0, 1
        for o in self.outs:
            if o["kind"] == "join":
                res.append((arrays[i], arrays[i + 1], int(c[pos + 1])))
                i += 2
                pos += 2
            else:
                nk = len(o["keys"])
                keys = arrays[i:i + nk]
                i += nk
                outs = {oid: arr for (oid, *_), arr in zip(o["prog"].outputs, arrays[i:i + len(o["outs"])])}
                i += len(o["outs"])
                res.append((outs, keys, int(c[pos])))
                pos += 1
        return res, int(counts.numel() * 8 + total)

    def _device_buf(self, name, nbytes):
        bufs = self.__dict__.setdefault("_dev_bufs", {})
        b = bufs.get(name)
        if b is None or b.numel() < nbytes:
            b = bufs[name] = torch.empty(max(nbytes, 1 << 16), dtype=torch.uint8, device=self.dev)
        return b[:nbytes]

    def _pinned(self, name, n, dtype):
        bufs = self.__dict__.setdefault("_host_bufs", {})
        b = bufs.get(name)
        if b is None or b.numel() < n or b.dtype != dtype:
            b = bufs[name] = torch.empty(max(n, 1024), dtype=dtype, pin_memory=True)
        return b[:n]

    def results(self):
        self.check_error()
        res = []
        for o in self.outs:
            if o["kind"] == "join":
                m = int(o["count"].item())
                res.append((o["keys"][:m].cpu().numpy(), o["vals"][:m].cpu().numpy(), int(o["groups"].item())))
            else:
                g = int(o["groups"].item())
                prog = o["prog"]
                outs = {oid: col[:g].cpu().numpy() for (oid, *_), col in zip(prog.outputs, o["outs"])}
                res.append((outs, [k[:g].cpu().numpy() for k in o["keys"]], g))
        return res

    def item_timeline(self) -> np.ndarray:
        """One run outside any graph with the per-item timeline on (see tqpk.batch.Batch.item_timeline)."""
        self._trace = torch.zeros(self.n_items * 4, dtype=torch.int64, device=self.dev)
        try:
            self.run()
            torch.cuda.synchronize()
        finally:
            tr, self._trace = self._trace, None
        t = tr.cpu().numpy().reshape(-1, 4)
        out = np.zeros(self.n_items, dtype=[("inst", "i4"), ("phase", "i4"), ("begin", "i8"), ("end", "i8"),
                                            ("t_deq", "f8"), ("t_ready", "f8"), ("t_done", "f8"), ("sm", "i4")])
        for f in ("inst", "phase", "begin", "end"):
            out[f] = self.items_np[f]
        t0 = t[:, 0].min()
        out["t_deq"], out["t_ready"], out["t_done"] = (t[:, 0] - t0) / 1e3, (t[:, 1] - t0) / 1e3, (t[:, 2] - t0) / 1e3
        out["sm"] = t[:, 3]
        return out
