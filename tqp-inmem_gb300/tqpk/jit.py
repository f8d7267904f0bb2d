"""Query-specialised kernels: CUDA C++ generated per query, compiled with NVRTC.

The interpreting kernels in libtqpk evaluate the predicate, expression and
accumulator programs instruction by instruction for every row.  For the hot
loops (filter + group-by accumulation, the fused join probe) this module
emits the query's program as straight-line code instead: column loads of four
rows at a time (128-bit when aligned), the predicate as one boolean
expression with its literals inlined as exact hex floats, SSA arithmetic with
the same IEEE round-to-nearest operations (``__dadd_rn`` ...), and one
accumulator update per aggregate with its table offset folded in.  The
results are identical to the interpreting kernels' (same operations, same
table encodings); only the instruction count per row changes.

``tqpk_jit_compile`` (libtqpk) compiles with NVRTC for sm_103a and loads the
cubin; kernels are cached by their source text.  When NVRTC is not available
the callers keep using the interpreting kernels.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import struct
import threading
from typing import Dict, List, Optional, Sequence, Tuple

from . import _lib as L

_CMP_OP = {L.LT: "<", L.LE: "<=", L.GT: ">", L.GE: ">=", L.EQ: "==", L.NE: "!="}
_CTYPE = {L.I8: "signed char", L.U8: "unsigned char", L.BOOL: "unsigned char", L.I32: "int", L.I64: "long long",
          L.F64: "double"}
_lock = threading.Lock()
_cache: Dict[str, int] = {}
_available: Optional[bool] = None

PRELUDE = r"""
typedef long long i64;
typedef unsigned long long u64;
typedef unsigned int u32;
__device__ __forceinline__ u64 d2u(double d) { return (u64)__double_as_longlong(d); }
__device__ __forceinline__ double u2d(u64 u) { return __longlong_as_double((long long)u); }
__device__ __forceinline__ u64 ford(double d) { u64 u = d2u(d); return (u >> 63) ? ~u : (u | (1ull << 63)); }
__device__ __forceinline__ bool iscl(double x, double lit, double allowed) {
  double e = fabs(__dsub_rn(x, lit));
  return (x == lit) || (isfinite(e) && e <= allowed);
}
template <class T> struct V4 { T v[4]; };
// four consecutive rows r0..r0+3 (r0 % 4 == 0); rows >= n read as 0
__device__ __forceinline__ V4<double> ld4(const double* p, i64 r0, i64 n, bool vec) {
  V4<double> o;
  if (vec && r0 + 4 <= n) {
    const double2* q = reinterpret_cast<const double2*>(p + r0);
    double2 a = q[0], b = q[1];
    o.v[0] = a.x; o.v[1] = a.y; o.v[2] = b.x; o.v[3] = b.y;
  } else {
    for (int j = 0; j < 4; ++j) o.v[j] = (r0 + j < n) ? p[r0 + j] : 0.0;
  }
  return o;
}
__device__ __forceinline__ V4<long long> ld4(const long long* p, i64 r0, i64 n, bool vec) {
  V4<long long> o;
  if (vec && r0 + 4 <= n) {
    const longlong2* q = reinterpret_cast<const longlong2*>(p + r0);
    longlong2 a = q[0], b = q[1];
    o.v[0] = a.x; o.v[1] = a.y; o.v[2] = b.x; o.v[3] = b.y;
  } else {
    for (int j = 0; j < 4; ++j) o.v[j] = (r0 + j < n) ? p[r0 + j] : 0;
  }
  return o;
}
__device__ __forceinline__ V4<int> ld4(const int* p, i64 r0, i64 n, bool vec) {
  V4<int> o;
  if (vec && r0 + 4 <= n) {
    int4 a = *reinterpret_cast<const int4*>(p + r0);
    o.v[0] = a.x; o.v[1] = a.y; o.v[2] = a.z; o.v[3] = a.w;
  } else {
    for (int j = 0; j < 4; ++j) o.v[j] = (r0 + j < n) ? p[r0 + j] : 0;
  }
  return o;
}
template <class B>
__device__ __forceinline__ V4<B> ld4b(const B* p, i64 r0, i64 n, bool vec) {
  V4<B> o;
  if (vec && r0 + 4 <= n) {
    unsigned w = *reinterpret_cast<const unsigned*>(p + r0);
    for (int j = 0; j < 4; ++j) o.v[j] = (B)((w >> (8 * j)) & 0xff);
  } else {
    for (int j = 0; j < 4; ++j) o.v[j] = (r0 + j < n) ? p[r0 + j] : (B)0;
  }
  return o;
}
__device__ __forceinline__ V4<signed char> ld4(const signed char* p, i64 r0, i64 n, bool vec) { return ld4b(p, r0, n, vec); }
__device__ __forceinline__ V4<unsigned char> ld4(const unsigned char* p, i64 r0, i64 n, bool vec) { return ld4b(p, r0, n, vec); }
"""


def available() -> bool:
    """NVRTC can be opened and TQPK_JIT is not set to 0."""
    global _available
    import os
    if os.environ.get("TQPK_JIT", "1") == "0":
        return False
    if _available is None:
        _available = bool(L.load().tqpk_jit_available())
    return _available


def _aligned(*ts) -> int:
    return int(all(t.data_ptr() % 16 == 0 for t in ts if t is not None))


def run_groupby(spec, pred, plan, ws, n: int, stream: int, pred_tensors=(), key_tensors=(), col_tensors=()):
    """Accumulation pass of ops.groupby as a query-specialised kernel (table in ws)."""
    lib = L.load()
    src, name, T, smem = groupby_source(spec, pred.struct if pred is not None else None, plan)
    h = compile_kernel(src, name)
    a = _Args()
    if pred is not None:
        for c in range(pred.struct.n_cols):
            a.ptr(pred.struct.cols[c])
    for k in range(spec.n_keys):
        a.ptr(spec.keys[k])
    for c in range(spec.n_cols):
        a.ptr(spec.cols[c])
    a.i64(n)
    a.ptr(lib.tqpk_groupby_table(ws.data_ptr()))
    a.i32(_aligned(*pred_tensors) if pred is not None else 1)
    a.i32(_aligned(*key_tensors))
    a.i32(_aligned(*col_tensors))
    grid = occupancy_grid(h, T, smem, (n + 3) // 4)
    launch(h, grid, T, smem, a, stream, L.KID_GROUPBY)


def probe_supported(fk_dtype_code: int) -> bool:
    return fk_dtype_code in (L.I32, L.I64)


def _hexf(x: float) -> str:
    return f"({float(x).hex()})" if x == x and abs(x) != float("inf") else (
        "__longlong_as_double(0x%016xLL)" % struct.unpack("<Q", struct.pack("<d", x))[0])


def _hexf32(x: float) -> str:
    import numpy as np
    return "__int_as_float(0x%08x)" % struct.unpack("<I", struct.pack("<f", np.float32(x)))[0]


def check_compiles(src: str) -> Tuple[bool, str]:
    """Compiles without loading (works without a GPU): (ok, log)."""
    log = C.create_string_buffer(1 << 16)
    rc = L.load().tqpk_jit_check(src.encode(), log, len(log))
    return rc == 0, log.value.decode(errors="replace")


def compile_kernel(src: str, name: str) -> int:
    key = hashlib.sha256((name + "\0" + src).encode()).hexdigest()
    with _lock:
        h = _cache.get(key)
        if h is not None:
            return h
        handle = C.c_void_p()
        log = C.create_string_buffer(1 << 16)
        rc = L.load().tqpk_jit_compile(src.encode(), name.encode(), C.byref(handle), log, len(log))
        if rc != 0:
            raise RuntimeError(f"query kernel compile failed ({rc}): {log.value.decode(errors='replace')[:2000]}")
        _cache[key] = handle.value
        return handle.value


class _Args:
    """Kernel parameters for cudaLaunchKernel (keeps the ctypes values alive)."""

    def __init__(self):
        self.vals: List = []

    def ptr(self, p):
        self.vals.append(C.c_void_p(p))

    def i64(self, v):
        self.vals.append(C.c_int64(int(v)))

    def i32(self, v):
        self.vals.append(C.c_int32(int(v)))

    def array(self):
        arr = (C.c_void_p * len(self.vals))()
        for i, v in enumerate(self.vals):
            arr[i] = C.cast(C.pointer(v), C.c_void_p)
        return arr


def launch(handle: int, grid: int, block: int, smem: int, args: _Args, stream: int, timing_kid: int = 0):
    arr = args.array()
    L.check(L.load().tqpk_jit_launch(handle, grid, block, smem, arr, timing_kid, stream), "tqpk_jit_launch")


def occupancy_grid(handle: int, block: int, smem: int, work_units: int) -> int:
    lib = L.load()
    per_sm = max(1, lib.tqpk_jit_occupancy(handle, block, smem))
    g = (work_units + block - 1) // block
    return max(1, min(g, per_sm * lib.tqpk_num_sms()))


# ---------------------------------------------------------------------------- code pieces
def _pred_code(P, prefix: str) -> Tuple[List[int], str]:
    """Boolean C++ expression of row j for a tqpk_predicate; returns (column slots used, code)."""
    st: List[str] = []
    used = set()
    for k in range(P.n_insn):
        I = P.insn[k]
        if I.op == L.P_CMP:
            used.add(I.col)
            x = f"{prefix}{I.col}.v[j]"
            dt = P.dtypes[I.col]
            if I.cmp == L.ISCLOSE:
                st.append(f"iscl({x}, {_hexf(I.lit_f)}, {_hexf(I.lit_aux)})")
            elif I.domain == L.DOM_F64:
                xx = x if dt == L.F64 else f"(double){x}"
                st.append(f"({xx} {_CMP_OP[I.cmp]} {_hexf(I.lit_f)})")
            elif I.domain == L.DOM_F32:
                st.append(f"((float){x} {_CMP_OP[I.cmp]} {_hexf32(I.lit_f)})")
            else:
                st.append(f"((i64){x} {_CMP_OP[I.cmp]} ({I.lit_i}LL))")
        elif I.op == L.P_CMPCOL:
            used.add(I.col)
            used.add(int(I.lit_i))
            a, b = f"{prefix}{I.col}.v[j]", f"{prefix}{int(I.lit_i)}.v[j]"
            t = "double" if I.domain == L.DOM_F64 else "i64"
            st.append(f"(({t}){a} {_CMP_OP[I.cmp]} ({t}){b})")
        elif I.op == L.P_MASK:
            used.add(I.col)
            st.append(f"({prefix}{I.col}.v[j] != 0)")
        elif I.op == L.P_TRUE:
            st.append("true")
        elif I.op == L.P_FALSE:
            st.append("false")
        elif I.op == L.P_NOT:
            st.append(f"(!{st.pop()})")
        else:
            b, a = st.pop(), st.pop()
            st.append(f"({a} {'&&' if I.op == L.P_AND else '||'} {b})")
    return sorted(used), (st[0] if st else "true")


def _expr_code(S, upto: int, colpfx: str) -> Tuple[List[int], List[str]]:
    """Statements computing registers r0..r{upto-1} for row j; returns (columns used, lines)."""
    lines, used = [], set()
    for i in range(upto):
        X = S.expr[i]
        f = X.type == L.F64
        t = "double" if f else "i64"
        if X.op == L.X_COL:
            used.add(X.col)
            src = f"{colpfx}{X.col}.v[j]"
            lines.append(f"const {t} r{i} = ({t}){src};")
        elif X.op == L.X_CONST:
            lines.append(f"const {t} r{i} = {_hexf(X.cf) if f else str(int(X.ci)) + 'LL'};")
        elif X.op == L.X_TOF64:
            lines.append(f"const double r{i} = (double)r{X.a};")
        else:
            if f:
                fn = {L.X_ADD: "__dadd_rn", L.X_SUB: "__dsub_rn", L.X_MUL: "__dmul_rn", L.X_DIV: "__ddiv_rn"}[X.op]
                lines.append(f"const double r{i} = {fn}(r{X.a}, r{X.b});")
            else:
                op = {L.X_ADD: "+", L.X_SUB: "-", L.X_MUL: "*"}[X.op]
                lines.append(f"const i64 r{i} = r{X.a} {op} r{X.b};")
    return sorted(used), lines


def _load_lines(cols: Sequence[int], dtypes, pfx: str, ptr_pfx: str, n: str, vec: str) -> List[str]:
    return [f"const V4<{_CTYPE[dtypes[c]]}> {pfx}{c} = ld4((const {_CTYPE[dtypes[c]]}*){ptr_pfx}{c}, r0, {n}, {vec});"
            for c in cols]


def _acc_init(a) -> str:
    if a.kind in (L.ACC_MIN, L.ACC_MAX):
        if a.type == L.F64:
            import numpy as np
            u = struct.unpack("<Q", struct.pack("<d", a.init_f))[0]
            u = (~u & ((1 << 64) - 1)) if (u >> 63) else (u | (1 << 63))
            return f"0x{u:016x}ull"
        return f"(u64)({int(a.init_i)}LL)"
    return "0ull"


def _acc_value(a) -> str:
    """Accumulator encoding of this row's contribution (register r{reg})."""
    if a.kind == L.ACC_COUNT_ROWS:
        return "1ull"
    r = f"r{a.reg}"
    if a.kind == L.ACC_SUM:
        return f"d2u({r})" if a.type == L.F64 else f"(u64){r}"
    if a.kind == L.ACC_COUNT_NOTNULL:
        return f"(u64)({r} != -64.0)" if a.type == L.F64 else f"(u64)({r} != -64LL)"
    return f"ford({r})" if a.type == L.F64 else f"(u64){r}"


def _combine(a, x: str, y: str) -> str:
    if a.kind == L.ACC_SUM:
        return f"d2u(__dadd_rn(u2d({x}), u2d({y})))" if a.type == L.F64 else f"({x} + {y})"
    if a.kind in (L.ACC_COUNT_ROWS, L.ACC_COUNT_NOTNULL):
        return f"({x} + {y})"
    fn = "min" if a.kind == L.ACC_MIN else "max"
    return f"{fn}({x}, {y})" if a.type == L.F64 else f"(u64){fn}((i64)({x}), (i64)({y}))"


def _merge_atomic(a, p: str, v: str) -> str:
    if a.kind == L.ACC_SUM:
        return (f"atomicAdd((double*)({p}), u2d({v}));" if a.type == L.F64
                else f"atomicAdd((unsigned long long*)({p}), (unsigned long long)({v}));")
    if a.kind in (L.ACC_COUNT_ROWS, L.ACC_COUNT_NOTNULL):
        return f"atomicAdd((unsigned long long*)({p}), (unsigned long long)({v}));"
    fn = "atomicMin" if a.kind == L.ACC_MIN else "atomicMax"
    return (f"{fn}((unsigned long long*)({p}), (unsigned long long)({v}));" if a.type == L.F64
            else f"{fn}((long long*)({p}), (long long)({v}));")


# ---------------------------------------------------------------------------- group-by accumulation
def groupby_source(spec, pred, plan) -> Tuple[str, str, int, int]:
    """CUDA source of the filter + group-by accumulation for one query.

    Returns (source, kernel name, threads, dynamic shared bytes).  The table
    layout ([n_accs][slots] in the plan's workspace) and encodings are the
    interpreting kernel's, so the library's count/emit stages read it."""
    S = spec
    A, K = S.n_accs, int(plan.slots)
    private = plan.mode in (L.GB_DENSE_PRIVATE, L.GB_GLOBAL_ONE)
    T = int(plan.threads) if private else 256
    smem = K * A * 8 * T if private else 0
    pcols, pexpr = _pred_code(pred, "p") if pred is not None else ([], "true")
    ecols, elines = _expr_code(S, S.n_expr, "c")
    kcols = list(range(S.n_keys))
    name = "tqpk_q_groupby"
    src = [PRELUDE, f'extern "C" __global__ void __launch_bounds__({T}) {name}(']
    params = [f"const void* __restrict__ pp{c}" for c in range(pred.n_cols if pred is not None else 0)]
    params += [f"const void* __restrict__ kp{k}" for k in kcols]
    params += [f"const void* __restrict__ cp{c}" for c in range(S.n_cols)]
    params += ["i64 n", "u64* __restrict__ gacc", "int vp", "int vk", "int vc"]
    src.append("    " + ",\n    ".join(params) + ") {")
    src.append(f"  constexpr int T = {T}; constexpr int A = {A}; constexpr i64 K = {K}LL;")
    if private:
        src.append("  extern __shared__ u64 sm[];")
        inits = " : ".join(f"(a == {i}) ? {_acc_init(S.accs[i])}" for i in range(A)) + " : 0ull"
        src.append(f"  for (i64 i = threadIdx.x; i < K * A * T; i += T) {{ const int a = (int)((i / T) % A); sm[i] = {inits}; }}")
        src.append("  __syncthreads();")
    src.append("  const i64 groups = (n + 3) >> 2;")
    src.append("  for (i64 g = blockIdx.x * (i64)T + threadIdx.x; g < groups; g += (i64)gridDim.x * T) {")
    src.append("    const i64 r0 = g << 2;")
    if pred is not None:
        src += ["    " + l for l in _load_lines(pcols, pred.dtypes, "P", "pp", "n", "vp != 0")]
    src += ["    " + l for l in _load_lines(kcols, S.key_dtypes, "Kc", "kp", "n", "vk != 0")]
    src += ["    " + l for l in _load_lines(ecols, S.col_dtypes, "Cv", "cp", "n", "vc != 0")]
    src.append("#pragma unroll")
    src.append("    for (int j = 0; j < 4; ++j) {")
    src.append("      if (r0 + j >= n) break;")
    src.append(f"      if (!({_rename(pexpr, 'p', 'P')})) continue;")
    slot = " + ".join(f"((i64)Kc{k}.v[j] - ({int(plan.key_min[k])}LL)) * {int(plan.key_stride[k])}LL" for k in kcols) or "0"
    src.append(f"      const i64 slot = {slot};")
    src += ["      " + _rename(l, "c", "Cv") for l in elines]
    for a in range(A):
        acc = S.accs[a]
        v = _acc_value(acc)
        if private:
            cell = f"sm[(slot * A + {a}) * T + threadIdx.x]"
            src.append(f"      {cell} = {_combine(acc, cell, v)};")
        else:
            src.append("      " + _merge_atomic(acc, f"&gacc[{a} * K + slot]", v))
    src.append("    }")
    src.append("  }")
    if private:
        src.append("  __syncthreads();")
        src.append("  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;")
        src.append("  for (i64 c = warp; c < K * A; c += T / 32) {")
        src.append("    const int a = (int)(c % A); const i64 s = c / A;")
        src.append("    switch (a) {")
        for a in range(A):
            acc = S.accs[a]
            init = _acc_init(acc)
            src.append(f"    case {a}: {{")
            src.append(f"      u64 v = {init};")
            src.append(f"      for (int t = lane; t < T; t += 32) v = {_combine(acc, 'v', 'sm[c * T + t]')};")
            src.append("      for (int o = 16; o; o >>= 1) { const u64 w = __shfl_xor_sync(0xffffffffu, v, o); "
                       f"v = {_combine(acc, 'v', 'w')}; }}")
            src.append(f"      if (lane == 0 && v != {init}) {_merge_atomic(acc, f'&gacc[{a} * K + s]', 'v')}")
            src.append("      break; }")
        src.append("    }")
        src.append("  }")
    src.append("}")
    return "\n".join(src), name, T, smem


def _rename(code: str, old_prefix: str, new_prefix: str) -> str:
    """Renames the tile variables of a code piece (p0 -> P0, c3 -> Cv3)."""
    import re
    return re.sub(rf"\b{old_prefix}(\d+)\.v\[j\]", rf"{new_prefix}\1.v[j]", code)


# ---------------------------------------------------------------------------- fused join probe
def join_probe_source(spec, val_reg: int, pred) -> Tuple[str, str]:
    """CUDA source of the fused probe + aggregate (directory lookup, value, FP64 sum, occupancy)."""
    S = spec
    pcols, pexpr = _pred_code(pred, "p") if pred is not None else ([], "true")
    ecols, elines = _expr_code(S, val_reg + 1, "c")
    vt = "double" if S.expr[val_reg].type == L.F64 else "i64"
    name = "tqpk_q_join_probe"
    params = [f"const void* __restrict__ pp{c}" for c in range(pred.n_cols if pred is not None else 0)]
    params += [f"const void* __restrict__ cp{c}" for c in range(S.n_cols)]
    params += ["const void* __restrict__ fk", "int fk_dt", "i64 np", "i64 key_min", "i64 slots",
               "const int* __restrict__ dir", "double* __restrict__ sum", "u32* __restrict__ occ",
               "int vp", "int vc", "int vf"]
    fk_load = ("const V4<i64> F = (fk_dt == 4) ? ld4((const long long*)fk, r0, np, vf != 0) : "
               "[&]{ V4<int> t = ld4((const int*)fk, r0, np, vf != 0); V4<i64> o; "
               "for (int q = 0; q < 4; ++q) o.v[q] = t.v[q]; return o; }();")
    src = [PRELUDE, f'extern "C" __global__ void __launch_bounds__(256) {name}(', "    " + ",\n    ".join(params) + ") {",
           "  const i64 n8 = (np + 7) >> 3;",
           "  for (i64 g = blockIdx.x * (i64)blockDim.x + threadIdx.x; g < n8; g += (i64)gridDim.x * blockDim.x) {",
           "    i64 sl[2][4]; unsigned m[2];",
           "#pragma unroll",
           "    for (int u = 0; u < 2; ++u) {",
           "      const i64 r0 = ((g << 1) + u) << 2;",
           "      m[u] = 0;",
           "      if (r0 >= np) continue;"]
    src += ["      " + l for l in _load_lines(pcols, pred.dtypes, "P", "pp", "np", "vp != 0")] if pred is not None else []
    src += ["      " + fk_load,
            "#pragma unroll",
            "      for (int j = 0; j < 4; ++j) {",
            "        sl[u][j] = F.v[j] - key_min;",
            f"        const bool ok = (r0 + j < np) && ({_rename(pexpr, 'p', 'P')}) && sl[u][j] >= 0 && sl[u][j] < slots;",
            "        m[u] |= (unsigned)ok << j;",
            "      }",
            "    }",
            "#pragma unroll",
            "    for (int u = 0; u < 2; ++u)",
            "#pragma unroll",
            "      for (int j = 0; j < 4; ++j)",
            "        if (((m[u] >> j) & 1u) && __ldg(&dir[sl[u][j]]) < 0) m[u] &= ~(1u << j);",
            "#pragma unroll",
            "    for (int u = 0; u < 2; ++u) {",
            "      if (!m[u]) continue;",
            "      const i64 r0 = ((g << 1) + u) << 2;"]
    src += ["      " + l for l in _load_lines(ecols, S.col_dtypes, "Cv", "cp", "np", "vc != 0")]
    src += ["#pragma unroll", "      for (int j = 0; j < 4; ++j) {", "        if (!((m[u] >> j) & 1u)) continue;"]
    src += ["        " + _rename(l, "c", "Cv") for l in elines]
    src += [f"        atomicAdd(&sum[sl[u][j]], (double)r{val_reg});", "        occ[sl[u][j]] = 1u;",
            "      }", "    }", "  }", "}"]
    return "\n".join(src), name
