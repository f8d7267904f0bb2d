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
// an opaque move: integer tests on a double's bits stay integer (a plain reinterpretation lets the
// compiler fold them into FP64 compares, which run at 1/64 rate on this part)
__device__ __forceinline__ u64 d2u(double d) { u64 u; asm("mov.b64 %0, %1;" : "=l"(u) : "d"(d)); return u; }
__device__ __forceinline__ double u2d(u64 u) { return __longlong_as_double((long long)u); }
__device__ __forceinline__ u64 ford(double d) { u64 u = d2u(d); return (u >> 63) ? ~u : (u | (1ull << 63)); }
__device__ __forceinline__ bool iscl(double x, double lit, double allowed) {
  double e = fabs(__dsub_rn(x, lit));
  return (x == lit) || (isfinite(e) && e <= allowed);
}
// reductions into global memory whose result nobody reads: `red.global`, applied at the L2 without a
// reply.  An atomicAdd through a pointer the compiler cannot place in global memory (a table pointer
// loaded from a descriptor) becomes a generic atomic that returns its old value, and the warp waits
// for the round trip.
__device__ __forceinline__ void gred_add(double* p, double v) {
  asm volatile("red.global.add.f64 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "d"(v) : "memory");
}
__device__ __forceinline__ void gred_add(u64* p, u64 v) {
  asm volatile("red.global.add.u64 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
__device__ __forceinline__ void gred_add(unsigned* p, unsigned v) {
  asm volatile("red.global.add.u32 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "r"(v) : "memory");
}
__device__ __forceinline__ void gred_min(u64* p, u64 v) {
  asm volatile("red.global.min.u64 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
__device__ __forceinline__ void gred_max(u64* p, u64 v) {
  asm volatile("red.global.max.u64 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
__device__ __forceinline__ void gred_min(i64* p, i64 v) {
  asm volatile("red.global.min.s64 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
__device__ __forceinline__ void gred_max(i64* p, i64 v) {
  asm volatile("red.global.max.s64 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
// bulk copies (TMA, 1-D) into shared memory, completed on an mbarrier
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(smem_u32(b)), "r"(parity) : "memory");
  return ok != 0;
}
// Year of day d (days since 1990-01-01): 1990 before that day, else the proleptic
// Gregorian year by H. Hinnant's civil_from_days (400-year eras of 146097 days).
__device__ __forceinline__ i64 tqpk_year(i64 d) {
  if (d < 0) return 1990;
  const i64 z = d + 7305 + 719468, era = z / 146097, doe = z - era * 146097;
  const i64 yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  const i64 doy = doe - (365 * yoe + yoe / 4 - yoe / 100), mp = (5 * doy + 2) / 153;
  return yoe + era * 400 + (mp >= 10 ? 1 : 0);
}
// 16-byte asynchronous global -> shared copy (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}
// read-only loads that leave L1 to other data (a lookup structure the kernel keeps there)
__device__ __forceinline__ int ld_na(const int* p) {
  int v; asm("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(p)); return v;
}
__device__ __forceinline__ long long ld_na(const long long* p) {
  long long v; asm("ld.global.nc.L1::no_allocate.b64 %0, [%1];" : "=l"(v) : "l"(p)); return v;
}
__device__ __forceinline__ double ld_na(const double* p) {
  double v; asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p)); return v;
}
// predicate literals, bound at launch (one compiled kernel serves every constant)
struct PL { long long i[32]; double f[32]; double a[32]; };
template <class T> struct V4 { T v[4]; };
// column stream loads; a kernel source may define TQPK_LD as __ldcs (evict-first) so the
// streamed columns do not push directories and group tables out of L2
#ifndef TQPK_LD
#define TQPK_LD(p) (*(p))
#endif
// four consecutive rows r0..r0+3 (r0 % 4 == 0); rows >= n read as 0
__device__ __forceinline__ V4<double> ld4(const double* p, i64 r0, i64 n, bool vec) {
  V4<double> o;
  if (vec && r0 + 4 <= n) {
    const double2* q = reinterpret_cast<const double2*>(p + r0);
    double2 a = TQPK_LD(q), b = TQPK_LD(q + 1);
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
    longlong2 a = TQPK_LD(q), b = TQPK_LD(q + 1);
    o.v[0] = a.x; o.v[1] = a.y; o.v[2] = b.x; o.v[3] = b.y;
  } else {
    for (int j = 0; j < 4; ++j) o.v[j] = (r0 + j < n) ? p[r0 + j] : 0;
  }
  return o;
}
__device__ __forceinline__ V4<int> ld4(const int* p, i64 r0, i64 n, bool vec) {
  V4<int> o;
  if (vec && r0 + 4 <= n) {
    int4 a = TQPK_LD(reinterpret_cast<const int4*>(p + r0));
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
    unsigned w = TQPK_LD(reinterpret_cast<const unsigned*>(p + r0));
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


_gb_memo: Dict[bytes, Tuple[int, int, int]] = {}


def _shape_key(*structs) -> bytes:
    """The bytes of ctypes structs with their pointer arrays cleared: what a generated
    kernel's source depends on (pointers and literals are launch arguments)."""
    out = []
    for st in structs:
        if st is None:
            out.append(b"-")
            continue
        c = type(st).from_buffer_copy(st)
        for fname, ftype in type(st)._fields_:
            if fname in ("cols", "keys", "n_rows", "ws_bytes", "key_range"):   # pointers, plan sizes
                setattr(c, fname, ftype())
            elif fname == "insn" and isinstance(st, L.Predicate):  # comparison literals are bound at launch
                for i in range(c.n_insn):
                    if c.insn[i].op == L.P_CMP:
                        c.insn[i].lit_i, c.insn[i].lit_f, c.insn[i].lit_aux = 0, 0.0, 0.0
        out.append(bytes(c))
    return b"|".join(out)


def run_groupby(spec, pred, plan, ws, n: int, stream: int, pred_tensors=(), key_tensors=(), col_tensors=(),
                err_ptr=None):
    """Accumulation pass of ops.groupby as a query-specialised kernel (table in ws).  The
    generated kernel is looked up by the shape of the spec, predicate and plan, so a
    repeated query shape skips the source generation."""
    lib = L.load()
    key = _shape_key(spec, pred.struct if pred is not None else None, plan)
    hit = _gb_memo.get(key)
    if hit is None:
        src, name, T, smem = groupby_source(spec, pred.struct if pred is not None else None, plan)
        hit = (compile_kernel(src, name), T, smem)
        _gb_memo[key] = hit
    h, T, smem = hit
    a = _Args()
    if pred is not None:
        for c in range(pred.struct.n_cols):
            a.ptr(pred.struct.cols[c])
    a.blob(pred_lits(pred.struct if pred is not None else None))
    for k in range(spec.n_keys):
        a.ptr(spec.keys[k])
    for c in range(spec.n_cols):
        a.ptr(spec.cols[c])
    a.i64(n)
    a.ptr(lib.tqpk_groupby_table(ws.data_ptr()))
    a.i32(_aligned(*pred_tensors) if pred is not None else 1)
    a.i32(_aligned(*key_tensors))
    a.i32(_aligned(*col_tensors))
    a.ptr(err_ptr)
    grid = occupancy_grid(h, T, smem, (n + 3) // 4)
    launch(h, grid, T, smem, a, stream, L.KID_GROUPBY)


def probe_supported(fk_dtype_code: int) -> bool:
    return fk_dtype_code in (L.I32, L.I64)


def _hexf(x: float) -> str:
    return f"({float(x).hex()})" if x == x and abs(x) != float("inf") else (
        "__longlong_as_double(0x%016xLL)" % struct.unpack("<Q", struct.pack("<d", x))[0])


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


class PredLits(C.Structure):
    """The literals of a predicate program (struct PL of the generated code)."""
    _fields_ = [("i", C.c_int64 * 32), ("f", C.c_double * 32), ("a", C.c_double * 32)]


def pred_lits(P) -> PredLits:
    out = PredLits()
    if P is not None:
        for k in range(P.n_insn):
            out.i[k], out.f[k], out.a[k] = P.insn[k].lit_i, P.insn[k].lit_f, P.insn[k].lit_aux
    return out


class _Args:
    """Kernel parameters for cudaLaunchKernel (keeps the ctypes values alive)."""

    def __init__(self):
        self.vals: List = []

    def blob(self, v):
        """A by-value struct parameter (a ctypes Structure)."""
        self.vals.append(v)

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


_occ_cache: Dict[Tuple[int, int, int], int] = {}


def occupancy_grid(handle: int, block: int, smem: int, work_units: int) -> int:
    """Blocks for work_units threads, capped at one full wave (resident CTAs per SM, from the
    occupancy API once per kernel and launch shape, x SMs)."""
    key = (handle, block, smem)
    cap = _occ_cache.get(key)
    if cap is None:
        lib = L.load()
        cap = _occ_cache[key] = max(1, lib.tqpk_jit_occupancy(handle, block, smem)) * lib.tqpk_num_sms()
    g = (work_units + block - 1) // block
    return max(1, min(g, cap))


# ---------------------------------------------------------------------------- code pieces
def _pred_code(P, prefix: str, lits: str = "lp") -> Tuple[List[int], str]:
    """Boolean C++ expression of row j for a tqpk_predicate; returns (column slots used, code).

    Comparison literals are read from the kernel's PL parameter `lits`
    (instruction k's literal at index k), so the compiled kernel depends on
    the predicate's shape only and each launch binds its own constants."""
    st: List[str] = []
    used = set()
    for k in range(P.n_insn):
        I = P.insn[k]
        if I.op == L.P_CMP:
            used.add(I.col)
            x = f"{prefix}{I.col}.v[j]"
            dt = P.dtypes[I.col]
            if I.cmp == L.ISCLOSE:
                st.append(f"iscl({x}, {lits}.f[{k}], {lits}.a[{k}])")
            elif I.domain == L.DOM_F64:
                xx = x if dt == L.F64 else f"(double){x}"
                st.append(f"({xx} {_CMP_OP[I.cmp]} {lits}.f[{k}])")
            elif I.domain == L.DOM_F32:
                st.append(f"((float){x} {_CMP_OP[I.cmp]} __double2float_rn({lits}.f[{k}]))")
            else:
                st.append(f"((i64){x} {_CMP_OP[I.cmp]} {lits}.i[{k}])")
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


def _reg_uses(S) -> Dict[int, int]:
    """How many expression operands and accumulators read each register."""
    uses: Dict[int, int] = {}
    for i in range(S.n_expr):
        X = S.expr[i]
        if X.op in (L.X_ADD, L.X_SUB, L.X_MUL, L.X_DIV, L.X_SELECT):
            uses[X.a] = uses.get(X.a, 0) + 1
            uses[X.b] = uses.get(X.b, 0) + 1
        if X.op in (L.X_TOF64, L.X_YEAR):
            uses[X.a] = uses.get(X.a, 0) + 1
        if X.op == L.X_SELECT:
            uses[X.col] = uses.get(X.col, 0) + 1
    for a in range(S.n_accs):
        if S.accs[a].kind != L.ACC_COUNT_ROWS:
            uses[S.accs[a].reg] = uses.get(S.accs[a].reg, 0) + 1
    return uses


def _one_minus(S, r: int) -> Optional[int]:
    """b when register r is the F64 (1.0 - r_b), else None."""
    X = S.expr[r]
    if X.op != L.X_SUB or X.type != L.F64:
        return None
    one = S.expr[X.a]
    if one.op != L.X_CONST or one.type != L.F64 or one.cf != 1.0:
        return None
    return X.b


def _contractions(S, upto: int) -> Dict[int, Tuple[int, int]]:
    """F64 products x * (1.0 - y) whose (1.0 - y) is read by nothing else: {register: (x, y, the
    (1.0 - y) register)}.
    The group-by evaluates them as fma(-x, y, x), x - x*y rounded once, where the plain form
    rounds (1 - y) and the product: within an ulp of the term, and one FP64 instruction fewer
    per row on the FP64-bound accumulation (the sums are compared at 1e-12 relative).  Per-row
    results (projections, join values) keep the plain form."""
    uses = _reg_uses(S)
    into_acc = {S.accs[a].reg for a in _fusable_products(S)}   # those become fma(x, t, acc) instead
    out = {}
    for i in range(upto):
        X = S.expr[i]
        if X.op != L.X_MUL or X.type != L.F64 or i in into_acc:
            continue
        for x, t in ((X.a, X.b), (X.b, X.a)):
            y = _one_minus(S, t)
            if y is not None and uses.get(t, 0) == 1 and t < i and x < i:
                out[i] = (x, y, t)
                break
    return out


def _expr_code(S, upto: int, colpfx: str, contract: bool = False) -> Tuple[List[int], List[str]]:
    """Statements computing registers r0..r{upto-1} for row j; returns (columns used, lines).
    contract: products x * (1 - y) as one fused multiply-add (see _contractions)."""
    lines, used = [], set()
    fused = _contractions(S, upto) if contract else {}
    skip = {t for (_, _, t) in fused.values()}
    for i in range(upto):
        X = S.expr[i]
        if i in skip:
            continue                  # (1 - y), folded into the fused multiply-add that reads it
        if i in fused:
            x, y, _ = fused[i]
            lines.append(f"const double r{i} = __fma_rn(-r{x}, r{y}, r{x});")
            continue
        if X.type == L.F32:          # float32 register: torch's default float dtype, round-to-nearest
            if X.op == L.X_CONST:            # the Python number cast to float32, as torch does
                lines.append(f"const float r{i} = __double2float_rn({_hexf(X.cf)});")
            elif X.op == L.X_TOF32:
                lines.append(f"const float r{i} = __ll2float_rn(r{X.a});")
            elif X.op == L.X_SELECT:
                lines.append(f"const float r{i} = r{X.a} != 0 ? r{X.b} : r{X.col};")
            else:
                fn = {L.X_ADD: "__fadd_rn", L.X_SUB: "__fsub_rn", L.X_MUL: "__fmul_rn", L.X_DIV: "__fdiv_rn"}[X.op]
                lines.append(f"const float r{i} = {fn}(r{X.a}, r{X.b});")
            continue
        if X.op == L.X_F32TOF64:
            lines.append(f"const double r{i} = (double)r{X.a};")
            continue
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
        elif X.op == L.X_SELECT:
            lines.append(f"const {t} r{i} = r{X.a} != 0 ? r{X.b} : r{X.col};")
        elif X.op == L.X_YEAR:
            lines.append(f"const i64 r{i} = tqpk_year(r{X.a});")
        else:
            if f:
                fn = {L.X_ADD: "__dadd_rn", L.X_SUB: "__dsub_rn", L.X_MUL: "__dmul_rn", L.X_DIV: "__ddiv_rn"}[X.op]
                lines.append(f"const double r{i} = {fn}(r{X.a}, r{X.b});")
            else:
                op = {L.X_ADD: "+", L.X_SUB: "-", L.X_MUL: "*"}[X.op]
                cast = {L.I8: "(signed char)", L.U8: "(unsigned char)", L.I32: "(int)"}.get(X.wrap, "")
                expr = f"(u64)r{X.a} {op} (u64)r{X.b}" if X.op != L.X_MUL else f"r{X.a} {op} r{X.b}"
                lines.append(f"const i64 r{i} = (i64){cast}({expr});" if cast else f"const i64 r{i} = r{X.a} {op} r{X.b};")
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


def _merge_atomic(a, p: str, v: str, glob: bool = False) -> str:
    """Atomic merge of v (accumulator encoding) into the cell at p; glob: p is in global memory and
    the merge is a reduction without a reply (the shared-memory tables keep the atomics)."""
    if glob:
        if a.kind == L.ACC_SUM and a.type == L.F64:
            return f"gred_add((double*)({p}), u2d({v}));"
        if a.kind in (L.ACC_SUM, L.ACC_COUNT_ROWS, L.ACC_COUNT_NOTNULL):
            return f"gred_add((u64*)({p}), (u64)({v}));"
        fn = "gred_min" if a.kind == L.ACC_MIN else "gred_max"
        return f"{fn}((u64*)({p}), (u64)({v}));" if a.type == L.F64 else f"{fn}((i64*)({p}), (i64)({v}));"
    if a.kind == L.ACC_SUM:
        return (f"atomicAdd((double*)({p}), u2d({v}));" if a.type == L.F64
                else f"atomicAdd((unsigned long long*)({p}), (unsigned long long)({v}));")
    if a.kind in (L.ACC_COUNT_ROWS, L.ACC_COUNT_NOTNULL):
        return f"atomicAdd((unsigned long long*)({p}), (unsigned long long)({v}));"
    fn = "atomicMin" if a.kind == L.ACC_MIN else "atomicMax"
    return (f"{fn}((unsigned long long*)({p}), (unsigned long long)({v}));" if a.type == L.F64
            else f"{fn}((long long*)({p}), (long long)({v}));")


def _fusable_products(S) -> Dict[int, Tuple[int, int]]:
    """Float sum accumulators whose value is an F64 product read by nothing else: {acc:
    (x, y)}.  Accumulating it as fma(x, y, acc) rounds once where the product + add round
    twice (0.5 ulp of the term; the sums are compared at 1e-12 relative), and saves one
    FP64 instruction per row on the FP64-bound group-by."""
    uses = _reg_uses(S)
    out = {}
    for a in range(S.n_accs):
        acc = S.accs[a]
        if acc.kind != L.ACC_SUM or acc.type != L.F64:
            continue
        X = S.expr[acc.reg]
        if X.op == L.X_MUL and X.type == L.F64 and uses.get(acc.reg, 0) == 1:
            out[a] = (X.a, X.b)
    return out


# ---------------------------------------------------------------------------- group-by accumulation
def groupby_source(spec, pred, plan) -> Tuple[str, str, int, int]:
    """CUDA source of the filter + group-by accumulation for one query.

    Returns (source, kernel name, threads, dynamic shared bytes).  The table
    layout ([n_accs][slots] in the plan's workspace) and encodings are the
    interpreting kernel's, so the library's count/emit stages read it."""
    S = spec
    A, K = S.n_accs, int(plan.slots)
    private = plan.mode in (L.GB_DENSE_PRIVATE, L.GB_GLOBAL_ONE)
    shared = plan.mode == L.GB_DENSE_SHARED          # one table per CTA, shared-memory atomics
    T = int(plan.threads) if private else 256
    smem = K * A * 8 * T if private else (K * A * 8 if shared else 0)
    pcols, pexpr = _pred_code(pred, "p") if pred is not None else ([], "true")
    ecols, elines = _expr_code(S, S.n_expr, "c", contract=True)
    kcols = list(range(S.n_keys))
    name = "tqpk_q_groupby"
    src = [PRELUDE, f'extern "C" __global__ void __launch_bounds__({T}) {name}(']
    params = [f"const void* __restrict__ pp{c}" for c in range(pred.n_cols if pred is not None else 0)]
    params += ["const PL lp"]
    params += [f"const void* __restrict__ kp{k}" for k in kcols]
    params += [f"const void* __restrict__ cp{c}" for c in range(S.n_cols)]
    params += ["i64 n", "u64* __restrict__ gacc", "int vp", "int vk", "int vc", "int* __restrict__ err"]
    src.append("    " + ",\n    ".join(params) + ") {")
    src.append(f"  constexpr int T = {T}; constexpr int A = {A}; constexpr i64 K = {K}LL;")
    inits = " : ".join(f"(a == {i}) ? {_acc_init(S.accs[i])}" for i in range(A)) + " : 0ull"
    if private:
        src.append("  extern __shared__ u64 sm[];")
        src.append(f"  for (i64 i = threadIdx.x; i < K * A * T; i += T) {{ const int a = (int)((i / T) % A); sm[i] = {inits}; }}")
        src.append("  __syncthreads();")
    elif shared:
        src.append("  extern __shared__ u64 sm[];")
        src.append(f"  for (i64 i = threadIdx.x; i < K * A; i += T) {{ const int a = (int)(i % A); sm[i] = {inits}; }}")
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
    # a key outside the plan's domain (key domains given as table statistics) would index past
    # the table: the row is skipped and TQPK_EINVAL recorded in *err (when given)
    if kcols:
        src.append("      if (" + " || ".join(f"(u64)((i64)Kc{k}.v[j] - ({int(plan.key_min[k])}LL)) >= "
                                              f"{int(plan.key_range[k])}ull" for k in kcols)
                   + ") { if (err) atomicCAS(err, 0, -1); continue; }")
    slot = " + ".join(f"((i64)Kc{k}.v[j] - ({int(plan.key_min[k])}LL)) * {int(plan.key_stride[k])}LL" for k in kcols) or "0"
    src.append(f"      const i64 slot = {slot};")
    src += ["      " + _rename(l, "c", "Cv") for l in elines]
    fused = _fusable_products(S) if private else {}
    for a in range(A):
        acc = S.accs[a]
        v = _acc_value(acc)
        if private:
            cell = f"sm[(slot * A + {a}) * T + threadIdx.x]"
            if a in fused:             # sum of a product used nowhere else: one fused multiply-add
                x, y = fused[a]
                src.append(f"      {cell} = d2u(__fma_rn(r{x}, r{y}, u2d({cell})));")
            else:
                src.append(f"      {cell} = {_combine(acc, cell, v)};")
        elif shared:
            src.append("      " + _merge_atomic(acc, f"&sm[slot * A + {a}]", v))
        else:
            src.append("      " + _merge_atomic(acc, f"&gacc[{a} * K + slot]", v, glob=True))
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
            src.append(f"      if (lane == 0 && v != {init}) {_merge_atomic(acc, f'&gacc[{a} * K + s]', 'v', glob=True)}")
            src.append("      break; }")
        src.append("    }")
        src.append("  }")
    elif shared:
        src.append("  __syncthreads();")
        src.append("  for (i64 c = threadIdx.x; c < K * A; c += T) {")
        src.append("    const int a = (int)(c % A); const i64 s = c / A; const u64 v = sm[c];")
        src.append("    switch (a) {")
        for a in range(A):
            acc = S.accs[a]
            src.append(f"    case {a}: if (v != {_acc_init(acc)}) {_merge_atomic(acc, f'&gacc[{a} * K + s]', 'v', glob=True)} break;")
        src.append("    }")
        src.append("  }")
    src.append("}")
    return "\n".join(src), name, T, smem


def _rename(code: str, old_prefix: str, new_prefix: str) -> str:
    """Renames the tile variables of a code piece (p0 -> P0, c3 -> Cv3)."""
    import re
    return re.sub(rf"\b{old_prefix}(\d+)\.v\[j\]", rf"{new_prefix}\1.v[j]", code)


# ---------------------------------------------------------------------------- fused join probe
def _gather_pred(pred, prefix: str, lits: str, ptr_pfx: str, row: str, live: str) -> Tuple[List[str], str]:
    """A predicate over dimension columns read through a row index (row[j], j live):
    (statements declaring the V4 tiles, boolean expression of row j)."""
    cols, expr = _pred_code(pred, prefix, lits)
    lines = []
    for c in cols:
        t = _CTYPE[pred.dtypes[c]]
        lines.append(f"V4<{t}> G{prefix}{c};")
        lines.append(f"for (int j = 0; j < 4; ++j) G{prefix}{c}.v[j] = (({live} >> j) & 1u) ? "
                     f"__ldg((const {t}*){ptr_pfx}{c} + {row}[j]) : ({t})0;")
    return lines, _rename(expr, prefix, "G" + prefix)


def _dense_tail(S, val_reg: int, ecols, elines, n: str, key: str, extra: List[str], U: int = 2,
                smem_vals: Optional[Dict[int, str]] = None, neg_zero_as_zero: bool = False,
                l1_no_allocate: bool = False, sum_stmt: Optional[str] = None) -> List[str]:
    """Warp-dense value pass: the warp's matched rows (queued as row offsets and
    slots in shared memory) are spread over all 32 lanes, so each FP64
    instruction and atomic runs with full lanes instead of the ~1 in 4 a
    row-per-lane loop leaves active after the predicate and the lookups.
    Each lane holds U groups of 4 rows; value column c is read from global
    memory, or from the shared-memory stage smem_vals[c] (indexed by the row's
    offset in the warp's 128 * U rows).  sum_stmt replaces the reduction of the value (the
    double `vz`) into sum[slot]."""
    import re
    lines = [f"    const unsigned nm = {' + '.join(f'__popc(m[{u}])' for u in range(U))};",
             "    unsigned incl = nm;",
             "#pragma unroll",
             "    for (int o = 1; o < 32; o <<= 1) { const unsigned t = __shfl_up_sync(0xffffffffu, incl, o); "
             "if (lane >= o) incl += t; }",
             "    const unsigned total = __shfl_sync(0xffffffffu, incl, 31);",
             "    unsigned pos = incl - nm;",
             "#pragma unroll",
             f"    for (int u = 0; u < {U}; ++u)",
             "#pragma unroll",
             "      for (int j = 0; j < 4; ++j)",
             f"        if ((m[u] >> j) & 1u) {{ q_off[wid][pos] = (lane * {4 * U} + u * 4 + j); "
             f"q_slot[wid][pos] = (int){key}[u][j]; ++pos; }}",
             "    __syncwarp();",
             "    for (unsigned i = lane; i < total; i += 32) {",
             "      const int off = q_off[wid][i];",
             "      const i64 row = wrow + off;",
             "      const i64 slot = q_slot[wid][i];"]
    for c in ecols:
        t = _CTYPE[S.col_dtypes[c]]
        if smem_vals is not None:
            lines.append(f"      const {t} Cs{c} = (({smem_vals[c]}))[off];")
        elif l1_no_allocate and S.col_dtypes[c] in (L.F64, L.I64, L.I32):
            lines.append(f"      const {t} Cs{c} = ld_na((const {t}*)cp{c} + row);")
        else:
            lines.append(f"      const {t} Cs{c} = __ldg((const {t}*)cp{c} + row);")
    for l in elines:
        lines.append("      " + re.sub(r"\bc(\d+)\.v\[j\]", r"Cs\1", l))
    if sum_stmt is not None:
        lines.append(f"      const double vz = (double)r{val_reg};")
        lines.append("      " + sum_stmt)
    elif neg_zero_as_zero:     # the sums start at -0.0 (the empty marker); add a -0.0 value as +0.0
        lines.append(f"      const double vz = (double)r{val_reg};")
        lines.append("      gred_add(&sum[slot], d2u(vz) == 0x8000000000000000ull ? 0.0 : vz);")
    else:
        lines.append(f"      gred_add(&sum[slot], (double)r{val_reg});")
    lines += ["      " + x for x in extra]
    lines += ["    }", "    __syncwarp();"]
    return lines


PROBE_U = 1          # 4-row groups per lane in the register probe: 4 rows, 32 registers, full occupancy


def probe_units(n: int) -> int:
    """Threads the register probes need for n rows (4 * PROBE_U rows per thread)."""
    return (int(n) + 4 * PROBE_U - 1) // (4 * PROBE_U)


def _stage_values(S, ecols, rows: int, n: str) -> Tuple[List[str], List[str], Dict[int, str]]:
    """Shared-memory stages of the value columns filled by cp.async (global -> shared,
    16-byte pieces, no registers held while the lookups are in flight): declarations,
    per-u copy statements (r0 = the 4-row group, sidx = its offset in the warp's rows),
    and the _dense_tail smem_vals map."""
    decl, copy, sv = [], [], {}
    for c in ecols:
        t = _CTYPE[S.col_dtypes[c]]
        es = {L.F64: 8, L.I64: 8, L.I32: 4}.get(S.col_dtypes[c])
        decl.append(f"  __shared__ __align__(16) {t} q_v{c}[8][{32 * rows}];")
        sv[c] = f"q_v{c}[wid]"
        if es is None:
            copy.append(f"for (int j = 0; j < 4; ++j) q_v{c}[wid][sidx + j] = (r0 + j < {n}) ? "
                        f"((const {t}*)cp{c})[r0 + j] : ({t})0;")
            continue
        pieces = 4 * es // 16
        copy.append(f"if (vc != 0 && r0 + 4 <= {n}) {{")
        for q in range(pieces):
            copy.append(f"  cp_async16(&q_v{c}[wid][sidx + {q * 16 // es}], (const {t}*)cp{c} + r0 + {q * 16 // es});")
        copy.append("} else {")
        copy.append(f"  for (int j = 0; j < 4; ++j) q_v{c}[wid][sidx + j] = (r0 + j < {n}) ? ((const {t}*)cp{c})[r0 + j] : ({t})0;")
        copy.append("}")
    return decl, copy, sv


def join_probe_source(spec, val_reg: int, pred, bpred=None, U: int = PROBE_U, min_blocks: int = 0,
                      stream_cs: bool = False, stage_vals: bool = False, occ_sentinel: bool = False,
                      dir_bits: bool = False) -> Tuple[str, str]:
    """CUDA source of the fused probe + aggregate (directory lookup, value, FP64 sum, occupancy).

    The directory holds build row indices (negative = no row).  `bpred`, when
    given, is a predicate over build-side columns evaluated through the row
    index (a resident directory serving queries with their own build filter).
    Each lane filters and looks up 4U consecutive rows (4-row vector loads);
    the warp then computes the value and updates the group of its matched rows
    densely (_dense_tail).  min_blocks > 0 asks the compiler for that many
    resident CTAs per SM (__launch_bounds__ register cap); stream_cs loads the
    probe columns with evict-first hints; stage_vals copies the value columns of
    every row to shared memory with cp.async at the top of the iteration (the
    value gather after the lookup leaves the dependent chain); occ_sentinel writes no
    occupancy word (the sums start at -0.0 and carry it; pipeline stage bit 3); dir_bits
    means `dir` is the build side's membership bitmap (tqpk_directory_bits; the group slot
    is the key, so membership is all the probe asks) and the value loads that are not
    staged bypass L1, which the bitmap keeps."""
    if dir_bits and bpred is not None:
        raise ValueError("a membership bitmap carries no build row for a probe-time build predicate")
    S = spec
    pcols, pexpr = _pred_code(pred, "p") if pred is not None else ([], "true")
    ecols, elines = _expr_code(S, val_reg + 1, "c")
    name = "tqpk_q_join_probe"
    params = [f"const void* __restrict__ pp{c}" for c in range(pred.n_cols if pred is not None else 0)]
    params += ["const PL lp"]
    if bpred is not None:
        params += [f"const void* __restrict__ bp{c}" for c in range(bpred.n_cols)]
        params += ["const PL lb"]
    params += [f"const void* __restrict__ cp{c}" for c in range(S.n_cols)]
    params += ["const void* __restrict__ fk", "int fk_dt", "i64 np", "i64 key_min", "i64 slots",
               "const unsigned* __restrict__ dir" if dir_bits else "const int* __restrict__ dir",
               "double* __restrict__ sum", "u32* __restrict__ occ", "int vp", "int vc", "int vf"]
    fk_load = ("const V4<i64> F = (fk_dt == 4) ? ld4((const long long*)fk, r0, np, vf != 0) : "
               "[&]{ V4<int> t = ld4((const int*)fk, r0, np, vf != 0); V4<i64> o; "
               "for (int q = 0; q < 4; ++q) o.v[q] = t.v[q]; return o; }();")
    rows = 4 * U                                   # rows per lane
    qt = "unsigned char" if 32 * rows <= 256 else "unsigned short"
    lb = f"256, {min_blocks}" if min_blocks else "256"
    hint = "#define TQPK_LD(p) __ldcs(p)\n" if stream_cs else ""
    sdecl, scopy, smem_vals = _stage_values(S, ecols, rows, "np") if stage_vals else ([], [], None)
    src = [hint + PRELUDE, f'extern "C" __global__ void __launch_bounds__({lb}) {name}(',
           "    " + ",\n    ".join(params) + ") {",
           f"  __shared__ {qt} q_off[8][{32 * rows}];",
           f"  __shared__ int q_slot[8][{32 * rows}];"] + sdecl + [
           "  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;",
           f"  const i64 nr = (np + {rows - 1}) / {rows};",
           "  const i64 stride = (i64)gridDim.x * blockDim.x;",
           "  for (i64 w0 = blockIdx.x * (i64)blockDim.x + (threadIdx.x & ~31); w0 < nr; w0 += stride) {",
           f"    const i64 g = w0 + lane, wrow = w0 * {rows};",
           f"    i64 sl[{U}][4]; int rw[{U}][4]; unsigned m[{U}];",
           "#pragma unroll",
           f"    for (int u = 0; u < {U}; ++u) {{",
           f"      const i64 r0 = g * {rows} + u * 4;",
           "      m[u] = 0;",
           "      if (r0 >= np) continue;"]
    if stage_vals:
        src += [f"      const int sidx = lane * {rows} + u * 4;"] + ["      " + l for l in scopy]
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
            f"    for (int u = 0; u < {U}; ++u)",
            "#pragma unroll",
            "      for (int j = 0; j < 4; ++j) {",
            ("        rw[u][j] = ((m[u] >> j) & 1u) ? (int)((__ldg(&dir[sl[u][j] >> 5]) >> (sl[u][j] & 31)) & 1u) - 1 : -1;"
             if dir_bits else "        rw[u][j] = ((m[u] >> j) & 1u) ? __ldg(&dir[sl[u][j]]) : -1;"),
            "        if (rw[u][j] < 0) m[u] &= ~(1u << j);",
            "      }"]
    if bpred is not None:
        glines, gexpr = _gather_pred(bpred, "b", "lb", "bp", "rw[u]", "m[u]")
        src += ["#pragma unroll", f"    for (int u = 0; u < {U}; ++u) {{", "      if (!m[u]) continue;"]
        src += ["      " + l for l in glines]
        src += ["#pragma unroll", "      for (int j = 0; j < 4; ++j)",
                f"        if (((m[u] >> j) & 1u) && !({gexpr})) m[u] &= ~(1u << j);", "    }"]
    if stage_vals:
        src += ["    cp_async_wait_all();", "    __syncwarp();"]
    src += _dense_tail(S, val_reg, ecols, elines, "np", "sl", [] if occ_sentinel else ["occ[slot] = 1u;"], U=U,
                       smem_vals=smem_vals, neg_zero_as_zero=occ_sentinel, l1_no_allocate=dir_bits)
    src += ["  }", "}"]
    return "\n".join(src), name


TMA_ROWS = 128       # probe rows per staged chunk (one warp's rows: 4 per lane)


def join_probe_tma_source(spec, val_reg: int, pred, bpred, fk_code: int, ST: int = 4) -> Tuple[str, str, int]:
    """The fused probe + aggregate with its column streams staged by TMA, one ring per warp.

    Every warp owns ST shared-memory stages and walks its own chunks of 128
    probe rows (chunk c = global warp + i x all warps).  Its lane 0 copies a
    chunk's column slices into a stage with 1-D bulk copies (cp.async.bulk,
    completion counted on the stage's mbarrier) ST chunks ahead, so each warp
    keeps ST x (24 B x 128) of HBM reads in flight while it filters, looks up
    the directory and aggregates the chunk it has; no CTA-wide barrier is
    involved after set-up.  The value pass is warp-dense and reads the values
    from the stage.  The last warp of the grid handles the rows after the
    last full chunk with plain loads.  Every stage wait is bounded: on expiry
    the warp records TQPK_ETIMEOUT in *err, waits (bounded) for its copies in
    flight and stops.  Returns (source, name, dynamic shared bytes)."""
    S = spec
    R = TMA_ROWS
    pcols, pexpr = _pred_code(pred, "p") if pred is not None else ([], "true")
    ecols, elines = _expr_code(S, val_reg + 1, "c")
    name = "tqpk_q_join_probe_tma"
    fkt = _CTYPE[fk_code]
    size = {L.I8: 1, L.U8: 1, L.BOOL: 1, L.I32: 4, L.I64: 8, L.F64: 8}
    cols = [("pp", c, pred.dtypes[c]) for c in pcols] + [("fk", 0, fk_code)] + \
           [("cp", c, S.col_dtypes[c]) for c in ecols]
    off, layout = 0, {}
    for kind, c, dt in cols:
        layout[(kind, c)] = (off, dt)
        off += R * size[dt]
    stage = off                                         # bytes of one stage (multiple of 128)
    params = [f"const void* __restrict__ pp{c}" for c in range(pred.n_cols if pred is not None else 0)]
    params += ["const PL lp"]
    if bpred is not None:
        params += [f"const void* __restrict__ bp{c}" for c in range(bpred.n_cols)]
        params += ["const PL lb"]
    params += [f"const void* __restrict__ cp{c}" for c in range(S.n_cols)]
    params += ["const void* __restrict__ fk", "int fk_dt", "i64 np", "i64 key_min", "i64 slots",
               "const int* __restrict__ dir", "double* __restrict__ sum", "u32* __restrict__ occ",
               "int vp", "int vc", "int vf", "int* __restrict__ err"]

    def issue(ind):
        out = [f"{ind}mbar_expect_tx(&bar[wid][st], {stage}u);"]
        for kind, c, dt in cols:
            o, _ = layout[(kind, c)]
            src = "fk" if kind == "fk" else f"{kind}{c}"
            out.append(f"{ind}bulk_g2s(ring + st * {stage} + {o}, (const unsigned char*){src} + ch * "
                       f"{R * size[dt]}ll, {R * size[dt]}u, &bar[wid][st]);")
        return out

    body = ["    const unsigned char* S0 = ring + st * " + str(stage) + ";",
            f"    const i64 wrow = ch * {R};",
            "    i64 sl[1][4]; int rw[1][4]; unsigned m[1];",
            "    {",
            "      const int u = 0;",
            "      const int lr = lane * 4;"]
    for c in pcols:
        o, dt = layout[("pp", c)]
        body.append(f"      const V4<{_CTYPE[dt]}> P{c} = ld4((const {_CTYPE[dt]}*)(S0 + {o}) + lr, 0, 4, true);")
    o, _ = layout[("fk", 0)]
    body += [f"      const V4<{fkt}> F = ld4((const {fkt}*)(S0 + {o}) + lr, 0, 4, true);",
             "      m[0] = 0;",
             "#pragma unroll",
             "      for (int j = 0; j < 4; ++j) {",
             "        sl[0][j] = (i64)F.v[j] - key_min;",
             f"        const bool ok = ({_rename(pexpr, 'p', 'P')}) && sl[0][j] >= 0 && sl[0][j] < slots;",
             "        m[0] |= (unsigned)ok << j;",
             "      }",
             "#pragma unroll",
             "      for (int j = 0; j < 4; ++j) {",
             "        rw[0][j] = ((m[0] >> j) & 1u) ? __ldg(&dir[sl[0][j]]) : -1;",
             "        if (rw[0][j] < 0) m[0] &= ~(1u << j);",
             "      }"]
    if bpred is not None:
        glines, gexpr = _gather_pred(bpred, "b", "lb", "bp", "rw[u]", "m[u]")
        body += ["      if (m[0]) {"] + ["        " + l for l in glines]
        body += ["#pragma unroll", "        for (int j = 0; j < 4; ++j)",
                 f"          if (((m[u] >> j) & 1u) && !({gexpr})) m[u] &= ~(1u << j);", "      }"]
    body += ["    }"]
    smem_vals = {c: f"(const {_CTYPE[layout[('cp', c)][1]]}*)(S0 + {layout[('cp', c)][0]})" for c in ecols}
    body += _dense_tail(S, val_reg, ecols, elines, "np", "sl", ["occ[slot] = 1u;"], U=1, smem_vals=smem_vals)
    # rows after the last full chunk: the grid's last warp, plain loads
    tail = ["  if (blockIdx.x == gridDim.x - 1 && wid == 7) {",
            f"    for (i64 w0 = (nch * {R} >> 2); w0 < ((np + 3) >> 2); w0 += 32) {{",
            "      const i64 g = w0 + lane, wrow = w0 << 2;",
            "      i64 sl[1][4]; int rw[1][4]; unsigned m[1];",
            "      {",
            "        const int u = 0;",
            "        const i64 r0 = g << 2;",
            "        m[0] = 0;",
            "        if (r0 < np) {"]
    tail += ["          " + l for l in _load_lines(pcols, pred.dtypes, "P", "pp", "np", "false")] if pred is not None else []
    tail += [f"          const V4<{fkt}> F = ld4((const {fkt}*)fk, r0, np, false);",
             "#pragma unroll",
             "          for (int j = 0; j < 4; ++j) {",
             "            sl[0][j] = (i64)F.v[j] - key_min;",
             f"            const bool ok = (r0 + j < np) && ({_rename(pexpr, 'p', 'P')}) && sl[0][j] >= 0 && sl[0][j] < slots;",
             "            m[0] |= (unsigned)ok << j;",
             "          }",
             "        }",
             "#pragma unroll",
             "        for (int j = 0; j < 4; ++j) {",
             "          rw[0][j] = ((m[0] >> j) & 1u) ? __ldg(&dir[sl[0][j]]) : -1;",
             "          if (rw[0][j] < 0) m[0] &= ~(1u << j);",
             "        }"]
    if bpred is not None:
        glines, gexpr = _gather_pred(bpred, "b", "lb", "bp", "rw[u]", "m[u]")
        tail += ["        if (m[0]) {"] + ["          " + l for l in glines]
        tail += ["#pragma unroll", "          for (int j = 0; j < 4; ++j)",
                 f"            if (((m[u] >> j) & 1u) && !({gexpr})) m[u] &= ~(1u << j);", "        }"]
    tail += ["      }"]
    tail += ["  " + l for l in _dense_tail(S, val_reg, ecols, elines, "np", "sl", ["occ[slot] = 1u;"], U=1)]
    tail += ["    }", "  }"]
    src = [PRELUDE, f'extern "C" __global__ void __launch_bounds__(256) {name}(',
           "    " + ",\n    ".join(params) + ") {",
           "  extern __shared__ __align__(1024) unsigned char stg[];",
           f"  __shared__ __align__(8) unsigned long long bar[8][{ST}];",
           f"  __shared__ unsigned char q_off[8][{R}];",
           f"  __shared__ int q_slot[8][{R}];",
           "  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;",
           f"  unsigned char* ring = stg + wid * {ST * stage};",
           f"  const i64 nch = np / {R};",
           "  const i64 gw = (i64)blockIdx.x * 8 + wid, nw = (i64)gridDim.x * 8;",
           "  if (threadIdx.x == 0) {",
           f"    for (int w = 0; w < 8; ++w) for (int st = 0; st < {ST}; ++st) mbar_init(&bar[w][st], 1);",
           "    mbar_fence_init();",
           "  }",
           "  __syncthreads();",
           "  unsigned pend = 0, ppar = 0;      // lane 0: stages with a copy in flight and their phase parity",
           "  if (lane == 0)",
           f"    for (int st = 0; st < {ST}; ++st) {{",
           "      const i64 ch = gw + st * nw;",
           "      if (ch >= nch) break;"]
    src += issue("      ")
    src += ["      pend |= 1u << st;",
            "    }",
            "  int stop = 0;",
            "  for (i64 it = 0;; ++it) {",
            "    const i64 ch = gw + it * nw;",
            "    if (ch >= nch) break;",
            f"    const int st = (int)(it % {ST});",
            f"    const unsigned par = (unsigned)((it / {ST}) & 1);",
            "    if (lane == 0) {",
            "      int spins = 0;",
            "      while (!mbar_try_wait(&bar[wid][st], par))",
            "        if (++spins > (1 << 20)) { atomicCAS(err, 0, -3); stop = 1; break; }",
            "      if (!stop) pend &= ~(1u << st);",
            "    }",
            "    stop = __shfl_sync(0xffffffffu, stop, 0);",
            "    if (stop) break;"]
    src += body
    src += ["    if (lane == 0) {                 // every lane is done with the stage (the tail's __syncwarp)",
            f"      const i64 ch2 = ch + {ST} * nw;",
            "      if (ch2 < nch) {",
            "        const i64 ch = ch2;"]
    src += issue("        ")
    src += ["        pend |= 1u << st;",
            f"        ppar = (ppar & ~(1u << st)) | ((unsigned)(((it + {ST}) / {ST}) & 1) << st);",
            "      }",
            "    }",
            "  }",
            "  if (stop) {",
            "    // give this warp's copies still in flight a bounded time to land before it exits",
            "    if (lane == 0)",
            f"      for (int st = 0; st < {ST}; ++st) {{",
            "        if (!((pend >> st) & 1u)) continue;",
            "        int spins = 0;",
            "        while (!mbar_try_wait(&bar[wid][st], (ppar >> st) & 1u) && ++spins < (1 << 16)) {}",
            "      }",
            "    __syncwarp();",
            "    return;",
            "  }"]
    src += tail
    src += ["}"]
    return "\n".join(src), name, 8 * ST * stage


def project_source(spec, outputs) -> Tuple[str, str]:
    """CUDA source of a projection: every row's expression registers written to output
    columns.  outputs: [(register, dtype code)].  Integer results pass through float64 on
    the way out, as project.py:38-58 stores every result as float64 and casts it back."""
    S = spec
    upto = max(r for r, _ in outputs) + 1
    ecols, elines = _expr_code(S, upto, "c")
    name = "tqpk_q_project"
    params = [f"const void* __restrict__ cp{c}" for c in range(S.n_cols)]
    params += [f"void* __restrict__ op{o}" for o in range(len(outputs))]
    params += ["i64 n", "int vc"]
    src = [PRELUDE, f'extern "C" __global__ void __launch_bounds__(256) {name}(', "    " + ",\n    ".join(params) + ") {",
           "  for (i64 g = blockIdx.x * (i64)blockDim.x + threadIdx.x; g < ((n + 3) >> 2); g += (i64)gridDim.x * blockDim.x) {",
           "    const i64 r0 = g << 2;"]
    src += ["    " + l for l in _load_lines(ecols, S.col_dtypes, "Cv", "cp", "n", "vc != 0")]
    src += ["#pragma unroll", "    for (int j = 0; j < 4; ++j) {", "      if (r0 + j >= n) break;",
            "      const i64 row = r0 + j;            // r0.. below are expression registers"]
    src += ["      " + _rename(l, "c", "Cv") for l in elines]
    for o, (reg, dt) in enumerate(outputs):
        t = _CTYPE[dt]
        f64 = S.expr[reg].type == L.F64
        val = f"r{reg}" if (f64 or dt == L.F64) else f"(double)r{reg}"
        src.append(f"      (({t}*)op{o})[row] = ({t})({val});")
    src += ["    }", "  }", "}"]
    return "\n".join(src), name


def join_probe_args(a: "_Args", spec, pred, bpred, fk, np_: int, key_min: int, slots: int, dir_ptr: int,
                    sum_ptr: int, occ_ptr: int, pred_tensors=(), bpred_tensors=(), col_tensors=()):
    """Parameters of join_probe_source's kernel, in order."""
    if pred is not None:
        for c in range(pred.n_cols):
            a.ptr(pred.cols[c])
    a.blob(pred_lits(pred))
    if bpred is not None:
        for c in range(bpred.n_cols):
            a.ptr(bpred.cols[c])
        a.blob(pred_lits(bpred))
    for c in range(spec.n_cols):
        a.ptr(spec.cols[c])
    a.ptr(fk.data_ptr())
    a.i32(L.I64 if fk.dtype.itemsize == 8 else L.I32)
    a.i64(np_)
    a.i64(key_min)
    a.i64(slots)
    a.ptr(dir_ptr)
    a.ptr(sum_ptr)
    a.ptr(occ_ptr)
    a.i32(_aligned(*pred_tensors) if pred is not None else 1)
    a.i32(_aligned(*col_tensors))
    a.i32(_aligned(fk))
    return a


def join_build_bits_source(pred) -> Tuple[str, str]:
    """CUDA source of the fused join's build stage in the membership-bitmap form, the build
    predicate compiled in (the library's k_pl_build_bits interprets it: ~110 instructions a row):
    every group sum set to -0.0 (the empty marker), one `red.or` per passing build row into the
    bitmap (bit s of word s / 32 for key key_min + s), the passing rows counted (one atomic per
    CTA), an out-of-domain key reported as TQPK_EINVAL (-1) in *err.  A repeated key shows later
    as fewer bits set than rows counted (the top-k's check)."""
    pcols, pexpr = _pred_code(pred, "p") if pred is not None else ([], "true")
    name = "tqpk_q_join_build_bits"
    params = [f"const void* __restrict__ pp{c}" for c in range(pred.n_cols if pred is not None else 0)]
    params += ["const PL lp", "const void* __restrict__ bk", "int bk_dt", "i64 nb", "i64 key_min", "i64 slots",
               "unsigned* __restrict__ bits", "double* __restrict__ sum", "u64* __restrict__ passing",
               "int* __restrict__ err", "int vp", "int vk"]
    key_load = ("const V4<i64> K = (bk_dt == 4) ? ld4((const long long*)bk, r0, nb, vk != 0) : "
                "[&]{ V4<int> t = ld4((const int*)bk, r0, nb, vk != 0); V4<i64> o; "
                "for (int q = 0; q < 4; ++q) o.v[q] = t.v[q]; return o; }();")
    src = [PRELUDE,
           "__device__ __forceinline__ void gred_or(unsigned* p, unsigned v) {",
           '  asm volatile("red.global.or.b32 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "r"(v) : "memory");',
           "}",
           f'extern "C" __global__ void __launch_bounds__(256) {name}(',
           "    " + ",\n    ".join(params) + ") {",
           "  __shared__ unsigned s_pass;",
           "  if (threadIdx.x == 0) s_pass = 0;",
           "  const i64 tid = blockIdx.x * (i64)blockDim.x + threadIdx.x, nthr = (i64)gridDim.x * blockDim.x;",
           "  {  // the sums start at -0.0, 16-byte stores",
           "    const double e = __longlong_as_double((long long)0x8000000000000000ull);",
           "    const bool v2 = (reinterpret_cast<unsigned long long>(sum) & 15u) == 0;",
           "    const i64 pairs = v2 ? slots / 2 : 0;",
           "    for (i64 i = tid; i < pairs; i += nthr) reinterpret_cast<double2*>(sum)[i] = make_double2(e, e);",
           "    for (i64 i = 2 * pairs + tid; i < slots; i += nthr) sum[i] = e;",
           "  }",
           "  __syncthreads();",
           "  unsigned npass = 0;",
           "  for (i64 g = tid; g < ((nb + 3) >> 2); g += nthr) {",
           "    const i64 r0 = g << 2;"]
    src += ["    " + l for l in _load_lines(pcols, pred.dtypes, "P", "pp", "nb", "vp != 0")] if pred is not None else []
    src += ["    " + key_load,
            "#pragma unroll",
            "    for (int j = 0; j < 4; ++j) {",
            f"      if (r0 + j >= nb || !({_rename(pexpr, 'p', 'P')})) continue;",
            "      const i64 slot = K.v[j] - key_min;",
            "      if (slot < 0 || slot >= slots) { atomicCAS(err, 0, -1); continue; }",
            "      gred_or(&bits[slot >> 5], 1u << (slot & 31));",
            "      ++npass;",
            "    }",
            "  }",
            "  npass = __reduce_add_sync(0xffffffffu, npass);",
            "  if ((threadIdx.x & 31) == 0 && npass) atomicAdd(&s_pass, npass);",
            "  __syncthreads();",
            "  if (threadIdx.x == 0 && s_pass) atomicAdd(passing, (u64)s_pass);",
            "}"]
    return "\n".join(src), name


def join_build_bits_args(a: "_Args", pred, bk, nb: int, key_min: int, slots: int, bits_ptr: int, sum_ptr: int,
                         passing_ptr: int, err_ptr: int, pred_tensors=()):
    """Parameters of join_build_bits_source's kernel, in order."""
    if pred is not None:
        for c in range(pred.n_cols):
            a.ptr(pred.cols[c])
    a.blob(pred_lits(pred))
    a.ptr(bk.data_ptr() if nb else None)
    a.i32(L.I64 if bk.dtype.itemsize == 8 else L.I32)
    a.i64(nb)
    a.i64(key_min)
    a.i64(slots)
    a.ptr(bits_ptr)
    a.ptr(sum_ptr)
    a.ptr(passing_ptr)
    a.ptr(err_ptr)
    a.i32(_aligned(*pred_tensors) if pred is not None else 1)
    a.i32(_aligned(bk))
    return a


# ---------------------------------------------------------------------------- star probe
def star_probe_source(spec, val_reg: int, fpred, apred, U: int = PROBE_U, min_blocks: int = 0,
                      early_fb: bool = False, stream_cs: bool = False, composed: bool = False,
                      a_bits: bool = False) -> Tuple[str, str]:
    """CUDA source of the star probe: fact -> A (row directory, A predicate through the
    row) -> B (directory of the C foreign key) -> C (row directory), then FP64 sum and
    count per C slot, computed warp-densely over the matched rows (_dense_tail).
    Directories: A and C hold row indices (negative = none), B holds the C key
    (INT_MIN = none).  early_fb loads the fkB column together with fkA, so the
    B lookup does not wait for a second column round trip after the A lookup;
    stream_cs loads the fact columns with evict-first hints; composed means B's directory
    already holds only C keys that have a C row (tqpk_directory_compose), so the C lookup
    is left out of the chain; a_bits means dir_a is A's membership bitmap
    (tqpk_directory_bits: 1 bit per key, 250 KB for 2 M keys, mostly L1-resident) in place
    of its row directory, which needs A's filter applied at build (apred None); the B lookups
    and the value loads then bypass L1 so that the bitmap keeps it."""
    if a_bits and apred is not None:
        raise ValueError("a membership bitmap carries no A row for a probe-time A predicate")
    S = spec
    pcols, pexpr = _pred_code(fpred, "p") if fpred is not None else ([], "true")
    ecols, elines = _expr_code(S, val_reg + 1, "c")
    name = "tqpk_q_star_probe"
    params = [f"const void* __restrict__ pp{c}" for c in range(fpred.n_cols if fpred is not None else 0)]
    params += ["const PL lp"]
    if apred is not None:
        params += [f"const void* __restrict__ ap{c}" for c in range(apred.n_cols)]
        params += ["const PL la"]
    params += [f"const void* __restrict__ cp{c}" for c in range(S.n_cols)]
    params += ["const int* __restrict__ fka", "const int* __restrict__ fkb", "i64 nf",
               "i64 a_min", "i64 a_slots", "const unsigned* __restrict__ dir_a" if a_bits else "const int* __restrict__ dir_a",
               "i64 b_min", "i64 b_slots", "const int* __restrict__ dir_b",
               "i64 c_min", "i64 c_slots", "const int* __restrict__ dir_c",
               "double* __restrict__ sum", "u32* __restrict__ cnt", "int vp", "int vc", "int vf"]
    rows = 4 * U
    qt = "unsigned char" if 32 * rows <= 256 else "unsigned short"
    lb = f"256, {min_blocks}" if min_blocks else "256"
    hint = "#define TQPK_LD(p) __ldcs(p)\n" if stream_cs else ""
    src = [hint + PRELUDE, f'extern "C" __global__ void __launch_bounds__({lb}) {name}(', "    " + ",\n    ".join(params) + ") {",
           f"  __shared__ {qt} q_off[8][{32 * rows}];",
           f"  __shared__ int q_slot[8][{32 * rows}];",
           "  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;",
           f"  const i64 nr = (nf + {rows - 1}) / {rows};",
           "  const i64 stride = (i64)gridDim.x * blockDim.x;",
           "  for (i64 w0 = blockIdx.x * (i64)blockDim.x + (threadIdx.x & ~31); w0 < nr; w0 += stride) {",
           f"    const i64 g = w0 + lane, wrow = w0 * {rows};",
           f"    i64 k[{U}][4]; int rw[{U}][4]; unsigned m[{U}];"]
    if early_fb:
        src += [f"    V4<int> FBs[{U}];"]
    src += [
           "#pragma unroll",
           f"    for (int u = 0; u < {U}; ++u) {{",
           f"      const i64 r0 = g * {rows} + u * 4;",
           "      m[u] = 0;",
           "      if (r0 >= nf) continue;"]
    src += ["      " + l for l in _load_lines(pcols, fpred.dtypes, "P", "pp", "nf", "vp != 0")] if fpred is not None else []
    src += ["      const V4<int> FA = ld4(fka, r0, nf, vf != 0);"]
    src += ["      FBs[u] = ld4(fkb, r0, nf, vf != 0);"] if early_fb else []
    src += ["#pragma unroll",
            "      for (int j = 0; j < 4; ++j) {",
            "        k[u][j] = (i64)FA.v[j] - a_min;",
            f"        const bool ok = (r0 + j < nf) && ({_rename(pexpr, 'p', 'P')}) && k[u][j] >= 0 && k[u][j] < a_slots;",
            "        m[u] |= (unsigned)ok << j;",
            "      }",
            "    }",
            "#pragma unroll",
            f"    for (int u = 0; u < {U}; ++u)",
            "#pragma unroll",
            "      for (int j = 0; j < 4; ++j) {",
            ("        rw[u][j] = ((m[u] >> j) & 1u) ? (int)((__ldg(&dir_a[k[u][j] >> 5]) >> (k[u][j] & 31)) & 1u) - 1 : -1;"
             if a_bits else "        rw[u][j] = ((m[u] >> j) & 1u) ? __ldg(&dir_a[k[u][j]]) : -1;"),
            "        if (rw[u][j] < 0) m[u] &= ~(1u << j);",
            "      }"]
    if apred is not None:
        glines, gexpr = _gather_pred(apred, "a", "la", "ap", "rw[u]", "m[u]")
        src += ["#pragma unroll", f"    for (int u = 0; u < {U}; ++u) {{", "      if (!m[u]) continue;"]
        src += ["      " + l for l in glines]
        src += ["#pragma unroll", "      for (int j = 0; j < 4; ++j)",
                f"        if (((m[u] >> j) & 1u) && !({gexpr})) m[u] &= ~(1u << j);", "    }"]
    src += ["#pragma unroll",
            f"    for (int u = 0; u < {U}; ++u) {{",
            "      if (!m[u]) continue;",
            f"      const i64 r0 = g * {rows} + u * 4;",
            "      const V4<int> FB = FBs[u];" if early_fb else "      const V4<int> FB = ld4(fkb, r0, nf, vf != 0);",
            "#pragma unroll",
            "      for (int j = 0; j < 4; ++j) {",
            "        const i64 sb = (i64)FB.v[j] - b_min;",
            "        const bool ok = ((m[u] >> j) & 1u) && sb >= 0 && sb < b_slots;",
            f"        const int fc = ok ? {'ld_na' if a_bits else '__ldg'}(&dir_b[sb]) : (int)0x80000000;",
            "        k[u][j] = (i64)fc - c_min;",
            "        if (fc == (int)0x80000000 || k[u][j] < 0 || k[u][j] >= c_slots) m[u] &= ~(1u << j);",
            "      }",
            "    }",
            ]
    if not composed:
        src += ["#pragma unroll",
                f"    for (int u = 0; u < {U}; ++u)",
                "#pragma unroll",
                "      for (int j = 0; j < 4; ++j)",
                "        if (((m[u] >> j) & 1u) && __ldg(&dir_c[k[u][j]]) < 0) m[u] &= ~(1u << j);"]
    src += _dense_tail(S, val_reg, ecols, elines, "nf", "k", ["gred_add(&cnt[slot], 1u);"], U=U,
                       l1_no_allocate=a_bits)
    src += ["  }", "}"]
    return "\n".join(src), name
