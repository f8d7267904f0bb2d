// common.cuh - shared device/host helpers of libtqpk (sm_103a).
//
// * dtype-generic column loads (constants.py dtype map: int8 strings, int64
//   ints, float64 decimals, int32 dates, plus uint8 flags)
// * the bounded decoupled look-back used by every ordered (stable) output:
//   stream compaction, join pair emission, group emission and the radix sort
// * block scans and the predicate-program interpreter (filter.py:14-162)
//
// Every spin on another CTA's flag is bounded (kSpinLimit polls with a short
// sleep, well under a second in total); on expiry the waiting CTA records
// TQPK_ETIMEOUT in the caller's error word, publishes what it has so that its
// successors also finish, and the host turns the error word into a status.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tqpk.h"

namespace tqpk {

// ---------------------------------------------------------------- host side
int num_sms();                        // SM count of the current device (cached)
extern thread_local int64_t g_launches;

#define TQPK_CHECK_LAUNCH()                                   \
  do {                                                        \
    ++::tqpk::g_launches;                                     \
    if (cudaPeekAtLastError() != cudaSuccess) {               \
      (void)cudaGetLastError();                               \
      return TQPK_ECUDA;                                      \
    }                                                         \
  } while (0)

#define TQPK_CUDA(x)                                          \
  do {                                                        \
    if ((x) != cudaSuccess) {                                 \
      (void)cudaGetLastError();                               \
      return TQPK_ECUDA;                                      \
    }                                                         \
  } while (0)

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
inline int dtype_size(int dt) {
  switch (dt) {
    case TQPK_I8: case TQPK_U8: case TQPK_BOOL: return 1;
    case TQPK_I32: return 4;
    case TQPK_I64: case TQPK_F64: return 8;
  }
  return 0;
}
inline bool is_int_dtype(int dt) {
  return dt == TQPK_I8 || dt == TQPK_U8 || dt == TQPK_I32 || dt == TQPK_I64 || dt == TQPK_BOOL;
}

// Bump allocator over a caller-provided workspace (256-byte aligned pieces).
struct WsCursor {
  char* base;
  size_t size, off = 0;
  WsCursor(void* b, size_t s) : base(static_cast<char*>(b)), size(s) {}
  template <class T>
  T* take(size_t count) {
    size_t o = align_up(off, 256);
    size_t bytes = align_up(count * sizeof(T), 256);
    if (o + bytes > size) return nullptr;
    off = o + bytes;
    return reinterpret_cast<T*>(base + o);
  }
};

// -------------------------------------------------------------- device side
constexpr int kSpinLimit = 1 << 21;   // polls of 64-256 ns each: well under a second
constexpr uint64_t kFlagAgg = 1ull << 62;
constexpr uint64_t kFlagInc = 2ull << 62;
constexpr uint64_t kValMask = (1ull << 62) - 1;

__device__ __forceinline__ uint64_t ld_acquire(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint64_t* p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void set_error(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// The bits of a double through an opaque move: integer tests on those bits (the sign, -0.0, the
// NaN exponent) stay integer instructions.  Through a plain reinterpretation the compiler may fold
// such tests back into FP64 compares, and FP64 runs at 1/64 of the FP32 rate on this part
// (measured: 2 FP64-pipe instructions per item in a top-k key transform, 7.2 against 2.8 us
// per CTA).
__device__ __forceinline__ uint64_t d2u(double d) {
  uint64_t u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(d));
  return u;
}
__device__ __forceinline__ double u2d(uint64_t u) { return __longlong_as_double(static_cast<long long>(u)); }

// Reductions into global memory whose result nobody reads: `red.global`, applied at the L2 with no
// reply.  An atomicAdd through a pointer the compiler cannot place in global memory (one loaded
// from a descriptor or selected between shared and global tables) is a generic atomic that returns
// its old value, and the issuing warp waits for the round trip (measured on a 9.3 K-group batched
// group-by: every update an L2 round trip, 122 stall cycles per issued instruction).
__device__ __forceinline__ void gred_add(double* p, double v) {
  asm volatile("red.global.add.f64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "d"(v) : "memory");
}
__device__ __forceinline__ void gred_add(uint64_t* p, uint64_t v) {
  asm volatile("red.global.add.u64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
__device__ __forceinline__ void gred_add(unsigned* p, unsigned v) {
  asm volatile("red.global.add.u32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "r"(v) : "memory");
}
__device__ __forceinline__ void gred_min_u64(uint64_t* p, uint64_t v) {
  asm volatile("red.global.min.u64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
__device__ __forceinline__ void gred_max_u64(uint64_t* p, uint64_t v) {
  asm volatile("red.global.max.u64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
__device__ __forceinline__ void gred_min_s64(uint64_t* p, int64_t v) {
  asm volatile("red.global.min.s64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
__device__ __forceinline__ void gred_max_s64(uint64_t* p, int64_t v) {
  asm volatile("red.global.max.s64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}
// Merge of a value (accumulator encoding: F64 sums as bits, F64 min/max as order keys) into a
// global table cell.
__device__ __forceinline__ void acc_merge_global(uint64_t* p, const tqpk_acc& a, uint64_t v) {
  switch (a.kind) {
    case TQPK_ACC_SUM:
      if (a.type == TQPK_F64) gred_add(reinterpret_cast<double*>(p), u2d(v));
      else gred_add(p, v);
      break;
    case TQPK_ACC_COUNT_ROWS:
    case TQPK_ACC_COUNT_NOTNULL: gred_add(p, v); break;
    case TQPK_ACC_MIN:
      if (a.type == TQPK_F64) gred_min_u64(p, v);
      else gred_min_s64(p, static_cast<int64_t>(v));
      break;
    case TQPK_ACC_MAX:
      if (a.type == TQPK_F64) gred_max_u64(p, v);
      else gred_max_s64(p, static_cast<int64_t>(v));
      break;
  }
}

// Order-preserving map of a double onto uint64 (for min/max atomics and the
// radix sort): negative values have all bits flipped, others the sign bit.
__device__ __forceinline__ uint64_t f64_ordered(double d) {
  uint64_t u = d2u(d);
  return (u & (1ull << 63)) ? ~u : (u | (1ull << 63));
}
__device__ __forceinline__ double f64_from_ordered(uint64_t o) {
  uint64_t u = (o & (1ull << 63)) ? (o & ~(1ull << 63)) : ~o;
  return u2d(u);
}

// The bits of a float64 with -0.0 folded onto +0.0 and every NaN onto one quiet NaN, in integer
// instructions only: on this part FP64 compares run at 1/64 of the FP32 rate, which made
// comparisons the cost of passes that only rank or hash doubles.
__device__ __forceinline__ uint64_t f64_canon_bits(uint64_t b) {
  if ((b << 1) == 0) return 0;                                            // +-0.0
  if ((b & 0x7ff0000000000000ull) == 0x7ff0000000000000ull && (b & 0x000fffffffffffffull))
    return 0x7ff8000000000000ull;                                         // NaN
  return b;
}

// Order-preserving uint64 image of a key of any dtype for sorting: signed ints
// flip the sign bit; float64 flips sign-magnitude with -0.0 -> +0.0 and every
// NaN mapped to the largest value (torch.sort's order); descending = bitwise
// complement, which keeps equal keys in input order under a stable sort.
__device__ __forceinline__ uint64_t sort_key_bits(uint64_t raw, int is_f64, int desc) {
  uint64_t u;
  if (is_f64) {
    const uint64_t b = f64_canon_bits(raw);
    u = (b & (1ull << 63)) ? ~b : (b | (1ull << 63));
  } else {
    u = raw ^ (1ull << 63);
  }
  return desc ? ~u : u;
}

// ---- column loads -----------------------------------------------------------
__device__ __forceinline__ int64_t ld_int(const void* p, int dt, int64_t i) {
  switch (dt) {
    case TQPK_I8: return static_cast<const int8_t*>(p)[i];
    case TQPK_U8:
    case TQPK_BOOL: return static_cast<const uint8_t*>(p)[i];
    case TQPK_I32: return static_cast<const int32_t*>(p)[i];
    case TQPK_I64: return static_cast<const int64_t*>(p)[i];
    case TQPK_F64: return static_cast<int64_t>(static_cast<const double*>(p)[i]);
  }
  return 0;
}
__device__ __forceinline__ double ld_f64(const void* p, int dt, int64_t i) {
  if (dt == TQPK_F64) return static_cast<const double*>(p)[i];
  return static_cast<double>(ld_int(p, dt, i));
}
__device__ __forceinline__ uint64_t sort_key(const void* keys, int dt, int64_t i, int desc) {
  const uint64_t raw = dt == TQPK_F64 ? d2u(static_cast<const double*>(keys)[i])
                                      : static_cast<uint64_t>(ld_int(keys, dt, i));
  return sort_key_bits(raw, dt == TQPK_F64, desc);
}

// Loads four consecutive rows r0..r0+3 (r0 % 4 == 0); rows >= n read as 0.
// `vec` means the base pointer is 16-byte aligned, so a full group can use
// 128-bit loads.
__device__ __forceinline__ void ld4_int(const void* p, int dt, int64_t r0, int64_t n, bool vec,
                                        int64_t (&x)[4]) {
  const bool full = vec && (r0 + 4 <= n);
  if (full) {
    switch (dt) {
      case TQPK_I32: {
        int4 v = *reinterpret_cast<const int4*>(static_cast<const int32_t*>(p) + r0);
        x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
        return;
      }
      case TQPK_I64: {
        const longlong2* q = reinterpret_cast<const longlong2*>(static_cast<const int64_t*>(p) + r0);
        longlong2 a = q[0], b = q[1];
        x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
        return;
      }
      case TQPK_U8:
      case TQPK_BOOL: {
        uint32_t w = *reinterpret_cast<const uint32_t*>(static_cast<const uint8_t*>(p) + r0);
        x[0] = w & 0xff; x[1] = (w >> 8) & 0xff; x[2] = (w >> 16) & 0xff; x[3] = w >> 24;
        return;
      }
      case TQPK_I8: {
        uint32_t w = *reinterpret_cast<const uint32_t*>(static_cast<const uint8_t*>(p) + r0);
        x[0] = (int8_t)(w & 0xff); x[1] = (int8_t)((w >> 8) & 0xff);
        x[2] = (int8_t)((w >> 16) & 0xff); x[3] = (int8_t)(w >> 24);
        return;
      }
      default: break;
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) x[j] = (r0 + j < n) ? ld_int(p, dt, r0 + j) : 0;
}

__device__ __forceinline__ void ld4_f64(const void* p, int64_t r0, int64_t n, bool vec, double (&x)[4]) {
  if (vec && r0 + 4 <= n) {
    const double2* q = reinterpret_cast<const double2*>(static_cast<const double*>(p) + r0);
    double2 a = q[0], b = q[1];
    x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
    return;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) x[j] = (r0 + j < n) ? static_cast<const double*>(p)[r0 + j] : 0.0;
}

// ---- row expressions ---------------------------------------------------------
// Straight-line expression program (tqpk_expr_insn) evaluated for one row.
// Programs of up to NR instructions run fully unrolled with operands picked
// by compile-time selects, so the register file stays in registers; longer
// programs use the generic loop (a small local-memory array).
static __device__ __noinline__ uint64_t expr_div(uint64_t a, uint64_t b) {
  return static_cast<uint64_t>(__double_as_longlong(__ddiv_rn(__longlong_as_double(a), __longlong_as_double(b))));
}

// Year of day d (days since 1990-01-01).  Days before 1990 fall in the first
// bucket (1990), as torch.bucketize over the year edges puts them.  Otherwise
// the proleptic Gregorian year, by H. Hinnant's civil_from_days method: days
// since 0000-03-01 split into 400-year eras of 146097 days, the year of the era
// from the day of the era, and January/February counted in the next year.
__host__ __device__ __forceinline__ int64_t expr_year(int64_t d) {
  if (d < 0) return 1990;
  const int64_t z = d + 7305 + 719468;           // 1970-01-01 is day 719468 after 0000-03-01
  const int64_t era = z / 146097;
  const int64_t doe = z - era * 146097;
  const int64_t yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  const int64_t doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
  const int64_t mp = (5 * doy + 2) / 153;
  return yoe + era * 400 + (mp >= 10 ? 1 : 0);
}

__device__ __forceinline__ uint64_t f32_bits(float x) { return static_cast<uint64_t>(__float_as_uint(x)); }
__device__ __forceinline__ float bits_f32(uint64_t u) { return __uint_as_float(static_cast<unsigned>(u)); }

// float32 registers (torch's default float dtype: integer with a Python float, integer true division)
__device__ __forceinline__ uint64_t expr_apply_f32(const tqpk_expr_insn& X, uint64_t a, uint64_t b) {
  switch (X.op) {
    case TQPK_X_CONST: return f32_bits(__double2float_rn(X.cf));
    case TQPK_X_TOF32: return f32_bits(__ll2float_rn(static_cast<long long>(a)));
    case TQPK_X_ADD: return f32_bits(__fadd_rn(bits_f32(a), bits_f32(b)));
    case TQPK_X_SUB: return f32_bits(__fsub_rn(bits_f32(a), bits_f32(b)));
    case TQPK_X_MUL: return f32_bits(__fmul_rn(bits_f32(a), bits_f32(b)));
    case TQPK_X_DIV: return f32_bits(__fdiv_rn(bits_f32(a), bits_f32(b)));
  }
  return 0;
}

// An int64 result narrowed to torch's result dtype (two's complement wrap of int8 / uint8 / int32).
__device__ __forceinline__ uint64_t int_wrap(uint64_t v, int wrap) {
  switch (wrap) {
    case TQPK_I8: return static_cast<uint64_t>(static_cast<int64_t>(static_cast<int8_t>(v)));
    case TQPK_U8: return static_cast<uint64_t>(static_cast<uint8_t>(v));
    case TQPK_I32: return static_cast<uint64_t>(static_cast<int64_t>(static_cast<int32_t>(v)));
  }
  return v;
}

__device__ __forceinline__ uint64_t expr_apply(const tqpk_expr_insn& X, uint64_t a, uint64_t b, uint64_t c,
                                              const void* const* cols, const int* dts, int64_t row) {
  const bool f = X.type == TQPK_F64;
  if (X.type == TQPK_F32 && X.op != TQPK_X_SELECT) return expr_apply_f32(X, a, b);
  if (X.wrap && X.type == TQPK_I64 && X.op >= TQPK_X_ADD && X.op <= TQPK_X_MUL) {
    const uint64_t r = X.op == TQPK_X_ADD ? a + b : X.op == TQPK_X_SUB ? a - b
                     : static_cast<uint64_t>(static_cast<int64_t>(a) * static_cast<int64_t>(b));
    return int_wrap(r, X.wrap);
  }
  switch (X.op) {
    case TQPK_X_F32TOF64:
      return static_cast<uint64_t>(__double_as_longlong(static_cast<double>(bits_f32(a))));
    case TQPK_X_SELECT: return a != 0 ? b : c;
    case TQPK_X_YEAR: return static_cast<uint64_t>(expr_year(static_cast<int64_t>(a)));
    case TQPK_X_COL:
      return f ? static_cast<uint64_t>(__double_as_longlong(ld_f64(cols[X.col], dts[X.col], row)))
               : static_cast<uint64_t>(ld_int(cols[X.col], dts[X.col], row));
    case TQPK_X_CONST: return f ? static_cast<uint64_t>(__double_as_longlong(X.cf)) : static_cast<uint64_t>(X.ci);
    case TQPK_X_TOF64:
      return static_cast<uint64_t>(__double_as_longlong(static_cast<double>(static_cast<int64_t>(a))));
    case TQPK_X_ADD:
      return f ? static_cast<uint64_t>(__double_as_longlong(__dadd_rn(__longlong_as_double(a), __longlong_as_double(b))))
               : a + b;
    case TQPK_X_SUB:
      return f ? static_cast<uint64_t>(__double_as_longlong(__dsub_rn(__longlong_as_double(a), __longlong_as_double(b))))
               : a - b;
    case TQPK_X_MUL:
      return f ? static_cast<uint64_t>(__double_as_longlong(__dmul_rn(__longlong_as_double(a), __longlong_as_double(b))))
               : static_cast<uint64_t>(static_cast<int64_t>(a) * static_cast<int64_t>(b));
    case TQPK_X_DIV: return expr_div(a, b);
  }
  return 0;
}

template <int NR>
__device__ __forceinline__ void expr_eval_small(const tqpk_expr_insn* E, int n, const void* const* cols,
                                                const int* dts, int64_t row, uint64_t (&r)[NR]) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    r[i] = 0;
    if (i < n) {
      const tqpk_expr_insn& X = E[i];
      uint64_t a = 0, b = 0, c = 0;
#pragma unroll
      for (int j = 0; j < i; ++j) {
        a = (X.a == j) ? r[j] : a;
        b = (X.b == j) ? r[j] : b;
        c = (X.col == j) ? r[j] : c;
      }
      r[i] = expr_apply(X, a, b, c, cols, dts, row);
    }
  }
}

template <int NR>
__device__ __forceinline__ uint64_t reg_pick(const uint64_t (&r)[NR], int idx) {
  uint64_t v = 0;
#pragma unroll
  for (int j = 0; j < NR; ++j) v = (idx == j) ? r[j] : v;
  return v;
}

__device__ __forceinline__ void expr_eval_generic(const tqpk_expr_insn* E, int n, const void* const* cols,
                                                  const int* dts, int64_t row, uint64_t* r) {
  for (int i = 0; i < n; ++i) {
    const tqpk_expr_insn& X = E[i];
    const bool two = (X.op >= TQPK_X_ADD && X.op <= TQPK_X_DIV) || X.op == TQPK_X_SELECT;
    r[i] = expr_apply(X, (X.op >= TQPK_X_ADD) ? r[X.a] : 0, two ? r[X.b] : 0, X.op == TQPK_X_SELECT ? r[X.col] : 0,
                      cols, dts, row);
  }
}

// Column preloading for 4-row groups: the first kPreCols columns of a program
// are loaded with 128-bit loads for four rows at once (all loads issued
// before any use), and X_COL instructions read them from registers.
constexpr int kPreCols = 4;

struct ColTile4 {
  uint64_t v[kPreCols][4];
};

__device__ __forceinline__ void load_cols4(const tqpk_groupby_spec& S, int64_t r0, int64_t n, bool vec, ColTile4& T) {
#pragma unroll
  for (int c = 0; c < kPreCols; ++c) {
    if (c < S.n_cols) {
      if (S.col_dtypes[c] == TQPK_F64) {
        double x[4];
        ld4_f64(S.cols[c], r0, n, vec, x);
#pragma unroll
        for (int j = 0; j < 4; ++j) T.v[c][j] = static_cast<uint64_t>(__double_as_longlong(x[j]));
      } else {
        int64_t x[4];
        ld4_int(S.cols[c], S.col_dtypes[c], r0, n, vec, x);
#pragma unroll
        for (int j = 0; j < 4; ++j) T.v[c][j] = static_cast<uint64_t>(x[j]);
      }
    }
  }
}

// Evaluates registers 0..n-1 for row j of a preloaded tile (n <= NR; every
// X_COL must name a preloaded column).
template <int NR>
__device__ __forceinline__ void expr_eval_tile(const tqpk_expr_insn* E, int n, const int* dts, const ColTile4& T, int j,
                                               uint64_t (&r)[NR]) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    r[i] = 0;
    if (i < n) {
      const tqpk_expr_insn& X = E[i];
      if (X.op == TQPK_X_COL) {
        uint64_t raw = 0;
#pragma unroll
        for (int cc = 0; cc < kPreCols; ++cc) raw = (X.col == cc) ? T.v[cc][j] : raw;
        if (X.type == TQPK_F64 && dts[X.col] != TQPK_F64)
          raw = static_cast<uint64_t>(__double_as_longlong(static_cast<double>(static_cast<int64_t>(raw))));
        r[i] = raw;
      } else {
        uint64_t a = 0, b = 0, c = 0;
#pragma unroll
        for (int q = 0; q < i; ++q) {
          a = (X.a == q) ? r[q] : a;
          b = (X.b == q) ? r[q] : b;
          c = (X.col == q) ? r[q] : c;
        }
        r[i] = expr_apply(X, a, b, c, nullptr, dts, 0);
      }
    }
  }
}

// True when the program's columns are all preloadable (and it fits NR=16 registers).
__device__ __forceinline__ bool tile_ok(const tqpk_groupby_spec& S) { return S.n_cols <= kPreCols && S.n_expr <= 16; }

// Value of register `out` for one row as a double (integers converted).
__device__ __forceinline__ double expr_value(const tqpk_groupby_spec& S, int64_t row, int out) {
  const bool f = S.expr[out].type == TQPK_F64;
  uint64_t v;
  if (out < 16) {
    uint64_t r[16];
    expr_eval_small<16>(S.expr, out + 1, S.cols, S.col_dtypes, row, r);
    v = reg_pick<16>(r, out);
  } else {
    uint64_t r[TQPK_MAX_EXPR];
    expr_eval_generic(S.expr, out + 1, S.cols, S.col_dtypes, row, r);
    v = r[out];
  }
  return f ? __longlong_as_double(static_cast<long long>(v)) : static_cast<double>(static_cast<int64_t>(v));
}

// ---- predicate interpreter (filter.py:14-162) -------------------------------
template <class T>
__device__ __forceinline__ bool cmp_op(int op, T a, T b) {
  switch (op) {
    case TQPK_LT: return a < b;
    case TQPK_LE: return a <= b;
    case TQPK_GT: return a > b;
    case TQPK_GE: return a >= b;
    case TQPK_EQ: return a == b;
    case TQPK_NE: return a != b;
  }
  return false;
}

// One comparison leaf over four rows -> 4-bit mask.
__device__ __forceinline__ uint32_t pred_leaf4(const tqpk_predicate& P, const tqpk_pred_insn& I,
                                               int64_t r0, int64_t n, bool vec) {
  const void* col = P.cols[I.col];
  const int dt = P.dtypes[I.col];
  uint32_t m = 0;
  if (I.domain == TQPK_DOM_F64) {
    double x[4];
    if (dt == TQPK_F64) {
      ld4_f64(col, r0, n, vec, x);
    } else {
      int64_t xi[4];
      ld4_int(col, dt, r0, n, vec, xi);
#pragma unroll
      for (int j = 0; j < 4; ++j) x[j] = static_cast<double>(xi[j]);
    }
    if (I.cmp == TQPK_ISCLOSE) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        double err = fabs(__dsub_rn(x[j], I.lit_f));
        bool c = (x[j] == I.lit_f) || (isfinite(err) && err <= I.lit_aux);
        m |= (uint32_t)c << j;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) m |= (uint32_t)cmp_op<double>(I.cmp, x[j], I.lit_f) << j;
    }
  } else {
    int64_t xi[4];
    ld4_int(col, dt, r0, n, vec, xi);
    if (I.domain == TQPK_DOM_F32) {
      const float lit = static_cast<float>(I.lit_f);  // exact: the host stores a float32 value
#pragma unroll
      for (int j = 0; j < 4; ++j) m |= (uint32_t)cmp_op<float>(I.cmp, static_cast<float>(xi[j]), lit) << j;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) m |= (uint32_t)cmp_op<int64_t>(I.cmp, xi[j], I.lit_i) << j;
    }
  }
  return m;
}

// ---- string predicates on int8 [N, w] rows (w = P.widths[col]) ----
__device__ __forceinline__ bool str_all_cmp(const int8_t* row, int w, const uint8_t* lit, int cmp) {
  for (int j = 0; j < w; ++j)
    if (!cmp_op<int64_t>(cmp, (int64_t)row[j], (int64_t)(int8_t)lit[j])) return false;
  return true;
}
__device__ __forceinline__ bool str_at(const int8_t* row, const uint8_t* lit, int len) {
  for (int j = 0; j < len; ++j)
    if (row[j] != (int8_t)lit[j]) return false;
  return true;
}
__device__ __forceinline__ bool str_contains(const int8_t* row, int w, const uint8_t* lit, int len) {
  for (int pos = 0; pos + len <= w; ++pos)
    if (str_at(row + pos, lit, len)) return true;
  return false;
}
__device__ __forceinline__ bool str_like2(const int8_t* row, int w, const uint8_t* a, int na, const uint8_t* b,
                                          int nb) {
  bool seen = false;                        // an occurrence of a ends at or before pos + na
  for (int pos = 0; pos + na + nb <= w; ++pos) {
    seen = seen || str_at(row + pos, a, na);
    if (seen && str_at(row + pos + na, b, nb)) return true;
  }
  return false;
}
static __device__ uint32_t str_leaf4(const tqpk_predicate& P, const tqpk_pred_insn& I, int64_t r0, int64_t n) {
  const int w = P.widths[I.col];
  const int64_t stride = P.strides[I.col] > 0 ? P.strides[I.col] : w;
  const int8_t* base = static_cast<const int8_t*>(P.cols[I.col]);
  const uint64_t L = (uint64_t)I.lit_i;
  uint32_t m = 0;
  for (int j = 0; j < 4; ++j) {
    if (r0 + j >= n) break;
    const int8_t* row = base + (r0 + j) * stride;
    bool ok;
    switch (I.op) {
      case TQPK_P_STRCMP: ok = str_all_cmp(row, w, P.strpool + (L & 0xffffffffu), I.cmp); break;
      case TQPK_P_PREFIX: ok = str_at(row, P.strpool + (L & 0xffffffffu), (int)(L >> 32)); break;
      case TQPK_P_CONTAINS: ok = str_contains(row, w, P.strpool + (L & 0xffffffffu), (int)(L >> 32)); break;
      default:
        ok = str_like2(row, w, P.strpool + (L & 0xffff), (int)((L >> 16) & 0xffff), P.strpool + ((L >> 32) & 0xffff),
                       (int)(L >> 48));
    }
    m |= (uint32_t)ok << j;
  }
  return m;
}

// Evaluates the predicate for rows r0..r0+3 -> 4-bit mask (rows >= n are 0).
__device__ __forceinline__ uint32_t eval_pred4(const tqpk_predicate& P, int64_t r0, int64_t n, bool vec) {
  if (P.n_insn == 1 && P.insn[0].op == TQPK_P_CMP) {  // one comparison: no stack
    const int64_t valid = n - r0;
    const uint32_t vm = valid >= 4 ? 0xfu : (valid <= 0 ? 0u : ((1u << valid) - 1));
    return pred_leaf4(P, P.insn[0], r0, n, vec) & vm;
  }
  uint32_t st[TQPK_MAX_PRED];
  int sp = 0;
  for (int k = 0; k < P.n_insn; ++k) {
    const tqpk_pred_insn& I = P.insn[k];
    switch (I.op) {
      case TQPK_P_CMP: st[sp++] = pred_leaf4(P, I, r0, n, vec); break;
      case TQPK_P_AND: --sp; st[sp - 1] &= st[sp]; break;
      case TQPK_P_OR: --sp; st[sp - 1] |= st[sp]; break;
      case TQPK_P_NOT: st[sp - 1] = ~st[sp - 1]; break;
      case TQPK_P_TRUE: st[sp++] = 0xfu; break;
      case TQPK_P_FALSE: st[sp++] = 0u; break;
      case TQPK_P_CMPCOL: {
        const int c2 = (int)I.lit_i;
        uint32_t m = 0;
        if (I.domain == TQPK_DOM_F64) {
          for (int j = 0; j < 4; ++j) {
            if (r0 + j >= n) break;
            const double a = ld_f64(P.cols[I.col], P.dtypes[I.col], r0 + j);
            const double b = ld_f64(P.cols[c2], P.dtypes[c2], r0 + j);
            m |= (uint32_t)cmp_op<double>(I.cmp, a, b) << j;
          }
        } else {
          int64_t a[4], b[4];
          ld4_int(P.cols[I.col], P.dtypes[I.col], r0, n, vec, a);
          ld4_int(P.cols[c2], P.dtypes[c2], r0, n, vec, b);
#pragma unroll
          for (int j = 0; j < 4; ++j) m |= (uint32_t)cmp_op<int64_t>(I.cmp, a[j], b[j]) << j;
        }
        st[sp++] = m;
        break;
      }
      case TQPK_P_MASK: {
        int64_t x[4];
        ld4_int(P.cols[I.col], TQPK_U8, r0, n, vec, x);
        st[sp++] = (x[0] != 0) | ((x[1] != 0) << 1) | ((x[2] != 0) << 2) | ((x[3] != 0) << 3);
        break;
      }
      case TQPK_P_STRCMP:
      case TQPK_P_PREFIX:
      case TQPK_P_CONTAINS:
      case TQPK_P_LIKE2: st[sp++] = str_leaf4(P, I, r0, n); break;
    }
  }
  int64_t valid = n - r0;
  uint32_t vm = valid >= 4 ? 0xfu : (valid <= 0 ? 0u : ((1u << valid) - 1));
  return (sp > 0 ? st[0] : 0xfu) & vm;
}

// Row filter: a u8 mask column, a predicate program, or neither (all rows).
struct RowFilter {
  const uint8_t* mask;
  int use_pred;
  int mask_vec;
  int pred_vec;
};

__device__ __forceinline__ uint32_t filter4(const RowFilter& F, const tqpk_predicate& P, int64_t r0, int64_t n) {
  if (F.use_pred) return eval_pred4(P, r0, n, F.pred_vec);
  int64_t valid = n - r0;
  uint32_t vm = valid >= 4 ? 0xfu : (valid <= 0 ? 0u : ((1u << valid) - 1));
  if (!F.mask) return vm;
  int64_t x[4];
  ld4_int(F.mask, TQPK_U8, r0, n, F.mask_vec, x);
  return ((x[0] != 0) | ((x[1] != 0) << 1) | ((x[2] != 0) << 2) | ((x[3] != 0) << 3)) & vm;
}

// ---- scans --------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T warp_incl_scan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide exclusive scan (BLOCK threads). `sw` holds BLOCK/32 + 1 values.
template <int BLOCK, class T>
__device__ __forceinline__ T block_excl_scan(T v, T& total, T* sw) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T inc = warp_incl_scan(v);
  if (lane == 31) sw[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < BLOCK / 32 ? sw[lane] : T(0);
    T wi = warp_incl_scan(w);
    if (lane < BLOCK / 32) sw[lane] = wi - w;
    if (lane == BLOCK / 32 - 1) sw[BLOCK / 32] = wi;
  }
  __syncthreads();
  T r = sw[warp] + inc - v;
  total = sw[BLOCK / 32];
  __syncthreads();
  return r;
}

// Decoupled look-back (single-pass prefix over tiles in tile order).  Called
// by all 32 lanes of one warp; returns the exclusive prefix of `tile` and
// publishes its inclusive prefix.  status[] must start zeroed.
__device__ __forceinline__ uint64_t lookback_warp(uint64_t* status, int64_t tile, uint64_t aggregate, int* err,
                                                  int spin_limit = kSpinLimit) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_release(&status[0], kFlagInc | aggregate);
    return 0;
  }
  if (lane == 0) st_release(&status[tile], kFlagAgg | aggregate);
  uint64_t excl = 0;
  int64_t base = tile - 1;
  int spins = 0;
  while (true) {
    const int64_t p = base - lane;
    const uint64_t s = (p >= 0) ? ld_acquire(&status[p]) : kFlagInc;
    const uint32_t inc = __ballot_sync(0xffffffffu, (s >> 62) == 2);
    const uint32_t zero = __ballot_sync(0xffffffffu, (s >> 62) == 0);
    const uint32_t need = inc ? (((inc & (0u - inc)) << 1) - 1u) : 0xffffffffu;
    if (zero & need) {
      if (++spins > spin_limit) {
        if (lane == 0) set_error(err, TQPK_ETIMEOUT);
        break;
      }
      __nanosleep(64);
      continue;
    }
    uint64_t v = ((need >> lane) & 1u) ? (s & kValMask) : 0ull;
    excl += warp_sum(v);
    if (inc) break;
    base -= 32;
  }
  if (lane == 0) st_release(&status[tile], kFlagInc | ((excl + aggregate) & kValMask));
  return excl;
}

// Per-thread variant (one independent chain per thread, e.g. one radix digit
// per thread).  status is indexed status[tile * stride + lane_id].
__device__ __forceinline__ uint64_t lookback_thread(uint64_t* status, int64_t tile, int stride, int id,
                                                    uint64_t aggregate, int* err) {
  if (tile == 0) {
    st_release(&status[id], kFlagInc | aggregate);
    return 0;
  }
  st_release(&status[tile * stride + id], kFlagAgg | aggregate);
  uint64_t excl = 0;
  int64_t p = tile - 1;
  int spins = 0;
  while (p >= 0) {
    const uint64_t s = ld_acquire(&status[p * stride + id]);
    const uint64_t f = s >> 62;
    if (f == 0) {
      if (++spins > kSpinLimit) {
        set_error(err, TQPK_ETIMEOUT);
        break;
      }
      __nanosleep(64);
      continue;
    }
    excl += s & kValMask;
    if (f == 2) break;
    --p;
  }
  st_release(&status[tile * stride + id], kFlagInc | ((excl + aggregate) & kValMask));
  return excl;
}

// ---------------------------------------------------- kernel timing hook
// tqpk_timing_begin(id) makes every launch of kernel `id` record a pair of
// CUDA events around itself on its own stream; tqpk_timing_end() sums them.
enum { KID_NONE = 0, KID_FILTER_MASK = 1, KID_COMPACT = 2, KID_GROUPBY = 3, KID_SORT_PASS = 4, KID_JOIN_PROBE = 5,
       KID_PIPE_PROBE = 6, KID_PIPE_BUILD = 7, KID_PIPE_TOPK = 8, KID_STAR_PROBE = 9, KID_BATCH = 10 };
void timing_before(int kid, cudaStream_t s);
void timing_after(int kid, cudaStream_t s);

// ---------------------------------------------------- shared host helpers
constexpr int kBlock = 256;
constexpr int kItems = 16;                 // rows per thread in an ordered tile
constexpr int kTile = kBlock * kItems;     // 4096 rows per tile

struct ColSet {
  int n;
  const void* in[TQPK_MAX_COLS];
  void* out[TQPK_MAX_COLS];
  int size[TQPK_MAX_COLS];
};

struct KeySet {
  int n;
  const void* col[TQPK_MAX_KEYS];
  int dt[TQPK_MAX_KEYS];
};

bool pred_vec_ok(const tqpk_predicate* p);
int check_pred(const tqpk_predicate* p);
RowFilter make_filter(const tqpk_predicate* pred, const uint8_t* mask);
const tqpk_predicate* pred_or_empty(const tqpk_predicate* p);
int grid_for(int64_t work_items, int per_sm);
int key_ranges(const tqpk_predicate* pred, const uint8_t* mask, int64_t n, int nk, const void* const* cols,
               const int32_t* dts, int64_t* h_min, int64_t* h_max, int64_t* h_count, void* scratch,
               cudaStream_t s);
size_t compact_status_bytes(int64_t n);
int compact_launch(const tqpk_predicate* pred, const uint8_t* mask, int64_t n, const ColSet& C, int64_t* d_count,
                   void* ws, size_t ws_bytes, cudaStream_t s);
size_t sort_ws_bytes(int64_t n);
bool spec_cols_vec(const tqpk_groupby_spec* S);   // all spec columns 16-byte aligned

// Grid of one full wave: resident CTAs per SM (occupancy API) x SMs, capped by
// the work (one thread per work unit).
template <class K>
inline int occ_grid(K kernel, int64_t work_units, size_t smem = 0) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem) != cudaSuccess || per_sm < 1) {
    (void)cudaGetLastError();
    per_sm = 2;
  }
  int64_t g = (work_units + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)per_sm * num_sms();
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}
int sort_pairs(const void* keys, int dt, int desc, const int64_t* perm_in, int64_t n, void* ws, size_t ws_bytes,
               cudaStream_t s, const int64_t** result);

}  // namespace tqpk
