// groupby.cu - kernel (d): group-by aggregation fused with the filter.
//
// Reference: operators/aggregate.py:236-393.  The reference compacts every
// input column with the filter mask (vortex_pipeline.py:58), hashes the key
// tuple with random coefficients and sorts it (torch.unique(dim=0), :318-327),
// then makes one full pass per aggregate (bincount / scatter_reduce, :122-195)
// with the expression temporaries materialised (:203-233).
//
// Here one pass reads each needed column once; rows failing the filter are
// skipped in registers (never compacted), the expression program runs in
// registers, and every accumulator is updated in the same pass.  Groups are
// addressed by a mixed-radix slot computed from the key ranges (one cheap
// min/max pre-pass over the key columns), so no hashing or sorting is needed
// and the groups come out in ascending key-tuple order:
//
//   DENSE_PRIVATE  slots*accs small: every thread owns a private copy of the
//                  table in shared memory (plain loads/stores, no atomics --
//                  shared-memory f64 atomics serialise badly on GB300).
//   DENSE_SHARED   up to ~12k slot*accs: one table per CTA, shared atomics.
//   DENSE_GLOBAL   up to max(4*rows, 2^20) slots: global (L2) atomics.
//   HASH           larger (sparse) key spaces: the packed mixed-radix key in an
//                  open-addressing table of >= 2 x rows slots, groups sorted
//                  by packed key at emit (the same ascending key-tuple order).
//
// FP64 work is the limit on GB300 (FP64 runs at 1/64 of the FP32 rate), so
// the expression program is straight-line with shared subexpressions and no
// FP64 atomics in shared memory.
#include <algorithm>

#include "common.cuh"

namespace tqpk {

struct GbDev {
  int nk;
  int64_t kmin[TQPK_MAX_KEYS];
  int64_t kstride[TQPK_MAX_KEYS];
  int64_t krange[TQPK_MAX_KEYS];
  int64_t slots;
};

__device__ __forceinline__ uint64_t acc_init(const tqpk_acc& a) {
  if (a.kind == TQPK_ACC_MIN || a.kind == TQPK_ACC_MAX)
    return a.type == TQPK_F64 ? f64_ordered(a.init_f) : static_cast<uint64_t>(a.init_i);
  return 0ull;
}

// Plain (owner-only) update of one accumulator cell.
// x is the raw register value (float64 or int64 bits) of the accumulated expression.
__device__ __forceinline__ void acc_plain(uint64_t* p, const tqpk_acc& a, uint64_t x) {
  switch (a.kind) {
    case TQPK_ACC_SUM:
      if (a.type == TQPK_F64) *p = d2u(__dadd_rn(u2d(*p), u2d(x)));
      else *p += x;
      break;
    case TQPK_ACC_COUNT_ROWS: *p += 1; break;
    case TQPK_ACC_COUNT_NOTNULL:
      if (a.type == TQPK_F64) *p += (u2d(x) != (double)TQPK_NULL_INDEX);
      else *p += (static_cast<int64_t>(x) != TQPK_NULL_INDEX);
      break;
    case TQPK_ACC_MIN:
      if (a.type == TQPK_F64) *p = min(*p, f64_ordered(u2d(x)));
      else *p = static_cast<uint64_t>(min(static_cast<int64_t>(*p), static_cast<int64_t>(x)));
      break;
    case TQPK_ACC_MAX:
      if (a.type == TQPK_F64) *p = max(*p, f64_ordered(u2d(x)));
      else *p = static_cast<uint64_t>(max(static_cast<int64_t>(*p), static_cast<int64_t>(x)));
      break;
  }
}

// Merge a value (already in accumulator encoding) into a shared cell atomically.
__device__ __forceinline__ void acc_merge_atomic(uint64_t* p, const tqpk_acc& a, uint64_t v) {
  switch (a.kind) {
    case TQPK_ACC_SUM:
      if (a.type == TQPK_F64) atomicAdd(reinterpret_cast<double*>(p), u2d(v));
      else atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
      break;
    case TQPK_ACC_COUNT_ROWS:
    case TQPK_ACC_COUNT_NOTNULL: atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v); break;
    case TQPK_ACC_MIN:
      if (a.type == TQPK_F64) atomicMin(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
      else atomicMin(reinterpret_cast<long long*>(p), (long long)v);
      break;
    case TQPK_ACC_MAX:
      if (a.type == TQPK_F64) atomicMax(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
      else atomicMax(reinterpret_cast<long long*>(p), (long long)v);
      break;
  }
}

// Accumulator encoding of one row's contribution.
__device__ __forceinline__ uint64_t acc_value(const tqpk_acc& a, uint64_t x) {
  switch (a.kind) {
    case TQPK_ACC_SUM: return x;
    case TQPK_ACC_COUNT_ROWS: return 1ull;
    case TQPK_ACC_COUNT_NOTNULL:
      return a.type == TQPK_F64 ? (u2d(x) != (double)TQPK_NULL_INDEX) : (static_cast<int64_t>(x) != TQPK_NULL_INDEX);
    default: return a.type == TQPK_F64 ? f64_ordered(u2d(x)) : x;
  }
}

template <int MODE>
__device__ __forceinline__ void acc_row(const tqpk_groupby_spec& S, uint64_t* sm, uint64_t* gacc, int64_t K,
                                        int64_t slot, int a, uint64_t x) {
  if (MODE == 1) {
    acc_plain(&sm[(slot * S.n_accs + a) * blockDim.x + threadIdx.x], S.accs[a], x);
  } else if (MODE == 2) {
    acc_merge_atomic(&sm[slot * S.n_accs + a], S.accs[a], acc_value(S.accs[a], x));
  } else {
    acc_merge_global(&gacc[(int64_t)a * K + slot], S.accs[a], acc_value(S.accs[a], x));
  }
}

__device__ __forceinline__ uint64_t combine_plain(const tqpk_acc& a, uint64_t x, uint64_t y) {
  switch (a.kind) {
    case TQPK_ACC_SUM: return a.type == TQPK_F64 ? d2u(__dadd_rn(u2d(x), u2d(y))) : x + y;
    case TQPK_ACC_COUNT_ROWS:
    case TQPK_ACC_COUNT_NOTNULL: return x + y;
    case TQPK_ACC_MIN:
      return a.type == TQPK_F64 ? min(x, y) : (uint64_t)min((int64_t)x, (int64_t)y);
    default: return a.type == TQPK_F64 ? max(x, y) : (uint64_t)max((int64_t)x, (int64_t)y);
  }
}

enum { MODE_PRIVATE = 1, MODE_SHARED = 2, MODE_GLOBAL = 3 };

template <int MODE>
__global__ void __launch_bounds__(256) k_groupby_dense(const __grid_constant__ tqpk_groupby_spec S,
                                                       const __grid_constant__ tqpk_predicate P, RowFilter F,
                                                       int64_t n, GbDev G, uint64_t* __restrict__ gacc,
                                                       int keys_vec, int cols_vec) {
  extern __shared__ uint64_t sm[];
  const int A = S.n_accs;
  const int T = blockDim.x;
  const int64_t K = G.slots;
  if (MODE == MODE_PRIVATE) {
    for (int64_t i = threadIdx.x; i < K * A * T; i += T) sm[i] = acc_init(S.accs[(i / T) % A]);
  } else if (MODE == MODE_SHARED) {
    for (int64_t i = threadIdx.x; i < K * A; i += T) sm[i] = acc_init(S.accs[i % A]);
  }
  __syncthreads();
  const int64_t groups = (n + 3) >> 2;
  const bool small = S.n_expr <= 16;
  const bool tile = tile_ok(S);
  for (int64_t g = blockIdx.x * (int64_t)T + threadIdx.x; g < groups; g += (int64_t)gridDim.x * T) {
    const int64_t r0 = g << 2;
    const uint32_t b = filter4(F, P, r0, n);
    if (!b) continue;
    int64_t slot[4] = {0, 0, 0, 0};
    for (int k = 0; k < G.nk; ++k) {
      int64_t x[4];
      ld4_int(S.keys[k], S.key_dtypes[k], r0, n, keys_vec, x);
#pragma unroll
      for (int j = 0; j < 4; ++j) slot[j] += (x[j] - G.kmin[k]) * G.kstride[k];
    }
    if (tile) {
      ColTile4 T;
      load_cols4(S, r0, n, cols_vec, T);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (!((b >> j) & 1u)) continue;
        uint64_t r[16];
        expr_eval_tile<16>(S.expr, S.n_expr, S.col_dtypes, T, j, r);
        for (int a = 0; a < A; ++a) acc_row<MODE>(S, sm, gacc, K, slot[j], a, reg_pick<16>(r, S.accs[a].reg));
      }
      continue;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((b >> j) & 1u)) continue;
      if (small) {
        uint64_t r[16];
        expr_eval_small<16>(S.expr, S.n_expr, S.cols, S.col_dtypes, r0 + j, r);
        for (int a = 0; a < A; ++a) acc_row<MODE>(S, sm, gacc, K, slot[j], a, reg_pick<16>(r, S.accs[a].reg));
      } else {
        uint64_t r[TQPK_MAX_EXPR];
        expr_eval_generic(S.expr, S.n_expr, S.cols, S.col_dtypes, r0 + j, r);
        for (int a = 0; a < A; ++a) acc_row<MODE>(S, sm, gacc, K, slot[j], a, r[S.accs[a].reg]);
      }
    }
  }
  if (MODE == MODE_GLOBAL) return;
  __syncthreads();
  // Flush the CTA's table into the global accumulators.
  if (MODE == MODE_PRIVATE) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = T >> 5;
    for (int64_t c = warp; c < K * A; c += nw) {
      const tqpk_acc& a = S.accs[c % A];
      uint64_t v = acc_init(a);
      for (int t = lane; t < T; t += 32) v = combine_plain(a, v, sm[c * T + t]);
#pragma unroll
      for (int o = 16; o; o >>= 1) v = combine_plain(a, v, __shfl_xor_sync(0xffffffffu, v, o));
      if (lane == 0 && v != acc_init(a)) acc_merge_global(&gacc[(c % A) * K + c / A], a, v);
    }
  } else {
    for (int64_t c = threadIdx.x; c < K * A; c += T) {
      const tqpk_acc& a = S.accs[c % A];
      const uint64_t v = sm[c];
      if (v != acc_init(a)) acc_merge_global(&gacc[(c % A) * K + c / A], a, v);
    }
  }
}

// ---------------------------------------------------------------- sparse key spaces
// When the mixed-radix key space is far larger than the rows (several wide keys),
// the packed key (the same mixed-radix number, < 2^62) is the key of an
// open-addressing table of C = 2^k >= 2 x rows slots in global memory (linear
// probing, atomicCAS claims an empty slot), and the accumulators live at the
// claimed slot.  The groups are then sorted by packed key, which is the
// ascending key-tuple order of the dense modes.
constexpr uint64_t kHashEmpty = ~0ull;

__device__ __forceinline__ int64_t hash_slot(uint64_t packed, int64_t C) {
  return (int64_t)((packed * 0x9E3779B97F4A7C15ull) >> 20) & (C - 1);
}

__global__ void k_fill_u64(uint64_t* p, int64_t n, uint64_t v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

__global__ void __launch_bounds__(256) k_groupby_hash(const __grid_constant__ tqpk_groupby_spec S,
                                                      const __grid_constant__ tqpk_predicate P, RowFilter F, int64_t n,
                                                      GbDev G, uint64_t* __restrict__ gacc,
                                                      unsigned long long* __restrict__ hkeys, int keys_vec,
                                                      int cols_vec, int* err) {
  const int A = S.n_accs;
  const int64_t C = G.slots;
  const int64_t groups = (n + 3) >> 2;
  const bool small = S.n_expr <= 16;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = g << 2;
    const uint32_t b = filter4(F, P, r0, n);
    if (!b) continue;
    uint64_t packed[4] = {0, 0, 0, 0};
    for (int k = 0; k < G.nk; ++k) {
      int64_t x[4];
      ld4_int(S.keys[k], S.key_dtypes[k], r0, n, keys_vec, x);
#pragma unroll
      for (int j = 0; j < 4; ++j) packed[j] += (uint64_t)(x[j] - G.kmin[k]) * (uint64_t)G.kstride[k];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((b >> j) & 1u)) continue;
      int64_t h = hash_slot(packed[j], C);
      int64_t probes = 0;
      while (true) {
        const unsigned long long cur = __ldcg(&hkeys[h]);
        if (cur == packed[j]) break;
        if (cur == kHashEmpty) {
          const unsigned long long prev = atomicCAS(&hkeys[h], kHashEmpty, (unsigned long long)packed[j]);
          if (prev == kHashEmpty || prev == packed[j]) break;
        }
        h = (h + 1) & (C - 1);
        if (++probes > C) { set_error(err, TQPK_ECAPACITY); h = -1; break; }   // table full: cannot happen (C >= 2 rows)
      }
      if (h < 0) continue;
      if (small) {
        uint64_t r[16];
        expr_eval_small<16>(S.expr, S.n_expr, S.cols, S.col_dtypes, r0 + j, r);
        for (int a = 0; a < A; ++a)
          acc_merge_global(&gacc[(int64_t)a * C + h], S.accs[a], acc_value(S.accs[a], reg_pick<16>(r, S.accs[a].reg)));
      } else {
        uint64_t r[TQPK_MAX_EXPR];
        expr_eval_generic(S.expr, S.n_expr, S.cols, S.col_dtypes, r0 + j, r);
        for (int a = 0; a < A; ++a)
          acc_merge_global(&gacc[(int64_t)a * C + h], S.accs[a], acc_value(S.accs[a], r[S.accs[a].reg]));
      }
    }
  }
}

// Appends (packed key, slot) of every occupied slot (unordered).
__global__ void k_hash_collect(const uint64_t* __restrict__ count0, const unsigned long long* __restrict__ hkeys,
                               int64_t C, int64_t* __restrict__ pk, int64_t* __restrict__ cslot,
                               unsigned long long* counter, int64_t cap) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < C;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = base + lane;
    const bool occ = s < C && count0[s] != 0;
    const unsigned bal = __ballot_sync(0xffffffffu, occ);
    if (!bal) continue;
    unsigned long long at = 0;
    if (lane == 0) at = atomicAdd(counter, (unsigned long long)__popc(bal));
    at = __shfl_sync(0xffffffffu, at, 0) + __popc(bal & ((1u << lane) - 1u));
    if (occ && (int64_t)at < cap) {
      pk[at] = (int64_t)hkeys[s];
      cslot[at] = s;
    }
  }
}

__global__ void k_init_accs(const __grid_constant__ tqpk_groupby_spec S, uint64_t* gacc, int64_t K) {
  const int64_t total = K * S.n_accs;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    gacc[i] = acc_init(S.accs[i / K]);
}

// Counts occupied slots (accumulator 0 is the row count).
__global__ void k_count_groups(const uint64_t* cnt, int64_t K, unsigned long long* groups) {
  unsigned local = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < K; i += (int64_t)gridDim.x * blockDim.x)
    local += cnt[i] != 0;
  local = __reduce_add_sync(0xffffffffu, local);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(groups, (unsigned long long)local);
}

__global__ void k_count_one(unsigned long long* groups) { *groups = 1; }

__global__ void k_groups_or_error(const int* err, const unsigned long long* groups, int64_t* out) {
  *out = *err ? (int64_t)*err : (int64_t)*groups;
}

struct EmitOut {
  int n;
  int op[TQPK_MAX_ACCS];
  int a[TQPK_MAX_ACCS];
  int b[TQPK_MAX_ACCS];
  int dt[TQPK_MAX_ACCS];
  void* col[TQPK_MAX_ACCS];
  void* key[TQPK_MAX_KEYS];
  int key_dt[TQPK_MAX_KEYS];
};

__device__ __forceinline__ void store_as(void* col, int dt, int64_t i, uint64_t v, bool is_f64) {
  switch (dt) {
    case TQPK_F64: static_cast<double*>(col)[i] = is_f64 ? u2d(v) : (double)(int64_t)v; break;
    case TQPK_I64: static_cast<int64_t*>(col)[i] = is_f64 ? (int64_t)u2d(v) : (int64_t)v; break;
    case TQPK_I32: static_cast<int32_t*>(col)[i] = (int32_t)(int64_t)v; break;
    case TQPK_I8: static_cast<int8_t*>(col)[i] = (int8_t)(int64_t)v; break;
    default: static_cast<uint8_t*>(col)[i] = (uint8_t)(int64_t)v; break;
  }
}

// Ordered emission of the occupied slots (ascending slot = ascending key tuple).
__global__ void __launch_bounds__(kBlock) k_emit_dense(const __grid_constant__ tqpk_groupby_spec S, GbDev G,
                                                       const uint64_t* __restrict__ gacc, int force_one,
                                                       const __grid_constant__ EmitOut E, uint64_t* status,
                                                       int* tile_ctr, int* err) {
  __shared__ int s_tile;
  __shared__ uint64_t s_excl;
  __shared__ int sw[kBlock / 32 + 1];
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1);
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t K = G.slots;
  const int64_t s0 = tile * kTile + threadIdx.x * kItems;
  uint32_t bits = 0;
  for (int j = 0; j < kItems; ++j) {
    const int64_t s = s0 + j;
    if (s < K && (gacc[s] != 0 || force_one)) bits |= 1u << j;
  }
  int total;
  const int excl = block_excl_scan<kBlock, int>(__popc(bits), total, sw);
  if (threadIdx.x < 32) {
    uint64_t e = lookback_warp(status, tile, (uint64_t)total, err);
    if (threadIdx.x == 0) s_excl = e;
  }
  // The tile's groups in output order (entry r: the slot offset in the tile; its output row is
  // s_excl + r), then every (group, column) pair on its own thread.  A group's outputs (an average is an FP64
  // division, a key a division of the slot index) are independent, and on this part FP64 runs at
  // 1/64 rate: one thread per group made a few groups a long serial chain (6 groups, 8 outputs:
  // 25 us for one CTA).
  __shared__ uint16_t e_off[kTile];
  {
    int r = excl;
    uint32_t b = bits;
    while (b) {
      const int j = __ffs(b) - 1;
      b &= b - 1;
      e_off[r++] = (uint16_t)(threadIdx.x * kItems + j);
    }
  }
  __syncthreads();
  const int per = G.nk + E.n;                       // columns written per group
  const bool small = K < (int64_t(1) << 31);       // slot indices fit 32 bits: 32-bit key decoding
  for (int w = threadIdx.x; w < total * per; w += kBlock) {
    const int r = w / per, c = w - r * per;
    const int64_t s = tile * kTile + e_off[r];
    const int64_t pos = (int64_t)s_excl + r;
    if (c < G.nk) {
      const int k = c;
      const int64_t q = small ? (int64_t)(((uint32_t)s / (uint32_t)G.kstride[k]) % (uint32_t)G.krange[k])
                              : (s / G.kstride[k]) % G.krange[k];
      store_as(E.key[k], E.key_dt[k], pos, (uint64_t)(G.kmin[k] + q), false);
      continue;
    }
    const int o = c - G.nk;
    const tqpk_acc& a = S.accs[E.a[o]];
    uint64_t v = gacc[(int64_t)E.a[o] * K + s];
    bool f = a.type == TQPK_F64 && a.kind != TQPK_ACC_COUNT_ROWS && a.kind != TQPK_ACC_COUNT_NOTNULL;
    if (f && (a.kind == TQPK_ACC_MIN || a.kind == TQPK_ACC_MAX)) v = d2u(f64_from_ordered(v));
    if (E.op[o] == TQPK_OUT_AVG) {
      const double num = f ? u2d(v) : (double)(int64_t)v;
      const double den = (double)(int64_t)gacc[(int64_t)E.b[o] * K + s];
      v = d2u(__ddiv_rn(num, den));
      f = true;
    } else if (a.kind == TQPK_ACC_COUNT_ROWS || a.kind == TQPK_ACC_COUNT_NOTNULL) {
      f = false;
    }
    store_as(E.col[o], E.dt[o], pos, v, f);
  }
}

// Groups of a hash table in key order: position j holds slot cslot[perm[j]].
__global__ void k_emit_hash(const __grid_constant__ tqpk_groupby_spec S, GbDev G, const uint64_t* __restrict__ gacc,
                            int64_t groups, const int64_t* __restrict__ pk, const int64_t* __restrict__ cslot,
                            const int64_t* __restrict__ perm, const __grid_constant__ EmitOut E) {
  const int64_t C = G.slots;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < groups; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm[j];
    const int64_t s = cslot[i];
    const uint64_t packed = (uint64_t)pk[i];
    for (int k = 0; k < G.nk; ++k) {
      const int64_t key = G.kmin[k] + (int64_t)((packed / (uint64_t)G.kstride[k]) % (uint64_t)G.krange[k]);
      store_as(E.key[k], E.key_dt[k], j, (uint64_t)key, false);
    }
    for (int o = 0; o < E.n; ++o) {
      const tqpk_acc& a = S.accs[E.a[o]];
      uint64_t v = gacc[(int64_t)E.a[o] * C + s];
      bool f = a.type == TQPK_F64 && a.kind != TQPK_ACC_COUNT_ROWS && a.kind != TQPK_ACC_COUNT_NOTNULL;
      if (f && (a.kind == TQPK_ACC_MIN || a.kind == TQPK_ACC_MAX)) v = d2u(f64_from_ordered(v));
      if (E.op[o] == TQPK_OUT_AVG) {
        const double num = f ? u2d(v) : (double)(int64_t)v;
        const double den = (double)(int64_t)gacc[(int64_t)E.b[o] * C + s];
        v = d2u(__ddiv_rn(num, den));
        f = true;
      } else if (a.kind == TQPK_ACC_COUNT_ROWS || a.kind == TQPK_ACC_COUNT_NOTNULL) {
        f = false;
      }
      store_as(E.col[o], E.dt[o], j, v, f);
    }
  }
}

// Hash-mode workspace: [512 header][acc table A x C][keys C][packed keys C][slots C][sort workspace]
struct HashLayout {
  uint64_t* gacc;
  unsigned long long* hkeys;
  int64_t* pk;
  int64_t* cslot;
  void* sort_ws;
  size_t sort_bytes;
};

static size_t hash_ws_bytes(int64_t C, int A) {
  return 512 + align_up((size_t)C * A * 8, 256) + 3 * align_up((size_t)C * 8, 256) + sort_ws_bytes(C / 2 + 1) + 256;
}

static HashLayout hash_layout(void* ws, int64_t C, int A) {
  HashLayout H;
  char* p = static_cast<char*>(ws) + 512;
  H.gacc = reinterpret_cast<uint64_t*>(p);
  p += align_up((size_t)C * A * 8, 256);
  H.hkeys = reinterpret_cast<unsigned long long*>(p);
  p += align_up((size_t)C * 8, 256);
  H.pk = reinterpret_cast<int64_t*>(p);
  p += align_up((size_t)C * 8, 256);
  H.cslot = reinterpret_cast<int64_t*>(p);
  p += align_up((size_t)C * 8, 256);
  H.sort_ws = p;
  H.sort_bytes = sort_ws_bytes(C / 2 + 1);
  return H;
}

// ---------------------------------------------------------------- host side
static GbDev to_dev(const tqpk_gb_plan& p, int nk) {
  GbDev G;
  G.nk = nk;
  for (int k = 0; k < TQPK_MAX_KEYS; ++k) {
    G.kmin[k] = p.key_min[k];
    G.kstride[k] = p.key_stride[k] ? p.key_stride[k] : 1;
    G.krange[k] = p.key_range[k] ? p.key_range[k] : 1;
  }
  G.slots = p.slots;
  return G;
}

// has_rows: the key and value columns are read (empty inputs may carry null column pointers)
static int check_spec(const tqpk_groupby_spec* S, bool has_rows = true) {
  if (!S) return TQPK_EINVAL;
  if (S->n_keys < 0 || S->n_keys > TQPK_MAX_KEYS || S->n_cols < 0 || S->n_cols > TQPK_MAX_COLS ||
      S->n_expr < 0 || S->n_expr > TQPK_MAX_EXPR || S->n_accs < 1 || S->n_accs > TQPK_MAX_ACCS)
    return TQPK_EINVAL;
  if (S->accs[0].kind != TQPK_ACC_COUNT_ROWS) return TQPK_EINVAL;  // accumulator 0 marks occupied groups
  for (int k = 0; k < S->n_keys; ++k) {
    if (!is_int_dtype(S->key_dtypes[k])) return TQPK_EDTYPE;
    if (has_rows && !S->keys[k]) return TQPK_EINVAL;
  }
  for (int c = 0; c < S->n_cols; ++c) {
    if (!dtype_size(S->col_dtypes[c])) return TQPK_EDTYPE;
    if (has_rows && !S->cols[c]) return TQPK_EINVAL;
  }
  for (int i = 0; i < S->n_expr; ++i) {
    const tqpk_expr_insn& X = S->expr[i];
    if (X.type != TQPK_F64 && X.type != TQPK_I64 && X.type != TQPK_F32) return TQPK_EDTYPE;
    if (X.op == TQPK_X_COL && (X.col < 0 || X.col >= S->n_cols || X.type == TQPK_F32)) return TQPK_EINVAL;
    if (X.op >= TQPK_X_ADD && X.op <= TQPK_X_DIV && (X.a < 0 || X.a >= i || X.b < 0 || X.b >= i)) return TQPK_EINVAL;
    if (X.op >= TQPK_X_ADD && X.op <= TQPK_X_DIV && (S->expr[X.a].type != X.type || S->expr[X.b].type != X.type))
      return TQPK_EDTYPE;                    // operands of the register's own type (conversions are explicit)
    if (X.op == TQPK_X_TOF64 && (X.a < 0 || X.a >= i || X.type != TQPK_F64 || S->expr[X.a].type != TQPK_I64))
      return TQPK_EINVAL;
    if (X.op == TQPK_X_TOF32 && (X.a < 0 || X.a >= i || X.type != TQPK_F32 || S->expr[X.a].type != TQPK_I64))
      return TQPK_EINVAL;
    if (X.op == TQPK_X_F32TOF64 && (X.a < 0 || X.a >= i || X.type != TQPK_F64 || S->expr[X.a].type != TQPK_F32))
      return TQPK_EINVAL;
    if (X.op == TQPK_X_DIV && X.type == TQPK_I64) return TQPK_EUNSUPPORTED;
    if (X.wrap && (X.type != TQPK_I64 || X.op < TQPK_X_ADD || X.op > TQPK_X_MUL ||
                   (X.wrap != TQPK_I8 && X.wrap != TQPK_U8 && X.wrap != TQPK_I32)))
      return TQPK_EINVAL;
    if (X.op == TQPK_X_SELECT) {
      if (X.a < 0 || X.a >= i || X.b < 0 || X.b >= i || X.col < 0 || X.col >= i) return TQPK_EINVAL;
      if (S->expr[X.a].type != TQPK_I64 || S->expr[X.b].type != X.type || S->expr[X.col].type != X.type)
        return TQPK_EDTYPE;
    }
    if (X.op == TQPK_X_YEAR && (X.a < 0 || X.a >= i || X.type != TQPK_I64 || S->expr[X.a].type != TQPK_I64))
      return TQPK_EINVAL;
    if (X.op < TQPK_X_COL || X.op > TQPK_X_F32TOF64) return TQPK_EINVAL;
  }
  for (int a = 0; a < S->n_accs; ++a) {
    const tqpk_acc& A = S->accs[a];
    if (A.kind < TQPK_ACC_SUM || A.kind > TQPK_ACC_MAX) return TQPK_EINVAL;
    if (A.kind != TQPK_ACC_COUNT_ROWS && (A.reg < 0 || A.reg >= S->n_expr)) return TQPK_EINVAL;
    if (A.kind != TQPK_ACC_COUNT_ROWS && S->expr[A.reg].type == TQPK_F32) return TQPK_EDTYPE;  // accumulate float64
  }
  return TQPK_OK;
}

constexpr int64_t kPrivateBudget = 96 * 1024;  // bytes of shared memory per CTA for private tables

// Slots, table placement and workspace of a plan from the key ranges and the row count.
static int plan_from_ranges(const tqpk_groupby_spec* S, const int64_t* mn, const int64_t* mx, int64_t rows,
                            tqpk_gb_plan* plan) {
  plan->n_rows = rows;
  int64_t K = 1;
  bool overflow = false;
  for (int k = S->n_keys - 1; k >= 0; --k) {
    const int64_t range = rows ? (mx[k] - mn[k] + 1) : 1;
    if (range <= 0 || range > (int64_t(1) << 40)) overflow = true;
    plan->key_min[k] = rows ? mn[k] : 0;
    plan->key_range[k] = range;
    plan->key_stride[k] = K;
    if (!overflow && K > (int64_t(1) << 62) / range) overflow = true;
    if (!overflow) K *= range;
  }
  if (S->n_keys > 0 && rows == 0) K = 1;  // no group at all; keep a 1-slot table
  const int64_t A = S->n_accs;
  if (S->n_keys == 0) {
    plan->mode = TQPK_GB_GLOBAL_ONE;
  } else if (overflow || K > std::max<int64_t>(4 * rows, int64_t(1) << 20)) {
    plan->mode = TQPK_GB_HASH;  // key space too sparse for a dense table
  } else if (K * A * 8 * 256 <= kPrivateBudget) {
    plan->mode = TQPK_GB_DENSE_PRIVATE;
  } else if (K * A * 8 * 128 <= kPrivateBudget) {
    plan->mode = TQPK_GB_DENSE_PRIVATE;
  } else if (K * A * 8 <= kPrivateBudget) {
    plan->mode = TQPK_GB_DENSE_SHARED;
  } else {
    plan->mode = TQPK_GB_DENSE_GLOBAL;
  }
  if (plan->mode == TQPK_GB_GLOBAL_ONE) K = 1;
  plan->threads = (plan->mode == TQPK_GB_DENSE_PRIVATE && K * A * 8 * 256 > kPrivateBudget) ? 128 : 256;
  if (plan->mode == TQPK_GB_GLOBAL_ONE) plan->threads = (K * A * 8 * 256 <= kPrivateBudget) ? 256 : 128;
  plan->slots = K;
  if (plan->mode == TQPK_GB_HASH) {
    if (overflow) {            // the packed key would not fit 62 bits
      plan->ws_bytes = 0;
      return TQPK_EUNSUPPORTED;
    }
    int64_t C = 1024;
    while (C < 2 * rows) C <<= 1;
    plan->slots = C;
    plan->threads = 256;
    plan->ws_bytes = hash_ws_bytes(C, (int)A);
    return TQPK_OK;
  }
  plan->ws_bytes = 512 + align_up((size_t)(K * A * 8), 256) + compact_status_bytes(K);
  return TQPK_OK;
}

}  // namespace tqpk

using namespace tqpk;

extern "C" int tqpk_groupby_plan(const tqpk_groupby_spec* S, const tqpk_predicate* pred, const uint8_t* mask,
                                 int64_t n, tqpk_gb_plan* plan, void* scratch, tqpk_stream stream) {
  int rc = check_spec(S, n > 0);
  if (rc) return rc;
  if (n > 0 && (rc = check_pred(pred))) return rc;   // an empty input never evaluates its predicate
  if (!plan || n < 0) return TQPK_EINVAL;
  *plan = tqpk_gb_plan{};
  int64_t mn[TQPK_MAX_KEYS], mx[TQPK_MAX_KEYS], rows = 0;
  rc = key_ranges(pred, mask, n, S->n_keys, S->keys, S->key_dtypes, mn, mx, &rows, scratch,
                  static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  return plan_from_ranges(S, mn, mx, rows, plan);
}

// The plan of a key domain known without a pass over the data (table statistics:
// [key_min[k], key_max[k]] per key), for callers that run the group-by with no host
// synchronisation (a captured graph, a serving loop).  n_rows is the row count the
// hash-mode sizing assumes (the input's rows); dense modes do not depend on it.
extern "C" int tqpk_groupby_plan_domains(const tqpk_groupby_spec* S, const int64_t* key_min, const int64_t* key_max,
                                         int64_t n_rows, tqpk_gb_plan* plan) {
  int rc = check_spec(S, false);
  if (rc) return rc;
  if (!plan || n_rows < 0 || (S->n_keys > 0 && (!key_min || !key_max))) return TQPK_EINVAL;
  for (int k = 0; k < S->n_keys; ++k)
    if (key_max[k] < key_min[k]) return TQPK_EINVAL;
  *plan = tqpk_gb_plan{};
  return plan_from_ranges(S, key_min, key_max, std::max<int64_t>(n_rows, 1), plan);
}

extern "C" int tqpk_groupby_run(const tqpk_groupby_spec* S, const tqpk_gb_plan* plan, const tqpk_predicate* pred,
                                const uint8_t* mask, int64_t n, void* ws, size_t ws_bytes, int64_t* h_groups,
                                tqpk_stream stream) {
  int rc = check_spec(S, n > 0);
  if (rc) return rc;
  if (n > 0 && (rc = check_pred(pred))) return rc;   // an empty input never evaluates its predicate
  if (!plan || !ws || ws_bytes < plan->ws_bytes || !h_groups || n < 0) return !ws || ws_bytes < (plan ? plan->ws_bytes : 0) ? TQPK_ENOMEM : TQPK_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (plan->mode == TQPK_GB_HASH) {
    if (!plan->ws_bytes) return TQPK_EUNSUPPORTED;
    const int64_t C = plan->slots;
    HashLayout H = hash_layout(ws, C, S->n_accs);
    char* base = static_cast<char*>(ws);
    unsigned long long* d_groups = reinterpret_cast<unsigned long long*>(base);
    int* err = reinterpret_cast<int*>(base + 8);
    TQPK_CUDA(cudaMemsetAsync(base, 0, 16, s));
    k_init_accs<<<grid_for(C * S->n_accs, 4), kBlock, 0, s>>>(*S, H.gacc, C);
    TQPK_CHECK_LAUNCH();
    k_fill_u64<<<grid_for(C, 4), kBlock, 0, s>>>(reinterpret_cast<uint64_t*>(H.hkeys), C, kHashEmpty);
    TQPK_CHECK_LAUNCH();
    if (n > 0 && plan->n_rows > 0) {
      bool kvec = true;
      for (int k = 0; k < S->n_keys; ++k) kvec = kvec && aligned16(S->keys[k]);
      const GbDev G = to_dev(*plan, S->n_keys);
      timing_before(KID_GROUPBY, s);
      k_groupby_hash<<<grid_for((n + 3) / 4, 8), 256, 0, s>>>(*S, *pred_or_empty(pred), make_filter(pred, mask), n, G,
                                                               H.gacc, H.hkeys, kvec, spec_cols_vec(S) ? 1 : 0, err);
      timing_after(KID_GROUPBY, s);
      TQPK_CHECK_LAUNCH();
      k_count_groups<<<grid_for(C, 4), kBlock, 0, s>>>(H.gacc, C, d_groups);
      TQPK_CHECK_LAUNCH();
    }
    unsigned long long h[2] = {0, 0};
    TQPK_CUDA(cudaMemcpyAsync(h, base, 16, cudaMemcpyDeviceToHost, s));
    TQPK_CUDA(cudaStreamSynchronize(s));
    const int e = (int)(h[1] & 0xffffffffu);
    if (e) return e;
    *h_groups = (int64_t)h[0];
    return TQPK_OK;
  }
  const int64_t K = plan->slots, A = S->n_accs;
  char* base = static_cast<char*>(ws);
  unsigned long long* d_groups = reinterpret_cast<unsigned long long*>(base);
  uint64_t* gacc = reinterpret_cast<uint64_t*>(base + 512);
  TQPK_CUDA(cudaMemsetAsync(d_groups, 0, 8, s));
  k_init_accs<<<grid_for(K * A, 4), kBlock, 0, s>>>(*S, gacc, K);
  TQPK_CHECK_LAUNCH();
  const GbDev G = to_dev(*plan, S->n_keys);
  const RowFilter F = make_filter(pred, mask);
  bool kvec = true;
  for (int k = 0; k < S->n_keys; ++k) kvec = kvec && aligned16(S->keys[k]);
  const tqpk_predicate& P = *pred_or_empty(pred);
  if (n > 0 && plan->n_rows > 0) {
    const int T = plan->threads;
    const int64_t groups4 = (n + 3) / 4;
    if (plan->mode == TQPK_GB_DENSE_PRIVATE || plan->mode == TQPK_GB_GLOBAL_ONE) {
      const size_t smem = (size_t)(K * A * 8 * T);
      TQPK_CUDA(cudaFuncSetAttribute(k_groupby_dense<MODE_PRIVATE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
      int g = (int)std::min<int64_t>((groups4 + T - 1) / T, (int64_t)num_sms() * 2);
      timing_before(KID_GROUPBY, s);
      k_groupby_dense<MODE_PRIVATE><<<std::max(g, 1), T, smem, s>>>(*S, P, F, n, G, gacc, kvec, spec_cols_vec(S) ? 1 : 0);
      timing_after(KID_GROUPBY, s);
    } else if (plan->mode == TQPK_GB_DENSE_SHARED) {
      const size_t smem = (size_t)(K * A * 8);
      TQPK_CUDA(cudaFuncSetAttribute(k_groupby_dense<MODE_SHARED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
      int g = (int)std::min<int64_t>((groups4 + 255) / 256, (int64_t)num_sms() * 2);
      timing_before(KID_GROUPBY, s);
      k_groupby_dense<MODE_SHARED><<<std::max(g, 1), 256, smem, s>>>(*S, P, F, n, G, gacc, kvec, spec_cols_vec(S) ? 1 : 0);
      timing_after(KID_GROUPBY, s);
    } else {
      int g = grid_for(groups4, 8);
      timing_before(KID_GROUPBY, s);
      k_groupby_dense<MODE_GLOBAL><<<g, 256, 0, s>>>(*S, P, F, n, G, gacc, kvec, spec_cols_vec(S) ? 1 : 0);
      timing_after(KID_GROUPBY, s);
    }
    TQPK_CHECK_LAUNCH();
  }
  int64_t groups = 0;
  if (S->n_keys == 0) {
    groups = 1;  // a global aggregate always has one group (aggregate.py:291-295)
  } else if (plan->n_rows > 0) {
    k_count_groups<<<grid_for(K, 4), kBlock, 0, s>>>(gacc, K, d_groups);
    TQPK_CHECK_LAUNCH();
    unsigned long long h = 0;
    TQPK_CUDA(cudaMemcpyAsync(&h, d_groups, 8, cudaMemcpyDeviceToHost, s));
    TQPK_CUDA(cudaStreamSynchronize(s));
    groups = (int64_t)h;
  } else {
    TQPK_CUDA(cudaStreamSynchronize(s));
  }
  *h_groups = groups;
  return TQPK_OK;
}

extern "C" int tqpk_groupby_emit(const tqpk_groupby_spec* S, const tqpk_gb_plan* plan, void* ws, int64_t groups,
                                 void* const* out_keys, int32_t n_out, const int32_t* ops, void* const* out_cols,
                                 tqpk_stream stream) {
  int rc = check_spec(S, false);
  if (rc) return rc;
  if (!plan || !ws || n_out < 0 || n_out > TQPK_MAX_ACCS || groups < 0) return TQPK_EINVAL;
  if (plan->mode == TQPK_GB_HASH && !plan->ws_bytes) return TQPK_EUNSUPPORTED;
  if (groups == 0) return TQPK_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  EmitOut E;
  E.n = n_out;
  for (int o = 0; o < n_out; ++o) {
    E.op[o] = ops[4 * o];
    E.a[o] = ops[4 * o + 1];
    E.b[o] = ops[4 * o + 2];
    E.dt[o] = ops[4 * o + 3];
    E.col[o] = out_cols[o];
    if (E.a[o] < 0 || E.a[o] >= S->n_accs || !E.col[o] || !dtype_size(E.dt[o])) return TQPK_EINVAL;
    if (E.op[o] == TQPK_OUT_AVG && (E.b[o] < 0 || E.b[o] >= S->n_accs)) return TQPK_EINVAL;
  }
  for (int k = 0; k < S->n_keys; ++k) {
    if (!out_keys[k]) return TQPK_EINVAL;
    E.key[k] = out_keys[k];
    E.key_dt[k] = S->key_dtypes[k];
  }
  const int64_t K = plan->slots, A = S->n_accs;
  char* base = static_cast<char*>(ws);
  if (plan->mode == TQPK_GB_HASH) {
    // the occupied slots (unordered), sorted by packed key = ascending key tuple
    HashLayout H = hash_layout(ws, K, (int)A);
    unsigned long long* counter = reinterpret_cast<unsigned long long*>(base + 16);
    TQPK_CUDA(cudaMemsetAsync(counter, 0, 8, s));
    k_hash_collect<<<grid_for(K, 4), kBlock, 0, s>>>(H.gacc, H.hkeys, K, H.pk, H.cslot, counter, groups);
    TQPK_CHECK_LAUNCH();
    const int64_t* perm = nullptr;
    int rc2 = sort_pairs(H.pk, TQPK_I64, 0, nullptr, groups, H.sort_ws, H.sort_bytes, s, &perm);
    if (rc2) return rc2;
    const GbDev G = to_dev(*plan, S->n_keys);
    k_emit_hash<<<grid_for(groups, 4), kBlock, 0, s>>>(*S, G, H.gacc, groups, H.pk, H.cslot, perm, E);
    TQPK_CHECK_LAUNCH();
    TQPK_CUDA(cudaStreamSynchronize(s));
    return TQPK_OK;
  }
  uint64_t* gacc = reinterpret_cast<uint64_t*>(base + 512);
  void* cws = base + 512 + align_up((size_t)(K * A * 8), 256);
  const int64_t tiles = (K + kTile - 1) / kTile;
  WsCursor cur(cws, compact_status_bytes(K));
  int* ctl = cur.take<int>(64);
  uint64_t* status = cur.take<uint64_t>(tiles);
  if (!ctl || !status) return TQPK_ENOMEM;
  TQPK_CUDA(cudaMemsetAsync(cws, 0, cur.off, s));
  const GbDev G = to_dev(*plan, S->n_keys);
  k_emit_dense<<<(int)tiles, kBlock, 0, s>>>(*S, G, gacc, S->n_keys == 0 ? 1 : 0, E, status, ctl, ctl + 1);
  TQPK_CHECK_LAUNCH();
  int err = 0;
  TQPK_CUDA(cudaMemcpyAsync(&err, ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  return err ? err : TQPK_OK;
}

// tqpk_groupby_emit without a host synchronisation: the group count is
// counted on the device and written to *d_groups_out (a negative status
// there if the emit's look-back failed).  The output columns must hold
// plan->slots rows (the largest possible group count).
extern "C" int tqpk_groupby_emit_async(const tqpk_groupby_spec* S, const tqpk_gb_plan* plan, void* ws,
                                       void* const* out_keys, int32_t n_out, const int32_t* ops,
                                       void* const* out_cols, int64_t* d_groups_out, tqpk_stream stream) {
  int rc = check_spec(S, false);
  if (rc) return rc;
  if (!plan || !ws || !d_groups_out || n_out < 0 || n_out > TQPK_MAX_ACCS) return TQPK_EINVAL;
  if (plan->mode == TQPK_GB_HASH) return TQPK_EUNSUPPORTED;
  EmitOut E;
  E.n = n_out;
  for (int o = 0; o < n_out; ++o) {
    E.op[o] = ops[4 * o];
    E.a[o] = ops[4 * o + 1];
    E.b[o] = ops[4 * o + 2];
    E.dt[o] = ops[4 * o + 3];
    E.col[o] = out_cols[o];
    if (E.a[o] < 0 || E.a[o] >= S->n_accs || !E.col[o] || !dtype_size(E.dt[o])) return TQPK_EINVAL;
    if (E.op[o] == TQPK_OUT_AVG && (E.b[o] < 0 || E.b[o] >= S->n_accs)) return TQPK_EINVAL;
  }
  for (int k = 0; k < S->n_keys; ++k) {
    if (!out_keys[k]) return TQPK_EINVAL;
    E.key[k] = out_keys[k];
    E.key_dt[k] = S->key_dtypes[k];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t K = plan->slots, A = S->n_accs;
  char* base = static_cast<char*>(ws);
  unsigned long long* d_groups = reinterpret_cast<unsigned long long*>(base);
  uint64_t* gacc = reinterpret_cast<uint64_t*>(base + 512);
  void* cws = base + 512 + align_up((size_t)(K * A * 8), 256);
  const int64_t tiles = (K + kTile - 1) / kTile;
  WsCursor cur(cws, compact_status_bytes(K));
  int* ctl = cur.take<int>(64);
  uint64_t* status = cur.take<uint64_t>(tiles);
  if (!ctl || !status) return TQPK_ENOMEM;
  TQPK_CUDA(cudaMemsetAsync(cws, 0, cur.off, s));
  TQPK_CUDA(cudaMemsetAsync(d_groups, 0, 8, s));
  if (S->n_keys == 0) {
    k_count_one<<<1, 1, 0, s>>>(d_groups);
  } else {
    k_count_groups<<<grid_for(K, 4), kBlock, 0, s>>>(gacc, K, d_groups);
  }
  TQPK_CHECK_LAUNCH();
  const GbDev G = to_dev(*plan, S->n_keys);
  k_emit_dense<<<(int)tiles, kBlock, 0, s>>>(*S, G, gacc, S->n_keys == 0 ? 1 : 0, E, status, ctl, ctl + 1);
  TQPK_CHECK_LAUNCH();
  k_groups_or_error<<<1, 1, 0, s>>>(ctl + 1, d_groups, d_groups_out);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

// Stages of tqpk_groupby_run for callers that launch their own accumulation
// kernel (the runtime-compiled one): prepare zeroes/initialises the table,
// count counts the occupied slots (synchronises).
extern "C" int tqpk_groupby_prepare(const tqpk_groupby_spec* S, const tqpk_gb_plan* plan, void* ws, size_t ws_bytes,
                                    tqpk_stream stream) {
  int rc = check_spec(S, false);
  if (rc) return rc;
  if (!plan || !ws) return TQPK_EINVAL;
  if (ws_bytes < plan->ws_bytes) return TQPK_ENOMEM;
  if (plan->mode == TQPK_GB_HASH) return TQPK_EUNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  TQPK_CUDA(cudaMemsetAsync(base, 0, 8, s));
  k_init_accs<<<grid_for(plan->slots * S->n_accs, 4), kBlock, 0, s>>>(*S, reinterpret_cast<uint64_t*>(base + 512),
                                                                       plan->slots);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

extern "C" int tqpk_groupby_count(const tqpk_groupby_spec* S, const tqpk_gb_plan* plan, void* ws, int64_t* h_groups,
                                  tqpk_stream stream) {
  if (!S || !plan || !ws || !h_groups) return TQPK_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  if (S->n_keys == 0) {
    *h_groups = 1;
    return TQPK_OK;
  }
  unsigned long long* d_groups = reinterpret_cast<unsigned long long*>(base);
  k_count_groups<<<grid_for(plan->slots, 4), kBlock, 0, s>>>(reinterpret_cast<const uint64_t*>(base + 512),
                                                            plan->slots, d_groups);
  TQPK_CHECK_LAUNCH();
  unsigned long long h = 0;
  TQPK_CUDA(cudaMemcpyAsync(&h, d_groups, 8, cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  *h_groups = (int64_t)h;
  return TQPK_OK;
}

// Device address of the accumulator table inside a plan's workspace ([n_accs][slots], 8 bytes each).
extern "C" void* tqpk_groupby_table(void* ws) { return ws ? static_cast<char*>(ws) + 512 : nullptr; }
