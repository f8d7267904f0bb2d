// batch.cu - many independent query instances in one persistent launch.
//
// Each instance is one of the two pipeline shapes the plain path runs with
// several launches and host synchronisations per operator (main.py's
// per-operator loop):
//   JOIN     Filter(build), Filter(probe), Join on a unique key, sum(expr) by
//            build key, top-k             -> phases BUILD, PROBE, TOPK
//   GROUPBY  Filter, group by dense keys with the aggregate program, emit the
//            groups in key order           -> phases AGG, COUNT, EMIT
// Every phase of every instance is cut into work items (row or slot ranges,
// sized per instance by the caller's tuning table).  The items are queued
// phase-major: all phase-0 items of all instances, then phase 1, then
// phase 2.  CTAs of one persistent grid take items with an atomic ticket;
// before running an item of phase p, a CTA waits (bounded, with a sleep)
// until every phase p-1 item of the same instance has finished.  Every such
// item was taken earlier by a running CTA, so the wait always ends; on expiry
// the CTA records TQPK_ETIMEOUT and goes on.  The whole batch is one kernel
// (plus the memsets of the instance tables) and can be captured in a CUDA
// graph by the caller.
#include <string.h>

#include <algorithm>

#include "topk.cuh"

namespace tqpk {

enum { BT_JOIN = 1, BT_GROUPBY = 2 };
constexpr int kBatchSmem = 96 * 1024;   // dynamic shared memory of the batch kernel

struct BatchInst {
  int type;
  int k, desc;
  int gb_mode;            // GROUPBY: 1 = per-thread private tables, 2 = one shared-memory table per item, 3 = global atomics
  int64_t n_items[3];
  // JOIN
  const void* b_keys; int b_dt; int64_t nb;
  const void* p_fk; int p_dt; int64_t np;
  int64_t key_min, slots;
  int val_reg;
  int* dir; double* sum; unsigned* occ;
  int64_t* out_keys; double* out_vals; int64_t* out_count;
  // GROUPBY
  int64_t n;
  int nk;
  int64_t kmin[TQPK_MAX_KEYS], kstride[TQPK_MAX_KEYS], krange[TQPK_MAX_KEYS];
  int64_t gslots;
  uint64_t* gacc;                       // [n_accs][gslots]
  int64_t range_slots;                  // slots per COUNT/EMIT item
  int64_t* range_count;                 // [n_items[1]] occupied slots per range
  int n_out;
  int out_op[TQPK_MAX_ACCS], out_a[TQPK_MAX_ACCS], out_b[TQPK_MAX_ACCS], out_dt[TQPK_MAX_ACCS];
  void* out_col[TQPK_MAX_ACCS];
  void* out_key[TQPK_MAX_KEYS];
  int key_dt[TQPK_MAX_KEYS];
  int64_t* out_groups;
  // shared
  int pred_vec0, pred_vec1;
  tqpk_predicate pred0;                 // JOIN: build filter; GROUPBY: the filter
  tqpk_predicate pred1;                 // JOIN: probe filter
  tqpk_groupby_spec spec;               // JOIN: value program; GROUPBY: full program
};

struct WorkItem {
  int inst, phase;
  int64_t begin, end;
};

__device__ __forceinline__ uint32_t batch_mask4(const tqpk_predicate& P, int vec, int64_t r0, int64_t n) {
  if (P.n_insn) return eval_pred4(P, r0, n, vec);
  const int64_t valid = n - r0;
  return valid >= 4 ? 0xfu : (valid <= 0 ? 0u : ((1u << valid) - 1));
}

// ---- accumulator helpers (same encoding as groupby.cu) -----------------------
__device__ __forceinline__ uint64_t b_acc_init(const tqpk_acc& a) {
  if (a.kind == TQPK_ACC_MIN || a.kind == TQPK_ACC_MAX)
    return a.type == TQPK_F64 ? f64_ordered(a.init_f) : static_cast<uint64_t>(a.init_i);
  return 0ull;
}
__device__ __forceinline__ uint64_t b_acc_value(const tqpk_acc& a, uint64_t x) {
  switch (a.kind) {
    case TQPK_ACC_SUM: return x;
    case TQPK_ACC_COUNT_ROWS: return 1ull;
    case TQPK_ACC_COUNT_NOTNULL:
      return a.type == TQPK_F64 ? (u2d(x) != (double)TQPK_NULL_INDEX) : (static_cast<int64_t>(x) != TQPK_NULL_INDEX);
    default: return a.type == TQPK_F64 ? f64_ordered(u2d(x)) : x;
  }
}
__device__ __forceinline__ uint64_t b_combine(const tqpk_acc& a, uint64_t x, uint64_t y) {
  switch (a.kind) {
    case TQPK_ACC_SUM: return a.type == TQPK_F64 ? d2u(__dadd_rn(u2d(x), u2d(y))) : x + y;
    case TQPK_ACC_COUNT_ROWS:
    case TQPK_ACC_COUNT_NOTNULL: return x + y;
    case TQPK_ACC_MIN: return a.type == TQPK_F64 ? min(x, y) : (uint64_t)min((int64_t)x, (int64_t)y);
    default: return a.type == TQPK_F64 ? max(x, y) : (uint64_t)max((int64_t)x, (int64_t)y);
  }
}
__device__ __forceinline__ void b_merge_atomic(uint64_t* p, const tqpk_acc& a, uint64_t v) {
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

// ---- phase bodies ----------------------------------------------------------------
__device__ void join_build_item(const BatchInst& I, int64_t b, int64_t e, int* err) {
  for (int64_t r0 = b + 4 * (int64_t)threadIdx.x; r0 < e; r0 += 4 * (int64_t)blockDim.x) {
    uint32_t m = batch_mask4(I.pred0, I.pred_vec0, r0, I.nb);
    if (!m) continue;
    int64_t x[4];
    ld4_int(I.b_keys, I.b_dt, r0, I.nb, false, x);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((m >> j) & 1u) || r0 + j >= e) continue;
      const int64_t s = x[j] - I.key_min;
      if (s < 0 || s >= I.slots) { set_error(err, TQPK_EINVAL); continue; }
      if (atomicCAS(&I.dir[s], -1, (int)(r0 + j)) != -1) set_error(err, TQPK_EUNSUPPORTED);
    }
  }
}

__device__ void join_probe_item(const BatchInst& I, int64_t b, int64_t e) {
  for (int64_t r0 = b + 4 * (int64_t)threadIdx.x; r0 < e; r0 += 4 * (int64_t)blockDim.x) {
    uint32_t m = batch_mask4(I.pred1, I.pred_vec1, r0, I.np);
    if (!m) continue;
    int64_t x[4];
    ld4_int(I.p_fk, I.p_dt, r0, I.np, false, x);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((m >> j) & 1u) || r0 + j >= e) continue;
      const int64_t s = x[j] - I.key_min;
      if (s < 0 || s >= I.slots || __ldcg(&I.dir[s]) < 0) continue;
      atomicAdd(&I.sum[s], expr_value(I.spec, r0 + j, I.val_reg));
      I.occ[s] = 1u;
    }
  }
}

// One CTA: top-k of the instance's occupied slots (k <= 32).
__device__ void join_topk_item(const BatchInst& I, uint64_t* sk, int64_t* si) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  DenseSumSource src{I.sum, I.occ, I.slots, I.desc};
  WarpList<1> L;
  L.init();
  unsigned valid = 0;
  for (int64_t base = warp * 32; base < I.slots; base += blockDim.x) {
    uint64_t key = ~0ull;
    const bool ok = src.get(base + lane, key);
    valid += ok;
    L.offer(I.k, key, base + lane, ok);
  }
  valid = __reduce_add_sync(0xffffffffu, valid);
  sk[warp * 32 + lane] = L.key[0];
  si[warp * 32 + lane] = L.idx[0];
  __shared__ unsigned long long s_valid;
  if (threadIdx.x == 0) s_valid = 0;
  __syncthreads();
  if (lane == 0) atomicAdd(&s_valid, (unsigned long long)valid);
  __syncthreads();
  if (warp == 0) {
    WarpList<1> M;
    M.init();
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      const int64_t ii = si[w * 32 + lane];
      M.offer(I.k, sk[w * 32 + lane], ii, lane < I.k && ii >= 0);
    }
    const bool v = lane < I.k && M.idx[0] >= 0;
    const int cnt = __popc(__ballot_sync(0xffffffffu, v));
    if (v) {
      I.out_keys[lane] = I.key_min + M.idx[0];
      I.out_vals[lane] = __ldcg(&I.sum[M.idx[0]]);
    }
    if (lane == 0) {
      *I.out_count = cnt;
      if (I.out_groups) *I.out_groups = (int64_t)s_valid;
    }
  }
}

__device__ void gb_agg_item(const BatchInst& I, int64_t b, int64_t e, uint64_t* sm) {
  const tqpk_groupby_spec& S = I.spec;
  const int A = S.n_accs;
  const int T = blockDim.x;
  const int64_t K = I.gslots;
  const bool priv = I.gb_mode == 1;
  const bool shared = I.gb_mode == 2;   // one table per CTA (per item), shared-memory atomics
  if (priv) {
    for (int64_t i = threadIdx.x; i < K * A * T; i += T) sm[i] = b_acc_init(S.accs[(i / T) % A]);
    __syncthreads();
  } else if (shared) {
    for (int64_t i = threadIdx.x; i < K * A; i += T) sm[i] = b_acc_init(S.accs[i % A]);
    __syncthreads();
  }
  const bool small = S.n_expr <= 16;
  for (int64_t r0 = b + 4 * (int64_t)threadIdx.x; r0 < e; r0 += 4 * (int64_t)T) {
    uint32_t m = batch_mask4(I.pred0, I.pred_vec0, r0, I.n);
    if (!m) continue;
    int64_t slot[4] = {0, 0, 0, 0};
    for (int k = 0; k < I.nk; ++k) {
      int64_t x[4];
      ld4_int(S.keys[k], S.key_dtypes[k], r0, I.n, false, x);
#pragma unroll
      for (int j = 0; j < 4; ++j) slot[j] += (x[j] - I.kmin[k]) * I.kstride[k];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((m >> j) & 1u) || r0 + j >= e) continue;
      uint64_t r8[16];
      uint64_t rg[TQPK_MAX_EXPR];
      if (small) expr_eval_small<16>(S.expr, S.n_expr, S.cols, S.col_dtypes, r0 + j, r8);
      else expr_eval_generic(S.expr, S.n_expr, S.cols, S.col_dtypes, r0 + j, rg);
      for (int a = 0; a < A; ++a) {
        const uint64_t x = small ? reg_pick<16>(r8, S.accs[a].reg) : rg[S.accs[a].reg];
        const tqpk_acc& ac = S.accs[a];
        if (priv) {
          uint64_t* p = &sm[(slot[j] * A + a) * T + threadIdx.x];
          *p = b_combine(ac, *p, b_acc_value(ac, x));
        } else if (shared) {
          b_merge_atomic(&sm[slot[j] * A + a], ac, b_acc_value(ac, x));
        } else {
          acc_merge_global(&I.gacc[(int64_t)a * K + slot[j]], ac, b_acc_value(ac, x));
        }
      }
    }
  }
  if (shared) {
    __syncthreads();
    for (int64_t c = threadIdx.x; c < K * A; c += T) {
      const tqpk_acc& a = S.accs[c % A];
      const uint64_t v = sm[c];
      if (v != b_acc_init(a)) acc_merge_global(&I.gacc[(c % A) * K + c / A], a, v);
    }
    __syncthreads();
    return;
  }
  if (!priv) return;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = T >> 5;
  for (int64_t c = warp; c < K * A; c += nw) {
    const tqpk_acc& a = S.accs[c % A];
    uint64_t v = b_acc_init(a);
    for (int t = lane; t < T; t += 32) v = b_combine(a, v, sm[c * T + t]);
#pragma unroll
    for (int o = 16; o; o >>= 1) v = b_combine(a, v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0 && v != b_acc_init(a)) acc_merge_global(&I.gacc[(c % A) * K + c / A], a, v);
  }
}

__device__ void gb_count_item(const BatchInst& I, int64_t item, int64_t b, int64_t e) {
  unsigned local = 0;
  for (int64_t s = b + threadIdx.x; s < e; s += blockDim.x) local += __ldcg(&I.gacc[s]) != 0;  // acc 0: row count
  local = __reduce_add_sync(0xffffffffu, local);
  __shared__ unsigned long long s_cnt;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(&s_cnt, (unsigned long long)local);
  __syncthreads();
  if (threadIdx.x == 0) I.range_count[item] = (int64_t)s_cnt;
}

__device__ __forceinline__ void b_store(void* col, int dt, int64_t i, uint64_t v, bool is_f64) {
  switch (dt) {
    case TQPK_F64: static_cast<double*>(col)[i] = is_f64 ? u2d(v) : (double)(int64_t)v; break;
    case TQPK_I64: static_cast<int64_t*>(col)[i] = is_f64 ? (int64_t)u2d(v) : (int64_t)v; break;
    case TQPK_I32: static_cast<int32_t*>(col)[i] = (int32_t)(int64_t)v; break;
    case TQPK_I8: static_cast<int8_t*>(col)[i] = (int8_t)(int64_t)v; break;
    default: static_cast<uint8_t*>(col)[i] = (uint8_t)(int64_t)v; break;
  }
}

__device__ void gb_emit_item(const BatchInst& I, int64_t item, int64_t b, int64_t e) {
  __shared__ int64_t s_base;
  __shared__ int sw[kBlock / 32 + 1];
  if (threadIdx.x == 0) {
    int64_t base = 0;
    for (int64_t r = 0; r < item; ++r) base += __ldcg(&I.range_count[r]);
    s_base = base;
    if (item == I.n_items[2] - 1 && I.out_groups) *I.out_groups = base + __ldcg(&I.range_count[item]);
  }
  __syncthreads();
  const tqpk_groupby_spec& S = I.spec;
  const int64_t K = I.gslots;
  for (int64_t t0 = b; t0 < e; t0 += blockDim.x) {
    const int64_t s = t0 + threadIdx.x;
    const bool occ = s < e && __ldcg(&I.gacc[s]) != 0;
    int total;
    const int ex = block_excl_scan<kBlock, int>(occ ? 1 : 0, total, sw);
    if (occ) {
      const int64_t pos = s_base + ex;
      for (int k = 0; k < I.nk; ++k)
        b_store(I.out_key[k], I.key_dt[k], pos, (uint64_t)(I.kmin[k] + (s / I.kstride[k]) % I.krange[k]), false);
      for (int o = 0; o < I.n_out; ++o) {
        const tqpk_acc& a = S.accs[I.out_a[o]];
        uint64_t v = __ldcg(&I.gacc[(int64_t)I.out_a[o] * K + s]);
        bool f = a.type == TQPK_F64 && a.kind != TQPK_ACC_COUNT_ROWS && a.kind != TQPK_ACC_COUNT_NOTNULL;
        if (f && (a.kind == TQPK_ACC_MIN || a.kind == TQPK_ACC_MAX)) v = d2u(f64_from_ordered(v));
        if (I.out_op[o] == TQPK_OUT_AVG) {
          const double num = f ? u2d(v) : (double)(int64_t)v;
          const double den = (double)(int64_t)__ldcg(&I.gacc[(int64_t)I.out_b[o] * K + s]);
          v = d2u(__ddiv_rn(num, den));
          f = true;
        }
        b_store(I.out_col[o], I.out_dt[o], pos, v, f);
      }
    }
    if (threadIdx.x == 0) s_base += total;
    __syncthreads();
  }
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void __launch_bounds__(kBlock) k_batch(const BatchInst* __restrict__ insts,
                                                  const WorkItem* __restrict__ items, int n_items,
                                                  unsigned* ticket, unsigned* done, int* err,
                                                  uint64_t* __restrict__ trace) {
  extern __shared__ uint64_t bsm[];
  __shared__ int s_item;
  __shared__ uint64_t tk_k[kBlock];
  __shared__ int64_t tk_i[kBlock];
  while (true) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(ticket, 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) return;
    const WorkItem W = items[it];
    const BatchInst& I = insts[W.inst];
    uint64_t t0 = 0, t1 = 0;
    if (trace && threadIdx.x == 0) t0 = global_ns();
    if (W.phase > 0 && threadIdx.x == 0) {
      const unsigned need = (unsigned)I.n_items[W.phase - 1];
      const uint64_t* flag = reinterpret_cast<const uint64_t*>(&done[(W.inst * 4 + W.phase - 1) * 2]);
      int spins = 0;
      while ((unsigned)ld_acquire(flag) < need) {
        if (++spins > kSpinLimit) { set_error(err, TQPK_ETIMEOUT); break; }
        __nanosleep(128);
      }
    }
    __syncthreads();
    if (trace && threadIdx.x == 0) t1 = global_ns();
    if (I.type == BT_JOIN) {
      if (W.phase == 0) join_build_item(I, W.begin, W.end, err);
      else if (W.phase == 1) join_probe_item(I, W.begin, W.end);
      else join_topk_item(I, tk_k, tk_i);
    } else {
      if (W.phase == 0) gb_agg_item(I, W.begin, W.end, bsm);
      else if (W.phase == 1) gb_count_item(I, W.begin / I.range_slots, W.begin, W.end);
      else gb_emit_item(I, W.begin / I.range_slots, W.begin, W.end);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(reinterpret_cast<unsigned long long*>(&done[(W.inst * 4 + W.phase) * 2]), 1ull);
      if (trace) {
        unsigned sm;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
        trace[4 * it + 0] = t0;
        trace[4 * it + 1] = t1;
        trace[4 * it + 2] = global_ns();
        trace[4 * it + 3] = sm;
      }
    }
  }
}

static uint64_t* g_batch_trace = nullptr;

__global__ void k_batch_init_gacc(const BatchInst* insts, int n_inst) {
  for (int i = blockIdx.y; i < n_inst; i += gridDim.y) {
    const BatchInst& I = insts[i];
    if (I.type != BT_GROUPBY) continue;
    const int64_t total = I.gslots * I.spec.n_accs;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < total; j += (int64_t)gridDim.x * blockDim.x)
      I.gacc[j] = b_acc_init(I.spec.accs[j / I.gslots]);
  }
}

static size_t join_ws(int64_t slots) { return align_up(slots * 4, 256) * 2 + align_up(slots * 8, 256) + 256; }

static size_t gb_ws(int64_t slots, int n_accs, int64_t ranges) {
  return align_up((size_t)slots * n_accs * 8, 256) + align_up((size_t)ranges * 8, 256) + 256;
}

}  // namespace tqpk

using namespace tqpk;

extern "C" size_t tqpk_batch_record_bytes(void) { return sizeof(BatchInst); }

extern "C" size_t tqpk_batch_join_workspace_bytes(int64_t key_min, int64_t key_max) {
  return key_max < key_min ? 256 : join_ws(key_max - key_min + 1);
}

extern "C" int tqpk_batch_describe_join(void* h_rec, const void* d_build_keys, int32_t build_dtype, int64_t nb,
                                        const tqpk_predicate* h_build_pred, int64_t key_min, int64_t key_max,
                                        const void* d_probe_fk, int32_t probe_dtype, int64_t np,
                                        const tqpk_predicate* h_probe_pred, const tqpk_groupby_spec* h_values,
                                        int32_t value_reg, int32_t k, int32_t descending, void* d_ws,
                                        size_t ws_bytes, int64_t* d_out_keys, double* d_out_vals,
                                        int64_t* d_out_count, int64_t* d_groups_out, int64_t build_rows_per_item,
                                        int64_t probe_rows_per_item) {
  if (!h_rec || !h_values || !d_ws || !d_out_keys || !d_out_vals || !d_out_count || k < 1 || k > 32 || nb < 0 ||
      np < 0 || key_max < key_min || build_rows_per_item < 4 || probe_rows_per_item < 4)
    return TQPK_EINVAL;
  if ((nb && !d_build_keys) || (np && !d_probe_fk)) return TQPK_EINVAL;
  if (!is_int_dtype(build_dtype) || !is_int_dtype(probe_dtype)) return TQPK_EDTYPE;
  if (value_reg < 0 || value_reg >= h_values->n_expr) return TQPK_EINVAL;
  int rc = check_pred(h_build_pred);
  if (!rc) rc = check_pred(h_probe_pred);
  if (rc) return rc;
  const int64_t slots = key_max - key_min + 1;
  if (slots > (int64_t(1) << 31)) return TQPK_EUNSUPPORTED;
  if (ws_bytes < join_ws(slots)) return TQPK_ENOMEM;
  BatchInst I;
  memset(&I, 0, sizeof(I));
  I.type = BT_JOIN;
  I.k = k;
  I.desc = descending ? 1 : 0;
  I.b_keys = d_build_keys; I.b_dt = build_dtype; I.nb = nb;
  I.p_fk = d_probe_fk; I.p_dt = probe_dtype; I.np = np;
  I.key_min = key_min; I.slots = slots;
  I.val_reg = value_reg;
  WsCursor c(d_ws, ws_bytes);
  I.dir = c.take<int>(slots);
  I.occ = c.take<unsigned>(slots);
  I.sum = c.take<double>(slots);
  I.out_keys = d_out_keys; I.out_vals = d_out_vals; I.out_count = d_out_count; I.out_groups = d_groups_out;
  build_rows_per_item = (build_rows_per_item + 3) / 4 * 4;
  probe_rows_per_item = (probe_rows_per_item + 3) / 4 * 4;
  I.n_items[0] = (nb + build_rows_per_item - 1) / build_rows_per_item;
  I.n_items[1] = (np + probe_rows_per_item - 1) / probe_rows_per_item;
  I.n_items[2] = 1;
  I.range_slots = build_rows_per_item;   // remembered for item generation
  I.gslots = probe_rows_per_item;
  I.pred0 = *pred_or_empty(h_build_pred);
  I.pred1 = *pred_or_empty(h_probe_pred);
  I.pred_vec0 = pred_vec_ok(h_build_pred);
  I.pred_vec1 = pred_vec_ok(h_probe_pred);
  I.spec = *h_values;
  memcpy(h_rec, &I, sizeof(I));
  return TQPK_OK;
}

extern "C" size_t tqpk_batch_groupby_workspace_bytes(const tqpk_groupby_spec* h_spec, const int64_t* key_min,
                                                     const int64_t* key_max, int64_t slots_per_item) {
  if (!h_spec || h_spec->n_accs < 1 || slots_per_item < 1) return 0;
  int64_t K = 1;
  for (int kk = 0; kk < h_spec->n_keys; ++kk) K *= (key_max[kk] - key_min[kk] + 1);
  return gb_ws(K, h_spec->n_accs, (K + slots_per_item - 1) / slots_per_item);
}

extern "C" int tqpk_batch_describe_groupby(void* h_rec, const tqpk_groupby_spec* S, const tqpk_predicate* h_pred,
                                           int64_t n, const int64_t* key_min, const int64_t* key_max, void* d_ws,
                                           size_t ws_bytes, void* const* h_out_keys, int32_t n_out,
                                           const int32_t* h_out_ops, void* const* h_out_cols,
                                           int64_t* d_groups_out, int64_t rows_per_item, int64_t slots_per_item,
                                           int32_t prefer_private) {
  if (!h_rec || !S || !d_ws || n < 0 || n_out < 0 || n_out > TQPK_MAX_ACCS || rows_per_item < 4 ||
      slots_per_item < 32 || S->n_accs < 1 || S->accs[0].kind != TQPK_ACC_COUNT_ROWS || S->n_keys < 1 ||
      S->n_keys > TQPK_MAX_KEYS)
    return TQPK_EINVAL;
  int rc = check_pred(h_pred);
  if (rc) return rc;
  BatchInst I;
  memset(&I, 0, sizeof(I));
  I.type = BT_GROUPBY;
  I.n = n;
  I.nk = S->n_keys;
  int64_t K = 1;
  for (int kk = S->n_keys - 1; kk >= 0; --kk) {
    const int64_t range = key_max[kk] - key_min[kk] + 1;
    if (range < 1 || range > (int64_t(1) << 31) || K > (int64_t(1) << 40) / range) return TQPK_EUNSUPPORTED;
    I.kmin[kk] = key_min[kk];
    I.krange[kk] = range;
    I.kstride[kk] = K;
    K *= range;
    I.key_dt[kk] = S->key_dtypes[kk];
    if (!h_out_keys[kk]) return TQPK_EINVAL;
    I.out_key[kk] = h_out_keys[kk];
  }
  I.gslots = K;
  I.range_slots = (slots_per_item + 31) / 32 * 32;
  const int64_t ranges = (K + I.range_slots - 1) / I.range_slots;
  if (ws_bytes < gb_ws(K, S->n_accs, ranges)) return TQPK_ENOMEM;
  WsCursor c(d_ws, ws_bytes);
  I.gacc = c.take<uint64_t>((size_t)K * S->n_accs);
  I.range_count = c.take<int64_t>(ranges);
  I.gb_mode = (prefer_private && K * S->n_accs * 8 * kBlock <= kBatchSmem) ? 1
              : (K * S->n_accs * 8 <= kBatchSmem ? 2 : 3);
  I.n_out = n_out;
  for (int o = 0; o < n_out; ++o) {
    I.out_op[o] = h_out_ops[4 * o];
    I.out_a[o] = h_out_ops[4 * o + 1];
    I.out_b[o] = h_out_ops[4 * o + 2];
    I.out_dt[o] = h_out_ops[4 * o + 3];
    I.out_col[o] = h_out_cols[o];
    if (!I.out_col[o] || I.out_a[o] < 0 || I.out_a[o] >= S->n_accs || !dtype_size(I.out_dt[o])) return TQPK_EINVAL;
  }
  I.out_groups = d_groups_out;
  rows_per_item = (rows_per_item + 3) / 4 * 4;
  I.n_items[0] = (n + rows_per_item - 1) / rows_per_item;
  I.n_items[1] = ranges;
  I.n_items[2] = ranges;
  I.nb = rows_per_item;   // remembered for item generation
  I.pred0 = *pred_or_empty(h_pred);
  I.pred_vec0 = pred_vec_ok(h_pred);
  I.spec = *S;
  memcpy(h_rec, &I, sizeof(I));
  return TQPK_OK;
}

// Phase-major work items for a set of described instances; returns the count
// (or the required count when it exceeds cap).
extern "C" int64_t tqpk_batch_items(const void* h_recs, int32_t n_inst, void* h_items, int64_t cap) {
  const BatchInst* R = static_cast<const BatchInst*>(h_recs);
  WorkItem* out = static_cast<WorkItem*>(h_items);
  int64_t m = 0;
  for (int phase = 0; phase < 3; ++phase) {
    for (int i = 0; i < n_inst; ++i) {
      const BatchInst& I = R[i];
      int64_t n, step;
      if (I.type == BT_JOIN) {
        n = phase == 0 ? I.nb : (phase == 1 ? I.np : 1);
        step = phase == 0 ? I.range_slots : (phase == 1 ? I.gslots : 1);
      } else {
        n = phase == 0 ? I.n : I.gslots;
        step = phase == 0 ? I.nb : I.range_slots;
      }
      for (int64_t j = 0; j < I.n_items[phase]; ++j) {
        if (m < cap && out) out[m] = WorkItem{i, phase, j * step, std::min(n, (j + 1) * step)};
        ++m;
      }
    }
  }
  return m;
}

// Bytes of the control block (ticket, error word, per-instance phase counters).
extern "C" size_t tqpk_batch_ctl_bytes(int32_t n_inst) { return 64 + (size_t)n_inst * 32; }

// Resets every instance's tables and the control block on `stream` (memsets and one
// init kernel: capturable).  h_recs is the host copy of the records in d_insts.
extern "C" int tqpk_batch_reset(const void* h_recs, const void* d_insts, int32_t n_inst, void* d_ctl,
                                tqpk_stream stream) {
  if (!h_recs || !d_insts || !d_ctl || n_inst < 1) return TQPK_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const BatchInst* R = static_cast<const BatchInst*>(h_recs);
  bool any_gb = false;
  for (int i = 0; i < n_inst; ++i) {
    const BatchInst& I = R[i];
    if (I.type == BT_JOIN) {
      TQPK_CUDA(cudaMemsetAsync(I.dir, 0xff, I.slots * 4, s));
      TQPK_CUDA(cudaMemsetAsync(I.occ, 0, I.slots * 4, s));
      TQPK_CUDA(cudaMemsetAsync(I.sum, 0, I.slots * 8, s));
    } else {
      any_gb = true;
    }
  }
  if (any_gb) {
    k_batch_init_gacc<<<dim3(64, std::min(n_inst, 1024)), kBlock, 0, s>>>(static_cast<const BatchInst*>(d_insts), n_inst);
    TQPK_CHECK_LAUNCH();
  }
  TQPK_CUDA(cudaMemsetAsync(d_ctl, 0, tqpk_batch_ctl_bytes(n_inst), s));
  return TQPK_OK;
}

extern "C" int tqpk_batch_run(const void* d_insts, int32_t n_inst, const void* d_items, int32_t n_items,
                              void* d_ctl, int32_t grid, tqpk_stream stream) {
  if (!d_insts || !d_items || !d_ctl || n_inst < 1 || n_items < 1 || grid < 1) return TQPK_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned* ctl = static_cast<unsigned*>(d_ctl);
  TQPK_CUDA(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, kBatchSmem));
  timing_before(KID_BATCH, s);
  k_batch<<<grid, kBlock, kBatchSmem, s>>>(static_cast<const BatchInst*>(d_insts),
                                           static_cast<const WorkItem*>(d_items), n_items, ctl, ctl + 16,
                                           reinterpret_cast<int*>(ctl + 1), g_batch_trace);
  timing_after(KID_BATCH, s);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

// Reads the batch error word (synchronises).
extern "C" int tqpk_batch_error(const void* d_ctl, int* h_err, tqpk_stream stream) {
  if (!d_ctl || !h_err) return TQPK_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TQPK_CUDA(cudaMemcpyAsync(h_err, static_cast<const unsigned*>(d_ctl) + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  return TQPK_OK;
}

extern "C" int32_t tqpk_batch_grid(void) { return num_sms() * 2; }

// Per-item timeline for tuning: when d_trace is set (32 bytes per work item),
// later tqpk_batch_run launches record for item i the global timer (ns) at
// dequeue, after its dependency wait and at completion, and the SM id.
// NULL turns it off.  A launch captured in a graph keeps the setting it had.
extern "C" int tqpk_batch_set_trace(void* d_trace) {
  g_batch_trace = static_cast<uint64_t*>(d_trace);
  return TQPK_OK;
}
