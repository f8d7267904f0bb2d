// pipeline.cu - fused filter -> join -> group-by -> top-k (the plan shape
// main.py:152-253 executes as Filter, Filter, Join, Aggregate, take ordered).
//
// The reference materialises every intermediate: two masks, the compacted
// inputs (vortex_pipeline.py:58), the join pairs and gathered columns
// (hashjoin.py:153-175), the group ids (aggregate.py:325), the per-aggregate
// temporaries and a full sort for the limit (sort.py:26-42).  Here, for a
// join whose build keys are unique (a primary key) the group key of
// "group by build key" is the build row itself, so the whole plan is:
//
//   build   one pass over the build side: predicate inline, dir[key-min] = row
//           (a direct-address directory over the base table's key domain,
//           L2-resident for millions of keys); a repeated key is flagged
//   probe   one pass over the probe side: predicate inline, directory lookup,
//           the value expression (loaded only for matched rows) and the group
//           accumulators (FP64 sum, count) updated with L2 atomics
//   top-k   one kernel: per-warp register top-k lists merged per CTA, and the
//           last CTA to finish merges the per-CTA lists (no grid-wide wait)
//
// No host synchronisation happens inside; the caller reads the k results and
// the group count once at the end.  Output order equals a stable descending
// sort of the groups in ascending key order (the reference's aggregate order
// for one non-negative key), i.e. ties resolve to the smaller key.
#include <algorithm>

#include "common.cuh"

namespace tqpk {

struct PipeJoinArgs {
  const void* b_keys;
  int b_dt;
  int64_t nb;
  int64_t key_min;
  int64_t slots;
  const void* p_fk;
  int p_dt;
  int64_t np;
  int val_reg;
  int k;
  int desc;
  int b_pvec;  // build predicate columns are 16-byte aligned
  int p_pvec;  // probe predicate columns are 16-byte aligned
};

__global__ void __launch_bounds__(kBlock) k_pl_build(const __grid_constant__ tqpk_predicate P, PipeJoinArgs A,
                                                     int* __restrict__ dir, int* err_dup) {
  const int64_t groups = (A.nb + 3) >> 2;
  const bool vec = ((reinterpret_cast<uintptr_t>(A.b_keys) & 15u) == 0);
  const bool pvec = A.b_pvec != 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = g << 2;
    uint32_t b = P.n_insn ? eval_pred4(P, r0, A.nb, pvec) : (A.nb - r0 >= 4 ? 0xfu : ((1u << (A.nb - r0)) - 1));
    if (!b) continue;
    int64_t x[4];
    ld4_int(A.b_keys, A.b_dt, r0, A.nb, vec, x);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((b >> j) & 1u)) continue;
      const int64_t slot = x[j] - A.key_min;
      if (slot < 0 || slot >= A.slots) { set_error(err_dup, TQPK_EINVAL); continue; }
      if (atomicCAS(&dir[slot], -1, (int)(r0 + j)) != -1) set_error(err_dup, TQPK_EUNSUPPORTED);
    }
  }
}

// Expression of one probe row (straight-line program of the spec).
__device__ __forceinline__ double pl_value(const tqpk_groupby_spec& S, int64_t row, int reg_out) {
  uint64_t reg[TQPK_MAX_EXPR];
  for (int i = 0; i <= reg_out; ++i) {
    const tqpk_expr_insn& X = S.expr[i];
    uint64_t r = 0;
    const bool f = X.type == TQPK_F64;
    switch (X.op) {
      case TQPK_X_COL:
        r = f ? d2u(ld_f64(S.cols[X.col], S.col_dtypes[X.col], row))
              : static_cast<uint64_t>(ld_int(S.cols[X.col], S.col_dtypes[X.col], row));
        break;
      case TQPK_X_CONST: r = f ? d2u(X.cf) : static_cast<uint64_t>(X.ci); break;
      case TQPK_X_TOF64: r = d2u(static_cast<double>(static_cast<int64_t>(reg[X.a]))); break;
      case TQPK_X_ADD: r = f ? d2u(__dadd_rn(u2d(reg[X.a]), u2d(reg[X.b]))) : reg[X.a] + reg[X.b]; break;
      case TQPK_X_SUB: r = f ? d2u(__dsub_rn(u2d(reg[X.a]), u2d(reg[X.b]))) : reg[X.a] - reg[X.b]; break;
      case TQPK_X_MUL:
        r = f ? d2u(__dmul_rn(u2d(reg[X.a]), u2d(reg[X.b])))
              : static_cast<uint64_t>(static_cast<int64_t>(reg[X.a]) * static_cast<int64_t>(reg[X.b]));
        break;
      case TQPK_X_DIV: r = d2u(__ddiv_rn(u2d(reg[X.a]), u2d(reg[X.b]))); break;
    }
    reg[i] = r;
  }
  const tqpk_expr_insn& X = S.expr[reg_out];
  return X.type == TQPK_F64 ? u2d(reg[reg_out]) : static_cast<double>(static_cast<int64_t>(reg[reg_out]));
}

__global__ void __launch_bounds__(kBlock) k_pl_probe_agg(const __grid_constant__ tqpk_predicate P,
                                                         const __grid_constant__ tqpk_groupby_spec S, PipeJoinArgs A,
                                                         const int* __restrict__ dir, double* __restrict__ sum,
                                                         unsigned* __restrict__ cnt,
                                                         unsigned long long* __restrict__ groups) {
  const int64_t ngroups4 = (A.np + 3) >> 2;
  const bool vec = ((reinterpret_cast<uintptr_t>(A.p_fk) & 15u) == 0);
  unsigned new_groups = 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ngroups4;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = g << 2;
    uint32_t b = P.n_insn ? eval_pred4(P, r0, A.np, A.p_pvec != 0) : (A.np - r0 >= 4 ? 0xfu : ((1u << (A.np - r0)) - 1));
    if (!b) continue;
    int64_t x[4];
    ld4_int(A.p_fk, A.p_dt, r0, A.np, vec, x);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((b >> j) & 1u)) continue;
      const int64_t slot = x[j] - A.key_min;
      if (slot < 0 || slot >= A.slots) continue;
      if (__ldg(&dir[slot]) < 0) continue;
      const double v = pl_value(S, r0 + j, A.val_reg);
      atomicAdd(&sum[slot], v);
      if (atomicAdd(&cnt[slot], 1u) == 0u) ++new_groups;
    }
  }
  new_groups = __reduce_add_sync(0xffffffffu, new_groups);
  if ((threadIdx.x & 31) == 0 && new_groups) atomicAdd(groups, (unsigned long long)new_groups);
}

// ---- top-k (k <= 32): a sorted list distributed over a warp, lane i = i-th best.
// Order: smaller ordered key first, then smaller slot (ties keep key order).
__device__ __forceinline__ bool better(uint64_t ka, int64_t sa, uint64_t kb, int64_t sb) {
  return ka < kb || (ka == kb && sa < sb);
}

struct WarpTopK {
  uint64_t key;   // this lane's list entry
  int64_t slot;   // -1 = empty
};

__device__ __forceinline__ void warp_topk_insert(WarpTopK& L, int k, uint64_t ck, int64_t cs, bool valid) {
  const int lane = threadIdx.x & 31;
  uint32_t pending = __ballot_sync(0xffffffffu, valid);
  while (pending) {
    const int src = __ffs(pending) - 1;
    pending &= pending - 1;
    const uint64_t k0 = __shfl_sync(0xffffffffu, ck, src);
    const int64_t s0 = __shfl_sync(0xffffffffu, cs, src);
    // position = number of list entries better than the candidate
    const bool mine_better = (lane < k) && L.slot >= 0 && better(L.key, L.slot, k0, s0);
    const int pos = __popc(__ballot_sync(0xffffffffu, mine_better));
    if (pos >= k) continue;
    const uint64_t up_k = __shfl_up_sync(0xffffffffu, L.key, 1);
    const int64_t up_s = __shfl_up_sync(0xffffffffu, L.slot, 1);
    if (lane > pos && lane < k) { L.key = up_k; L.slot = up_s; }
    if (lane == pos) { L.key = k0; L.slot = s0; }
  }
}

__device__ __forceinline__ uint64_t order_key(double v, int desc) {
  if (v == 0.0) v = 0.0;
  uint64_t b = d2u(v);
  if (isnan(v)) b = 0x7ff8000000000000ull;
  const uint64_t u = (b & (1ull << 63)) ? ~b : (b | (1ull << 63));
  return desc ? ~u : u;
}

__global__ void __launch_bounds__(kBlock) k_pl_topk(const double* __restrict__ sum, const unsigned* __restrict__ cnt,
                                                    int64_t slots, int k, int desc, uint64_t* cand_key,
                                                    int64_t* cand_slot, unsigned* done, int64_t key_min,
                                                    int64_t* out_keys, double* out_vals, int64_t* out_count,
                                                    const unsigned long long* groups) {
  __shared__ uint64_t sk[kBlock / 32][32];
  __shared__ int64_t ss[kBlock / 32][32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpTopK L{~0ull, -1};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + warp * 32; base < slots; base += stride) {
    const int64_t s = base + lane;
    const bool ok = s < slots && cnt[s] != 0;
    const uint64_t key = ok ? order_key(sum[s], desc) : ~0ull;
    // quick reject against the current k-th entry
    const uint64_t kth_k = __shfl_sync(0xffffffffu, L.key, k - 1);
    const int64_t kth_s = __shfl_sync(0xffffffffu, L.slot, k - 1);
    const bool cand = ok && (kth_s < 0 || better(key, s, kth_k, kth_s));
    warp_topk_insert(L, k, key, s, cand);
  }
  sk[warp][lane] = L.key;
  ss[warp][lane] = L.slot;
  __syncthreads();
  if (warp == 0) {
    WarpTopK M{~0ull, -1};
    for (int w = 0; w < kBlock / 32; ++w) {
      const bool v = lane < k && ss[w][lane] >= 0;
      warp_topk_insert(M, k, sk[w][lane], ss[w][lane], v);
    }
    if (lane < k) {
      cand_key[blockIdx.x * 32 + lane] = M.key;
      cand_slot[blockIdx.x * 32 + lane] = M.slot;
    }
    __threadfence();
    unsigned prev = 0;
    if (lane == 0) prev = atomicAdd(done, 1u);
    prev = __shfl_sync(0xffffffffu, prev, 0);
    if (lane == 0) last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || warp != 0) return;
  __threadfence();
  WarpTopK F{~0ull, -1};
  for (int c = 0; c < (int)gridDim.x; ++c) {
    const bool v = lane < k;
    const uint64_t ck = v ? *((volatile uint64_t*)&cand_key[c * 32 + lane]) : ~0ull;
    const int64_t cs = v ? *((volatile int64_t*)&cand_slot[c * 32 + lane]) : -1;
    warp_topk_insert(F, k, ck, cs, v && cs >= 0);
  }
  const int64_t G = (int64_t)*groups;
  const int64_t m = G < k ? G : k;
  if (lane < m && F.slot >= 0) {
    out_keys[lane] = key_min + F.slot;
    out_vals[lane] = sum[F.slot];
  }
  if (lane == 0) {
    *out_count = m;
    *done = 0;  // leave the counter ready for the next launch
  }
}

struct PipeLayout {
  int* dir;
  double* sum;
  unsigned* cnt;
  unsigned long long* groups;
  int* err;
  unsigned* done;
  uint64_t* cand_key;
  int64_t* cand_slot;
};

static size_t pipe_bytes(int64_t slots, int grid) {
  return 4096 + align_up(slots * 4, 256) + align_up(slots * 8, 256) + align_up(slots * 4, 256) +
         2 * align_up((size_t)grid * 32 * 8, 256);
}

static bool pipe_layout(void* ws, size_t bytes, int64_t slots, int grid, PipeLayout& L) {
  WsCursor c(ws, bytes);
  int* hdr = c.take<int>(64);
  if (!hdr) return false;
  L.groups = reinterpret_cast<unsigned long long*>(hdr);
  L.err = hdr + 2;
  L.done = reinterpret_cast<unsigned*>(hdr + 3);
  L.dir = c.take<int>(slots);
  L.sum = c.take<double>(slots);
  L.cnt = c.take<unsigned>(slots);
  L.cand_key = c.take<uint64_t>((size_t)grid * 32);
  L.cand_slot = c.take<int64_t>((size_t)grid * 32);
  return L.cand_slot != nullptr;
}

static int topk_grid() { return num_sms() * 2; }

}  // namespace tqpk

using namespace tqpk;

extern "C" size_t tqpk_pipeline_join_agg_topk_workspace_bytes(int64_t key_min, int64_t key_max) {
  if (key_max < key_min) return 4096;
  return pipe_bytes(key_max - key_min + 1, topk_grid());
}

extern "C" int tqpk_pipeline_join_agg_topk(const void* d_build_keys, int32_t build_dtype, int64_t nb,
                                           const tqpk_predicate* h_build_pred, int64_t key_min, int64_t key_max,
                                           const void* d_probe_fk, int32_t probe_dtype, int64_t np,
                                           const tqpk_predicate* h_probe_pred, const tqpk_groupby_spec* h_values,
                                           int32_t value_reg, int32_t k, int32_t descending, void* d_ws,
                                           size_t ws_bytes, int64_t* d_out_keys, double* d_out_vals,
                                           int64_t* d_out_count, int64_t* d_groups_out, tqpk_stream stream) {
  if (nb < 0 || np < 0 || k < 1 || k > 32 || !h_values || !d_ws || !d_out_keys || !d_out_vals || !d_out_count)
    return TQPK_EINVAL;
  if ((nb > 0 && !d_build_keys) || (np > 0 && !d_probe_fk)) return TQPK_EINVAL;
  if (!is_int_dtype(build_dtype) || !is_int_dtype(probe_dtype)) return TQPK_EDTYPE;
  if (key_max < key_min || key_max - key_min + 1 > (int64_t(1) << 31)) return TQPK_EUNSUPPORTED;
  if (value_reg < 0 || value_reg >= h_values->n_expr) return TQPK_EINVAL;
  int rc = check_pred(h_build_pred);
  if (!rc) rc = check_pred(h_probe_pred);
  if (rc) return rc;
  const int64_t slots = key_max - key_min + 1;
  const int grid = topk_grid();
  if (ws_bytes < pipe_bytes(slots, grid)) return TQPK_ENOMEM;
  PipeLayout L;
  if (!pipe_layout(d_ws, ws_bytes, slots, grid, L)) return TQPK_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  PipeJoinArgs A;
  A.b_keys = d_build_keys;
  A.b_dt = build_dtype;
  A.nb = nb;
  A.key_min = key_min;
  A.slots = slots;
  A.p_fk = d_probe_fk;
  A.p_dt = probe_dtype;
  A.np = np;
  A.val_reg = value_reg;
  A.k = k;
  A.desc = descending ? 1 : 0;
  A.b_pvec = pred_vec_ok(h_build_pred) ? 1 : 0;
  A.p_pvec = pred_vec_ok(h_probe_pred) ? 1 : 0;
  TQPK_CUDA(cudaMemsetAsync(L.groups, 0, 16, s));
  TQPK_CUDA(cudaMemsetAsync(L.dir, 0xff, slots * 4, s));
  TQPK_CUDA(cudaMemsetAsync(L.sum, 0, slots * 8, s));
  TQPK_CUDA(cudaMemsetAsync(L.cnt, 0, slots * 4, s));
  if (nb > 0) {
    timing_before(KID_PIPE_BUILD, s);
    k_pl_build<<<grid_for((nb + 3) / 4, 8), kBlock, 0, s>>>(*pred_or_empty(h_build_pred), A, L.dir, L.err);
    timing_after(KID_PIPE_BUILD, s);
    TQPK_CHECK_LAUNCH();
  }
  if (np > 0) {
    timing_before(KID_PIPE_PROBE, s);
    k_pl_probe_agg<<<grid_for((np + 3) / 4, 8), kBlock, 0, s>>>(*pred_or_empty(h_probe_pred), *h_values, A, L.dir,
                                                               L.sum, L.cnt, L.groups);
    timing_after(KID_PIPE_PROBE, s);
    TQPK_CHECK_LAUNCH();
  }
  timing_before(KID_PIPE_TOPK, s);
  k_pl_topk<<<grid, kBlock, 0, s>>>(L.sum, L.cnt, slots, k, A.desc, L.cand_key, L.cand_slot, L.done, key_min,
                                    d_out_keys, d_out_vals, d_out_count, L.groups);
  timing_after(KID_PIPE_TOPK, s);
  TQPK_CHECK_LAUNCH();
  if (d_groups_out) TQPK_CUDA(cudaMemcpyAsync(d_groups_out, L.groups, 8, cudaMemcpyDeviceToDevice, s));
  return TQPK_OK;
}

extern "C" int tqpk_pipeline_error(const void* d_ws, int* h_err, tqpk_stream stream) {
  if (!d_ws || !h_err) return TQPK_EINVAL;
  const int* hdr = static_cast<const int*>(d_ws);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TQPK_CUDA(cudaMemcpyAsync(h_err, hdr + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  return TQPK_OK;
}
