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

#include "topk.cuh"

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
  int v_pvec;  // value columns are 16-byte aligned
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
    int old[4];           // the four claims in flight together, their results read afterwards
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t slot = x[j] - A.key_min;
      const bool in = (b >> j) & 1u, put = in && slot >= 0 && slot < A.slots;
      if (in && !put) set_error(err_dup, TQPK_EINVAL);
      old[j] = put ? atomicCAS(&dir[slot], -1, (int)(r0 + j)) : -1;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (old[j] != -1) set_error(err_dup, TQPK_EUNSUPPORTED);
  }
}

// The build side's membership bitmap: one atomicOr per passing build row, its result unused (a
// reduction the L2 applies without a reply).  The same grid first sets every group sum to -0.0
// (the empty sum), so no separate fill pass runs.  The passing rows are counted (one atomic per
// CTA); the top-k pass counts the bits set, and fewer bits than rows means a repeated key.
__global__ void __launch_bounds__(kBlock) k_pl_build_bits(const __grid_constant__ tqpk_predicate P, PipeJoinArgs A,
                                                          unsigned* __restrict__ bits, double* __restrict__ sum,
                                                          unsigned long long* passing, int* err) {
  __shared__ unsigned s_pass;
  if (threadIdx.x == 0) s_pass = 0;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nthr = (int64_t)gridDim.x * blockDim.x;
  {
    const double2 e2 = make_double2(u2d(DenseSumSource::kEmptySum), u2d(DenseSumSource::kEmptySum));
    const bool vec = (reinterpret_cast<uintptr_t>(sum) & 15u) == 0;
    const int64_t pairs = vec ? A.slots / 2 : 0;
    for (int64_t i = tid; i < pairs; i += nthr) reinterpret_cast<double2*>(sum)[i] = e2;
    for (int64_t i = 2 * pairs + tid; i < A.slots; i += nthr) sum[i] = e2.x;
  }
  __syncthreads();
  const int64_t groups = (A.nb + 3) >> 2;
  const bool vec = ((reinterpret_cast<uintptr_t>(A.b_keys) & 15u) == 0);
  const bool pvec = A.b_pvec != 0;
  unsigned npass = 0;
  for (int64_t g = tid; g < groups; g += nthr) {
    const int64_t r0 = g << 2;
    uint32_t b = P.n_insn ? eval_pred4(P, r0, A.nb, pvec) : (A.nb - r0 >= 4 ? 0xfu : ((1u << (A.nb - r0)) - 1));
    if (!b) continue;
    int64_t x[4];
    ld4_int(A.b_keys, A.b_dt, r0, A.nb, vec, x);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((b >> j) & 1u)) continue;
      const int64_t slot = x[j] - A.key_min;
      if (slot < 0 || slot >= A.slots) { set_error(err, TQPK_EINVAL); continue; }
      atomicOr(&bits[slot >> 5], 1u << (slot & 31));
      ++npass;
    }
  }
  npass = __reduce_add_sync(0xffffffffu, npass);
  if ((threadIdx.x & 31) == 0 && npass) atomicAdd(&s_pass, npass);
  __syncthreads();
  if (threadIdx.x == 0 && s_pass) atomicAdd(passing, (unsigned long long)s_pass);
}

__global__ void __launch_bounds__(kBlock) k_pl_probe_agg(const __grid_constant__ tqpk_predicate P,
                                                         const __grid_constant__ tqpk_groupby_spec S, PipeJoinArgs A,
                                                         const int* __restrict__ dir, double* __restrict__ sum,
                                                         unsigned* __restrict__ cnt,
                                                         unsigned long long* __restrict__ groups) {
  // Two 4-row groups per thread per iteration: every load of the 8 rows
  // (filter column, fk, directory, value columns) is issued before the
  // atomics, so each thread keeps several independent misses in flight.
  constexpr int U = 2;
  const int64_t n8 = (A.np + 4 * U - 1) / (4 * U);
  const bool vec = ((reinterpret_cast<uintptr_t>(A.p_fk) & 15u) == 0);
  const bool tile = tile_ok(S);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n8; g += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m[U];
    int64_t x[U][4];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t r0 = (g * U + u) << 2;
      m[u] = P.n_insn ? eval_pred4(P, r0, A.np, A.p_pvec != 0)
                      : (A.np - r0 >= 4 ? 0xfu : (A.np - r0 <= 0 ? 0u : ((1u << (A.np - r0)) - 1)));
      if (m[u]) ld4_int(A.p_fk, A.p_dt, r0, A.np, vec, x[u]);
    }
    int64_t slot[U][4];
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        slot[u][j] = x[u][j] - A.key_min;
        const bool ok = ((m[u] >> j) & 1u) && slot[u][j] >= 0 && slot[u][j] < A.slots;
        if (!ok || __ldg(&dir[slot[u][j]]) < 0) m[u] &= ~(1u << j);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (!m[u]) continue;
      const int64_t r0 = (g * U + u) << 2;
      double v[4];
      if (tile) {
        ColTile4 T;
        load_cols4(S, r0, A.np, A.v_pvec != 0, T);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uint64_t r[16];
          expr_eval_tile<16>(S.expr, A.val_reg + 1, S.col_dtypes, T, j, r);
          const uint64_t raw = reg_pick<16>(r, A.val_reg);
          v[j] = S.expr[A.val_reg].type == TQPK_F64 ? u2d(raw) : (double)(int64_t)raw;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = ((m[u] >> j) & 1u) ? expr_value(S, r0 + j, A.val_reg) : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (!((m[u] >> j) & 1u)) continue;
        gred_add(&sum[slot[u][j]], v[j]);
        cnt[slot[u][j]] = 1u;  // occupancy (the top-k pass counts the groups)
      }
    }
  }
}

constexpr int kPipeMaxK = 256;

struct PipeLayout {
  int* dir;
  double* sum;
  unsigned* cnt;
  unsigned long long* groups;
  int* err;
  unsigned* done;
  int64_t* top_count;
  unsigned long long* passing;
  int64_t* top_idx;
  uint64_t* cand_key;
  int64_t* cand_slot;
};

static size_t pipe_bytes(int64_t slots, int grid) {
  return 4096 + align_up(slots * 4, 256) + align_up(slots * 8, 256) + align_up(slots * 4, 256) +
         align_up(kPipeMaxK * 8, 256) + 2 * align_up(std::max<size_t>((size_t)grid * kPipeMaxK, kTopkCand) * 8, 256);
}

static bool pipe_layout(void* ws, size_t bytes, int64_t slots, int grid, PipeLayout& L) {
  WsCursor c(ws, bytes);
  int* hdr = c.take<int>(64);
  if (!hdr) return false;
  L.groups = reinterpret_cast<unsigned long long*>(hdr);      // hdr[0..1]
  L.err = hdr + 2;                                            // hdr[2]
  L.done = reinterpret_cast<unsigned*>(hdr + 3);              // hdr[3]
  L.top_count = reinterpret_cast<int64_t*>(hdr + 4);          // hdr[4..5]; the top-k's bound hdr[6..7], its
                                                              // arrival counter hdr[8], bits set hdr[10..11]
  L.passing = reinterpret_cast<unsigned long long*>(hdr + 12); // hdr[12..13]: passing build rows
  L.dir = c.take<int>(slots);
  L.sum = c.take<double>(slots);
  L.cnt = c.take<unsigned>(slots);
  L.top_idx = c.take<int64_t>(kPipeMaxK);
  L.cand_key = c.take<uint64_t>(std::max<size_t>((size_t)grid * kPipeMaxK, kTopkCand));
  L.cand_slot = c.take<int64_t>(std::max<size_t>((size_t)grid * kPipeMaxK, kTopkCand));
  return L.cand_slot != nullptr;
}

static int topk_grid() { return topk_grid_size(); }

}  // namespace tqpk

using namespace tqpk;

extern "C" size_t tqpk_pipeline_join_agg_topk_workspace_bytes(int64_t key_min, int64_t key_max) {
  if (key_max < key_min) return 4096;
  return pipe_bytes(key_max - key_min + 1, topk_grid());
}

__global__ void k_pl_fill_u64(uint64_t* p, int64_t n, uint64_t v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

static int pipeline_join(int stages, const void* d_build_keys, int32_t build_dtype, int64_t nb,
                         const tqpk_predicate* h_build_pred, int64_t key_min, int64_t key_max, const void* d_probe_fk,
                         int32_t probe_dtype, int64_t np, const tqpk_predicate* h_probe_pred,
                         const tqpk_groupby_spec* h_values, int32_t value_reg, int32_t k, int32_t descending,
                         void* d_ws, size_t ws_bytes, int64_t* d_out_keys, double* d_out_vals, int64_t* d_out_count,
                         int64_t* d_groups_out, tqpk_stream stream) {
  if (nb < 0 || np < 0 || k < 1 || k > kPipeMaxK || !h_values || !d_ws || !d_out_keys || !d_out_vals || !d_out_count)
    return TQPK_EINVAL;
  if ((nb > 0 && !d_build_keys) || (np > 0 && !d_probe_fk)) return TQPK_EINVAL;
  if (!is_int_dtype(build_dtype) || !is_int_dtype(probe_dtype)) return TQPK_EDTYPE;
  if (key_max < key_min || key_max - key_min + 1 > (int64_t(1) << 31)) return TQPK_EUNSUPPORTED;
  if (value_reg < 0 || value_reg >= h_values->n_expr) return TQPK_EINVAL;
  // a side with no rows never evaluates its predicate (its columns may be empty, null tensors)
  int rc = nb > 0 ? check_pred(h_build_pred) : TQPK_OK;
  if (!rc && np > 0) rc = check_pred(h_probe_pred);
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
  A.v_pvec = spec_cols_vec(h_values) ? 1 : 0;
  const bool sentinel = (stages & 8) != 0;   // occupancy carried by the sums (see DenseSumSource)
  const bool bits = (stages & 16) != 0;      // membership bitmap in place of the row directory
  if (bits && (stages & 2)) return TQPK_EINVAL;
  if ((stages & 32) && !bits) return TQPK_EINVAL;   // a caller-launched build writes the bitmap form
  if (stages & 1) {
  TQPK_CUDA(cudaMemsetAsync(L.groups, 0, 56, s));   // hdr[0..13]
  if (bits)
    TQPK_CUDA(cudaMemsetAsync(L.dir, 0, ((slots + 31) / 32) * 4, s));
  else
    TQPK_CUDA(cudaMemsetAsync(L.dir, 0xff, slots * 4, s));
  if (bits && !sentinel) return TQPK_EINVAL;        // the bitmap build fills the sentinel sums
  if (bits) {
    // the build kernel fills the sums
  } else if (sentinel) {
    k_pl_fill_u64<<<grid_for(slots, 4), kBlock, 0, s>>>(reinterpret_cast<uint64_t*>(L.sum), slots,
                                                        DenseSumSource::kEmptySum);
    TQPK_CHECK_LAUNCH();
  } else {
    TQPK_CUDA(cudaMemsetAsync(L.sum, 0, slots * 8, s));
    TQPK_CUDA(cudaMemsetAsync(L.cnt, 0, slots * 4, s));
  }
  if (bits && (stages & 32)) {
    // the caller launches the build (tqpk_pipeline_join_words gives it the counters)
  } else if (bits) {                                 // also fills the sums: runs with no build rows too
    timing_before(KID_PIPE_BUILD, s);
    k_pl_build_bits<<<grid_for(std::max<int64_t>((nb + 3) / 4, slots / 2), 8), kBlock, 0, s>>>(
        *pred_or_empty(h_build_pred), A, reinterpret_cast<unsigned*>(L.dir), L.sum, L.passing, L.err);
    timing_after(KID_PIPE_BUILD, s);
    TQPK_CHECK_LAUNCH();
  } else if (nb > 0) {
    timing_before(KID_PIPE_BUILD, s);
    k_pl_build<<<grid_for((nb + 3) / 4, 8), kBlock, 0, s>>>(*pred_or_empty(h_build_pred), A, L.dir, L.err);
    timing_after(KID_PIPE_BUILD, s);
    TQPK_CHECK_LAUNCH();
  }
  }
  if ((stages & 2) && np > 0) {
    timing_before(KID_PIPE_PROBE, s);
    k_pl_probe_agg<<<occ_grid(k_pl_probe_agg, (np + 7) / 8), kBlock, 0, s>>>(*pred_or_empty(h_probe_pred), *h_values,
                                                                           A, L.dir, L.sum, L.cnt, L.groups);
    timing_after(KID_PIPE_PROBE, s);
    TQPK_CHECK_LAUNCH();
  }
  if (stages & 4) {
    // the top-k's bound, arrival counter and bits-set count (hdr[6..11]) and the group count
    TQPK_CUDA(cudaMemsetAsync(L.top_count + 1, 0, 24, s));
    TQPK_CUDA(cudaMemsetAsync(L.groups, 0, 8, s));
    DenseSumSource src{L.sum, sentinel ? nullptr : L.cnt, slots, A.desc};
    TopkOut O{L.top_idx, L.top_count, L.cand_key, L.cand_slot, L.done, L.groups,
              reinterpret_cast<unsigned long long*>(L.top_count + 1), reinterpret_cast<unsigned*>(L.top_count + 2)};
    O.emit_keys = d_out_keys;          // the top rows straight from the top-k's last CTA
    O.emit_vals = d_out_vals;
    O.emit_count = d_out_count;
    O.emit_sum = L.sum;
    O.emit_key_min = key_min;
    O.err = L.err;                     // the single-launch top-k's bounded barrier reports here
    if (bits) {                        // occupancy also needs the slot's bit; the bit count checks the build
      src.bits = reinterpret_cast<const unsigned*>(L.dir);
      O.bits_set = reinterpret_cast<unsigned long long*>(L.top_count + 3);
      O.bits_expected = L.passing;
    }
    timing_before(KID_PIPE_TOPK, s);
    int trc = topk_warp_launch(0, &src, k, grid, O, s);
    timing_after(KID_PIPE_TOPK, s);
    if (trc) return trc;
  }
  if ((stages & 4) && d_groups_out) TQPK_CUDA(cudaMemcpyAsync(d_groups_out, L.groups, 8, cudaMemcpyDeviceToDevice, s));
  return TQPK_OK;
}

extern "C" int tqpk_pipeline_join_agg_topk(const void* d_build_keys, int32_t build_dtype, int64_t nb,
                                           const tqpk_predicate* h_build_pred, int64_t key_min, int64_t key_max,
                                           const void* d_probe_fk, int32_t probe_dtype, int64_t np,
                                           const tqpk_predicate* h_probe_pred, const tqpk_groupby_spec* h_values,
                                           int32_t value_reg, int32_t k, int32_t descending, void* d_ws,
                                           size_t ws_bytes, int64_t* d_out_keys, double* d_out_vals,
                                           int64_t* d_out_count, int64_t* d_groups_out, tqpk_stream stream) {
  return pipeline_join(7, d_build_keys, build_dtype, nb, h_build_pred, key_min, key_max, d_probe_fk, probe_dtype, np,
                       h_probe_pred, h_values, value_reg, k, descending, d_ws, ws_bytes, d_out_keys, d_out_vals,
                       d_out_count, d_groups_out, stream);
}

// Same pipeline, run stage by stage: bit 0 = reset + build, bit 1 = probe +
// aggregate, bit 2 = top-k + emit.  A caller with its own probe kernel runs
// stages 1 and 4 around it (tqpk_pipeline_join_tables gives the tables).
extern "C" int tqpk_pipeline_join_agg_topk_stages(int32_t stages, const void* d_build_keys, int32_t build_dtype,
                                                  int64_t nb, const tqpk_predicate* h_build_pred, int64_t key_min,
                                                  int64_t key_max, const void* d_probe_fk, int32_t probe_dtype,
                                                  int64_t np, const tqpk_predicate* h_probe_pred,
                                                  const tqpk_groupby_spec* h_values, int32_t value_reg, int32_t k,
                                                  int32_t descending, void* d_ws, size_t ws_bytes,
                                                  int64_t* d_out_keys, double* d_out_vals, int64_t* d_out_count,
                                                  int64_t* d_groups_out, tqpk_stream stream) {
  return pipeline_join(stages, d_build_keys, build_dtype, nb, h_build_pred, key_min, key_max, d_probe_fk, probe_dtype,
                       np, h_probe_pred, h_values, value_reg, k, descending, d_ws, ws_bytes, d_out_keys, d_out_vals,
                       d_out_count, d_groups_out, stream);
}

// Device addresses of the directory (int32), sums (f64) and occupancy (u32) in the workspace.
extern "C" int tqpk_pipeline_join_tables(void* d_ws, size_t ws_bytes, int64_t key_min, int64_t key_max, void** dir,
                                         void** sum, void** occ) {
  PipeLayout L;
  if (!d_ws || key_max < key_min || !pipe_layout(d_ws, ws_bytes, key_max - key_min + 1, topk_grid(), L))
    return TQPK_EINVAL;
  *dir = L.dir;
  *sum = L.sum;
  *occ = L.cnt;
  return TQPK_OK;
}

extern "C" int tqpk_pipeline_join_words(void* d_ws, size_t ws_bytes, int64_t key_min, int64_t key_max, int32_t** err,
                                        uint64_t** passing) {
  PipeLayout L;
  if (!d_ws || !err || !passing || key_max < key_min ||
      !pipe_layout(d_ws, ws_bytes, key_max - key_min + 1, topk_grid(), L))
    return TQPK_EINVAL;
  *err = L.err;
  *passing = reinterpret_cast<uint64_t*>(L.passing);
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
