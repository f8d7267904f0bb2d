// dense.cu - resident key directories and dense slot tables.
//
// A dimension table joined on its primary key becomes a direct-address
// directory over the key domain [key_min, key_min + slots): dir[key - min]
// holds the row index (or a payload column such as the next hop's foreign
// key).  Built once when the table is loaded, it stays in HBM and serves every
// later join against that table: the per-query build predicate is evaluated
// through the row index at probe time instead of being baked into the
// directory.  This is the "built join table" of the reference's sort-based
// join (operators/hashjoin.py:24-177 sorts the build keys on every call); the
// directory replaces the sort + searchsorted for a unique key.
//
// The group tables these probes fill are dense too (one FP64 sum and one
// count per directory slot), and tqpk_dense_topk turns such a table into the
// k best groups without a host round trip: the warp-list top-k of topk.cuh,
// ties to the smaller key, plus a device-side group count.
//
// tqpk_groupby_emit_async is the group-by emit stage without its host
// synchronisation, for callers (the serving loop) that keep many queries in
// flight and read the group count later from device memory.
#include <algorithm>

#include "topk.cuh"

namespace tqpk {

__global__ void __launch_bounds__(kBlock) k_dir_build(const __grid_constant__ tqpk_predicate P, const void* keys,
                                                      int dt, const void* payload, int pdt, int64_t n, int64_t kmin,
                                                      int64_t slots, int empty, int fail_value, int pvec,
                                                      const int* __restrict__ next, int64_t next_min,
                                                      int64_t next_slots, int* __restrict__ dir, int* err) {
  const int64_t groups = (n + 3) >> 2;
  const bool kvec = ((reinterpret_cast<uintptr_t>(keys) & 15u) == 0);
  const bool plvec = ((reinterpret_cast<uintptr_t>(payload) & 15u) == 0);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = g << 2;
    const uint32_t live = n - r0 >= 4 ? 0xfu : ((1u << (n - r0)) - 1);
    const uint32_t pass = P.n_insn ? eval_pred4(P, r0, n, pvec) : live;
    int64_t x[4];
    ld4_int(keys, dt, r0, n, kvec, x);
    int64_t pl[4] = {r0, r0 + 1, r0 + 2, r0 + 3};
    if (payload) ld4_int(payload, pdt, r0, n, plvec, pl);
    // The four rows' next-table lookups, then their four claims, are issued before any result is
    // used: each is an L2 round trip, and one row after another a thread would wait for eight.
    int64_t slot[4];
    bool put[4], ok[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      slot[j] = x[j] - kmin;
      const bool in = (live >> j) & 1u;
      put[j] = in && slot[j] >= 0 && slot[j] < slots;
      if (in && !put[j]) set_error(err, TQPK_EINVAL);
      // a payload outside int32, or equal to the empty marker, cannot name a key of the
      // next (int32) domain: the row stays in the directory as a non-matching entry
      ok[j] = put[j] && ((pass >> j) & 1u) && pl[j] >= (int64_t)INT32_MIN && pl[j] <= (int64_t)INT32_MAX &&
              pl[j] != (int64_t)empty;
    }
    if (next) {                // composed with the next table: keep a payload key that has a row there
      int nx[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t q = pl[j] - next_min;
        ok[j] = ok[j] && q >= 0 && q < next_slots;
        nx[j] = ok[j] ? __ldg(&next[q]) : -1;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) ok[j] = ok[j] && nx[j] >= 0;
    }
    int old[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) old[j] = put[j] ? atomicCAS(&dir[slot[j]], empty, ok[j] ? (int)pl[j] : fail_value) : empty;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (old[j] != empty) set_error(err, TQPK_EUNSUPPORTED);  // repeated key
  }
}

__global__ void k_dir_fill(int* p, int64_t n, int v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void k_dense_emit(const int64_t* idx, const int64_t* count, const double* sum, const unsigned* cnt,
                             int64_t key_min, int k, int64_t* out_keys, double* out_vals, int64_t* out_cnts,
                             int64_t* out_count, const unsigned long long* groups, int64_t* out_groups) {
  const int64_t m = *count;
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    if (j < m) {
      out_keys[j] = key_min + idx[j];
      out_vals[j] = __ldcg(&sum[idx[j]]);
      if (out_cnts) out_cnts[j] = __ldcg(&cnt[idx[j]]);
    }
  }
  if (threadIdx.x == 0) {
    *out_count = m;
    if (out_groups) *out_groups = (int64_t)*groups;
  }
}

constexpr int kDenseMaxK = 256;

}  // namespace tqpk

using namespace tqpk;

static int directory_build(const void* d_keys, int32_t key_dtype, int64_t n, const tqpk_predicate* h_pred,
                           const void* d_payload, int32_t payload_dtype, int64_t key_min, int64_t slots,
                           int32_t empty, int32_t fail_value, const int32_t* d_next, int64_t next_min,
                           int64_t next_slots, int32_t* d_dir, int32_t* d_err, tqpk_stream stream) {
  if (n < 0 || slots < 1 || slots > (int64_t(1) << 31) || !d_dir || !d_err || (n > 0 && !d_keys)) return TQPK_EINVAL;
  if (d_next && (!d_payload || next_slots < 1)) return TQPK_EINVAL;
  if (!is_int_dtype(key_dtype) || (d_payload && !is_int_dtype(payload_dtype))) return TQPK_EDTYPE;
  if (!d_payload && n > (int64_t)INT32_MAX) return TQPK_EUNSUPPORTED;  // row indices travel as int32
  if (fail_value == empty) return TQPK_EINVAL;
  int rc = n > 0 ? check_pred(h_pred) : TQPK_OK;
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TQPK_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int32_t), s));
  k_dir_fill<<<grid_for(slots, 4), kBlock, 0, s>>>(d_dir, slots, empty);
  TQPK_CHECK_LAUNCH();
  if (n > 0) {
    k_dir_build<<<grid_for((n + 3) / 4, 8), kBlock, 0, s>>>(*pred_or_empty(h_pred), d_keys, key_dtype, d_payload,
                                                           payload_dtype, n, key_min, slots, empty, fail_value,
                                                           pred_vec_ok(h_pred) ? 1 : 0, d_next, next_min, next_slots,
                                                           d_dir, d_err);
    TQPK_CHECK_LAUNCH();
  }
  return TQPK_OK;
}

extern "C" int tqpk_directory_build(const void* d_keys, int32_t key_dtype, int64_t n, const tqpk_predicate* h_pred,
                                    const void* d_payload, int32_t payload_dtype, int64_t key_min, int64_t slots,
                                    int32_t empty, int32_t fail_value, int32_t* d_dir, int32_t* d_err,
                                    tqpk_stream stream) {
  return directory_build(d_keys, key_dtype, n, h_pred, d_payload, payload_dtype, key_min, slots, empty, fail_value,
                         nullptr, 0, 0, d_dir, d_err, stream);
}

extern "C" int tqpk_directory_build_next(const void* d_keys, int32_t key_dtype, int64_t n,
                                         const tqpk_predicate* h_pred, const void* d_payload, int32_t payload_dtype,
                                         int64_t key_min, int64_t slots, int32_t empty, int32_t fail_value,
                                         const int32_t* d_next, int64_t next_min, int64_t next_slots,
                                         int32_t* d_dir, int32_t* d_err, tqpk_stream stream) {
  if (!d_next) return TQPK_EINVAL;
  return directory_build(d_keys, key_dtype, n, h_pred, d_payload, payload_dtype, key_min, slots, empty, fail_value,
                         d_next, next_min, next_slots, d_dir, d_err, stream);
}

// dir[i] (a key of the next table's domain) keeps its value only when the next
// table's directory has a row there (next[v - next_min] >= 0); otherwise it
// becomes fail_value.  `empty` and `fail_value` entries stay as they are.
__global__ void k_dir_compose(int* __restrict__ dir, int64_t n, const int* __restrict__ next, int64_t next_min,
                              int64_t next_slots, int empty, int fail_value) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int v = dir[i];
    if (v == empty || v == fail_value) continue;
    const int64_t k = (int64_t)v - next_min;
    if (k < 0 || k >= next_slots || next[k] < 0) dir[i] = fail_value;
  }
}

extern "C" int tqpk_directory_compose(int32_t* d_dir, int64_t slots, const int32_t* d_next, int64_t next_min,
                                      int64_t next_slots, int32_t empty, int32_t fail_value, tqpk_stream stream) {
  if (slots < 0 || next_slots < 0 || (slots > 0 && !d_dir) || (next_slots > 0 && !d_next)) return TQPK_EINVAL;
  if (empty == fail_value) return TQPK_EINVAL;
  if (slots == 0) return TQPK_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_dir_compose<<<grid_for(slots, 8), kBlock, 0, s>>>(d_dir, slots, d_next, next_min, next_slots, empty, fail_value);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

// One bit per directory slot, set where the slot names a row (dir[s] >= 0): a warp
// reads 32 consecutive slots and writes their ballot as one word.
__global__ void k_dir_bits(const int* __restrict__ dir, int64_t n, uint32_t* __restrict__ bits) {
  const int lane = threadIdx.x & 31;
  const int64_t words = (n + 31) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < words; w += nwarps) {
    const int64_t i = (w << 5) + lane;
    const unsigned b = __ballot_sync(0xffffffffu, i < n && dir[i] >= 0);
    if (lane == 0) bits[w] = b;
  }
}

extern "C" int tqpk_directory_bits(const int32_t* d_dir, int64_t slots, uint32_t* d_bits, tqpk_stream stream) {
  if (slots < 0 || (slots > 0 && (!d_dir || !d_bits))) return TQPK_EINVAL;
  if (slots == 0) return TQPK_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_dir_bits<<<grid_for(((slots + 31) >> 5) * 32, 8), kBlock, 0, s>>>(d_dir, slots, d_bits);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

extern "C" size_t tqpk_dense_topk_workspace_bytes(int32_t k) {
  k = std::max(1, std::min(k, kDenseMaxK));
  return 1024 + align_up((size_t)k * 8, 256) + 2 * align_up(topk_cand_entries(k) * 8, 256) + 1024;
}

extern "C" int tqpk_dense_topk(const double* d_sum, const uint32_t* d_cnt, int64_t slots, int64_t key_min, int32_t k,
                               int32_t descending, void* d_ws, size_t ws_bytes, int64_t* d_out_keys,
                               double* d_out_vals, int64_t* d_out_counts, int64_t* d_out_count,
                               int64_t* d_out_groups, tqpk_stream stream) {
  if (slots < 0 || k < 1 || k > kDenseMaxK || !d_ws || !d_out_keys || !d_out_vals || !d_out_count) return TQPK_EINVAL;
  if (slots > 0 && (!d_sum || !d_cnt)) return TQPK_EINVAL;
  if (ws_bytes < tqpk_dense_topk_workspace_bytes(k)) return TQPK_ENOMEM;
  const int grid = topk_grid_size();
  WsCursor c(d_ws, ws_bytes);
  unsigned* hdr = c.take<unsigned>(64);
  int64_t* top_idx = c.take<int64_t>(k);
  uint64_t* cand_key = c.take<uint64_t>(topk_cand_entries(k));
  int64_t* cand_idx = c.take<int64_t>(topk_cand_entries(k));
  if (!cand_idx) return TQPK_ENOMEM;
  unsigned* ticket = hdr;
  unsigned long long* groups = reinterpret_cast<unsigned long long*>(hdr + 2);
  int64_t* count = reinterpret_cast<int64_t*>(hdr + 4);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TQPK_CUDA(cudaMemsetAsync(hdr, 0, 256, s));
  DenseSumSource src{d_sum, reinterpret_cast<const unsigned*>(d_cnt), slots, descending ? 1 : 0};
  TopkOut O{top_idx, count, cand_key, cand_idx, ticket, groups, reinterpret_cast<unsigned long long*>(hdr + 6),
            hdr + 8};
  timing_before(KID_PIPE_TOPK, s);
  int rc = topk_warp_launch(0, &src, k, grid, O, s);
  timing_after(KID_PIPE_TOPK, s);
  if (rc) return rc;
  k_dense_emit<<<1, 256, 0, s>>>(top_idx, count, d_sum, reinterpret_cast<const unsigned*>(d_cnt), key_min, k,
                                 d_out_keys, d_out_vals, d_out_counts, d_out_count, groups, d_out_groups);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}
