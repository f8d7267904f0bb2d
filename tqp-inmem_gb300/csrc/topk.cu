// topk.cu - launchers of the warp-list top-k (topk.cuh) and tqpk_topk_stable.
#include <algorithm>

#include "topk.cuh"

namespace tqpk {

__device__ __forceinline__ bool ArraySource::get(int64_t i, uint64_t& k) const {
  if (i >= n) return false;
  const int64_t src = perm ? perm[i] : i;
  k = sort_key(keys, dt, src, desc);
  return true;
}

// Test hook (tqpk_debug_topk_barrier): the poll limit of the single-launch top-k's grid barrier and
// a number of arrivals it also waits for that never come.
static int g_tk_spin_limit = kSpinLimit;
static int g_tk_missing = 0;

// CTAs of k_tk_fused<Src> that fit on the device at once (the cooperative launch's limit).
template <class Src>
static int fused_capacity() {
  static int cap = -1;
  if (cap < 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tk_fused<Src>, 256, 0) != cudaSuccess) {
      (void)cudaGetLastError();
      per_sm = 0;
    }
    cap = per_sm * num_sms();
  }
  return cap;
}

template <int R, class Src>
static int launch_r(const Src& src, int k, int grid, TopkOut O, cudaStream_t s) {
  (void)grid;
  // groups of G items (a multiple of 4), at most kTopkGroups of them
  int64_t G = 4;
  while (G * kTopkGroups < src.n) G <<= 1;
  const int ng = (int)std::max<int64_t>(1, (src.n + G - 1) / G);
  if (R == 1 && G <= kTopkFusedMaxG && O.err && ng <= fused_capacity<Src>()) {
    // one cooperative launch: all ng CTAs resident together, so the grid barrier inside completes
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.gridDim = dim3(ng);
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    TQPK_CUDA(cudaLaunchKernelEx(&cfg, k_tk_fused<Src>, src, G, k, O, g_tk_spin_limit, g_tk_missing));
    return TQPK_OK;
  }
  k_tk_group_best<Src><<<ng, 256, 0, s>>>(src, G, k, O);
  TQPK_CHECK_LAUNCH();
  k_tk_filter<R, Src><<<ng, 256, 0, s>>>(src, G, k, O);     // the same groups
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

template <class Src>
static int launch_src(const Src& src, int k, int grid, TopkOut O, cudaStream_t s) {
  if (k <= 32) return launch_r<1>(src, k, grid, O, s);
  if (k <= 64) return launch_r<2>(src, k, grid, O, s);
  if (k <= 128) return launch_r<4>(src, k, grid, O, s);
  if (k <= 256) return launch_r<8>(src, k, grid, O, s);
  return TQPK_EUNSUPPORTED;
}

int topk_warp_launch(int kind, const void* src, int k, int grid, TopkOut O, cudaStream_t s) {
  if (kind == 0) return launch_src(*static_cast<const DenseSumSource*>(src), k, grid, O, s);
  return launch_src(*static_cast<const ArraySource*>(src), k, grid, O, s);
}

__global__ void k_topk_positions_to_perm(const int64_t* idx, const int64_t* count, const int64_t* perm_in,
                                         int64_t* perm_out, int64_t k) {
  const int64_t m = *count;
  for (int64_t j = threadIdx.x; j < k; j += blockDim.x) {
    if (j < m) perm_out[j] = perm_in ? perm_in[idx[j]] : idx[j];
  }
}

}  // namespace tqpk

using namespace tqpk;

// Test hook: the poll limit of the single-launch top-k's grid barrier, and arrivals it also waits
// for that never come (its bounded wait then runs out: TQPK_ETIMEOUT in the caller's error word).
// (kSpinLimit, 0) restores the defaults.  Not thread-safe; for tests only.
extern "C" int tqpk_debug_topk_barrier(int32_t spin_limit, int32_t missing) {
  if (spin_limit < 0 || spin_limit > kSpinLimit || missing < 0 || missing > 1024) return TQPK_EINVAL;
  g_tk_spin_limit = spin_limit;
  g_tk_missing = missing;
  return TQPK_OK;
}

extern "C" size_t tqpk_topk_workspace_bytes(int64_t n, int64_t k) {
  if (n < 0) n = 0;
  if (k <= 256) return topk_scratch_bytes((int)std::max<int64_t>(k, 1)) + 1024;
  return sort_ws_bytes(n);
}

extern "C" int tqpk_topk_stable(const void* d_keys, int32_t dt, int32_t desc, const int64_t* d_perm_in, int64_t n,
                                int64_t k, int64_t* d_perm_out, void* ws, size_t ws_bytes, tqpk_stream stream) {
  if (n < 0 || k < 0 || (n > 0 && k > 0 && (!d_keys || !d_perm_out || !ws))) return TQPK_EINVAL;
  if (!dtype_size(dt)) return TQPK_EDTYPE;
  const int64_t m = std::min(n, k);
  if (m == 0) return TQPK_OK;
  if (ws_bytes < tqpk_topk_workspace_bytes(n, k)) return TQPK_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (k > 256) {
    const int64_t* res = nullptr;
    int rc = sort_pairs(d_keys, dt, desc ? 1 : 0, d_perm_in, n, ws, ws_bytes, s, &res);
    if (rc) return rc;
    TQPK_CUDA(cudaMemcpyAsync(d_perm_out, res, m * sizeof(int64_t), cudaMemcpyDeviceToDevice, s));
    return TQPK_OK;
  }
  const int grid = topk_grid_size();
  WsCursor cur(ws, ws_bytes);
  unsigned* ticket = cur.take<unsigned>(64);
  int64_t* count = cur.take<int64_t>(4);
  int64_t* idx = cur.take<int64_t>(k);
  uint64_t* ck = cur.take<uint64_t>(topk_cand_entries((int)k));
  int64_t* ci = cur.take<int64_t>(topk_cand_entries((int)k));
  if (!ci) return TQPK_ENOMEM;
  TQPK_CUDA(cudaMemsetAsync(ticket, 0, 256, s));
  ArraySource src{d_keys, dt, d_perm_in, n, desc ? 1 : 0};
  TopkOut O{idx, count, ck, ci, ticket, nullptr, reinterpret_cast<unsigned long long*>(ticket + 8), ticket + 16};
  timing_before(KID_PIPE_TOPK, s);
  int rc = topk_warp_launch(1, &src, (int)k, grid, O, s);
  timing_after(KID_PIPE_TOPK, s);
  if (rc) return rc;
  k_topk_positions_to_perm<<<1, 256, 0, s>>>(idx, count, d_perm_in, d_perm_out, m);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}
