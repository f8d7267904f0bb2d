// sort.cu - kernel (b): stable LSD radix sort of (key, row) pairs, and (e) top-k.
//
// Reference: operators/sort.py:22-42 runs one stable torch.sort per key (last
// key first), permuting `perm` each time, then slices perm[:limit].
// tqpk_argsort_stable is one iteration of that loop: it sorts
// keys[perm_in[i]] stably and returns the permuted perm_in, so the caller's
// LSD key loop needs no extra gathers.
//
// Algorithm (one-sweep style):
//   prepare : gather keys through perm_in, map them onto order-preserving
//             uint64 (signed ints: sign flip; float64: sign-magnitude flip with
//             -0.0 -> +0.0 and NaN canonicalised to the largest value;
//             descending: bitwise complement, which keeps ties stable) and
//             histogram all eight 8-bit digits in the same read.
//   scan    : exclusive digit offsets per pass; passes whose digit is constant
//             over all keys are skipped (e.g. int32 keys in a narrow range).
//   pass    : 4096-key tiles; per warp, match_any ranks equal digits in item
//             order (stable), per-digit warp prefixes in shared memory, then a
//             decoupled look-back per digit across tiles gives the global
//             position in a single read of the tile.
#include <algorithm>

#include "common.cuh"

namespace tqpk {

constexpr int kRadix = 256;
constexpr int kPasses = 8;

__global__ void __launch_bounds__(kBlock) k_sort_prepare(const void* keys, int dt, int desc, const int64_t* perm_in,
                                                         int64_t n, uint64_t* kout, int64_t* vout,
                                                         unsigned* hist /*[8][256]*/) {
  __shared__ unsigned sh[kPasses * kRadix];
  for (int i = threadIdx.x; i < kPasses * kRadix; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t src = perm_in ? perm_in[i] : i;
    const uint64_t k = sort_key(keys, dt, src, desc);
    kout[i] = k;
    vout[i] = src;
#pragma unroll
    for (int p = 0; p < kPasses; ++p) atomicAdd(&sh[p * kRadix + ((k >> (8 * p)) & 255)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kPasses * kRadix; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// One block of 256 threads: offsets[p][d] = exclusive scan; trivial[p] = one digit holds every key.
__global__ void k_sort_scan(const unsigned* hist, int64_t n, int64_t* offsets, int* trivial) {
  __shared__ int64_t sw[kBlock / 32 + 1];
  for (int p = 0; p < kPasses; ++p) {
    const int64_t c = hist[p * kRadix + threadIdx.x];
    int64_t total;
    const int64_t e = block_excl_scan<kBlock, int64_t>(c, total, sw);
    offsets[p * kRadix + threadIdx.x] = e;
    const int all = __syncthreads_or(c == n);
    if (threadIdx.x == 0) trivial[p] = all;
  }
}

constexpr int kSortItems = 16;
constexpr int kSortTile = kBlock * kSortItems;  // 4096 keys

__global__ void __launch_bounds__(kBlock) k_sort_pass(const uint64_t* __restrict__ kin, const int64_t* __restrict__ vin,
                                                      uint64_t* __restrict__ kout, int64_t* __restrict__ vout,
                                                      int64_t n, int shift, const int64_t* __restrict__ offsets,
                                                      uint64_t* status, int* tile_ctr, int* err) {
  __shared__ unsigned wcnt[kBlock / 32][kRadix];
  __shared__ int64_t gbase[kRadix];
  __shared__ int s_tile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < (kBlock / 32) * kRadix; i += kBlock) (&wcnt[0][0])[i] = 0;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1);
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t wbase = tile * kSortTile + (int64_t)warp * (32 * kSortItems);
  uint64_t k[kSortItems];
  int64_t v[kSortItems];
  unsigned rank[kSortItems];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const int64_t i = wbase + j * 32 + lane;
    const bool ok = i < n;
    k[j] = ok ? kin[i] : 0;
    v[j] = ok ? vin[i] : 0;
    const unsigned d = ok ? (unsigned)((k[j] >> shift) & 255) : 256u + lane;  // out-of-range lanes: unique digit
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned r = __popc(peers & lt);
    unsigned base = 0;
    if (ok) base = wcnt[warp][d];
    __syncwarp();
    if (ok && lane == 31 - __clz(peers)) wcnt[warp][d] = base + __popc(peers);
    __syncwarp();
    rank[j] = base + r;
  }
  __syncthreads();
  {  // thread d owns digit d: warp prefixes and the tile's count
    const int d = threadIdx.x;
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < kBlock / 32; ++w) {
      const unsigned c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
    const uint64_t excl = lookback_thread(status, tile, kRadix, d, run, err);
    gbase[d] = offsets[d] + (int64_t)excl;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const int64_t i = wbase + j * 32 + lane;
    if (i < n) {
      const unsigned d = (unsigned)((k[j] >> shift) & 255);
      const int64_t pos = gbase[d] + wcnt[warp][d] + rank[j];
      kout[pos] = k[j];
      vout[pos] = v[j];
    }
  }
}

// Small sorts (n <= kSmallSort, e.g. the groups of an aggregate result): one
// CTA sorts (key, position) pairs with a bitonic network in shared memory.
// Ties fall to the smaller position, so the result is the stable order, and
// the host never waits (no trivial-pass flags, no look-back error word).
constexpr int kSmallSort = 2048;

__global__ void __launch_bounds__(1024) k_sort_small(const void* keys, int dt, int desc, const int64_t* perm_in,
                                                     int n, int64_t* perm_out) {
  __shared__ uint64_t sk[kSmallSort];
  __shared__ uint16_t si[kSmallSort];
  __shared__ int64_t pin[kSmallSort];
  int P = 1;
  while (P < n) P <<= 1;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    if (i < n) {
      const int64_t row = perm_in ? perm_in[i] : i;
      pin[i] = row;
      sk[i] = sort_key(keys, dt, row, desc);
      si[i] = static_cast<uint16_t>(i);
    } else {
      sk[i] = ~0ull;
      si[i] = 0xffffu;
    }
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool up = (i & k) == 0;
          const uint64_t ka = sk[i], kb = sk[ixj];
          const uint16_t ia = si[i], ib = si[ixj];
          const bool greater = ka > kb || (ka == kb && ia > ib);
          if (greater == up) {
            sk[i] = kb; sk[ixj] = ka;
            si[i] = ib; si[ixj] = ia;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm_out[i] = pin[si[i]];
}

size_t sort_ws_bytes(int64_t n) {
  const int64_t tiles = (n + kSortTile - 1) / kSortTile;
  size_t b = 0;
  b += 4 * align_up(sizeof(int64_t) * (size_t)(n > 0 ? n : 1), 256);  // keys A/B (u64) + vals A/B (i64)
  b += align_up(kPasses * kRadix * sizeof(unsigned), 256);
  b += align_up(kPasses * kRadix * sizeof(int64_t), 256);
  b += align_up(64 * sizeof(int), 256);
  b += align_up((size_t)(tiles > 0 ? tiles : 1) * kRadix * sizeof(uint64_t), 256);
  return b + 1024;
}

// Sorts and leaves the permutation in *result (one of the two value buffers).
int sort_pairs(const void* keys, int dt, int desc, const int64_t* perm_in, int64_t n, void* ws, size_t ws_bytes,
               cudaStream_t s, const int64_t** result) {
  const int64_t tiles = (n + kSortTile - 1) / kSortTile;
  WsCursor cur(ws, ws_bytes);
  uint64_t* ka = cur.take<uint64_t>(n);
  uint64_t* kb = cur.take<uint64_t>(n);
  int64_t* va = cur.take<int64_t>(n);
  int64_t* vb = cur.take<int64_t>(n);
  unsigned* hist = cur.take<unsigned>(kPasses * kRadix);
  int64_t* offsets = cur.take<int64_t>(kPasses * kRadix);
  int* ctl = cur.take<int>(64);  // [0..7] trivial flags, [8] tile counter, [9] error word
  uint64_t* status = cur.take<uint64_t>((size_t)(tiles > 0 ? tiles : 1) * kRadix);
  if (!status) return TQPK_ENOMEM;
  TQPK_CUDA(cudaMemsetAsync(hist, 0, kPasses * kRadix * sizeof(unsigned), s));
  TQPK_CUDA(cudaMemsetAsync(ctl, 0, 64 * sizeof(int), s));
  k_sort_prepare<<<grid_for(n, 4), kBlock, 0, s>>>(keys, dt, desc, perm_in, n, ka, va, hist);
  TQPK_CHECK_LAUNCH();
  k_sort_scan<<<1, kBlock, 0, s>>>(hist, n, offsets, ctl);
  TQPK_CHECK_LAUNCH();
  int h[kPasses];
  TQPK_CUDA(cudaMemcpyAsync(h, ctl, sizeof(h), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  uint64_t *kin = ka, *kout = kb;
  int64_t *vin = va, *vout = vb;
  for (int p = 0; p < kPasses; ++p) {
    if (h[p]) continue;
    TQPK_CUDA(cudaMemsetAsync(status, 0, (size_t)tiles * kRadix * sizeof(uint64_t), s));
    TQPK_CUDA(cudaMemsetAsync(ctl + 8, 0, sizeof(int), s));
    k_sort_pass<<<(int)tiles, kBlock, 0, s>>>(kin, vin, kout, vout, n, 8 * p, offsets + p * kRadix, status, ctl + 8,
                                             ctl + 9);
    TQPK_CHECK_LAUNCH();
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  int err = 0;
  TQPK_CUDA(cudaMemcpyAsync(&err, ctl + 9, sizeof(int), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  if (err) return err;
  *result = vin;
  return TQPK_OK;
}

}  // namespace tqpk

using namespace tqpk;

extern "C" size_t tqpk_sort_workspace_bytes(int64_t n) { return sort_ws_bytes(n < 0 ? 0 : n); }

extern "C" int tqpk_argsort_stable(const void* d_keys, int32_t dt, int32_t desc, const int64_t* d_perm_in, int64_t n,
                                   int64_t* d_perm_out, void* ws, size_t ws_bytes, tqpk_stream stream) {
  if (n < 0 || (n > 0 && (!d_keys || !d_perm_out))) return TQPK_EINVAL;
  if (!dtype_size(dt)) return TQPK_EDTYPE;
  if (n == 0) return TQPK_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n <= kSmallSort) {   // no workspace needed
    k_sort_small<<<1, 1024, 0, s>>>(d_keys, dt, desc ? 1 : 0, d_perm_in, (int)n, d_perm_out);
    TQPK_CHECK_LAUNCH();
    return TQPK_OK;
  }
  if (!ws) return TQPK_EINVAL;
  if (ws_bytes < sort_ws_bytes(n)) return TQPK_ENOMEM;
  if ((n + kSortTile - 1) / kSortTile > INT32_MAX) return TQPK_EUNSUPPORTED;
  const int64_t* res = nullptr;
  int rc = sort_pairs(d_keys, dt, desc ? 1 : 0, d_perm_in, n, ws, ws_bytes, s, &res);
  if (rc) return rc;
  TQPK_CUDA(cudaMemcpyAsync(d_perm_out, res, n * sizeof(int64_t), cudaMemcpyDeviceToDevice, s));
  return TQPK_OK;
}

