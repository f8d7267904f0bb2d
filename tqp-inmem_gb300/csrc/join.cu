// join.cu - kernel (c): equi-join probe emitting (build_row, probe_row) pairs.
//
// Reference: operators/hashjoin.py:24-177 sorts the build keys, takes
// unique_consecutive + counts + an exclusive prefix, binary-searches every
// probe key (searchsorted), expands duplicates through a padded (m, lmax)
// arange matrix with masked_select / repeat_interleave (several host syncs),
// re-checks key equality and gathers the output columns.
//
// Here the build side is turned into a directory once:
//   DIRECT  dense key range (<= max(4*rows, 2^24) slots): slot = key - min.
//           Unique keys: dir[slot] = build row.  Duplicate keys: the passing
//           build rows are radix-sorted stably by key (CSR, ascending row
//           inside a key) and dir[slot] = start of the key's run.
//   SORTED  sparse keys: the same stable sort, plus the distinct keys and run
//           starts; the probe binary-searches the distinct keys (the
//           reference's searchsorted, on a deduplicated array).
// The probe is one single-pass kernel per join type: each thread looks up 16
// probe rows, the per-row match counts are scanned in the block and across
// tiles with the decoupled look-back, and the pairs are written by ascending
// probe row, as the reference's are, then ascending build row (the reference
// sorts build keys with an unstable torch.sort, hashjoin.py:43, so its order
// of one key's duplicate build rows is not fixed; this is the stable one).  Rows
// failing either side's filter mask are skipped in place: the inputs are
// never compacted, and the emitted ids index the original columns.
#include <algorithm>

#include "common.cuh"

namespace tqpk {

struct JoinDir {
  int mode, unique;
  int64_t key_min, slots, n_unique, nb_rows;
  const int64_t* dir;       // DIRECT: row (unique) or run start (dups), -1 = empty
  const int* cnt;           // DIRECT: rows per slot
  const int64_t* csr;       // build rows sorted by (key, row)
  const int64_t* ukeys;     // SORTED: distinct keys
  const int64_t* ustart;    // SORTED: run starts (n_unique + 1 entries)
};

// A compaction leaves a negative status in its count when a look-back gave up.
__global__ void k_count_status(const int64_t* count, int* err) {
  if (*count < 0) set_error(err, (int)*count);
}

__global__ void k_join_init_dir(int64_t* dir, int* cnt, int64_t slots) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < slots; i += (int64_t)gridDim.x * blockDim.x) {
    dir[i] = -1;
    cnt[i] = 0;
  }
}

__global__ void __launch_bounds__(kBlock) k_join_build_direct(const void* keys, int dt, RowFilter F, int64_t nb,
                                                              int64_t kmin, int64_t* dir, int* cnt, int* dup) {
  const int64_t groups = (nb + 3) >> 2;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = g << 2;
    int64_t valid = nb - r0;
    uint32_t b = valid >= 4 ? 0xfu : ((1u << valid) - 1);
    if (F.mask) {
      int64_t m[4];
      ld4_int(F.mask, TQPK_U8, r0, nb, F.mask_vec, m);
      b &= (m[0] != 0) | ((m[1] != 0) << 1) | ((m[2] != 0) << 2) | ((m[3] != 0) << 3);
    }
    if (!b) continue;
    int64_t x[4];
    ld4_int(keys, dt, r0, nb, false, x);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!((b >> j) & 1u)) continue;
      const int64_t slot = x[j] - kmin;
      const int old = atomicAdd(&cnt[slot], 1);
      if (old) *dup = 1;
      dir[slot] = r0 + j;
    }
  }
}

// After the stable sort: csr[i] = i-th build row in (key, row) order.
__global__ void k_join_runs(const void* keys, int dt, const int64_t* csr, int64_t m, int64_t kmin, int direct,
                            int64_t* dir, int64_t* head_flag_rows) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = ld_int(keys, dt, csr[i]);
    const bool head = (i == 0) || ld_int(keys, dt, csr[i - 1]) != k;
    if (direct) {
      if (head) dir[k - kmin] = i;
    } else {
      head_flag_rows[i] = head ? 1 : 0;
    }
  }
}

// SORTED mode: distinct keys + run starts from the head flags (ordered).
__global__ void __launch_bounds__(kBlock) k_join_unique(const void* keys, int dt, const int64_t* csr,
                                                        const int64_t* head, int64_t m, int64_t* ukeys,
                                                        int64_t* ustart, int64_t* nu, uint64_t* status,
                                                        int* tile_ctr, int* err) {
  __shared__ int s_tile;
  __shared__ uint64_t s_excl;
  __shared__ int sw[kBlock / 32 + 1];
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1);
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t i0 = tile * kTile + threadIdx.x * kItems;
  uint32_t bits = 0;
  for (int j = 0; j < kItems; ++j)
    if (i0 + j < m && head[i0 + j]) bits |= 1u << j;
  int total;
  const int excl = block_excl_scan<kBlock, int>(__popc(bits), total, sw);
  if (threadIdx.x < 32) {
    uint64_t e = lookback_warp(status, tile, (uint64_t)total, err);
    if (threadIdx.x == 0) s_excl = e;
  }
  __syncthreads();
  int64_t pos = (int64_t)s_excl + excl;
  while (bits) {
    const int j = __ffs(bits) - 1;
    bits &= bits - 1;
    ukeys[pos] = ld_int(keys, dt, csr[i0 + j]);
    ustart[pos] = i0 + j;
    ++pos;
  }
  if (tile == (int64_t)gridDim.x - 1 && threadIdx.x == 0) {
    *nu = (int64_t)(s_excl + total);
    ustart[s_excl + total] = m;
  }
}

// Looks up one probe key: returns the match count and the first match's
// position (a build row when unique, else an index into csr).
__device__ __forceinline__ int64_t join_lookup(const JoinDir& D, int64_t key, int64_t& first) {
  if (D.mode == TQPK_JOIN_DIRECT) {
    const int64_t slot = key - D.key_min;
    if (slot < 0 || slot >= D.slots) return 0;
    if (D.unique) {
      first = D.dir[slot];
      return first >= 0 ? 1 : 0;
    }
    const int c = D.cnt[slot];
    if (c) first = D.dir[slot];
    return c;
  }
  int64_t lo = 0, hi = D.n_unique;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (D.ukeys[mid] < key) lo = mid + 1; else hi = mid;
  }
  if (lo >= D.n_unique || D.ukeys[lo] != key) return 0;
  first = D.ustart[lo];
  return D.ustart[lo + 1] - D.ustart[lo];
}

template <int JT>
__global__ void __launch_bounds__(kBlock) k_join_probe(JoinDir D, const void* pkeys, int pdt, RowFilter F, int64_t np,
                                                       int64_t* __restrict__ out_b, int64_t* __restrict__ out_p,
                                                       int64_t capacity, const int64_t* base_ptr, int64_t* total_out,
                                                       uint64_t* status, int* tile_ctr, int* err) {
  __shared__ int s_tile;
  __shared__ uint64_t s_excl;
  __shared__ int64_t sw[kBlock / 32 + 1];
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1);
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t r0 = tile * kTile + threadIdx.x * kItems;
  int64_t cnt[kItems], first[kItems];
  int64_t mine = 0;
  const bool kvec = ((reinterpret_cast<uintptr_t>(pkeys) & 15u) == 0);
#pragma unroll
  for (int q = 0; q < kItems / 4; ++q) {
    const int64_t g0 = r0 + 4 * q;
    int64_t valid = np - g0;
    uint32_t b = valid >= 4 ? 0xfu : (valid <= 0 ? 0u : ((1u << valid) - 1));
    if (F.mask && b) {
      int64_t m[4];
      ld4_int(F.mask, TQPK_U8, g0, np, F.mask_vec, m);
      b &= (m[0] != 0) | ((m[1] != 0) << 1) | ((m[2] != 0) << 2) | ((m[3] != 0) << 3);
    }
    int64_t x[4] = {0, 0, 0, 0};
    if (b) ld4_int(pkeys, pdt, g0, np, kvec, x);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t c = 0, f = 0;
      if ((b >> j) & 1u) {
        c = join_lookup(D, x[j], f);
        if (JT == TQPK_JT_SEMI) c = c ? 1 : 0;
        if (JT == TQPK_JT_ANTI) c = c ? 0 : 1;
      }
      cnt[4 * q + j] = c;
      first[4 * q + j] = f;
      mine += c;
    }
  }
  int64_t total;
  const int64_t excl = block_excl_scan<kBlock, int64_t>(mine, total, sw);
  if (threadIdx.x < 32) {
    uint64_t e = lookback_warp(status, tile, (uint64_t)total, err);
    if (threadIdx.x == 0) s_excl = e;
  }
  __syncthreads();
  const int64_t base = (base_ptr ? *base_ptr : 0);
  const bool one_per_row = JT != TQPK_JT_INNER || (D.mode == TQPK_JOIN_DIRECT && D.unique);   // block-uniform
  if (one_per_row) {
    // at most one output per row, so the tile's outputs fit kTile slots: each thread places its
    // outputs at its block offset in shared memory, then the block writes them contiguously
    // (coalesced) instead of every lane storing its own run
    __shared__ int64_t s_out[kTile];
    const int64_t gbase = base + (int64_t)s_excl;
    int64_t lp = excl;
#pragma unroll
    for (int j = 0; j < kItems; ++j)
      if (cnt[j]) s_out[lp++] = r0 + j;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < total; i += kBlock)
      if (gbase + i < capacity) out_p[gbase + i] = s_out[i];
    if (JT == TQPK_JT_INNER || (JT == TQPK_JT_ANTI && out_b)) {
      __syncthreads();
      lp = excl;
#pragma unroll
      for (int j = 0; j < kItems; ++j)
        if (cnt[j]) s_out[lp++] = (JT == TQPK_JT_INNER) ? first[j] : (int64_t)TQPK_NULL_INDEX;
      __syncthreads();
      for (int64_t i = threadIdx.x; i < total; i += kBlock)
        if (gbase + i < capacity) out_b[gbase + i] = s_out[i];
    }
  } else {
    int64_t pos = base + (int64_t)s_excl + excl;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
      const int64_t c = cnt[j];
      for (int64_t t = 0; t < c; ++t, ++pos) {
        if (pos >= capacity) continue;
        out_p[pos] = r0 + j;
        if (JT == TQPK_JT_INNER) out_b[pos] = D.csr[first[j] + t];
      }
    }
  }
  if (tile == (int64_t)gridDim.x - 1 && threadIdx.x == 0) *total_out = base + (int64_t)(s_excl + total);
}

__global__ void k_gather(int ncols, const __grid_constant__ ColSet C, const int64_t* __restrict__ idx, int64_t n,
                         int null_aware) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx[j];
    const bool isnull = null_aware && i == TQPK_NULL_INDEX;
    for (int c = 0; c < ncols; ++c) {
      switch (C.size[c]) {
        case 1: static_cast<uint8_t*>(C.out[c])[j] = isnull ? (uint8_t)(int8_t)TQPK_NULL_INDEX : static_cast<const uint8_t*>(C.in[c])[i]; break;
        case 4: static_cast<int32_t*>(C.out[c])[j] = isnull ? TQPK_NULL_INDEX : static_cast<const int32_t*>(C.in[c])[i]; break;
        case 8: static_cast<int64_t*>(C.out[c])[j] = isnull ? TQPK_NULL_INDEX : static_cast<const int64_t*>(C.in[c])[i]; break;
        default: static_cast<double*>(C.out[c])[j] = isnull ? (double)TQPK_NULL_INDEX : static_cast<const double*>(C.in[c])[i]; break;
      }
    }
  }
}

// ---------------------------------------------------------------- host side
struct BuildLayout {
  int* hdr;            // [0] dup flag, [1] error, [2] tile counter
  int64_t* nu;         // distinct keys (SORTED)
  int64_t* dir;
  int* cnt;
  int64_t* csr;
  int64_t* ukeys;
  int64_t* ustart;
  int64_t* head;
  void* sort_ws;
  size_t sort_bytes;
  uint64_t* status;
};

static bool layout(const tqpk_join_plan& p, void* ws, size_t bytes, BuildLayout& L) {
  WsCursor c(ws, bytes);
  const int64_t m = p.nb_rows > 0 ? p.nb_rows : 1;
  L.hdr = c.take<int>(64);
  L.nu = c.take<int64_t>(4);
  L.dir = c.take<int64_t>(p.mode == TQPK_JOIN_DIRECT ? p.slots : 1);
  L.cnt = c.take<int>(p.mode == TQPK_JOIN_DIRECT ? p.slots : 1);
  L.csr = c.take<int64_t>(m);
  L.ukeys = c.take<int64_t>(p.mode == TQPK_JOIN_SORTED ? m : 1);
  L.ustart = c.take<int64_t>(p.mode == TQPK_JOIN_SORTED ? m + 1 : 1);
  L.head = c.take<int64_t>(p.mode == TQPK_JOIN_SORTED ? m : 1);
  L.status = c.take<uint64_t>((m + kTile - 1) / kTile + 1);
  L.sort_bytes = sort_ws_bytes(m);
  L.sort_ws = c.take<char>(L.sort_bytes);
  return L.sort_ws != nullptr;
}

static size_t layout_bytes(const tqpk_join_plan& p) {
  const int64_t m = p.nb_rows > 0 ? p.nb_rows : 1;
  size_t b = 256 + 256;
  if (p.mode == TQPK_JOIN_DIRECT) b += align_up(p.slots * 8, 256) + align_up(p.slots * 4, 256);
  else b += 512;
  b += align_up(m * 8, 256);
  if (p.mode == TQPK_JOIN_SORTED) b += align_up(m * 8, 256) + align_up((m + 1) * 8, 256) + align_up(m * 8, 256);
  else b += 768;
  b += align_up(((m + kTile - 1) / kTile + 1) * 8, 256);
  b += align_up(sort_ws_bytes(m), 256);
  return b + 2048;
}

static JoinDir make_dir(const tqpk_join_plan& p, const BuildLayout& L) {
  JoinDir D;
  D.mode = p.mode;
  D.unique = p.unique;
  D.key_min = p.key_min;
  D.slots = p.slots;
  D.n_unique = p.n_unique;
  D.nb_rows = p.nb_rows;
  D.dir = L.dir;
  D.cnt = L.cnt;
  D.csr = L.csr;
  D.ukeys = L.ukeys;
  D.ustart = L.ustart;
  return D;
}

}  // namespace tqpk

using namespace tqpk;

extern "C" int tqpk_join_plan_build(const void* keys, int32_t dt, const uint8_t* mask, int64_t nb, tqpk_join_plan* plan,
                                    void* scratch, tqpk_stream stream) {
  if (!plan || nb < 0 || (nb > 0 && !keys)) return TQPK_EINVAL;
  if (!is_int_dtype(dt)) return TQPK_EDTYPE;
  *plan = tqpk_join_plan{};
  int64_t mn = 0, mx = -1, rows = 0;
  const void* cols[1] = {keys};
  const int32_t dts[1] = {dt};
  int rc = key_ranges(nullptr, mask, nb, 1, cols, dts, &mn, &mx, &rows, scratch, static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  plan->nb_rows = rows;
  plan->key_min = rows ? mn : 0;
  plan->key_max = rows ? mx : -1;
  const int64_t range = rows ? (mx - mn + 1) : 1;
  // direct addressing costs 12 B per slot of the key range; up to 2^24 slots (~200 MB) that is
  // cheaper than a binary search per probe row even for a sparse build side (a filtered
  // dimension of 2 M keys joined by a 60 M-row fact table: 7.6 ms sorted, ~0.1 ms direct)
  const bool dense = rows == 0 || (range > 0 && range <= std::max<int64_t>(4 * rows, int64_t(1) << 24) &&
                                   range < (int64_t(1) << 31));
  plan->mode = dense ? TQPK_JOIN_DIRECT : TQPK_JOIN_SORTED;
  plan->slots = dense ? range : 0;
  plan->unique = 1;
  plan->ws_bytes = layout_bytes(*plan);
  return TQPK_OK;
}

extern "C" int tqpk_join_build(tqpk_join_plan* plan, const void* keys, int32_t dt, const uint8_t* mask, int64_t nb,
                               void* ws, size_t ws_bytes, tqpk_stream stream) {
  if (!plan || nb < 0 || (nb > 0 && !keys)) return TQPK_EINVAL;
  if (!is_int_dtype(dt)) return TQPK_EDTYPE;
  if (!ws || ws_bytes < plan->ws_bytes) return TQPK_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BuildLayout L;
  if (!layout(*plan, ws, ws_bytes, L)) return TQPK_ENOMEM;
  TQPK_CUDA(cudaMemsetAsync(L.hdr, 0, 64 * sizeof(int), s));
  RowFilter F = make_filter(nullptr, mask);
  bool need_sort = plan->mode == TQPK_JOIN_SORTED;
  if (plan->mode == TQPK_JOIN_DIRECT) {
    k_join_init_dir<<<grid_for(plan->slots, 4), kBlock, 0, s>>>(L.dir, L.cnt, plan->slots);
    TQPK_CHECK_LAUNCH();
    if (plan->nb_rows > 0) {
      k_join_build_direct<<<grid_for((nb + 3) / 4, 8), kBlock, 0, s>>>(keys, dt, F, nb, plan->key_min, L.dir, L.cnt,
                                                                      L.hdr);
      TQPK_CHECK_LAUNCH();
    }
    int h[2] = {0, 0};   // [0] a repeated key, [1] error word: one read
    TQPK_CUDA(cudaMemcpyAsync(h, L.hdr, sizeof(h), cudaMemcpyDeviceToHost, s));
    TQPK_CUDA(cudaStreamSynchronize(s));
    if (h[1]) return h[1];
    plan->unique = h[0] ? 0 : 1;
    need_sort = h[0] != 0;
    if (!need_sort) return TQPK_OK;
  }
  if (need_sort && plan->nb_rows > 0) {
    plan->unique = 0;
    // Passing build rows in row order, then a stable sort by key -> CSR.
    ColSet C;
    C.n = 1;
    C.in[0] = nullptr;
    C.out[0] = L.csr;
    C.size[0] = 0;  // row ids
    int64_t* d_m = L.nu + 1;
    int rc = compact_launch(nullptr, mask, nb, C, d_m, L.sort_ws, L.sort_bytes, s);  // no mask: all rows
    if (rc) return rc;
    k_count_status<<<1, 1, 0, s>>>(d_m, L.hdr + 1);   // a failed compaction's status joins the error word
    TQPK_CHECK_LAUNCH();
    const int64_t* sorted = nullptr;
    rc = sort_pairs(keys, dt, 0, L.csr, plan->nb_rows, L.sort_ws, L.sort_bytes, s, &sorted);
    if (rc) return rc;
    TQPK_CUDA(cudaMemcpyAsync(L.csr, sorted, plan->nb_rows * 8, cudaMemcpyDeviceToDevice, s));
    const int direct = plan->mode == TQPK_JOIN_DIRECT;
    k_join_runs<<<grid_for(plan->nb_rows, 4), kBlock, 0, s>>>(keys, dt, L.csr, plan->nb_rows, plan->key_min, direct,
                                                             L.dir, L.head);
    TQPK_CHECK_LAUNCH();
    if (!direct) {
      const int64_t tiles = (plan->nb_rows + kTile - 1) / kTile;
      TQPK_CUDA(cudaMemsetAsync(L.status, 0, (tiles + 1) * 8, s));
      TQPK_CUDA(cudaMemsetAsync(L.hdr + 2, 0, sizeof(int), s));
      k_join_unique<<<(int)tiles, kBlock, 0, s>>>(keys, dt, L.csr, L.head, plan->nb_rows, L.ukeys, L.ustart, L.nu,
                                                  L.status, L.hdr + 2, L.hdr + 1);
      TQPK_CHECK_LAUNCH();
      int64_t nu = 0;
      TQPK_CUDA(cudaMemcpyAsync(&nu, L.nu, 8, cudaMemcpyDeviceToHost, s));
      TQPK_CUDA(cudaStreamSynchronize(s));
      plan->n_unique = nu;
    }
  }
  int err = 0;
  TQPK_CUDA(cudaMemcpyAsync(&err, L.hdr + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  return err ? err : TQPK_OK;
}

extern "C" size_t tqpk_join_probe_workspace_bytes(int64_t np) {
  const int64_t tiles = (np + kTile - 1) / kTile;
  return 1024 + 2 * align_up((size_t)(tiles + 1) * 8, 256);
}

extern "C" int tqpk_join_probe(const tqpk_join_plan* plan, const void* build_ws, const void* pkeys, int32_t pdt,
                               const uint8_t* pmask, int64_t np, int32_t jt, int64_t* out_b, int64_t* out_p,
                               int64_t capacity, int64_t* h_count, void* pws, size_t pws_bytes, tqpk_stream stream) {
  if (!plan || !build_ws || np < 0 || (np > 0 && !pkeys) || !h_count || capacity < 0) return TQPK_EINVAL;
  if (jt < TQPK_JT_INNER || jt > TQPK_JT_OUTER) return TQPK_EINVAL;
  if ((jt == TQPK_JT_INNER || jt == TQPK_JT_OUTER) && capacity > 0 && !out_b) return TQPK_EINVAL;
  if (capacity > 0 && !out_p) return TQPK_EINVAL;
  if (!is_int_dtype(pdt)) return TQPK_EDTYPE;
  if (!pws || pws_bytes < tqpk_join_probe_workspace_bytes(np)) return TQPK_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BuildLayout L;
  if (!layout(*plan, const_cast<void*>(build_ws), plan->ws_bytes, L)) return TQPK_ENOMEM;
  const JoinDir D = make_dir(*plan, L);
  const int64_t tiles = (np + kTile - 1) / kTile;
  WsCursor cur(pws, pws_bytes);
  int* ctl = cur.take<int>(64);        // [0] tile counter A, [1] error, [2] tile counter B
  int64_t* totals = cur.take<int64_t>(8);
  uint64_t* status_a = cur.take<uint64_t>(tiles + 1);
  uint64_t* status_b = cur.take<uint64_t>(tiles + 1);
  if (!status_b) return TQPK_ENOMEM;
  TQPK_CUDA(cudaMemsetAsync(pws, 0, cur.off, s));
  *h_count = 0;
  if (np == 0) return TQPK_OK;
  const RowFilter F = make_filter(nullptr, pmask);
  const bool empty_build = plan->nb_rows == 0;
  if (jt == TQPK_JT_INNER || jt == TQPK_JT_OUTER) {
    if (!empty_build) {
      timing_before(KID_JOIN_PROBE, s);
      k_join_probe<TQPK_JT_INNER><<<(int)tiles, kBlock, 0, s>>>(D, pkeys, pdt, F, np, out_b, out_p, capacity, nullptr,
                                                               totals, status_a, ctl, ctl + 1);
      timing_after(KID_JOIN_PROBE, s);
      TQPK_CHECK_LAUNCH();
    }
    if (jt == TQPK_JT_OUTER) {
      JoinDir E = D;
      if (empty_build) { E.mode = TQPK_JOIN_DIRECT; E.unique = 1; E.slots = 0; }
      k_join_probe<TQPK_JT_ANTI><<<(int)tiles, kBlock, 0, s>>>(E, pkeys, pdt, F, np, out_b, out_p, capacity, totals,
                                                              totals + 1, status_b, ctl + 2, ctl + 1);
      TQPK_CHECK_LAUNCH();
    }
  } else if (jt == TQPK_JT_SEMI) {
    if (!empty_build) {
      k_join_probe<TQPK_JT_SEMI><<<(int)tiles, kBlock, 0, s>>>(D, pkeys, pdt, F, np, nullptr, out_p, capacity, nullptr,
                                                              totals, status_a, ctl, ctl + 1);
      TQPK_CHECK_LAUNCH();
    }
  } else {
    JoinDir E = D;
    if (empty_build) { E.mode = TQPK_JOIN_DIRECT; E.unique = 1; E.slots = 0; }
    k_join_probe<TQPK_JT_ANTI><<<(int)tiles, kBlock, 0, s>>>(E, pkeys, pdt, F, np, nullptr, out_p, capacity, nullptr,
                                                            totals, status_a, ctl, ctl + 1);
    TQPK_CHECK_LAUNCH();
  }
  int64_t h[2] = {0, 0};
  int err = 0;
  TQPK_CUDA(cudaMemcpyAsync(h, totals, sizeof(h), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaMemcpyAsync(&err, ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  if (err) return err;
  *h_count = (jt == TQPK_JT_OUTER) ? h[1] : h[0];
  return *h_count > capacity ? TQPK_ECAPACITY : TQPK_OK;
}

extern "C" int tqpk_gather(int32_t ncols, const void* const* cols_in, const int32_t* dts, const int64_t* idx,
                           int64_t n_idx, int32_t null_aware, void* const* cols_out, tqpk_stream stream) {
  if (ncols < 0 || ncols > TQPK_MAX_COLS || n_idx < 0 || (n_idx > 0 && !idx)) return TQPK_EINVAL;
  if (n_idx == 0 || ncols == 0) return TQPK_OK;
  ColSet C;
  C.n = ncols;
  for (int c = 0; c < ncols; ++c) {
    const int sz = dtype_size(dts[c]);
    if (!sz) return TQPK_EDTYPE;
    if (!cols_in[c] || !cols_out[c]) return TQPK_EINVAL;
    C.in[c] = cols_in[c];
    C.out[c] = cols_out[c];
    C.size[c] = (dts[c] == TQPK_F64) ? 9 : sz;  // 9: float64 (null fill is -64.0)
  }
  k_gather<<<grid_for(n_idx, 8), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(ncols, C, idx, n_idx, null_aware);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}
