// filter.cu - kernel (a): predicate evaluation and stable stream compaction.
//
// Reference: operators/filter.py:14-204 evaluates a predicate tree with one
// ATen launch per tree node and stores a bool mask; IO/vortex_pipeline.py:58
// later compacts every consumer column with tensor[mask] (nonzero + gather,
// one host sync per column).  Here the whole predicate program runs in one
// pass with 128-bit loads over groups of four rows, and compaction of up to
// 16 columns is one single-pass kernel: per-thread popc of a 16-row mask, a
// block scan, and a decoupled look-back across 4096-row tiles so the output
// keeps row order (what tensor[mask] gives).
#include <stdio.h>

#include "common.cuh"

namespace tqpk {

thread_local int64_t g_launches = 0;

namespace {
struct Timing {
  int kid = KID_NONE;
  int n = 0;
  cudaEvent_t ev[2 * 4096];
  bool created = false;
};
Timing g_timing;
}  // namespace

void timing_before(int kid, cudaStream_t s) {
  if (g_timing.kid != kid || g_timing.n >= 4096) return;
  cudaEventRecord(g_timing.ev[2 * g_timing.n], s);
}
void timing_after(int kid, cudaStream_t s) {
  if (g_timing.kid != kid || g_timing.n >= 4096) return;
  cudaEventRecord(g_timing.ev[2 * g_timing.n + 1], s);
  ++g_timing.n;
}

int num_sms() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cached[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
    cached[dev] = v;
  }
  return cached[dev];
}

__global__ void __launch_bounds__(kBlock) k_filter_mask(const __grid_constant__ tqpk_predicate P, int64_t n,
                                                        uint8_t* __restrict__ mask, unsigned long long* count,
                                                        int vec, int mask_vec) {
  const int64_t groups = (n + 3) >> 2;
  unsigned local = 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = g << 2;
    const uint32_t b = eval_pred4(P, r0, n, vec);
    local += __popc(b);
    if (mask_vec && r0 + 4 <= n) {
      const uint32_t w = (b & 1u) | ((b & 2u) << 7) | ((b & 4u) << 14) | ((b & 8u) << 21);
      *reinterpret_cast<uint32_t*>(mask + r0) = w;
    } else {
      for (int j = 0; j < 4 && r0 + j < n; ++j) mask[r0 + j] = (b >> j) & 1u;
    }
  }
  if (count) {
    local = __reduce_add_sync(0xffffffffu, local);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, (unsigned long long)local);
  }
}

// Control block of one compaction (zeroed before the launch).
struct CompactCtl {
  int tile_ctr;      // next tile to take
  int err;           // first error status of any CTA
  int finished;      // CTAs done
  int pad;
  int64_t kept;      // rows kept, written by the CTA of the last tile
};
constexpr size_t kCompactCtlBytes = 256;   // one WsCursor piece
static_assert(sizeof(CompactCtl) <= kCompactCtlBytes, "control block");

// Test hook (tqpk_debug_compact_wait): the poll limit of the look-back, and a tile whose CTA
// publishes nothing, so that its successors' waits run out.  Defaults: kSpinLimit, none.
static int g_dbg_spin_limit = kSpinLimit;
static int64_t g_dbg_stall_tile = -1;

// One 4096-row tile of k_compact: the tile's mask bits, its block scan, the look-back for its
// output offset, then the kept rows of every column in row order.
__device__ __forceinline__ void compact_tile(const tqpk_predicate& P, const RowFilter& F, int64_t n, const ColSet& C,
                                             uint64_t* status, CompactCtl* ctl, int spin_limit, int64_t tile,
                                             uint64_t& s_excl, int* sw) {
  const int64_t r0 = tile * kTile + threadIdx.x * kItems;
  uint32_t bits = 0;
#pragma unroll
  for (int q = 0; q < kItems / 4; ++q) bits |= filter4(F, P, r0 + 4 * q, n) << (4 * q);
  int total;
  const int excl = block_excl_scan<kBlock, int>(__popc(bits), total, sw);
  if (threadIdx.x < 32) {
    uint64_t e = lookback_warp(status, tile, (uint64_t)total, &ctl->err, spin_limit);
    if (threadIdx.x == 0) s_excl = e;
  }
  __syncthreads();
  const int64_t base = (int64_t)s_excl + excl;
  for (int c = 0; c < C.n; ++c) {
    int64_t pos = base;
    uint32_t b = bits;
    switch (C.size[c]) {
      case 1: {
        const uint8_t* in = static_cast<const uint8_t*>(C.in[c]);
        uint8_t* out = static_cast<uint8_t*>(C.out[c]);
        while (b) { int j = __ffs(b) - 1; b &= b - 1; out[pos++] = in[r0 + j]; }
        break;
      }
      case 4: {
        const uint32_t* in = static_cast<const uint32_t*>(C.in[c]);
        uint32_t* out = static_cast<uint32_t*>(C.out[c]);
        while (b) { int j = __ffs(b) - 1; b &= b - 1; out[pos++] = in[r0 + j]; }
        break;
      }
      case 8: {
        const uint64_t* in = static_cast<const uint64_t*>(C.in[c]);
        uint64_t* out = static_cast<uint64_t*>(C.out[c]);
        while (b) { int j = __ffs(b) - 1; b &= b - 1; out[pos++] = in[r0 + j]; }
        break;
      }
      default: {  // size 0: the row index itself (int64), for row-id compaction
        int64_t* out = static_cast<int64_t*>(C.out[c]);
        while (b) { int j = __ffs(b) - 1; b &= b - 1; out[pos++] = r0 + j; }
        break;
      }
    }
  }
  if (tile == (int64_t)gridDim.x - 1 && threadIdx.x == 0) ctl->kept = (int64_t)(s_excl + total);
}

__global__ void __launch_bounds__(kBlock) k_compact(const __grid_constant__ tqpk_predicate P, RowFilter F, int64_t n,
                                                    const __grid_constant__ ColSet C, int64_t* count,
                                                    uint64_t* status, CompactCtl* ctl, int spin_limit,
                                                    int64_t stall_tile) {
  __shared__ int s_tile;
  __shared__ uint64_t s_excl;
  __shared__ int sw[kBlock / 32 + 1];
  if (threadIdx.x == 0) s_tile = atomicAdd(&ctl->tile_ctr, 1);
  __syncthreads();
  const int64_t tile = s_tile;
  if (tile != stall_tile) compact_tile(P, F, n, C, status, ctl, spin_limit, tile, s_excl, sw);
  // The last CTA to finish writes the result: the kept-row count, or the error status (negative)
  // when any look-back gave up.  Every CTA's error write precedes its fence and its increment.
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ctl->finished, 1) == (int)gridDim.x - 1) {
      __threadfence();
      const int e = *reinterpret_cast<volatile int*>(&ctl->err);
      const int64_t kept = *reinterpret_cast<volatile int64_t*>(&ctl->kept);
      *count = e ? (int64_t)e : kept;
    }
  }
}

// Min/max of up to four integer key columns over the rows passing a filter,
// plus the passing-row count.  out = [min0..min3, max0..max3].
__global__ void k_init_range(int64_t* out, unsigned long long* count) {
  if (threadIdx.x < TQPK_MAX_KEYS) {
    out[threadIdx.x] = INT64_MAX;
    out[TQPK_MAX_KEYS + threadIdx.x] = INT64_MIN;
  }
  if (threadIdx.x == 0) *count = 0;
}

__global__ void __launch_bounds__(kBlock) k_key_range(const __grid_constant__ tqpk_predicate P, RowFilter F, int64_t n,
                                                      KeySet K, int64_t* out, unsigned long long* count, int vec) {
  int64_t mn[TQPK_MAX_KEYS], mx[TQPK_MAX_KEYS];
#pragma unroll
  for (int k = 0; k < TQPK_MAX_KEYS; ++k) { mn[k] = INT64_MAX; mx[k] = INT64_MIN; }
  unsigned cnt = 0;
  const int64_t groups = (n + 3) >> 2;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = g << 2;
    const uint32_t b = filter4(F, P, r0, n);
    if (!b) continue;
    cnt += __popc(b);
#pragma unroll
    for (int k = 0; k < TQPK_MAX_KEYS; ++k) {
      if (k >= K.n) break;
      int64_t x[4];
      ld4_int(K.col[k], K.dt[k], r0, n, vec, x);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if ((b >> j) & 1u) { mn[k] = min(mn[k], x[j]); mx[k] = max(mx[k], x[j]); }
    }
  }
  for (int k = 0; k < K.n; ++k) {
    int64_t a = mn[k], z = mx[k];
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      a = min(a, (int64_t)__shfl_xor_sync(0xffffffffu, (long long)a, o));
      z = max(z, (int64_t)__shfl_xor_sync(0xffffffffu, (long long)z, o));
    }
    if ((threadIdx.x & 31) == 0 && a <= z) {
      atomicMin(reinterpret_cast<long long*>(&out[k]), (long long)a);
      atomicMax(reinterpret_cast<long long*>(&out[TQPK_MAX_KEYS + k]), (long long)z);
    }
  }
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(count, (unsigned long long)cnt);
}

// ---------------------------------------------------------------- host side
bool pred_vec_ok(const tqpk_predicate* p) {
  if (!p) return true;
  for (int c = 0; c < p->n_cols; ++c)
    if (!aligned16(p->cols[c])) return false;
  return true;
}

int check_pred(const tqpk_predicate* p) {
  if (!p) return TQPK_OK;
  if (p->n_insn < 0 || p->n_insn > TQPK_MAX_PRED || p->n_cols < 0 || p->n_cols > TQPK_MAX_COLS) return TQPK_EINVAL;
  int depth = 0;
  for (int k = 0; k < p->n_insn; ++k) {
    const tqpk_pred_insn& I = p->insn[k];
    switch (I.op) {
      case TQPK_P_CMP:
      case TQPK_P_MASK:
        if (I.col < 0 || I.col >= p->n_cols || !p->cols[I.col]) return TQPK_EINVAL;
        if (!dtype_size(p->dtypes[I.col])) return TQPK_EDTYPE;
        if (I.op == TQPK_P_CMP && I.domain == TQPK_DOM_F64 && p->dtypes[I.col] != TQPK_F64 &&
            I.cmp == TQPK_ISCLOSE)
          return TQPK_EINVAL;
        if (I.op == TQPK_P_MASK && dtype_size(p->dtypes[I.col]) != 1) return TQPK_EDTYPE;
        ++depth;
        break;
      case TQPK_P_CMPCOL:
        if (I.col < 0 || I.col >= p->n_cols || !p->cols[I.col] || I.lit_i < 0 || I.lit_i >= p->n_cols ||
            !p->cols[I.lit_i] || I.cmp == TQPK_ISCLOSE)
          return TQPK_EINVAL;
        if (!dtype_size(p->dtypes[I.col]) || !dtype_size(p->dtypes[I.lit_i])) return TQPK_EDTYPE;
        ++depth;
        break;
      case TQPK_P_STRCMP:
      case TQPK_P_PREFIX:
      case TQPK_P_CONTAINS:
      case TQPK_P_LIKE2: {
        if (I.col < 0 || I.col >= p->n_cols || !p->cols[I.col]) return TQPK_EINVAL;
        if (dtype_size(p->dtypes[I.col]) != 1) return TQPK_EDTYPE;
        const int64_t w = p->widths[I.col];
        const uint64_t L = (uint64_t)I.lit_i;
        if (w <= 0 || p->strides[I.col] < 0 || (p->strides[I.col] > 0 && p->strides[I.col] < w)) return TQPK_EINVAL;
        bool ok;
        if (I.op == TQPK_P_STRCMP) {
          ok = (L & 0xffffffffu) + w <= TQPK_MAX_STRPOOL && I.cmp >= TQPK_LT && I.cmp <= TQPK_NE;
        } else if (I.op == TQPK_P_LIKE2) {
          ok = (L & 0xffff) + ((L >> 16) & 0xffff) <= TQPK_MAX_STRPOOL &&
               ((L >> 32) & 0xffff) + (L >> 48) <= TQPK_MAX_STRPOOL;
        } else {
          ok = (L & 0xffffffffu) + (L >> 32) <= TQPK_MAX_STRPOOL && (I.op != TQPK_P_PREFIX || (int64_t)(L >> 32) <= w);
        }
        if (!ok) return TQPK_EINVAL;
        ++depth;
        break;
      }
      case TQPK_P_TRUE:
      case TQPK_P_FALSE: ++depth; break;
      case TQPK_P_AND:
      case TQPK_P_OR:
        if (depth < 2) return TQPK_EINVAL;
        --depth;
        break;
      case TQPK_P_NOT:
        if (depth < 1) return TQPK_EINVAL;
        break;
      default: return TQPK_EINVAL;
    }
  }
  return (p->n_insn == 0 || depth == 1) ? TQPK_OK : TQPK_EINVAL;
}

bool spec_cols_vec(const tqpk_groupby_spec* S) {
  if (!S) return true;
  for (int c = 0; c < S->n_cols; ++c)
    if (!aligned16(S->cols[c])) return false;
  return true;
}

RowFilter make_filter(const tqpk_predicate* pred, const uint8_t* mask) {
  RowFilter F;
  F.mask = mask;
  F.use_pred = (pred != nullptr && mask == nullptr) ? 1 : 0;
  F.mask_vec = mask ? ((reinterpret_cast<uintptr_t>(mask) & 3u) == 0) : 0;
  F.pred_vec = pred_vec_ok(pred) ? 1 : 0;
  return F;
}

const tqpk_predicate* pred_or_empty(const tqpk_predicate* p) {
  static const tqpk_predicate empty = {};
  return p ? p : &empty;
}

int grid_for(int64_t work_items, int per_sm) {
  int64_t g = (work_items + kBlock - 1) / kBlock;
  int64_t cap = (int64_t)num_sms() * per_sm;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

// Shared by the group-by and join planners: min/max of key columns over the
// filtered rows.  scratch holds 8 int64 + 1 counter; synchronises.
int key_ranges(const tqpk_predicate* pred, const uint8_t* mask, int64_t n, int nk, const void* const* cols,
               const int32_t* dts, int64_t* h_min, int64_t* h_max, int64_t* h_count, void* scratch,
               cudaStream_t s) {
  if (nk < 0 || nk > TQPK_MAX_KEYS || !scratch) return TQPK_EINVAL;
  if (n == 0) {  // no rows: empty ranges (min > max); empty tensors may carry null pointers
    for (int k = 0; k < nk; ++k) {
      h_min[k] = 0;
      h_max[k] = -1;
    }
    *h_count = 0;
    return TQPK_OK;
  }
  KeySet K;
  K.n = nk;
  bool vec = true;
  for (int k = 0; k < nk; ++k) {
    if (!cols[k] || !is_int_dtype(dts[k])) return cols[k] ? TQPK_EDTYPE : TQPK_EINVAL;
    K.col[k] = cols[k];
    K.dt[k] = dts[k];
    vec = vec && aligned16(cols[k]);
  }
  int64_t* out = static_cast<int64_t*>(scratch);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(out + 2 * TQPK_MAX_KEYS);
  k_init_range<<<1, 32, 0, s>>>(out, cnt);
  TQPK_CHECK_LAUNCH();
  if (n > 0) {
    RowFilter F = make_filter(pred, mask);
    k_key_range<<<grid_for((n + 3) / 4, 4), kBlock, 0, s>>>(*pred_or_empty(pred), F, n, K, out, cnt, vec ? 1 : 0);
    TQPK_CHECK_LAUNCH();
  }
  int64_t host[2 * TQPK_MAX_KEYS + 1];
  TQPK_CUDA(cudaMemcpyAsync(host, out, sizeof(host), cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < nk; ++k) {
    h_min[k] = host[k];
    h_max[k] = host[TQPK_MAX_KEYS + k];
  }
  *h_count = host[2 * TQPK_MAX_KEYS];
  return TQPK_OK;
}

// Stable compaction used inside the library (groups, join rows).
// Workspace of one compaction: the control block, then one status word per tile (both
// 256-byte aligned pieces, as compact_launch takes them).
size_t compact_status_bytes(int64_t n) { return kCompactCtlBytes + align_up(((n + kTile - 1) / kTile) * 8, 256); }

int compact_launch(const tqpk_predicate* pred, const uint8_t* mask, int64_t n, const ColSet& C, int64_t* d_count,
                   void* ws, size_t ws_bytes, cudaStream_t s) {
  const int64_t tiles = (n + kTile - 1) / kTile;
  WsCursor cur(ws, ws_bytes);
  CompactCtl* ctl = reinterpret_cast<CompactCtl*>(cur.take<unsigned char>(kCompactCtlBytes));
  uint64_t* status = cur.take<uint64_t>(tiles > 0 ? tiles : 1);
  if (!ctl || !status) return TQPK_ENOMEM;
  TQPK_CUDA(cudaMemsetAsync(ws, 0, cur.off, s));
  if (tiles == 0) {
    TQPK_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int64_t), s));
    return TQPK_OK;
  }
  if (tiles > INT32_MAX) return TQPK_EUNSUPPORTED;
  RowFilter F = make_filter(pred, mask);
  k_compact<<<(int)tiles, kBlock, 0, s>>>(*pred_or_empty(pred), F, n, C, d_count, status, ctl, g_dbg_spin_limit,
                                          g_dbg_stall_tile);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

}  // namespace tqpk

using namespace tqpk;

extern "C" int tqpk_version(void) { return 1; }

extern "C" const char* tqpk_status_string(int status) {
  switch (status) {
    case TQPK_OK: return "ok";
    case TQPK_EINVAL: return "invalid argument";
    case TQPK_ENOMEM: return "workspace too small";
    case TQPK_ETIMEOUT: return "bounded device wait expired";
    case TQPK_EDTYPE: return "unsupported dtype";
    case TQPK_ECUDA: return "CUDA error";
    case TQPK_ECAPACITY: return "output capacity too small";
    case TQPK_EUNSUPPORTED: return "unsupported shape";
  }
  return "unknown status";
}

extern "C" int64_t tqpk_launch_count(void) { return g_launches; }

extern "C" int tqpk_timing_begin(int32_t kernel_id) {
  if (!g_timing.created) {
    for (int i = 0; i < 2 * 4096; ++i) TQPK_CUDA(cudaEventCreate(&g_timing.ev[i]));
    g_timing.created = true;
  }
  g_timing.kid = kernel_id;
  g_timing.n = 0;
  return TQPK_OK;
}

extern "C" int tqpk_timing_end(double* h_total_ms, int32_t* h_launches) {
  if (!h_total_ms || !h_launches) return TQPK_EINVAL;
  double total = 0.0;
  for (int i = 0; i < g_timing.n; ++i) {
    TQPK_CUDA(cudaEventSynchronize(g_timing.ev[2 * i + 1]));
    float ms = 0.f;
    TQPK_CUDA(cudaEventElapsedTime(&ms, g_timing.ev[2 * i], g_timing.ev[2 * i + 1]));
    total += ms;
  }
  *h_total_ms = total;
  *h_launches = g_timing.n;
  g_timing.kid = KID_NONE;
  g_timing.n = 0;
  return TQPK_OK;
}

extern "C" int tqpk_abi_sizes(int64_t* out, int n) {
  const int64_t sizes[] = {sizeof(tqpk_pred_insn), sizeof(tqpk_predicate), sizeof(tqpk_expr_insn), sizeof(tqpk_acc),
                           sizeof(tqpk_groupby_spec), sizeof(tqpk_gb_plan), sizeof(tqpk_join_plan)};
  const int k = (int)(sizeof(sizes) / sizeof(sizes[0]));
  for (int i = 0; i < n && i < k; ++i) out[i] = sizes[i];
  return k;
}

extern "C" int tqpk_filter_mask(const tqpk_predicate* h_pred, int64_t n, uint8_t* d_mask,
                                unsigned long long* d_count, tqpk_stream stream) {
  if (!h_pred || n < 0 || (n > 0 && !d_mask)) return TQPK_EINVAL;
  int rc = check_pred(h_pred);
  if (rc) return rc;
  if (n == 0) return TQPK_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int mask_vec = (reinterpret_cast<uintptr_t>(d_mask) & 3u) == 0;
  timing_before(KID_FILTER_MASK, s);
  k_filter_mask<<<grid_for((n + 3) / 4, 8), kBlock, 0, s>>>(*h_pred, n, d_mask, d_count, pred_vec_ok(h_pred) ? 1 : 0,
                                                          mask_vec);
  timing_after(KID_FILTER_MASK, s);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

// Test hook: the poll limit of the compaction's look-back, and a tile whose CTA publishes nothing
// (its successors' bounded waits then run out and the call's count becomes TQPK_ETIMEOUT).
// (kSpinLimit or less, -1) restores the defaults.  Not thread-safe; for tests only.
extern "C" int tqpk_debug_compact_wait(int32_t spin_limit, int64_t stall_tile) {
  if (spin_limit < 0 || spin_limit > kSpinLimit || stall_tile < -1) return TQPK_EINVAL;
  g_dbg_spin_limit = spin_limit;
  g_dbg_stall_tile = stall_tile;
  return TQPK_OK;
}

// [min, max] of one integer column over all n rows (one host synchronisation); d_scratch holds
// 256 bytes.  An empty column gives min > max.
extern "C" int tqpk_key_range(const void* d_col, int32_t dtype, int64_t n, void* d_scratch, int64_t* h_min,
                              int64_t* h_max, tqpk_stream stream) {
  if (n < 0 || !d_scratch || !h_min || !h_max || (n > 0 && !d_col)) return TQPK_EINVAL;
  int64_t cnt = 0;
  const void* cols[1] = {d_col};
  const int32_t dts[1] = {dtype};
  return key_ranges(nullptr, nullptr, n, 1, cols, dts, h_min, h_max, &cnt, d_scratch,
                    static_cast<cudaStream_t>(stream));
}

extern "C" size_t tqpk_compact_workspace_bytes(int64_t n) { return compact_status_bytes(n < 0 ? 0 : n); }

extern "C" int tqpk_compact(const tqpk_predicate* h_pred, const uint8_t* d_mask, int64_t n, int32_t ncols,
                            const void* const* h_cols_in, const int32_t* h_dtypes, void* const* h_cols_out,
                            int64_t* d_count, void* d_ws, size_t ws_bytes, tqpk_stream stream) {
  if (n < 0 || ncols < 0 || ncols > TQPK_MAX_COLS || !d_count || !d_ws) return TQPK_EINVAL;
  if (n == 0) {  // nothing to keep; empty tensors may carry null pointers
    TQPK_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int64_t), static_cast<cudaStream_t>(stream)));
    return TQPK_OK;
  }
  if (!h_pred && !d_mask) return TQPK_EINVAL;
  int rc = check_pred(h_pred);
  if (rc) return rc;
  ColSet C;
  C.n = ncols;
  for (int c = 0; c < ncols; ++c) {
    const int sz = dtype_size(h_dtypes[c]);
    if (!sz && h_dtypes[c] != TQPK_ROWID) return TQPK_EDTYPE;
    if (n > 0 && ((sz && !h_cols_in[c]) || !h_cols_out[c])) return TQPK_EINVAL;
    C.in[c] = h_cols_in[c];
    C.out[c] = h_cols_out[c];
    C.size[c] = sz;
  }
  return compact_launch(d_mask ? nullptr : h_pred, d_mask, n, C, d_count, d_ws, ws_bytes,
                        static_cast<cudaStream_t>(stream));
}

namespace tqpk {
__global__ void k_mark_rows(const int64_t* __restrict__ idx, int64_t n_idx, uint8_t* __restrict__ flags, int64_t n) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n_idx; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx[j];
    if (i >= 0 && i < n) flags[i] = 1;
  }
}
}  // namespace tqpk

// flags[idx[j]] = 1 for every j (indices outside [0, n) are skipped): the rows a set of
// join pairs touches, for the semi / anti / outer forms of a join with extra conditions.
extern "C" int tqpk_mark_rows(const int64_t* d_idx, int64_t n_idx, uint8_t* d_flags, int64_t n, tqpk_stream stream) {
  if (n_idx < 0 || n < 0 || (n_idx > 0 && (!d_idx || !d_flags))) return TQPK_EINVAL;
  if (n_idx == 0) return TQPK_OK;
  k_mark_rows<<<grid_for(n_idx, 4), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(d_idx, n_idx, d_flags, n);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}
