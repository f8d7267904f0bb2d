// topk.cuh - kernel (e): stable top-k with warp-resident sorted lists.
//
// Reference: operators/sort.py:41-42 sorts everything (stable) and keeps
// perm[:limit].  The stable top-k order is lexicographic on
// (order-preserving key, position), smaller first, so ties keep input order.
//
// Items are cut by a threshold found from group bests, the few survivors are
// sorted in one CTA (see k_tk_group_best below).  WarpList keeps a warp's best
// k entries as a sorted list striped over the warp (entry p = row p/32 of lane
// p%32, R rows per lane, k <= 32*R); a batch of 32 candidates is compared
// against the current k-th entry and the survivors are inserted one by one
// (rank by ballot/popc, shift by shuffles).  It serves the tie-heavy fallback
// and the batched kernels.
#pragma once

#include "common.cuh"

namespace tqpk {

__device__ __forceinline__ bool tk_better(uint64_t ka, int64_t ia, uint64_t kb, int64_t ib) {
  return ka < kb || (ka == kb && ia < ib);
}

template <int R>
struct WarpList {
  uint64_t key[R];
  int64_t idx[R];  // -1 = empty
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int r = 0; r < R; ++r) { key[r] = ~0ull; idx[r] = -1; }
  }
  // entry at position p (warp-uniform p)
  __device__ __forceinline__ void at(int p, uint64_t& k, int64_t& i) const {
    const int rr = p >> 5, ll = p & 31;
    k = ~0ull;
    i = -1;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint64_t kk = __shfl_sync(0xffffffffu, key[r], ll);
      const int64_t ii = __shfl_sync(0xffffffffu, idx[r], ll);
      if (r == rr) { k = kk; i = ii; }
    }
  }
  __device__ __forceinline__ void insert(int k, uint64_t ck, int64_t ci) {
    const int lane = threadIdx.x & 31;
    int pos = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const bool b = (r * 32 + lane < k) && idx[r] >= 0 && tk_better(key[r], idx[r], ck, ci);
      pos += __popc(__ballot_sync(0xffffffffu, b));
    }
    if (pos >= k) return;
#pragma unroll
    for (int r = R - 1; r >= 0; --r) {
      uint64_t uk = __shfl_up_sync(0xffffffffu, key[r], 1);
      int64_t ui = __shfl_up_sync(0xffffffffu, idx[r], 1);
      if (r > 0) {
        const uint64_t pk = __shfl_sync(0xffffffffu, key[r - 1], 31);
        const int64_t pi = __shfl_sync(0xffffffffu, idx[r - 1], 31);
        if (lane == 0) { uk = pk; ui = pi; }
      }
      const int p = r * 32 + lane;
      if (p > pos && p < k) { key[r] = uk; idx[r] = ui; }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (r * 32 + lane == pos) { key[r] = ck; idx[r] = ci; }
  }
  // Inserts the valid lanes' candidates that beat the current k-th entry.
  // ext is a key bound known from elsewhere (some list already holds k keys
  // <= ext): strictly larger keys cannot reach the top k and are skipped.
  __device__ __forceinline__ void offer(int k, uint64_t ck, int64_t ci, bool valid, uint64_t ext = ~0ull) {
    uint64_t tk;
    int64_t ti;
    at(k - 1, tk, ti);
    const bool cand = valid && ck <= ext && (ti < 0 || tk_better(ck, ci, tk, ti));
    uint32_t pending = __ballot_sync(0xffffffffu, cand);
    while (pending) {
      const int src = __ffs(pending) - 1;
      pending &= pending - 1;
      const uint64_t k0 = __shfl_sync(0xffffffffu, ck, src);
      const int64_t i0 = __shfl_sync(0xffffffffu, ci, src);
      insert(k, k0, i0);
    }
  }
};

// Candidate sources -----------------------------------------------------------
// Occupied slots of a dense group table, keyed by their float64 sum.
struct DenseSumSource {
  const double* sum;
  const unsigned* cnt;   // occupancy: non-zero for groups that received a row; NULL: the sums
                         // start at -0.0 and every added value is +0.0 or non-zero, so a slot is
                         // occupied exactly when its bits are no longer those of -0.0
  int64_t n;
  int desc;
  const unsigned* bits = nullptr;   // when set, only slots whose bit is set can be occupied (the join's
                                    // build writes its passing keys' bits and initialises those sums)
  static constexpr uint64_t kEmptySum = 0x8000000000000000ull;
  __device__ __forceinline__ uint64_t order_key(double v) const {
    const uint64_t b = f64_canon_bits(d2u(v));       // integer instructions only (no FP64 compares)
    const uint64_t u = (b & (1ull << 63)) ? ~b : (b | (1ull << 63));
    return desc ? ~u : u;
  }
  // The membership nibble of slots i0..i0+3 (i0 % 4 == 0): all ones without a bitmap.
  __device__ __forceinline__ unsigned bits4(int64_t i0) const {
    if (!bits) return 0xfu;
    return (__ldcg(&bits[i0 >> 5]) >> (i0 & 31)) & 0xfu;
  }
  __device__ __forceinline__ bool get(int64_t i, uint64_t& k) const {
    if (i >= n) return false;
    if (bits && !((__ldcg(&bits[i >> 5]) >> (i & 31)) & 1u)) return false;
    if (!cnt) {
      const double v = __ldcg(&sum[i]);
      if (d2u(v) == kEmptySum) return false;
      k = order_key(v);
      return true;
    }
    if (__ldcg(&cnt[i]) == 0) return false;   // L2 loads: the table may have been written
    k = order_key(__ldcg(&sum[i]));           // earlier in the same launch by other CTAs
    return true;
  }
  // Slots i0..i0+3 (i0 % 4 == 0): the occupancy and sum loads are issued
  // together (16-byte vectors when aligned), so a warp keeps 3 independent
  // loads per lane in flight instead of two dependent ones per slot.
  __device__ __forceinline__ unsigned get4(int64_t i0, uint64_t* k) const {
    unsigned c[4];
    double v[4];
    if (!cnt) {
      if (i0 + 4 <= n && (reinterpret_cast<uintptr_t>(sum) & 15u) == 0) {
        const double2 a = __ldcg(reinterpret_cast<const double2*>(sum + i0));
        const double2 b = __ldcg(reinterpret_cast<const double2*>(sum + i0 + 2));
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = (i0 + q < n) ? __ldcg(&sum[i0 + q]) : u2d(kEmptySum);
      }
      unsigned ok = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        k[q] = order_key(v[q]);
        ok |= (d2u(v[q]) != kEmptySum ? 1u : 0u) << q;
      }
      return ok & bits4(i0);
    }
    if (i0 + 4 <= n && ((reinterpret_cast<uintptr_t>(cnt) | reinterpret_cast<uintptr_t>(sum)) & 15u) == 0) {
      const uint4 cc = __ldcg(reinterpret_cast<const uint4*>(cnt + i0));
      const double2 a = __ldcg(reinterpret_cast<const double2*>(sum + i0));
      const double2 b = __ldcg(reinterpret_cast<const double2*>(sum + i0 + 2));
      c[0] = cc.x; c[1] = cc.y; c[2] = cc.z; c[3] = cc.w;
      v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        c[q] = (i0 + q < n) ? __ldcg(&cnt[i0 + q]) : 0u;
        v[q] = (i0 + q < n) ? __ldcg(&sum[i0 + q]) : 0.0;
      }
    }
    unsigned ok = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      k[q] = order_key(v[q]);
      ok |= (c[q] != 0u ? 1u : 0u) << q;
    }
    return ok & bits4(i0);
  }
};

// keys[perm_in[i]] (perm_in may be null) of any dtype, position i.
struct ArraySource {
  const void* keys;
  int dt;
  const int64_t* perm;
  int64_t n;
  int desc;
  __device__ __forceinline__ bool get(int64_t i, uint64_t& k) const;
  __device__ __forceinline__ unsigned bits4(int64_t) const { return 0xfu; }
  __device__ __forceinline__ unsigned get4(int64_t i0, uint64_t* k) const {
    unsigned ok = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) ok |= (get(i0 + q, k[q]) ? 1u : 0u) << q;
    return ok;
  }
};

struct TopkOut {
  int64_t* out_idx;     // positions (or slots) of the best entries
  int64_t* out_count;   // min(k, valid items)
  uint64_t* cand_key;   // [grid][k]
  int64_t* cand_idx;
  unsigned* ticket;
  unsigned long long* valid_total;  // number of valid items seen (may be null)
  unsigned long long* bound;        // the cut (written by the first pass)
  unsigned* arrive;                 // [2] CTAs done with the group-best and the filter pass (zeroed before the launch)
  // Optional, for a dense group table: the last CTA also writes (key_min + slot, sum[slot]) of the
  // top rows and their number (emit_keys null: not written) ...
  int64_t* emit_keys = nullptr;
  double* emit_vals = nullptr;
  int64_t* emit_count = nullptr;
  const double* emit_sum = nullptr;
  int64_t emit_key_min = 0;
  // ... and checks that the membership bits set (counted into bits_set, zeroed before the launch)
  // are as many as the rows that set them (bits_expected): fewer means a repeated key, reported
  // as TQPK_EUNSUPPORTED in *err.  bits_set null: no check.
  unsigned long long* bits_set = nullptr;
  const unsigned long long* bits_expected = nullptr;
  int* err = nullptr;
};

// ---------------------------------------------------------------------------
// Threshold top-k (the default): one pass over the items cuts them into at
// most kTopkGroups groups of G consecutive items and keeps each group's best
// key; the k-th best of those group bests is a cut T with at least k items
// at or below it (every one of those k groups holds one), so the top k are
// all among the items with key <= T.  For independent keys only about k
// items pass T.  A second pass appends them to a candidate list (at most
// kTopkCap), and the last CTA of that pass sorts the list bitonically by
// (key, index) in shared memory.  When ties push more than kTopkSortCap items
// under the cut, that CTA falls back to the warp lists over all items (same
// result, slower).  For k > 32 the cut is computed by the last CTA of the
// first pass and the top-k is two launches; for k <= 32 every CTA of the
// second pass derives the cut from the group bests (tk_bin_cut), and when
// each CTA's group fits one sweep of its threads the two passes run as one
// cooperative launch with a grid barrier between them (k_tk_fused below).
constexpr int kTopkCap = 4096;
constexpr int kTopkGroups = 512;     // >= 2 x the largest k: the cut stays near the k-th item
constexpr int kTopkCand = kTopkCap + kTopkGroups;   // cand_key entries used: candidates, then group bests

__device__ __forceinline__ void block_min_u64(uint64_t& v, uint64_t* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; ++w) v = red[w] < v ? red[w] : v;
    red[0] = v;
  }
  __syncthreads();
  v = red[0];
}

// True in the last CTA of the grid to get here, after every other CTA has made its
// writes visible; all threads of every CTA call it once, at the end of the kernel.  No CTA
// waits for another: the others have finished.
__device__ __forceinline__ bool tk_last_cta(unsigned* arrive) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(arrive, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// The cut for k > 32: the k-th best of the ng group bests (bitonic sort of the bests in one CTA).
__device__ __forceinline__ void tk_cut(int ng, int k, TopkOut O) {
  __shared__ uint64_t v[kTopkGroups];
  for (int i = threadIdx.x; i < kTopkGroups; i += blockDim.x) v[i] = i < ng ? __ldcg(&O.cand_key[kTopkCap + i]) : ~0ull;
  __syncthreads();
  for (int size = 2; size <= kTopkGroups; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < kTopkGroups / 2; t += blockDim.x) {
        const int i = 2 * t - (t & (stride - 1)), j = i + stride;
        const bool up = (i & size) == 0;
        const uint64_t a = v[i], b = v[j];
        if ((a > b) == up) { v[i] = b; v[j] = a; }
      }
      __syncthreads();
    }
  if (threadIdx.x == 0) *O.bound = v[(k <= kTopkGroups ? k : kTopkGroups) - 1];
}

// One CTA's walk over items [b0, b1) in quads (4 items per thread, 256 threads): kTopkQuads
// quads per thread are loaded before any is looked at, so a thread keeps that many loads in
// flight (the passes are latency-bound on tables resident in L2).  f(key, index, lane_has_item)
// runs for every item slot in warp-uniform order (lanes without an item pass false), so f may use
// warp collectives; valid / nbits count the items and the membership bits seen.
constexpr int kTopkQuads = 4;
template <class Src, class F>
__device__ __forceinline__ void tk_scan_group(const Src& src, int64_t b0, int64_t b1, bool count_bits, F f,
                                              unsigned& valid, unsigned& nbits) {
  for (int64_t c0 = b0 + threadIdx.x * 4; c0 - threadIdx.x * 4 < b1; c0 += 4 * 256 * kTopkQuads) {
    uint64_t key[kTopkQuads][4];
    unsigned ok[kTopkQuads];
#pragma unroll
    for (int u = 0; u < kTopkQuads; ++u) {
      const int64_t i0 = c0 + u * 1024;
      ok[u] = 0;
      if (i0 < b1) {
        const unsigned tail = i0 + 4 <= b1 ? 0xfu : (1u << (b1 - i0)) - 1u;
        ok[u] = src.get4(i0, key[u]) & tail;
        if (count_bits) nbits += __popc(src.bits4(i0) & tail);
      }
    }
#pragma unroll
    for (int u = 0; u < kTopkQuads; ++u) {
      valid += __popc(ok[u]);
#pragma unroll
      for (int q = 0; q < 4; ++q) f(key[u][q], c0 + u * 1024 + q, ((ok[u] >> q) & 1u) != 0);
    }
  }
}

// Pass 1: each CTA keeps the best key of its group of G items; the last CTA to finish
// computes the cut from all groups' bests.
template <class Src>
__global__ void __launch_bounds__(256) k_tk_group_best(Src src, int64_t G, int k, TopkOut O) {
  __shared__ uint64_t red[8];
  const int64_t b0 = (int64_t)blockIdx.x * G, b1 = b0 + G < src.n ? b0 + G : src.n;
  __shared__ unsigned s_valid, s_bits;
  if (threadIdx.x == 0) { s_valid = 0; s_bits = 0; }
  __syncthreads();
  uint64_t best = ~0ull;
  unsigned valid = 0, nbits = 0;
  tk_scan_group(src, b0, b1, O.bits_set != nullptr, [&](uint64_t key, int64_t, bool has) {
    if (has && key < best) best = key;          // slots without an item carry no key
  }, valid, nbits);
  // one atomic per CTA for each count: per-warp atomics on one address serialise in the L2
  valid = __reduce_add_sync(0xffffffffu, valid);
  nbits = __reduce_add_sync(0xffffffffu, nbits);
  if ((threadIdx.x & 31) == 0) {
    if (valid) atomicAdd(&s_valid, valid);
    if (nbits) atomicAdd(&s_bits, nbits);
  }
  block_min_u64(best, red);        // its barriers order the shared counts too
  if (threadIdx.x == 0) {
    O.cand_key[kTopkCap + blockIdx.x] = best;
    if (blockIdx.x == 0) *O.ticket = 0;          // the candidate counter of the next pass
    if (s_valid && O.valid_total) atomicAdd(O.valid_total, (unsigned long long)s_valid);
    if (s_bits && O.bits_set) atomicAdd(O.bits_set, (unsigned long long)s_bits);
  }
  if (k <= 32) return;              // the filter pass derives its cut from the group bests itself
  if (tk_last_cta(O.arrive)) tk_cut((int)gridDim.x, k, O);
}

// The cut for k <= 32, computed by every CTA of the filter pass from the ng group bests (no
// serial step between the passes): the groups that hold an item are dealt round-robin into k
// bins and the cut is the largest of the bins' smallest keys.  Each bin's smallest key belongs to
// an item of its own group, so at least k items lie at or under the cut, and the top k are among
// them; for independent keys about k ln k items pass.  Fewer than k non-empty groups: ~0 (every
// item passes).  Called by all threads.
__device__ __forceinline__ uint64_t tk_bin_cut(int ng, int k, const TopkOut& O) {
  __shared__ unsigned long long bin[32];
  __shared__ unsigned s_ne;
  __shared__ unsigned long long s_cut;
  if (threadIdx.x < 32) bin[threadIdx.x] = ~0ull;
  if (threadIdx.x == 0) { s_ne = 0; s_cut = 0; }
  __syncthreads();
  // the rank of a non-empty group among the non-empty ones decides its bin: groups are read in
  // index order in chunks of 256, each chunk's non-empty ones numbered by a block scan
  __shared__ int wsum[8];
  for (int base = 0; base < ng; base += 256) {
    const int g = base + threadIdx.x;
    const uint64_t v = g < ng ? __ldcg(&O.cand_key[kTopkCap + g]) : ~0ull;
    const bool ne = v != ~0ull;
    const unsigned m = __ballot_sync(0xffffffffu, ne);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wsum[warp] = __popc(m);
    __syncthreads();
    int before = s_ne;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    if (ne) atomicMin(&bin[(before + __popc(m & ((1u << lane) - 1u))) % k], (unsigned long long)v);
    __syncthreads();
    if (threadIdx.x == 0) for (int w = 0; w < 8; ++w) s_ne += wsum[w];
    __syncthreads();
  }
  if (threadIdx.x < 32) {
    unsigned long long c = threadIdx.x < k ? bin[threadIdx.x] : 0ull;
#pragma unroll
    for (int o = 16; o; o >>= 1) { const unsigned long long w = __shfl_xor_sync(0xffffffffu, c, o); c = w > c ? w : c; }
    if (threadIdx.x == 0) s_cut = s_ne >= (unsigned)k ? c : ~0ull;
  }
  __syncthreads();
  return s_cut;
}

constexpr int kTopkSortCap = 2048;   // candidates the final CTA sorts in shared memory

// The last CTA's outputs: the count, the optional dense-table rows (key_min + slot, sum) and the
// membership-bit check.  si[0..m) holds the winners' indices.  tk_finish: every thread of the
// CTA; tk_finish_warp: one warp.
__device__ __forceinline__ void tk_emit(int j, const TopkOut& O, const int64_t* si) {
  if (O.emit_keys) {
    O.emit_keys[j] = O.emit_key_min + si[j];
    O.emit_vals[j] = __ldcg(&O.emit_sum[si[j]]);
  }
}
__device__ __forceinline__ void tk_counts(int m, const TopkOut& O) {
  *O.out_count = m;
  if (O.emit_count) *O.emit_count = m;
  if (O.bits_set && O.bits_expected && O.err && atomicAdd(O.bits_set, 0ull) != __ldcg(O.bits_expected))
    set_error(O.err, TQPK_EUNSUPPORTED);     // fewer bits than passing build rows: a repeated key
}
__device__ __forceinline__ void tk_finish(int m, const TopkOut& O, const int64_t* si) {
  for (int j = threadIdx.x; j < m; j += blockDim.x) tk_emit(j, O, si);
  if (threadIdx.x == 0) tk_counts(m, O);
}
__device__ __forceinline__ void tk_finish_warp(int m, const TopkOut& O, const int64_t* si) {
  for (int j = threadIdx.x & 31; j < m; j += 32) tk_emit(j, O, si);
  if ((threadIdx.x & 31) == 0) tk_counts(m, O);
}

// The final step, in one CTA: sort the candidates under the cut by (key, index), or, when
// ties put more than kTopkSortCap items under it, warp lists over every item.
template <int R, class Src>
__device__ __forceinline__ void tk_final(const Src& src, int k, TopkOut O) {
  __shared__ uint64_t sk[kTopkSortCap];
  __shared__ int64_t si[kTopkSortCap];
  const unsigned cnt = __ldcg(O.ticket);
  if (cnt <= 256u) {
    // few candidates: each thread ranks one against all of them (one pass over shared memory,
    // two barriers) and writes it at its rank when that is among the first k
    if (threadIdx.x < cnt) {
      sk[threadIdx.x] = __ldcg(&O.cand_key[threadIdx.x]);
      si[threadIdx.x] = __ldcg(&O.cand_idx[threadIdx.x]);
    }
    __syncthreads();
    int rank = 0;
    uint64_t mk = 0;
    int64_t mi = 0;
    if (threadIdx.x < cnt) {
      mk = sk[threadIdx.x];
      mi = si[threadIdx.x];
      for (int j = 0; j < (int)cnt; ++j) rank += tk_better(sk[j], si[j], mk, mi) ? 1 : 0;
    }
    __syncthreads();
    if (threadIdx.x < cnt && rank < k) {
      O.out_idx[rank] = mi;
      si[rank] = mi;
    }
    __syncthreads();
    tk_finish((int)cnt < k ? (int)cnt : k, O, si);
    return;
  }
  if (cnt <= (unsigned)kTopkSortCap) {
    int P = 2;
    while (P < (int)cnt) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      const bool in = i < (int)cnt;
      sk[i] = in ? __ldcg(&O.cand_key[i]) : ~0ull;
      si[i] = in ? __ldcg(&O.cand_idx[i]) : INT64_MAX;
    }
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int t = threadIdx.x; t < P / 2; t += blockDim.x) {
          const int i = 2 * t - (t & (stride - 1)), j = i + stride;
          const bool up = (i & size) == 0;
          const uint64_t ka = sk[i], kb = sk[j];
          const int64_t ia = si[i], ib = si[j];
          if (tk_better(kb, ib, ka, ia) == up) { sk[i] = kb; sk[j] = ka; si[i] = ib; si[j] = ia; }
        }
        __syncthreads();
      }
    const int m = (int)cnt < k ? (int)cnt : k;
    for (int j = threadIdx.x; j < m; j += blockDim.x) O.out_idx[j] = si[j];
    tk_finish(m, O, si);
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpList<R> L;
  L.init();
  for (int64_t base = warp * 128; base < src.n; base += 8 * 128) {
    const int64_t i0 = base + lane * 4;
    uint64_t key[4];
    const unsigned ok = src.get4(i0, key);
#pragma unroll
    for (int q = 0; q < 4; ++q) L.offer(k, key[q], i0 + q, (ok >> q) & 1u);
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    sk[warp * 32 * R + r * 32 + lane] = L.key[r];
    si[warp * 32 * R + r * 32 + lane] = L.idx[r];
  }
  __syncthreads();
  if (warp != 0) return;
  WarpList<R> M;
  M.init();
  for (int w = 0; w < 8; ++w)
    for (int r = 0; r < R; ++r) {
      const int p = r * 32 + lane;
      const int64_t ii = si[w * 32 * R + p];
      M.offer(k, sk[w * 32 * R + p], ii, p < k && ii >= 0);
    }
  int c = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int p = r * 32 + lane;
    const bool v = p < k && M.idx[r] >= 0;
    c += __popc(__ballot_sync(0xffffffffu, v));
    if (v) {
      O.out_idx[p] = M.idx[r];
      si[p] = M.idx[r];
    }
  }
  __syncwarp();
  tk_finish_warp(c, O, si);
}

// Pass 2: the items at or under the cut are appended to the candidate list; the last CTA
// to finish sorts them (tk_final).  Same groups of G items as pass 1, 256 threads per CTA
// (tk_final's 8 warps).
template <int R, class Src>
__global__ void __launch_bounds__(256) k_tk_filter(Src src, int64_t G, int k, TopkOut O) {
  const int lane = threadIdx.x & 31;
  const uint64_t cut = k <= 32 ? tk_bin_cut((int)gridDim.x, k, O) : __ldcg(O.bound);
  const int64_t b0 = (int64_t)blockIdx.x * G, b1 = b0 + G < src.n ? b0 + G : src.n;
  unsigned valid = 0, nbits = 0;
  tk_scan_group(src, b0, b1, false, [&](uint64_t key, int64_t idx, bool has) {
    const bool pass = has && key <= cut;
    const unsigned bal = __ballot_sync(0xffffffffu, pass);
    if (!bal) return;
    unsigned at = 0;
    if (lane == 0) at = atomicAdd(O.ticket, (unsigned)__popc(bal));
    at = __shfl_sync(0xffffffffu, at, 0) + __popc(bal & ((1u << lane) - 1u));
    if (pass && at < (unsigned)kTopkCap) {
      O.cand_key[at] = key;
      O.cand_idx[at] = idx;
    }
  }, valid, nbits);
  if (tk_last_cta(O.arrive + 1)) tk_final<R>(src, k, O);
}

// Both passes in one cooperative launch, for k <= 32 and groups of at most one tk_scan_group
// sweep (G <= 4096 items: kTopkQuads quads per thread): each thread loads its items once and
// keeps their keys in registers across a grid barrier, after which every CTA derives the cut from
// the group bests (tk_bin_cut) and filters the keys it holds.  One launch and one pass over the
// table instead of two.  The barrier wait is bounded: on expiry the CTA records TQPK_ETIMEOUT in
// *O.err (required) and leaves.
constexpr int64_t kTopkFusedMaxG = 4 * 256 * kTopkQuads;
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
template <class Src>
__global__ void __launch_bounds__(256) k_tk_fused(Src src, int64_t G, int k, TopkOut O, int spin_limit,
                                                  int missing) {
  __shared__ uint64_t red[8];
  __shared__ unsigned s_valid, s_bits;
  __shared__ int s_fail;
  const int lane = threadIdx.x & 31;
  const int64_t b0 = (int64_t)blockIdx.x * G, b1 = b0 + G < src.n ? b0 + G : src.n;
  if (threadIdx.x == 0) { s_valid = 0; s_bits = 0; s_fail = 0; }
  __syncthreads();
  uint64_t key[kTopkQuads][4];
  unsigned ok[kTopkQuads];
  unsigned valid = 0, nbits = 0;
  const int64_t c0 = b0 + threadIdx.x * 4;
#pragma unroll
  for (int u = 0; u < kTopkQuads; ++u) {
    const int64_t i0 = c0 + u * 1024;
    ok[u] = 0;
    if (i0 < b1) {
      const unsigned tail = i0 + 4 <= b1 ? 0xfu : (1u << (b1 - i0)) - 1u;
      ok[u] = src.get4(i0, key[u]) & tail;
      if (O.bits_set) nbits += __popc(src.bits4(i0) & tail);
    }
  }
  uint64_t best = ~0ull;
#pragma unroll
  for (int u = 0; u < kTopkQuads; ++u) {
    valid += __popc(ok[u]);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (((ok[u] >> q) & 1u) && key[u][q] < best) best = key[u][q];
  }
  valid = __reduce_add_sync(0xffffffffu, valid);
  nbits = __reduce_add_sync(0xffffffffu, nbits);
  if (lane == 0) {
    if (valid) atomicAdd(&s_valid, valid);
    if (nbits) atomicAdd(&s_bits, nbits);
  }
  block_min_u64(best, red);
  if (threadIdx.x == 0) {
    O.cand_key[kTopkCap + blockIdx.x] = best;
    if (blockIdx.x == 0) *O.ticket = 0;
    if (s_valid && O.valid_total) atomicAdd(O.valid_total, (unsigned long long)s_valid);
    if (s_bits && O.bits_set) atomicAdd(O.bits_set, (unsigned long long)s_bits);
    // grid barrier: every CTA's group best (and the ticket reset) before any cut is taken
    __threadfence();
    atomicAdd(O.arrive, 1u);
    int spins = 0;
    while (ld_acquire_u32(O.arrive) < gridDim.x + (unsigned)missing) {   // missing > 0: a test hook
      if (++spins > spin_limit) { s_fail = 1; set_error(O.err, TQPK_ETIMEOUT); break; }
      __nanosleep(64);
    }
  }
  __syncthreads();
  if (s_fail) return;
  const uint64_t cut = tk_bin_cut((int)gridDim.x, k, O);
#pragma unroll
  for (int u = 0; u < kTopkQuads; ++u)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool pass = ((ok[u] >> q) & 1u) && key[u][q] <= cut;
      const unsigned bal = __ballot_sync(0xffffffffu, pass);
      if (!bal) continue;
      unsigned at = 0;
      if (lane == 0) at = atomicAdd(O.ticket, (unsigned)__popc(bal));
      at = __shfl_sync(0xffffffffu, at, 0) + __popc(bal & ((1u << lane) - 1u));
      if (pass && at < (unsigned)kTopkCap) {
        O.cand_key[at] = key[u][q];
        O.cand_idx[at] = c0 + u * 1024 + q;
      }
    }
  if (tk_last_cta(O.arrive + 1)) tk_final<1>(src, k, O);
}

// Host launcher: k <= 256.  The cand arrays hold topk_cand_entries(k) entries each;
// O.ticket, O.bound, O.arrive[0..1], O.valid_total and O.bits_set must be zero before the call.
int topk_warp_launch(int kind, const void* src, int k, int grid, TopkOut O, cudaStream_t s);
inline int topk_grid_size() { return num_sms(); }
inline size_t topk_cand_entries(int k) {
  const size_t a = (size_t)topk_grid_size() * k;
  return a > (size_t)kTopkCand ? a : (size_t)kTopkCand;
}
inline size_t topk_scratch_bytes(int k) {
  // ticket block + count + k indices + two candidate arrays, each 256-byte aligned
  return 2 * align_up(topk_cand_entries(k) * 8, 256) + align_up((size_t)k * 8, 256) + 1024;
}

}  // namespace tqpk
