// keys.cu - group codes of arbitrary key tuples, and row gathers of string columns.
//
// The reference stacks the group-by key columns side by side, a 2-D string
// column contributing its w bytes as w columns (aggregate.py:291-311), then
// numbers the distinct rows of that stack (:313-333).  Key tuples that do not
// fit the dense mixed-radix slots or the packed 62-bit hash of groupby.cu
// (string keys, float keys, more than TQPK_MAX_KEYS keys) are numbered here:
//
//   1. k_key_insert: each row passing the mask hashes its key tuple and claims
//      or finds its entry of an open-addressing table (capacity a power of two
//      >= 2n).  An entry is one 64-bit word, (24-bit fingerprint << 40) |
//      (representative row + 1), claimed with one compare-and-swap; a
//      fingerprint match is confirmed by comparing the whole key tuple with
//      the representative row's, so distinct tuples never share a group.
//   2. k_key_collect: occupied entries are numbered (group ids in table order).
//   3. The groups are ordered by key tuple with the library's stable radix sort,
//      least significant key first: one pass per numeric key, one per 8 bytes
//      of a string key (big-endian words of the bytes, an int8 column's with
//      the sign bit flipped, so unsigned word order is the byte order of the
//      reference's stacked columns).
//   4. k_key_codes: every row gets the rank of its group; d_reps[rank] is the
//      group's representative row.
//
// A dense group-by over the codes (domain [0, G)) then produces the groups in
// ascending key-tuple order, and the key outputs are gathered from the
// representative rows (tqpk_gather_rows for string keys).
#include "common.cuh"

namespace tqpk {

constexpr int kMaxEncKeys = TQPK_MAX_COLS;
constexpr uint64_t kRowMask = (1ull << 40) - 1;

struct KeyTuple {
  const void* col[kMaxEncKeys];
  int dt[kMaxEncKeys];
  int width[kMaxEncKeys];   // bytes per row of a string key, 0 for a 1-D key
  int n;
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  // splitmix64 finaliser (S. Vigna): a bijective avalanche of 64 bits
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// The bits a key contributes to equality: integers by value, float64 with
// -0.0 folded onto +0.0 (torch.unique sees them equal).
__device__ __forceinline__ uint64_t key_bits(const void* p, int dt, int64_t row) {
  if (dt == TQPK_F64) {
    const uint64_t b = static_cast<const uint64_t*>(p)[row];
    return (b << 1) == 0 ? 0 : b;                     // -0.0 as +0.0, in integer instructions
  }
  return static_cast<uint64_t>(ld_int(p, dt, row));
}

__device__ __forceinline__ uint64_t key_hash(const KeyTuple& K, int64_t row) {
  uint64_t h = 0x9e3779b97f4a7c15ull;
  for (int k = 0; k < K.n; ++k) {
    if (K.width[k]) {
      const uint8_t* s = static_cast<const uint8_t*>(K.col[k]) + row * K.width[k];
      uint64_t w = 0;
      int b = 0;
      for (int i = 0; i < K.width[k]; ++i) {
        w |= static_cast<uint64_t>(s[i]) << (8 * b);
        if (++b == 8) { h = mix64(h ^ w); w = 0; b = 0; }
      }
      if (b) h = mix64(h ^ w ^ (static_cast<uint64_t>(b) << 61));
    } else {
      h = mix64(h ^ key_bits(K.col[k], K.dt[k], row));
    }
  }
  return h;
}

__device__ __forceinline__ bool key_equal(const KeyTuple& K, int64_t a, int64_t b) {
  for (int k = 0; k < K.n; ++k) {
    if (K.width[k]) {
      const uint8_t* x = static_cast<const uint8_t*>(K.col[k]) + a * K.width[k];
      const uint8_t* y = static_cast<const uint8_t*>(K.col[k]) + b * K.width[k];
      for (int i = 0; i < K.width[k]; ++i)
        if (x[i] != y[i]) return false;
    } else if (key_bits(K.col[k], K.dt[k], a) != key_bits(K.col[k], K.dt[k], b)) {
      return false;
    }
  }
  return true;
}

__global__ void __launch_bounds__(kBlock) k_key_insert(const __grid_constant__ KeyTuple K, const uint8_t* mask, int64_t n,
                                                       uint64_t* __restrict__ table, int64_t cap,
                                                       int64_t* __restrict__ entry_of_row, int* err) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    if (mask && !mask[r]) { entry_of_row[r] = -1; continue; }
    const uint64_t h = key_hash(K, r);
    const uint64_t mine = ((h >> 40) << 40) | static_cast<uint64_t>(r + 1);
    int64_t p = static_cast<int64_t>(h & static_cast<uint64_t>(cap - 1));
    int64_t found = -1;
    for (int64_t probe = 0; probe < cap; ++probe) {
      uint64_t e = table[p];
      if (e == 0) {
        e = atomicCAS(reinterpret_cast<unsigned long long*>(&table[p]), 0ull, (unsigned long long)mine);
        if (e == 0) { found = p; break; }
      }
      if ((e >> 40) == (h >> 40) && key_equal(K, r, static_cast<int64_t>((e & kRowMask) - 1))) { found = p; break; }
      p = (p + 1) & (cap - 1);
    }
    if (found < 0) set_error(err, TQPK_ENOMEM);   // cannot happen at capacity >= 2n; kept as a bound
    entry_of_row[r] = found;
  }
}

__global__ void __launch_bounds__(kBlock) k_key_collect(const uint64_t* __restrict__ table, int64_t cap,
                                                        int64_t* __restrict__ gid_of_entry,
                                                        int64_t* __restrict__ rep_of_gid,
                                                        unsigned long long* counter) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < cap; p += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t e = table[p];
    if (e == 0) continue;
    const int64_t g = static_cast<int64_t>(atomicAdd(counter, 1ull));
    gid_of_entry[p] = g;
    rep_of_gid[g] = static_cast<int64_t>((e & kRowMask) - 1);
  }
}

// Sort key of pass (k, word) for group g: a numeric key's value (sorted in its
// own dtype) or one big-endian 8-byte word of a string key (as int64 whose
// sign-flipped bits give the unsigned order).
__global__ void k_key_sortword(const __grid_constant__ KeyTuple K, int k, int word, const int64_t* __restrict__ rep,
                               int64_t G, int64_t* __restrict__ out) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = rep[g];
    if (K.width[k]) {
      const uint8_t* s = static_cast<const uint8_t*>(K.col[k]) + row * K.width[k];
      const uint8_t flip = K.dt[k] == TQPK_I8 ? 0x80u : 0u;   // int8 bytes order as signed values
      uint64_t w = 0;
      for (int i = 0; i < 8; ++i) {
        const int c = word * 8 + i;
        const uint64_t b = c < K.width[k] ? static_cast<uint64_t>(s[c] ^ flip) : 0ull;
        w = (w << 8) | b;
      }
      out[g] = static_cast<int64_t>(w ^ (1ull << 63));
    } else if (K.dt[k] == TQPK_F64) {
      out[g] = __double_as_longlong(static_cast<const double*>(K.col[k])[row]);
    } else {
      out[g] = ld_int(K.col[k], K.dt[k], row);
    }
  }
}

__global__ void k_key_rank(const int64_t* __restrict__ perm, int64_t G, const int64_t* __restrict__ rep_of_gid,
                           int64_t* __restrict__ rank_of_gid, int64_t* __restrict__ reps_out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < G; i += (int64_t)gridDim.x * blockDim.x) {
    rank_of_gid[perm[i]] = i;
    reps_out[i] = rep_of_gid[perm[i]];
  }
}

__global__ void k_key_codes(const int64_t* __restrict__ entry_of_row, int64_t n, const int64_t* __restrict__ gid_of_entry,
                            const int64_t* __restrict__ rank_of_gid, int32_t* __restrict__ codes) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = entry_of_row[r];
    codes[r] = e < 0 ? 0 : static_cast<int32_t>(rank_of_gid[gid_of_entry[e]]);
  }
}

// Word `word` of each row of an int8/uint8 [n, w] column as a sort key: bytes
// word*8 .. word*8+7 big-endian (an int8 column's with the sign bit of each
// byte flipped; zero past w), stored as int64 with its top bit flipped, so the
// library's int64 sort orders rows as the byte columns compare, most
// significant first.
__global__ void k_string_words(const uint8_t* __restrict__ src, int64_t n, int w, int word, uint8_t flip,
                               int64_t* __restrict__ out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t* s = src + r * w;
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) {
      const int c = word * 8 + i;
      v = (v << 8) | (c < w ? static_cast<uint64_t>(s[c] ^ flip) : 0ull);
    }
    out[r] = static_cast<int64_t>(v ^ (1ull << 63));
  }
}

__global__ void k_gather_rows(const uint8_t* __restrict__ src, int64_t row_bytes, const int64_t* __restrict__ idx,
                              int64_t n_idx, int64_t n_src, uint8_t* __restrict__ dst, int* err) {
  const int64_t total = n_idx * row_bytes;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i / row_bytes, b = i - j * row_bytes;
    const int64_t r = idx[j];
    if (r < 0 || r >= n_src) {
      set_error(err, TQPK_EINVAL);
      dst[i] = 0;
      continue;
    }
    dst[i] = src[r * row_bytes + b];
  }
}

static int64_t key_capacity(int64_t n) {
  int64_t c = 1024;
  while (c < 2 * n) c <<= 1;
  return c;
}

}  // namespace tqpk

using namespace tqpk;

extern "C" size_t tqpk_key_encode_workspace_bytes(int64_t n) {
  if (n < 0) n = 0;
  const int64_t cap = key_capacity(n);
  return align_up(cap * 8, 256) * 2 + align_up(n * 8, 256) * 6 + sort_ws_bytes(n) + 4096;
}

extern "C" int tqpk_key_encode(int32_t n_keys, const void* const* h_keys, const int32_t* h_dtypes,
                               const int32_t* h_widths, const uint8_t* d_mask, int64_t n, int32_t* d_codes,
                               int64_t* d_reps, int64_t* h_groups, void* d_ws, size_t ws_bytes,
                               tqpk_stream stream) {
  if (n_keys < 1 || n_keys > kMaxEncKeys || n < 0 || !h_keys || !h_dtypes || !h_widths || !h_groups) return TQPK_EINVAL;
  if (n >= (int64_t)kRowMask || n > (int64_t)INT32_MAX) return TQPK_EUNSUPPORTED;
  KeyTuple K{};
  K.n = n_keys;
  for (int k = 0; k < n_keys; ++k) {
    if (h_widths[k] < 0) return TQPK_EINVAL;
    if (h_widths[k] > 0 && dtype_size(h_dtypes[k]) != 1) return TQPK_EDTYPE;
    if (!dtype_size(h_dtypes[k])) return TQPK_EDTYPE;
    if (n > 0 && !h_keys[k]) return TQPK_EINVAL;
    K.col[k] = h_keys[k];
    K.dt[k] = h_dtypes[k];
    K.width[k] = h_widths[k];
  }
  *h_groups = 0;
  if (n == 0) return TQPK_OK;
  if (!d_codes || !d_reps || !d_ws) return TQPK_EINVAL;
  if (ws_bytes < tqpk_key_encode_workspace_bytes(n)) return TQPK_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t cap = key_capacity(n);
  WsCursor ws(d_ws, ws_bytes);
  uint64_t* table = ws.take<uint64_t>(cap);
  int64_t* gid_of_entry = ws.take<int64_t>(cap);
  int64_t* entry_of_row = ws.take<int64_t>(n);
  int64_t* rep_of_gid = ws.take<int64_t>(n);
  int64_t* rank_of_gid = ws.take<int64_t>(n);
  int64_t* perm_a = ws.take<int64_t>(n);
  int64_t* perm_b = ws.take<int64_t>(n);
  int64_t* words = ws.take<int64_t>(n);
  int* ctl = ws.take<int>(4);
  void* sort_ws = ws.take<char>(sort_ws_bytes(n));
  if (!sort_ws || !ctl) return TQPK_ENOMEM;
  unsigned long long* counter = reinterpret_cast<unsigned long long*>(ctl);   // ctl[0..1]
  int* err = ctl + 2;
  TQPK_CUDA(cudaMemsetAsync(table, 0, cap * 8, s));
  TQPK_CUDA(cudaMemsetAsync(ctl, 0, 16, s));
  k_key_insert<<<grid_for(n, 8), kBlock, 0, s>>>(K, d_mask, n, table, cap, entry_of_row, err);
  TQPK_CHECK_LAUNCH();
  k_key_collect<<<grid_for(cap, 8), kBlock, 0, s>>>(table, cap, gid_of_entry, rep_of_gid, counter);
  TQPK_CHECK_LAUNCH();
  int64_t host[2] = {0, 0};
  TQPK_CUDA(cudaMemcpyAsync(host, ctl, 16, cudaMemcpyDeviceToHost, s));
  TQPK_CUDA(cudaStreamSynchronize(s));
  const int64_t G = host[0];
  const int e = static_cast<int>(host[1] & 0xffffffff);
  if (e) return e;
  *h_groups = G;
  if (G == 0) return TQPK_OK;
  // least significant pass first: keys from last to first, words of a string from last to first
  int64_t* cur = nullptr;
  for (int k = n_keys - 1; k >= 0; --k) {
    const int nw = K.width[k] ? (K.width[k] + 7) / 8 : 1;
    const int dt = (K.width[k] == 0 && K.dt[k] == TQPK_F64) ? TQPK_F64 : TQPK_I64;
    for (int w = nw - 1; w >= 0; --w) {
      k_key_sortword<<<grid_for(G, 4), kBlock, 0, s>>>(K, k, w, rep_of_gid, G, words);
      TQPK_CHECK_LAUNCH();
      int64_t* out = (cur == perm_a) ? perm_b : perm_a;
      const int rc = tqpk_argsort_stable(words, dt, 0, cur, G, out, sort_ws, sort_ws_bytes(n), stream);
      if (rc) return rc;
      cur = out;
    }
  }
  k_key_rank<<<grid_for(G, 4), kBlock, 0, s>>>(cur, G, rep_of_gid, rank_of_gid, d_reps);
  TQPK_CHECK_LAUNCH();
  k_key_codes<<<grid_for(n, 8), kBlock, 0, s>>>(entry_of_row, n, gid_of_entry, rank_of_gid, d_codes);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

extern "C" int tqpk_gather_rows(const void* d_src, int64_t n_src, int64_t row_bytes, const int64_t* d_idx, int64_t n_idx,
                                void* d_dst, tqpk_stream stream) {
  if (n_src < 0 || n_idx < 0 || row_bytes <= 0) return TQPK_EINVAL;
  if (n_idx == 0) return TQPK_OK;
  if (!d_src || !d_idx || !d_dst) return TQPK_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_gather_rows<<<grid_for(n_idx * row_bytes, 8), kBlock, 0, s>>>(static_cast<const uint8_t*>(d_src), row_bytes, d_idx,
                                                                  n_idx, n_src, static_cast<uint8_t*>(d_dst), nullptr);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}

extern "C" int tqpk_string_words(const void* d_src, int64_t n, int32_t width, int32_t word, int32_t signed_bytes,
                                 int64_t* d_out, tqpk_stream stream) {
  if (n < 0 || width <= 0 || word < 0 || word * 8 >= width) return TQPK_EINVAL;
  if (n == 0) return TQPK_OK;
  if (!d_src || !d_out) return TQPK_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_string_words<<<grid_for(n, 8), kBlock, 0, s>>>(static_cast<const uint8_t*>(d_src), n, width, word,
                                                   signed_bytes ? 0x80u : 0u, d_out);
  TQPK_CHECK_LAUNCH();
  return TQPK_OK;
}
