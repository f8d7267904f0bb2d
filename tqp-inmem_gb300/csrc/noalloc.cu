// noalloc.cu - stream compaction that allocates nothing.
//
// tqpk_compact needs a small scratch area (a tile counter, an error word and
// one look-back status word per 4096-row tile) that its caller allocates.
// Some callers cannot allocate device memory at the moment they want to run
// the operator: code running inside a host runtime that owns all device
// memory through its own arena and gives out none for library scratch,
// request paths that forbid allocation after start-up because cudaMalloc /
// cudaFree can synchronise the device and stall unrelated work, or foreign
// language bindings that only hold the input and output buffers they were
// handed.  tqpk_compact_noalloc serves them: its scratch is the file-scope
// device array below, so a call only needs the inputs and outputs.
//
// Limits and sharing:
//  * the array is 1 MiB: a 256-byte control block and the look-back status
//    words of at most tqpk_compact_noalloc_max_rows() rows (536,739,840);
//    larger inputs are rejected with TQPK_ENOMEM before anything is launched;
//  * a look-back wait that runs out leaves the negative status TQPK_ETIMEOUT
//    in *d_count instead of a row count, as tqpk_compact does;
//  * every GPU that loads this library keeps the array resident until the
//    process exits;
//  * all calls on a device share the one array and it keeps whatever the
//    previous call left, so each call first clears the part it uses on its
//    own stream; two calls whose work overlaps on the GPU (different streams
//    or threads without ordering between them) race on the array and must be
//    serialised by the caller;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture starts on the device.
#include <mutex>

#include "common.cuh"

namespace tqpk {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;  // 1 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};
}  // namespace

// Device address of the scratch array for the current device (looked up once per device).
static int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    (void)cudaGetLastError();
    return TQPK_ECUDA;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      (void)cudaGetLastError();
      return TQPK_ECUDA;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return TQPK_OK;
}

}  // namespace tqpk

using namespace tqpk;

extern "C" int64_t tqpk_compact_noalloc_max_rows(void) {
  // The compaction's workspace (compact_status_bytes) is a 256-byte control block followed by one
  // 8-byte look-back status word per 4096-row tile, rounded up to 256 bytes: the array holds
  // (1 MiB - 256) / 8 = 131,040 tiles.
  const int64_t rows = (int64_t)((kNoAllocScratchBytes - 256) / 8) * kTile;
  return compact_status_bytes(rows) <= kNoAllocScratchBytes ? rows : 0;
}

extern "C" int tqpk_compact_noalloc(const tqpk_predicate* h_pred, const uint8_t* d_mask, int64_t n, int32_t ncols,
                                    const void* const* h_cols_in, const int32_t* h_dtypes, void* const* h_cols_out,
                                    int64_t* d_count, tqpk_stream stream) {
  if (n < 0 || ncols < 0 || ncols > TQPK_MAX_COLS || !d_count) return TQPK_EINVAL;
  if (n > tqpk_compact_noalloc_max_rows()) return TQPK_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n == 0) {
    TQPK_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int64_t), s));
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
    if ((sz && !h_cols_in[c]) || !h_cols_out[c]) return TQPK_EINVAL;
    C.in[c] = h_cols_in[c];
    C.out[c] = h_cols_out[c];
    C.size[c] = sz;
  }
  void* scratch = nullptr;
  if ((rc = noalloc_scratch(&scratch))) return rc;
  // compact_launch clears the control words and the status words it uses on `s`
  return compact_launch(d_mask ? nullptr : h_pred, d_mask, n, C, d_count, scratch, kNoAllocScratchBytes, s);
}
