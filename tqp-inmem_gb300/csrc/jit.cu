// jit.cu - runtime compilation of query-specialised kernels (NVRTC).
//
// The operators' predicate, expression and accumulator programs are data
// (include/tqpk.h).  The interpreting kernels pay for that on every row:
// opcode dispatch, operand selection and small local arrays.  For the hot
// kernels the host instead generates CUDA C++ in which the query's program
// is straight-line code with its literals inlined, compiles it here with
// NVRTC for sm_103a, loads the cubin with the runtime's library API and
// launches it on the caller's stream.  NVRTC is opened with dlopen, so the
// library has no link-time dependency on it; without it the interpreting
// kernels run instead (the same results, more instructions per row).
#include <atomic>
#include <dlfcn.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace tqpk {
namespace {

typedef int nvrtcResult_t;
typedef struct _nvrtcProgram* nvrtcProgram_t;

struct Nvrtc {
  void* so = nullptr;
  nvrtcResult_t (*create)(nvrtcProgram_t*, const char*, const char*, int, const char* const*, const char* const*);
  nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char* const*);
  nvrtcResult_t (*log_size)(nvrtcProgram_t, size_t*);
  nvrtcResult_t (*log)(nvrtcProgram_t, char*);
  nvrtcResult_t (*cubin_size)(nvrtcProgram_t, size_t*);
  nvrtcResult_t (*cubin)(nvrtcProgram_t, char*);
  nvrtcResult_t (*destroy)(nvrtcProgram_t*);
  bool tried = false;
};

Nvrtc g_nvrtc;
std::mutex g_jit_mu;

bool nvrtc_open() {
  if (g_nvrtc.tried) return g_nvrtc.so != nullptr;
  g_nvrtc.tried = true;
  const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                         "/usr/local/cuda/lib64/libnvrtc.so", "/usr/local/cuda/targets/sbsa-linux/lib/libnvrtc.so.13",
                         "/usr/local/cuda/targets/x86_64-linux/lib/libnvrtc.so.13"};
  for (const char* n : names) {
    g_nvrtc.so = dlopen(n, RTLD_NOW | RTLD_LOCAL);
    if (g_nvrtc.so) break;
  }
  if (!g_nvrtc.so) return false;
  auto sym = [](const char* s) { return dlsym(g_nvrtc.so, s); };
  g_nvrtc.create = reinterpret_cast<decltype(g_nvrtc.create)>(sym("nvrtcCreateProgram"));
  g_nvrtc.compile = reinterpret_cast<decltype(g_nvrtc.compile)>(sym("nvrtcCompileProgram"));
  g_nvrtc.log_size = reinterpret_cast<decltype(g_nvrtc.log_size)>(sym("nvrtcGetProgramLogSize"));
  g_nvrtc.log = reinterpret_cast<decltype(g_nvrtc.log)>(sym("nvrtcGetProgramLog"));
  g_nvrtc.cubin_size = reinterpret_cast<decltype(g_nvrtc.cubin_size)>(sym("nvrtcGetCUBINSize"));
  g_nvrtc.cubin = reinterpret_cast<decltype(g_nvrtc.cubin)>(sym("nvrtcGetCUBIN"));
  g_nvrtc.destroy = reinterpret_cast<decltype(g_nvrtc.destroy)>(sym("nvrtcDestroyProgram"));
  if (!g_nvrtc.create || !g_nvrtc.compile || !g_nvrtc.log_size || !g_nvrtc.log || !g_nvrtc.cubin_size ||
      !g_nvrtc.cubin || !g_nvrtc.destroy) {
    dlclose(g_nvrtc.so);
    g_nvrtc.so = nullptr;
    return false;
  }
  return true;
}

struct JitKernel {
  cudaLibrary_t lib;
  cudaKernel_t kernel;
  std::atomic<size_t> smem_allowed{0};   // dynamic shared memory the kernel has been opened up to
};

// Raises the kernel's dynamic shared-memory limit once per new maximum: the attribute call
// costs tens of microseconds of host time, too much to repeat on every launch.
static cudaError_t allow_smem(JitKernel* k, size_t smem) {
  if (smem <= k->smem_allowed.load(std::memory_order_relaxed)) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(k->kernel),
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) k->smem_allowed.store(smem, std::memory_order_relaxed);
  return e;
}

}  // namespace
}  // namespace tqpk

using namespace tqpk;

extern "C" int tqpk_jit_available(void) {
  std::lock_guard<std::mutex> lock(g_jit_mu);
  return nvrtc_open() ? 1 : 0;
}

// Compiles `src` for the current device's architecture family (sm_103a) and
// loads kernel `name` (an extern "C" __global__).  *h_handle receives an
// opaque handle; the compile log (if any) goes to log[0..log_len).
extern "C" int tqpk_jit_compile(const char* src, const char* name, void** h_handle, char* log, size_t log_len) {
  if (!src || !name || !h_handle) return TQPK_EINVAL;
  std::lock_guard<std::mutex> lock(g_jit_mu);
  if (!nvrtc_open()) return TQPK_EUNSUPPORTED;
  nvrtcProgram_t prog = nullptr;
  if (g_nvrtc.create(&prog, src, "tqpk_query.cu", 0, nullptr, nullptr) != 0) return TQPK_ECUDA;
  const char* opts[] = {"-arch=sm_103a", "-std=c++17", "--fmad=false", "-default-device", "-lineinfo"};
  const nvrtcResult_t rc = g_nvrtc.compile(prog, 5, opts);
  size_t ls = 0;
  g_nvrtc.log_size(prog, &ls);
  if (log && log_len) {
    std::vector<char> buf(ls + 1, 0);
    if (ls) g_nvrtc.log(prog, buf.data());
    snprintf(log, log_len, "%s", buf.data());
  }
  if (rc != 0) {
    g_nvrtc.destroy(&prog);
    return TQPK_EINVAL;
  }
  size_t n = 0;
  g_nvrtc.cubin_size(prog, &n);
  std::vector<char> cubin(n);
  g_nvrtc.cubin(prog, cubin.data());
  g_nvrtc.destroy(&prog);
  JitKernel* k = new JitKernel();
  if (cudaLibraryLoadData(&k->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess ||
      cudaLibraryGetKernel(&k->kernel, k->lib, name) != cudaSuccess) {
    (void)cudaGetLastError();
    delete k;
    return TQPK_ECUDA;
  }
  *h_handle = k;
  return TQPK_OK;
}

// Compiles only (no device needed): 0 when `src` compiles, with the log in `log`.
extern "C" int tqpk_jit_check(const char* src, char* log, size_t log_len) {
  if (!src) return TQPK_EINVAL;
  std::lock_guard<std::mutex> lock(g_jit_mu);
  if (!nvrtc_open()) return TQPK_EUNSUPPORTED;
  nvrtcProgram_t prog = nullptr;
  if (g_nvrtc.create(&prog, src, "tqpk_query.cu", 0, nullptr, nullptr) != 0) return TQPK_ECUDA;
  const char* opts[] = {"-arch=sm_103a", "-std=c++17", "--fmad=false", "-default-device"};
  const nvrtcResult_t rc = g_nvrtc.compile(prog, 4, opts);
  size_t ls = 0;
  g_nvrtc.log_size(prog, &ls);
  if (log && log_len) {
    std::vector<char> buf(ls + 1, 0);
    if (ls) g_nvrtc.log(prog, buf.data());
    snprintf(log, log_len, "%s", buf.data());
  }
  g_nvrtc.destroy(&prog);
  return rc == 0 ? TQPK_OK : TQPK_EINVAL;
}

// Resident CTAs per SM of a compiled kernel (occupancy API).
extern "C" int tqpk_jit_occupancy(void* handle, int32_t block, size_t smem) {
  if (!handle) return 0;
  JitKernel* k = static_cast<JitKernel*>(handle);
  int per_sm = 0;
  if (smem > 0)   // dynamic + static shared memory may pass the 48 KB default even when smem alone does not
    (void)allow_smem(k, smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(k->kernel), block, smem) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return per_sm;
}

extern "C" int tqpk_jit_prefer_shared(void* handle, int32_t percent) {
  if (!handle || percent < 0 || percent > 100) return TQPK_EINVAL;
  JitKernel* k = static_cast<JitKernel*>(handle);
  TQPK_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void*>(k->kernel),
                                 cudaFuncAttributePreferredSharedMemoryCarveout, (int)percent));
  return TQPK_OK;
}

extern "C" int32_t tqpk_num_sms(void) { return num_sms(); }

// Launches a compiled kernel: args[i] points at the i-th kernel parameter.
// timing_kid tags the launch for tqpk_timing_begin (0 = untimed).
extern "C" int tqpk_jit_launch(void* handle, int32_t grid, int32_t block, size_t smem, void** args,
                               int32_t timing_kid, tqpk_stream stream) {
  if (!handle || grid < 1 || block < 1 || !args) return TQPK_EINVAL;
  JitKernel* k = static_cast<JitKernel*>(handle);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (smem > 0) TQPK_CUDA(allow_smem(k, smem));
  if (timing_kid) timing_before(timing_kid, s);
  const cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(k->kernel), dim3(grid), dim3(block), args,
                                         smem, s);
  if (timing_kid) timing_after(timing_kid, s);
  ++g_launches;
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return TQPK_ECUDA;
  }
  return TQPK_OK;
}
