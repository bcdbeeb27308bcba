// sphg_noalloc.cu -- sphg_sort_pairs_noalloc: the radix sort of sphg_sort.cu
// with its scratch in a fixed device array instead of cudaMallocAsync.
//
// For callers that cannot allocate device memory at the time they sort: code
// that runs while a CUDA graph is being captured with a memory policy that
// forbids allocation nodes, allocators that own all device memory themselves
// (memory pools handed a fixed budget, real-time loops that must never block
// in the driver's allocator), or plug-ins whose host forbids cudaMalloc.
// The caller still passes the input and output buffers.
//
// The scratch lives in one file-scope __device__ array; every GPU that loads
// the library holds it until the process exits.  Its size bounds n to
// kNoAllocMaxPairs.  Host code cannot use the array's name as a device
// address (it names a host-side shadow), so the address is fetched with
// cudaGetSymbolAddress once per device context and cached together with the
// context's id: after a cudaDeviceReset the device gets a new context, the
// module (and the array) is loaded again, possibly at another address, and the
// next call looks the address up again.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/sphg.h"
#include "sphg_sort.cuh"
#include "sphg_step.cuh"

namespace {

constexpr int64_t kNoAllocMaxPairs = SPHG_SORT_NOALLOC_MAX_PAIRS;
constexpr size_t kHistWords = sphg::sort_scratch_words_c(kNoAllocMaxPairs);
constexpr size_t kScratchWords = kHistWords + 2 * (size_t)kNoAllocMaxPairs;
static_assert(kScratchWords * 4 == SPHG_SORT_NOALLOC_SCRATCH_BYTES, "documented scratch size");

// [histograms, tile counters, error word, look-back words | ping-pong keys | ping-pong values]
static __device__ __align__(256) uint32_t g_noalloc_sort_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct ScratchAddr {
  uint32_t* ptr = nullptr;
  unsigned long long ctx_id = 0;  // id of the context ptr belongs to (0: unknown)
};
ScratchAddr g_scratch[kMaxDevices];

// Driver entry points that identify the current context, fetched through the
// runtime (the library does not link the driver library itself).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
bool g_ctx_fns_tried = false;

// Id of the calling thread's current context, 0 when it cannot be told.
unsigned long long current_context_id() {
  if (!g_ctx_fns_tried) {
    g_ctx_fns_tried = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_id = reinterpret_cast<CtxGetIdFn>(f);
  }
  if (!g_ctx_current || !g_ctx_id) return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (g_ctx_current(&c) != CUDA_SUCCESS || !c) return 0;
  if (g_ctx_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

sphg_status noalloc_fail(sphg_status st, const std::string& msg) {
  sphg::set_last_error(msg);
  return st;
}

// Device address of the scratch array in the current device's context: looked
// up at the first call on a device, and again when the device's context has
// changed since (cudaDeviceReset).
sphg_status scratch_for_current_device(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(SPHG_CUDA_ERROR, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(SPHG_CAPACITY, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_mu);
  ScratchAddr& c = g_scratch[dev];
  const unsigned long long ctx = current_context_id();
  if (!c.ptr || ctx == 0 || ctx != c.ctx_id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_sort_scratch);
    if (e != cudaSuccess || !p)
      return noalloc_fail(SPHG_CUDA_ERROR, std::string("cudaGetSymbolAddress of the sort scratch: ") +
                                              cudaGetErrorString(e));
    c.ptr = static_cast<uint32_t*>(p);
    c.ctx_id = current_context_id();  // the lookup made the context current if it was not
  }
  *out = c.ptr;
  return SPHG_OK;
}

}  // namespace

extern "C" {

sphg_status sphg_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in,
                                    uint32_t* keys_out, uint32_t* vals_out, int64_t n,
                                    int32_t bits, void* stream) {
  if (n < 0 || bits < 1 || bits > 32) return noalloc_fail(SPHG_INVALID_ARG, "n < 0 or bits outside 1..32");
  if (n > kNoAllocMaxPairs)
    return noalloc_fail(SPHG_CAPACITY, "sphg_sort_pairs_noalloc sorts at most " +
                                           std::to_string(kNoAllocMaxPairs) + " pairs, got " +
                                           std::to_string(n));
  if (n == 0) return SPHG_OK;
  if (!keys_in || !keys_out || !vals_out) return noalloc_fail(SPHG_INVALID_ARG, "null buffer");
  uint32_t* scratch = nullptr;
  sphg_status st = scratch_for_current_device(&scratch);
  if (st != SPHG_OK) return st;
  // The sort clears its histograms, tile counters, error word and look-back
  // words itself (stream-ordered memsets, no allocation) before each use.
  uint32_t* keys_tmp = scratch + kHistWords;
  uint32_t* vals_tmp = keys_tmp + kNoAllocMaxPairs;
  cudaError_t e = sphg::radix_sort_pairs(keys_in, vals_in, keys_out, vals_out, keys_tmp, vals_tmp,
                                         scratch, n, bits, (cudaStream_t)stream, nullptr, nullptr, nullptr,
                                         true);
  if (e != cudaSuccess) return noalloc_fail(SPHG_CUDA_ERROR, std::string("radix sort launch: ") + cudaGetErrorString(e));
  return SPHG_OK;
}

}  // extern "C"
