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
// address (it names a host-side shadow), so the address is fetched once per
// device with cudaGetSymbolAddress and cached.
#include <cstdint>
#include <mutex>
#include <string>

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
uint32_t* g_scratch_ptr[kMaxDevices] = {};

sphg_status noalloc_fail(sphg_status st, const std::string& msg) {
  sphg::set_last_error(msg);
  return st;
}

// Device address of the scratch array on the current device (fetched once per device).
sphg_status scratch_for_current_device(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(SPHG_CUDA_ERROR, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(SPHG_CAPACITY, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_sort_scratch);
    if (e != cudaSuccess || !p)
      return noalloc_fail(SPHG_CUDA_ERROR, std::string("cudaGetSymbolAddress of the sort scratch: ") +
                                              cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_scratch_ptr[dev];
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
  // The sort clears its histograms, tile counters and look-back words itself
  // (stream-ordered memsets, no allocation) before each use.
  uint32_t* keys_tmp = scratch + kHistWords;
  uint32_t* vals_tmp = keys_tmp + kNoAllocMaxPairs;
  cudaError_t e = sphg::radix_sort_pairs(keys_in, vals_in, keys_out, vals_out, keys_tmp, vals_tmp,
                                         scratch, n, bits, (cudaStream_t)stream);
  if (e != cudaSuccess) return noalloc_fail(SPHG_CUDA_ERROR, std::string("radix sort launch: ") + cudaGetErrorString(e));
  return SPHG_OK;
}

}  // extern "C"
