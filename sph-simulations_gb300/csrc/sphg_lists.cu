// sphg_lists.cu -- CSR neighbour lists of the current (sorted) state, in the
// reference's order: self included, stencil x offset outer, y offset inner,
// j ascending (MultipassNeighborLists: count CountNeighborsPerParticle
// core/algorithmic/MultipassNeighborLists.h:63-121, offsets CalculateOffsets
// :47-61, fill AssignIndices :123-181).  The reference GPU version
// (core/acceleration/cuNeighborLists.cu) drops the particle itself and leaves
// its index buffer uninitialised; this one follows the CPU semantics.
//
// Three passes: count (stencil walk), a device-wide exclusive scan to int64
// offsets, fill (same walk).
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sphg.h"
#include "sphg_neighbor.cuh"
#include "sphg_step.cuh"

namespace sphg {

constexpr int kListThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

template <int PREC, bool BATCHED>
__global__ void __launch_bounds__(kListThreads) lists_count(StepArgs a, int32_t* counts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const InstDesc d = inst_of<BATCHED>(a, i);
  int cx, cy, c = 0;
  for_each_neighbor<PREC, true>(a, d, a.keyA[i], a.posA[i], cx, cy,
                                [&](uint32_t, float, float, float, uint32_t) { ++c; });
  counts[i] = c;
}

template <int PREC, bool BATCHED>
__global__ void __launch_bounds__(kListThreads) lists_fill(StepArgs a, const int64_t* offs,
                                                           int32_t* idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const InstDesc d = inst_of<BATCHED>(a, i);
  int64_t o = offs[i];
  int cx, cy;
  for_each_neighbor<PREC, true>(a, d, a.keyA[i], a.posA[i], cx, cy,
                                [&](uint32_t j, float, float, float, uint32_t) { idx[o++] = (int32_t)j; });
}

// Exclusive scan of int32 counts into int64 offsets (offs[n] = total).
__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t* warp_tot, int64_t& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int64_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  total = warp_tot[(blockDim.x >> 5) - 1];
  int64_t r = (w ? warp_tot[w - 1] : 0) + x - v;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles(const int32_t* counts, int64_t n,
                                                           int64_t* offs, int64_t* tile_sums) {
  __shared__ int64_t wt[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? counts[base + k] : 0;
    s += v[k];
  }
  int64_t total;
  int64_t pre = block_excl_scan(s, wt, total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) offs[base + k] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_tile_sums(int64_t* tile_sums, int ntiles,
                                                               int64_t* total_out) {
  __shared__ int64_t wt[32];
  int64_t carry = 0;
  for (int b = 0; b < ntiles; b += kScanThreads) {
    int t = b + threadIdx.x;
    int64_t v = t < ntiles ? tile_sums[t] : 0;
    int64_t tot;
    int64_t e = block_excl_scan(v, wt, tot);
    if (t < ntiles) tile_sums[t] = carry + e;
    carry += tot;
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void scan_add(int64_t* offs, int64_t n, const int64_t* tile_sums,
                         const int64_t* total) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) offs[i] += tile_sums[i / kScanTile];
  if (i == n) offs[n] = *total;
}

}  // namespace sphg

namespace sphg {

int lists_impl(const StepArgs& a, int precision, int64_t* offs, int32_t* idx, int64_t* total,
               cudaStream_t st, std::string* err) {
  const int64_t n = a.n;
  if (total) *total = 0;
  if (n == 0) {
    if (offs) offs[0] = 0;
    return SPHG_OK;
  }
  const int ntiles = (int)((n + kScanTile - 1) / kScanTile);
  int32_t* dcounts = nullptr;
  int64_t* doffs = nullptr;
  int64_t* dsums = nullptr;
  int32_t* didx = nullptr;
  auto cleanup = [&]() {
    if (dcounts) cudaFreeAsync(dcounts, st);
    if (doffs) cudaFreeAsync(doffs, st);
    if (dsums) cudaFreeAsync(dsums, st);
    if (didx) cudaFreeAsync(didx, st);
  };
  auto ck = [&](cudaError_t e, const char* what) -> bool {
    if (e == cudaSuccess) return true;
    *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
  };
  const unsigned g = (unsigned)((n + kListThreads - 1) / kListThreads);
  bool ok = ck(cudaMallocAsync((void**)&dcounts, n * sizeof(int32_t), st), "cudaMallocAsync") &&
            ck(cudaMallocAsync((void**)&doffs, (n + 1) * sizeof(int64_t), st), "cudaMallocAsync") &&
            ck(cudaMallocAsync((void**)&dsums, (ntiles + 1) * sizeof(int64_t), st), "cudaMallocAsync");
  if (!ok) { cleanup(); return SPHG_OOM; }
  const bool batched = (a.ninst > 1 || a.force_batched);
  if (precision) {
    if (batched) lists_count<1, true><<<g, kListThreads, 0, st>>>(a, dcounts);
    else lists_count<1, false><<<g, kListThreads, 0, st>>>(a, dcounts);
  } else {
    if (batched) lists_count<0, true><<<g, kListThreads, 0, st>>>(a, dcounts);
    else lists_count<0, false><<<g, kListThreads, 0, st>>>(a, dcounts);
  }
  scan_tiles<<<ntiles, kScanThreads, 0, st>>>(dcounts, n, doffs, dsums);
  scan_tile_sums<<<1, kScanThreads, 0, st>>>(dsums, ntiles, dsums + ntiles);
  scan_add<<<(unsigned)((n + 1 + 255) / 256), 256, 0, st>>>(doffs, n, dsums, dsums + ntiles);
  int64_t tot = 0;
  ok = ck(cudaGetLastError(), "list count/scan launch") &&
       ck(cudaMemcpyAsync(&tot, dsums + ntiles, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "copy") &&
       ck(cudaStreamSynchronize(st), "sync");
  if (!ok) { cleanup(); return SPHG_CUDA_ERROR; }
  if (total) *total = tot;
  if (offs) {
    ok = ck(cudaMemcpyAsync(offs, doffs, (n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st), "copy");
    if (!ok) { cleanup(); return SPHG_CUDA_ERROR; }
  }
  if (idx && tot > 0) {
    ok = ck(cudaMallocAsync((void**)&didx, tot * sizeof(int32_t), st), "cudaMallocAsync");
    if (!ok) { cleanup(); return SPHG_OOM; }
    if (precision) {
      if (batched) lists_fill<1, true><<<g, kListThreads, 0, st>>>(a, doffs, didx);
      else lists_fill<1, false><<<g, kListThreads, 0, st>>>(a, doffs, didx);
    } else {
      if (batched) lists_fill<0, true><<<g, kListThreads, 0, st>>>(a, doffs, didx);
      else lists_fill<0, false><<<g, kListThreads, 0, st>>>(a, doffs, didx);
    }
    ok = ck(cudaGetLastError(), "list fill launch") &&
         ck(cudaMemcpyAsync(idx, didx, tot * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "copy");
    if (!ok) { cleanup(); return SPHG_CUDA_ERROR; }
  }
  cleanup();
  if (!ck(cudaStreamSynchronize(st), "sync")) return SPHG_CUDA_ERROR;
  return SPHG_OK;
}

}  // namespace sphg
