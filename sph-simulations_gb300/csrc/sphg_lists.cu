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

// Lists mode: the same walk, entries packed as j << 5 | tag (stencil offset and
// periodic-wrap bit, read back by the density and force passes); at most cap
// entries are written (the buffer was sized at the pre-loop), and a list that
// runs past it sets *overflow, which the synchronising calls report.
template <int PREC, bool BATCHED>
__global__ void __launch_bounds__(kListThreads) lists_fill_packed(StepArgs a, const int64_t* offs,
                                                                  uint32_t* idx, int64_t cap,
                                                                  uint32_t* overflow) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const InstDesc d = inst_of<BATCHED>(a, i);
  int64_t o = offs[i];
  int cx, cy;
  for_each_neighbor<PREC, true>(a, d, a.keyA[i], a.posA[i], cx, cy,
                                [&](uint32_t j, float, float, float, uint32_t tag) {
                                  if (o < cap) idx[o] = (j << 5) | tag;
                                  ++o;
                                });
  if (o > cap && overflow) *overflow = 1u;
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

// Delta codec of CSR lists (Codifier::Encode, core/encoders/Encoder.h:27-44):
// the first index of a list verbatim, then idx[k] - idx[k-1] - 1, which needs
// each list ascending.  One thread per list.
__global__ void lists_sort_ascending(const int64_t* offs, int32_t* idx, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = offs[i], e = offs[i + 1];
  for (int64_t q = b + 1; q < e; ++q) {  // insertion sort: lists hold a few dozen entries
    const int32_t v = idx[q];
    int64_t r = q - 1;
    while (r >= b && idx[r] > v) {
      idx[r + 1] = idx[r];
      --r;
    }
    idx[r + 1] = v;
  }
}

__global__ void delta_encode_kernel(const int64_t* offs, const int32_t* idx, int64_t n, int32_t* enc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = offs[i], e = offs[i + 1];
  if (b >= e) return;
  int32_t prev = idx[b];
  enc[b] = prev;
  for (int64_t q = b + 1; q < e; ++q) {
    const int32_t v = idx[q];
    enc[q] = v - prev - 1;
    prev = v;
  }
}

__global__ void delta_decode_kernel(const int64_t* offs, const int32_t* enc, int64_t n, int32_t* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = offs[i], e = offs[i + 1];
  if (b >= e) return;
  int32_t v = enc[b];
  out[b] = v;
  for (int64_t q = b + 1; q < e; ++q) {
    v = v + enc[q] + 1;
    out[q] = v;
  }
}

cudaError_t launch_delta(bool encode, const int64_t* offs, const int32_t* in, int64_t n, int32_t* out,
                         cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const unsigned g = (unsigned)((n + 255) / 256);
  if (encode) delta_encode_kernel<<<g, 256, 0, st>>>(offs, in, n, out);
  else delta_decode_kernel<<<g, 256, 0, st>>>(offs, in, n, out);
  return cudaGetLastError();
}

int lists_scan_tiles(int64_t n) { return (int)((n + kScanTile - 1) / kScanTile); }

cudaError_t launch_lists_count_scan(const StepArgs& a, int precision, int32_t* counts, int64_t* offs,
                                    int64_t* sums, cudaStream_t st) {
  const int64_t n = a.n;
  if (n == 0) return cudaSuccess;
  const int ntiles = lists_scan_tiles(n);
  const unsigned g = (unsigned)((n + kListThreads - 1) / kListThreads);
  const bool batched = (a.ninst > 1 || a.force_batched);
  if (precision) {
    if (batched) lists_count<1, true><<<g, kListThreads, 0, st>>>(a, counts);
    else lists_count<1, false><<<g, kListThreads, 0, st>>>(a, counts);
  } else {
    if (batched) lists_count<0, true><<<g, kListThreads, 0, st>>>(a, counts);
    else lists_count<0, false><<<g, kListThreads, 0, st>>>(a, counts);
  }
  scan_tiles<<<ntiles, kScanThreads, 0, st>>>(counts, n, offs, sums);
  scan_tile_sums<<<1, kScanThreads, 0, st>>>(sums, ntiles, sums + ntiles);
  scan_add<<<(unsigned)((n + 1 + 255) / 256), 256, 0, st>>>(offs, n, sums, sums + ntiles);
  return cudaGetLastError();
}

cudaError_t launch_lists_fill_packed(const StepArgs& a, int precision, const int64_t* offs,
                                     uint32_t* idx, int64_t cap, uint32_t* overflow, cudaStream_t st) {
  const int64_t n = a.n;
  if (n == 0) return cudaSuccess;
  const unsigned g = (unsigned)((n + kListThreads - 1) / kListThreads);
  const bool batched = (a.ninst > 1 || a.force_batched);
  if (precision) {
    if (batched) lists_fill_packed<1, true><<<g, kListThreads, 0, st>>>(a, offs, idx, cap, overflow);
    else lists_fill_packed<1, false><<<g, kListThreads, 0, st>>>(a, offs, idx, cap, overflow);
  } else {
    if (batched) lists_fill_packed<0, true><<<g, kListThreads, 0, st>>>(a, offs, idx, cap, overflow);
    else lists_fill_packed<0, false><<<g, kListThreads, 0, st>>>(a, offs, idx, cap, overflow);
  }
  return cudaGetLastError();
}

}  // namespace sphg

namespace sphg {

int lists_impl(const StepArgs& a, int precision, int64_t* offs, int32_t* idx, int64_t* total,
               cudaStream_t st, std::string* err, bool encoded) {
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
    if (encoded) {  // ascending lists, delta-coded in place of the counts buffer
      int32_t* denc = nullptr;
      ok = ck(cudaMallocAsync((void**)&denc, tot * sizeof(int32_t), st), "cudaMallocAsync");
      if (!ok) { cleanup(); return SPHG_OOM; }
      lists_sort_ascending<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(doffs, didx, n);
      ok = ck(launch_delta(true, doffs, didx, n, denc, st), "delta encode launch") &&
           ck(cudaMemcpyAsync(idx, denc, tot * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "copy");
      cudaFreeAsync(denc, st);
      if (!ok) { cleanup(); return SPHG_CUDA_ERROR; }
    } else {
      ok = ck(cudaGetLastError(), "list fill launch") &&
           ck(cudaMemcpyAsync(idx, didx, tot * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "copy");
    }
    if (!ok) { cleanup(); return SPHG_CUDA_ERROR; }
  }
  cleanup();
  if (!ck(cudaStreamSynchronize(st), "sync")) return SPHG_CUDA_ERROR;
  return SPHG_OK;
}

}  // namespace sphg
