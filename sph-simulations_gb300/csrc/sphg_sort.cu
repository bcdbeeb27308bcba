// sphg_sort.cu -- stable LSD radix sort of (uint32 key, uint32 value) pairs,
// written for this library (no CUB/Thrust).  It replaces the
// thrust::sort_by_key of cuSortContainerByCellID
// (core/acceleration/cuFindNeighbors.cu:82-100), sorting the slot index
// instead of six payload arrays; the payload is gathered once afterwards.
//
// One pass per 8-bit digit, three kernels per pass:
//   sort_hist      per-tile digit histogram (warp-aggregated shared atomics)
//   sort_dscan     per-digit exclusive scan over tiles (one CTA per digit)
//   sort_scatter   stable in-tile ranking (__match_any_sync + popc across the
//                  tile's rounds and warps) and scatter to the global offsets
// Tiles are 2048 keys (256 threads x 8 items, striped so that a round of 256
// consecutive keys is ranked before the next round -> stability).
#include <cstdint>
#include <cuda_runtime.h>

#include "sphg_sort.cuh"

namespace sphg {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;
constexpr int kWarps = kSortThreads / 32;

__global__ void __launch_bounds__(kSortThreads) sort_hist(const uint32_t* __restrict__ keys,
                                                          int64_t n, int shift,
                                                          uint32_t* __restrict__ tile_hist,
                                                          int ntiles, uint32_t* epoch) {
  __shared__ uint32_t h[kRadix];
  if (epoch && blockIdx.x == 0 && threadIdx.x == 0) *epoch += 1u;
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kTile;
  const int lane = threadIdx.x & 31;
  for (int k = 0; k < kSortItems; ++k) {
    int64_t i = base + (int64_t)k * kSortThreads + threadIdx.x;
    bool valid = i < n;
    uint32_t d = valid ? (__ldg(keys + i) >> shift) & (kRadix - 1) : kRadix;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && lane == __ffs(peers) - 1) atomicAdd(&h[d], (uint32_t)__popc(peers));
  }
  __syncthreads();
  tile_hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// One CTA per digit: exclusive scan of tile_hist[d][0..ntiles), total -> digit_total[d].
__global__ void __launch_bounds__(1024) sort_dscan(uint32_t* __restrict__ tile_hist, int ntiles,
                                                   uint32_t* __restrict__ digit_total) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t carry_s;
  uint32_t* row = tile_hist + (int64_t)blockIdx.x * ntiles;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (int base = 0; base < ntiles; base += 1024) {
    int t = base + threadIdx.x;
    uint32_t v = t < ntiles ? row[t] : 0;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t s = warp_sums[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      warp_sums[lane] = s;  // inclusive over warps
    }
    __syncthreads();
    uint32_t carry = carry_s;
    uint32_t excl = carry + (warp ? warp_sums[warp - 1] : 0) + x - v;
    if (t < ntiles) row[t] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = carry + warp_sums[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) digit_total[blockIdx.x] = carry_s;
}

__global__ void __launch_bounds__(kSortThreads) sort_scatter(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int64_t n, int shift,
    const uint32_t* __restrict__ tile_hist, const uint32_t* __restrict__ digit_total,
    int ntiles) {
  __shared__ uint32_t base_s[kRadix];
  __shared__ uint32_t running[kRadix];
  __shared__ uint32_t warp_cnt[kWarps][kRadix];
  __shared__ uint32_t wsum[kWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // global start of digit tid = exclusive scan of digit_total + this tile's offset
  uint32_t tot = digit_total[tid];
  uint32_t x = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  running[tid] = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) warp_cnt[w][tid] = 0;
  __syncthreads();
  uint32_t wpre = 0;
  for (int w = 0; w < warp; ++w) wpre += wsum[w];
  base_s[tid] = wpre + x - tot + tile_hist[(int64_t)tid * ntiles + blockIdx.x];
  __syncthreads();

  const int64_t base = (int64_t)blockIdx.x * kTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int k = 0; k < kSortItems; ++k) {
    int64_t i = base + (int64_t)k * kSortThreads + tid;
    bool valid = i < n;
    uint32_t key = 0, val = 0, d = kRadix;
    if (valid) {
      key = __ldg(keys_in + i);
      val = vals_in ? __ldg(vals_in + i) : (uint32_t)i;
      d = (key >> shift) & (kRadix - 1);
    }
    unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t rank = __popc(peers & lt_mask);
    if (valid && lane == __ffs(peers) - 1) warp_cnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t pre = 0;
      for (int w = 0; w < warp; ++w) pre += warp_cnt[w][d];
      uint32_t pos = base_s[d] + running[d] + pre + rank;
      keys_out[pos] = key;
      vals_out[pos] = val;
    }
    __syncthreads();
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      s += warp_cnt[w][tid];
      warp_cnt[w][tid] = 0;
    }
    running[tid] += s;
    __syncthreads();
  }
}

int sort_num_tiles(int64_t n) { return (int)((n + kTile - 1) / kTile); }

size_t sort_scratch_words(int64_t n) {
  return (size_t)kRadix * (size_t)sort_num_tiles(n) + kRadix;
}

cudaError_t radix_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in,
                             uint32_t* keys_out, uint32_t* vals_out, uint32_t* keys_tmp,
                             uint32_t* vals_tmp, uint32_t* scratch, int64_t n, int bits,
                             cudaStream_t stream, uint32_t* epoch) {
  if (n <= 0) return cudaSuccess;
  const int passes = bits <= 0 ? 1 : (bits + 7) / 8;
  const int ntiles = sort_num_tiles(n);
  uint32_t* tile_hist = scratch;
  uint32_t* digit_total = scratch + (size_t)kRadix * ntiles;
  const uint32_t* kin = keys_in;
  const uint32_t* vin = vals_in;
  for (int p = 0; p < passes; ++p) {
    // the last pass lands in keys_out/vals_out
    bool to_out = ((passes - 1 - p) % 2) == 0;
    uint32_t* ko = to_out ? keys_out : keys_tmp;
    uint32_t* vo = to_out ? vals_out : vals_tmp;
    const int shift = 8 * p;
    sort_hist<<<ntiles, kSortThreads, 0, stream>>>(kin, n, shift, tile_hist, ntiles,
                                                   p == 0 ? epoch : nullptr);
    sort_dscan<<<kRadix, 1024, 0, stream>>>(tile_hist, ntiles, digit_total);
    sort_scatter<<<ntiles, kSortThreads, 0, stream>>>(kin, vin, ko, vo, n, shift, tile_hist,
                                                      digit_total, ntiles);
    kin = ko;
    vin = vo;
  }
  return cudaGetLastError();
}

}  // namespace sphg
