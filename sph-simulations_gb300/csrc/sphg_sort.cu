// sphg_sort.cu -- stable LSD radix sort of (uint32 key, uint32 value) pairs,
// written for this library (no CUB/Thrust).  It replaces the
// thrust::sort_by_key of cuSortContainerByCellID
// (core/acceleration/cuFindNeighbors.cu:82-100), sorting the slot index
// instead of six payload arrays; the payload is gathered once afterwards.
//
// One-sweep structure, 8-bit digits:
//   sort_hist_all   one read of the keys -> digit histograms of every pass
//   sort_pass       one kernel per pass: a CTA takes the next tile of 2048 keys
//                   (tile ids handed out in start order by an atomic counter),
//                   ranks them stably in registers (__match_any_sync + popc,
//                   rounds of 256 consecutive keys), publishes its per-digit
//                   counts, finds its global offsets by a decoupled look-back
//                   over the preceding tiles' published counts, and scatters.
// The look-back only waits on tiles that started earlier (so it cannot
// deadlock); each wait is bounded and sets an error word if it gives up.
#include <cstdint>
#include <cuda_runtime.h>

#include "sphg_sort.cuh"

namespace sphg {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;
constexpr int kWarps = kSortThreads / 32;
constexpr int kMaxPasses = 4;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPre = 2u << 30;
constexpr uint32_t kValMask = kFlagAgg - 1u;
constexpr int kSpinLimit = 1 << 22;

static inline int passes_for(int bits) { return bits <= 0 ? 1 : (bits + 7) / 8; }

int sort_num_tiles(int64_t n) { return (int)((n + kTile - 1) / kTile); }

// scratch: [passes x 256 histogram][passes tile counters][error word][pad to 256]
//          [passes x ntiles x 256 look-back words]
static inline size_t head_words() { return (size_t)kMaxPasses * kRadix + 256; }

size_t sort_scratch_words(int64_t n) {
  return head_words() + (size_t)kMaxPasses * kRadix * (size_t)sort_num_tiles(n);
}
static_assert(kMaxPasses * kRadix + 256 == 1280 && kTile == 2048, "sort_scratch_words_c layout");

// Digit histograms of every pass in one read of the keys.  Each thread counts
// a run of 16 consecutive keys; nearly sorted input has long runs of equal
// digits, so one shared atomic per run and pass replaces one per key.
constexpr int kHistPerThread = 16;

__global__ void __launch_bounds__(kSortThreads) sort_hist_all(const uint32_t* __restrict__ keys,
                                                              int64_t n, int passes,
                                                              uint32_t* __restrict__ ghist,
                                                              const uint32_t* skip) {
  if (skip && *skip) return;
  __shared__ uint32_t h[kMaxPasses][kRadix];
  for (int p = 0; p < kMaxPasses; ++p) h[p][threadIdx.x] = 0;
  __syncthreads();
  const int64_t chunk = (int64_t)kSortThreads * kHistPerThread;
  for (int64_t b = (int64_t)blockIdx.x * chunk; b < n; b += (int64_t)gridDim.x * chunk) {
    const int64_t s0 = b + (int64_t)threadIdx.x * kHistPerThread;
    uint32_t k[kHistPerThread];
    // 16-byte loads only where the address allows them: a caller's buffer may
    // start at any 4-byte boundary (a view such as keys + 1)
    if (s0 + kHistPerThread <= n && ((reinterpret_cast<uintptr_t>(keys + s0) & 15u) == 0)) {
#pragma unroll
      for (int q = 0; q < kHistPerThread; q += 4) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(keys + s0 + q));
        k[q] = v.x; k[q + 1] = v.y; k[q + 2] = v.z; k[q + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int q = 0; q < kHistPerThread; ++q) k[q] = s0 + q < n ? __ldg(keys + s0 + q) : 0u;
    }
    const int m = (int)(s0 >= n ? 0 : (n - s0 < kHistPerThread ? n - s0 : kHistPerThread));
    for (int p = 0; p < passes; ++p) {
      uint32_t run_d = 0, run_c = 0;
#pragma unroll
      for (int q = 0; q < kHistPerThread; ++q) {
        if (q >= m) break;
        const uint32_t d = (k[q] >> (8 * p)) & (kRadix - 1);
        if (run_c && d != run_d) {
          atomicAdd(&h[p][run_d], run_c);
          run_c = 0;
        }
        run_d = d;
        ++run_c;
      }
      if (run_c) atomicAdd(&h[p][run_d], run_c);
    }
  }
  __syncthreads();
  for (int p = 0; p < passes; ++p)
    if (h[p][threadIdx.x]) atomicAdd(&ghist[p * kRadix + threadIdx.x], h[p][threadIdx.x]);
}

template <int ITEMS>
__global__ void __launch_bounds__(kSortThreads) sort_pass(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int64_t n, int pass,
    const uint32_t* __restrict__ ghist, uint32_t* tile_counter, uint32_t* lookback,
    uint32_t* err, uint32_t* epoch, const uint32_t* skip) {
  if (skip && *skip) return;  // the incremental re-sort handled this step
  __shared__ uint32_t s_tile;
  __shared__ uint32_t base_s[kRadix];
  __shared__ uint32_t running[kRadix];
  __shared__ uint32_t warp_cnt[kWarps][kRadix];
  __shared__ uint32_t wsum[kWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int shift = 8 * pass;

  if (tid == 0) s_tile = atomicAdd(tile_counter + pass, 1u);
  // start of digit tid in the output: exclusive scan of this pass's histogram
  const uint32_t tot = ghist[pass * kRadix + tid];
  uint32_t x = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  running[tid] = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) warp_cnt[w][tid] = 0;
  __syncthreads();
  uint32_t dstart = x - tot;
  for (int w = 0; w < warp; ++w) dstart += wsum[w];
  const uint32_t tile = s_tile;
  const int64_t base = (int64_t)tile * (kSortThreads * ITEMS);
  if (epoch && tile == 0 && tid == 0) *epoch += 1u;  // nobody reads the epoch during the sort

  // load the tile (striped: round k holds keys base + k*256 + tid)
  uint32_t key[ITEMS], val[ITEMS], rank[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int64_t i = base + (int64_t)k * kSortThreads + tid;
    if (i < n) {
      key[k] = __ldg(keys_in + i);
      val[k] = vals_in ? __ldg(vals_in + i) : (uint32_t)i;
    } else {
      key[k] = 0;
      val[k] = 0;
    }
  }
  // stable in-tile ranks
  const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const bool valid = base + (int64_t)k * kSortThreads + tid < n;
    const uint32_t d = valid ? (key[k] >> shift) & (kRadix - 1) : kRadix;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && lane == __ffs(peers) - 1) warp_cnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t pre = 0;
      for (int w = 0; w < warp; ++w) pre += warp_cnt[w][d];
      rank[k] = running[d] + pre + __popc(peers & lt_mask);
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

  // publish this tile's count of digit tid, then look back for the exclusive prefix
  const uint32_t cnt = running[tid];
  uint32_t* my = lookback + (size_t)tile * kRadix + tid;
  uint32_t excl = 0;
  if (tile == 0) {
    atomicExch(my, kFlagPre | cnt);
  } else {
    atomicExch(my, kFlagAgg | cnt);
    // walk back eight predecessors per round trip: add their counts until one
    // carries an inclusive prefix
    int64_t t = (int64_t)tile - 1;
    int spins = 0;
    bool done = false;
    while (!done && t >= 0) {
      uint32_t w[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        w[q] = (t - q >= 0) ? *((const volatile uint32_t*)(lookback + (size_t)(t - q) * kRadix + tid))
                            : kFlagPre;
      int used = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        if (done || used < q) continue;  // stop at the first word not yet published
        const uint32_t v = w[q];
        if ((v & (kFlagAgg | kFlagPre)) == 0) continue;
        excl += v & kValMask;
        used = q + 1;
        if (v & kFlagPre) done = true;
      }
      t -= used;
      if (!done && used < 8 && t >= 0) {
        if (++spins > kSpinLimit) {  // give up: flag the error, treat the rest as zero
          atomicExch(err, 1u);
          break;
        }
        __nanosleep(32);
      }
    }
    atomicExch(my, kFlagPre | (excl + cnt));
  }
  base_s[tid] = dstart + excl;
  __syncthreads();

#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int64_t i = base + (int64_t)k * kSortThreads + tid;
    if (i < n) {
      const uint32_t d = (key[k] >> shift) & (kRadix - 1);
      const uint32_t pos = base_s[d] + rank[k];
      keys_out[pos] = key[k];
      vals_out[pos] = val[k];
    }
  }
}

cudaError_t radix_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in,
                             uint32_t* keys_out, uint32_t* vals_out, uint32_t* keys_tmp,
                             uint32_t* vals_tmp, uint32_t* scratch, int64_t n, int bits,
                             cudaStream_t stream, uint32_t* epoch, const uint32_t* hist,
                             const uint32_t* skip, bool clear_err) {
  if (n <= 0) return cudaSuccess;
  const int passes = passes_for(bits);
  // big inputs: 4096-key tiles halve the look-back chain; small ones: 2048 for parallelism
  const int items = n >= (1 << 18) ? 16 : 8;
  const int ntiles = (int)((n + kSortThreads * items - 1) / (kSortThreads * items));
  uint32_t* ghist = scratch;
  uint32_t* tile_counter = scratch + kMaxPasses * kRadix;
  uint32_t* err = tile_counter + kMaxPasses;
  uint32_t* lookback = scratch + head_words();
  // tile counters and look-back words start at zero every sort; so does the
  // histogram unless the caller accumulated it already.  The error word is
  // cleared too when clear_err is set (stand-alone sorts); a step's sort leaves
  // it alone so it stays set until the handle reports it.
  cudaError_t e;
  const size_t head_clear = kMaxPasses + (clear_err ? 1 : 0);
  if (hist) {
    e = cudaMemsetAsync(tile_counter, 0, sizeof(uint32_t) * head_clear, stream);
  } else {
    e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * (kMaxPasses * kRadix + head_clear), stream);
  }
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(lookback, 0, sizeof(uint32_t) * (size_t)passes * kRadix * ntiles, stream);
  if (e != cudaSuccess) return e;
  if (!hist) {
    const int64_t hchunks = (n + kSortThreads * kHistPerThread - 1) / (kSortThreads * kHistPerThread);
    const int hist_blocks = (int)(hchunks < 608 ? hchunks : 608);
    sort_hist_all<<<hist_blocks, kSortThreads, 0, stream>>>(keys_in, n, passes, ghist, skip);
    hist = ghist;
  }
  const uint32_t* kin = keys_in;
  const uint32_t* vin = vals_in;
  for (int p = 0; p < passes; ++p) {
    const bool to_out = ((passes - 1 - p) % 2) == 0;  // the last pass lands in keys_out
    uint32_t* ko = to_out ? keys_out : keys_tmp;
    uint32_t* vo = to_out ? vals_out : vals_tmp;
    if (items == 16)
      sort_pass<16><<<ntiles, kSortThreads, 0, stream>>>(kin, vin, ko, vo, n, p, hist, tile_counter,
                                                         lookback + (size_t)p * kRadix * ntiles, err,
                                                         p == 0 ? epoch : nullptr, skip);
    else
      sort_pass<8><<<ntiles, kSortThreads, 0, stream>>>(kin, vin, ko, vo, n, p, hist, tile_counter,
                                                        lookback + (size_t)p * kRadix * ntiles, err,
                                                        p == 0 ? epoch : nullptr, skip);
    kin = ko;
    vin = vo;
  }
  return cudaGetLastError();
}

uint32_t* sort_error_word(uint32_t* scratch) { return scratch + kMaxPasses * kRadix + kMaxPasses; }

}  // namespace sphg
