// sphg_movers.cu -- incremental re-sort of a nearly sorted state.
//
// Between two main-loop iterations a particle moves a small fraction of a
// cell, so almost every particle keeps its cell key.  The stable sort of the
// new keys (GenericNeighborSearch::SortParticleIds,
// core/alg/GenericNeighborSearch.h:69-76, with ties in previous-slot order)
// is then a merge of two sorted sequences:
//   * stayers: slots whose key did not change -- already in (key, slot) order,
//     because the current state is sorted;
//   * movers: slots whose key changed -- few, ranked here by counting.
// A stayer's new position is its rank among stayers plus the number of movers
// ordered before it; a mover's is its rank among movers plus the number of
// stayers ordered before it.  The force pass records which slots moved (one
// bit per slot, and a count per group of 8,192 slots); when more than
// kMoverCap slots moved, the full radix sort runs instead (its kernels read the
// same decision word and skip themselves otherwise).
//
// Kernels: movers_compact (mover list in slot order, movers before each word,
// decision), movers_rank_place (a warp per mover: its rank by counting the
// smaller movers, the stayers before it from the current cell-range table --
// or a warp-wide search of the keys when its new cell is empty), movers_merge
// (final position of every stayer).
#include <cstdint>

#include <cuda_runtime.h>

#include "sphg_common.cuh"
#include "sphg_movers.cuh"

namespace sphg {

namespace {

constexpr int kCompactThreads = 256;
constexpr int kCompactWords = 1;  // words per thread: 256 x 1 word = one group of 8,192 slots
static_assert(kCompactThreads * kCompactWords * 32 == (1 << kGroupShift), "one block per group");
constexpr int kRankThreads = 256;  // 8 movers per block
constexpr int kStayThreads = 128;
constexpr int kMergeSlots = 4;  // slots per thread of movers_merge

__device__ __forceinline__ uint32_t movers_before(const MoverArgs& a, int64_t p, uint32_t m) {
  if (p >= a.n) return m;
  const int64_t w = p >> 5;
  const uint32_t below = (1u << (p & 31)) - 1u;
  return a.wprefix[w] + __popc(a.mask[w] & below);
}

// Slot `from` of the integrated state (its values p, v, id) to sorted position `to`.
__device__ __forceinline__ void place_values(const MoverArgs& a, int64_t from, int64_t to, uint32_t key, float2 p,
                                             float2 v, int32_t id) {
  a.keyS[to] = key;
  a.perm[to] = (uint32_t)from;
  a.posA[to] = p;
  a.velpA[to] = make_float4(v.x, v.y, 0.f, 0.f);
  if (a.idsA) a.idsA[to] = id;
}

__device__ __forceinline__ void place(const MoverArgs& a, int64_t from, int64_t to, uint32_t key) {
  place_values(a, from, to, key, a.posB[from], a.velB[from], a.idsA ? a.idsB[from] : 0);
}

// Movers ordered before va and before vb: counts in [0, m] of the sorted mover
// list, by warp-wide 32-way searches (two dependent rounds for 8,192 movers);
// the two searches are interleaved so their load rounds overlap.
__device__ __forceinline__ void warp_count_below2(const unsigned long long* __restrict__ ms, uint32_t m,
                                                  unsigned long long va, unsigned long long vb, int lane,
                                                  uint32_t& ra, uint32_t& rb) {
  uint32_t la = 0, ha = m, lb = 0, hb = m;
  while (ha - la > 32 || hb - lb > 32) {
    const bool wa = ha - la > 32, wb = hb - lb > 32;
    const uint32_t sa = (ha - la + 31) / 32, sb = (hb - lb + 31) / 32;
    const uint32_t pa = la + (uint32_t)(lane + 1) * sa - 1, pb = lb + (uint32_t)(lane + 1) * sb - 1;
    const bool lessa = wa && pa < ha && __ldg(ms + pa) < va;
    const bool lessb = wb && pb < hb && __ldg(ms + pb) < vb;
    const uint32_t ca = __popc(__ballot_sync(0xffffffffu, lessa));
    const uint32_t cb = __popc(__ballot_sync(0xffffffffu, lessb));
    if (wa) {
      const uint32_t nh = la + (ca + 1) * sa - 1;
      la += ca * sa;
      if (nh < ha) ha = nh;
    }
    if (wb) {
      const uint32_t nh = lb + (cb + 1) * sb - 1;
      lb += cb * sb;
      if (nh < hb) hb = nh;
    }
  }
  const bool lessa = la + (uint32_t)lane < ha && __ldg(ms + la + lane) < va;
  const bool lessb = lb + (uint32_t)lane < hb && __ldg(ms + lb + lane) < vb;
  ra = la + __popc(__ballot_sync(0xffffffffu, lessa));
  rb = lb + __popc(__ballot_sync(0xffffffffu, lessb));
}

// One synchronisation for the whole block: the mover words are loaded first
// (independent of the counts), then the totals over all groups and over the
// groups before this one and the scan of the words' counts are reduced warp by
// warp, and combined once.
__global__ void __launch_bounds__(kCompactThreads) movers_compact(MoverArgs a) {
  __shared__ uint32_t red_tot[kCompactThreads / 32], red_pre[kCompactThreads / 32], scan[kCompactThreads / 32];
  const int g = blockIdx.x;
  const int ngroups = (int)gridDim.x;
  const int64_t nwords = (a.n + 31) >> 5;
  const int64_t w0 = ((int64_t)g << (kGroupShift - 5)) + (int64_t)threadIdx.x * kCompactWords;
  uint32_t mw[kCompactWords];
  uint32_t c = 0;
#pragma unroll
  for (int q = 0; q < kCompactWords; ++q) {
    mw[q] = (w0 + q < nwords) ? a.mask[w0 + q] : 0u;
    c += __popc(mw[q]);
  }
  // movers in all groups, and in the groups before this one
  uint32_t pre = 0, tot = 0;
  for (int k = threadIdx.x; k < ngroups; k += blockDim.x) {
    const uint32_t v = a.gsum[k];
    tot += v;
    if (k < g) pre += v;
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  tot = __reduce_add_sync(0xffffffffu, tot);
  pre = __reduce_add_sync(0xffffffffu, pre);
  uint32_t x = c;  // inclusive scan of the per-thread counts within the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) {
    red_tot[wp] = tot;
    red_pre[wp] = pre;
    scan[wp] = x;
  }
  __syncthreads();
  tot = pre = 0;
  uint32_t wbase = 0;
#pragma unroll
  for (int k = 0; k < kCompactThreads / 32; ++k) {
    tot += red_tot[k];
    pre += red_pre[k];
    if (k < wp) wbase += scan[k];
  }
  const bool inc = tot <= (uint32_t)kMoverCap;
  if (g == 0 && threadIdx.x == 0) {
    a.ctl[0] = inc ? 1u : 0u;
    a.ctl[1] = tot;
    if (inc) *a.epoch += 1u;  // the step epoch the skipped radix sort would have bumped
    if (a.cond) cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, inc ? 0u : 1u);
  }
  if (!inc) return;
  uint32_t r = pre + wbase + x - c;
#pragma unroll
  for (int q = 0; q < kCompactWords; ++q) {
    const int64_t w = w0 + q;
    if (w >= nwords) break;
    a.wprefix[w] = r;
    uint32_t bits = mw[q];
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1;
      const uint32_t slot = (uint32_t)((w << 5) + b);
      if (r < tot && slot < a.n) a.movers[r] = ((uint64_t)a.keyB[slot] << 32) | slot;
      else a.ctl[2] = 1u;  // inconsistent mover record: nothing is written out of bounds
      ++r;
    }
  }
}

// One warp per mover: its rank among the movers (the lanes split the
// comparisons against the whole mover list, L1-cached), then its final
// position = rank + the stayers ordered before it, found by a warp-wide
// 32-way search of the slots' (key, slot) order (four or five dependent
// rounds instead of twenty for a million slots).
__global__ void __launch_bounds__(kRankThreads) movers_rank_place(MoverArgs a) {
  cudaGridDependencySynchronize();  // the mover list and decision of movers_compact
  if (!a.ctl[0]) return;
  const uint32_t m = a.ctl[1];
  const int lane = threadIdx.x & 31;
  const uint32_t r = blockIdx.x * (kRankThreads / 32) + (threadIdx.x >> 5);
  if (r >= m) return;
  const unsigned long long v = __ldg(a.movers + r);
  uint32_t c = 0;
  for (uint32_t q = lane; q < m; q += 32) c += __ldg(a.movers + q) < v;
  const uint32_t rank = __reduce_add_sync(0xffffffffu, c);
  const uint32_t k = (uint32_t)(v >> 32), sl = (uint32_t)v;
  // p = number of slots s with (keyA[s], s) < (k, sl).  When cell k holds
  // particles in the current order, its range [start, end) gives p directly
  // (movers_compact has bumped the epoch, so the current ranges carry the
  // previous one); otherwise a warp-wide search of the keys finds it.
  const uint4 cr = __ldg(a.ranges + k);
  if (cr.z == *a.epoch - 1u && cr.x < cr.y && cr.y <= a.n) {
    if (lane == 0) {
      const int64_t p = sl < cr.x ? cr.x : (sl > cr.y ? cr.y : sl);
      if (rank < m) a.msorted[rank] = v;
      const int64_t fin = (int64_t)rank + (p - (int64_t)movers_before(a, p, m));
      if (rank < m && fin >= 0 && fin < a.n && sl < a.n) place(a, sl, fin, k);
      else a.ctl[2] = 1u;
    }
    return;
  }
  int64_t lo = 0, hi = a.n;
  while (hi - lo > 32) {
    const int64_t step = (hi - lo + 31) / 32;
    const int64_t pos = lo + (int64_t)(lane + 1) * step - 1;
    bool less = false;
    if (pos < hi) {
      const uint32_t kp = a.keyA[pos];
      less = kp < k || (kp == k && pos < (int64_t)sl);
    }
    const int cnt = __popc(__ballot_sync(0xffffffffu, less));
    const int64_t nlo = lo + (int64_t)cnt * step;
    const int64_t nhi = lo + (int64_t)(cnt + 1) * step - 1;
    lo = nlo;
    if (nhi < hi) hi = nhi;
  }
  bool less = false;
  if (lo + lane < hi) {
    const int64_t pos = lo + lane;
    const uint32_t kp = a.keyA[pos];
    less = kp < k || (kp == k && pos < (int64_t)sl);
  }
  const int64_t p = lo + __popc(__ballot_sync(0xffffffffu, less));
  if (lane == 0) {
    if (rank < m) a.msorted[rank] = v;
    const int64_t fin = (int64_t)rank + (p - (int64_t)movers_before(a, p, m));
    if (rank < m && fin >= 0 && fin < a.n && sl < a.n) place(a, sl, fin, k);
    else a.ctl[2] = 1u;
  }
}

// Each block places kMergeSlots x kStayThreads consecutive slots, those that kept their
// key (the movers are placed already): a stayer's position is its rank among
// stayers + the movers ordered before it.  The movers ordered before any slot
// of the block lie between the counts of its first and last slot, found by
// warp 0 with two interleaved warp-wide searches while the other threads load
// their slots' state; each thread then refines inside that (usually empty)
// interval.  Four slots per thread (strided by the block size, so every load
// and store stays coalesced) keep all blocks resident in one wave.
__global__ void __launch_bounds__(kStayThreads) movers_merge(MoverArgs a) {
  cudaGridDependencySynchronize();  // the sorted movers of movers_rank_place
  if (!a.ctl[0]) return;
  const uint32_t m = a.ctl[1];
  const int64_t base = (int64_t)blockIdx.x * (kStayThreads * kMergeSlots);
  if (base >= a.n) return;
  const int64_t last = min(base + kStayThreads * kMergeSlots, a.n) - 1;
  __shared__ uint32_t bounds[2];
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const unsigned long long v0 = ((unsigned long long)a.keyA[base] << 32) | (uint32_t)base;
    const unsigned long long v1 = ((unsigned long long)a.keyA[last] << 32) | (uint32_t)last;
    uint32_t lo, hi;
    warp_count_below2(a.msorted, m, v0, v1, lane, lo, hi);
    if (lane == 0) {
      bounds[0] = lo;
      bounds[1] = hi;
    }
  }
  uint32_t key[kMergeSlots], before[kMergeSlots];
  float2 p[kMergeSlots], vel[kMergeSlots];
  int32_t id[kMergeSlots];
  bool stay[kMergeSlots];
#pragma unroll
  for (int u = 0; u < kMergeSlots; ++u) {
    const int64_t i = base + (int64_t)u * kStayThreads + threadIdx.x;
    stay[u] = false;
    key[u] = 0;
    before[u] = 0;
    id[u] = 0;
    p[u] = vel[u] = make_float2(0.f, 0.f);
    if (i < a.n) {
      const uint32_t mw = a.mask[i >> 5];
      stay[u] = !((mw >> (i & 31)) & 1u);
      if (stay[u]) {
        key[u] = a.keyA[i];
        before[u] = a.wprefix[i >> 5] + __popc(mw & ((1u << (i & 31)) - 1u));
        p[u] = a.posB[i];
        vel[u] = a.velB[i];
        if (a.idsA) id[u] = a.idsB[i];
      }
    }
  }
  __syncthreads();
  const uint32_t blo = bounds[0], bhi = bounds[1];
#pragma unroll
  for (int u = 0; u < kMergeSlots; ++u) {
    if (!stay[u]) continue;
    const int64_t i = base + (int64_t)u * kStayThreads + threadIdx.x;
    const unsigned long long v = ((unsigned long long)key[u] << 32) | (uint32_t)i;
    uint32_t lo = blo, hi = bhi;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (a.msorted[mid] < v) lo = mid + 1;
      else hi = mid;
    }
    const int64_t fin = i - (int64_t)before[u] + lo;
    if (fin >= 0 && fin < a.n) place_values(a, i, fin, key[u], p[u], vel[u], id[u]);
    else a.ctl[2] = 1u;
  }
}

}  // namespace

int mover_groups(int64_t n) { return (int)((n + (1 << kGroupShift) - 1) >> kGroupShift); }

cudaError_t launch_movers(const MoverArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  const int64_t cap = a.n < kMoverCap ? a.n : kMoverCap;
  const int per_block = kRankThreads / 32;
  movers_compact<<<mover_groups(a.n), kCompactThreads, 0, st>>>(a);
  cudaError_t e = launch_pdl(movers_rank_place, dim3((unsigned)((cap + per_block - 1) / per_block)),
                             dim3(kRankThreads), 0, st, a);
  if (e != cudaSuccess) return e;
  const int64_t merge_block = (int64_t)kStayThreads * kMergeSlots;
  e = launch_pdl(movers_merge, dim3((unsigned)((a.n + merge_block - 1) / merge_block)), dim3(kStayThreads), 0, st,
                 a);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace sphg
