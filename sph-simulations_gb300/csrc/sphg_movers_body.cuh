// sphg_movers_body.cuh -- the incremental re-sort's per-block work, shared by
// the stand-alone merge kernel (sphg_movers.cu) and the fused single-launch
// iteration (sphg_step.cu).  The algorithm is described in sphg_movers.cu.
//
// COHERENT: the caller is a kernel that rewrites keyA and the cell-range table
// later in the same launch (the fused iteration); their loads then bypass the
// incoherent L1 / texture path (ld.global.cg), so no stale line of them is left
// in an SM's L1 for the later phases' reads.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "sphg_common.cuh"
#include "sphg_movers.cuh"

namespace sphg {

constexpr int kMergeThreads = 128;
#ifndef SPHG_MERGE_SLOTS
#define SPHG_MERGE_SLOTS 4
#endif
constexpr int kMergeSlots = SPHG_MERGE_SLOTS;               // slots per thread
constexpr int kMergeBlockSlots = kMergeThreads * kMergeSlots;  // 512 slots, 16 mask words
constexpr int kSpanCap = 256;                               // movers inside a block's key span kept in shared memory
// The stand-alone merge kernel's first blocks place the movers (a warp each,
// from the start of the launch: their chain of dependent loads overlaps the
// other blocks' work), the others only the unchanged slots: at most
// kMoverBlocks of them (1M dam break: 17.7 -> 14.9 us against every block
// placing its share of the movers after its unchanged slots).
constexpr int kMoverBlocks = 512;
static_assert(kMergeBlockSlots / 32 <= kMergeThreads, "one thread per mask word of the block");

template <bool COHERENT, class T>
__device__ __forceinline__ T merge_load(const T* p) {
  if constexpr (COHERENT) return __ldcg(p);
  else return __ldg(p);
}

// Slot `from` of the integrated state (its values p, v, id) to sorted position
// `to` (COHERENT: stores that bypass L1, read by a later phase of the launch).
template <bool COHERENT, class V>
__device__ __forceinline__ void merge_store(V* p, V v) {
  if constexpr (COHERENT) __stcg(p, v);
  else *p = v;
}
template <bool COHERENT>
__device__ __forceinline__ void merge_place(const MoverArgs& a, int64_t from, int64_t to, uint32_t key, float2 p,
                                            float2 v, int32_t id) {
  merge_store<COHERENT>(a.keyS + to, key);
  merge_store<COHERENT>(a.perm + to, (uint32_t)from);
  merge_store<COHERENT>(a.posA + to, p);
  merge_store<COHERENT>(a.velpA + to, make_float4(v.x, v.y, 0.f, 0.f));
  if (a.idsA) merge_store<COHERENT>(a.idsA + to, id);
}

// Position of (k, sl) among the slots of the current sorted order: the number
// of slots s with (keyA[s], s) < (k, sl).  When cell k holds particles now its
// range [start, end) gives it directly (an entry is current when the key at
// its start is k: a cell that is empty now has no slot with key k); otherwise
// a warp-wide 32-way search of the keys finds it.  All lanes return the value.
template <bool COHERENT>
__device__ __forceinline__ int64_t merge_current_position(const MoverArgs& a, uint32_t k, uint32_t sl, int lane) {
  const uint4 cr = merge_load<COHERENT>(a.ranges + k);
  if (cr.x < cr.y && cr.y <= (uint64_t)a.n && merge_load<COHERENT>(a.keyA + cr.x) == k)
    return sl < cr.x ? (int64_t)cr.x : (sl > cr.y ? (int64_t)cr.y : (int64_t)sl);
  int64_t lo = 0, hi = a.n;
  while (hi - lo > 32) {
    const int64_t step = (hi - lo + 31) / 32;
    const int64_t pos = lo + (int64_t)(lane + 1) * step - 1;
    bool less = false;
    if (pos < hi) {
      const uint32_t kp = merge_load<COHERENT>(a.keyA + pos);
      less = kp < k || (kp == k && pos < (int64_t)sl);
    }
    const int cnt = __popc(__ballot_sync(0xffffffffu, less));
    const int64_t nhi = lo + (int64_t)(cnt + 1) * step - 1;
    lo += (int64_t)cnt * step;
    if (nhi < hi) hi = nhi;
  }
  bool less = false;
  if (lo + lane < hi) {
    const int64_t pos = lo + lane;
    const uint32_t kp = merge_load<COHERENT>(a.keyA + pos);
    less = kp < k || (kp == k && pos < (int64_t)sl);
  }
  return lo + __popc(__ballot_sync(0xffffffffu, less));
}

// The decision, by every block from the force pass's count: merge when at most
// kMoverCap slots changed.  The leader records it (decision word, count, the
// step epoch the skipped radix sort would have bumped, the graph's conditional).
__device__ __forceinline__ bool merge_decide(const MoverArgs& a, bool leader, uint32_t* total) {
  const uint32_t t = *(volatile const uint32_t*)a.count;
  const bool inc = t <= (uint32_t)kMoverCap;
  if (leader) {
    a.ctl[0] = inc ? 1u : 0u;
    a.ctl[1] = t;
    if (inc) atomicAdd(a.epoch, 1u);
    if (a.cond) cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, inc ? 0u : 1u);
  }
  *total = t;
  return inc;
}

// Mover q of the list (key << 32 | slot): its rank among the movers, its
// current position and the movers below that, then its state to its final
// position.  The whole warp calls it.
template <bool COHERENT>
__device__ __forceinline__ void merge_mover(const MoverArgs& a, uint32_t q, uint32_t m, int lane) {
  const unsigned long long* __restrict__ ml = a.movers;
  const unsigned long long e = __ldg(ml + q);
  const uint32_t k = (uint32_t)(e >> 32), sl = (uint32_t)e;
  const int64_t pcur = merge_current_position<COHERENT>(a, k, sl, lane);
  uint32_t rank = 0, movers_below = 0;
  for (uint32_t r = lane; r < m; r += 32) {
    const unsigned long long f = __ldg(ml + r);
    rank += f < e;
    movers_below += (int64_t)(uint32_t)f < pcur;
  }
  rank = __reduce_add_sync(0xffffffffu, rank);
  movers_below = __reduce_add_sync(0xffffffffu, movers_below);
  if (lane == 0) {
    const int64_t fin = (int64_t)rank + pcur - (int64_t)movers_below;
    if (fin >= 0 && fin < a.n && sl < a.n)
      merge_place<COHERENT>(a, sl, fin, k, a.posB[sl], a.velB[sl], a.idsA ? a.idsB[sl] : 0);
    else
      a.ctl[2] = 1u;
  }
}

// Merge block blk of nblk (slots [blk * 512, blk * 512 + 512) and its share of
// the m movers; nblk = 0: the unchanged slots only); every thread of the block
// calls it.
template <bool COHERENT>
__device__ __forceinline__ void merge_block(const MoverArgs& a, int64_t blk, uint32_t nblk, uint32_t m) {
  const unsigned long long* __restrict__ ml = a.movers;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = blk * kMergeBlockSlots;
  const int64_t last = min(base + kMergeBlockSlots, a.n) - 1;

  __shared__ unsigned long long span[kSpanCap];
  __shared__ uint32_t nspan, red_a[kMergeThreads / 32], red_b[kMergeThreads / 32];
  __shared__ uint32_t wpre[kMergeBlockSlots / 32], wbits[kMergeBlockSlots / 32];
  __syncthreads();  // (a block calling again reuses the shared arrays)
  if (tid == 0) nspan = 0;
  // the block's stayers: state loaded first (independent of the counts)
  uint32_t key[kMergeSlots];
  float2 p[kMergeSlots], vel[kMergeSlots];
  int32_t id[kMergeSlots];
  bool stay[kMergeSlots];
#pragma unroll
  for (int u = 0; u < kMergeSlots; ++u) {
    const int64_t i = base + (int64_t)u * kMergeThreads + tid;
    stay[u] = false;
    key[u] = 0;
    id[u] = 0;
    p[u] = vel[u] = make_float2(0.f, 0.f);
    if (i < a.n) {
      const uint32_t mw = __ldg(a.mask + (i >> 5));
      stay[u] = !((mw >> (i & 31)) & 1u);
      if (stay[u]) {
        key[u] = merge_load<COHERENT>(a.keyA + i);
        p[u] = a.posB[i];
        vel[u] = a.velB[i];
        if (a.idsA) id[u] = a.idsB[i];
      }
    }
  }
  if (tid < kMergeBlockSlots / 32) {
    const int64_t w = (base >> 5) + tid;
    wbits[tid] = (w << 5) < a.n ? __ldg(a.mask + w) : 0u;
  }
  const unsigned long long v0 = ((unsigned long long)merge_load<COHERENT>(a.keyA + base) << 32) | (uint32_t)base;
  const unsigned long long v1 = ((unsigned long long)merge_load<COHERENT>(a.keyA + last) << 32) | (uint32_t)last;
  __syncthreads();
  // over the mover list: movers before the block's first slot, movers ordered
  // before its first (key, slot), and the movers inside its (key, slot) span
  uint32_t ca = 0, cb = 0;
  for (uint32_t q = tid; q < m; q += kMergeThreads) {
    const unsigned long long e = __ldg(ml + q);
    ca += (uint32_t)e < (uint64_t)base;
    cb += e < v0;
    if (e >= v0 && e <= v1) {
      const uint32_t at = atomicAdd(&nspan, 1u);
      if (at < kSpanCap) span[at] = e;
    }
  }
  ca = __reduce_add_sync(0xffffffffu, ca);
  cb = __reduce_add_sync(0xffffffffu, cb);
  if (lane == 0) {
    red_a[warp] = ca;
    red_b[warp] = cb;
  }
  if (tid == 0) {
    uint32_t run = 0;
    for (int w = 0; w < kMergeBlockSlots / 32; ++w) {
      wpre[w] = run;
      run += __popc(wbits[w]);
    }
  }
  __syncthreads();
  uint32_t before_block = 0, before_v0 = 0;
#pragma unroll
  for (int w = 0; w < kMergeThreads / 32; ++w) {
    before_block += red_a[w];
    before_v0 += red_b[w];
  }
  const uint32_t ns = nspan;
#pragma unroll
  for (int u = 0; u < kMergeSlots; ++u) {
    if (!stay[u]) continue;
    const int64_t i = base + (int64_t)u * kMergeThreads + tid;
    const int wl = (int)((i - base) >> 5);
    const uint32_t slot_before = before_block + wpre[wl] + __popc(wbits[wl] & ((1u << (i & 31)) - 1u));
    const unsigned long long v = ((unsigned long long)key[u] << 32) | (uint32_t)i;
    uint32_t key_before = before_v0;
    if (ns <= (uint32_t)kSpanCap) {
      for (uint32_t q = 0; q < ns; ++q) key_before += span[q] < v;
    } else {  // many movers inside this block's span: count over the whole list
      key_before = 0;
      for (uint32_t q = 0; q < m; ++q) key_before += __ldg(ml + q) < v;
    }
    const int64_t fin = i - (int64_t)slot_before + key_before;
    if (fin >= 0 && fin < a.n) merge_place<COHERENT>(a, i, fin, key[u], p[u], vel[u], id[u]);
    else a.ctl[2] = 1u;
  }
  // the movers, shared out over the blocks: one warp each
  if (nblk == 0) return;  // placed by blocks of their own (merge_movers)
  const uint32_t per = (m + nblk - 1) / nblk;
  const uint32_t q0 = (uint32_t)blk * per, q1 = min(q0 + per, m);
  for (uint32_t q = q0 + warp; q < q1; q += kMergeThreads / 32) merge_mover<COHERENT>(a, q, m, lane);
}

// Movers wq, wq + nw, ... of the list, one warp each (every lane calls it).
template <bool COHERENT>
__device__ __forceinline__ void merge_movers(const MoverArgs& a, uint32_t wq, uint32_t nw, uint32_t m) {
  const int lane = threadIdx.x & 31;
  for (uint32_t q = wq; q < m; q += nw) merge_mover<COHERENT>(a, q, m, lane);
}

}  // namespace sphg
