// sphg_step.cu -- the per-step SPH kernels for sm_103a.
//
// Step pipeline (one launch each, plus the re-sort of sphg_movers.cu or the
// radix sort of sphg_sort.cu):
//   step_keys      cell key of every particle (first iteration after an upload;
//                  afterwards the force pass computes the next keys)
//                  (GenericNeighborSearch::SetParticleCellIds, GenericNeighborSearch.h:201-231)
//   [re-sort]      stable order of (key, slot): merge of the slots that changed
//                  cell, or the full radix sort (SortParticleIds, :69-76)
//   step_reorder   cell ranges (and, after a full sort, the gather of the state
//                  into key order) (SortContainer :111-191, SetCellRanges :93-108)
//   step_density   3x3-stencil density + EOS pressure, stores p/rho^2 and 1/rho
//                  (ApproximateDensity GenericForceComputation.tpp:35-130,
//                   CalculatePressure :23-32, cuInvertDensity)
//   step_force     pressure + viscosity (+ artificial viscosity) + gravity,
//                  fused with the next step's symplectic-Euler update and walls
//                  (ComputeForces :134-253, Integrator.cpp:7-46)
//   step_diag      step-header diagnostics, when asked for (StepHeader,
//                  app/simulation_configuration.h:152-158)
//
// Neighbour decisions and cell keys are the reference's FP64 decisions made
// exactly from FP32 state: the FP32 value decides unless it lies in a thin
// band around the threshold, where the reference's FP64 expression is
// evaluated (sphg_common.cuh).
#include <algorithm>
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "sphg_movers.cuh"
#include "sphg_movers_body.cuh"
#include "sphg_neighbor.cuh"
#include "sphg_step.cuh"

namespace sphg {

constexpr int kThreads = 128;  // 128-thread blocks: measured a little faster than 256 and 512 for the passes

// Stores of the phase outputs that a later phase of the fused single-launch
// iteration (step_fused) reads: there they bypass L1 (st.global.cg), so no
// SM keeps a partial line of data other SMs write in the same launch.
template <bool FUSED, class V>
__device__ __forceinline__ void st_out(V* p, V v) {
  if constexpr (FUSED) __stcg(p, v);
  else *p = v;
}

// ---------------------------------------------------------------- keys
template <int PREC, bool BATCHED>
__global__ void __launch_bounds__(kThreads) step_keys(StepArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < a.n;
  uint32_t key = 0;
  if (valid) {
    const InstDesc d = inst_of<BATCHED>(a, i);
    float2 p = a.posB[i];
    const int cmx = d.periodic ? d.nxr - 1 : d.nx - 1;
    const int cmy = d.periodic ? d.nyr - 1 : d.ny - 1;
    int cx, cy;
    if (PREC == 0) {
      cx = cell_coord(p.x, d.lo_x, d.inv_cs_x, d.lo_xd, d.cs_xd, cmx);
      cy = cell_coord(p.y, d.lo_y, d.inv_cs_y, d.lo_yd, d.cs_yd, cmy);
    } else {
      int ox, oy;
      decode_code(d, a.keyA[i] - d.cell_base, ox, oy);
      int kx = offset_cells(p.x, d.inv_cs_x, d.cs_xd);
      int ky = offset_cells(p.y, d.inv_cs_y, d.cs_yd);
      cx = ox + kx;
      cy = oy + ky;
      int sx = kx, sy = ky;  // cells the offset moves by
      if (d.periodic) {
        cx = ((cx % d.nxr) + d.nxr) % d.nxr;
        cy = ((cy % d.nyr) + d.nyr) % d.nyr;
      } else {
        cx = cx < 0 ? 0 : (cx > cmx ? cmx : cx);
        cy = cy < 0 ? 0 : (cy > cmy ? cmy : cy);
        sx = cx - ox;
        sy = cy - oy;
      }
      if (sx) p.x = offset_shift_d(p.x, sx, d.cs_xd);
      if (sy) p.y = offset_shift_d(p.y, sy, d.cs_yd);
      a.posB[i] = p;
    }
    key = d.cell_base + local_code(d, cx, cy);
    a.keyB[i] = key;
  }
}

// ---------------------------------------------------------------- reorder + cell ranges
// kReorderSlots slots per thread, strided by the block size (coalesced), their
// keys loaded before any is used.
constexpr int kReorderSlots = 4;

template <bool FUSED>
__device__ __forceinline__ void reorder_slot(const StepArgs& a, int64_t i, uint32_t k, uint32_t kprev,
                                             uint32_t knext, bool gather, uint32_t ep) {
  st_out<FUSED>(a.keyA + i, k);
  if (gather) {  // after a full sort (a merge scattered the state already)
    const uint32_t src = a.perm[i];
    st_out<FUSED>(a.posA + i, a.posB[src]);
    const float2 v = a.velB[src];
    st_out<FUSED>(a.velpA + i, make_float4(v.x, v.y, 0.f, 0.f));
    if (a.track_ids) st_out<FUSED>(a.idsA + i, a.idsB[src]);
  }
  uint32_t* r = reinterpret_cast<uint32_t*>(a.ranges);
  if (k != kprev) {
    st_out<FUSED>(r + 4 * (size_t)k, (uint32_t)i);
    st_out<FUSED>(r + 4 * (size_t)k + 2, ep);
  }
  if (k != knext) st_out<FUSED>(r + 4 * (size_t)k + 1, (uint32_t)(i + 1));
  if (a.tile_bits) {
    const int sh = 2 * a.tile_bits;
    const uint32_t t = k >> sh;
    uint32_t* tr = reinterpret_cast<uint32_t*>(a.tile_ranges);
    if (kprev == kNoIndex || (kprev >> sh) != t) {
      tr[2 * (size_t)t] = (uint32_t)i;
      a.tile_list[atomicAdd(a.tile_count, 1u)] = t;
    }
    if (knext == kNoIndex || (knext >> sh) != t) tr[2 * (size_t)t + 1] = (uint32_t)(i + 1);
  }
}

// Reorder block blk: slots [blk * 512, blk * 512 + 512).
template <bool FUSED>
__device__ __forceinline__ void reorder_block(const StepArgs& a, int64_t blk) {
  const int64_t base = blk * (kThreads * kReorderSlots) + threadIdx.x;
  uint32_t k[kReorderSlots], kp[kReorderSlots], kn[kReorderSlots];
#pragma unroll
  for (int u = 0; u < kReorderSlots; ++u) {
    const int64_t i = base + (int64_t)u * kThreads;
    k[u] = kp[u] = kn[u] = kNoIndex;
    if (i < a.n) {
      k[u] = a.keyS[i];
      kp[u] = i > 0 ? a.keyS[i - 1] : kNoIndex;
      kn[u] = i + 1 < a.n ? a.keyS[i + 1] : kNoIndex;
    }
  }
  const bool gather = !(a.merged && *a.merged);
  const uint32_t ep = *a.epoch;
#pragma unroll
  for (int u = 0; u < kReorderSlots; ++u) {
    const int64_t i = base + (int64_t)u * kThreads;
    if (i < a.n) reorder_slot<FUSED>(a, i, k[u], kp[u], kn[u], gather, ep);
  }
}

__global__ void __launch_bounds__(kThreads) step_reorder(StepArgs a) {
  cudaGridDependencySynchronize();  // the sorted keys (and the decision word) of the re-sort
  allow_next_kernel(a.early_next);
  // the mover count of this iteration's force pass starts at zero (this
  // iteration's re-sort, the kernel before, has read the last one)
  if (a.mover_count && blockIdx.x == 0 && threadIdx.x == 0) *a.mover_count = 0;
  reorder_block<false>(a, blockIdx.x);
}

// ---------------------------------------------------------------- density + pressure
// Pair vector x_i - x_j of a recorded neighbour entry (j << 5 | tag): the tag's
// stencil offset k = 3 (c1 + 1) + (c2 + 1) moves the split offsets into one
// cell frame; bit 4 marks a periodic wrap (plain positions: minimum image).
template <int PREC>
__device__ __forceinline__ void entry_vec(const InstDesc& d, float2 pi, float2 pj, uint32_t e,
                                          float& dx, float& dy) {
  if (PREC == 0 && (e & 16u)) {
    wrapped_pair(d, pi, pj, dx, dy);
  } else {
    const uint32_t k = e & 15u;
    const int c1 = (int)(k / 3) - 1, c2 = (int)(k % 3) - 1;
    const float shx = (PREC == 1) ? (c1 == 0 ? 0.f : (c1 > 0 ? d.cs_x : -d.cs_x)) : 0.f;
    const float shy = (PREC == 1) ? (c2 == 0 ? 0.f : (c2 > 0 ? d.cs_y : -d.cs_y)) : 0.f;
    dx = (pi.x - pj.x) - shx;
    dy = (pi.y - pj.y) - shy;
  }
}

#ifndef SPHG_DENSITY_TRIM
#define SPHG_DENSITY_TRIM 1
#endif
// 1: the split walk skips the particle itself by splitting its own cell, the
// prefetch past the last candidate reads the padding entry of the positions,
// and the record is unconditional (the step's density pass always records)
constexpr bool kDensityTrim = SPHG_DENSITY_TRIM != 0;


template <int PREC, bool BATCHED, bool CSR, int T = kThreads>
__global__ void __launch_bounds__(T) step_density(StepArgs a);

// Density + pressure of particle i (i < n); FUSED: the outputs bypass L1 (st_out).
template <int PREC, bool BATCHED, bool CSR, int T, bool FUSED>
__device__ __forceinline__ void density_particle(const StepArgs& a, int64_t i) {
  typename std::conditional<BATCHED, const InstDesc&, const InstDesc>::type d = inst_ref<BATCHED>(a, i);
  if (BATCHED && !d.active) return;  // a finished served instance
  const uint32_t key = a.keyA[i];
  const float2 pi = a.posA[i];
  typename std::conditional<PREC == 1, CSum, PSum>::type S;
  int cx, cy;
  const float inv_h2 = d.inv_h2;
  if constexpr (CSR) {
    // MPListsForceComputation::ApproximateDensity: the list in its order, self included
    const int64_t b = min(a.csr_offs[i], a.csr_cap), e = min(a.csr_offs[i + 1], a.csr_cap);
    for (int64_t q = b; q < e; ++q) {
      const uint32_t ent = __ldg(a.csr_idx + q);
      float dx, dy;
      entry_vec<PREC>(d, pi, __ldg(a.posA + (ent >> 5)), ent, dx, dy);
      const float r2 = fmaf(dx, dx, dy * dy);
      const float t = fmaf(-r2, inv_h2, 1.0f);
      S.add(t * t * t);
    }
  } else {
    __shared__ uint4 s_cells[10][T];  // per thread: its non-empty stencil cells (own cell split at itself)
    uint32_t* __restrict__ nbr = a.nbr;
    const uint32_t slots = (uint32_t)a.nbr_slots;
    const size_t n = (size_t)a.n;
    uint32_t cnt = 0;
    auto accept = [&](uint32_t e, float r2) {  // e = j << 5 | stencil tag
      const float t = fmaf(-r2, inv_h2, 1.0f);
      S.add(t * t * t);
      if (nbr && (e >> 5) != (uint32_t)i) {  // record the pair for the force pass
        if (cnt < slots) st_out<FUSED>(nbr + cnt * n + i, e);
        ++cnt;
      }
    };
    if (nbr && n < ((size_t)1 << 27)) {
      // One loop over the candidates of the non-empty stencil cells, cells in
      // the stencil order and j ascending within a cell.  A warp then runs about
      // max over its lanes of the candidate total instead of the sum over the
      // nine cells of the per-cell maxima (cells hold 1-4 particles, so
      // per-cell loops keep half the lanes idle).  The cells are queued in
      // shared memory as {j0 << 5 | tag, j1 << 5 | tag, shift x, shift y}; the
      // position of the next candidate is loaded one iteration ahead; pairs are
      // accumulated branch-free (about a third of the candidates are accepted,
      // so a branch would be taken by some lane nearly always).  In split
      // precision the particle's own term W(0) = 1 is the first term of the
      // compensated sum (which then needs only Fast2Sum) and is skipped in the
      // walk; plain sums add it where the walk meets it.
      const int tid = threadIdx.x;
      const uint32_t code = key - d.cell_base;
      decode_code(d, code, cx, cy);
      const uint32_t ep = *a.epoch;
      uint32_t c[9], valid, wrapmask;
      stencil_keys(d, code, cx, cy, c, valid, wrapmask);
      uint4 r[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) r[k] = ((valid >> k) & 1u) ? __ldg(a.ranges + c[k]) : make_uint4(0, 0, 0, 0);
      int nseg = 0;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        if (r[k].z == ep && r[k].y > r[k].x) {
          const int c1 = k / 3 - 1, c2 = k % 3 - 1;
          const uint32_t tag = (uint32_t)k | ((PREC == 0 && ((wrapmask >> k) & 1u)) ? 16u : 0u);
          const float shx = (PREC == 1) ? (c1 == 0 ? 0.f : (c1 > 0 ? d.cs_x : -d.cs_x)) : 0.f;
          const float shy = (PREC == 1) ? (c2 == 0 ? 0.f : (c2 > 0 ? d.cs_y : -d.cs_y)) : 0.f;
          if (kDensityTrim && PREC == 1 && k == 4) {
            // own cell without the particle itself (its term W(0) = 1 is added
            // first): [start, i) and (i, end), whichever are not empty
            const uint32_t self = (uint32_t)i;
            if (self > r[k].x)
              s_cells[nseg++][tid] = make_uint4((r[k].x << 5) | tag, (self << 5) | tag, 0u, 0u);
            if (self + 1 < r[k].y)
              s_cells[nseg++][tid] = make_uint4(((self + 1) << 5) | tag, (r[k].y << 5) | tag, 0u, 0u);
            continue;
          }
          s_cells[nseg][tid] = make_uint4((r[k].x << 5) | tag, (r[k].y << 5) | tag, __float_as_uint(shx),
                                          __float_as_uint(shy));
          ++nseg;
        }
      }
      const float2* __restrict__ pos = a.posA;
      const float h2_lo = d.h2_lo, h2_hi = d.h2_hi;
      const bool record = nbr != nullptr;
      const uint32_t self = (uint32_t)i;
      uint32_t* rp = record ? nbr + i : nullptr;  // next record slot: nbr[cnt * n + i]
      bool border = false;
      if (PREC == 1) S.add(1.0f);  // own term W(0) first (plain sums keep the walk's order)
      if (nseg > 0) {  // plain: always (the particle's own cell holds it); split: any other particle near
        uint4 w = s_cells[0][tid];
        int q = 1;
        uint32_t jj = w.x, je = w.y;
        float shx = __uint_as_float(w.z), shy = __uint_as_float(w.w);
        float2 pj = __ldg(pos + (jj >> 5));
        while (true) {
          uint32_t jn = jj + 32u, jen = je;
          float shxn = shx, shyn = shy;
          bool more = true;
          if (jn == je) {
            if (q == nseg) {
              more = false;
            } else {
              w = s_cells[q][tid];
              ++q;
              jn = w.x;
              jen = w.y;
              shxn = __uint_as_float(w.z);
              shyn = __uint_as_float(w.w);
            }
          }
          // one candidate ahead (past the last one: the end of its cell, at most
          // slot n -- the positions hold one entry more)
          const float2 pn = __ldg(pos + ((kDensityTrim || more ? jn : jj) >> 5));
          const uint32_t j = jj >> 5;
          const float2 dxy = sub2(sub2(pi, pj), make_float2(shx, shy));
          float dx = dxy.x, dy = dxy.y;
          float r2;
          bool in;
          if (PREC == 0 && (jj & 16u)) {  // plain position reached through the periodic boundary
            in = wrapped_pair(d, pi, pj, dx, dy);
            r2 = fmaf(dx, dx, dy * dy);
          } else {
            r2 = fmaf(dx, dx, dy * dy);
            in = r2 < h2_lo;
            border |= !in && r2 <= h2_hi;
          }
          // split: the walk never meets the particle itself; the step always records
          const bool other = (kDensityTrim && PREC == 1) || j != self;
          const float t = fmaf(-r2, inv_h2, 1.0f);
          S.add_fast((PREC == 1 ? in && other : in) ? t * t * t : 0.0f);
          const bool rec = in && other && (kDensityTrim || record);
          if (rec && cnt < slots) {
            st_out<FUSED>(rp, jj);
            rp += n;
          }
          cnt += rec ? 1u : 0u;
          if (!more) break;
          jj = jn;
          je = jen;
          shx = shxn;
          shy = shyn;
          pj = pn;
        }
      }
      if (border) {  // rare: pairs in the FP64 band, the same cells in the same order
#pragma unroll 1
        for (int s = 0; s < nseg; ++s) {
          const uint4 w = s_cells[s][tid];
          const uint32_t tag = w.x & 31u;
          if (PREC == 0 && (tag & 16u)) continue;
          const int c1 = (int)(tag / 3) - 1, c2 = (int)(tag % 3) - 1;
          const float sx = __uint_as_float(w.z), sy = __uint_as_float(w.w);
          for (uint32_t e = w.x; e != w.y; e += 32u) {
            const float2 pj = __ldg(pos + (e >> 5));
            const float dx = (pi.x - pj.x) - sx;
            const float dy = (pi.y - pj.y) - sy;
            const float r2 = fmaf(dx, dx, dy * dy);
            if (r2 >= h2_lo && r2 <= h2_hi && pair_inside<PREC>(d, pi, pj, c1, c2, r2)) accept(e, r2);
          }
        }
      }
    } else {
      for_each_neighbor<PREC>(a, d, key, pi, cx, cy, [&](uint32_t j, float, float, float r2, uint32_t tag) {
        accept((j << 5) | tag, r2);
      });
    }
    if (nbr) st_out<FUSED>(a.ncount + i, cnt);
  }
  float rho, drho;
  if constexpr (PREC == 1) {
    rho = d.wd * S.value();
    drho = fmaf(d.wd, S.s, -d.rho0) + d.wd * S.c;
  } else {
    rho = d.wd * S.value();
    drho = rho - d.rho0;
  }
  const float inv = 1.0f / rho;
  const float P = d.k * drho * inv * inv;
  st_out<FUSED>(a.rho + i, rho);
  st_out<FUSED>(reinterpret_cast<float2*>(a.velpA + i) + 1, make_float2(P, inv));
}

template <int PREC, bool BATCHED, bool CSR, int T>
__global__ void __launch_bounds__(T) step_density(StepArgs a) {
  cudaGridDependencySynchronize();  // the sorted state and cell ranges of the reorder
  allow_next_kernel(a.early_next);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  density_particle<PREC, BATCHED, CSR, T, false>(a, i);
}

// ---------------------------------------------------------------- density, two particles of a cell per thread
// The same computation as step_density's flattened stencil walk, arranged so
// that one thread carries two particles of one cell: they share the cell's
// stencil, its range loads, its queue of non-empty cells and every candidate's
// position load, while each keeps its own sum, neighbour record and self test
// -- so every particle visits the same candidates in the same order with the
// same arithmetic as in step_density (bit-identical results).  A block takes
// 256 consecutive slots, splits each run of equal keys (a cell, or the part of
// it inside the block) into pairs from its first slot, and hands the pairs
// and the odd particles out to its threads in slot order.
// slots per block: two per thread


// One particle's running state of the walk.
template <int PREC>
struct WalkAcc {
  typename std::conditional<PREC == 1, CSum, PSum>::type S;
  uint32_t cnt = 0;
  uint32_t* rp = nullptr;  // next record slot: nbr[cnt * n + i]
};

// Rare: pairs of particle pi inside the FP64 band around h^2, over the same
// queued cells in the same order (step_density's second pass).
template <int PREC, int T, class Acc>
__device__ __forceinline__ void band_pass(const InstDesc& d, const float2* __restrict__ pos,
                                          const uint4 (*cells)[T], int nseg, int tid, float2 pi,
                                          uint32_t self, Acc& A, uint32_t slots, size_t n, bool record) {
  const float h2_lo = d.h2_lo, h2_hi = d.h2_hi, inv_h2 = d.inv_h2;
#pragma unroll 1
  for (int s = 0; s < nseg; ++s) {
    const uint4 w = cells[s][tid];
    const uint32_t tag = w.x & 31u;
    if (PREC == 0 && (tag & 16u)) continue;
    const int c1 = (int)(tag / 3) - 1, c2 = (int)(tag % 3) - 1;
    const float sx = __uint_as_float(w.z), sy = __uint_as_float(w.w);
    for (uint32_t e = w.x; e != w.y; e += 32u) {
      const float2 pj = __ldg(pos + (e >> 5));
      const float dx = (pi.x - pj.x) - sx;
      const float dy = (pi.y - pj.y) - sy;
      const float r2 = fmaf(dx, dx, dy * dy);
      if (r2 >= h2_lo && r2 <= h2_hi && pair_inside<PREC>(d, pi, pj, c1, c2, r2)) {
        const float t = fmaf(-r2, inv_h2, 1.0f);
        A.S.add(t * t * t);
        if (record && (e >> 5) != self) {
          if (A.cnt < slots) *A.rp = e;
          A.rp += n;
          ++A.cnt;
        }
      }
    }
  }
}

template <int PREC>
__device__ __forceinline__ void density_epilogue(const StepArgs& a, const InstDesc& d, int64_t i,
                                                 const typename std::conditional<PREC == 1, CSum, PSum>::type& S) {
  float rho, drho;
  if constexpr (PREC == 1) {
    rho = d.wd * S.value();
    drho = fmaf(d.wd, S.s, -d.rho0) + d.wd * S.c;
  } else {
    rho = d.wd * S.value();
    drho = rho - d.rho0;
  }
  const float inv = 1.0f / rho;
  const float P = d.k * drho * inv * inv;
  a.rho[i] = rho;
  reinterpret_cast<float2*>(a.velpA + i)[1] = make_float2(P, inv);
}

template <int PREC, bool BATCHED, int T = kThreads>
__global__ void __launch_bounds__(T) step_density_pairs(StepArgs a) {
  constexpr int kPairSlots = 2 * T;
  cudaGridDependencySynchronize();  // the sorted state and cell ranges of the reorder
  allow_next_kernel(a.early_next);
  __shared__ uint32_t s_key[kPairSlots];
  __shared__ uint16_t s_chunk[kPairSlots];  // offset of each pair's (or odd particle's) first slot | partner << 15
  __shared__ uint32_t s_wmax[T / 32], s_wcnt[T / 32];
  __shared__ uint4 s_cells[9][T];   // per thread: the non-empty stencil cells of its cell
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t b0 = (int64_t)blockIdx.x * kPairSlots;
  const int nb = (int)min((int64_t)kPairSlots, a.n - b0);
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int o = u * T + tid;
    s_key[o] = o < nb ? __ldg(a.keyA + b0 + o) : kNoIndex;
  }
  __syncthreads();
  // runs of equal keys inside the block: start of each slot's run by a max-scan
  // (thread t holds offsets 2t, 2t+1), pairs counted from the run's start
  const int o0 = 2 * tid, o1 = o0 + 1;
  const uint32_t k0 = s_key[o0], k1 = s_key[o1];
  const int st0 = (o0 == 0 || s_key[o0 - 1] != k0) ? o0 : 0;
  const int st1 = (k1 != k0) ? o1 : 0;
  int m = max(st0, st1);
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, m, d);
    if (lane >= d) m = max(m, y);
  }
  if (lane == 31) s_wmax[warp] = m;
  int excl = __shfl_up_sync(0xffffffffu, m, 1);
  if (lane == 0) excl = 0;
  __syncthreads();
  for (int w = 0; w < warp; ++w) excl = max(excl, (int)s_wmax[w]);
  const int rs0 = max(excl, st0), rs1 = max(rs0, st1);
  const bool lead0 = o0 < nb && ((o0 - rs0) & 1) == 0;
  const bool lead1 = o1 < nb && ((o1 - rs1) & 1) == 0;
  const bool part0 = lead0 && o1 < nb && k1 == k0;
  const bool part1 = lead1 && o1 + 1 < nb && s_key[o1 + 1] == k1;
  const uint32_t c = (lead0 ? 1u : 0u) + (lead1 ? 1u : 0u);
  uint32_t x = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) s_wcnt[warp] = x;
  __syncthreads();
  uint32_t at = x - c, nchunks = 0;
  for (int w = 0; w < T / 32; ++w) {
    if (w < warp) at += s_wcnt[w];
    nchunks += s_wcnt[w];
  }
  if (lead0) s_chunk[at++] = (uint16_t)(o0 | (part0 ? 0x8000 : 0));
  if (lead1) s_chunk[at] = (uint16_t)(o1 | (part1 ? 0x8000 : 0));
  __syncthreads();

  uint32_t* __restrict__ nbr = a.nbr;
  const uint32_t slots = (uint32_t)a.nbr_slots;
  const size_t n = (size_t)a.n;
  const bool record = nbr != nullptr;
  const float2* __restrict__ pos = a.posA;
  for (uint32_t q = tid; q < nchunks; q += T) {
    const uint32_t ce = s_chunk[q];
    const int off = (int)(ce & 0x7fffu);
    const bool hasB = (ce >> 15) != 0;
    const int64_t iA = b0 + off, iB = hasB ? iA + 1 : iA;
    typename std::conditional<BATCHED, const InstDesc&, const InstDesc>::type d = inst_ref<BATCHED>(a, iA);
    if (BATCHED && !d.active) continue;  // a finished served instance
    const uint32_t key = s_key[off];
    const float2 pA = pos[iA], pB = pos[iB];
    const float inv_h2 = d.inv_h2;
    int cx, cy;
    const uint32_t code = key - d.cell_base;
    decode_code(d, code, cx, cy);
    const uint32_t ep = *a.epoch;
    uint32_t cs[9], valid, wrapmask;
    stencil_keys(d, code, cx, cy, cs, valid, wrapmask);
    uint4 r[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) r[k] = ((valid >> k) & 1u) ? __ldg(a.ranges + cs[k]) : make_uint4(0, 0, 0, 0);
    int nseg = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      if (r[k].z == ep && r[k].y > r[k].x) {
        const int c1 = k / 3 - 1, c2 = k % 3 - 1;
        const uint32_t tag = (uint32_t)k | ((PREC == 0 && ((wrapmask >> k) & 1u)) ? 16u : 0u);
        const float shx = (PREC == 1) ? (c1 == 0 ? 0.f : (c1 > 0 ? d.cs_x : -d.cs_x)) : 0.f;
        const float shy = (PREC == 1) ? (c2 == 0 ? 0.f : (c2 > 0 ? d.cs_y : -d.cs_y)) : 0.f;
        s_cells[nseg][tid] = make_uint4((r[k].x << 5) | tag, (r[k].y << 5) | tag, __float_as_uint(shx),
                                        __float_as_uint(shy));
        ++nseg;
      }
    }
    const float h2_lo = d.h2_lo, h2_hi = d.h2_hi;
    WalkAcc<PREC> A, B;
    A.rp = record ? nbr + iA : nullptr;
    B.rp = record ? nbr + iB : nullptr;
    bool border = false;
    if (PREC == 1) {  // own terms W(0) first (plain sums keep the walk's order)
      A.S.add(1.0f);
      B.S.add(1.0f);
    }
    if (nseg > 0) {  // always: the particles' own cell holds them
      uint4 w = s_cells[0][tid];
      int qq = 1;
      uint32_t jj = w.x, je = w.y;
      float shx = __uint_as_float(w.z), shy = __uint_as_float(w.w);
      float2 pj = __ldg(pos + (jj >> 5));
      while (true) {
        uint32_t jn = jj + 32u, jen = je;
        float shxn = shx, shyn = shy;
        bool more = true;
        if (jn == je) {
          if (qq == nseg) {
            more = false;
          } else {
            w = s_cells[qq][tid];
            ++qq;
            jn = w.x;
            jen = w.y;
            shxn = __uint_as_float(w.z);
            shyn = __uint_as_float(w.w);
          }
        }
        const float2 pn = __ldg(pos + ((more ? jn : jj) >> 5));  // one candidate ahead
        const uint32_t j = jj >> 5;
        float dxa = (pA.x - pj.x) - shx, dya = (pA.y - pj.y) - shy;
        float dxb = (pB.x - pj.x) - shx, dyb = (pB.y - pj.y) - shy;
        float r2a, r2b;
        bool ina, inb;
        if (PREC == 0 && (jj & 16u)) {  // plain positions reached through the periodic boundary
          ina = wrapped_pair(d, pA, pj, dxa, dya);
          inb = wrapped_pair(d, pB, pj, dxb, dyb);
          r2a = fmaf(dxa, dxa, dya * dya);
          r2b = fmaf(dxb, dxb, dyb * dyb);
        } else {
          r2a = fmaf(dxa, dxa, dya * dya);
          r2b = fmaf(dxb, dxb, dyb * dyb);
          ina = r2a < h2_lo;
          inb = r2b < h2_lo;
          border |= (!ina && r2a <= h2_hi) || (!inb && r2b <= h2_hi);
        }
        const bool oa = j != (uint32_t)iA, ob = j != (uint32_t)iB;
        const float ta = fmaf(-r2a, inv_h2, 1.0f), tb = fmaf(-r2b, inv_h2, 1.0f);
        A.S.add_fast((PREC == 1 ? ina && oa : ina) ? ta * ta * ta : 0.0f);
        B.S.add_fast((PREC == 1 ? inb && ob : inb) ? tb * tb * tb : 0.0f);
        const bool ra = ina && oa && record, rb = hasB && inb && ob && record;
        if (ra && A.cnt < slots) {
          *A.rp = jj;
          A.rp += n;
        }
        if (rb && B.cnt < slots) {
          *B.rp = jj;
          B.rp += n;
        }
        A.cnt += ra ? 1u : 0u;
        B.cnt += rb ? 1u : 0u;
        if (!more) break;
        jj = jn;
        je = jen;
        shx = shxn;
        shy = shyn;
        pj = pn;
      }
    }
    if (border) {
      band_pass<PREC, T>(d, pos, s_cells, nseg, tid, pA, (uint32_t)iA, A, slots, n, record);
      if (hasB) band_pass<PREC, T>(d, pos, s_cells, nseg, tid, pB, (uint32_t)iB, B, slots, n, record);
    }
    if (record) a.ncount[iA] = A.cnt;
    density_epilogue<PREC>(a, d, iA, A.S);
    if (hasB) {
      if (record) a.ncount[iB] = B.cnt;
      density_epilogue<PREC>(a, d, iB, B.S);
    }
  }
}

// ---------------------------------------------------------------- forces (+ integration)
// The pairs are the neighbours the density pass recorded (j << 5 | stencil
// tag per entry); a particle with more than the recorded slots walks the
// stencil again.
#ifndef SPHG_FORCE_BATCH
#define SPHG_FORCE_BATCH 4
#endif
constexpr int kForceBatch = SPHG_FORCE_BATCH;  // recorded neighbours gathered together
#ifndef SPHG_FORCE_TAIL
#define SPHG_FORCE_TAIL 1
#endif
#ifndef SPHG_SKIP_ZERO_VISCOSITY
#define SPHG_SKIP_ZERO_VISCOSITY 1
#endif
constexpr bool kSkipZeroViscosity = SPHG_SKIP_ZERO_VISCOSITY != 0;


template <int PREC, bool BATCHED, int MODE, bool CSR>
__device__ __forceinline__ uint32_t force_one(const StepArgs& a, int64_t i, const float2* unit);

// Threads per SM the force pass is compiled for.  Split precision: 1,152
// (nine 128-thread blocks, 56 registers) for one instance and 1,024 (eight
// blocks, 64 registers; the instance lookup spills a few bytes) for the batched
// variants -- measured on the GB300 against 1,024 / the compiler's own 72
// registers: 29.8 against 31.7 us on the 1M dam break, 0.408 against 0.420 ms
// per batch_256 iteration.  Plain positions need more registers: 1,024 for one
// instance, the compiler's choice batched (fewer spill).
#ifndef SPHG_FORCE_THREADS_PER_SM
#define SPHG_FORCE_THREADS_PER_SM 1152
#endif
#ifndef SPHG_FORCE_BATCHED_THREADS_PER_SM
#define SPHG_FORCE_BATCHED_THREADS_PER_SM 1024
#endif
constexpr int force_threads_per_sm(int prec, bool batched) {
  return prec == 1 ? (batched ? SPHG_FORCE_BATCHED_THREADS_PER_SM : SPHG_FORCE_THREADS_PER_SM) : (batched ? 0 : 1024);
}
template <int PREC, bool BATCHED, int MODE, bool CSR>
__device__ __forceinline__ void force_slot(const StepArgs& a, int64_t i, const float2* unit);

template <int PREC, bool BATCHED, int MODE, bool CSR, int T = kThreads>

__global__ void __launch_bounds__(T, force_threads_per_sm(PREC, BATCHED) / T) step_force(StepArgs a) {
  // unit stencil offsets (c1, c2) of the tags k = 3 (c1 + 1) + (c2 + 1) of the
  // recorded neighbours: one shared-memory load per pair instead of decoding k
  __shared__ float2 unit[16];
  if (threadIdx.x < 16) {
    const int k = threadIdx.x;
    unit[k] = k < 9 ? make_float2((float)(k / 3 - 1), (float)(k % 3 - 1)) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  cudaGridDependencySynchronize();  // densities, pressures and neighbour lists of the density pass
  allow_next_kernel(a.early_next);
  force_slot<PREC, BATCHED, MODE, CSR>(a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, unit);
}

// Force pass of slot i (every thread of a warp calls it, i may be >= n): the
// forces and, in integrate mode, the update, the new key and the mover record.
template <int PREC, bool BATCHED, int MODE, bool CSR>
__device__ __forceinline__ void force_slot(const StepArgs& a, int64_t i, const float2* unit) {
  // slots of a finished served instance are skipped (no pair, no integration, no mover bit)
  const bool valid = i < a.n && (!BATCHED || inst_ref<BATCHED>(a, i).active);
  const bool track = MODE == kForceIntegrate && a.mover_mask != nullptr;
  uint32_t key = 0;
  if (valid) key = force_one<PREC, BATCHED, MODE, CSR>(a, i, unit);
  if (track) {
    // slots whose cell key changed, for the incremental re-sort: one bit per
    // slot (a warp holds 32 consecutive slots) and (key, slot) appended to the
    // mover list, one atomic per warp
    const unsigned moved = __ballot_sync(0xffffffffu, valid && key != a.keyA[i]);
    const int lane = threadIdx.x & 31;
    if (lane == 0 && i < a.n) a.mover_mask[i >> 5] = moved;  // every word of the slots, skipped ones included
    if (moved) {
      uint32_t at = 0;
      if (lane == 0) at = atomicAdd(a.mover_count, (uint32_t)__popc(moved));
      at = __shfl_sync(0xffffffffu, at, 0) + (uint32_t)__popc(moved & ((1u << lane) - 1u));
      if (((moved >> lane) & 1u) && at < (uint32_t)kMoverCap)
        a.mover_list[at] = ((unsigned long long)key << 32) | (uint32_t)i;
    }
  }
}

// Forces on particle i; in integrate mode also the update and the new key
// (returned), in force-only mode the acceleration is stored.
template <int PREC, bool BATCHED, int MODE, bool CSR>
__device__ __forceinline__ uint32_t force_one(const StepArgs& a, int64_t i, const float2* unit) {
  // one instance: a copy of the kernel-argument descriptor; batched: a reference
  typename std::conditional<BATCHED, const InstDesc&, const InstDesc>::type d = inst_ref<BATCHED>(a, i);
  const uint32_t key = a.keyA[i];
  const float2 pi = a.posA[i];
  const float4 vi = a.velpA[i];
  // one (compensated) sum per axis of every pair's pressure + viscosity (+ alpha)
  // term, both axes in paired instructions
  typename std::conditional<PREC == 1, CSum2, PSum2>::type f;
  const float h = d.h, kp = d.kp, kv = d.kv, tol2 = d.tol2;
  const float alpha_c0 = d.alpha_c0;
  const float rho_i = 1.0f / vi.w;
  const float4* __restrict__ velp = a.velpA;
  auto pair_v = [&](const float4 vj, float dx, float dy) {
    const float r2 = fmaf(dx, dx, dy * dy);
    const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
    const float r = r2 * rinv;
    const float hr = h - r;
    // viscosity (Laplacian): mu m / (rho_j pi h^6) 45 (h - r) (v_j - v_i); skipped when MU = 0 (the dam
    // breaks' artificial viscosity replaces it), a branch uniform over the instance
    float2 t = make_float2(0.f, 0.f);
    if (!kSkipZeroViscosity || kv != 0.f) {
      const float vm = kv * vj.w * hr;
      t = mul2(make_float2(vm, vm), sub2(make_float2(vj.x, vj.y), make_float2(vi.x, vi.y)));
    }
    if (r2 > tol2) {
      // pressure (spiky gradient, symmetric p / rho^2 form)
      float s = kp * (vi.z + vj.z);
      if (alpha_c0 > 0.f) {
        const float vr = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy;
        if (vr < 0.f) {
          // Monaghan: Pi_ij = -alpha c0 h vr / ((r^2 + eps h^2) rho_bar), rho_bar = (rho_i + rho_j) / 2,
          // with rho_j = 1 / w_j: 1 / (rho_i + 1 / w_j) = w_j / (rho_i w_j + 1) -- one division
          const float pij = -2.0f * alpha_c0 * h * vr * __fdividef(vj.w, (r2 + d.eps_h2) * fmaf(rho_i, vj.w, 1.0f));
          s = fmaf(d.ka, pij, s);
        }
      }
      s *= hr * hr * rinv;
      t = fma2(make_float2(s, s), make_float2(dx, dy), t);
    }
    f.add(t);
  };
  auto pair = [&](uint32_t j, float dx, float dy) { pair_v(__ldg(velp + j), dx, dy); };
  int cx, cy;
  const uint32_t cnt = CSR ? 0u : (a.nbr ? a.ncount[i] : 0xffffffffu);
  if constexpr (CSR) {
    // MPListsForceComputation::ComputeForces: the list in its order (self skipped:
    // its pressure term is excluded by r > TOL and its viscosity term is zero)
    decode_code(d, key - d.cell_base, cx, cy);
    const int64_t b = min(a.csr_offs[i], a.csr_cap), e = min(a.csr_offs[i + 1], a.csr_cap);
    for (int64_t q = b; q < e; ++q) {
      const uint32_t ent = __ldg(a.csr_idx + q);
      const uint32_t j = ent >> 5;
      if (j == (uint32_t)i) continue;
      float dx, dy;
      entry_vec<PREC>(d, pi, __ldg(a.posA + j), ent, dx, dy);
      pair(j, dx, dy);
    }
  } else if (cnt <= (uint32_t)a.nbr_slots) {  // (not CSR: the lists mode has no record)
    // the density pass recorded this particle's neighbours (stencil order)
    decode_code(d, key - d.cell_base, cx, cy);
    const size_t n = (size_t)a.n;
    // kForceBatch neighbours at a time, their gathers in flight together.  The
    // lanes of a warp all run the warp's largest count: whole batches, then
    // (SPHG_FORCE_TAIL) a batch of two and a single one for the rest; a lane's
    // missing entries are the particle itself (stencil cell 4, no shift), whose
    // pair term is exactly zero (r = 0, v_j = v_i), so the sums are the same
    // whatever the batching.
    const uint32_t wmax = __reduce_max_sync(__activemask(), cnt);
    const uint32_t self_e = ((uint32_t)i << 5) | 4u;
    auto batch = [&](auto width, uint32_t q) {
      constexpr int B = decltype(width)::value;
      uint32_t e[B];
      float2 pj[B];
      float4 vj[B];
#pragma unroll
      for (int u = 0; u < B; ++u) e[u] = q + u < cnt ? __ldg(a.nbr + (q + u) * n + i) : self_e;
#pragma unroll
      for (int u = 0; u < B; ++u) {
        pj[u] = __ldg(a.posA + (e[u] >> 5));
        vj[u] = __ldg(velp + (e[u] >> 5));
      }
#pragma unroll
      for (int u = 0; u < B; ++u) {
        float dx, dy;
        if (PREC == 1) {  // split: the offsets moved into one cell frame by the tag's stencil offset
          const float2 o = unit[e[u] & 15u];  // (c1, c2) in {-1, 0, 1}: o * cs is exact
          const float2 dxy = fma2(make_float2(-o.x, -o.y), make_float2(d.cs_x, d.cs_y), sub2(pi, pj[u]));
          dx = dxy.x;
          dy = dxy.y;
        } else {
          entry_vec<PREC>(d, pi, pj[u], e[u], dx, dy);
        }
        pair_v(vj[u], dx, dy);
      }
    };
#if SPHG_FORCE_TAIL
    uint32_t q = 0;
    for (; q + kForceBatch <= wmax; q += kForceBatch) batch(std::integral_constant<int, kForceBatch>(), q);
    if (q + 2 <= wmax) {
      batch(std::integral_constant<int, 2>(), q);
      q += 2;
    }
    if (q < wmax) batch(std::integral_constant<int, 1>(), q);
#else
    for (uint32_t q = 0; q < wmax; q += kForceBatch) batch(std::integral_constant<int, kForceBatch>(), q);
#endif
  } else {
    // more neighbours than the density pass could record (or no record): the
    // stencil walk, pairs in the walk's order
    for_each_neighbor<PREC>(a, d, key, pi, cx, cy, [&](uint32_t j, float dx, float dy, float, uint32_t) {
      if (j != (uint32_t)i) pair(j, dx, dy);
    });
  }
  const float2 acc = add2(make_float2(d.gx, d.gy), f.value());
  const float ax = acc.x, ay = acc.y;
  if (MODE == kForceOnly) {
    a.acc[i] = make_float2(ax, ay);
    return 0;
  }
  return integrate_and_key<PREC>(a, d, i, cx, cy, pi, vi, ax, ay);
}

// ---------------------------------------------------------------- the iteration in one launch
// step_fused runs re-sort (merge) -> cell ranges -> density -> forces +
// integration as four phases of ONE cooperative launch, separated by grid-wide
// barriers, instead of four kernels: for small and medium workloads the
// kernel boundaries cost as much as the work.  Every phase is the same device
// code as its stand-alone kernel (the same bits), over the blocks in a
// grid-stride loop.  Data a phase writes and a later phase of the same launch
// reads is stored past L1 (st.global.cg) and the merge reads the keys and cell
// ranges the reorder will rewrite past L1 (ld.global.cg): no SM holds a stale
// line of them.  When more than kMoverCap slots changed, the launch only
// records that (merge_decide) and the full radix sort runs, followed by the
// launch in "post" mode (ranges, density, forces).
constexpr int kBarrierSpinLimit = 1 << 22;  // about a quarter second of 64 ns sleeps

// Grid-wide barrier of a cooperative launch: bar[0] counts arrivals, bar[1] is
// the generation the last arrival advances.  Bounded: a wait that gives up
// sets *err (reported as SPHG_TIMEOUT) and lets the block go on.
__device__ __forceinline__ void grid_barrier(uint32_t* bar, uint32_t* err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t gen = atomicAdd(bar + 1, 0u);
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      int spins = 0;
      while (*(volatile uint32_t*)(bar + 1) == gen) {
        if (++spins > kBarrierSpinLimit) {
          atomicExch(err, 1u);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

template <int PREC, bool BATCHED>
__global__ void __launch_bounds__(kThreads, BATCHED ? 6 : 8) step_fused(StepArgs a, MoverArgs m, uint32_t* bar, uint32_t* err,
                                                          int post) {
  __shared__ float2 unit[16];
  if (threadIdx.x < 16) {
    const int k = threadIdx.x;
    unit[k] = k < 9 ? make_float2((float)(k / 3 - 1), (float)(k % 3 - 1)) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int64_t G = gridDim.x;
  if (!post) {
    uint32_t movers = 0;
    if (!merge_decide(m, blockIdx.x == 0 && threadIdx.x == 0, &movers)) return;  // the full sort runs instead
    const int64_t nb = (a.n + kMergeBlockSlots - 1) / kMergeBlockSlots;
    for (int64_t b = blockIdx.x; b < nb; b += G) merge_block<true>(m, b, (uint32_t)nb, movers);
    grid_barrier(bar, err);
  } else if (a.merged && *(volatile const uint32_t*)a.merged) {
    return;  // stream-launched iteration that merged: nothing left for the post launch
  }
  if (a.mover_count && blockIdx.x == 0 && threadIdx.x == 0) atomicExch(a.mover_count, 0u);
  const int64_t nr = (a.n + kThreads * kReorderSlots - 1) / (kThreads * kReorderSlots);
  for (int64_t b = blockIdx.x; b < nr; b += G) reorder_block<true>(a, b);
  grid_barrier(bar, err);
  const int64_t np = (a.n + kThreads - 1) / kThreads;
  for (int64_t b = blockIdx.x; b < np; b += G) {
    const int64_t i = b * kThreads + threadIdx.x;
    if (i < a.n) density_particle<PREC, BATCHED, false, kThreads, true>(a, i);
  }
  grid_barrier(bar, err);
  for (int64_t b = blockIdx.x; b < np; b += G)
    force_slot<PREC, BATCHED, kForceIntegrate, false>(a, b * kThreads + threadIdx.x, unit);
}

// ---------------------------------------------------------------- diagnostics
constexpr int kDiagThreads = 256;
constexpr int kDiagBatch = 4;

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Float-float arithmetic (Knuth's TwoSum, Dekker's Fast2Sum, products split
// exactly with an FMA) for the per-thread part of the diagnostics.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
struct FFSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v, float err) {
    float t, e;
    two_sum(s, v, t, e);
    s = t;
    c = __fadd_rn(c, __fadd_rn(e, err));
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// Per (chunk, instance) block.  The conservation sums (kinetic energy,
// momentum) and max |v|^2 carry the FP32 velocities' exact squares in
// float-float (FP32 pipes) through the whole reduction -- per thread, across a
// warp, the block, and the chunks -- and become FP64 only in the six final
// values; the in-domain count is decided in FP32 and redone in FP64 (out of
// line) only within a thin band of a wall; counts are integers.  Every
// reduction has a fixed shape, so the values are deterministic.
static __device__ __noinline__ bool inside_d(double x, double y, double lox, double hix, double loy, double hiy) {
  return !(x < lox || x > hix) && !(y < loy || y > hiy);
}

// One chunk's (or one warp's) partial: three float-float sums, the largest
// |v|^2 as a normalised float-float pair, two counts.  48 bytes, the size of
// six doubles per chunk of the partials buffer.
struct DiagPart {
  FFSum e2, mx, my;
  float mh, ml;
  uint32_t inside, bad, pad0, pad1;
};
static_assert(sizeof(DiagPart) == 6 * sizeof(double), "a chunk's slot of the partials buffer");

__device__ __forceinline__ void ff_add(FFSum& a, const FFSum& b) {  // a += b
  float t, e;
  two_sum(a.s, b.s, t, e);
  a.s = t;
  a.c = __fadd_rn(a.c, __fadd_rn(b.c, e));
}
__device__ __forceinline__ void part_add(DiagPart& a, const DiagPart& b) {
  ff_add(a.e2, b.e2);
  ff_add(a.mx, b.mx);
  ff_add(a.my, b.my);
  if (b.mh > a.mh || (b.mh == a.mh && b.ml > a.ml)) {
    a.mh = b.mh;
    a.ml = b.ml;
  }
  a.inside += b.inside;
  a.bad += b.bad;
}
__device__ __forceinline__ DiagPart part_shfl_down(const DiagPart& a, int o) {
  DiagPart b;
  b.e2.s = __shfl_down_sync(0xffffffffu, a.e2.s, o);
  b.e2.c = __shfl_down_sync(0xffffffffu, a.e2.c, o);
  b.mx.s = __shfl_down_sync(0xffffffffu, a.mx.s, o);
  b.mx.c = __shfl_down_sync(0xffffffffu, a.mx.c, o);
  b.my.s = __shfl_down_sync(0xffffffffu, a.my.s, o);
  b.my.c = __shfl_down_sync(0xffffffffu, a.my.c, o);
  b.mh = __shfl_down_sync(0xffffffffu, a.mh, o);
  b.ml = __shfl_down_sync(0xffffffffu, a.ml, o);
  b.inside = __shfl_down_sync(0xffffffffu, a.inside, o);
  b.bad = __shfl_down_sync(0xffffffffu, a.bad, o);
  return b;
}
// The block's sum in thread 0 (fixed shape: lanes by halving, then the warps in order).
__device__ __forceinline__ DiagPart part_block_reduce(DiagPart v, DiagPart* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part_add(v, part_shfl_down(v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 1; k < kDiagThreads / 32; ++k) part_add(v, sh[k]);
  return v;
}

// A partial written by another block of this launch (past L1).
__device__ __forceinline__ DiagPart load_part(const DiagPart* p) {
  const uint4* q = reinterpret_cast<const uint4*>(p);
  uint4 w[3] = {__ldcg(q), __ldcg(q + 1), __ldcg(q + 2)};
  DiagPart r;
  memcpy(&r, w, sizeof(r));
  return r;
}

// One launch: every (chunk, instance) block reduces its particles into a
// partial; the last block of an instance to finish (a ticket counter, reset
// by it for the next launch) reduces the instance's partials into its six
// FP64 values {E_k, max |v|^2, N inside, m sum vx, m sum vy, non-finite
// count}, written to out[inst * 6 ..] or, with a header slot, to the slot's
// array at step k -- whose index the last instance to finish then advances.
template <int PREC, bool SLOT>
__global__ void __launch_bounds__(kDiagThreads) step_diag(StepArgs a, int chunks, double* partials,
                                                          uint32_t* tickets, double* out, HeaderSlot* slot) {
  // block -> (instance, chunk): one instance: the grid's x; several: the
  // layout's table (about 4,096 particles a block for every instance, so a
  // small instance of a mixed batch is not spread over as many blocks as the
  // largest one)
  int inst = 0, chunk = blockIdx.x;
  if (a.diag_tab) {
    const uint32_t t = __ldg(a.diag_tab + blockIdx.x);
    inst = (int)(t >> 12);
    chunk = (int)(t & 4095u);
  }
  const InstDesc& d = (a.ninst == 1) ? a.d0 : a.desc[inst];
  const int64_t cnt = d.end - d.begin;
  const int ck = a.diag_tab ? diag_instance_chunks(cnt, chunks) : chunks;
  const int64_t per = (cnt + ck - 1) / ck;
  const int64_t b = d.begin + per * chunk;
  const int64_t e = min((int64_t)d.end, b + per);
  // the instance constants used per particle, in registers
  const float lo_x = d.lo_x, hi_x = d.hi_x, lo_y = d.lo_y, hi_y = d.hi_y;
  const float cs_x = d.cs_x, cs_y = d.cs_y, Lx = d.Lx, Ly = d.Ly;
  const uint32_t cell_base = d.cell_base;
  const int order = d.order, nx = d.nx;
  const float band = 1.0e-6f * fmaxf(fabsf(hi_x - lo_x), fabsf(hi_y - lo_y));
  DiagPart v = {};
  // kDiagBatch particles per thread at a time: all their loads are issued
  // before any of them is used (the rare FP64 wall test is an out-of-line call
  // the compiler cannot move loads across)
  for (int64_t i0 = b + threadIdx.x; i0 < e; i0 += (int64_t)kDiagBatch * blockDim.x) {
    float2 vb[kDiagBatch];  // (vx, vy) of velpA
    float2 pb[kDiagBatch];
    float rb[kDiagBatch];
    uint32_t kb[kDiagBatch];
#pragma unroll
    for (int u = 0; u < kDiagBatch; ++u) {
      const int64_t i = i0 + (int64_t)u * blockDim.x;
      const bool ok = i < e;
      vb[u] = ok ? reinterpret_cast<const float2*>(a.velpA)[2 * i] : make_float2(0.f, 0.f);
      pb[u] = ok ? a.posA[i] : make_float2(0.5f * (lo_x + hi_x), 0.5f * (lo_y + hi_y));
      rb[u] = ok ? a.rho[i] : 1.f;
      kb[u] = (PREC == 1 && ok) ? a.keyA[i] : cell_base;
    }
#pragma unroll
    for (int u = 0; u < kDiagBatch; ++u) {
      if (i0 + (int64_t)u * blockDim.x >= e) break;
      const float2 vel = vb[u];
      const float2 p = pb[u];
      const float rho = rb[u];
      const float p1 = vel.x * vel.x, e1 = fmaf(vel.x, vel.x, -p1);
      const float p2 = vel.y * vel.y, e2 = fmaf(vel.y, vel.y, -p2);
      v.e2.add(p1, e1);
      v.e2.add(p2, e2);
      v.mx.add(vel.x, 0.f);
      v.my.add(vel.y, 0.f);
      float h, l;
      two_sum(p1, p2, h, l);
      l += e1 + e2;
      fast_two_sum(h, l, h, l);
      if (h > v.mh || (h == v.mh && l > v.ml)) {
        v.mh = h;
        v.ml = l;
      }
      int cx = 0, cy = 0;
      const float x = p.x, y = p.y;  // position, or offset in cell (cx, cy)
      float lox = lo_x, hix = hi_x, loy = lo_y, hiy = hi_y;
      if (PREC == 1) {
        const uint32_t code = kb[u] - cell_base;
        if (order == 0) {
          cx = (int)compact1by1(code);
          cy = (int)compact1by1(code >> 1);
        } else {
          cx = (int)(code % (uint32_t)nx);
          cy = (int)(code / (uint32_t)nx);
        }
        lox = -(float)cx * cs_x;  // the walls in the cell's frame
        hix = Lx - (float)cx * cs_x;
        loy = -(float)cy * cs_y;
        hiy = Ly - (float)cy * cs_y;
      }
      const bool fin = isfinite(x) && isfinite(y) && isfinite(vel.x) && isfinite(vel.y) && isfinite(rho);
      bool in = fin && x >= lox && x <= hix && y >= loy && y <= hiy;
      const bool near = fin && (fabsf(x - lox) <= band || fabsf(x - hix) <= band || fabsf(y - loy) <= band ||
                                fabsf(y - hiy) <= band);
      if (near) {
        const double xd = PREC == 1 ? d.lo_xd + cx * d.cs_xd + (double)x : (double)x;
        const double yd = PREC == 1 ? d.lo_yd + cy * d.cs_yd + (double)y : (double)y;
        in = inside_d(xd, yd, d.lo_xd, d.hi_xd, d.lo_yd, d.hi_yd);
      }
      v.inside += in ? 1u : 0u;
      v.bad += fin ? 0u : 1u;
    }
  }
  __shared__ DiagPart sh[kDiagThreads / 32];
  __shared__ bool last;
  v = part_block_reduce(v, sh);
  DiagPart* parts = reinterpret_cast<DiagPart*>(partials) + (size_t)inst * chunks;
  if (threadIdx.x == 0) {
    parts[chunk] = v;
    __threadfence();
    last = atomicAdd(tickets + inst, 1u) == (uint32_t)ck - 1u;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  DiagPart f = {};
  for (int c = threadIdx.x; c < ck; c += blockDim.x) part_add(f, load_part(parts + c));
  f = part_block_reduce(f, sh);
  if (threadIdx.x != 0) return;
  tickets[inst] = 0;
  const double m = d.mass_d;
  const double r[6] = {0.5 * m * f.e2.value(), (double)f.mh + (double)f.ml, (double)f.inside, m * f.mx.value(),
                       m * f.my.value(), (double)f.bad};
  if (!SLOT) {
    for (int q = 0; q < 6; ++q) out[inst * 6 + q] = r[q];
    return;
  }
  const size_t k = *(volatile uint32_t*)&slot->k;
  for (int q = 0; q < 6; ++q) slot->out[(k * a.ninst + inst) * 6 + q] = r[q];
  __threadfence();
  if (atomicAdd(&slot->done, 1u) == (uint32_t)a.ninst - 1u) {
    slot->done = 0;
    slot->k += 1;
    __threadfence();
  }
}

// CFL inputs per (chunk, instance): FP64 maxima of |v|^2 and |a|^2 (a from the
// force-only pass), reduced over chunks by step_cfl_final.
__global__ void __launch_bounds__(kDiagThreads) step_cfl_partial(StepArgs a, int chunks, double* partials) {
  const int inst = blockIdx.y;
  const InstDesc d = (a.ninst == 1) ? a.d0 : a.desc[inst];
  const int64_t cnt = d.end - d.begin;
  const int64_t per = (cnt + chunks - 1) / chunks;
  const int64_t b = d.begin + per * blockIdx.x;
  const int64_t e = min((int64_t)d.end, b + per);
  double v2 = 0.0, a2 = 0.0;
  for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    const float4 v = a.velpA[i];
    const float2 f = a.acc[i];
    v2 = fmax(v2, (double)v.x * v.x + (double)v.y * v.y);
    a2 = fmax(a2, (double)f.x * f.x + (double)f.y * f.y);
  }
  v2 = warp_max(v2);
  a2 = warp_max(a2);
  __shared__ double sh[2][kDiagThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][w] = v2;
    sh[1][w] = a2;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double m = 0.0;
    for (int k = 0; k < kDiagThreads / 32; ++k) m = fmax(m, sh[threadIdx.x][k]);
    partials[((size_t)inst * chunks + blockIdx.x) * 6 + threadIdx.x] = m;
  }
}

__global__ void step_cfl_final(int ninst, int chunks, const double* partials, double* out) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= ninst) return;
  double v2 = 0.0, a2 = 0.0;
  for (int c = 0; c < chunks; ++c) {
    v2 = fmax(v2, partials[((size_t)inst * chunks + c) * 6]);
    a2 = fmax(a2, partials[((size_t)inst * chunks + c) * 6 + 1]);
  }
  out[inst * 6] = v2;
  out[inst * 6 + 1] = a2;
}

// ---------------------------------------------------------------- stand-alone keys
__global__ void cell_keys_plain(InstDesc d, const float* __restrict__ x,
                                const float* __restrict__ y, int64_t n, int32_t* keys) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int cmx = d.periodic ? d.nxr - 1 : d.nx - 1;
  const int cmy = d.periodic ? d.nyr - 1 : d.ny - 1;
  int cx = cell_coord(x[i], d.lo_x, d.inv_cs_x, d.lo_xd, d.cs_xd, cmx);
  int cy = cell_coord(y[i], d.lo_y, d.inv_cs_y, d.lo_yd, d.cs_yd, cmy);
  keys[i] = (int32_t)local_code(d, cx, cy);
}

// ---------------------------------------------------------------- launchers
static inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

#define SPHG_DISPATCH2(PREC_RT, BATCH_RT, KERNEL, ...)                      \
  do {                                                                    \
    if (PREC_RT) {                                                        \
      if (BATCH_RT) KERNEL<1, true __VA_ARGS__><<<g, kThreads, 0, s>>>(a); \
      else KERNEL<1, false __VA_ARGS__><<<g, kThreads, 0, s>>>(a);        \
    } else {                                                              \
      if (BATCH_RT) KERNEL<0, true __VA_ARGS__><<<g, kThreads, 0, s>>>(a); \
      else KERNEL<0, false __VA_ARGS__><<<g, kThreads, 0, s>>>(a);        \
    }                                                                     \
  } while (0)

// The same with programmatic dependent launch (the kernel synchronises on its
// predecessor's grid itself).
#define SPHG_DISPATCH2_PDL(PREC_RT, BATCH_RT, KERNEL, ...)                                   \
  do {                                                                                      \
    cudaError_t e_ = cudaSuccess;                                                           \
    if (PREC_RT) {                                                                          \
      if (BATCH_RT) e_ = launch_pdl(KERNEL<1, true __VA_ARGS__>, dim3(g), dim3(kThreads), 0, s, a);  \
      else e_ = launch_pdl(KERNEL<1, false __VA_ARGS__>, dim3(g), dim3(kThreads), 0, s, a);          \
    } else {                                                                                \
      if (BATCH_RT) e_ = launch_pdl(KERNEL<0, true __VA_ARGS__>, dim3(g), dim3(kThreads), 0, s, a);  \
      else e_ = launch_pdl(KERNEL<0, false __VA_ARGS__>, dim3(g), dim3(kThreads), 0, s, a);          \
    }                                                                                       \
    if (e_ != cudaSuccess) return e_;                                                       \
  } while (0)

cudaError_t launch_keys(const StepArgs& a, int precision, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const unsigned g = blocks_for(a.n, kThreads);
  SPHG_DISPATCH2(precision, (a.ninst > 1 || a.force_batched), step_keys);
  return cudaGetLastError();
}

cudaError_t launch_reorder(const StepArgs& a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  cudaError_t e = launch_pdl(step_reorder, dim3(blocks_for(a.n, kThreads * kReorderSlots)), dim3(kThreads), 0, s, a);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// The sorted-mode density pass with T-thread blocks: two particles of a cell
// per thread (pairs) or one.
template <int T>
static cudaError_t density_sorted(const StepArgs& a, int precision, bool b, bool pairs, cudaStream_t s) {
  if (pairs) {
    const dim3 g(blocks_for(a.n, 2 * T)), t(T);
    if (precision) return b ? launch_pdl(step_density_pairs<1, true, T>, g, t, 0, s, a)
                            : launch_pdl(step_density_pairs<1, false, T>, g, t, 0, s, a);
    return b ? launch_pdl(step_density_pairs<0, true, T>, g, t, 0, s, a)
             : launch_pdl(step_density_pairs<0, false, T>, g, t, 0, s, a);
  }
  const dim3 g(blocks_for(a.n, T)), t(T);
  if (precision) return b ? launch_pdl(step_density<1, true, false, T>, g, t, 0, s, a)
                          : launch_pdl(step_density<1, false, false, T>, g, t, 0, s, a);
  return b ? launch_pdl(step_density<0, true, false, T>, g, t, 0, s, a)
           : launch_pdl(step_density<0, false, false, T>, g, t, 0, s, a);
}

cudaError_t launch_density(const StepArgs& a, int precision, cudaStream_t s, bool csr) {
  if (a.n == 0) return cudaSuccess;
  const bool b = (a.ninst > 1 || a.force_batched);
  cudaError_t e;
  if (csr) {
    const unsigned g = blocks_for(a.n, kThreads);
    SPHG_DISPATCH2(precision, b, step_density, , true);
    return cudaGetLastError();
  }
  // the pairs kernel needs the neighbour record (below 2^27 particles)
  const bool pairs = a.cell_pairs && a.n < ((int64_t)1 << 27);
  switch (a.block) {
    case 64: e = density_sorted<64>(a, precision, b, pairs, s); break;
    case 256: e = density_sorted<256>(a, precision, b, pairs, s); break;
    default: e = density_sorted<kThreads>(a, precision, b, pairs, s); break;
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// The sorted-mode force + integration pass with T-thread blocks.
template <int T>
static cudaError_t force_sorted(const StepArgs& a, int precision, bool b, cudaStream_t s) {
  const dim3 g(blocks_for(a.n, T)), t(T);
  if (precision) return b ? launch_pdl(step_force<1, true, kForceIntegrate, false, T>, g, t, 0, s, a)
                          : launch_pdl(step_force<1, false, kForceIntegrate, false, T>, g, t, 0, s, a);
  return b ? launch_pdl(step_force<0, true, kForceIntegrate, false, T>, g, t, 0, s, a)
           : launch_pdl(step_force<0, false, kForceIntegrate, false, T>, g, t, 0, s, a);
}

cudaError_t launch_force(const StepArgs& a, int precision, int mode, cudaStream_t s, bool csr) {
  if (a.n == 0) return cudaSuccess;
  const unsigned g = blocks_for(a.n, kThreads);
  const bool b = (a.ninst > 1 || a.force_batched);
  if (csr) {
    if (mode == kForceOnly) SPHG_DISPATCH2(precision, b, step_force, , kForceOnly, true);
    else SPHG_DISPATCH2(precision, b, step_force, , kForceIntegrate, true);
  } else if (mode == kForceOnly) {
    SPHG_DISPATCH2(precision, b, step_force, , kForceOnly, false);
  } else {
    cudaError_t e;
    switch (a.block) {
      case 64: e = force_sorted<64>(a, precision, b, s); break;
      case 256: e = force_sorted<256>(a, precision, b, s); break;
      default: e = force_sorted<kThreads>(a, precision, b, s); break;
    }
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

int diag_chunks(int64_t max_inst_n, int ninst, int cap) {
  int64_t c;
  if (ninst > 1) {
    c = (max_inst_n + 4095) / 4096;  // about 16 particles per thread (diag_instance_chunks)
  } else {
    // one instance: two blocks per SM, all resident at once and equally loaded
    static const int sms = [] {
      int dev = 0, v = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        v = 152;
      }
      return v;
    }();
    c = std::min<int64_t>((max_inst_n + 255) / 256, 2 * (int64_t)sms);
  }
  if (c < 1) c = 1;
  if (c > cap) c = cap;
  return (int)c;
}

cudaError_t launch_diagnostics(const StepArgs& a, int precision, double* partials, uint32_t* tickets, int chunks,
                               double* out, cudaStream_t s) {
  const dim3 g = a.diag_tab ? dim3(a.diag_blocks) : dim3(chunks, a.ninst);
  if (precision) step_diag<1, false><<<g, kDiagThreads, 0, s>>>(a, chunks, partials, tickets, out, nullptr);
  else step_diag<0, false><<<g, kDiagThreads, 0, s>>>(a, chunks, partials, tickets, out, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_diagnostics_slot(const StepArgs& a, int precision, double* partials, uint32_t* tickets,
                                    int chunks, HeaderSlot* slot, cudaStream_t s) {
  const dim3 g = a.diag_tab ? dim3(a.diag_blocks) : dim3(chunks, a.ninst);
  if (precision) step_diag<1, true><<<g, kDiagThreads, 0, s>>>(a, chunks, partials, tickets, nullptr, slot);
  else step_diag<0, true><<<g, kDiagThreads, 0, s>>>(a, chunks, partials, tickets, nullptr, slot);
  return cudaGetLastError();
}

cudaError_t launch_cfl(const StepArgs& a, double* partials, int chunks, double* out, cudaStream_t s) {
  dim3 g(chunks, a.ninst);
  step_cfl_partial<<<g, kDiagThreads, 0, s>>>(a, chunks, partials);
  step_cfl_final<<<blocks_for(a.ninst, 128), 128, 0, s>>>(a.ninst, chunks, partials, out);
  return cudaGetLastError();
}

cudaError_t launch_cell_keys_plain(const InstDesc& d, const float* x, const float* y, int64_t n,
                                   int32_t* keys, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cell_keys_plain<<<blocks_for(n, kThreads), kThreads, 0, s>>>(d, x, y, n, keys);
  return cudaGetLastError();
}

// Co-resident blocks of step_fused (0: it cannot be launched cooperatively).
template <int PREC, bool BATCHED>
static int fused_max_blocks() {
  static int cached = -1;
  if (cached >= 0) return cached;
  int dev = 0, sms = 0, per = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, step_fused<PREC, BATCHED>, kThreads, 0) != cudaSuccess) {
    cudaGetLastError();
    return cached = 0;
  }
  return cached = per * sms;
}

int fused_blocks(const StepArgs& a, int precision) {
  const bool b = (a.ninst > 1 || a.force_batched);
  const int mx = precision ? (b ? fused_max_blocks<1, true>() : fused_max_blocks<1, false>())
                           : (b ? fused_max_blocks<0, true>() : fused_max_blocks<0, false>());
  const int64_t need = (a.n + kThreads - 1) / kThreads;
  return (int)std::min<int64_t>(mx, std::max<int64_t>(need, 1));
}

cudaError_t launch_fused(const StepArgs& a, const MoverArgs& m, int precision, uint32_t* bar, uint32_t* err, bool post,
                         cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const int g = fused_blocks(a, precision);
  if (g <= 0) return cudaErrorNotSupported;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g);
  cfg.blockDim = dim3(kThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const bool b = (a.ninst > 1 || a.force_batched);
  const int p = post ? 1 : 0;
  cudaError_t e;
  if (precision) e = b ? cudaLaunchKernelEx(&cfg, step_fused<1, true>, a, m, bar, err, p)
                       : cudaLaunchKernelEx(&cfg, step_fused<1, false>, a, m, bar, err, p);
  else e = b ? cudaLaunchKernelEx(&cfg, step_fused<0, true>, a, m, bar, err, p)
             : cudaLaunchKernelEx(&cfg, step_fused<0, false>, a, m, bar, err, p);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace sphg
