// sphg_tiled.cu -- cell-tile density and force kernels (Morton order).
//
// A tile is an aligned 2^TB x 2^TB block of cells.  In Morton order its keys
// are one contiguous range, so its particles are one contiguous run of the
// sorted arrays.  One CTA per non-empty tile:
//   1. looks up the particle ranges of the (2^TB + 2)^2 cells of the tile and
//      its one-cell halo (one range-table load per cell, all cells in parallel);
//   2. copies the tile's own particles (one coalesced copy of the run) and the
//      halo cells' particles into shared memory;
//   3. sweeps every particle of the tile against its 3x3 stencil in shared
//      memory, in the reference's order (x offset outer, y offset inner, j
//      ascending; GenericForceComputation.tpp:56-70 / :160-200).
// The force kernel also integrates the particle (Integrator.cpp:7-46) and
// computes the cell key of the integrated position for the next sort
// (GenericNeighborSearch.h:201-231), so no separate key pass is needed.
// Tiles whose staged particles exceed the shared-memory capacity fall back to
// the global-memory stencil walk of sphg_neighbor.cuh for their particles.
#include <cstdint>
#include <type_traits>

#include <cuda_runtime.h>

#include "sphg_neighbor.cuh"
#include "sphg_step.cuh"

namespace sphg {

constexpr int kTileThreads = 256;

struct TileFrame {
  int cx0, cy0;  // first cell of the tile
};

// Frame cell (u, v) of a tile -> global cell, or false when no particle of the
// tile can have it in its stencil (outside the grid / beyond the periodic wrap).
__device__ __forceinline__ bool frame_cell(const InstDesc& d, int gx, int gy, int& ox, int& oy,
                                           int& wrapx, int& wrapy) {
  wrapx = wrapy = 0;
  if (d.periodic) {
    if (gx == -1) { gx = d.nxr - 1; wrapx = 1; }
    else if (gx == d.nxr) { gx = 0; wrapx = -1; }
    else if (gx < -1 || gx > d.nxr) return false;
    if (gy == -1) { gy = d.nyr - 1; wrapy = 1; }
    else if (gy == d.nyr) { gy = 0; wrapy = -1; }
    else if (gy < -1 || gy > d.nyr) return false;
  } else {
    if (gx < 0 || gx >= d.nx || gy < 0 || gy >= d.ny) return false;
  }
  ox = gx;
  oy = gy;
  return true;
}

// Block-wide exclusive scan of one value per thread (blockDim.x == kTileThreads).
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t* wsum, uint32_t& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < kTileThreads / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kTileThreads / 32) wsum[lane] = t;
  }
  __syncthreads();
  total = wsum[kTileThreads / 32 - 1];
  uint32_t r = (w ? wsum[w - 1] : 0) + x - v;
  __syncthreads();
  return r;
}

template <int PREC, bool BATCHED, bool FORCE, int TB>
__global__ void __launch_bounds__(kTileThreads) tile_kernel(StepArgs a) {
  constexpr int TW = 1 << TB;
  constexpr int FW = TW + 2;
  constexpr int NF = FW * FW;
  constexpr int RPT = (NF + kTileThreads - 1) / kTileThreads;  // frame cells per thread
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t* fstart = reinterpret_cast<uint32_t*>(smem_raw);  // [NF] staging start
  uint32_t* fcount = fstart + NF;                             // [NF] particles
  uint32_t* fglob = fcount + NF;                              // [NF] global start
  uint32_t* hpre = fglob + NF;                                // [NF] halo prefix (frame order)
  int8_t* fwrap = reinterpret_cast<int8_t*>(hpre + NF);       // [NF] reached through the periodic wrap
  __shared__ uint32_t wsum[32];
  const int cap = a.tile_cap;
  float2* spos = reinterpret_cast<float2*>(smem_raw + (((size_t)NF * 17 + 15) & ~(size_t)15));
  float4* svel = reinterpret_cast<float4*>(spos + cap);

  const uint32_t ntiles = *a.tile_count;
  const uint32_t ep = *a.epoch;
  for (uint32_t tt = blockIdx.x; tt < ntiles; tt += gridDim.x) {
    const uint32_t T = a.tile_list[tt];
    const uint2 tr = a.tile_ranges[T];
    const uint32_t ts = tr.x;
    const uint32_t n_int = tr.y - tr.x;
    const InstDesc d = BATCHED ? a.desc[find_instance(a.begins, a.ninst, (int)ts)] : a.d0;
    int cx0, cy0;
    decode_code(d, (T << (2 * TB)) - d.cell_base, cx0, cy0);

    // 1. range entries of the tile and its halo, all frame cells at once
    uint32_t halo_cnt[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const int f = r * kTileThreads + threadIdx.x;
      halo_cnt[r] = 0;
      if (f < NF) {
        const int u = f % FW, v = f / FW;
        int gx, gy, wx, wy;
        uint32_t cnt = 0, gs = 0;
        if (frame_cell(d, cx0 - 1 + u, cy0 - 1 + v, gx, gy, wx, wy)) {
          const uint4 e = __ldg(a.ranges + d.cell_base + local_code(d, gx, gy));
          if (e.z == ep) {
            cnt = e.y - e.x;
            gs = e.x;
          }
        }
        const bool interior = (wx == 0 && wy == 0) && u >= 1 && u <= TW && v >= 1 && v <= TW;
        fcount[f] = cnt;
        fglob[f] = gs;
        fwrap[f] = (int8_t)((wx != 0) || (wy != 0));
        if (interior) fstart[f] = gs - ts;
        else halo_cnt[r] = cnt;
      }
    }
    uint32_t halo_sum = 0;
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      uint32_t tot;
      const uint32_t pre = block_scan_excl(halo_cnt[r], wsum, tot) + halo_sum;
      const int f = r * kTileThreads + threadIdx.x;
      if (f < NF) {
        hpre[f] = pre;
        if (halo_cnt[r]) fstart[f] = n_int + pre;
      }
      halo_sum += tot;
    }
    const bool staged = (n_int + halo_sum) <= (uint32_t)cap;
    __syncthreads();

    if (staged) {
      // 2. stage the tile's run and the halo particles (one flat pass each)
      for (uint32_t k = threadIdx.x; k < n_int; k += kTileThreads) {
        spos[k] = __ldg(a.posA + ts + k);
        if (FORCE) svel[k] = __ldg(a.velpA + ts + k);
      }
      for (uint32_t hq = threadIdx.x; hq < halo_sum; hq += kTileThreads) {
        int lo = 0, hi = NF - 1;  // last frame cell with hpre <= hq
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (hpre[mid] <= hq) lo = mid; else hi = mid - 1;
        }
        const uint32_t g = fglob[lo] + (hq - hpre[lo]);
        spos[n_int + hq] = __ldg(a.posA + g);
        if (FORCE) svel[n_int + hq] = __ldg(a.velpA + g);
      }
      __syncthreads();
    }

    // 3. sweep the tile's particles
    for (uint32_t k = threadIdx.x; k < n_int; k += kTileThreads) {
      const uint32_t i = ts + k;
      const uint32_t key = a.keyA[i];
      int cx, cy;
      decode_code(d, key - d.cell_base, cx, cy);
      const float2 pi = staged ? spos[k] : a.posA[i];
      float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
      if (FORCE) vi = staged ? svel[k] : a.velpA[i];
      typedef typename std::conditional<PREC == 1, CSum, PSum>::type Sum;
      Sum S, fpx, fpy, fvx, fvy, fax, fay;
      const float inv_h2 = d.inv_h2, h = d.h, kp = d.kp, kv = d.kv, tol2 = d.tol2;
      const float alpha_c0 = d.alpha_c0;
      auto visit = [&](float dx, float dy, float r2, float4 vj, bool self) {
        if (!FORCE) {
          const float t = fmaf(-r2, inv_h2, 1.0f);
          S.add(t * t * t);
          return;
        }
        if (self) return;
        const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
        const float r = r2 * rinv;
        const float hr = h - r;
        if (r2 > tol2) {
          const float s = kp * hr * hr * rinv * (vi.z + vj.z);
          fpx.add(s * dx);
          fpy.add(s * dy);
        }
        const float vm = kv * vj.w * hr;
        fvx.add(vm * (vj.x - vi.x));
        fvy.add(vm * (vj.y - vi.y));
        if (alpha_c0 > 0.f && r2 > tol2) {
          const float vr = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy;
          if (vr < 0.f) {
            const float muij = h * vr / (r2 + d.eps_h2);
            const float rho_bar = 0.5f * (1.0f / vi.w + 1.0f / vj.w);
            const float pij = -alpha_c0 * muij / rho_bar;
            const float s = d.ka * hr * hr * rinv * pij;
            fax.add(s * dx);
            fay.add(s * dy);
          }
        }
      };
      if (staged) {
        const int lx = cx - cx0, ly = cy - cy0;
#pragma unroll 1
        for (int k9 = 0; k9 < 9; ++k9) {
          const int c1 = k9 / 3 - 1, c2 = k9 % 3 - 1;
          const int f = (lx + 1 + c1) + FW * (ly + 1 + c2);
          const uint32_t cnt = fcount[f];
          if (cnt == 0) continue;
          const uint32_t s0 = fstart[f];
          const bool wrapped = (PREC == 0) && fwrap[f];
          const float shx = (PREC == 1) ? (c1 == 0 ? 0.f : (c1 > 0 ? d.cs_x : -d.cs_x)) : 0.f;
          const float shy = (PREC == 1) ? (c2 == 0 ? 0.f : (c2 > 0 ? d.cs_y : -d.cs_y)) : 0.f;
          for (uint32_t q = s0; q < s0 + cnt; ++q) {
            const float2 pj = spos[q];
            float dx = (pi.x - pj.x) - shx;
            float dy = (pi.y - pj.y) - shy;
            if (!wrapped) {
              const float r2 = fmaf(dx, dx, dy * dy);
              if (pair_inside<PREC>(d, pi, pj, c1, c2, r2)) visit(dx, dy, r2, FORCE ? svel[q] : vi, q == k);
            } else if (wrapped_pair(d, pi, pj, dx, dy)) {
              visit(dx, dy, fmaf(dx, dx, dy * dy), FORCE ? svel[q] : vi, q == k);
            }
          }
        }
      } else {
        int ccx, ccy;
        for_each_neighbor<PREC>(a, d, key, pi, ccx, ccy, [&](uint32_t j, float dx, float dy, float r2, uint32_t) {
          visit(dx, dy, r2, FORCE ? __ldg(a.velpA + j) : vi, j == i);
        });
      }

      if (!FORCE) {
        float rho, drho;
        if constexpr (PREC == 1) {
          rho = d.wd * S.value();
          drho = fmaf(d.wd, S.s, -d.rho0) + d.wd * S.c;
        } else {
          rho = d.wd * S.value();
          drho = rho - d.rho0;
        }
        const float inv = 1.0f / rho;
        a.rho[i] = rho;
        reinterpret_cast<float2*>(a.velpA + i)[1] = make_float2(d.k * drho * inv * inv, inv);
        continue;
      }
      float ax = d.gx + fpx.value();
      float ay = d.gy + fpy.value();
      ax += fvx.value();
      ay += fvy.value();
      if (alpha_c0 > 0.f) {
        ax += fax.value();
        ay += fay.value();
      }
      integrate_and_key<PREC>(a, d, i, cx, cy, pi, vi, ax, ay);
    }
    __syncthreads();  // the staging buffers are reused by the next tile
  }
}

size_t tile_smem_bytes(int tb, int cap, bool force) {
  const int fw = (1 << tb) + 2, nf = fw * fw;
  size_t head = ((size_t)nf * 17 + 15) & ~(size_t)15;
  return head + (size_t)cap * (force ? (8 + 16) : 8);
}

template <int PREC, bool BATCHED, bool FORCE, int TB>
static cudaError_t launch_tiles_t(const StepArgs& a, cudaStream_t s) {
  const size_t smem = tile_smem_bytes(TB, a.tile_cap, FORCE);
  auto k = tile_kernel<PREC, BATCHED, FORCE, TB>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.tile_grid, kTileThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <bool FORCE, int TB>
static cudaError_t launch_tiles_tb(const StepArgs& a, int precision, cudaStream_t s) {
  const bool b = (a.ninst > 1 || a.force_batched);
  if (precision) return b ? launch_tiles_t<1, true, FORCE, TB>(a, s) : launch_tiles_t<1, false, FORCE, TB>(a, s);
  return b ? launch_tiles_t<0, true, FORCE, TB>(a, s) : launch_tiles_t<0, false, FORCE, TB>(a, s);
}

cudaError_t launch_tiled(const StepArgs& a, int precision, bool force, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  switch (a.tile_bits) {
    case 3: return force ? launch_tiles_tb<true, 3>(a, precision, s) : launch_tiles_tb<false, 3>(a, precision, s);
    case 4: return force ? launch_tiles_tb<true, 4>(a, precision, s) : launch_tiles_tb<false, 4>(a, precision, s);
    case 5: return force ? launch_tiles_tb<true, 5>(a, precision, s) : launch_tiles_tb<false, 5>(a, precision, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sphg
