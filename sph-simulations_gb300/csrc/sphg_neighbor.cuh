// sphg_neighbor.cuh -- the 3x3 cell-stencil neighbour walk shared by the
// density, force and neighbour-list kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sphg_common.cuh"
#include "sphg_step.cuh"

namespace sphg {

// Constants of the instance owning slot i (by value so they live in registers).
template <bool BATCHED>
__device__ __forceinline__ InstDesc inst_of(const StepArgs& a, int64_t i) {
  if (!BATCHED) return a.d0;
  return a.desc[find_instance(a.begins, a.ninst, (int)i)];
}

// ---------------------------------------------------------------- neighbour walk
// Visits every j with |x_i - x_j| <= h in the reference's stencil order
// (x offset outer, y offset inner, j ascending; GenericForceComputation.tpp:56-70),
// calling visit(j, dx, dy, r2) with dx = x_i - x_j.
template <int PREC, class F>
__device__ __forceinline__ void for_each_neighbor(const StepArgs& a, const InstDesc& d,
                                                  uint32_t key, float2 pi, int& cx, int& cy,
                                                  F&& visit) {
  decode_code(d, key - d.cell_base, cx, cy);
  const uint32_t n = (uint32_t)a.n;
  const uint2* __restrict__ ranges = a.ranges;
  const uint32_t* __restrict__ keys = a.keyA;
  const float2* __restrict__ pos = a.posA;
#pragma unroll 1
  for (int c1 = -1; c1 <= 1; ++c1) {
    int jx = cx + c1;
    bool wx = false;
    if (d.periodic) {
      if (jx < 0) { jx += d.nxr; wx = true; }
      else if (jx >= d.nxr) { jx -= d.nxr; wx = true; }
    } else if (jx < 0 || jx >= d.nx) {
      continue;
    }
#pragma unroll 1
    for (int c2 = -1; c2 <= 1; ++c2) {
      int jy = cy + c2;
      bool wy = false;
      if (d.periodic) {
        if (jy < 0) { jy += d.nyr; wy = true; }
        else if (jy >= d.nyr) { jy -= d.nyr; wy = true; }
      } else if (jy < 0 || jy >= d.ny) {
        continue;
      }
      const uint32_t c = d.cell_base + local_code(d, jx, jy);
      const uint2 r = __ldg(ranges + c);
      if (r.x >= n || __ldg(keys + r.x) != c) continue;
      const bool wrapped = (PREC == 0) && (wx || wy);
      const float shx = (PREC == 1) ? (float)c1 * d.cs_x : 0.f;
      const float shy = (PREC == 1) ? (float)c2 * d.cs_y : 0.f;
      for (uint32_t j = r.x; j < r.y; ++j) {
        const float2 pj = __ldg(pos + j);
        float dx = (pi.x - pj.x) - shx;
        float dy = (pi.y - pj.y) - shy;
        if (!wrapped) {
          const float r2 = fmaf(dx, dx, dy * dy);
          bool in;
          if (r2 < d.h2_lo) in = true;
          else if (r2 > d.h2_hi) in = false;
          else {
            double ddx = __dsub_rn(__dsub_rn((double)pi.x, (double)pj.x), (double)c1 * ((PREC == 1) ? d.cs_xd : 0.0));
            double ddy = __dsub_rn(__dsub_rn((double)pi.y, (double)pj.y), (double)c2 * ((PREC == 1) ? d.cs_yd : 0.0));
            in = exact_inside_d(ddx, ddy, d.h2_d);
          }
          if (in) visit(j, dx, dy, r2);
        } else {
          double ddx = __dsub_rn((double)pi.x, (double)pj.x);
          double ddy = __dsub_rn((double)pi.y, (double)pj.y);
          if (ddx > 0.5 * d.Lx_d) ddx -= d.Lx_d; else if (ddx < -0.5 * d.Lx_d) ddx += d.Lx_d;
          if (ddy > 0.5 * d.Ly_d) ddy -= d.Ly_d; else if (ddy < -0.5 * d.Ly_d) ddy += d.Ly_d;
          if (exact_inside_d(ddx, ddy, d.h2_d)) {
            dx = (float)ddx;
            dy = (float)ddy;
            visit(j, dx, dy, fmaf(dx, dx, dy * dy));
          }
        }
      }
    }
  }
}

}  // namespace sphg
