// sphg_neighbor.cuh -- the 3x3 cell-stencil neighbour walk and the fused
// integration epilogue shared by the density, force and neighbour-list kernels.
//
// Cell ranges: one 16-byte entry per global cell key, {start, end, epoch, 0}.
// The reorder kernel writes the entries of the occupied cells with the current
// step's epoch (bumped by the sort); an entry whose epoch is not the current
// one belongs to a cell that is empty now.  The table is never cleared.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sphg_common.cuh"
#include "sphg_step.cuh"

namespace sphg {

// Constants of the instance owning slot i (by value so they live in registers).
// Batched: the instance of the first slot of i's 256-slot block from a table
// built with the layout, then forward over the (rare) instance starts inside
// the block -- instances hold at least hundreds of slots, so one or two loads.
template <bool BATCHED>
__device__ __forceinline__ InstDesc inst_of(const StepArgs& a, int64_t i) {
  if (!BATCHED) return a.d0;
  int k = __ldg(a.inst_tab + (i >> kInstTabShift));
  while (k + 1 < a.ninst && __ldg(a.begins + k + 1) <= (int32_t)i) ++k;
  return a.desc[k];
}

// The same as a reference: batched kernels read each constant where it is used
// (L1-cached) instead of holding the whole descriptor in registers.
template <bool BATCHED>
__device__ __forceinline__ const InstDesc& inst_ref(const StepArgs& a, int64_t i) {
  if (!BATCHED) return a.d0;
  int k = __ldg(a.inst_tab + (i >> kInstTabShift));
  while (k + 1 < a.ninst && __ldg(a.begins + k + 1) <= (int32_t)i) ++k;
  return a.desc[k];
}

static __device__ __noinline__ int offset_cells_d(float o, double cs_d) {
  return (int)floor(__ddiv_rn((double)o, cs_d));
}

// Offset o moved k cells: o - k cs in FP64, rounded to FP32 and kept inside
// [0, cs) of the FP64 cell size (a rounding up to cs is stepped back one ulp),
// so the reconstructed position lo + c cs + o stays in cell c.  Out of line:
// runs only for particles that changed cell.
static __device__ __noinline__ float offset_shift_d(float o, int k, double cs_d) {
  float r = __double2float_rn(__dsub_rn((double)o, (double)k * cs_d));
  if ((double)r >= cs_d) r = nextafterf(r, 0.0f);
  return r;
}

// floor(o / cs) for a split-precision offset, FP64 near integer boundaries.
// |q| < 1/2 (an offset at or near the cell's low edge, e.g. a particle resting
// on a wall) is decided by the sign alone: o / cs lies in (-1, 1), so the FP64
// floor is 0 for o >= 0 and -1 for o < 0.
__device__ __forceinline__ int offset_cells(float o, float inv_cs, double cs_d) {
  float q = o * inv_cs;
  float fq = floorf(q);
  float fr = q - fq;
  if (fr > 1.0e-6f && fr < 1.0f - 1.0e-6f && fabsf(q) < 1.0e6f) return (int)fq;
  if (fabsf(q) < 0.5f) return o < 0.0f ? -1 : 0;
  if (!(fabsf(q) < 1.0e6f)) return 0;  // NaN / runaway: keep the cell; diagnostics flag the state
  return offset_cells_d(o, cs_d);
}

// Stencil cell (cx + c1, cy + c2) -> global key, with the wall bounds of the
// reference (padded Morton grid) or the periodic wrap.  wrap is set when the
// cell was reached through the periodic boundary.
__device__ __forceinline__ bool stencil_cell(const InstDesc& d, int cx, int cy, int c1, int c2,
                                             uint32_t& c, bool& wrap) {
  int jx = cx + c1, jy = cy + c2;
  wrap = false;
  if (d.periodic) {
    if (jx < 0) { jx += d.nxr; wrap = true; }
    else if (jx >= d.nxr) { jx -= d.nxr; wrap = true; }
    if (jy < 0) { jy += d.nyr; wrap = true; }
    else if (jy >= d.nyr) { jy -= d.nyr; wrap = true; }
  } else if (jx < 0 || jx >= d.nx || jy < 0 || jy >= d.ny) {
    return false;
  }
  c = d.cell_base + local_code(d, jx, jy);
  return true;
}

// FP64 test of the reference on one pair: dx = (xi - xj) - sx in FP64, where sx
// is the stencil offset of j's cell in split precision (0, +cs or -cs; chosen,
// never multiplied).  Kept out of line so nothing of it is hoisted into the
// FP32 hot loops (FP64 issues at 1/64 of the FP32 rate).
static __device__ __noinline__ bool pair_inside_d(float xi, float yi, float xj, float yj,
                                                  double sx, double sy, double h2_d) {
  const double ddx = __dsub_rn(__dsub_rn((double)xi, (double)xj), sx);
  const double ddy = __dsub_rn(__dsub_rn((double)yi, (double)yj), sy);
  return exact_inside_d(ddx, ddy, h2_d);
}

// Pair test of the reference, r2 <= h2 in FP64, decided in FP32 outside a thin
// band around h^2.  (c1, c2) is the stencil offset of j's cell.
template <int PREC>
__device__ __forceinline__ bool pair_inside(const InstDesc& d, float2 pi, float2 pj, int c1,
                                            int c2, float r2) {
  if (r2 < d.h2_lo) return true;
  if (r2 > d.h2_hi) return false;
  double sx = 0.0, sy = 0.0;
  if (PREC == 1) {
    sx = c1 == 0 ? 0.0 : (c1 > 0 ? d.cs_xd : -d.cs_xd);
    sy = c2 == 0 ? 0.0 : (c2 > 0 ? d.cs_yd : -d.cs_yd);
  }
  return pair_inside_d(pi.x, pi.y, pj.x, pj.y, sx, sy, d.h2_d);
}

// Plain positions reached through the periodic boundary: minimum image in FP64
// (out of line, no FP64 multiply, so nothing is hoisted into the hot loops).
static __device__ __noinline__ bool wrapped_pair_d(float xi, float yi, float xj, float yj,
                                                   double Lx, double Ly, double hLx, double hLy,
                                                   double h2_d, float* dx, float* dy) {
  double ddx = __dsub_rn((double)xi, (double)xj);
  double ddy = __dsub_rn((double)yi, (double)yj);
  if (ddx > hLx) ddx = __dsub_rn(ddx, Lx); else if (ddx < -hLx) ddx = __dadd_rn(ddx, Lx);
  if (ddy > hLy) ddy = __dsub_rn(ddy, Ly); else if (ddy < -hLy) ddy = __dadd_rn(ddy, Ly);
  if (!exact_inside_d(ddx, ddy, h2_d)) return false;
  *dx = (float)ddx;
  *dy = (float)ddy;
  return true;
}

// x_i - x_j by the minimum image of one periodic axis of length L (FP32 exact,
// positions in [0, L)): the FP64 computation's value rounded to FP32, from FP32
// operations.  Valid when the wrap decision is clear of |d| = L/2 and the
// operand near 0 is 0 or at least 2^-28 L: the FP64 result is then exact, the
// operand near L minus L is exact (Sterbenz), and one FP32 operation rounds the
// exact value.  false: leave it to FP64.
__device__ __forceinline__ bool min_image_f32(float xi, float xj, float L, float& out) {
  const float hL = 0.5f * L;
  const float d0 = xi - xj;  // the exact difference rounded
  const float ad = fabsf(d0);
  const float margin = 1.0e-6f * hL;  // > the rounding of d0: the same side of L/2 as the exact difference
  if (ad < hL - margin) {
    out = d0;
    return true;
  }
  if (ad <= hL + margin) return false;
  const bool down = d0 > 0.f;  // x_i near L: d - L; x_j near L: d + L
  const float near0 = down ? xj : xi, nearL = down ? xi : xj;
  if (!(near0 >= 0.f) || (near0 != 0.f && near0 < L * 0x1p-28f) || !(nearL >= hL && nearL <= 2.0f * L)) return false;
  const float t = nearL - L;  // exact
  out = down ? t - xj : xi - t;
  return true;
}

__device__ __forceinline__ bool wrapped_pair(const InstDesc& d, float2 pi, float2 pj, float& dx,
                                             float& dy) {
  if (d.wrap_f32) {
    // FP32 minimum images; the FP64 decision only inside the band around h^2
    float ex, ey;
    if (min_image_f32(pi.x, pj.x, d.Lx, ex) && min_image_f32(pi.y, pj.y, d.Ly, ey)) {
      dx = ex;
      dy = ey;
      const float r2 = fmaf(ex, ex, ey * ey);
      if (r2 < d.h2_lo) return true;
      if (r2 > d.h2_hi) return false;
    }
  }
  return wrapped_pair_d(pi.x, pi.y, pj.x, pj.y, d.Lx_d, d.Ly_d, d.half_Lx_d, d.half_Ly_d,
                        d.h2_d, &dx, &dy);
}

// ---------------------------------------------------------------- neighbour walk
// The nine stencil keys of cell (cx, cy) with code `code`, in the reference's
// order k = 3 * (c1 + 1) + (c2 + 1).  Morton neighbours come from dilated
// integer arithmetic on the code (+-1 on the interleaved x or y bits), row-major
// ones from +-1 / +-nx.  valid bit k: the cell exists; wrap bit k: reached
// through the periodic boundary.
__device__ __forceinline__ void stencil_keys(const InstDesc& d, uint32_t code, int cx, int cy,
                                             uint32_t (&c)[9], uint32_t& valid, uint32_t& wrap) {
  valid = 0;
  wrap = 0;
  // periodic, away from the wrap: the walls' stencil with every cell present
  const bool inner = d.periodic && cx > 0 && cx + 1 < d.nxr && cy > 0 && cy + 1 < d.nyr;
  if ((!d.periodic || inner) && d.order == 0) {
    const uint32_t X = code & 0x55555555u, Y = code & 0xAAAAAAAAu;
    const uint32_t xs[3] = {(X - 1u) & 0x55555555u, X, ((X | 0xAAAAAAAAu) + 1u) & 0x55555555u};
    const uint32_t ys[3] = {(Y - 1u) & 0xAAAAAAAAu, Y, ((Y | 0x55555555u) + 1u) & 0xAAAAAAAAu};
    const bool xo[3] = {cx > 0, true, cx + 1 < d.nx};
    const bool yo[3] = {cy > 0, true, cy + 1 < d.ny};
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      c[k] = d.cell_base + (xs[k / 3] | ys[k % 3]);
      if (xo[k / 3] && yo[k % 3]) valid |= 1u << k;
    }
    return;
  }
  if (!d.periodic || inner) {  // row-major
    const uint32_t base = d.cell_base + code;
    const bool xo[3] = {cx > 0, true, cx + 1 < d.nx};
    const bool yo[3] = {cy > 0, true, cy + 1 < d.ny};
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      c[k] = base + (uint32_t)((k / 3 - 1) + (k % 3 - 1) * d.nx);
      if (xo[k / 3] && yo[k % 3]) valid |= 1u << k;
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) {  // periodic: wrap each axis
    bool w;
    if (stencil_cell(d, cx, cy, k / 3 - 1, k % 3 - 1, c[k], w)) valid |= 1u << k;
    if (w) wrap |= 1u << k;
  }
}

// Visits every j with |x_i - x_j| <= h, calling visit(j, dx, dy, r2, tag) with
// dx = x_i - x_j and tag = stencil cell k (0..8, k = 3 (c1 + 1) + (c2 + 1)) plus
// 16 when the cell was reached through the periodic boundary.  The nine range entries are loaded before any particle so
// their latencies overlap.
// ORDERED: strictly the reference's stencil order (x offset outer, y offset
// inner, j ascending; GenericForceComputation.tpp:56-70), the FP64 decision
// made in place -- used where the order is part of the result (neighbour
// lists).  Otherwise pairs inside the thin FP64 band around h^2 are skipped by
// the main pass and decided by a second pass over the same cells, which keeps
// the FP64 code out of the hot loop; only the summation order of those rare
// pairs differs.
template <int PREC, bool ORDERED = false, class F>
__device__ __forceinline__ void for_each_neighbor(const StepArgs& a, const InstDesc& d,
                                                  uint32_t key, float2 pi, int& cx, int& cy,
                                                  F&& visit) {
  const uint32_t code = key - d.cell_base;
  decode_code(d, code, cx, cy);
  const uint32_t ep = *a.epoch;
  const uint4* __restrict__ ranges = a.ranges;
  const float2* __restrict__ pos = a.posA;
  uint32_t c[9], valid, wrapmask;
  stencil_keys(d, code, cx, cy, c, valid, wrapmask);
  uint32_t rs[9], re[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    rs[k] = re[k] = 0;
    if ((valid >> k) & 1u) {
      const uint4 e = __ldg(ranges + c[k]);
      if (e.z == ep) {
        rs[k] = e.x;
        re[k] = e.y;
      }
    }
  }
  bool border = false;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int c1 = k / 3 - 1, c2 = k % 3 - 1;
    const bool wrapped = (PREC == 0) && ((wrapmask >> k) & 1u);
    const float shx = (PREC == 1) ? (c1 == 0 ? 0.f : (c1 > 0 ? d.cs_x : -d.cs_x)) : 0.f;
    const float shy = (PREC == 1) ? (c2 == 0 ? 0.f : (c2 > 0 ? d.cs_y : -d.cs_y)) : 0.f;
    auto candidate = [&](uint32_t j, float2 pj) {
      float dx = (pi.x - pj.x) - shx;
      float dy = (pi.y - pj.y) - shy;
      if (wrapped) {
        if (wrapped_pair(d, pi, pj, dx, dy)) visit(j, dx, dy, fmaf(dx, dx, dy * dy), (uint32_t)k | 16u);
        return;
      }
      const float r2 = fmaf(dx, dx, dy * dy);
      if (r2 < d.h2_lo) {
        visit(j, dx, dy, r2, (uint32_t)k);
      } else if (r2 <= d.h2_hi) {
        if (ORDERED) {
          if (pair_inside<PREC>(d, pi, pj, c1, c2, r2)) visit(j, dx, dy, r2, (uint32_t)k);
        } else {
          border = true;
        }
      }
    };
    for (uint32_t j = rs[k]; j < re[k]; ++j) candidate(j, __ldg(pos + j));
  }
  if (ORDERED || !border) return;
#pragma unroll 1
  for (int k = 0; k < 9; ++k) {  // rare: pairs in the FP64 band
    if ((PREC == 0) && ((wrapmask >> k) & 1u)) continue;
    const int c1 = k / 3 - 1, c2 = k % 3 - 1;
    const float shx = (PREC == 1) ? (c1 == 0 ? 0.f : (c1 > 0 ? d.cs_x : -d.cs_x)) : 0.f;
    const float shy = (PREC == 1) ? (c2 == 0 ? 0.f : (c2 > 0 ? d.cs_y : -d.cs_y)) : 0.f;
    uint32_t s = 0, e = 0;
#pragma unroll
    for (int q = 0; q < 9; ++q)
      if (q == k) { s = rs[q]; e = re[q]; }
    for (uint32_t j = s; j < e; ++j) {
      const float2 pj = __ldg(pos + j);
      const float dx = (pi.x - pj.x) - shx;
      const float dy = (pi.y - pj.y) - shy;
      const float r2 = fmaf(dx, dx, dy * dy);
      if (r2 >= d.h2_lo && r2 <= d.h2_hi && pair_inside<PREC>(d, pi, pj, c1, c2, r2))
        visit(j, dx, dy, r2, (uint32_t)k);
    }
  }
}

// ---------------------------------------------------------------- integration epilogue
// Symplectic Euler (UpdateVelocities then UpdatePositions) with the boundary
// of Integrator::ApplyBoundaryConditions (Integrator.cpp:30-46: per axis high
// then low) or the periodic wrap, then the cell key of the new position for
// the next sort (SetParticleCellIds).  Split precision keeps the position as
// (cell, offset) and renormalises the offset into the new cell.
template <int PREC>
__device__ __forceinline__ uint32_t integrate_and_key(const StepArgs& a, const InstDesc& d, int64_t i,
                                                  int cx, int cy, float2 pi, float4 vi, float ax,
                                                  float ay) {
  const float dt = d.dt;
  const float2 v = fma2(make_float2(dt, dt), make_float2(ax, ay), make_float2(vi.x, vi.y));
  const float2 xy = fma2(make_float2(dt, dt), v, pi);
  float vx = v.x, vy = v.y;
  float x = xy.x, y = xy.y;
  if (d.periodic) {
    if (PREC == 0) {
      if (x >= d.hi_x) x -= d.Lx;
      if (x < d.lo_x) x += d.Lx;
      if (y >= d.hi_y) y -= d.Ly;
      if (y < d.lo_y) y += d.Ly;
    }
  } else {
    float whx, wlx, why, wly;  // walls in the particle's frame
    if (PREC == 0) {
      whx = d.hi_x; wlx = d.lo_x; why = d.hi_y; wly = d.lo_y;
    } else {
      whx = d.Lx - (float)cx * d.cs_x;
      wlx = -(float)cx * d.cs_x;
      why = d.Ly - (float)cy * d.cs_y;
      wly = -(float)cy * d.cs_y;
    }
    if (x > whx) { x = whx; vx = -vx; }
    if (x < wlx) { x = wlx; vx = -vx; }
    if (y > why) { y = why; vy = -vy; }
    if (y < wly) { y = wly; vy = -vy; }
  }
  const int cmx = d.periodic ? d.nxr - 1 : d.nx - 1;
  const int cmy = d.periodic ? d.nyr - 1 : d.ny - 1;
  int nx_, ny_;
  if (PREC == 0) {
    nx_ = cell_coord(x, d.lo_x, d.inv_cs_x, d.lo_xd, d.cs_xd, cmx);
    ny_ = cell_coord(y, d.lo_y, d.inv_cs_y, d.lo_yd, d.cs_yd, cmy);
  } else {
    const int kx = offset_cells(x, d.inv_cs_x, d.cs_xd);
    const int ky = offset_cells(y, d.inv_cs_y, d.cs_yd);
    nx_ = cx + kx;
    ny_ = cy + ky;
    int sx, sy;  // cells the offset moves by
    if (d.periodic) {
      sx = kx;
      sy = ky;
      nx_ = ((nx_ % d.nxr) + d.nxr) % d.nxr;
      ny_ = ((ny_ % d.nyr) + d.nyr) % d.nyr;
    } else {
      nx_ = nx_ < 0 ? 0 : (nx_ > cmx ? cmx : nx_);
      ny_ = ny_ < 0 ? 0 : (ny_ > cmy ? cmy : ny_);
      sx = nx_ - cx;
      sy = ny_ - cy;
    }
    if (sx) x = offset_shift_d(x, sx, d.cs_xd);
    if (sy) y = offset_shift_d(y, sy, d.cs_yd);
  }
  const uint32_t key = d.cell_base + local_code(d, nx_, ny_);
  a.posB[i] = make_float2(x, y);
  a.velB[i] = make_float2(vx, vy);
  a.keyB[i] = key;
  if (a.track_ids) a.idsB[i] = a.idsA[i];
  return key;
}

}  // namespace sphg
