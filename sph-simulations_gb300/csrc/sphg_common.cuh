// sphg_common.cuh -- device-side data layout and helpers shared by the SPH
// step kernels.
//
// Layout in HBM (structure of arrays, one entry per particle slot, all
// instances of a handle concatenated in instance order):
//   pos    float2  position (plain) or in-cell offset (split precision)
//   velp   float4  (vx, vy, P = p/rho^2, 1/rho)  -- written by reorder (xy) and density (zw)
//   rho    float   density
//   key    uint32  global cell key = instance cell_base + Morton/row-major code
//   range  uint2   per global key: [start, end) of its particles in the sorted order
//                  (valid only when key[start] == that key; never cleared)
// and a second copy of pos/vel ("next" state) written by the fused
// force+integrate kernel and consumed by the next sort.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sphg {

constexpr uint32_t kNoIndex = 0xFFFFFFFFu;

// Per-instance constants, precomputed on the host in FP64 (sphg_api.cu).
struct __align__(16) InstDesc {
  int32_t begin, end;     // particle slots [begin, end)
  uint32_t cell_base;     // first global key of this instance
  uint32_t key_span;      // number of keys owned by this instance
  int32_t nx, ny;         // grid extent used by the stencil bounds (Morton: padded)
  int32_t nxr, nyr;       // real cell counts ceil(L/cs) (periodic wrap)
  int32_t order;          // 0 Morton, 1 row-major
  int32_t periodic;       // 0 walls, 1 periodic
  int32_t active;         // 0: a finished served instance awaiting compaction (its slots are skipped)
  int32_t wrap_f32;       // periodic, lo = 0, both lengths exact in FP32: minimum images from FP32 operations
  float lo_x, lo_y, hi_x, hi_y;
  float cs_x, cs_y, inv_cs_x, inv_cs_y;
  float Lx, Ly;
  float h, inv_h2;
  float h2_lo, h2_hi;     // band around h^2 inside which the FP64 test decides
  float wd;               // m * 315 / (64 pi h^3):  rho = wd * sum_j (1 - r^2/h^2)^3
  float kp;               // m * 1.5 * 15 / (pi h^6):  pressure pair factor
  float kv;               // m * 45 mu / (pi h^6):     viscosity pair factor
  float ka;               // m * 3 * 15 / (pi h^6):    artificial-viscosity pair factor
  float k, rho0, tol2;    // EOS stiffness, rest density, TOL^2
  float gx, gy, dt;
  float alpha_c0;         // alpha * c0 (0 = off)
  float eps_h2;           // 0.01 h^2
  double lo_xd, lo_yd, cs_xd, cs_yd, Lx_d, Ly_d, h2_d;
  double mass_d, hi_xd, hi_yd;
  double half_Lx_d, half_Ly_d;  // periodic minimum image
  double inv_cs_xd, inv_cs_yd;  // 1 / cs (FP64): cell index of an FP64 position without a division
};

// ---------------------------------------------------------------- Morton codes
// Bit interleave of 16-bit coordinates: x to even bits, y to odd bits
// (the same code as MortonOrder::MortonCode2d for coordinates < 2^16).
__device__ __forceinline__ uint32_t part1by1(uint32_t x) {
  x &= 0x0000ffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}
__device__ __forceinline__ uint32_t compact1by1(uint32_t x) {
  x &= 0x55555555u;
  x = (x | (x >> 1)) & 0x33333333u;
  x = (x | (x >> 2)) & 0x0f0f0f0fu;
  x = (x | (x >> 4)) & 0x00ff00ffu;
  x = (x | (x >> 8)) & 0x0000ffffu;
  return x;
}

__device__ __forceinline__ uint32_t local_code(const InstDesc& d, int cx, int cy) {
  if (d.order == 0) return (part1by1((uint32_t)cy) << 1) | part1by1((uint32_t)cx);
  return (uint32_t)cx + (uint32_t)cy * (uint32_t)d.nx;
}

__device__ __forceinline__ void decode_code(const InstDesc& d, uint32_t code, int& cx, int& cy) {
  if (d.order == 0) {
    cx = (int)compact1by1(code);
    cy = (int)compact1by1(code >> 1);
  } else {
    cx = (int)(code % (uint32_t)d.nx);
    cy = (int)(code / (uint32_t)d.nx);
  }
}

// ---------------------------------------------------------------- exact cell index
// floor((x - lo) / cs) exactly as the reference's FP64 code computes it
// (GenericNeighborSearch.h:216-222), from an FP32 position: the FP32 quotient
// decides unless it lies within a few ulp of a cell edge, where the FP64
// expression decides.  Clamped to [0, cmax] (the reference clamps above only).
static __device__ __noinline__ int cell_coord_d(float x, double lo_d, double cs_d) {
  return (int)floor(__ddiv_rn(__dsub_rn((double)x, lo_d), cs_d));
}

__device__ __forceinline__ int cell_coord(float x, float lo, float inv_cs, double lo_d,
                                          double cs_d, int cmax) {
  float q = (x - lo) * inv_cs;
  if (!(q < (float)cmax + 1.0f)) return cmax;  // also NaN
  float tol = 5.0e-7f * (fabsf(x) + fabsf(lo)) * inv_cs + 1.0e-30f;
  // clearly below 1 (a particle at or near the low wall): the FP64 quotient is
  // below 1, its floor 0 or negative, clamped to 0
  if (q < 1.0f - tol) return 0;
  float fq = floorf(q);
  float fr = q - fq;
  int c;
  if (fr > tol && fr < 1.0f - tol) {
    c = (int)fq;
  } else {
    c = cell_coord_d(x, lo_d, cs_d);  // out of line: keeps FP64 off the common path
  }
  return c < 0 ? 0 : (c > cmax ? cmax : c);
}

// FP64 distance test of the reference: r2 = dx*dx + dy*dy (no contraction),
// inside when !(r2 > h2).
static __device__ __forceinline__ bool exact_inside_d(double dx, double dy, double h2_d) {
  double r2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  return !(r2 > h2_d);
}

// ---------------------------------------------------------------- compensated sums
struct CSum {
  float s, c;
  __device__ __forceinline__ CSum() : s(0.f), c(0.f) {}
  __device__ __forceinline__ void add(float t) {  // TwoSum (Knuth), error kept in c
    float sn = __fadd_rn(s, t);
    float bp = __fsub_rn(sn, s);
    float err = __fadd_rn(__fsub_rn(s, __fsub_rn(sn, bp)), __fsub_rn(t, bp));
    s = sn;
    c = __fadd_rn(c, err);
  }
  // Fast2Sum (Dekker): the rounding error of s + t is exactly t - ((s + t) - s)
  // when |s| >= |t|.  Valid for the density sum once it holds the particle's
  // own term W(0) = 1: every other term (1 - r^2/h^2)^3 of an accepted pair
  // lies in [0, 1] and none is negative.
  __device__ __forceinline__ void add_fast(float t) {
    const float sn = __fadd_rn(s, t);
    c = __fadd_rn(c, __fsub_rn(t, __fsub_rn(sn, s)));
    s = sn;
  }
  __device__ __forceinline__ float value() const { return s + c; }
};

// Paired FP32 arithmetic (one sm_100-family instruction for both components;
// each component rounds exactly as the scalar _rn operation does).
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// CSum of both axes at once: the same TwoSum per component in paired
// instructions (the same bits as two CSum).
struct CSum2 {
  float2 s, c;
  __device__ __forceinline__ CSum2() : s(make_float2(0.f, 0.f)), c(make_float2(0.f, 0.f)) {}
  __device__ __forceinline__ void add(float2 t) {
    const float2 sn = add2(s, t);
    const float2 bp = sub2(sn, s);
    const float2 err = add2(sub2(s, sub2(sn, bp)), sub2(t, bp));
    s = sn;
    c = add2(c, err);
  }
  __device__ __forceinline__ float2 value() const { return add2(s, c); }
};

struct PSum2 {
  float2 s;
  __device__ __forceinline__ PSum2() : s(make_float2(0.f, 0.f)) {}
  __device__ __forceinline__ void add(float2 t) { s = add2(s, t); }
  __device__ __forceinline__ float2 value() const { return s; }
};

struct PSum {
  float s;
  __device__ __forceinline__ PSum() : s(0.f) {}
  __device__ __forceinline__ void add(float t) { s += t; }
  __device__ __forceinline__ void add_fast(float t) { s += t; }
  __device__ __forceinline__ float value() const { return s; }
};

// Instance of particle slot i (binary search over instance begins; ninst is small).
__device__ __forceinline__ int find_instance(const int32_t* __restrict__ begins, int ninst, int i) {
  int lo = 0, hi = ninst - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(begins + mid) <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Lets the next kernel of the stream (launched with programmatic dependent
// launch) be scheduled now: its blocks take the SMs this grid's last blocks
// leave and wait in cudaGridDependencySynchronize() for this grid to finish
// (which still orders every memory access).  Called at the start of the step
// kernels when the state is small (a few waves a kernel: the tail and the next
// launch are a large share of it), not for large ones, where it measured slower
// (12,800 particles: 36.5 -> 34.4 us an iteration; 4.4M: 0.410 -> 0.419 ms).
constexpr int64_t kEarlyNextMaxN = (int64_t)1 << 19;
__device__ __forceinline__ void allow_next_kernel(int early) {
  if (early) cudaTriggerProgrammaticLaunchCompletion();
}

// Launch with programmatic dependent launch: the kernel may be scheduled while
// the previous kernel in the stream finishes; it must call
// cudaGridDependencySynchronize() before touching that kernel's results (a
// no-op when launched without the attribute).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
#ifdef SPHG_NO_PDL
  cfg.numAttrs = 0;
#else
  cfg.numAttrs = 1;
#endif
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace sphg
