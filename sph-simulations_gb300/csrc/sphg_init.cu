// sphg_init.cu -- initial states generated on the device.
//
// The reference builds its initial state on the host with LatticeCreator
// (core/container/Lattice.h:12-35: points d*i, i = 0..n-1 per direction, index
// i + nx*j).  sphg_upload_lattice builds the same lattice -- optionally with a
// seeded uniform jitter and a Taylor-Green velocity field -- directly in the
// handle's arrays, so a large or served state needs no host arrays and no
// host-to-device copy.  The result is what sphg_upload would produce from the
// same FP64 values: FP32 positions, or (split precision) the FP64 cell index
// floor((x - lo) / cs) clamped to the grid and the FP32 offset inside it.
//
// Jitter: particle p of an instance draws u = U(seed, 2p) and U(seed, 2p + 1)
// uniform in [-1, 1) from the SplitMix64 output function (Steele, Lea and
// Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014) of the
// counter seed + (counter + 1) * golden gamma, and moves the point by
// jitter * u * spacing.
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sphg.h"
#include "sphg_internal.cuh"

namespace sphg {
namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// uniform in [-1, 1) with 53 random bits
__device__ __forceinline__ double uniform_pm1(uint64_t seed, uint64_t counter) {
  const uint64_t z = splitmix64(seed + (counter + 1ull) * 0x9E3779B97F4A7C15ull);
  return __dsub_rn(__dmul_rn((double)(z >> 11), 0x1.0p-52), 1.0);
}

// Lattice point p of an instance in the device representation: FP32 position
// (plain) or FP32 offset in cell (cx, cy) (split), FP32 velocity, and the cell.
__device__ __forceinline__ void lattice_point(const sphg_lattice& L, const InstDesc& d, int64_t p, int precision,
                                              float2& pos, float2& vel, int& cx, int& cy) {
  const int64_t gi = p % L.nx, gj = p / L.nx;
  double ox = 0.0, oy = 0.0;
  if (L.jitter != 0.0) {
    ox = __dmul_rn(L.jitter, uniform_pm1(L.seed, 2ull * (uint64_t)p));
    oy = __dmul_rn(L.jitter, uniform_pm1(L.seed, 2ull * (uint64_t)p + 1ull));
  }
  const double x = __dadd_rn(L.x0, __dmul_rn(__dadd_rn((double)gi, ox), L.dx));
  const double y = __dadd_rn(L.y0, __dmul_rn(__dadd_rn((double)gj, oy), L.dy));
  double vx = 0.0, vy = 0.0;
  if (L.velocity == SPHG_VEL_TAYLOR_GREEN) {
    const double twopi = 6.283185307179586476925286766559;
    const double sx = sin(twopi * (x - d.lo_xd) / d.Lx_d), kx = cos(twopi * (x - d.lo_xd) / d.Lx_d);
    const double sy = sin(twopi * (y - d.lo_yd) / d.Ly_d), ky = cos(twopi * (y - d.lo_yd) / d.Ly_d);
    vx = L.u0 * sx * ky;
    vy = -L.u0 * kx * sy;
  }
  vel = make_float2((float)vx, (float)vy);
  const int cmx = d.periodic ? d.nxr - 1 : d.nx - 1;
  const int cmy = d.periodic ? d.nyr - 1 : d.ny - 1;
  // the position the cell is computed from: FP64 (split) or the FP32 one (plain)
  const double px = precision == SPHG_PRECISION_SPLIT ? x : (double)(float)x;
  const double py = precision == SPHG_PRECISION_SPLIT ? y : (double)(float)y;
  const double qx = floor(__ddiv_rn(__dsub_rn(px, d.lo_xd), d.cs_xd));
  const double qy = floor(__ddiv_rn(__dsub_rn(py, d.lo_yd), d.cs_yd));
  cx = !(qx < (double)cmx) ? cmx : (qx < 0.0 ? 0 : (int)qx);
  cy = !(qy < (double)cmy) ? cmy : (qy < 0.0 ? 0 : (int)qy);
  if (precision == SPHG_PRECISION_SPLIT) {
    float fx = __double2float_rn(__dsub_rn(__dsub_rn(x, d.lo_xd), __dmul_rn((double)cx, d.cs_xd)));
    float fy = __double2float_rn(__dsub_rn(__dsub_rn(y, d.lo_yd), __dmul_rn((double)cy, d.cs_yd)));
    if ((double)fx >= d.cs_xd) fx = nextafterf(fx, 0.0f);
    if ((double)fy >= d.cs_yd) fy = nextafterf(fy, 0.0f);
    pos = make_float2(fx, fy);
  } else {
    pos = make_float2((float)x, (float)y);
  }
}

__global__ void lattice_kernel(StepArgs a, const sphg_lattice* __restrict__ spec, int precision) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int inst = a.ninst == 1 ? 0 : find_instance(a.begins, a.ninst, (int)i);
  const InstDesc& d = a.ninst == 1 ? a.d0 : a.desc[inst];
  float2 pos, vel;
  int cx, cy;
  lattice_point(spec[inst], d, i - d.begin, precision, pos, vel, cx, cy);
  a.posB[i] = pos;
  a.velB[i] = vel;
  if (a.track_ids) a.idsB[i] = (int32_t)i;
  if (precision == SPHG_PRECISION_SPLIT) a.keyA[i] = d.cell_base + local_code(d, cx, cy);
}

// A served request's initial state straight into the admission staging:
// instance-local cell codes and creation indices.
__global__ void lattice_stage_kernel(InstDesc d, sphg_lattice L, int precision, int64_t n, float2* pos,
                                     float2* vel, uint32_t* key, int32_t* ids) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int cx, cy;
  lattice_point(L, d, p, precision, pos[p], vel[p], cx, cy);
  key[p] = local_code(d, cx, cy);
  if (ids) ids[p] = (int32_t)p;
}

}  // namespace
}  // namespace sphg

namespace sphg {
cudaError_t launch_lattice_stage(const InstDesc& d, const sphg_lattice& L, int precision, int64_t n, float2* pos,
                                 float2* vel, uint32_t* key, int32_t* ids, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  lattice_stage_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d, L, precision, n, pos, vel, key, ids);
  return cudaGetLastError();
}
}  // namespace sphg

// Validation shared by the handle and the server.
sphg_status sphg_detail::check_lattice(const sphg_lattice& L, int64_t count, int index) {
  if (L.nx < 0 || L.ny < 0 || L.nx * L.ny != count)
    return fail(SPHG_INVALID_ARG, "lattice " + std::to_string(index) + ": nx * ny differs from the particle count");
  if (!std::isfinite(L.x0) || !std::isfinite(L.y0) || !std::isfinite(L.dx) || !std::isfinite(L.dy) ||
      !std::isfinite(L.jitter) || !std::isfinite(L.u0))
    return fail(SPHG_NONFINITE, "lattice " + std::to_string(index) + ": non-finite parameter");
  if (L.velocity != SPHG_VEL_ZERO && L.velocity != SPHG_VEL_TAYLOR_GREEN)
    return fail(SPHG_INVALID_ARG, "lattice " + std::to_string(index) + ": unknown velocity field");
  return SPHG_OK;
}

extern "C" sphg_status sphg_upload_lattice(sphg_sim* s, const sphg_lattice* spec, void* stream) {
  using namespace sphg_detail;
  if (!s || !spec) return fail(SPHG_INVALID_ARG, "null argument");
  for (int i = 0; i < s->ninst; ++i) SPHG_TRY(check_lattice(spec[i], s->counts[i], i));
  cudaStream_t st = (cudaStream_t)stream;
  if (s->n > 0) {
    sphg_lattice* dspec = nullptr;
    SPHG_CUDA(cudaMallocAsync((void**)&dspec, sizeof(sphg_lattice) * s->ninst, st));
    cudaError_t e = cudaMemcpyAsync(dspec, spec, sizeof(sphg_lattice) * s->ninst, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      sphg::lattice_kernel<<<(unsigned)((s->n + 255) / 256), 256, 0, st>>>(s->args(), dspec, s->opt.precision);
      e = cudaGetLastError();
    }
    cudaFreeAsync(dspec, st);
    if (e != cudaSuccess) return fail(SPHG_CUDA_ERROR, std::string("lattice generation: ") + cudaGetErrorString(e));
    // digit histograms of the next sort restart with the generated state
    SPHG_CUDA(cudaMemsetAsync(s->scratch, 0, sizeof(uint32_t) * 4 * 256, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
  }
  s->uploaded = true;
  s->preloop_done = false;
  return SPHG_OK;
}
