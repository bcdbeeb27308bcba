// sphg_hostio.cu -- upload and download that read and write the caller's host
// arrays from the device.
//
// On a Grace-Blackwell node the GPU reaches pageable host memory directly
// (cudaDevAttrPageableMemoryAccess, address translation through the host's
// page tables), so the FP64 <-> device-representation conversion of
// sphg_upload / sphg_download runs as one kernel over the caller's arrays:
// no pinned staging copy and no host conversion loop.  Used when the device
// reports the capability (sphg_set_host_access can turn it off); the results
// are those of the staging path.
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/sphg.h"
#include "sphg_internal.cuh"
#include "sphg_neighbor.cuh"

namespace sphg {
namespace {

// floor(t / cs) exactly as the FP64 division rounds it, from t * (1 / cs):
// the product is within 3 ulp of the quotient, so away from an integer (and
// for |q| < 1e6) its floor is the quotient's; near one the division decides.
__device__ __forceinline__ double floor_div(double t, double cs, double inv_cs) {
  const double q = __dmul_rn(t, inv_cs);
  const double f = floor(q);
  const double r = __dsub_rn(q, f);
  if (r > 1.0e-9 && r < 1.0 - 1.0e-9 && fabs(q) < 1.0e6) return f;
  return floor(__ddiv_rn(t, cs));
}

// One particle of the caller's FP64 state into the device representation
// (false: not finite, nothing written).
__device__ __forceinline__ bool upload_one(const StepArgs& a, int precision, int64_t i, double xi, double yi,
                                           double vxi, double vyi, float2& pos, float2& vel, uint32_t& key) {
  if (!isfinite(xi) || !isfinite(yi) || !isfinite(vxi) || !isfinite(vyi)) return false;
  vel = make_float2((float)vxi, (float)vyi);
  if (precision == SPHG_PRECISION_SPLIT) {
    const InstDesc& d = inst_ref<true>(a, i);
    const int cmx = d.periodic ? d.nxr - 1 : d.nx - 1;
    const int cmy = d.periodic ? d.nyr - 1 : d.ny - 1;
    const double qx = floor_div(__dsub_rn(xi, d.lo_xd), d.cs_xd, d.inv_cs_xd);
    const double qy = floor_div(__dsub_rn(yi, d.lo_yd), d.cs_yd, d.inv_cs_yd);
    const int cx = !(qx < (double)cmx) ? cmx : (qx < 0.0 ? 0 : (int)qx);
    const int cy = !(qy < (double)cmy) ? cmy : (qy < 0.0 ? 0 : (int)qy);
    float fx = __double2float_rn(__dsub_rn(__dsub_rn(xi, d.lo_xd), __dmul_rn((double)cx, d.cs_xd)));
    float fy = __double2float_rn(__dsub_rn(__dsub_rn(yi, d.lo_yd), __dmul_rn((double)cy, d.cs_yd)));
    if ((double)fx >= d.cs_xd) fx = nextafterf(fx, 0.0f);
    if ((double)fy >= d.cs_yd) fy = nextafterf(fy, 0.0f);
    pos = make_float2(fx, fy);
    key = d.cell_base + local_code(d, cx, cy);
  } else {
    pos = make_float2((float)xi, (float)yi);
  }
  return true;
}

__global__ void upload_direct_kernel(StepArgs a, int precision, const double* __restrict__ x,
                                     const double* __restrict__ y, const double* __restrict__ vx,
                                     const double* __restrict__ vy, uint32_t* first_bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  float2 pos, vel;
  uint32_t key = 0;
  if (!upload_one(a, precision, i, x[i], y[i], vx[i], vy[i], pos, vel, key)) {
    atomicMin(first_bad, (uint32_t)i);
    return;
  }
  a.velB[i] = vel;
  a.posB[i] = pos;
  if (precision == SPHG_PRECISION_SPLIT) a.keyA[i] = key;
  if (a.track_ids) a.idsB[i] = (int32_t)i;
}

// Two consecutive particles a thread, 16-byte reads of the caller's arrays
// (all four 16-byte aligned; n odd: the last particle alone).
__global__ void upload_direct_kernel2(StepArgs a, int precision, const double2* __restrict__ x,
                                      const double2* __restrict__ y, const double2* __restrict__ vx,
                                      const double2* __restrict__ vy, uint32_t* first_bad) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i0 = 2 * t;
  if (i0 >= a.n) return;
  if (i0 + 1 == a.n) {  // the odd last particle
    const double* xs = reinterpret_cast<const double*>(x);
    const double* ys = reinterpret_cast<const double*>(y);
    const double* vxs = reinterpret_cast<const double*>(vx);
    const double* vys = reinterpret_cast<const double*>(vy);
    float2 pos, vel;
    uint32_t key = 0;
    if (!upload_one(a, precision, i0, xs[i0], ys[i0], vxs[i0], vys[i0], pos, vel, key)) {
      atomicMin(first_bad, (uint32_t)i0);
      return;
    }
    a.velB[i0] = vel;
    a.posB[i0] = pos;
    if (precision == SPHG_PRECISION_SPLIT) a.keyA[i0] = key;
    if (a.track_ids) a.idsB[i0] = (int32_t)i0;
    return;
  }
  const double2 xv = x[t], yv = y[t], vxv = vx[t], vyv = vy[t];
  float2 p0, p1, v0, v1;
  uint32_t k0 = 0, k1 = 0;
  const bool ok0 = upload_one(a, precision, i0, xv.x, yv.x, vxv.x, vyv.x, p0, v0, k0);
  const bool ok1 = upload_one(a, precision, i0 + 1, xv.y, yv.y, vxv.y, vyv.y, p1, v1, k1);
  if (!ok0 || !ok1) {
    atomicMin(first_bad, (uint32_t)(ok0 ? i0 + 1 : i0));
    if (!ok0 && !ok1) return;
  }
  if (ok0 && ok1) {
    reinterpret_cast<float4*>(a.velB)[t] = make_float4(v0.x, v0.y, v1.x, v1.y);
    reinterpret_cast<float4*>(a.posB)[t] = make_float4(p0.x, p0.y, p1.x, p1.y);
    if (precision == SPHG_PRECISION_SPLIT) reinterpret_cast<uint2*>(a.keyA)[t] = make_uint2(k0, k1);
    if (a.track_ids) reinterpret_cast<int2*>(a.idsB)[t] = make_int2((int32_t)i0, (int32_t)(i0 + 1));
    return;
  }
  const int64_t i = ok0 ? i0 : i0 + 1;  // the finite one of the pair
  a.velB[i] = ok0 ? v0 : v1;
  a.posB[i] = ok0 ? p0 : p1;
  if (precision == SPHG_PRECISION_SPLIT) a.keyA[i] = ok0 ? k0 : k1;
  if (a.track_ids) a.idsB[i] = (int32_t)i;
}

// Particle i of the device state in the caller's FP64 representation.
__device__ __forceinline__ void download_one(const StepArgs& a, int precision, int64_t i, double& px, double& py) {
  const float2 p = a.posA[i];
  px = p.x;
  py = p.y;
  if (precision == SPHG_PRECISION_SPLIT) {
    const InstDesc& d = inst_ref<true>(a, i);
    int cx, cy;
    decode_code(d, a.keyA[i] - d.cell_base, cx, cy);
    px = __dadd_rn(__dadd_rn(d.lo_xd, __dmul_rn((double)cx, d.cs_xd)), px);
    py = __dadd_rn(__dadd_rn(d.lo_yd, __dmul_rn((double)cy, d.cs_yd)), py);
  }
}

__global__ void download_direct_kernel(StepArgs a, int precision, double* __restrict__ x, double* __restrict__ y,
                                       double* __restrict__ vx, double* __restrict__ vy,
                                       double* __restrict__ rho, double* __restrict__ fx,
                                       double* __restrict__ fy, int32_t* __restrict__ ids) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  if (x || y) {
    double px, py;
    download_one(a, precision, i, px, py);
    if (x) x[i] = px;
    if (y) y[i] = py;
  }
  if (vx || vy) {
    const float4 v = a.velpA[i];
    if (vx) vx[i] = v.x;
    if (vy) vy[i] = v.y;
  }
  if (rho) rho[i] = a.rho[i];
  if (fx || fy) {
    const float2 f = a.acc[i];
    if (fx) fx[i] = f.x;
    if (fy) fy[i] = f.y;
  }
  if (ids) ids[i] = a.track_ids ? a.idsA[i] : -1;
}

// Two consecutive particles a thread, 16-byte writes of the caller's arrays
// (every given array 16-byte aligned, the ids 8-byte; n odd: the last one alone).
__global__ void download_direct_kernel2(StepArgs a, int precision, double* __restrict__ x, double* __restrict__ y,
                                        double* __restrict__ vx, double* __restrict__ vy,
                                        double* __restrict__ rho, double* __restrict__ fx,
                                        double* __restrict__ fy, int32_t* __restrict__ ids) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i0 = 2 * t;
  if (i0 >= a.n) return;
  if (i0 + 1 == a.n) {  // the odd last particle
    if (x || y) {
      double px, py;
      download_one(a, precision, i0, px, py);
      if (x) x[i0] = px;
      if (y) y[i0] = py;
    }
    if (vx || vy) {
      const float4 v = a.velpA[i0];
      if (vx) vx[i0] = v.x;
      if (vy) vy[i0] = v.y;
    }
    if (rho) rho[i0] = a.rho[i0];
    if (fx || fy) {
      const float2 f = a.acc[i0];
      if (fx) fx[i0] = f.x;
      if (fy) fy[i0] = f.y;
    }
    if (ids) ids[i0] = a.track_ids ? a.idsA[i0] : -1;
    return;
  }
  if (x || y) {
    double px0, py0, px1, py1;
    download_one(a, precision, i0, px0, py0);
    download_one(a, precision, i0 + 1, px1, py1);
    if (x) reinterpret_cast<double2*>(x)[t] = make_double2(px0, px1);
    if (y) reinterpret_cast<double2*>(y)[t] = make_double2(py0, py1);
  }
  if (vx || vy) {
    const float4 v0 = a.velpA[i0], v1 = a.velpA[i0 + 1];
    if (vx) reinterpret_cast<double2*>(vx)[t] = make_double2(v0.x, v1.x);
    if (vy) reinterpret_cast<double2*>(vy)[t] = make_double2(v0.y, v1.y);
  }
  if (rho) {
    const float2 r = reinterpret_cast<const float2*>(a.rho)[t];
    reinterpret_cast<double2*>(rho)[t] = make_double2(r.x, r.y);
  }
  if (fx || fy) {
    const float4 f = reinterpret_cast<const float4*>(a.acc)[t];
    if (fx) reinterpret_cast<double2*>(fx)[t] = make_double2(f.x, f.z);
    if (fy) reinterpret_cast<double2*>(fy)[t] = make_double2(f.y, f.w);
  }
  if (ids) {
    const int2 d = a.track_ids ? reinterpret_cast<const int2*>(a.idsA)[t] : make_int2(-1, -1);
    reinterpret_cast<int2*>(ids)[t] = d;
  }
}

bool aligned(const void* p, uintptr_t to) { return (reinterpret_cast<uintptr_t>(p) & (to - 1)) == 0; }

}  // namespace

cudaError_t launch_upload_direct(const StepArgs& a, int precision, const double* x, const double* y,
                                 const double* vx, const double* vy, uint32_t* first_bad, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (aligned(x, 16) && aligned(y, 16) && aligned(vx, 16) && aligned(vy, 16)) {
    const int64_t pairs = (a.n + 1) / 2;
    upload_direct_kernel2<<<(unsigned)((pairs + 255) / 256), 256, 0, st>>>(
        a, precision, reinterpret_cast<const double2*>(x), reinterpret_cast<const double2*>(y),
        reinterpret_cast<const double2*>(vx), reinterpret_cast<const double2*>(vy), first_bad);
  } else {
    upload_direct_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a, precision, x, y, vx, vy, first_bad);
  }
  return cudaGetLastError();
}

cudaError_t launch_download_direct(const StepArgs& a, int precision, double* x, double* y, double* vx, double* vy,
                                   double* rho, double* fx, double* fy, int32_t* ids, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (aligned(x, 16) && aligned(y, 16) && aligned(vx, 16) && aligned(vy, 16) && aligned(rho, 16) &&
      aligned(fx, 16) && aligned(fy, 16) && aligned(ids, 8)) {
    const int64_t pairs = (a.n + 1) / 2;
    download_direct_kernel2<<<(unsigned)((pairs + 255) / 256), 256, 0, st>>>(a, precision, x, y, vx, vy, rho, fx,
                                                                               fy, ids);
  } else {
    download_direct_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a, precision, x, y, vx, vy, rho, fx, fy,
                                                                           ids);
  }
  return cudaGetLastError();
}

}  // namespace sphg
