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

__global__ void upload_direct_kernel(StepArgs a, int precision, const double* __restrict__ x,
                                     const double* __restrict__ y, const double* __restrict__ vx,
                                     const double* __restrict__ vy, uint32_t* first_bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double xi = x[i], yi = y[i], vxi = vx[i], vyi = vy[i];
  if (!isfinite(xi) || !isfinite(yi) || !isfinite(vxi) || !isfinite(vyi)) {
    atomicMin(first_bad, (uint32_t)i);
    return;
  }
  a.velB[i] = make_float2((float)vxi, (float)vyi);
  if (a.track_ids) a.idsB[i] = (int32_t)i;
  if (precision == SPHG_PRECISION_SPLIT) {
    const InstDesc& d = inst_ref<true>(a, i);
    const int cmx = d.periodic ? d.nxr - 1 : d.nx - 1;
    const int cmy = d.periodic ? d.nyr - 1 : d.ny - 1;
    const double qx = floor(__ddiv_rn(__dsub_rn(xi, d.lo_xd), d.cs_xd));
    const double qy = floor(__ddiv_rn(__dsub_rn(yi, d.lo_yd), d.cs_yd));
    const int cx = !(qx < (double)cmx) ? cmx : (qx < 0.0 ? 0 : (int)qx);
    const int cy = !(qy < (double)cmy) ? cmy : (qy < 0.0 ? 0 : (int)qy);
    float fx = __double2float_rn(__dsub_rn(__dsub_rn(xi, d.lo_xd), __dmul_rn((double)cx, d.cs_xd)));
    float fy = __double2float_rn(__dsub_rn(__dsub_rn(yi, d.lo_yd), __dmul_rn((double)cy, d.cs_yd)));
    if ((double)fx >= d.cs_xd) fx = nextafterf(fx, 0.0f);
    if ((double)fy >= d.cs_yd) fy = nextafterf(fy, 0.0f);
    a.posB[i] = make_float2(fx, fy);
    a.keyA[i] = d.cell_base + local_code(d, cx, cy);
  } else {
    a.posB[i] = make_float2((float)xi, (float)yi);
  }
}

__global__ void download_direct_kernel(StepArgs a, int precision, double* __restrict__ x, double* __restrict__ y,
                                       double* __restrict__ vx, double* __restrict__ vy,
                                       double* __restrict__ rho, double* __restrict__ fx,
                                       double* __restrict__ fy, int32_t* __restrict__ ids) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  if (x || y) {
    const float2 p = a.posA[i];
    double px = p.x, py = p.y;
    if (precision == SPHG_PRECISION_SPLIT) {
      const InstDesc& d = inst_ref<true>(a, i);
      int cx, cy;
      decode_code(d, a.keyA[i] - d.cell_base, cx, cy);
      px = __dadd_rn(__dadd_rn(d.lo_xd, __dmul_rn((double)cx, d.cs_xd)), px);
      py = __dadd_rn(__dadd_rn(d.lo_yd, __dmul_rn((double)cy, d.cs_yd)), py);
    }
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

}  // namespace

cudaError_t launch_upload_direct(const StepArgs& a, int precision, const double* x, const double* y,
                                 const double* vx, const double* vy, uint32_t* first_bad, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  upload_direct_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a, precision, x, y, vx, vy, first_bad);
  return cudaGetLastError();
}

cudaError_t launch_download_direct(const StepArgs& a, int precision, double* x, double* y, double* vx, double* vy,
                                   double* rho, double* fx, double* fy, int32_t* ids, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  download_direct_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a, precision, x, y, vx, vy, rho, fx, fy,
                                                                         ids);
  return cudaGetLastError();
}

}  // namespace sphg
