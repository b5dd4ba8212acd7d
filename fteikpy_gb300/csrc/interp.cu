// Interpolation kernels: one thread per query point (the reference's prange
// over points, fteikpy/_interp/_interp3d.py:177-185 and friends).
#include "common.cuh"
#include "fteik_gb300.h"
#include "interp.cuh"
#include "runtime.h"

namespace fteik {

__global__ void interp3d_kernel(const double* ax0, int n0, const double* ax1, int n1,
                                const double* ax2, int n2, const double* v, long long vs,
                                const double* pts, int npts, double fval, double* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  out[p] = interp3_point(ax0, n0, ax1, n1, ax2, n2, v, vs, pts[3 * p], pts[3 * p + 1],
                         pts[3 * p + 2], fval);
}

__global__ void interp2d_kernel(const double* ax0, int n0, const double* ax1, int n1,
                                const double* v, long long vs, const double* pts, int npts,
                                double fval, double* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  out[p] = interp2_point(ax0, n0, ax1, n1, v, vs, pts[2 * p], pts[2 * p + 1], fval);
}

__global__ void vinterp3d_kernel(const double* ax0, int n0, const double* ax1, int n1,
                                 const double* ax2, int n2, const double* tt, long long tstride,
                                 const int* gidx, const double* pts, int npts,
                                 const double* src, const double* vzero, double fval,
                                 double* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int g = gidx ? gidx[p] : 0;
  out[p] = vinterp3_point(ax0, n0, ax1, n1, ax2, n2, tt + (long long)g * tstride, pts[3 * p],
                          pts[3 * p + 1], pts[3 * p + 2], src[3 * g], src[3 * g + 1],
                          src[3 * g + 2], vzero[g], fval);
}

__global__ void vinterp2d_kernel(const double* ax0, int n0, const double* ax1, int n1,
                                 const double* tt, long long tstride, const int* gidx,
                                 const double* pts, int npts, const double* src,
                                 const double* vzero, double fval, double* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int g = gidx ? gidx[p] : 0;
  out[p] = vinterp2_point(ax0, n0, ax1, n1, tt + (long long)g * tstride, pts[2 * p],
                          pts[2 * p + 1], src[2 * g], src[2 * g + 1], vzero[g], fval);
}

}  // namespace fteik

using namespace fteik;

static inline bool axes_ok(int n) { return n >= 2; }

extern "C" int fteik_interp3d(const double* ax0, int n0, const double* ax1, int n1,
                              const double* ax2, int n2, const double* v, long long vstride,
                              const double* points, int npts, double fill_value, double* out,
                              void* stream) {
  if (!axes_ok(n0) || !axes_ok(n1) || !axes_ok(n2) || npts < 0 || vstride < 1)
    return kInvalidArgument;
  if (npts == 0) return kOk;
  interp3d_kernel<<<(npts + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      ax0, n0, ax1, n1, ax2, n2, v, vstride, points, npts, fill_value, out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}

extern "C" int fteik_interp2d(const double* ax0, int n0, const double* ax1, int n1,
                              const double* v, long long vstride, const double* points, int npts,
                              double fill_value, double* out, void* stream) {
  if (!axes_ok(n0) || !axes_ok(n1) || npts < 0 || vstride < 1) return kInvalidArgument;
  if (npts == 0) return kOk;
  interp2d_kernel<<<(npts + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      ax0, n0, ax1, n1, v, vstride, points, npts, fill_value, out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}

extern "C" int fteik_vinterp3d(const double* ax0, int n0, const double* ax1, int n1,
                               const double* ax2, int n2, const double* tt, long long tt_stride,
                               const int* grid_index, const double* points, int npts,
                               const double* sources, const double* vzero, double fill_value,
                               double* out, void* stream) {
  if (!axes_ok(n0) || !axes_ok(n1) || !axes_ok(n2) || npts < 0) return kInvalidArgument;
  if (npts == 0) return kOk;
  vinterp3d_kernel<<<(npts + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      ax0, n0, ax1, n1, ax2, n2, tt, tt_stride, grid_index, points, npts, sources, vzero,
      fill_value, out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}

extern "C" int fteik_vinterp2d(const double* ax0, int n0, const double* ax1, int n1,
                               const double* tt, long long tt_stride, const int* grid_index,
                               const double* points, int npts, const double* sources,
                               const double* vzero, double fill_value, double* out,
                               void* stream) {
  if (!axes_ok(n0) || !axes_ok(n1) || npts < 0) return kInvalidArgument;
  if (npts == 0) return kOk;
  vinterp2d_kernel<<<(npts + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      ax0, n0, ax1, n1, tt, tt_stride, grid_index, points, npts, sources, vzero, fill_value,
      out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}
