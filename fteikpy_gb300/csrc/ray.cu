// A-posteriori ray tracing: fteikpy/_fteik/_ray3d.py, _ray2d.py and the
// step-shrinking helper _fteik/_common.py restated for the GPU, one thread per
// ray (the reference's prange over end points, _ray3d.py:145).
//
// Per step the reference interpolates each gradient component separately
// (_ray3d.py:60-62); the three calls share the query point, so the cell lookup
// and the 8 weights are computed once here and applied to the three
// components, which gives the same numbers.
//
// One intentional difference: when a honor_grid step lands exactly on the last
// node of an axis, the reference reads one element past the end of that axis
// (_ray3d.py:96-98, _ray2d.py:69-70); here the index is clamped to the last
// node, as the reference itself does when it sets up the first cell
// (_ray3d.py:46-48).
#include <math_constants.h>

#include "common.cuh"
#include "fteik_gb300.h"
#include "interp.cuh"
#include "runtime.h"

namespace fteik {

// numpy ndarray.min(): NaN if any element is NaN.
__device__ __forceinline__ double np_min(const double* a, int n) {
  double m = a[0];
  for (int q = 0; q < n; ++q) {
    if (a[q] != a[q]) return a[q];
    if (a[q] < m) m = a[q];
  }
  return m;
}

// shrink, _fteik/_common.py:4-28.
template <int ND>
__device__ __forceinline__ double shrink(const double* pcur, const double* delta,
                                         const double* lower, const double* upper) {
  double bl[ND], bu[ND];
  int nl = 0, nu = 0;
#pragma unroll
  for (int q = 0; q < ND; ++q) {
    const double tmp = pcur[q] - delta[q];
    if (tmp < lower[q]) bl[nl++] = (pcur[q] - lower[q]) / delta[q];
    if (tmp > upper[q]) bu[nu++] = (pcur[q] - upper[q]) / delta[q];
  }
  if (nl && nu) {
    const double a = np_min(bl, nl), b = np_min(bu, nu);
    return b < a ? b : a;
  }
  if (nl) return np_min(bl, nl);
  if (nu) return np_min(bu, nu);
  return 1.0;
}

struct Axes {
  const double* a[3];
  int n[3];
};

// Gradient direction at p: the three (or two) interpolated components.
template <int ND>
__device__ __forceinline__ void grad_at(const Axes& ax, const double* g, const double* p,
                                        double* out) {
  if (ND == 3) {
    if (!inside3(ax.a[0], ax.n[0], ax.a[1], ax.n[1], ax.a[2], ax.n[2], p[0], p[1], p[2])) {
      out[0] = out[1] = out[2] = CUDART_NAN;
      return;
    }
    const Cell3 c = locate3(ax.a[0], ax.n[0], ax.a[1], ax.n[1], ax.a[2], ax.n[2], p[0], p[1], p[2]);
    double w[8];
    weights3(c, p[0], p[1], p[2], w);
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      double q[8];
      corners3(g + comp, 3, c, ax.n[1], ax.n[2], q);
      out[comp] = blend3(c, q, w);
    }
  } else {
    if (!inside2(ax.a[0], ax.n[0], ax.a[1], ax.n[1], p[0], p[1])) {
      out[0] = out[1] = CUDART_NAN;
      return;
    }
    const Cell2 c = locate2(ax.a[0], ax.n[0], ax.a[1], ax.n[1], p[0], p[1]);
    double w[4];
    weights2(c, p[0], p[1], w);
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      double q[4];
      corners2(g + comp, 2, c, ax.n[1], q);
      double vq = q[0] * w[0];
      vq += q[1] * w[1];
      vq += q[2] * w[2];
      vq += q[3] * w[3];
      vq /= fabs((c.x2 - c.x1) * (c.y2 - c.y1));
      out[comp] = vq;
    }
  }
}

// Component `comp` of grad_at (the same lookup, weights and blend).
template <int ND>
__device__ __forceinline__ double grad_comp(const Axes& ax, const double* g, const double* p,
                                            int comp) {
  if (ND == 3) {
    if (!inside3(ax.a[0], ax.n[0], ax.a[1], ax.n[1], ax.a[2], ax.n[2], p[0], p[1], p[2]))
      return CUDART_NAN;
    const Cell3 c = locate3(ax.a[0], ax.n[0], ax.a[1], ax.n[1], ax.a[2], ax.n[2], p[0], p[1], p[2]);
    double w[8], q[8];
    weights3(c, p[0], p[1], p[2], w);
    corners3(g + comp, 3, c, ax.n[1], ax.n[2], q);
    return blend3(c, q, w);
  } else {
    if (!inside2(ax.a[0], ax.n[0], ax.a[1], ax.n[1], p[0], p[1])) return CUDART_NAN;
    const Cell2 c = locate2(ax.a[0], ax.n[0], ax.a[1], ax.n[1], p[0], p[1]);
    double w[4], q[4];
    weights2(c, p[0], p[1], w);
    corners2(g + comp, 2, c, ax.n[1], q);
    double vq = q[0] * w[0];
    vq += q[1] * w[1];
    vq += q[2] * w[2];
    vq += q[3] * w[3];
    vq /= fabs((c.x2 - c.x1) * (c.y2 - c.y1));
    return vq;
  }
}

// _ray3d / _ray2d, _ray3d.py:9-120 and _ray2d.py:9-91.
// L lanes trace one ray: with L = 4, lanes 0..ND-1 of the group each blend
// one gradient component and the group shares them, so a few rays (one
// source's receivers) take fewer dependent FP64 instructions per step; the
// other work is done identically by every lane and lane 0 writes.
template <int ND, int L>
__global__ void ray_kernel(Axes ax, const double* ttgrad, long long gstride, const int* gidx,
                           const double* ends, int nrays, const double* sources,
                           double stepsize, int max_step, int honor_grid, double* rays,
                           int* counts, int* status) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int r = (int)(tid / L);
  const int sub = (int)(tid % L);
  const bool writer = sub == 0;
  const unsigned gmask = L == 1 ? 0u : (((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1)));
  if (r >= nrays) return;
  const int gi = gidx ? gidx[r] : 0;
  const double* g = ttgrad + (long long)gi * gstride;
  double src[ND], pcur[ND], delta[ND], lower[ND], upper[ND];
  int isrc[ND];
#pragma unroll
  for (int q = 0; q < ND; ++q) {
    src[q] = sources[ND * gi + q];
    pcur[q] = ends[ND * r + q];
  }
  if (writer) counts[r] = 0;
#pragma unroll
  for (int q = 0; q < ND; ++q) {
    if (!(__ldg(ax.a[q]) <= pcur[q] && pcur[q] <= __ldg(ax.a[q] + ax.n[q] - 1))) {
      if (writer) status[r] = kEndPointOutOfBound;
      return;
    }
  }
  if (honor_grid) {
#pragma unroll
    for (int q = 0; q < ND; ++q) {
      const double* a = ax.a[q];
      const int n = ax.n[q];
      const int i = search_right_m1(a, n, pcur[q]);
      lower[q] = pcur[q] == __ldg(a + i) ? __ldg(a + imax(i - 1, 0)) : __ldg(a + i);
      upper[q] = __ldg(a + imin(i + 1, n - 1));
      isrc[q] = search_right_m1(a, n, src[q]);
    }
  }
  double* ray = rays + (long long)r * max_step * ND;
  int count = 1;
  if (writer) {
#pragma unroll
    for (int q = 0; q < ND; ++q) ray[q] = pcur[q];
  }
  // The reference loops until the ray reaches the source or max_step points
  // are recorded; with honor_grid a step inside a cell records nothing, so
  // the number of iterations is capped as well (a cap the reference does not
  // have), reported as max_step reached, so that no input can hang the GPU.
  const long long max_iter = 64LL * max_step + 4096;
  for (long long iter = 0;; ++iter) {
    if (iter >= max_iter) {
      if (writer) status[r] = kMaxStepReached;
      return;
    }
    const double dd = ND == 3 ? dist3(src[0], src[1], src[2], pcur[0], pcur[1], pcur[2])
                              : dist2(src[0], src[1], pcur[0], pcur[1]);
    if (!(dd >= stepsize)) break;
    double gv[ND];
    if (L == 1) {
      grad_at<ND>(ax, g, pcur, gv);
    } else {
      const double mine = sub < ND ? grad_comp<ND>(ax, g, pcur, sub) : 0.0;
#pragma unroll
      for (int q = 0; q < ND; ++q) gv[q] = __shfl_sync(gmask, mine, q, L);
    }
    double gsq = gv[0] * gv[0] + gv[1] * gv[1];
    if (ND == 3) gsq = gsq + gv[ND - 1] * gv[ND - 1];
    const double gn = sqrt(gsq);
    double gni;
    if (gn > 0.0)
      gni = 1.0 / gn;
    else
      break;
#pragma unroll
    for (int q = 0; q < ND; ++q) delta[q] = stepsize * gv[q] * gni;
    if (honor_grid) {
      const double fac = shrink<ND>(pcur, delta, lower, upper);
#pragma unroll
      for (int q = 0; q < ND; ++q) {
        double v = pcur[q] - fac * delta[q];
        const double lo = __ldg(ax.a[q]), hi = __ldg(ax.a[q] + ax.n[q] - 1);
        v = lo > v ? lo : v;  // max(pcur, axis[0])
        v = hi < v ? hi : v;  // min(., axis[-1])
        pcur[q] = v;
      }
      if (fac < 1.0) {
#pragma unroll
        for (int q = 0; q < ND; ++q) {
          if (fabs(pcur[q] - lower[q]) < 1.0e-8)
            pcur[q] = lower[q];
          else if (fabs(pcur[q] - upper[q]) < 1.0e-8)
            pcur[q] = upper[q];
        }
        bool hit = true;
#pragma unroll
        for (int q = 0; q < ND; ++q) {
          const double* a = ax.a[q];
          const int n = ax.n[q];
          const int i = search_right_m1(a, n, pcur[q]);
          lower[q] = pcur[q] == __ldg(a + i) ? __ldg(a + imax(i - 1, 0)) : __ldg(a + i);
          upper[q] = __ldg(a + imin(i + 1, n - 1));
          hit = hit && (i == isrc[q]);
        }
        if (writer) {
#pragma unroll
          for (int q = 0; q < ND; ++q) ray[count * ND + q] = pcur[q];
        }
        count += 1;
        if (hit) break;
      }
    } else {
#pragma unroll
      for (int q = 0; q < ND; ++q) {
        double v = pcur[q] - delta[q];
        const double lo = __ldg(ax.a[q]), hi = __ldg(ax.a[q] + ax.n[q] - 1);
        v = lo > v ? lo : v;
        v = hi < v ? hi : v;
        pcur[q] = v;
        if (writer) ray[count * ND + q] = v;
      }
      count += 1;
    }
    if (count >= max_step) {
      if (writer) status[r] = kMaxStepReached;
      return;
    }
  }
  if (writer) {
#pragma unroll
    for (int q = 0; q < ND; ++q) ray[count * ND + q] = src[q];
    counts[r] = count;
    status[r] = kOk;
  }
}

// Reverse each ray (source first, as ray3d returns ray[count::-1]) and pack
// the rays back to back.
template <int ND>
__global__ void ray_pack_kernel(const double* rays, int nrays, int max_step, const int* counts,
                                const long long* offsets, double* packed) {
  const int r = blockIdx.x;
  if (r >= nrays) return;
  const int c = counts[r];
  const double* src = rays + (long long)r * max_step * ND;
  double* dst = packed + offsets[r] * ND;
  for (int t = threadIdx.x; t <= c; t += blockDim.x) {
#pragma unroll
    for (int q = 0; q < ND; ++q) dst[t * ND + q] = src[(c - t) * ND + q];
  }
}

}  // namespace fteik

using namespace fteik;

template <int ND>
static int launch_rays(const double* const* axes, const int* n, const double* ttgrad,
                       long long grad_stride, const int* grid_index, const double* ends,
                       int nrays, const double* sources, double stepsize, int max_step,
                       int honor_grid, double* rays, int* counts, int* status, void* stream) {
  if (nrays < 0 || max_step < 2 || !(stepsize > 0.0)) return kInvalidArgument;
  Axes ax;
  for (int q = 0; q < 3; ++q) {
    ax.a[q] = q < ND ? axes[q] : nullptr;
    ax.n[q] = q < ND ? n[q] : 0;
    if (q < ND && n[q] < 2) return kInvalidArgument;
  }
  if (nrays == 0) return kOk;
  // Four lanes per ray while every ray's group fits on the GPU at once (one
  // source's receivers); one lane per ray for large batches, which are bound
  // by throughput rather than by the latency of a step.
  if ((long long)nrays * 4 <= 64LL * 1024) {
    const long long threads = (long long)nrays * 4;
    ray_kernel<ND, 4><<<(unsigned)((threads + 63) / 64), 64, 0, (cudaStream_t)stream>>>(
        ax, ttgrad, grad_stride, grid_index, ends, nrays, sources, stepsize, max_step,
        honor_grid, rays, counts, status);
  } else {
    ray_kernel<ND, 1><<<(nrays + 63) / 64, 64, 0, (cudaStream_t)stream>>>(
        ax, ttgrad, grad_stride, grid_index, ends, nrays, sources, stepsize, max_step,
        honor_grid, rays, counts, status);
  }
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}

extern "C" int fteik_ray3d(const double* ax0, int n0, const double* ax1, int n1, const double* ax2,
                           int n2, const double* ttgrad, long long grad_stride,
                           const int* grid_index, const double* ends, int nrays,
                           const double* sources, double stepsize, int max_step, int honor_grid,
                           double* rays, int* counts, int* status, void* stream) {
  const double* axes[3] = {ax0, ax1, ax2};
  const int n[3] = {n0, n1, n2};
  return launch_rays<3>(axes, n, ttgrad, grad_stride, grid_index, ends, nrays, sources, stepsize,
                        max_step, honor_grid, rays, counts, status, stream);
}

extern "C" int fteik_ray2d(const double* ax0, int n0, const double* ax1, int n1,
                           const double* ttgrad, long long grad_stride, const int* grid_index,
                           const double* ends, int nrays, const double* sources,
                           double stepsize, int max_step, int honor_grid, double* rays,
                           int* counts, int* status, void* stream) {
  const double* axes[3] = {ax0, ax1, nullptr};
  const int n[3] = {n0, n1, 0};
  return launch_rays<2>(axes, n, ttgrad, grad_stride, grid_index, ends, nrays, sources, stepsize,
                        max_step, honor_grid, rays, counts, status, stream);
}

extern "C" int fteik_ray_pack(int ndim, const double* rays, int nrays, int max_step,
                              const int* counts, const long long* offsets, double* packed,
                              void* stream) {
  if (nrays < 0 || (ndim != 2 && ndim != 3)) return kInvalidArgument;
  if (nrays == 0) return kOk;
  if (ndim == 3)
    ray_pack_kernel<3><<<nrays, 64, 0, (cudaStream_t)stream>>>(rays, nrays, max_step, counts,
                                                               offsets, packed);
  else
    ray_pack_kernel<2><<<nrays, 64, 0, (cudaStream_t)stream>>>(rays, nrays, max_step, counts,
                                                               offsets, packed);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}
