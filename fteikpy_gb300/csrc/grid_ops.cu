// Velocity-model preparation on the device: the resampling and smoothing that
// fteikpy's grids do with SciPy (fteikpy/_base.py:81-123, 165-212).
//
//  * resample: RegularGridInterpolator on the grid's own axes, evaluated at
//    the tensor grid of np.linspace points. The per-axis lower indices and
//    normalised distances (and 1 - distance) come from the host, which
//    computes them with NumPy; the kernel forms the 2^nd-corner sum in the
//    order of SciPy's _evaluate_linear (scipy/interpolate/_rgi.py): corners
//    in itertools.product order (last axis fastest), weight ((w0 * w1) * w2),
//    running sum from 0. "nearest" gathers the nearest node per axis.
//  * smooth: gaussian_filter as one 1D correlation per axis with the
//    Gaussian weights the host computes, in mode 'reflect'
//    (d c b a | a b c d | d c b a), origin 0.
#include <cstdint>

#include "common.cuh"
#include "fteik_gb300.h"
#include "runtime.h"

namespace fteik {

struct Dims3 {
  int n[3];   // input shape (unused trailing axes are 1)
  int m[3];   // output shape
  int off[3];  // start of each axis' table in the concatenated tables
};

__global__ void resample_linear_kernel(int nd, const double* v, Dims3 D, const int* idx,
                                       const double* y, const double* ym, double* out) {
  const long long total = (long long)D.m[0] * D.m[1] * D.m[2];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int q2 = (int)(q % D.m[2]);
    const int q1 = (int)((q / D.m[2]) % D.m[1]);
    const int q0 = (int)(q / ((long long)D.m[1] * D.m[2]));
    const int qq[3] = {q0, q1, q2};
    int lo[3];
    double wl[3], wu[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo[d] = d < nd ? idx[D.off[d] + qq[d]] : 0;
      wl[d] = d < nd ? ym[D.off[d] + qq[d]] : 1.0;
      wu[d] = d < nd ? y[D.off[d] + qq[d]] : 0.0;
    }
    double value = 0.0;
    const int ncorner = 1 << nd;
    for (int c = 0; c < ncorner; ++c) {
      // itertools.product order: bit (nd-1-d) of c selects the upper node of axis d
      long long at = 0;
      double w = 1.0;
      for (int d = 0; d < nd; ++d) {
        const int up = (c >> (nd - 1 - d)) & 1;
        at = at * D.n[d] + lo[d] + up;
        w = w * (up ? wu[d] : wl[d]);
      }
      value = value + __ldg(v + at) * w;
    }
    out[q] = value;
  }
}

__global__ void resample_nearest_kernel(int nd, const double* v, Dims3 D, const int* idx,
                                        double* out) {
  const long long total = (long long)D.m[0] * D.m[1] * D.m[2];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int q2 = (int)(q % D.m[2]);
    const int q1 = (int)((q / D.m[2]) % D.m[1]);
    const int q0 = (int)(q / ((long long)D.m[1] * D.m[2]));
    const int qq[3] = {q0, q1, q2};
    long long at = 0;
    for (int d = 0; d < nd; ++d) at = at * D.n[d] + idx[D.off[d] + qq[d]];
    out[q] = __ldg(v + at);
  }
}

// Index of position i on an axis of n nodes in mode 'reflect'.
__device__ __forceinline__ int reflect_index(int i, int n) {
  const int p = 2 * n;
  int m = i % p;
  if (m < 0) m += p;
  return m < n ? m : p - 1 - m;
}

// out[..., i, ...] = sum_j w[j] * in[..., reflect(i + j - r), ...] along
// `axis` (the array seen as [outer][n][inner]); r = (nw - 1) / 2.
__global__ void correlate1d_kernel(const double* in, long long outer, int n, long long inner,
                                   const double* w, int nw, double* out) {
  const long long total = outer * n * inner;
  const int r = (nw - 1) / 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long o = q / ((long long)n * inner);
    const long long rest = q - o * n * inner;
    const int i = (int)(rest / inner);
    const long long k = rest - (long long)i * inner;
    const double* line = in + o * n * inner + k;
    double s = 0.0;
    for (int j = 0; j < nw; ++j) s += __ldg(w + j) * __ldg(line + (long long)reflect_index(i + j - r, n) * inner);
    out[q] = s;
  }
}

static bool dims_ok(int nd, const int* dims) {
  if (nd < 1 || nd > 3 || !dims) return false;
  for (int d = 0; d < nd; ++d)
    if (dims[d] < 1) return false;
  return true;
}

}  // namespace fteik

using namespace fteik;

extern "C" int fteik_resample(int nd, int nearest, const double* values, const int* dims,
                              const int* out_dims, const int* idx, const double* y,
                              const double* ym, double* out, void* stream) {
  if (!dims_ok(nd, dims) || !dims_ok(nd, out_dims) || !values || !idx || !out ||
      (!nearest && (!y || !ym)))
    return kInvalidArgument;
  Dims3 D;
  int off = 0;
  for (int d = 0; d < 3; ++d) {
    D.n[d] = d < nd ? dims[d] : 1;
    D.m[d] = d < nd ? out_dims[d] : 1;
    D.off[d] = off;
    off += D.m[d];
  }
  // one output node per thread; the lower index + 1 must stay in the grid
  // for the linear weights (the host clips it to n - 2, or 0 on a 1-node axis)
  for (int d = 0; d < nd; ++d)
    if (!nearest && D.n[d] < 2) return kInvalidArgument;
  const long long total = (long long)D.m[0] * D.m[1] * D.m[2];
  cudaStream_t st = (cudaStream_t)stream;
  if (nearest)
    resample_nearest_kernel<<<grid_for(total, 256), 256, 0, st>>>(nd, values, D, idx, out);
  else
    resample_linear_kernel<<<grid_for(total, 256), 256, 0, st>>>(nd, values, D, idx, y, ym, out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}

extern "C" int fteik_correlate1d(int nd, const double* in, const int* dims, int axis,
                                 const double* weights, int nweights, double* out,
                                 void* stream) {
  if (!dims_ok(nd, dims) || axis < 0 || axis >= nd || !in || !out || !weights ||
      nweights < 1 || (nweights & 1) == 0 || in == out)
    return kInvalidArgument;
  long long outer = 1, inner = 1;
  for (int d = 0; d < axis; ++d) outer *= dims[d];
  for (int d = axis + 1; d < nd; ++d) inner *= dims[d];
  const long long total = outer * dims[axis] * inner;
  correlate1d_kernel<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(
      in, outer, dims[axis], inner, weights, nweights, out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}
