// Device-side interpolation shared by the interpolation and ray-tracing
// kernels: fteikpy/_interp/_interp2d.py, _interp3d.py, _vinterp2d.py,
// _vinterp3d.py restated operation by operation.
//
// Axis lookup: np.searchsorted(a, v, side="right") - 1 on an ascending axis.
// A float guess from the axis span picks the cell, then exact double
// comparisons against the stored axis values confirm it (falling back to a
// bisection), so the index is exactly the reference's for any ascending axis.
#pragma once
#include "common.cuh"

namespace fteik {

__device__ __forceinline__ int search_right_m1(const double* __restrict__ a, int n, double v) {
  if (!(v == v)) return n - 1;  // numpy orders NaN after every number
  const double a0 = __ldg(a), an = __ldg(a + n - 1);
  if (v < a0) return -1;
  if (v >= an) {
    // every element is <= v
    return n - 1;
  }
  // here a0 <= v < an, so the answer lies in [0, n-2]
  int g = (int)(__fdividef((float)(v - a0), (float)(an - a0)) * (float)(n - 1));
  g = g < 0 ? 0 : (g > n - 2 ? n - 2 : g);
  int lo, hi;  // invariant: a[lo] <= v < a[hi]
  if (__ldg(a + g) <= v) {
    if (v < __ldg(a + g + 1)) return g;
    lo = g + 1;
    hi = n - 1;
  } else {
    lo = 0;
    hi = g;
  }
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(a + mid) <= v)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ double dist3(double x1, double y1, double z1, double x2, double y2,
                                        double z2) {
  const double a = x1 - x2, b = y1 - y2, c = z1 - z2;
  return sqrt_rn(a * a + b * b + c * c);
}
__device__ __forceinline__ double dist2(double x1, double y1, double x2, double y2) {
  const double a = x1 - x2, b = y1 - y2;
  return sqrt_rn(a * a + b * b);
}

// Cell of a query point inside the axes (the bounds check done by the caller):
// corner coordinates and the "last node" flags of _interp3d.py:21-162.
struct Cell3 {
  int i1, j1, k1;
  bool ei, ej, ek;
  double x1, x2, y1, y2, z1, z2;
};

__device__ __forceinline__ Cell3 locate3(const double* x, int nx, const double* y, int ny,
                                         const double* z, int nz, double xq, double yq,
                                         double zq) {
  Cell3 c;
  c.i1 = search_right_m1(x, nx, xq);
  c.j1 = search_right_m1(y, ny, yq);
  c.k1 = search_right_m1(z, nz, zq);
  c.ei = c.i1 == nx - 1;
  c.ej = c.j1 == ny - 1;
  c.ek = c.k1 == nz - 1;
  c.x1 = __ldg(x + c.i1);
  c.y1 = __ldg(y + c.j1);
  c.z1 = __ldg(z + c.k1);
  c.x2 = c.ei ? 2.0 * c.x1 - __ldg(x + nx - 2) : __ldg(x + c.i1 + 1);
  c.y2 = c.ej ? 2.0 * c.y1 - __ldg(y + ny - 2) : __ldg(y + c.j1 + 1);
  c.z2 = c.ek ? 2.0 * c.z1 - __ldg(z + nz - 2) : __ldg(z + c.k1 + 1);
  return c;
}

__device__ __forceinline__ bool inside3(const double* x, int nx, const double* y, int ny,
                                        const double* z, int nz, double xq, double yq,
                                        double zq) {
  return (__ldg(x) <= xq && xq <= __ldg(x + nx - 1)) && (__ldg(y) <= yq && yq <= __ldg(y + ny - 1)) &&
         (__ldg(z) <= zq && zq <= __ldg(z + nz - 1));
}

// The 8 trilinear weights |(x? - xq)(y? - yq)(z? - zq)| of _interp3d.py:164-171,
// in the order 111, 211, 121, 221, 112, 212, 122, 222.
__device__ __forceinline__ void weights3(const Cell3& c, double xq, double yq, double zq,
                                         double (&w)[8]) {
  w[0] = fabs((c.x2 - xq) * (c.y2 - yq) * (c.z2 - zq));
  w[1] = fabs((c.x1 - xq) * (c.y2 - yq) * (c.z2 - zq));
  w[2] = fabs((c.x2 - xq) * (c.y1 - yq) * (c.z2 - zq));
  w[3] = fabs((c.x1 - xq) * (c.y1 - yq) * (c.z2 - zq));
  w[4] = fabs((c.x2 - xq) * (c.y2 - yq) * (c.z1 - zq));
  w[5] = fabs((c.x1 - xq) * (c.y2 - yq) * (c.z1 - zq));
  w[6] = fabs((c.x2 - xq) * (c.y1 - yq) * (c.z1 - zq));
  w[7] = fabs((c.x1 - xq) * (c.y1 - yq) * (c.z1 - zq));
}

// Corner values v111 .. v222 (1.0 past the last node) read with element
// stride vs, _interp3d.py:28-162.
__device__ __forceinline__ void corners3(const double* __restrict__ v, long long vs,
                                         const Cell3& c, int ny, int nz, double (&q)[8]) {
  const long long b = ((long long)c.i1 * ny + c.j1) * nz + c.k1;
  const long long di = (long long)ny * nz, dj = nz, dk = 1;
  q[0] = __ldg(v + b * vs);
  q[1] = c.ei ? 1.0 : __ldg(v + (b + di) * vs);
  q[2] = c.ej ? 1.0 : __ldg(v + (b + dj) * vs);
  q[3] = (c.ei || c.ej) ? 1.0 : __ldg(v + (b + di + dj) * vs);
  q[4] = c.ek ? 1.0 : __ldg(v + (b + dk) * vs);
  q[5] = (c.ei || c.ek) ? 1.0 : __ldg(v + (b + di + dk) * vs);
  q[6] = (c.ej || c.ek) ? 1.0 : __ldg(v + (b + dj + dk) * vs);
  q[7] = (c.ei || c.ej || c.ek) ? 1.0 : __ldg(v + (b + di + dj + dk) * vs);
}

__device__ __forceinline__ double blend3(const Cell3& c, const double (&q)[8],
                                         const double (&w)[8]) {
  double vq = q[0] * w[0];
#pragma unroll
  for (int t = 1; t < 8; ++t) vq += q[t] * w[t];
  vq /= fabs((c.x2 - c.x1) * (c.y2 - c.y1) * (c.z2 - c.z1));
  return vq;
}

// _interp3d, _interp3d.py:7-174.
__device__ __forceinline__ double interp3_point(const double* x, int nx, const double* y, int ny,
                                                const double* z, int nz, const double* v,
                                                long long vs, double xq, double yq, double zq,
                                                double fval) {
  if (!inside3(x, nx, y, ny, z, nz, xq, yq, zq)) return fval;
  const Cell3 c = locate3(x, nx, y, ny, z, nz, xq, yq, zq);
  double w[8], q[8];
  weights3(c, xq, yq, zq, w);
  corners3(v, vs, c, ny, nz, q);
  return blend3(c, q, w);
}

// _vinterp3d, _vinterp3d.py:7-264.
__device__ __forceinline__ double vinterp3_point(const double* x, int nx, const double* y,
                                                 int ny, const double* z, int nz,
                                                 const double* v, double xq, double yq,
                                                 double zq, double xs, double ys, double zs,
                                                 double vzero, double fval) {
  if (!inside3(x, nx, y, ny, z, nz, xq, yq, zq)) return fval;
  const int xsi = search_right_m1(x, nx, xs), ysi = search_right_m1(y, ny, ys),
            zsi = search_right_m1(z, nz, zs);
  const Cell3 c = locate3(x, nx, y, ny, z, nz, xq, yq, zq);
  if (xsi == c.i1 && ysi == c.j1 && zsi == c.k1) return vzero * dist3(xs, ys, zs, xq, yq, zq);
  double q[8];
  corners3(v, 1, c, ny, nz, q);
  double d[8];
  d[0] = dist3(xs, ys, zs, c.x1, c.y1, c.z1);
  d[1] = c.ei ? 0.0 : dist3(xs, ys, zs, c.x2, c.y1, c.z1);
  d[2] = c.ej ? 0.0 : dist3(xs, ys, zs, c.x1, c.y2, c.z1);
  d[3] = (c.ei || c.ej) ? 0.0 : dist3(xs, ys, zs, c.x2, c.y2, c.z1);
  d[4] = c.ek ? 0.0 : dist3(xs, ys, zs, c.x1, c.y1, c.z2);
  d[5] = (c.ei || c.ek) ? 0.0 : dist3(xs, ys, zs, c.x2, c.y1, c.z2);
  d[6] = (c.ej || c.ek) ? 0.0 : dist3(xs, ys, zs, c.x1, c.y2, c.z2);
  d[7] = (c.ei || c.ej || c.ek) ? 0.0 : dist3(xs, ys, zs, c.x2, c.y2, c.z2);
  bool all_nonzero = true;
#pragma unroll
  for (int t = 0; t < 8; ++t) all_nonzero = all_nonzero && (q[t] != 0.0);
  if (!all_nonzero) return vzero * dist3(xs, ys, zs, xq, yq, zq);
  double w[8];
  weights3(c, xq, yq, zq, w);
  double vq = d[0] / q[0] * w[0];
#pragma unroll
  for (int t = 1; t < 8; ++t) vq += d[t] / q[t] * w[t];
  vq /= fabs((c.x2 - c.x1) * (c.y2 - c.y1) * (c.z2 - c.z1));
  return dist3(xs, ys, zs, xq, yq, zq) / vq;
}

// ---- 2D ------------------------------------------------------------------------

struct Cell2 {
  int i1, j1;
  bool ei, ej;
  double x1, x2, y1, y2;
};

__device__ __forceinline__ bool inside2(const double* x, int nx, const double* y, int ny,
                                        double xq, double yq) {
  return (__ldg(x) <= xq && xq <= __ldg(x + nx - 1)) && (__ldg(y) <= yq && yq <= __ldg(y + ny - 1));
}

__device__ __forceinline__ Cell2 locate2(const double* x, int nx, const double* y, int ny,
                                         double xq, double yq) {
  Cell2 c;
  c.i1 = search_right_m1(x, nx, xq);
  c.j1 = search_right_m1(y, ny, yq);
  c.ei = c.i1 == nx - 1;
  c.ej = c.j1 == ny - 1;
  c.x1 = __ldg(x + c.i1);
  c.y1 = __ldg(y + c.j1);
  c.x2 = c.ei ? 2.0 * c.x1 - __ldg(x + nx - 2) : __ldg(x + c.i1 + 1);
  c.y2 = c.ej ? 2.0 * c.y1 - __ldg(y + ny - 2) : __ldg(y + c.j1 + 1);
  return c;
}

__device__ __forceinline__ void weights2(const Cell2& c, double xq, double yq, double (&w)[4]) {
  w[0] = fabs((c.x2 - xq) * (c.y2 - yq));
  w[1] = fabs((c.x1 - xq) * (c.y2 - yq));
  w[2] = fabs((c.x2 - xq) * (c.y1 - yq));
  w[3] = fabs((c.x1 - xq) * (c.y1 - yq));
}

__device__ __forceinline__ void corners2(const double* __restrict__ v, long long vs,
                                         const Cell2& c, int ny, double (&q)[4]) {
  const long long b = (long long)c.i1 * ny + c.j1;
  q[0] = __ldg(v + b * vs);
  q[1] = c.ei ? 1.0 : __ldg(v + (b + ny) * vs);
  q[2] = c.ej ? 1.0 : __ldg(v + (b + 1) * vs);
  q[3] = (c.ei || c.ej) ? 1.0 : __ldg(v + (b + ny + 1) * vs);
}

// _interp2d, _interp2d.py:7-74.
__device__ __forceinline__ double interp2_point(const double* x, int nx, const double* y, int ny,
                                                const double* v, long long vs, double xq,
                                                double yq, double fval) {
  if (!inside2(x, nx, y, ny, xq, yq)) return fval;
  const Cell2 c = locate2(x, nx, y, ny, xq, yq);
  double w[4], q[4];
  weights2(c, xq, yq, w);
  corners2(v, vs, c, ny, q);
  double vq = q[0] * w[0];
  vq += q[1] * w[1];
  vq += q[2] * w[2];
  vq += q[3] * w[3];
  vq /= fabs((c.x2 - c.x1) * (c.y2 - c.y1));
  return vq;
}

// _vinterp2d, _vinterp2d.py:7-108.
__device__ __forceinline__ double vinterp2_point(const double* x, int nx, const double* y,
                                                 int ny, const double* v, double xq, double yq,
                                                 double xs, double ys, double vzero,
                                                 double fval) {
  if (!inside2(x, nx, y, ny, xq, yq)) return fval;
  const int xsi = search_right_m1(x, nx, xs), ysi = search_right_m1(y, ny, ys);
  const Cell2 c = locate2(x, nx, y, ny, xq, yq);
  if (xsi == c.i1 && ysi == c.j1) return vzero * dist2(xs, ys, xq, yq);
  double q[4];
  corners2(v, 1, c, ny, q);
  double d[4];
  d[0] = dist2(xs, ys, c.x1, c.y1);
  d[1] = c.ei ? 0.0 : dist2(xs, ys, c.x2, c.y1);
  d[2] = c.ej ? 0.0 : dist2(xs, ys, c.x1, c.y2);
  d[3] = (c.ei || c.ej) ? 0.0 : dist2(xs, ys, c.x2, c.y2);
  if (!(q[0] != 0.0 && q[1] != 0.0 && q[2] != 0.0 && q[3] != 0.0))
    return vzero * dist2(xs, ys, xq, yq);
  double w[4];
  weights2(c, xq, yq, w);
  double vq = d[0] / q[0] * w[0];
  vq += d[1] / q[1] * w[1];
  vq += d[2] / q[2] * w[2];
  vq += d[3] / q[3] * w[3];
  vq /= fabs((c.x2 - c.x1) * (c.y2 - c.y1));
  return dist2(xs, ys, xq, yq) / vq;
}

}  // namespace fteik
