// A-posteriori ray tracing: fteikpy/_fteik/_ray3d.py, _ray2d.py and the
// step-shrinking helper _fteik/_common.py restated for the GPU, one thread per
// ray (the reference's prange over end points, _ray3d.py:145).
//
// Per step the reference interpolates each gradient component separately
// (_ray3d.py:60-62); the three calls share the query point, so the cell lookup
// and the 8 weights are computed once here and applied to the three
// components, which gives the same numbers.
//
// On GB300 one warp's FP64 instruction occupies the FP64 pipe for 64 cycles
// (a compare for about 105, a sqrt or a division for about 600), whatever the
// number of active lanes, so a ray step is timed by its FP64 instruction
// count.  Work that can leave the pipe without changing a result bit does:
// comparisons of positions against axis values use integer order keys, the
// cell guess is a float computation confirmed by exact comparisons, the
// "distance to the source >= stepsize" test compares the squared distance
// with the exact threshold of RN(sqrt(x)) >= stepsize (found on the host),
// and on axes with one spacing the blend's division by the cell volume uses
// the correctly rounded constant-divisor division of common.cuh.
//
// One intentional difference: when a honor_grid step lands exactly on the last
// node of an axis, the reference reads one element past the end of that axis
// (_ray3d.py:96-98, _ray2d.py:69-70); here the index is clamped to the last
// node, as the reference itself does when it sets up the first cell
// (_ray3d.py:46-48).
#include <math_constants.h>

#include <cmath>

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

// Order key of a non-NaN double in which -0.0 and +0.0 are equal:
// zkey(a) < zkey(b) <=> a < b.
__device__ __forceinline__ long long zkey(double x) {
  // |x|'s pattern from 32-bit words: a 64-bit mask of the sign bit would be
  // compiled as an FP64 absolute value
  const int h = __double2hiint(x);
  const long long m = ((long long)(h & 0x7fffffff) << 32) | (unsigned)__double2loint(x);
  return h < 0 ? -m : m;
}

// Per-axis constants of one launch, set up by every block in shared memory.
struct RayAxis {
  double lo, hi;       // first and last node
  long long klo, khi;  // their order keys
  float f0, fs;        // cell guess (float(v) - f0) * fs
  int uniform;         // every cell (and the last-node extension) has x2 - x1 == d
  double d;
};

// np.searchsorted(a, v, "right") - 1 for a finite v with lo <= v <= hi: the
// float guess, confirmed (or moved by one) with exact comparisons, else a
// bisection.
__device__ __forceinline__ int ray_search(const double* __restrict__ a, int n,
                                          const RayAxis& X, double v, long long kv) {
  if (kv >= X.khi) return n - 1;
  int g = (int)(((float)v - X.f0) * X.fs);
  g = g < 0 ? 0 : (g > n - 2 ? n - 2 : g);
  const long long kg = zkey(__ldg(a + g));
  int lo, hi;  // invariant: a[lo] <= v < a[hi]
  if (kg <= kv) {
    const long long kg1 = zkey(__ldg(a + g + 1));
    if (kv < kg1) return g;
    if (g + 2 > n - 1 || kv < zkey(__ldg(a + g + 2))) return g + 1;  // a[n-1] > v here
    lo = g + 2;
    hi = n - 1;
  } else {
    if (g > 0 && zkey(__ldg(a + g - 1)) <= kv) return g - 1;
    lo = 0;
    hi = g;
  }
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (zkey(__ldg(a + mid)) <= kv)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Per-launch state every block sets up in shared memory.
struct RayShared {
  RayAxis X[3];
  Recip vol;      // 1 / cell volume when every axis has one spacing
  int uni;        // 1: divide blends with `vol`
  double vol_c;   // the cell volume
};

// RN(x / cell volume) as _interp3d computes it: the constant-divisor
// division where it is exact (one spacing per axis, x normal and far from
// overflow and underflow), else IEEE division by the volume of cell c.
__device__ __forceinline__ double per_volume(double x, double vol_c, const Recip& R, bool uni) {
  const int e = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  if (uni && e >= 300 && e <= 1700) return div_by(x, R);
  return x / vol_c;
}

// Component `comp` of the gradient at p (the reference interpolates each
// component with _interp3d / _interp2d, _ray3d.py:60-62): NaN outside.
template <int ND>
__device__ __forceinline__ double grad_comp(const Axes& ax, const RayShared& S, const double* g,
                                            const double* p, const long long* kp, int comp) {
  bool inside = true;
#pragma unroll
  for (int q = 0; q < ND; ++q) inside = inside && S.X[q].klo <= kp[q] && kp[q] <= S.X[q].khi;
  if (!inside) return CUDART_NAN;
  if (ND == 3) {
    Cell3 c;
    c.i1 = ray_search(ax.a[0], ax.n[0], S.X[0], p[0], kp[0]);
    c.j1 = ray_search(ax.a[1], ax.n[1], S.X[1], p[1], kp[1]);
    c.k1 = ray_search(ax.a[2], ax.n[2], S.X[2], p[2], kp[2]);
    const int nx = ax.n[0], ny = ax.n[1], nz = ax.n[2];
    c.ei = c.i1 == nx - 1;
    c.ej = c.j1 == ny - 1;
    c.ek = c.k1 == nz - 1;
    c.x1 = __ldg(ax.a[0] + c.i1);
    c.y1 = __ldg(ax.a[1] + c.j1);
    c.z1 = __ldg(ax.a[2] + c.k1);
    c.x2 = c.ei ? 2.0 * c.x1 - __ldg(ax.a[0] + nx - 2) : __ldg(ax.a[0] + c.i1 + 1);
    c.y2 = c.ej ? 2.0 * c.y1 - __ldg(ax.a[1] + ny - 2) : __ldg(ax.a[1] + c.j1 + 1);
    c.z2 = c.ek ? 2.0 * c.z1 - __ldg(ax.a[2] + nz - 2) : __ldg(ax.a[2] + c.k1 + 1);
    double w[8], q[8];
    corners3(g + comp, 3, c, ny, nz, q);
    weights3(c, p[0], p[1], p[2], w);
    double vq = q[0] * w[0];
#pragma unroll
    for (int t = 1; t < 8; ++t) vq += q[t] * w[t];
    const double vol = S.uni ? S.vol_c : fabs((c.x2 - c.x1) * (c.y2 - c.y1) * (c.z2 - c.z1));
    return per_volume(vq, vol, S.vol, S.uni != 0);
  } else {
    Cell2 c;
    c.i1 = ray_search(ax.a[0], ax.n[0], S.X[0], p[0], kp[0]);
    c.j1 = ray_search(ax.a[1], ax.n[1], S.X[1], p[1], kp[1]);
    const int nx = ax.n[0], ny = ax.n[1];
    c.ei = c.i1 == nx - 1;
    c.ej = c.j1 == ny - 1;
    c.x1 = __ldg(ax.a[0] + c.i1);
    c.y1 = __ldg(ax.a[1] + c.j1);
    c.x2 = c.ei ? 2.0 * c.x1 - __ldg(ax.a[0] + nx - 2) : __ldg(ax.a[0] + c.i1 + 1);
    c.y2 = c.ej ? 2.0 * c.y1 - __ldg(ax.a[1] + ny - 2) : __ldg(ax.a[1] + c.j1 + 1);
    double w[4], q[4];
    corners2(g + comp, 2, c, ny, q);
    weights2(c, p[0], p[1], w);
    double vq = q[0] * w[0];
    vq += q[1] * w[1];
    vq += q[2] * w[2];
    vq += q[3] * w[3];
    const double vol = S.uni ? S.vol_c : fabs((c.x2 - c.x1) * (c.y2 - c.y1));
    return per_volume(vq, vol, S.vol, S.uni != 0);
  }
}

// All components at p (one lane per ray): the lookup and weights once.
template <int ND>
__device__ __forceinline__ void grad_at(const Axes& ax, const RayShared& S, const double* g,
                                        const double* p, const long long* kp, double* out) {
  bool inside = true;
#pragma unroll
  for (int q = 0; q < ND; ++q) inside = inside && S.X[q].klo <= kp[q] && kp[q] <= S.X[q].khi;
  if (!inside) {
#pragma unroll
    for (int q = 0; q < ND; ++q) out[q] = CUDART_NAN;
    return;
  }
  if (ND == 3) {
    Cell3 c;
    c.i1 = ray_search(ax.a[0], ax.n[0], S.X[0], p[0], kp[0]);
    c.j1 = ray_search(ax.a[1], ax.n[1], S.X[1], p[1], kp[1]);
    c.k1 = ray_search(ax.a[2], ax.n[2], S.X[2], p[2], kp[2]);
    const int nx = ax.n[0], ny = ax.n[1], nz = ax.n[2];
    c.ei = c.i1 == nx - 1;
    c.ej = c.j1 == ny - 1;
    c.ek = c.k1 == nz - 1;
    c.x1 = __ldg(ax.a[0] + c.i1);
    c.y1 = __ldg(ax.a[1] + c.j1);
    c.z1 = __ldg(ax.a[2] + c.k1);
    c.x2 = c.ei ? 2.0 * c.x1 - __ldg(ax.a[0] + nx - 2) : __ldg(ax.a[0] + c.i1 + 1);
    c.y2 = c.ej ? 2.0 * c.y1 - __ldg(ax.a[1] + ny - 2) : __ldg(ax.a[1] + c.j1 + 1);
    c.z2 = c.ek ? 2.0 * c.z1 - __ldg(ax.a[2] + nz - 2) : __ldg(ax.a[2] + c.k1 + 1);
    double w[8];
    weights3(c, p[0], p[1], p[2], w);
    const double vol = S.uni ? S.vol_c : fabs((c.x2 - c.x1) * (c.y2 - c.y1) * (c.z2 - c.z1));
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      double q[8];
      corners3(g + comp, 3, c, ny, nz, q);
      double vq = q[0] * w[0];
#pragma unroll
      for (int t = 1; t < 8; ++t) vq += q[t] * w[t];
      out[comp] = per_volume(vq, vol, S.vol, S.uni != 0);
    }
  } else {
    Cell2 c;
    c.i1 = ray_search(ax.a[0], ax.n[0], S.X[0], p[0], kp[0]);
    c.j1 = ray_search(ax.a[1], ax.n[1], S.X[1], p[1], kp[1]);
    const int nx = ax.n[0], ny = ax.n[1];
    c.ei = c.i1 == nx - 1;
    c.ej = c.j1 == ny - 1;
    c.x1 = __ldg(ax.a[0] + c.i1);
    c.y1 = __ldg(ax.a[1] + c.j1);
    c.x2 = c.ei ? 2.0 * c.x1 - __ldg(ax.a[0] + nx - 2) : __ldg(ax.a[0] + c.i1 + 1);
    c.y2 = c.ej ? 2.0 * c.y1 - __ldg(ax.a[1] + ny - 2) : __ldg(ax.a[1] + c.j1 + 1);
    double w[4];
    weights2(c, p[0], p[1], w);
    const double vol = S.uni ? S.vol_c : fabs((c.x2 - c.x1) * (c.y2 - c.y1));
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      double q[4];
      corners2(g + comp, 2, c, ny, q);
      double vq = q[0] * w[0];
      vq += q[1] * w[1];
      vq += q[2] * w[2];
      vq += q[3] * w[3];
      out[comp] = per_volume(vq, vol, S.vol, S.uni != 0);
    }
  }
}

// The block's shared set-up: axis ends and keys, the float guess, and
// whether every axis has a single spacing d (a[i+1] - a[i] == d for every
// cell and for the last-node extension 2*a[n-1] - a[n-2]), which makes every
// cell volume the same double.
template <int ND>
__device__ __forceinline__ void ray_setup(const Axes& ax, RayShared& S) {
  if (threadIdx.x < ND) {
    const int q = threadIdx.x;
    const double* a = ax.a[q];
    const int n = ax.n[q];
    RayAxis& X = S.X[q];
    X.lo = __ldg(a);
    X.hi = __ldg(a + n - 1);
    X.klo = zkey(X.lo);
    X.khi = zkey(X.hi);
    X.f0 = (float)X.lo;
    const float span = (float)X.hi - X.f0;
    X.fs = span > 0.0f ? (float)(n - 1) / span : 0.0f;
    X.d = __ldg(a + 1) - __ldg(a);
    X.uniform = deq((2.0 * X.hi - __ldg(a + n - 2)) - X.hi, X.d) ? 1 : 0;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < ND; ++q) {
    const double* a = ax.a[q];
    bool ok = true;
    for (int i = threadIdx.x; i < ax.n[q] - 1; i += blockDim.x)
      ok = ok && deq(__ldg(a + i + 1) - __ldg(a + i), S.X[q].d);
    if (!ok) S.X[q].uniform = 0;  // benign race: every writer stores 0
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    bool uni = true;
    double vol = 1.0;
#pragma unroll
    for (int q = 0; q < ND; ++q) {
      uni = uni && S.X[q].uniform;
      vol = vol * S.X[q].d;
    }
    vol = fabs(vol);
    // the constant-divisor division wants a normal divisor of moderate size
    const int e = (int)((__double_as_longlong(vol) >> 52) & 0x7ff);
    uni = uni && e >= 823 && e <= 1223;
    S.uni = uni ? 1 : 0;
    S.vol_c = vol;
    S.vol = make_recip(uni ? vol : 1.0);
  }
  __syncthreads();
}

// _ray3d / _ray2d, _ray3d.py:9-120 and _ray2d.py:9-91.
// L lanes trace one ray: with L = 4, lanes 0..ND-1 of the group each blend
// one gradient component and the group shares them, so a few rays (one
// source's receivers) take fewer dependent FP64 instructions per step; the
// other work is done identically by every lane and lane 0 writes.
// `dist_min` is the least double x with RN(sqrt(x)) >= stepsize, so the
// reference's `dist(src, p) >= stepsize` is `squared distance >= dist_min`.
template <int ND, int L>
__global__ void ray_kernel(Axes ax, const double* ttgrad, long long gstride, const int* gidx,
                           const double* ends, int nrays, const double* sources,
                           double stepsize, double dist_min, int max_step, int honor_grid,
                           double* rays, int* counts, int* status) {
  __shared__ RayShared S;
  ray_setup<ND>(ax, S);
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int r = (int)(tid / L);
  const int sub = (int)(tid % L);
  const bool writer = sub == 0;
  const unsigned gmask = L == 1 ? 0u : (((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1)));
  if (r >= nrays) return;
  const int gi = gidx ? gidx[r] : 0;
  const double* g = ttgrad + (long long)gi * gstride;
  const long long kmin = __double_as_longlong(dist_min);
  double src[ND], pcur[ND], delta[ND], lower[ND], upper[ND];
  long long kp[ND];
  int isrc[ND];
#pragma unroll
  for (int q = 0; q < ND; ++q) {
    src[q] = sources[ND * gi + q];
    pcur[q] = ends[ND * r + q];
  }
  if (writer) counts[r] = 0;
#pragma unroll
  for (int q = 0; q < ND; ++q) {
    if (!(S.X[q].lo <= pcur[q] && pcur[q] <= S.X[q].hi)) {
      if (writer) status[r] = kEndPointOutOfBound;
      return;
    }
    kp[q] = zkey(pcur[q]);
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
    // dist(src, pcur) >= stepsize: the squared distance is a sum of squares,
    // so as a bit pattern it orders like its value; NaN (a NaN position)
    // fails the reference's test
    double dsq;
    if (ND == 3) {
      const double a = src[0] - pcur[0], b = src[1] - pcur[1], c = src[2] - pcur[2];
      dsq = a * a + b * b + c * c;
    } else {
      const double a = src[0] - pcur[0], b = src[1] - pcur[1];
      dsq = a * a + b * b;
    }
    const long long db = __double_as_longlong(dsq);
    if (db < kmin || db > 0x7ff0000000000000LL) break;
    double gv[ND];
    if (L == 1) {
      grad_at<ND>(ax, S, g, pcur, kp, gv);
    } else {
      const double mine = sub < ND ? grad_comp<ND>(ax, S, g, pcur, kp, sub) : 0.0;
#pragma unroll
      for (int q = 0; q < ND; ++q) gv[q] = __shfl_sync(gmask, mine, q, L);
    }
    double gsq = gv[0] * gv[0] + gv[1] * gv[1];
    if (ND == 3) gsq = gsq + gv[ND - 1] * gv[ND - 1];
    // gn = sqrt(gsq) > 0 unless gsq is +0 or NaN (a sum of squares)
    const long long gb = __double_as_longlong(gsq);
    if (gb == 0 || gb > 0x7ff0000000000000LL) break;
    const double gni = 1.0 / sqrt_rn(gsq);
#pragma unroll
    for (int q = 0; q < ND; ++q) delta[q] = stepsize * gv[q] * gni;
    if (honor_grid) {
      const double fac = shrink<ND>(pcur, delta, lower, upper);
#pragma unroll
      for (int q = 0; q < ND; ++q) {
        double v = pcur[q] - fac * delta[q];
        const double lo = S.X[q].lo, hi = S.X[q].hi;
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
#pragma unroll
      for (int q = 0; q < ND; ++q) kp[q] = zkey(pcur[q]);
    } else {
#pragma unroll
      for (int q = 0; q < ND; ++q) {
        // max(axis[0], min(axis[-1], pcur - delta)) with the comparisons on
        // keys; a NaN compares false with both ends and stays
        double v = pcur[q] - delta[q];
        long long kv = zkey(v);
        const bool nan = (kv < 0 ? -kv : kv) > 0x7ff0000000000000LL;
        if (!nan && S.X[q].klo > kv) {
          v = S.X[q].lo;
          kv = S.X[q].klo;
        }
        if (!nan && S.X[q].khi < kv) {
          v = S.X[q].hi;
          kv = S.X[q].khi;
        }
        pcur[q] = v;
        kp[q] = kv;
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

// The same rays without honor_grid, four lanes per ray, where lane q of the
// group owns axis q (lanes past the last axis repeat it): its term of the
// squared distance, its cell search and corner coordinates, its two weight
// differences, its gradient component's blend, its coordinate's step and
// clamp, and its coordinate of each ray point.  The group exchanges only
// what the others need by shuffles, so a step issues each axis's integer
// work once instead of once per axis on every lane.  Every value is the same
// IEEE operation on the same operands as in ray_kernel, so the rays are the
// same bits.
template <int ND>
__global__ void ray_axis_kernel(Axes ax, const double* ttgrad, long long gstride,
                                const int* gidx, const double* ends, int nrays,
                                const double* sources, double stepsize, double dist_min,
                                int max_step, double* rays, int* counts, int* status) {
  __shared__ RayShared S;
  ray_setup<ND>(ax, S);
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int r = (int)(tid >> 2);
  const int sub = (int)(tid & 3);
  const int q = sub < ND ? sub : ND - 1;
  const int g0 = (threadIdx.x & 31) & ~3;  // first lane of the group
  const unsigned gmask = 0xfu << g0;
  const unsigned all_axes = (1u << ND) - 1u;
  if (r >= nrays) return;
  const int gi = gidx ? gidx[r] : 0;
  const double* g = ttgrad + (long long)gi * gstride;
  // (selects, not an index into the parameter block, which would copy it to
  // local memory)
  const double* a = q == 0 ? ax.a[0] : (q == 1 ? ax.a[1] : ax.a[ND - 1]);
  const int n = q == 0 ? ax.n[0] : (q == 1 ? ax.n[1] : ax.n[ND - 1]);
  const RayAxis& X = S.X[q];
  const double sq = sources[ND * gi + q];
  double p = ends[ND * r + q];
  const long long kmin = __double_as_longlong(dist_min);
  if (sub == 0) counts[r] = 0;
  if (((__ballot_sync(gmask, X.lo <= p && p <= X.hi) >> g0) & all_axes) != all_axes) {
    if (sub == 0) status[r] = kEndPointOutOfBound;
    return;
  }
  long long kp = zkey(p);
  double* ray = rays + (long long)r * max_step * ND;
  int count = 1;
  if (sub < ND) ray[q] = p;
  const long long max_iter = 64LL * max_step + 4096;
  for (long long iter = 0;; ++iter) {
    if (iter >= max_iter) {
      if (sub == 0) status[r] = kMaxStepReached;
      return;
    }
    // dist(src, pcur) >= stepsize on the squared distance (a*a + b*b) + c*c
    const double dq = sq - p;
    const double s2 = dq * dq;
    double dsq = __shfl_sync(gmask, s2, g0) + __shfl_sync(gmask, s2, g0 + 1);
    if (ND == 3) dsq = dsq + __shfl_sync(gmask, s2, g0 + 2);
    const long long db = __double_as_longlong(dsq);
    if (db < kmin || db > 0x7ff0000000000000LL) break;
    // outside the grid the gradient is NaN and the reference's loop ends
    if (((__ballot_sync(gmask, X.klo <= kp && kp <= X.khi) >> g0) & all_axes) != all_axes) break;
    // this lane's axis: cell, corner coordinates, weight differences
    const int c = ray_search(a, n, X, p, kp);
    const bool e = c == n - 1;
    const double x1 = __ldg(a + c);
    const double x2 = e ? 2.0 * x1 - __ldg(a + n - 2) : __ldg(a + c + 1);
    const double lo = x1 - p, hi = x2 - p, span = x2 - x1;
    double L[ND], H[ND];
    int ci[ND];
    bool ce[ND];
#pragma unroll
    for (int t = 0; t < ND; ++t) {
      L[t] = __shfl_sync(gmask, lo, g0 + t);
      H[t] = __shfl_sync(gmask, hi, g0 + t);
      const int packed = __shfl_sync(gmask, (c << 1) | (e ? 1 : 0), g0 + t);
      ci[t] = packed >> 1;
      ce[t] = (packed & 1) != 0;
    }
    double vol = S.vol_c;
    if (!S.uni) {
      vol = __shfl_sync(gmask, span, g0) * __shfl_sync(gmask, span, g0 + 1);
      if (ND == 3) vol = vol * __shfl_sync(gmask, span, g0 + 2);
      vol = fabs(vol);
    }
    double mine;
    if (ND == 3) {
      // weights3: |((x? - xq) * (y? - yq)) * (z? - zq)|, 111, 211, 121, 221, 112, ...
      const double hh = H[0] * H[1], lh = L[0] * H[1], hl = H[0] * L[1], ll = L[0] * L[1];
      double w[8];
      w[0] = fabs(hh * H[ND - 1]);
      w[1] = fabs(lh * H[ND - 1]);
      w[2] = fabs(hl * H[ND - 1]);
      w[3] = fabs(ll * H[ND - 1]);
      w[4] = fabs(hh * L[ND - 1]);
      w[5] = fabs(lh * L[ND - 1]);
      w[6] = fabs(hl * L[ND - 1]);
      w[7] = fabs(ll * L[ND - 1]);
      Cell3 cc;
      cc.i1 = ci[0];
      cc.j1 = ci[1];
      cc.k1 = ci[ND - 1];
      cc.ei = ce[0];
      cc.ej = ce[1];
      cc.ek = ce[ND - 1];
      double qv[8];
      corners3(g + q, 3, cc, ax.n[1], ax.n[ND - 1], qv);
      double vq = qv[0] * w[0];
#pragma unroll
      for (int t = 1; t < 8; ++t) vq += qv[t] * w[t];
      mine = per_volume(vq, vol, S.vol, S.uni != 0);
    } else {
      double w[4];
      w[0] = fabs(H[0] * H[1]);
      w[1] = fabs(L[0] * H[1]);
      w[2] = fabs(H[0] * L[1]);
      w[3] = fabs(L[0] * L[1]);
      Cell2 cc;
      cc.i1 = ci[0];
      cc.j1 = ci[1];
      cc.ei = ce[0];
      cc.ej = ce[1];
      double qv[4];
      corners2(g + q, 2, cc, ax.n[1], qv);
      double vq = qv[0] * w[0];
      vq += qv[1] * w[1];
      vq += qv[2] * w[2];
      vq += qv[3] * w[3];
      mine = per_volume(vq, vol, S.vol, S.uni != 0);
    }
    double gv[ND];
#pragma unroll
    for (int t = 0; t < ND; ++t) gv[t] = __shfl_sync(gmask, mine, g0 + t);
    double gsq = gv[0] * gv[0] + gv[1] * gv[1];
    if (ND == 3) gsq = gsq + gv[ND - 1] * gv[ND - 1];
    const long long gb = __double_as_longlong(gsq);
    if (gb == 0 || gb > 0x7ff0000000000000LL) break;
    const double gni = 1.0 / sqrt_rn(gsq);
    // this lane's coordinate: max(axis[0], min(axis[-1], p - stepsize * g * gni))
    double v = p - stepsize * mine * gni;
    long long kv = zkey(v);
    const bool nan = (kv < 0 ? -kv : kv) > 0x7ff0000000000000LL;
    if (!nan && X.klo > kv) {
      v = X.lo;
      kv = X.klo;
    }
    if (!nan && X.khi < kv) {
      v = X.hi;
      kv = X.khi;
    }
    p = v;
    kp = kv;
    if (sub < ND) ray[count * ND + q] = v;
    count += 1;
    if (count >= max_step) {
      if (sub == 0) status[r] = kMaxStepReached;
      return;
    }
  }
  if (sub < ND) ray[count * ND + q] = sq;
  if (sub == 0) {
    counts[r] = count;
    status[r] = kOk;
  }
}

// One warp per ray, for launches of at most one ray per SM sub-partition
// (one source's receivers), where a step's time is its chain of FP64
// instructions.  Lane q < ND owns axis q as in ray_axis_kernel.  The blend's
// weights and products, which the axis kernel repeats on each of a ray's
// lanes, are spread over the warp: lane NC c + t computes corner t's weight
// and its product with gradient component c's corner value.  Each sum stays
// sequential, in the reference's order, on its component's lane, and the
// squared norm takes each lane's square.  Every value is the same IEEE
// operation on the same operands as in ray_kernel, so the rays are the same
// bits, with about a third fewer FP64 instructions per step.
template <int ND>
__global__ void __launch_bounds__(128)
    ray_warp_kernel(Axes ax, const double* ttgrad, long long gstride, const int* gidx,
                    const double* ends, int nrays, const double* sources, double stepsize,
                    double dist_min, int max_step, double* rays, int* counts, int* status) {
  constexpr int NC = 1 << ND;  // corners of a cell
  __shared__ RayShared S;
  ray_setup<ND>(ax, S);
  const int lane = threadIdx.x & 31;
  const int r = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
  if (r >= nrays) return;
  const unsigned full = 0xffffffffu, all_axes = (1u << ND) - 1u;
  const int q = lane < ND ? lane : ND - 1;          // this lane's axis and component
  const int t = lane & (NC - 1);                    // corner of this lane's product
  const int pc = lane / NC < ND ? lane / NC : ND - 1;  // component of this lane's product
  const int gi = gidx ? gidx[r] : 0;
  const double* g = ttgrad + (long long)gi * gstride;
  const double* a = q == 0 ? ax.a[0] : (q == 1 ? ax.a[1] : ax.a[ND - 1]);
  const int n = q == 0 ? ax.n[0] : (q == 1 ? ax.n[1] : ax.n[ND - 1]);
  const RayAxis& X = S.X[q];
  const double sq = sources[ND * gi + q];
  double p = ends[ND * r + q];
  const long long kmin = __double_as_longlong(dist_min);
  if (lane == 0) counts[r] = 0;
  if ((__ballot_sync(full, X.lo <= p && p <= X.hi) & all_axes) != all_axes) {
    if (lane == 0) status[r] = kEndPointOutOfBound;
    return;
  }
  long long kp = zkey(p);
  double* ray = rays + (long long)r * max_step * ND;
  int count = 1;
  if (lane < ND) ray[q] = p;
  const long long max_iter = 64LL * max_step + 4096;
  for (long long iter = 0;; ++iter) {
    if (iter >= max_iter) {
      if (lane == 0) status[r] = kMaxStepReached;
      return;
    }
    // dist(src, pcur) >= stepsize on the squared distance (a*a + b*b) + c*c
    const double dq = sq - p;
    const double s2 = dq * dq;
    double dsq = __shfl_sync(full, s2, 0) + __shfl_sync(full, s2, 1);
    if (ND == 3) dsq = dsq + __shfl_sync(full, s2, 2);
    const long long db = __double_as_longlong(dsq);
    if (db < kmin || db > 0x7ff0000000000000LL) break;
    if ((__ballot_sync(full, X.klo <= kp && kp <= X.khi) & all_axes) != all_axes) break;
    // this lane's axis: cell, corner coordinates, weight differences
    const int c = ray_search(a, n, X, p, kp);
    const bool e = c == n - 1;
    const double x1 = __ldg(a + c);
    const double x2 = e ? 2.0 * x1 - __ldg(a + n - 2) : __ldg(a + c + 1);
    const double lo = x1 - p, hi = x2 - p, span = x2 - x1;
    double L[ND], H[ND];
    int ci[ND];
    bool ce[ND];
#pragma unroll
    for (int u = 0; u < ND; ++u) {
      L[u] = __shfl_sync(full, lo, u);
      H[u] = __shfl_sync(full, hi, u);
      const int packed = __shfl_sync(full, (c << 1) | (e ? 1 : 0), u);
      ci[u] = packed >> 1;
      ce[u] = (packed & 1) != 0;
    }
    double vol = S.vol_c;
    if (!S.uni) {
      vol = __shfl_sync(full, span, 0) * __shfl_sync(full, span, 1);
      if (ND == 3) vol = vol * __shfl_sync(full, span, 2);
      vol = fabs(vol);
    }
    // corner t's weight (weights3 / weights2: |(x? - xq)(y? - yq)(z? - zq)|)
    // and its product with component pc's value there (1.0 past the last node)
    double w, cv;
    if (ND == 3) {
      const double pair = ((t & 1) ? L[0] : H[0]) * ((t & 2) ? L[1] : H[1]);
      w = fabs(pair * ((t & 4) ? L[ND - 1] : H[ND - 1]));
      const int n1 = ax.n[1], n2 = ax.n[ND - 1];
      const long long b = ((long long)ci[0] * n1 + ci[1]) * n2 + ci[ND - 1];
      const long long off =
          ((t & 1) ? (long long)n1 * n2 : 0) + ((t & 2) ? n2 : 0) + ((t & 4) ? 1 : 0);
      const bool past = ((t & 1) && ce[0]) || ((t & 2) && ce[1]) || ((t & 4) && ce[ND - 1]);
      cv = past ? 1.0 : __ldg(g + (b + off) * 3 + pc);
    } else {
      w = fabs(((t & 1) ? L[0] : H[0]) * ((t & 2) ? L[1] : H[1]));
      const int n1 = ax.n[1];
      const long long b = (long long)ci[0] * n1 + ci[1];
      const long long off = ((t & 1) ? n1 : 0) + ((t & 2) ? 1 : 0);
      const bool past = ((t & 1) && ce[0]) || ((t & 2) && ce[1]);
      cv = past ? 1.0 : __ldg(g + (b + off) * 2 + pc);
    }
    const double prod = cv * w;
    // component q's blend, in the reference's order
    double vq = __shfl_sync(full, prod, q * NC);
#pragma unroll
    for (int u = 1; u < NC; ++u) vq += __shfl_sync(full, prod, q * NC + u);
    const double mine = per_volume(vq, vol, S.vol, S.uni != 0);
    const double m2 = mine * mine;
    double gsq = __shfl_sync(full, m2, 0) + __shfl_sync(full, m2, 1);
    if (ND == 3) gsq = gsq + __shfl_sync(full, m2, 2);
    const long long gb = __double_as_longlong(gsq);
    if (gb == 0 || gb > 0x7ff0000000000000LL) break;
    const double gni = 1.0 / sqrt_rn(gsq);
    // this lane's coordinate: max(axis[0], min(axis[-1], p - stepsize * g * gni))
    double v = p - stepsize * mine * gni;
    long long kv = zkey(v);
    const bool nan = (kv < 0 ? -kv : kv) > 0x7ff0000000000000LL;
    if (!nan && X.klo > kv) {
      v = X.lo;
      kv = X.klo;
    }
    if (!nan && X.khi < kv) {
      v = X.hi;
      kv = X.khi;
    }
    p = v;
    kp = kv;
    if (lane < ND) ray[count * ND + q] = v;
    count += 1;
    if (count >= max_step) {
      if (lane == 0) status[r] = kMaxStepReached;
      return;
    }
  }
  if (lane < ND) ray[count * ND + q] = sq;
  if (lane == 0) {
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

// The least double x >= 0 with RN(sqrt(x)) >= s (s > 0): RN(sqrt(.)) is
// monotone, so sqrt(x) >= s exactly when x >= this threshold.  The host's
// sqrt is the correctly rounded IEEE square root, as the device's is.
static double sqrt_threshold(double s) {
  double x = s * s;
  if (!(std::sqrt(x) >= s)) {
    while (!(std::sqrt(x) >= s)) x = std::nextafter(x, HUGE_VAL);
  } else {
    for (;;) {
      const double y = std::nextafter(x, 0.0);
      if (!(y >= 0.0) || y == x || !(std::sqrt(y) >= s)) break;
      x = y;
    }
  }
  return x;
}

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
  const double dist_min = sqrt_threshold(stepsize);
  // A warp per ray while each ray's warp has an SM sub-partition to itself;
  // four lanes per ray while every ray's group fits on the GPU at once (one
  // source's receivers); one lane per ray for large batches, which are bound
  // by throughput rather than by the latency of a step.  "ray_lanes" picks
  // one (32, 4 or 1; honor_grid rays run on one or four lanes).
  const long long lanes_opt = option_value(kOptRayLanes);
  const int lanes = lanes_opt > 0 ? (int)lanes_opt
                                  : ((long long)nrays <= 4LL * sm_count()
                                         ? 32
                                         : ((long long)nrays * 4 <= 64LL * 1024 ? 4 : 1));
  if (lanes == 32 && !honor_grid) {
    ray_warp_kernel<ND><<<(unsigned)((nrays + 3) / 4), 128, 0, (cudaStream_t)stream>>>(
        ax, ttgrad, grad_stride, grid_index, ends, nrays, sources, stepsize, dist_min, max_step,
        rays, counts, status);
  } else if (lanes >= 4) {
    const long long threads = (long long)nrays * 4;
    const unsigned blocks = (unsigned)((threads + 63) / 64);
    if (!honor_grid)
      ray_axis_kernel<ND><<<blocks, 64, 0, (cudaStream_t)stream>>>(
          ax, ttgrad, grad_stride, grid_index, ends, nrays, sources, stepsize, dist_min,
          max_step, rays, counts, status);
    else
      ray_kernel<ND, 4><<<blocks, 64, 0, (cudaStream_t)stream>>>(
          ax, ttgrad, grad_stride, grid_index, ends, nrays, sources, stepsize, dist_min,
          max_step, honor_grid, rays, counts, status);
  } else {
    ray_kernel<ND, 1><<<(nrays + 63) / 64, 64, 0, (cudaStream_t)stream>>>(
        ax, ttgrad, grad_stride, grid_index, ends, nrays, sources, stepsize, dist_min, max_step,
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
