// 2D FTeik solver for GB300: fteikpy/_fteik/_fteik2d.py rebuilt as CUDA.
//
// Layout (C order, float64 unless noted):
//   slow  [nz][nx] cells, tt [nsrc][NZ][NX] nodes, ttgrad [nsrc][NZ][NX][2],
//   rec   [nsrc][NZ][NX] uint8 branch record (sz+1)*3 + (sx+1) (ttsgn of
//         _fteik2d.py:178-187).
//
// Schedule.  The reference's 2D sweep is NOT a set of independent directional
// sweeps: for every column it runs the downward pass and then the upward pass
// before moving to the next column (_fteik2d.py:199-287), so each sweep is a
// single dependence chain of 4*nz*nx node updates, and reordering it changes
// the result (by up to 1e-2 relative on layered models).  The kernel therefore
// keeps the reference's order exactly: one thread walks one source's chain,
// and batches of sources run in parallel, one thread each.
#include <cstdint>

#include "common.cuh"
#include "fteik_gb300.h"
#include "runtime.h"

namespace fteik {

struct Ops2 {
  double dz, dx, dzi, dxi, dz2i, dx2i;  // sweep2d dargs, _fteik2d.py:193-197
  double s2, p2;                        // dz2i + dx2i, dz2i * dx2i
  double dzz, dxx, hyp;                 // dz**2, dx**2, (dx**2 + dz**2)**0.5
  Recip r2, rdz, rdx, rhyp;
};

static Ops2 make_ops2(double dz, double dx) {
  Ops2 o;
  o.dz = dz;
  o.dx = dx;
  o.dzi = 1.0 / dz;
  o.dxi = 1.0 / dx;
  o.dz2i = o.dzi / dz;
  o.dx2i = o.dxi / dx;
  o.s2 = o.dz2i + o.dx2i;
  o.p2 = o.dz2i * o.dx2i;
  o.dzz = dz * dz;
  o.dxx = dx * dx;
  o.hyp = __builtin_sqrt(o.dxx + o.dzz);
  o.r2 = make_recip(o.s2);
  o.rdz = make_recip(dz);
  o.rdx = make_recip(dx);
  o.rhyp = make_recip(o.hyp);
  return o;
}

struct Source2 {
  double zsa, xsa, vzero;
  int zsi, xsi, iflag, pad;
};

// t_ana / t_anad, _fteik2d.py:11-30.
__device__ __forceinline__ double t_ana2(int i, int j, double dz, double dx, double zsa,
                                         double xsa, double vzero) {
  double a = dz * ((double)i - zsa);
  double b = dx * ((double)j - xsa);
  return vzero * sqrt(a * a + b * b);
}
__device__ __forceinline__ double t_anad2(int i, int j, double dz, double dx, double zsa,
                                          double xsa, double vzero, double& tzc, double& txc) {
  double t = t_ana2(i, j, dz, dx, zsa, xsa, vzero);
  if (t > 0.0) {
    double tmp = vzero * vzero / t;
    tzc = ((double)i - zsa) * dz * tmp;
    txc = ((double)j - xsa) * dx * tmp;
  } else {
    tzc = txc = 0.0;
  }
  return t;
}

// delta, _fteik2d.py:33-67 (factored quadratic near the source).
__device__ double delta2(double t1, double tauv, double taue, double tauev, double t0c,
                         double tzc, double txc, double dzi, double dxi, double dz2i,
                         double dx2i, double vzero, double vref, int sgntz, int sgntx) {
  double ta = tauev + taue - tauv;
  double tb = tauev - taue + tauv;
  double apoly = dz2i + dx2i;
  double bpoly = 4.0 * ((double)sgntx * txc * dxi + (double)sgntz * tzc * dzi) -
                 2.0 * (ta * dx2i + tb * dz2i);
  double cpoly = ((ta * ta) * dx2i) + ((tb * tb) * dz2i) -
                 4.0 * ((double)sgntx * txc * dxi * ta + (double)sgntz * tzc * dzi * tb) +
                 4.0 * (vzero * vzero - vref * vref);
  double dpoly = bpoly * bpoly - 4.0 * apoly * cpoly;
  return dpoly >= 0.0 ? 0.5 * (sqrt(dpoly) - bpoly) / apoly + t0c : t1;
}

// Comparisons of the node update.  K = false: IEEE comparisons, which keep
// Python's NaN semantics (every comparison with NaN is false).  K = true:
// integer order keys (common.cuh), exact when no value is NaN or -0.0.  The
// sweeps produce neither from values that are neither (every radicand of the
// operators is positive by a wide margin under its guard, and every
// traveltime is a sum of non-negative terms), so the keys serve every source
// whose first propagation left only finite values in the grid; an FP64
// comparison costs more than an FP64 add on GB300, and this chain is one
// thread long.
__device__ __forceinline__ bool is_finite(double x) {
  return (__double_as_longlong(x) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}
template <bool K>
__device__ __forceinline__ bool lt2(double a, double b) {
  return K ? dlt(a, b) : a < b;
}
template <bool K>
__device__ __forceinline__ bool le2(double a, double b) {
  return K ? dle(a, b) : a <= b;
}
template <bool K>
__device__ __forceinline__ bool eq2(double a, double b) {
  return K ? deq(a, b) : a == b;
}

// The inputs of one node update that do not depend on the previous node of
// the pass: the previous column's te and tev, the node's own old value t0, and
// the five slowness cells of the operators.
struct In2 {
  double te, tev, t0, sz0, sz1, sx0, sx1, s2;
};

__device__ __forceinline__ In2 load_in2(const double* tt, const double* slow, int i, int j,
                                        int sgnvz, int sgnvx, int sgntz, int sgntx, int NZ,
                                        int NX) {
  const int nxc = NX - 1;
  const int i1 = i - sgnvz, j1 = j - sgnvx;
  const long long n = (long long)i * NX + j;
  In2 q;
  q.te = tt[n - sgntx];
  q.tev = tt[n - (long long)sgntz * NX - sgntx];
  q.t0 = tt[n];
  q.sz0 = __ldg(slow + (long long)i1 * nxc + imax(j - 1, 0));
  q.sz1 = __ldg(slow + (long long)i1 * nxc + imin(j, NX - 2));
  q.sx0 = __ldg(slow + (long long)imax(i - 1, 0) * nxc + j1);
  q.sx1 = __ldg(slow + (long long)imin(i, NZ - 2) * nxc + j1);
  q.s2 = __ldg(slow + (long long)i1 * nxc + j1);
  return q;
}

// One node update, _fteik2d.py:70-187, from tv (the previous node of the
// pass) and the other inputs, with the comparisons of policy K (above).
// Returns the node's value after the update.
template <bool GRAD, bool K>
__device__ __forceinline__ double node_update2d(double* tt, uint8_t* rec, const Ops2& o,
                                                const Source2& sp, int i, int j, int sgntz,
                                                int sgntx, int NX, double tv, const In2& q) {
  const long long n = (long long)i * NX + j;
  const double te = q.te, tev = q.tev;
  double vref = pmin(q.sz0, q.sz1);
  const double t1d1 = tv + o.dz * vref;
  vref = pmin(q.sx0, q.sx1);
  const double t1d2 = te + o.dx * vref;
  const double t1d = lt2<K>(t1d2, t1d1) ? t1d2 : t1d1;

  double t2d = kBig;
  vref = q.s2;
  const int di = i - sp.zsi, dj = j - sp.xsi;
  if (di > kEpsin || di < -kEpsin || dj > kEpsin || dj < -kEpsin) {
    // plane-wave operators, _fteik2d.py:121-142
    if (le2<K>(tv, te + o.dx * vref) && le2<K>(te, tv + o.dz * vref) && le2<K>(tev, te) &&
        le2<K>(tev, tv)) {
      const double ta = tev + te - tv;
      const double tb = tev - te + tv;
      const double d = ta - tb;
      t2d = div_dd((tb * o.dz2i + ta * o.dx2i) + sqrt(times4(vref * vref) * o.s2 - o.p2 * (d * d)),
                   o.r2);
    } else if (le2<K>(te - tev, div_dd(o.dzz * vref, o.rhyp)) && lt2<K>(0.0, te - tev)) {
      const double r = div_dd(te - tev, o.rdz);
      t2d = te + o.dx * sqrt(vref * vref - r * r);
    } else if (le2<K>(tv - tev, div_dd(o.dxx * vref, o.rhyp)) && lt2<K>(0.0, tv - tev)) {
      const double r = div_dd(tv - tev, o.rdx);
      t2d = tv + o.dz * sqrt(vref * vref - r * r);
    }
  } else {
    // spherical (factored) operator near the source, _fteik2d.py:144-171
    if (lt2<K>(tv, te + o.dx * vref) && lt2<K>(te, tv + o.dz * vref) && le2<K>(tev, te) &&
        le2<K>(tev, tv)) {
      double tzc, txc;
      const double t0c = t_anad2(i, j, o.dz, o.dx, sp.zsa, sp.xsa, sp.vzero, tzc, txc);
      const double tauv = tv - t_ana2(i - sgntz, j, o.dz, o.dx, sp.zsa, sp.xsa, sp.vzero);
      const double taue = te - t_ana2(i, j - sgntx, o.dz, o.dx, sp.zsa, sp.xsa, sp.vzero);
      const double tauev = tev - t_ana2(i - sgntz, j - sgntx, o.dz, o.dx, sp.zsa, sp.xsa, sp.vzero);
      t2d = delta2(t2d, tauv, taue, tauev, t0c, tzc, txc, o.dzi, o.dxi, o.dz2i, o.dx2i,
                   sp.vzero, vref, sgntz, sgntx);
      if (t2d < tv || t2d < te) t2d = kBig;
    }
  }
  const double t0 = q.t0;
  // min(t0, t1d, t2d) with Python's semantics: keep the earlier argument
  // unless a later one compares strictly smaller.
  double tnew = t0;
  if (lt2<K>(t1d, tnew)) tnew = t1d;
  if (lt2<K>(t2d, tnew)) tnew = t2d;
  if (!eq2<K>(tnew, t0)) {
    tt[n] = tnew;
    if (GRAD) {
      int a, b;
      if (eq2<K>(tnew, t1d1)) {
        a = sgntz; b = 0;
      } else if (eq2<K>(tnew, t1d2)) {
        a = 0; b = sgntx;
      } else {
        a = sgntz; b = sgntx;
      }
      rec[n] = (uint8_t)((a + 1) * 3 + (b + 1));
    }
  }
  return tnew;
}

// One pass over column j, rows i0, i0 + step, ..., i1 (inclusive), in the
// reference's order.  Only tv depends on the previous node; every other
// input of the next node is read while the current one is computed (the
// previous column is complete, and this column's old values were written by
// earlier passes), so the pass runs at the latency of the arithmetic chain.
template <bool GRAD, bool K>
__device__ __forceinline__ void column_pass2d(double* tt, uint8_t* rec, const double* slow,
                                              const Ops2& o, const Source2& sp, int j, int i0,
                                              int i1, int sgnvz, int sgnvx, int sgntz,
                                              int sgntx, int NZ, int NX) {
  const int step = sgntz;  // passes run in the direction of their upwind sign
  double tv = tt[(long long)(i0 - sgntz) * NX + j];
  In2 cur = load_in2(tt, slow, i0, j, sgnvz, sgnvx, sgntz, sgntx, NZ, NX);
  for (int i = i0;; i += step) {
    const bool more = i != i1;
    In2 nxt;
    if (more) nxt = load_in2(tt, slow, i + step, j, sgnvz, sgnvx, sgntz, sgntx, NZ, NX);
    tv = node_update2d<GRAD, K>(tt, rec, o, sp, i, j, sgntz, sgntx, NX, tv, cur);
    if (!more) break;
    cur = nxt;
  }
}

// The nsweep interleaved sweeps, _fteik2d.py:190-287 and 619-621.
template <bool GRAD, bool K>
__device__ __noinline__ void sweeps2d(double* tt, uint8_t* rec, const double* slow,
                                      const Ops2& o, const Source2& sp, int nsweep, int NZ,
                                      int NX) {
  for (int sw = 0; sw < nsweep; ++sw) {
    for (int j = 1; j < NX; ++j) {
      column_pass2d<GRAD, K>(tt, rec, slow, o, sp, j, 1, NZ - 1, 1, 1, 1, 1, NZ, NX);
      column_pass2d<GRAD, K>(tt, rec, slow, o, sp, j, NZ - 2, 0, 0, 1, -1, 1, NZ, NX);
    }
    for (int j = NX - 2; j >= 0; --j) {
      column_pass2d<GRAD, K>(tt, rec, slow, o, sp, j, 1, NZ - 1, 1, 0, 1, -1, NZ, NX);
      column_pass2d<GRAD, K>(tt, rec, slow, o, sp, j, NZ - 2, 0, 0, 0, -1, -1, NZ, NX);
    }
  }
}

// Source classification and first propagation, _fteik2d.py:296-617, for the
// source at src[0..1] into tt (pre-filled with Big; rec with "no sign").
// Returns the source's parameters for the sweeps.
template <bool GRAD>
__device__ Source2 first_propagation2d(const double* slow, const double* src, int nz, int nx,
                                       const Ops2& o, double* tt, uint8_t* rec) {
  const int NZ = nz + 1, NX = nx + 1;
#define TT(a, b) tt[(long long)(a)*NX + (b)]
#define SL(a, b) slow[(long long)(a)*nx + (b)]
#define SGN(a, b, sz_, sx_) \
  if (GRAD) rec[(long long)(a)*NX + (b)] = (uint8_t)(((sz_) + 1) * 3 + ((sx_) + 1))

  const double dz = o.dz, dx = o.dx;
#define TT(a, b) tt[(long long)(a)*NX + (b)]
#define SL(a, b) slow[(long long)(a)*nx + (b)]
#define SGN(a, b, sz_, sx_) \
  if (GRAD) rec[(long long)(a)*NX + (b)] = (uint8_t)(((sz_) + 1) * 3 + ((sx_) + 1))

  double zsa = src[0] / dz, xsa = src[1] / dx;
  zsa = zsa >= nz ? zsa - kEps : zsa;
  xsa = xsa >= nx ? xsa - kEps : xsa;
  const int zsi = imin((int)zsa, nz - 1);
  const int xsi = imin((int)xsa, nx - 1);
  const double vzero = SL(zsi, xsi);

  double dzu = fabs(zsa - (double)zsi);
  double dzd = 1.0 - dzu;
  double dxw = fabs(xsa - (double)xsi);
  double dxe = 1.0 - dxw;
  const double dzv_min = dzd < dzu ? dzd : dzu;
  const double dzh_min = dxe < dxw ? dxe : dxw;
  int iflag;
  if (dzv_min < kEps && dzh_min < kEps) {
    zsa = rint(zsa);
    xsa = rint(xsa);
    iflag = 1;
  } else if (dzv_min > kEps || dzh_min > kEps) {
    zsa = dzv_min < kEps ? rint(zsa) : zsa;
    xsa = dzh_min < kEps ? rint(xsa) : xsa;
    iflag = 2;
  } else {
    zsa = rint(zsa);
    xsa = rint(xsa);
    iflag = 3;
  }

  if (iflag == 2) {
    dzu = fabs(zsa - (double)zsi);
    dzd = 1.0 - dzu;
    dxw = fabs(xsa - (double)xsi);
    dxe = 1.0 - dxw;
    for (int q = 0; q < 4; ++q) {
      const int i = zsi + (q & 1), j = xsi + (q >> 1);
      double tzc, txc;
      TT(i, j) = t_anad2(i, j, dz, dx, zsa, xsa, vzero, tzc, txc);
    }
    double dxi = 1.0 / dx;
    double dx2i = dxi / dx;
    double dzi, dz2i, tzc, txc, t0c, vref, tauv, tauev, taue, td_prev, td_cur;
    // along row zsi (+1), eastwards, _fteik2d.py:379-435
    td_prev = vzero * dxe * dx;
    for (int j = xsi + 2; j < NX; ++j) {
      vref = SL(zsi, j - 1);
      td_cur = td_prev + dx * vref;
      tauv = td_cur - vzero * fabs((double)j - xsa) * dx;
      tauev = td_prev - vzero * fabs((double)j - xsa - 1.0) * dx;
      dzi = 1.0 / dzd;
      dz2i = dz / dzd / dzd;
      taue = TT(zsi + 1, j - 1) - t_ana2(zsi + 1, j - 1, dz, dx, zsa, xsa, vzero);
      t0c = t_anad2(zsi + 1, j, dz, dx, zsa, xsa, vzero, tzc, txc);
      TT(zsi + 1, j) = delta2(TT(zsi + 1, j), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i,
                              dx2i, vzero, vref, 1, 1);
      SGN(zsi + 1, j, 1, 1);
      if (dzu > 0.0) {
        dzi = 1.0 / dzu;
        dz2i = dz / dzu / dzu;
        taue = TT(zsi, j - 1) - t_ana2(zsi, j - 1, dz, dx, zsa, xsa, vzero);
        t0c = t_anad2(zsi, j, dz, dx, zsa, xsa, vzero, tzc, txc);
        TT(zsi, j) = delta2(TT(zsi, j), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i, dx2i,
                            vzero, vref, -1, 1);
        SGN(zsi, j, -1, 1);
      }
      td_prev = td_cur;
    }
    // westwards, _fteik2d.py:437-495
    td_prev = vzero * dxw * dx;
    for (int j = xsi - 1; j >= 0; --j) {
      vref = SL(zsi, j);
      td_cur = td_prev + dx * vref;
      tauv = td_cur - vzero * fabs((double)j - xsa) * dx;
      tauev = td_prev - vzero * fabs((double)j - xsa + 1.0) * dx;
      dzi = 1.0 / dzd;
      dz2i = dz / dzd / dzd;
      taue = TT(zsi + 1, j + 1) - t_ana2(zsi + 1, j + 1, dz, dx, zsa, xsa, vzero);
      t0c = t_anad2(zsi + 1, j, dz, dx, zsa, xsa, vzero, tzc, txc);
      TT(zsi + 1, j) = delta2(TT(zsi + 1, j), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i,
                              dx2i, vzero, vref, 1, -1);
      SGN(zsi + 1, j, 1, -1);
      if (dzu > 0.0) {
        dzi = 1.0 / dzu;
        dz2i = dz / dzu / dzu;
        // the reference reads row zsi + 1 here (_fteik2d.py:472-474)
        taue = TT(zsi + 1, j + 1) - t_ana2(zsi + 1, j + 1, dz, dx, zsa, xsa, vzero);
        t0c = t_anad2(zsi, j, dz, dx, zsa, xsa, vzero, tzc, txc);
        TT(zsi, j) = delta2(TT(zsi, j), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i, dx2i,
                            vzero, vref, -1, -1);
        SGN(zsi, j, -1, -1);
      }
      td_prev = td_cur;
    }
    // along column xsi (+1), downwards, _fteik2d.py:497-556
    dzi = 1.0 / dz;
    dz2i = dzi / dz;
    td_prev = vzero * dzd * dz;
    for (int i = zsi + 2; i < NZ; ++i) {
      vref = SL(i - 1, xsi);
      td_cur = td_prev + dz * vref;
      taue = td_cur - vzero * fabs((double)i - zsa) * dz;
      tauev = td_prev - vzero * fabs((double)i - zsa - 1.0) * dz;
      dxi = 1.0 / dxe;
      dx2i = dx / dxe / dxe;
      tauv = TT(i - 1, xsi + 1) - t_ana2(i - 1, xsi + 1, dz, dx, zsa, xsa, vzero);
      t0c = t_anad2(i, xsi + 1, dz, dx, zsa, xsa, vzero, tzc, txc);
      TT(i, xsi + 1) = delta2(TT(i, xsi + 1), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i,
                              dx2i, vzero, vref, 1, 1);
      SGN(i, xsi + 1, 1, 1);
      if (dxw > 0.0) {
        dxi = 1.0 / dxw;
        dx2i = dx / dxw / dxw;
        tauv = TT(i - 1, xsi) - t_ana2(i - 1, xsi, dz, dx, zsa, xsa, vzero);
        t0c = t_anad2(i, xsi, dz, dx, zsa, xsa, vzero, tzc, txc);
        TT(i, xsi) = delta2(TT(i, xsi), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i, dx2i,
                            vzero, vref, 1, -1);
        SGN(i, xsi, 1, -1);
      }
      td_prev = td_cur;
    }
    // upwards, _fteik2d.py:558-614
    td_prev = vzero * dzu * dz;
    for (int i = zsi - 1; i >= 0; --i) {
      vref = SL(i, xsi);
      td_cur = td_prev + dz * vref;
      taue = td_cur - vzero * fabs((double)i - zsa) * dz;
      tauev = td_prev - vzero * fabs((double)i - zsa + 1.0) * dz;
      dxi = 1.0 / dxe;
      dx2i = dx / dxe / dxe;
      tauv = TT(i + 1, xsi + 1) - t_ana2(i + 1, xsi + 1, dz, dx, zsa, xsa, vzero);
      t0c = t_anad2(i, xsi + 1, dz, dx, zsa, xsa, vzero, tzc, txc);
      TT(i, xsi + 1) = delta2(TT(i, xsi + 1), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i,
                              dx2i, vzero, vref, -1, 1);
      SGN(i, xsi + 1, -1, 1);
      if (dxw > 0.0) {
        dxi = 1.0 / dxw;
        dx2i = dx / dxw / dxw;
        tauv = TT(i + 1, xsi) - t_ana2(i + 1, xsi, dz, dx, zsa, xsa, vzero);
        t0c = t_anad2(i, xsi, dz, dx, zsa, xsa, vzero, tzc, txc);
        TT(i, xsi) = delta2(TT(i, xsi), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i, dx2i,
                            vzero, vref, -1, -1);
        SGN(i, xsi, -1, -1);
      }
      td_prev = td_cur;
    }
  } else {
    TT((int)zsa, (int)xsa) = 0.0;  // _fteik2d.py:616-617
  }
#undef TT
#undef SL
#undef SGN

  Source2 sp;
  sp.zsa = zsa;
  sp.xsa = xsa;
  sp.vzero = vzero;
  sp.zsi = zsi;
  sp.xsi = xsi;
  sp.iflag = iflag;
  sp.pad = 0;
  return sp;
}

// One thread per source: the first propagation, then the nsweep interleaved
// sweeps, _fteik2d.py:190-287 and 619-621.  tt is pre-filled with Big and rec
// with "no sign".
template <bool GRAD>
__global__ void __launch_bounds__(32) solve2d_kernel(const double* slow, const double* src,
                                                     int nsrc, int nz, int nx, int nsweep,
                                                     Ops2 o, double* tt_all, uint8_t* rec_all,
                                                     Source2* params, double* vzero_out,
                                                     bool keys) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsrc) return;
  const int NZ = nz + 1, NX = nx + 1;
  const long long nodes = (long long)NZ * NX;
  double* tt = tt_all + (long long)s * nodes;
  uint8_t* rec = GRAD ? rec_all + (long long)s * nodes : nullptr;
  const Source2 sp = first_propagation2d<GRAD>(slow, src + 2 * s, nz, nx, o, tt, rec);
  const int zsi = sp.zsi, xsi = sp.xsi;
  params[s] = sp;
  vzero_out[s] = sp.vzero;

  // The first propagation wrote rows zsi, zsi+1 and columns xsi, xsi+1 (the
  // rest is Big).  If all of them are finite, no NaN or infinity arises in
  // the sweeps and their comparisons can use integer keys.
  bool finite = keys;
  for (int jj = 0; jj < NX && finite; ++jj)
    for (int r = zsi; r <= imin(zsi + 1, NZ - 1); ++r) finite = finite && is_finite(tt[(long long)r * NX + jj]);
  for (int ii = 0; ii < NZ && finite; ++ii)
    for (int c = xsi; c <= imin(xsi + 1, NX - 1); ++c) finite = finite && is_finite(tt[(long long)ii * NX + c]);
  if (finite)
    sweeps2d<GRAD, true>(tt, rec, slow, o, sp, nsweep, NZ, NX);
  else
    sweeps2d<GRAD, false>(tt, rec, slow, o, sp, nsweep, NZ, NX);
}

// ----------------------------------------------------- one warp per source --
//
// For a few sources the chain's length is the solve's time, and every FP64
// instruction of it costs the full warp issue time whatever the number of
// active lanes.  Once column j - sgntx is final, every quantity of column j's
// updates that does not involve tv (the previous node of the pass) is known:
// the 1D candidates' terms, the plane operator's guards and partial sums,
// its radicand's constant term, and the whole second operator (its guard,
// sqrt and division).  Here the 32 lanes of a warp compute those for a chunk
// of rows at once into shared memory, and lane 0 then runs the chain on what
// depends on tv.  The operations and their operands are node_update2d's, so
// the results are the same bits.
constexpr int kChunk2 = 128;  // rows per precomputed chunk

template <int N>
struct Pre2T {
  double a1[N];    // dz * min slowness along z (t1d1 = tv + a1)
  double t1d2[N];  // te + dx * min slowness along x
  double c1[N];    // te + dx * vref (guard tv <= c1)
  double b[N];     // dz * vref (guard te <= tv + b)
  double p1[N];    // tev + te (ta = p1 - tv)
  double p2[N];    // tev - te (tb = p2 + tv)
  double x[N];     // 4 vref^2 (dz2i + dx2i), the radicand's constant term
  double te[N], tev[N], vref[N];
  double vv[N];    // vref * vref
  double d3[N];    // the third operator's guard bound
  double t2[N];    // the second operator's value, where it applies
  // Speculation: the whole update of the row evaluated with tv equal to the
  // previous node's value before this pass (tvs), giving tns and its branch
  // code cds.  When the previous node keeps its value in the pass (most
  // nodes of most passes), the chain's actual tv has the same bits as tvs
  // and lane 0 takes the result instead of evaluating the operators.
  double tvs[N], tns[N];
  unsigned char flags[N];  // 1: tev <= te; 2: the second operator applies
  unsigned char cds[N];
};
using Pre2 = Pre2T<kChunk2>;

// The precomputed terms the chain reads on every node, loaded into registers
// one node ahead (the rarer branches read shared memory directly).
struct Row2 {
  double a1, t1d2, c1, b, p1, p2, x, te, tev, tvs, tns;
  unsigned flags, cds;
};
template <class PreT>
__device__ __forceinline__ Row2 load_row2(const PreT& P, int q) {
  return Row2{P.a1[q], P.t1d2[q], P.c1[q], P.b[q],   P.p1[q],    P.p2[q],    P.x[q],
              P.te[q], P.tev[q],  P.tvs[q], P.tns[q], P.flags[q], P.cds[q]};
}

// node_update2d on precomputed row q: only the terms that involve tv.
// Returns the node's value after the update and, when it changes, its branch
// code (GRAD).
template <bool GRAD, bool K, class PreT>
__device__ __forceinline__ double eval_node2d(const Ops2& o, const Source2& sp, const PreT& P,
                                              const Row2& R, int q, int i, int j, int sgntz,
                                              int sgntx, double tv, double t0, unsigned& code) {
  const double t1d1 = tv + R.a1;
  const double t1d2 = R.t1d2;
  const double t1d = lt2<K>(t1d2, t1d1) ? t1d2 : t1d1;
  double t2d = kBig;
  const unsigned f = R.flags;
  const double tev = R.tev;
  const int di = i - sp.zsi, dj = j - sp.xsi;
  if (di > kEpsin || di < -kEpsin || dj > kEpsin || dj < -kEpsin) {
    if (le2<K>(tv, R.c1) && le2<K>(R.te, tv + R.b) && (f & 1u) && le2<K>(tev, tv)) {
      const double ta = R.p1 - tv;
      const double tb = R.p2 + tv;
      const double d = ta - tb;
      t2d = div_dd((tb * o.dz2i + ta * o.dx2i) + sqrt(R.x - o.p2 * (d * d)), o.r2);
    } else if (f & 2u) {
      t2d = P.t2[q];
    } else if (le2<K>(tv - tev, P.d3[q]) && lt2<K>(0.0, tv - tev)) {
      const double r = div_dd(tv - tev, o.rdx);
      t2d = tv + o.dz * sqrt(P.vv[q] - r * r);
    }
  } else {
    // spherical (factored) operator near the source, _fteik2d.py:144-171
    const double te = R.te, vref = P.vref[q];
    if (lt2<K>(tv, te + o.dx * vref) && lt2<K>(te, tv + o.dz * vref) && le2<K>(tev, te) &&
        le2<K>(tev, tv)) {
      double tzc, txc;
      const double t0c = t_anad2(i, j, o.dz, o.dx, sp.zsa, sp.xsa, sp.vzero, tzc, txc);
      const double tauv = tv - t_ana2(i - sgntz, j, o.dz, o.dx, sp.zsa, sp.xsa, sp.vzero);
      const double taue = te - t_ana2(i, j - sgntx, o.dz, o.dx, sp.zsa, sp.xsa, sp.vzero);
      const double tauev = tev - t_ana2(i - sgntz, j - sgntx, o.dz, o.dx, sp.zsa, sp.xsa, sp.vzero);
      t2d = delta2(t2d, tauv, taue, tauev, t0c, tzc, txc, o.dzi, o.dxi, o.dz2i, o.dx2i,
                   sp.vzero, vref, sgntz, sgntx);
      if (t2d < tv || t2d < te) t2d = kBig;
    }
  }
  double tnew = t0;
  if (lt2<K>(t1d, tnew)) tnew = t1d;
  if (lt2<K>(t2d, tnew)) tnew = t2d;
  if (GRAD && !eq2<K>(tnew, t0)) {
    int a, bb;
    if (eq2<K>(tnew, t1d1)) {
      a = sgntz; bb = 0;
    } else if (eq2<K>(tnew, t1d2)) {
      a = 0; bb = sgntx;
    } else {
      a = sgntz; bb = sgntx;
    }
    code = (unsigned)((a + 1) * 3 + (bb + 1));
  }
  return tnew;
}

template <bool GRAD, bool K, bool SPEC, class PreT>
__device__ __forceinline__ void precompute_row2d(PreT& P, int q, const double* tt,
                                                 const double* slow, const Ops2& o,
                                                 const Source2& sp, int i, int j, int sgnvz,
                                                 int sgnvx, int sgntz, int sgntx, int NZ,
                                                 int NX) {
  const In2 in = load_in2(tt, slow, i, j, sgnvz, sgnvx, sgntz, sgntx, NZ, NX);
  const double te = in.te, tev = in.tev;
  P.a1[q] = o.dz * pmin(in.sz0, in.sz1);
  P.t1d2[q] = te + o.dx * pmin(in.sx0, in.sx1);
  const double vref = in.s2;
  P.c1[q] = te + o.dx * vref;
  P.b[q] = o.dz * vref;
  P.p1[q] = tev + te;
  P.p2[q] = tev - te;
  const double vv = vref * vref;
  P.vv[q] = vv;
  P.x[q] = times4(vv) * o.s2;
  P.te[q] = te;
  P.tev[q] = tev;
  P.vref[q] = vref;
  P.d3[q] = div_dd(o.dxx * vref, o.rhyp);
  unsigned f = le2<K>(tev, te) ? 1u : 0u;
  const double dte = te - tev;
  if (le2<K>(dte, div_dd(o.dzz * vref, o.rhyp)) && lt2<K>(0.0, dte)) {
    const double r = div_dd(dte, o.rdz);
    P.t2[q] = te + o.dx * sqrt(vv - r * r);
    f |= 2u;
  }
  P.flags[q] = (unsigned char)f;
  if (SPEC) {
    // this lane's own writes above are visible to it
    const double tvs = tt[(long long)(i - sgntz) * NX + j];
    unsigned code = 0;
    P.tvs[q] = tvs;
    P.tns[q] = eval_node2d<GRAD, K>(o, sp, P, load_row2(P, q), q, i, j, sgntz, sgntx, tvs,
                                    in.t0, code);
    P.cds[q] = (unsigned char)code;
  }
}

// One pass over column j (rows i0, i0 + sgntz, ..., i1) by the whole warp.
// With SPEC, a row whose speculated tv has the bits of the actual one takes
// the speculated result (the same operations on the same operands, so the
// same bits); `hits` counts them.
template <bool GRAD, bool K, bool SPEC>
__device__ __forceinline__ void warp_pass2d(Pre2& P, double* tt, uint8_t* rec, const double* slow,
                                            const Ops2& o, const Source2& sp, int j, int i0,
                                            int i1, int sgnvz, int sgnvx, int sgntz, int sgntx,
                                            int NZ, int NX, unsigned long long& hits) {
  const int lane = threadIdx.x & 31;
  const int step = sgntz;
  const int len = (i1 - i0) * step + 1;
  double tv = 0.0;
  if (lane == 0) tv = tt[(long long)(i0 - sgntz) * NX + j];
  for (int c0 = 0; c0 < len; c0 += kChunk2) {
    const int m = imin(kChunk2, len - c0);
    for (int q = lane; q < m; q += 32)
      precompute_row2d<GRAD, K, SPEC>(P, q, tt, slow, o, sp, i0 + (c0 + q) * step, j, sgnvz,
                                      sgnvx, sgntz, sgntx, NZ, NX);
    __syncwarp();
    if (lane == 0) {
      int i = i0 + c0 * step;
      double t0n = tt[(long long)i * NX + j];
      Row2 rn = load_row2(P, 0);
      for (int q = 0; q < m; ++q, i += step) {
        const double t0 = t0n;
        const Row2 r = rn;
        if (q + 1 < m) {
          t0n = tt[(long long)(i + step) * NX + j];
          rn = load_row2(P, q + 1);
        }
        unsigned code;
        double tnew;
        if (SPEC && deq(tv, r.tvs)) {
          tnew = r.tns;
          code = r.cds;
          ++hits;
        } else {
          tnew = eval_node2d<GRAD, K>(o, sp, P, r, q, i, j, sgntz, sgntx, tv, t0, code);
        }
        if (!eq2<K>(tnew, t0)) {
          const long long n = (long long)i * NX + j;
          tt[n] = tnew;
          if (GRAD) rec[n] = (uint8_t)code;
        }
        tv = tnew;
      }
    }
    __syncwarp();
  }
}

template <bool GRAD, bool K, bool SPEC>
__device__ __noinline__ void warp_sweeps2d(Pre2& P, double* tt, uint8_t* rec, const double* slow,
                                           const Ops2& o, const Source2& sp, int nsweep, int NZ,
                                           int NX, unsigned long long* stats) {
  unsigned long long hits = 0;
  for (int sw = 0; sw < nsweep; ++sw) {
    for (int j = 1; j < NX; ++j) {
      warp_pass2d<GRAD, K, SPEC>(P, tt, rec, slow, o, sp, j, 1, NZ - 1, 1, 1, 1, 1, NZ, NX, hits);
      warp_pass2d<GRAD, K, SPEC>(P, tt, rec, slow, o, sp, j, NZ - 2, 0, 0, 1, -1, 1, NZ, NX,
                                 hits);
    }
    for (int j = NX - 2; j >= 0; --j) {
      warp_pass2d<GRAD, K, SPEC>(P, tt, rec, slow, o, sp, j, 1, NZ - 1, 1, 0, 1, -1, NZ, NX,
                                 hits);
      warp_pass2d<GRAD, K, SPEC>(P, tt, rec, slow, o, sp, j, NZ - 2, 0, 0, 0, -1, -1, NZ, NX,
                                 hits);
    }
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(stats, (unsigned long long)nsweep * 4ull * (unsigned long long)(NZ - 1) * (NX - 1));
    atomicAdd(stats + 1, hits);
  }
}

// One warp per source (blockIdx.x): lane 0 runs the first propagation, the
// warp checks it for non-finite values, then the sweeps run as above.
template <bool GRAD, bool SPEC>
__global__ void __launch_bounds__(32) solve2d_warp_kernel(const double* slow, const double* src,
                                                          int nz, int nx, int nsweep, Ops2 o,
                                                          double* tt_all, uint8_t* rec_all,
                                                          Source2* params, double* vzero_out,
                                                          bool keys, unsigned long long* stats) {
  __shared__ Pre2 P;
  __shared__ Source2 sps;
  const int s = blockIdx.x;
  const int lane = threadIdx.x;
  const int NZ = nz + 1, NX = nx + 1;
  const long long nodes = (long long)NZ * NX;
  double* tt = tt_all + (long long)s * nodes;
  uint8_t* rec = GRAD ? rec_all + (long long)s * nodes : nullptr;
  if (lane == 0) {
    const Source2 sp = first_propagation2d<GRAD>(slow, src + 2 * s, nz, nx, o, tt, rec);
    params[s] = sp;
    vzero_out[s] = sp.vzero;
    sps = sp;
  }
  __syncwarp();
  const Source2 sp = sps;
  bool finite = true;
  for (int jj = lane; jj < NX; jj += 32)
    for (int r = sp.zsi; r <= imin(sp.zsi + 1, NZ - 1); ++r)
      finite = finite && is_finite(tt[(long long)r * NX + jj]);
  for (int ii = lane; ii < NZ; ii += 32)
    for (int c = sp.xsi; c <= imin(sp.xsi + 1, NX - 1); ++c)
      finite = finite && is_finite(tt[(long long)ii * NX + c]);
  finite = __all_sync(0xffffffffu, finite) && keys;
  if (finite)
    warp_sweeps2d<GRAD, true, SPEC>(P, tt, rec, slow, o, sp, nsweep, NZ, NX, stats);
  else
    warp_sweeps2d<GRAD, false, SPEC>(P, tt, rec, slow, o, sp, nsweep, NZ, NX, stats);
}

// A block of 4 warps per source.  In the warp kernel the rows of a pass are
// precomputed chunk by chunk between stretches of the chain, which on the
// plain 2D workload puts a fifth of the time on the chain's path.  Here warp
// 0's lane 0 runs the chain while warps 1-3 precompute the pass's chunks of
// 32 rows ahead of it into a ring of shared-memory slots, each slot published
// with a tag (pass, chunk) once written.  A pass starts after a block barrier,
// when every input of its rows is final (the previous column, and this
// column's values after the previous pass), so only the first chunk's
// precompute stays on the chain's path.  The rows' operations are the warp
// kernel's, so the results are the same bits.
constexpr int kTeamRows2 = 32;                  // rows per chunk
constexpr int kTeamSlots2 = 8;                  // chunks in the ring
constexpr int kTeamWarps2 = 4;                  // the chain's warp and three producers
constexpr unsigned long long kTeamWaitNs2 = 10000000000ull;  // default bound of one wait: 10 s
using Pre2Ring = Pre2T<kTeamRows2 * kTeamSlots2>;

struct TeamSync2 {
  unsigned long long ready[kTeamSlots2];  // tag of the chunk each slot holds
  unsigned long long consumed;            // tag of the last chunk the chain finished
  int abort;                              // a wait gave up: the block stops
};

// Tags grow with (pass, chunk): pass from 1, chunk c < 2^26 - 1 (rows < 2^31).
__device__ __forceinline__ unsigned long long tag2(unsigned long long pass, int c) {
  return (pass << 26) | (unsigned long long)(c + 1);
}

// Wait until *p >= want. Gives up (false) when another thread of the block
// gave up, or after limit_ns, marking the block aborted.
__device__ __forceinline__ bool wait_tag2(const volatile unsigned long long* p,
                                          unsigned long long want, volatile int* abort,
                                          unsigned long long limit_ns) {
  if (*p >= want) return true;
  const unsigned long long t0 = globaltimer();
  for (;;) {
    __nanosleep(32);
    if (*p >= want) return true;
    if (*abort) return false;
    if (globaltimer() - t0 >= limit_ns) {
      *abort = 1;
      return false;
    }
  }
}

// One pass over column j (rows i0, i0 + sgntz, ..., i1), as warp_pass2d.
template <bool GRAD, bool K, bool SPEC>
__device__ __forceinline__ void team_pass2d(Pre2Ring& P, TeamSync2& S, double* tt, uint8_t* rec,
                                            const double* slow, const Ops2& o,
                                            const Source2& sp, int j, int i0, int i1, int sgnvz,
                                            int sgnvx, int sgntz, int sgntx, int NZ, int NX,
                                            unsigned long long pass, unsigned long long wait_ns,
                                            unsigned long long& hits) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int step = sgntz;
  const int len = (i1 - i0) * step + 1;
  const int nch = (len + kTeamRows2 - 1) / kTeamRows2;
  __syncthreads();  // the previous pass is complete
  if (*(volatile int*)&S.abort) return;
  if (warp > 0) {
    for (int c = warp - 1; c < nch; c += kTeamWarps2 - 1) {
      const int slot = c % kTeamSlots2;
      bool ok = true;
      if (c >= kTeamSlots2 && lane == 0)
        ok = wait_tag2(&S.consumed, tag2(pass, c - kTeamSlots2), &S.abort, wait_ns);
      if (__shfl_sync(0xffffffffu, ok ? 1 : 0, 0) == 0) return;
      __threadfence_block();
      const int r0 = c * kTeamRows2;
      const int m = imin(kTeamRows2, len - r0);
      if (lane < m)
        precompute_row2d<GRAD, K, SPEC>(P, slot * kTeamRows2 + lane, tt, slow, o, sp,
                                        i0 + (r0 + lane) * step, j, sgnvz, sgnvx, sgntz, sgntx,
                                        NZ, NX);
      __syncwarp();
      if (lane == 0) {
        __threadfence_block();
        *(volatile unsigned long long*)&S.ready[slot] = tag2(pass, c);
      }
    }
  } else if (lane == 0) {
    double tv = tt[(long long)(i0 - sgntz) * NX + j];
    int i = i0;
    for (int c = 0; c < nch; ++c) {
      const int slot = c % kTeamSlots2;
      if (!wait_tag2(&S.ready[slot], tag2(pass, c), &S.abort, wait_ns)) return;
      __threadfence_block();
      const int m = imin(kTeamRows2, len - c * kTeamRows2);
      const int qb = slot * kTeamRows2;
      double t0n = tt[(long long)i * NX + j];
      Row2 rn = load_row2(P, qb);
      for (int q = qb; q < qb + m; ++q, i += step) {
        const double t0 = t0n;
        const Row2 r = rn;
        if (q + 1 < qb + m) {
          t0n = tt[(long long)(i + step) * NX + j];
          rn = load_row2(P, q + 1);
        }
        unsigned code;
        double tnew;
        if (SPEC && deq(tv, r.tvs)) {
          tnew = r.tns;
          code = r.cds;
          ++hits;
        } else {
          tnew = eval_node2d<GRAD, K>(o, sp, P, r, q, i, j, sgntz, sgntx, tv, t0, code);
        }
        if (!eq2<K>(tnew, t0)) {
          const long long n = (long long)i * NX + j;
          tt[n] = tnew;
          if (GRAD) rec[n] = (uint8_t)code;
        }
        tv = tnew;
      }
      __threadfence_block();
      *(volatile unsigned long long*)&S.consumed = tag2(pass, c);
    }
  }
}

template <bool GRAD, bool K, bool SPEC>
__device__ __noinline__ void team_sweeps2d(Pre2Ring& P, TeamSync2& S, double* tt, uint8_t* rec,
                                           const double* slow, const Ops2& o, const Source2& sp,
                                           int nsweep, int NZ, int NX, unsigned long long wait_ns,
                                           unsigned long long* stats) {
  unsigned long long hits = 0, pass = 0;
  for (int sw = 0; sw < nsweep; ++sw) {
    for (int j = 1; j < NX; ++j) {
      team_pass2d<GRAD, K, SPEC>(P, S, tt, rec, slow, o, sp, j, 1, NZ - 1, 1, 1, 1, 1, NZ, NX,
                                 ++pass, wait_ns, hits);
      team_pass2d<GRAD, K, SPEC>(P, S, tt, rec, slow, o, sp, j, NZ - 2, 0, 0, 1, -1, 1, NZ, NX,
                                 ++pass, wait_ns, hits);
    }
    for (int j = NX - 2; j >= 0; --j) {
      team_pass2d<GRAD, K, SPEC>(P, S, tt, rec, slow, o, sp, j, 1, NZ - 1, 1, 0, 1, -1, NZ, NX,
                                 ++pass, wait_ns, hits);
      team_pass2d<GRAD, K, SPEC>(P, S, tt, rec, slow, o, sp, j, NZ - 2, 0, 0, 0, -1, -1, NZ, NX,
                                 ++pass, wait_ns, hits);
    }
  }
  if (threadIdx.x == 0) {
    atomicAdd(stats, (unsigned long long)nsweep * 4ull * (unsigned long long)(NZ - 1) * (NX - 1));
    atomicAdd(stats + 1, hits);
  }
}

// A block of kTeamWarps2 warps per source (blockIdx.x): thread 0 runs the
// first propagation, the block checks it for non-finite values, then the
// sweeps run as above.
template <bool GRAD, bool SPEC>
__global__ void __launch_bounds__(kTeamWarps2 * 32)
    solve2d_team_kernel(const double* slow, const double* src, int nz, int nx, int nsweep,
                        Ops2 o, double* tt_all, uint8_t* rec_all, Source2* params,
                        double* vzero_out, bool keys, unsigned long long wait_ns,
                        unsigned long long* stats, int* status) {
  __shared__ Pre2Ring P;
  __shared__ TeamSync2 S;
  __shared__ Source2 sps;
  const int s = blockIdx.x;
  const int tid = threadIdx.x;
  const int NZ = nz + 1, NX = nx + 1;
  const long long nodes = (long long)NZ * NX;
  double* tt = tt_all + (long long)s * nodes;
  uint8_t* rec = GRAD ? rec_all + (long long)s * nodes : nullptr;
  if (tid == 0) {
    const Source2 sp = first_propagation2d<GRAD>(slow, src + 2 * s, nz, nx, o, tt, rec);
    params[s] = sp;
    vzero_out[s] = sp.vzero;
    sps = sp;
    S.consumed = 0;
    S.abort = 0;
  }
  if (tid < kTeamSlots2) S.ready[tid] = 0;
  __syncthreads();
  const Source2 sp = sps;
  bool finite = true;
  for (int jj = tid; jj < NX; jj += blockDim.x)
    for (int r = sp.zsi; r <= imin(sp.zsi + 1, NZ - 1); ++r)
      finite = finite && is_finite(tt[(long long)r * NX + jj]);
  for (int ii = tid; ii < NZ; ii += blockDim.x)
    for (int c = sp.xsi; c <= imin(sp.xsi + 1, NX - 1); ++c)
      finite = finite && is_finite(tt[(long long)ii * NX + c]);
  finite = __syncthreads_and(finite ? 1 : 0) != 0 && keys;
  if (finite)
    team_sweeps2d<GRAD, true, SPEC>(P, S, tt, rec, slow, o, sp, nsweep, NZ, NX, wait_ns, stats);
  else
    team_sweeps2d<GRAD, false, SPEC>(P, S, tt, rec, slow, o, sp, nsweep, NZ, NX, wait_ns, stats);
  __syncthreads();
  if (tid == 0 && *(volatile int*)&S.abort) atomicCAS(status, 0, (int)kDeviceWaitTimeout);
}

__global__ void fill2d_kernel(double* tt, uint8_t* rec, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    tt[q] = kBig;
    if (rec) rec[q] = 4;
  }
}

// Gradient post-pass, _fteik2d.py:623-639.  With an off-grid source the 4
// nodes around it start from their analytic derivatives (_fteik2d.py:370-375).
__global__ void grad2d_kernel(const double* tt, const uint8_t* rec, const Source2* params,
                              int nsrc, int NZ, int NX, double dz, double dx, double* ttgrad) {
  const long long nodes = (long long)NZ * NX;
  const long long total = nodes * nsrc;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(q / nodes);
    const long long n = q - (long long)s * nodes;
    const int i = (int)(n / NX), j = (int)(n - (long long)i * NX);
    const Source2 p = params[s];
    double g0 = 0.0, g1 = 0.0;
    if (p.iflag == 2 && (unsigned)(i - p.zsi) <= 1u && (unsigned)(j - p.xsi) <= 1u)
      t_anad2(i, j, dz, dx, p.zsa, p.xsa, p.vzero, g0, g1);
    const int code = rec[q];
    const int cz = code / 3 - 1, cx = code % 3 - 1;
    const double tq = tt[q];
    if (cz != 0) g0 = (double)cz * (tq - tt[q - (long long)cz * NX]) / dz;
    if (cx != 0) g1 = (double)cx * (tq - tt[q - cx]) / dx;
    const double gn = sqrt(g0 * g0 + g1 * g1);
    if (gn > 0.0) {
      g0 /= gn;
      g1 /= gn;
    }
    ttgrad[2 * q] = g0;
    ttgrad[2 * q + 1] = g1;
  }
}

struct Layout2 {
  size_t status, params, src, rec, total;
};

static size_t align_up2(size_t x) { return (x + 255) & ~(size_t)255; }

static Layout2 layout2(int nz, int nx, int nsrc, int grad) {
  const size_t nodes = (size_t)(nz + 1) * (nx + 1);
  Layout2 L;
  size_t off = 0;
  L.status = off;  // int status; then at byte 8 the chain statistics (u64 nodes, u64 hits)
  off = align_up2(off + 32);
  L.params = off;
  off = align_up2(off + sizeof(Source2) * (size_t)nsrc);
  L.src = off;
  off = align_up2(off + sizeof(double) * 2 * (size_t)nsrc);
  L.rec = off;
  if (grad) off = align_up2(off + nodes * (size_t)nsrc);
  L.total = off;
  return L;
}

}  // namespace fteik

using namespace fteik;

extern "C" size_t fteik2d_workspace_bytes(int nz, int nx, int nsrc, int grad) {
  if (nz < 1 || nx < 1 || nsrc < 1) return 0;
  return layout2(nz, nx, nsrc, grad).total;
}

extern "C" int fteik2d_solve(const double* slow, int nz, int nx, double dz, double dx,
                             const double* sources, int nsrc, int nsweep, int grad, double* tt,
                             double* ttgrad, double* vzero, void* workspace,
                             size_t workspace_bytes, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nz < 2 || nx < 2 || nsrc < 1 || nsweep < 0 || !slow || !sources || !tt || !vzero ||
      !workspace || (grad && !ttgrad))
    return kInvalidArgument;
  if (!(dz > 1e-100 && dz < 1e100 && dx > 1e-100 && dx < 1e100)) return kInvalidArgument;
  const Layout2 L = layout2(nz, nx, nsrc, grad);
  if (workspace_bytes < L.total) return kWorkspaceTooSmall;
  for (int s = 0; s < nsrc; ++s) {  // _fteik2d.py:296-300
    const double z = sources[2 * s], x = sources[2 * s + 1];
    if (!((0.0 <= z && z <= dz * nz) && (0.0 <= x && x <= dx * nx))) return kSourceOutOfBound;
  }
  char* ws = (char*)workspace;
  const Ops2 o = make_ops2(dz, dx);
  Source2* params = (Source2*)(ws + L.params);
  double* src_dev = (double*)(ws + L.src);
  uint8_t* rec = grad ? (uint8_t*)(ws + L.rec) : nullptr;
  const long long nodes = (long long)(nz + 1) * (nx + 1);
  const long long ntot = nodes * nsrc;
  FTEIK_CHECK(cudaMemsetAsync(ws + L.status, 0, 32, st));
  FTEIK_CHECK(cudaMemcpyAsync(src_dev, sources, sizeof(double) * 2 * (size_t)nsrc,
                              cudaMemcpyHostToDevice, st));
  fill2d_kernel<<<grid_for(ntot, 256), 256, 0, st>>>(tt, rec, ntot);
  const int blocks = (nsrc + 31) / 32;
  const bool keys = option_value(kOptSweep2dKeys) != 0;
  // A warp per source while every source's warp has an SM sub-partition to
  // itself (its FP64 pipe is what the chain waits on); beyond that, one
  // thread per source, where each warp instruction serves 32 chains.
  const long long warp_opt = option_value(kOptSweep2dWarp);
  const int mode = warp_opt >= 0 ? (int)warp_opt
                                 : (nsrc <= sm_count() ? 2 : (nsrc <= 4 * sm_count() ? 1 : 0));
  const bool spec = option_value(kOptSweep2dSpec) != 0;
  unsigned long long* stats = (unsigned long long*)(ws + L.status + 8);
  if (mode == 2) {
    // a block per source while every source has an SM to itself
    int* status = (int*)(ws + L.status);
    const long long wopt = option_value(kOptSweep2dWaitNs);
    const unsigned long long wait_ns = wopt >= 0 ? (unsigned long long)wopt : kTeamWaitNs2;
#define FTEIK_T2(G, S)                                                                   \
  solve2d_team_kernel<G, S><<<nsrc, kTeamWarps2 * 32, 0, st>>>(                          \
      slow, src_dev, nz, nx, nsweep, o, tt, rec, params, vzero, keys, wait_ns, stats, status)
    if (grad) {
      if (spec) FTEIK_T2(true, true); else FTEIK_T2(true, false);
    } else {
      if (spec) FTEIK_T2(false, true); else FTEIK_T2(false, false);
    }
#undef FTEIK_T2
  } else if (mode == 1) {
#define FTEIK_W2(G, S)                                                                  \
  solve2d_warp_kernel<G, S><<<nsrc, 32, 0, st>>>(slow, src_dev, nz, nx, nsweep, o, tt, rec, \
                                                 params, vzero, keys, stats)
    if (grad) {
      if (spec) FTEIK_W2(true, true); else FTEIK_W2(true, false);
    } else {
      if (spec) FTEIK_W2(false, true); else FTEIK_W2(false, false);
    }
#undef FTEIK_W2
  } else if (grad) {
    solve2d_kernel<true><<<blocks, 32, 0, st>>>(slow, src_dev, nsrc, nz, nx, nsweep, o, tt, rec,
                                                 params, vzero, keys);
  } else {
    solve2d_kernel<false><<<blocks, 32, 0, st>>>(slow, src_dev, nsrc, nz, nx, nsweep, o, tt,
                                                  rec, params, vzero, keys);
  }
  FTEIK_CHECK(cudaGetLastError());
  if (grad) {
    grad2d_kernel<<<grid_for(ntot, 256), 256, 0, st>>>(tt, rec, params, nsrc, nz + 1, nx + 1,
                                                       dz, dx, ttgrad);
    FTEIK_CHECK(cudaGetLastError());
  }
  return fteik_workspace_status(workspace, stream);
}

extern "C" int fteik2d_chain_stats(const void* workspace, unsigned long long* nodes,
                                   unsigned long long* hits, void* stream) {
  if (!workspace || !nodes || !hits) return kInvalidArgument;
  unsigned long long v[2] = {0, 0};
  FTEIK_CHECK(cudaMemcpyAsync(v, (const char*)workspace + 8, sizeof(v), cudaMemcpyDeviceToHost,
                              (cudaStream_t)stream));
  FTEIK_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
  *nodes = v[0];
  *hits = v[1];
  return kOk;
}
