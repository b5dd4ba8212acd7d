// 3D FTeik solver for GB300: fteikpy/_fteik/_fteik3d.py rebuilt as CUDA.
//
// Layout in HBM (C order, float64 unless noted):
//   slow  [nz][nx][ny]                cells (shared by every source)
//   tt    [nsrc][NZ][NX][NY]          nodes, NZ = nz + 1 ...
//   ttgrad[nsrc][NZ][NX][NY][3]
//   rec   [nsrc][NZ][NX][NY] uint8    branch record: the sign triple that the
//                                     reference keeps in ttsgn
//                                     (_fteik3d.py:166-200), packed as
//                                     (sz+1)*9 + (sx+1)*3 + (sy+1)
//
// Schedule.  One directional sweep (_fteik3d.py:217-391) only reads the 7
// upwind neighbours of a node and the node itself (_fteik3d.py:68-74,162), so
// any order that visits a node after its upwind neighbours reproduces the
// reference's loop exactly.  The (j, k) plane is cut into 4 x 8 pencils that
// run through the whole depth; one warp owns one pencil, lane (lj, lk) owns one
// (j, k) column, and at step s lane (lj, lk) updates row r = s - lj - lk: a
// skewed wavefront inside the pencil where the upwind values of the same
// pencil arrive through warp shuffles of the three previous results.  Values
// from upwind pencils come from L2 after the upwind pencil has published its
// progress.  All 8 * nsweep sweeps of all sources run in ONE persistent launch:
// warps take (sweep, pencil, source) work items from a ticket counter in
// dependency order and wait (bounded) on per-pencil progress counters for
//   * the upwind pencils of the same sweep (read-after-write),
//   * their own pencil in the previous sweep, and the pencils that read it in
//     the previous sweep (write-after-read),
// so consecutive sweeps and all sources overlap without grid-wide barriers.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fteik_gb300.h"
#include "runtime.h"
#include "solve3d.cuh"

namespace fteik {

constexpr int kWarpsPerBlock = 4;
// Batches of at least this many sources read precomputed coefficient arrays.
constexpr int kCoefMinSources = 4;


// Plane operator of _fteik3d.py:113-117 (and its ZY / XY twins):
//   ((p*cp + q*cq) + sqrt(q4 - prod*(ta-tb)^2)) / sum,  q4 = 4*v^2*sum
__device__ __forceinline__ double plane_op(double p, double cp, double q, double cq, double d,
                                           double q4, double prod, const Recip& r) {
  double num = p * cp + q * cq;
  double rad = q4 - prod * (d * d);
  return div_dd(num + sqrt_rn(rad), r);
}


// Where the update gets its coefficients from.  Both give the same values:
//  * CoefArrays reads the precomputed arrays (one read each; pays off when
//    many sources share them, as they then stay in L2);
//  * CoefCells derives them from the 8 slowness cells around the node,
//    U[a][b][c] indexed upwind-first (a = 0 is the reference's cell row i1 =
//    i - sgnvz, a = 1 the other row of the pair {max(i-1,0), min(i,nz-2)};
//    b, c likewise along j, k), which stay in L2 for any number of sources.
template <class I>
struct CoefArraysT {
  const Coef3& C;
  I oz1, ox1, oy1, ozx, ozy, oxy, ot3;
  __device__ __forceinline__ double z1() const { return __ldg(C.z1 + oz1); }
  __device__ __forceinline__ double x1() const { return __ldg(C.x1 + ox1); }
  __device__ __forceinline__ double y1() const { return __ldg(C.y1 + oy1); }
  __device__ __forceinline__ double zxa() const { return __ldg(C.zxa + ozx); }
  __device__ __forceinline__ double zxb() const { return __ldg(C.zxb + ozx); }
  __device__ __forceinline__ double zxq() const { return __ldg(C.zxq + ozx); }
  __device__ __forceinline__ double zya() const { return __ldg(C.zya + ozy); }
  __device__ __forceinline__ double zyb() const { return __ldg(C.zyb + ozy); }
  __device__ __forceinline__ double zyq() const { return __ldg(C.zyq + ozy); }
  __device__ __forceinline__ double xya() const { return __ldg(C.xya + oxy); }
  __device__ __forceinline__ double xyb() const { return __ldg(C.xyb + oxy); }
  __device__ __forceinline__ double xyq() const { return __ldg(C.xyq + oxy); }
  __device__ __forceinline__ double t3() const { return __ldg(C.t3 + ot3); }
};
using CoefArrays = CoefArraysT<long long>;

struct CoefCells {
  double U[2][2][2];
  const Ops3& o;
  __device__ __forceinline__ double vzx() const { return pmin(U[0][0][0], U[0][0][1]); }
  __device__ __forceinline__ double vzy() const { return pmin(U[0][0][0], U[0][1][0]); }
  __device__ __forceinline__ double vxy() const { return pmin(U[0][0][0], U[1][0][0]); }
  __device__ __forceinline__ double z1() const {
    return o.dz * pmin(pmin(U[0][0][0], U[0][0][1]), pmin(U[0][1][0], U[0][1][1]));
  }
  __device__ __forceinline__ double x1() const {
    return o.dx * pmin(pmin(U[0][0][0], U[1][0][0]), pmin(U[0][0][1], U[1][0][1]));
  }
  __device__ __forceinline__ double y1() const {
    return o.dy * pmin(pmin(U[0][0][0], U[0][1][0]), pmin(U[1][0][0], U[1][1][0]));
  }
  __device__ __forceinline__ double zxa() const { return o.dx * vzx(); }
  __device__ __forceinline__ double zxb() const { return o.dz * vzx(); }
  __device__ __forceinline__ double zxq() const { const double v = vzx(); return times4(v * v) * o.szx; }
  __device__ __forceinline__ double zya() const { return o.dy * vzy(); }
  __device__ __forceinline__ double zyb() const { return o.dz * vzy(); }
  __device__ __forceinline__ double zyq() const { const double v = vzy(); return times4(v * v) * o.szy; }
  __device__ __forceinline__ double xya() const { return o.dy * vxy(); }
  __device__ __forceinline__ double xyb() const { return o.dx * vxy(); }
  __device__ __forceinline__ double xyq() const { const double v = vxy(); return times4(v * v) * o.sxy; }
  __device__ __forceinline__ double t3() const { return U[0][0][0] * U[0][0][0] * o.dsum * 9.0; }
};

// One node update, _fteik3d.py:38-200, with the slowness-only factors taken
// from the coefficient provider c (see Coef3 for which factor is which).
// Plane operator of plane P (0 ZX, 1 ZY, 2 XY, _fteik3d.py:106-143) on its
// inputs (u, w, x) = (tv, te, tev), (tv, tn, tnv) or (te, tn, ten), for a node
// whose guard holds; q4 = 4 v^2 (sum of the plane's two inverse squares).
// The reference forms ta = tev + te - tv, tb = tev - te + tv for ZX and
// ta = u - w + x, tb = w - u + x for ZY and XY; both are written as
// (p1 + p2) + p3 with negated operands (x - y is x + (-y) exactly), so one
// instruction sequence serves every plane when P differs between lanes.
__device__ __forceinline__ double plane3(int P, double u, double w, double x, double q4,
                                         const Ops3& o) {
  const bool zx = P == 0;
  // operands picked first, so that each sum is one add sequence for any P
  const double a1 = zx ? x : u, a2 = dflip(w, !zx), a3 = zx ? dneg(u) : x;
  const double b1 = zx ? x : w, b2 = dneg(zx ? w : u), b3 = zx ? u : x;
  const double ta = (a1 + a2) + a3;
  const double tb = (b1 + b2) + b3;
  const double p = zx ? tb : ta, q = zx ? ta : tb;
  const double cp = P == 2 ? o.dx2i : o.dz2i;
  const double cq = P == 0 ? o.dx2i : o.dy2i;
  const double prod = P == 0 ? o.dz2dx2 : P == 1 ? o.dz2dy2 : o.dx2dy2;
  const Recip& r = P == 0 ? o.rzx : P == 1 ? o.rzy : o.rxy;
  return plane_op(p, cp, q, cq, ta - tb, q4, prod, r);
}

// 3D operator, _fteik3d.py:145-159, for a node whose guard
// max(tv, te, tn) < min(t1d, t2d) holds; t2 = s^2 * dsum * 9.
__device__ __forceinline__ double op3d(double tv, double te, double tn, double tev, double ten,
                                       double tnv, double tnve, double t2, const Ops3& o) {
  const double htn = half(tn), hten = half(ten), htv = half(tv), htev = half(tev);
  const double htnv = half(tnv), hte = half(te);
  double ta = te - htn + hten - htv + htev - tnv + tnve;
  double tb = tv - htn + htnv - hte + htev - ten + tnve;
  double tc = tn - hte + hten - htv + htnv - tev + tnve;
  double dab = ta - tb, dbc = tb - tc, dac = ta - tc;
  double t3 = o.dz2dx2 * (dab * dab);
  t3 += o.dz2dy2 * (dbc * dbc);
  t3 += o.dx2dy2 * (dac * dac);
  if (!dle(t3, t2)) return kBig;
  double t1 = tb * o.dz2i + ta * o.dx2i + tc * o.dy2i;
  return div_dd(t1 + sqrt_rn(t2 - t3), o.rsum);
}

// Minimum with the old value and the branch record, _fteik3d.py:161-200.
template <bool GRAD>
__device__ __forceinline__ double finish3d(double t0, double t1d1, double t1d2, double t1d3,
                                           double t2d1, double t2d2, double t2d3, double t3d,
                                           int sz, int sx, int sy, uint8_t& code) {
  const double t1d = dmin(dmin(t1d1, t1d2), t1d3);
  const double t2d = dmin(dmin(t2d1, t2d2), t2d3);
  const double tnew = dmin(dmin(dmin(t0, t1d), t2d), t3d);
  if (GRAD && !deq(tnew, t0)) {
    int a, b, c;
    if (deq(tnew, t1d1)) {
      a = sz; b = 0; c = 0;
    } else if (deq(tnew, t1d2)) {
      a = 0; b = sx; c = 0;
    } else if (deq(tnew, t1d3)) {
      a = 0; b = 0; c = sy;
    } else if (deq(tnew, t2d1)) {
      a = sz; b = sx; c = 0;
    } else if (deq(tnew, t2d2)) {
      a = sz; b = 0; c = sy;
    } else if (deq(tnew, t2d3)) {
      a = 0; b = sx; c = sy;
    } else {
      a = sz; b = sx; c = sy;
    }
    code = (uint8_t)((a + 1) * 9 + (b + 1) * 3 + (c + 1));
  }
  return tnew;
}

// The bound tests below allow a slack of 2^-43 M, M the largest of their
// inputs (all >= 0).  mh, the largest of the inputs' high words (which order
// like the values), bounds M < D(mh + 1) (D(h): the double whose high word is h
// and low word 0), so slack_above(mh) = D(mh + 1 - 43 * 2^20) as a float is a
// safe upper bound of 2^-43 M.  A larger slack only makes the tests stricter.
__device__ __forceinline__ int hi_max8(double a, double b, double c, double d, double e,
                                       double f, double g, double h) {
  return max(max(max(__double2hiint(a), __double2hiint(b)), max(__double2hiint(c), __double2hiint(d))),
             max(max(__double2hiint(e), __double2hiint(f)), max(__double2hiint(g), __double2hiint(h))));
}
// The slack bound applies: M neither tiny (exponent field > 44) nor infinite
// or NaN.
__device__ __forceinline__ bool slack_applies(int mh) {
  const int e = mh >> 20;
  return e > 44 && e < 2047;
}
__device__ __forceinline__ float slack_above(int mh) {
  return f_above(__hiloint2double(mh - (43 << 20), 0));
}

// True when the node provably keeps t0 in this sweep, on a grid with equal
// spacings.  There every plane operator's value is its diagonal input plus a
// non-negative root term (_fteik3d.py:113-117 with dz2i = dx2i: ta + tb =
// 2 tev), and the 3D operator's is tnve plus one (ta + tb + tc = 3 tnve,
// _fteik3d.py:149-158); computed in double precision each lies within
// 2^-46 * M of that bound, M the largest input.  So if every 1D candidate is
// >= t0 and every diagonal input is >= t0 + 2^-43 * M, no operator can beat
// t0 (the minimum keeps t0 on ties) and the update is skipped.  (Also
// accepting nodes whose plane guards fail would catch more of them, but the
// guards' coefficient reads then run for every node and cost more than the
// extra skips save.)
// Both tests are decided with float bounds (f_below / f_above, directed
// float additions), so no FP64 instruction runs: t0 <= RN(tv + z1) follows
// from f_above(t0) <= f_below(tv) + f_below(z1) rounded down, and
// RN(t0 + 2^-43 M) <= tev from the rounded-up sum <= f_below(tev).  A test
// the floats cannot decide (values within about 2^-20 of each other) counts
// as failed, which only gives up a skip: the update then runs in full.  z1,
// x1, y1 are the 1D candidates' spacing-times-slowness terms (t1d1 = tv + z1,
// _fteik3d.py:76-104); mh is hi_max8 of the node's eight values.
__device__ __forceinline__ bool keeps_t0(double t0, int mh, double z1, double x1, double y1,
                                         double tv, double te, double tn, double tev, double ten,
                                         double tnv, double tnve) {
  const float t0u = f_above(t0);
  if (!(t0u <= __fadd_rd(f_below(tv), f_below(z1)) && t0u <= __fadd_rd(f_below(te), f_below(x1)) &&
        t0u <= __fadd_rd(f_below(tn), f_below(y1))))
    return false;
  if (!slack_applies(mh)) return false;
  const float thr = __fadd_ru(t0u, slack_above(mh));  // >= t0 + 2^-43 M
  return thr <= f_below(tev) && thr <= f_below(ten) && thr <= f_below(tnv) &&
         thr <= f_below(tnve);
}

// Operators that provably cannot beat t0, for a node that may change (equal
// spacings h).  A plane operator whose guard holds is at least its diagonal
// input plus h v (v its minimum slowness): with dz2i = dx2i = c its value is
// diag + sqrt(rad) / 2c (ta + tb = 2 diag, _fteik3d.py:113-117), and the
// guard |te - tv| < h v bounds (ta - tb)^2 = 4 (te - tv)^2 < 4 h^2 v^2, so
// rad = 8 c v^2 - c^2 (ta - tb)^2 > 4 c v^2 and sqrt(rad) / 2c > v / sqrt(c)
// = h v.  Computed in double the value stays within 2^-48 M of that bound, M
// the largest input (h v included), so an operator with diag + h v (the
// guard's own coefficient a = h v) >= t0 + 2^-43 M cannot beat t0.  The 3D
// operator is at least tnve likewise (ta + tb + tc = 3 tnve,
// _fteik3d.py:149-158).  Such an operator is left out (its value as Big)
// when that keeps the 3D operator's guard max(tv, te, tn) < min(t1d, t2d) as
// it is: the guard fails anyway (max(tv, te, tn) >= t1d), or the plane
// operator provably exceeds max(tv, te, tn) (diag + h v >= that max +
// 2^-43 M).  Its value, being >= t0, takes no part in the minimum or the
// branch record either.  a_zx, a_zy, a_xy: the planes' guard coefficients.
// Returns the mask of the plane operators (bit P) and of the 3D operator
// (bit 3) that may be left out; 0 when the bound does not apply (M tiny,
// infinite or NaN; mh is hi_max8 of the node's eight values).  The sums are
// bounded with floats rounded the safe way
// (f_above, f_below, __fadd_ru, __fadd_rd), so a test holds only when the
// FP64 sums would pass it too, and no FP64 instruction runs; the few tests
// the floats cannot decide leave their operator in.
__device__ __forceinline__ unsigned dead_operators(double t0, int mh, double t1d, double tv,
                                                   double te, double tn, double tev, double ten,
                                                   double tnv, double tnve, double a_zx,
                                                   double a_zy, double a_xy) {
  mh = max(max(mh, __double2hiint(a_zx)), max(__double2hiint(a_zy), __double2hiint(a_xy)));
  if (!slack_applies(mh)) return 0u;
  const float eps = slack_above(mh);                                   // >= 2^-43 M
  const float thr = __fadd_ru(f_above(t0), eps);                       // >= t0 + 2^-43 M
  const double mx = dmax(dmax(tv, te), tn);
  const bool no3d = dle(t1d, mx);
  const float thr_mx = __fadd_ru(f_above(mx), eps);
  // <= tev + a_zx, tnv + a_zy, ten + a_xy
  const float b_zx = __fadd_rd(f_below(tev), f_below(a_zx));
  const float b_zy = __fadd_rd(f_below(tnv), f_below(a_zy));
  const float b_xy = __fadd_rd(f_below(ten), f_below(a_xy));
  unsigned dead = 0u;
  if (thr <= b_zx && (no3d || thr_mx <= b_zx)) dead |= 1u;
  if (thr <= b_zy && (no3d || thr_mx <= b_zy)) dead |= 2u;
  if (thr <= b_xy && (no3d || thr_mx <= b_xy)) dead |= 4u;
  if (thr <= f_below(tnve)) dead |= 8u;
  return dead;
}

// One node update, _fteik3d.py:38-200.  Takes the three 1D candidates
// (_fteik3d.py:76-104: t1d1 = tv + c.z1() ...), which the caller computes
// first to test whether the node can change.  With `bounds` (equal
// spacings), operators that provably cannot beat t0 are left out
// (dead_operators; mh is hi_max8 of the node's eight values).
// A plane operator's guard u < v + a && v < u + b (_fteik3d.py:110,122,134:
// u, v the two face neighbours, a, b >= 0 the guard's spacing-times-slowness
// factors) with one addition instead of two.  The clause whose left operand
// is the smaller holds by itself, as RN(w + c) >= w for c >= 0; with u == v
// both hold exactly when u < RN(u + min(a, b)), RN(u + .) being monotone.
__device__ __forceinline__ bool plane_guard(double u, double v, double a, double b) {
  const bool ul = dlt(u, v), vl = dlt(v, u);
  const double lo = ul ? u : v, hi = ul ? v : u;
  const double c = ul ? b : (vl ? a : dmin(a, b));
  return dlt(hi, lo + c);
}

// The same guard decided with float bounds where they suffice: 1 when
// hi < RN(lo + c) (f_above(hi) < the float sum rounded down, which is a
// double <= lo + c), 0 when it fails (the rounded-up sum <= f_below(hi)), and
// -1 when the floats cannot tell (hi and lo + c within about 2^-20 of each
// other), where the caller runs plane_guard.  No FP64 instruction runs.
__device__ __forceinline__ int plane_guard_bound(double u, double v, double a, double b) {
  const bool ul = dlt(u, v), vl = dlt(v, u);
  const double lo = ul ? u : v, hi = ul ? v : u;
  const double c = ul ? b : (vl ? a : dmin(a, b));
  if (f_above(hi) < __fadd_rd(f_below(lo), f_below(c))) return 1;
  if (__fadd_ru(f_above(lo), f_above(c)) <= f_below(hi)) return 0;
  return -1;
}

template <bool GRAD, class CP>
__device__ __forceinline__ double node_update3d(double t1d1, double t1d2, double t1d3, double tv,
                                                double te, double tn, double tev, double ten,
                                                double tnv, double tnve, double t0, int mh,
                                                const CP& c, const Ops3& o, int sz, int sx,
                                                int sy, bool bounds, uint8_t& code) {
  const double t1d = dmin(dmin(t1d1, t1d2), t1d3);
  const double a_zx = c.zxa(), a_zy = c.zya(), a_xy = c.xya();
  int gzx = plane_guard_bound(tv, te, a_zx, c.zxb());
  int gzy = plane_guard_bound(tv, tn, a_zy, c.zyb());
  int gxy = plane_guard_bound(te, tn, a_xy, c.xyb());
  // The FP64 guard where the floats cannot decide: rare, so a branch that
  // the lanes here take together only when one of them needs it.
  if (__any_sync(__activemask(), (gzx | gzy | gxy) < 0)) {
    if (gzx < 0) gzx = plane_guard(tv, te, a_zx, c.zxb());
    if (gzy < 0) gzy = plane_guard(tv, tn, a_zy, c.zyb());
    if (gxy < 0) gxy = plane_guard(te, tn, a_xy, c.xyb());
  }
  const unsigned dead =
      bounds ? dead_operators(t0, mh, t1d, tv, te, tn, tev, ten, tnv, tnve, a_zx, a_zy, a_xy)
             : 0u;
  double t2d1 = kBig, t2d2 = kBig, t2d3 = kBig;
  if (gzx && !(dead & 1u)) t2d1 = plane3(0, tv, te, tev, c.zxq(), o);
  if (gzy && !(dead & 2u)) t2d2 = plane3(1, tv, tn, tnv, c.zyq(), o);
  if (gxy && !(dead & 4u)) t2d3 = plane3(2, te, tn, ten, c.xyq(), o);
  const double t2d = dmin(dmin(t2d1, t2d2), t2d3);
  double t3d = kBig;
  if (!(dead & 8u) && dlt(dmax(dmax(tv, te), tn), dmin(t1d, t2d)))
    t3d = op3d(tv, te, tn, tev, ten, tnv, tnve, c.t3(), o);
  return finish3d<GRAD>(t0, t1d1, t1d2, t1d3, t2d1, t2d2, t2d3, t3d, sz, sx, sy, code);
}

// Tape entry of a change of node sn (= source * nodes + n) in sweep e: its
// operator code, and the value t0 it replaced unless this is the node's first
// change (see Tape3).  A full overflow table flags FTEIK_TAPE_OVERFLOW, which
// also ends the solve early (its waits give up once the status is set): the
// caller retries with more history slots.
__device__ __forceinline__ void tape_record(const Tape3& P, int* status, long long sn, int e,
                                            uint8_t code, double t0) {
  uint8_t* rec = P.code + sn * P.E;
  const int m = tape_changes_before(rec, e) + 1;  // this change's number
  rec[e] = code;
  if (m < 2) return;
  if (m - 2 < P.H) {
    P.hist[sn * P.H + (m - 2)] = t0;
    return;
  }
  const unsigned long long key = tape_key(sn, m);
  unsigned long long h = tape_slot(key, P.mask);
  for (int q = 0; q < kTapeProbes; ++q) {
    const unsigned long long prev = atomicCAS(P.key + h, 0ull, key);
    if (prev == 0ull || prev == key) {
      P.val[h] = t0;
      return;
    }
    h = (h + 1) & P.mask;
  }
  atomicCAS(status, 0, (int)kTapeOverflow);
}

// One model of a multi-model launch (device table built by the host).
struct Model3 {
  Ops3 o;
  const double* slow;
  Coef3 C;
  const int* no_skip;  // this model's all-Big skip flag (see coef3d_kernel)
  int keep_test;       // equal spacings: test keeps_t0 before the 2D/3D operators
  int nz, nx, ny, NZ, NX, NY;
  long long nodes;
  int PJ, PK, T;
  unsigned stride;
};

// One (model, source) pair of a multi-model launch.
struct Job3 {
  double* tt;      // this source's traveltimes
  uint8_t* rec;    // its branch record (gradients) or null
  unsigned* prog;  // its pencils' progress counters
  int model, pad;
};

struct Sweep3Args {
  // one model, nsrc sources: item t = (sweep, pencil in diagonal order, source)
  double* tt;
  uint8_t* rec;
  Coef3 C;              // precomputed coefficients (COEF variant)
  const double* slow;   // slowness cells (cell variant)
  const int* no_skip;   // set by coef3d_kernel when the all-Big skip is not exact
  Tape3 tape;           // optional (tape.code null: none): the adjoint's record of every change
  unsigned* progress;
  const int* order;
  int nz, nx, ny;  // cells
  int NZ, NX, NY;  // nodes
  long long nodes;
  int nsrc, npencils, PJ, PK, total_steps;
  unsigned stride;
  int keep_test;  // equal spacings: test keeps_t0 before the 2D/3D operators
  Ops3 o;
  // several models: item t = (sweep, items[t % items_per_epoch])
  const Model3* models;
  const Job3* jobs;
  const int2* items;  // (job, JL << 16 | KL), by diagonal, then job
  unsigned items_per_epoch;
  int ngroups;        // team kernel: groups of kTeamWarps sources
  // both
  unsigned* ticket;
  int* status;
  int nepochs;
  int chunk;  // steps between two progress publications (a power of 2)
  long long spin_limit;
};

// The persistent sweep kernel.  PW is the pencil width along j (the pencil is
// PW x 32/PW columns); MULTI takes items from the multi-model tables.
template <bool GRAD, bool COEF, int PW, bool MULTI>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    sweep3d_kernel(const __grid_constant__ Sweep3Args A) {
  constexpr int PJW = PW, PKW = 32 / PW, LAG = PJW + PKW - 2;
  const int lane = threadIdx.x & 31;
  const int lj = lane / PKW, lk = lane % PKW;
  const unsigned per_epoch = MULTI ? A.items_per_epoch : (unsigned)A.npencils * A.nsrc;
  const unsigned total_items = (unsigned)A.nepochs * per_epoch;
  const unsigned cmask = (unsigned)A.chunk - 1u;

  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(A.ticket, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= total_items) break;
    const int e = (int)(t / per_epoch);
    const unsigned rem = t - (unsigned)e * per_epoch;
    // Geometry of this item's model and source.
    const Ops3* op;
    const double* slow;
    const int* no_skip;
    Coef3 C;
    double* tts;
    uint8_t* recs;
    unsigned* prog;
    int nx, ny, NZ, NX, NY, PJ, PK, T, JL, KL, src, keep_test;
    long long nodes;
    unsigned stride;
    if constexpr (MULTI) {
      const int2 it = A.items[rem];
      const Job3 jb = A.jobs[it.x];
      const Model3& M = A.models[jb.model];
      op = &M.o;
      slow = M.slow;
      no_skip = M.no_skip;
      if (COEF) C = M.C;
      tts = jb.tt;
      recs = jb.rec;
      prog = jb.prog;
      nx = M.nx; ny = M.ny;
      NZ = M.NZ; NX = M.NX; NY = M.NY;
      PJ = M.PJ; PK = M.PK; T = M.T;
      nodes = M.nodes;
      stride = M.stride;
      keep_test = M.keep_test;
      JL = it.y >> 16;
      KL = it.y & 0xffff;
      src = it.x;
    } else {
      const int p = (int)(rem / A.nsrc);
      src = (int)(rem - (unsigned)p * A.nsrc);
      op = &A.o;
      slow = A.slow;
      no_skip = A.no_skip;
      if (COEF) C = A.C;
      tts = A.tt + (long long)src * A.nodes;
      recs = GRAD ? A.rec + (long long)src * A.nodes : nullptr;
      prog = A.progress + (long long)src * A.npencils;
      nx = A.nx; ny = A.ny;
      NZ = A.NZ; NX = A.NX; NY = A.NY;
      PJ = A.PJ; PK = A.PK; T = A.total_steps;
      nodes = A.nodes;
      stride = A.stride;
      keep_test = A.keep_test;
      JL = A.order[p] >> 16;
      KL = A.order[p] & 0xffff;
    }
    const Ops3& o = *op;
    const int NXY = NX * NY;  // nodes < 2^31 (checked by the host)
    const int dir = e & 7;
    const int sz = dir < 4 ? 1 : -1, sx = (dir & 1) ? -1 : 1, sy = (dir & 2) ? -1 : 1;
    const int J = sx > 0 ? JL : PJ - 1 - JL;
    const int K = sy > 0 ? KL : PK - 1 - KL;
    unsigned* my_prog = prog + J * PK + K;
    const unsigned base = (unsigned)e * stride;

    // Dependencies on the previous sweep: this pencil, and the pencils that
    // read it (its downwind neighbours in the previous direction).
    bool ok = true;
    if (lane == 0 && e > 0) {
      const int pd = (e - 1) & 7;
      const int psx = (pd & 1) ? -1 : 1, psy = (pd & 2) ? -1 : 1;
      const unsigned done = base - stride + (unsigned)T;
      ok = wait_geq(my_prog, done, A.status, A.spin_limit);
      const int J2 = J + psx, K2 = K + psy;
      const bool hj = J2 >= 0 && J2 < PJ, hk = K2 >= 0 && K2 < PK;
      if (ok && hj) ok = wait_geq(prog + J2 * PK + K, done, A.status, A.spin_limit);
      if (ok && hk) ok = wait_geq(prog + J * PK + K2, done, A.status, A.spin_limit);
      if (ok && hj && hk) ok = wait_geq(prog + J2 * PK + K2, done, A.status, A.spin_limit);
    }
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    if (!ok) {
      __syncwarp();
      if (lane == 0) st_release(my_prog, base + (unsigned)T);
      continue;
    }

    // Upwind pencils of this sweep.
    const int Ju = J - sx, Ku = K - sy;
    const bool hJu = Ju >= 0 && Ju < PJ, hKu = Ku >= 0 && Ku < PK;
    const unsigned* prog_j = prog + Ju * PK + K;
    const unsigned* prog_k = prog + J * PK + Ku;
    const unsigned* prog_jk = prog + Ju * PK + Ku;

    const int j = sx > 0 ? J * PJW + lj : J * PJW + (PJW - 1) - lj;
    const int k = sy > 0 ? K * PKW + lk : K * PKW + (PKW - 1) - lk;
    const bool in_grid = j < NX && k < NY;
    const bool frozen_jk = (j == (sx > 0 ? 0 : NX - 1)) || (k == (sy > 0 ? 0 : NY - 1));
    // Offsets of the coefficient reads that depend on the column only (see
    // Coef3): j1, k1 are the upwind cell indices of the reference.
    const int j1 = sx > 0 ? j - 1 : j, k1 = sy > 0 ? k - 1 : k;
    const int jk = j * NY + k;
    const int j1k = j1 * NY + k, jk1 = j * NY + k1;
    const int j1k1 = j1 * NY + k1;
    // Slowness cell offsets around the column, upwind cell first (CoefCells).
    const int jm = imax(j - 1, 0), jp = imin(j, NX - 2);
    const int km = imax(k - 1, 0), kp = imin(k, NY - 2);
    const int NYc = ny, NXYc = nx * ny;
    const int ju = (sx > 0 ? jm : jp) * NYc, jo = (sx > 0 ? jp : jm) * NYc;
    const int ku = sy > 0 ? km : kp, ko = sy > 0 ? kp : km;
    const int dj = sx * NY, dk = sy;
    const int di = sz * NXY;
    const bool may_skip = *no_skip == 0;
    const long long big_bits = __double_as_longlong(kBig);

    double r1 = 0.0, r2 = 0.0, r3 = 0.0;
    for (int s = 0; s < T; ++s) {
      if (((unsigned)s & cmask) == 0) {
        // Upwind data needed by the steps s .. s+chunk-1 of this chunk.
        const int last = imin(s + (int)cmask, T - 1);
        bool w = true;
        if (lane == 0) {
          if (hJu) w = wait_geq(prog_j, base + (unsigned)imin(last + PJW, T), A.status, A.spin_limit);
          if (w && hKu)
            w = wait_geq(prog_k, base + (unsigned)imin(last + PKW, T), A.status, A.spin_limit);
          if (w && hJu && hKu)
            w = wait_geq(prog_jk, base + (unsigned)imin(last + LAG + 1, T), A.status,
                         A.spin_limit);
          if (w) __threadfence();
        }
        w = __shfl_sync(0xffffffffu, w ? 1 : 0, 0) != 0;
        __syncwarp();
        if (!w) break;
      }
      const double uj_1 = __shfl_up_sync(0xffffffffu, r1, PKW);
      const double uj_2 = __shfl_up_sync(0xffffffffu, r2, PKW);
      const double uk_1 = __shfl_up_sync(0xffffffffu, r1, 1);
      const double uk_2 = __shfl_up_sync(0xffffffffu, r2, 1);
      const double ujk_2 = __shfl_up_sync(0xffffffffu, r2, PKW + 1);
      const double ujk_3 = __shfl_up_sync(0xffffffffu, r3, PKW + 1);
      const int r = s - lj - lk;
      const bool act = in_grid && r >= 0 && r < NZ;
      const int i = sz > 0 ? r : NZ - 1 - r;
      const int n = i * NXY + jk;
      const double t0 = act ? ld_cg(tts + n) : 0.0;
      double res = t0;
      bool upd = act && r != 0 && !frozen_jk;
      double tv = 0.0, te = 0.0, tn = 0.0, tev = 0.0, tnv = 0.0, ten = 0.0, tnve = 0.0;
      if (upd) {
        tv = r1;
        te = lj > 0 ? uj_1 : ld_cg(tts + n - dj);
        tn = lk > 0 ? uk_1 : ld_cg(tts + n - dk);
        tev = lj > 0 ? uj_2 : ld_cg(tts + n - di - dj);
        tnv = lk > 0 ? uk_2 : ld_cg(tts + n - di - dk);
        ten = (lj > 0 && lk > 0) ? ujk_2 : ld_cg(tts + n - dj - dk);
        tnve = (lj > 0 && lk > 0) ? ujk_3 : ld_cg(tts + n - di - dj - dk);
        // A node whose value and 7 upwind neighbours all still hold Big keeps
        // Big (every operator then returns at least Big; coef3d_kernel checks
        // the scale condition that makes this exact).
        if (may_skip) {
          const long long b = __double_as_longlong(t0);
          const bool all_big = b == big_bits && __double_as_longlong(tv) == b &&
                               __double_as_longlong(te) == b && __double_as_longlong(tn) == b &&
                               __double_as_longlong(tev) == b && __double_as_longlong(tnv) == b &&
                               __double_as_longlong(ten) == b && __double_as_longlong(tnve) == b;
          upd = !all_big;
        }
      }
      if (__any_sync(0xffffffffu, upd)) {
        // Coefficients (see Coef3): read lazily from the arrays, or derived
        // from the 8 slowness cells around the node.
        const int i0 = i * NXY;
        const int i1 = (sz > 0 ? i - 1 : i) * NXY;
        const CoefArraysT<int> ca{C,        i1 + jk,  i0 + j1k,  i0 + jk1,
                                  i1 + j1k, i1 + jk1, i0 + j1k1, i1 + j1k1};
        CoefCells cc{{}, o};
        // the 1D candidates' spacing-times-slowness terms (t1d1 = tv + z1 ...)
        double z1 = 0.0, x1 = 0.0, y1 = 0.0;
        int mh = 0;  // hi_max8 of the node's values, for the bound tests
        bool go = upd;
        if (upd) {
          if (COEF) {
            z1 = ca.z1();
            x1 = ca.x1();
            y1 = ca.y1();
          } else {
            const int im = imax(i - 1, 0), ip = imin(i, NZ - 2);
            const long long iu = (sz > 0 ? im : ip) * NXYc, io = (sz > 0 ? ip : im) * NXYc;
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
              for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int c = 0; c < 2; ++c)
                  cc.U[a][b][c] = __ldg(slow + (a ? io : iu) + (b ? jo : ju) + (c ? ko : ku));
            z1 = cc.z1();
            x1 = cc.x1();
            y1 = cc.y1();
          }
          if (keep_test) {
            mh = hi_max8(t0, tv, te, tn, tev, ten, tnv, tnve);
            go = !keeps_t0(t0, mh, z1, x1, y1, tv, te, tn, tev, ten, tnv, tnve);
          }
        }
        if (__any_sync(0xffffffffu, go) && go) {
          const double t1d1 = tv + z1, t1d2 = te + x1, t1d3 = tn + y1;
          uint8_t code = 0;
          res = COEF ? node_update3d<GRAD>(t1d1, t1d2, t1d3, tv, te, tn, tev, ten, tnv, tnve, t0,
                                           mh, ca, o, sz, sx, sy, keep_test != 0, code)
                     : node_update3d<GRAD>(t1d1, t1d2, t1d3, tv, te, tn, tev, ten, tnv, tnve, t0,
                                           mh, cc, o, sz, sx, sy, keep_test != 0, code);
          if (!deq(res, t0)) {
            tts[n] = res;
            if (GRAD) recs[n] = code;
            if (!MULTI && A.tape.code)
              tape_record(A.tape, A.status, (long long)src * nodes + n, e, code, t0);
          }
        }
      }
      r3 = r2;
      r2 = r1;
      r1 = res;
      if (((unsigned)(s + 1) & cmask) == 0 || s + 1 == T) {
        __syncwarp();
        if (lane == 0) {
          __threadfence();
          st_release(my_prog, base + (unsigned)(s + 1));
        }
      }
    }
    // Completion (also after an aborted wait, so that no other warp blocks).
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      st_release(my_prog, base + (unsigned)T);
    }
  }
}

// ------------------------------------------------------------- team kernel --
//
// The same sweeps for batches of sources, with the operators compacted.  In
// the warp-per-pencil kernel above every 2D and 3D operator runs as a full
// warp instruction even when few lanes need it: a plane operator's guard
// holds in about half the lanes that update, the 3D operator's in a sixth,
// and unchanged nodes (keeps_t0) idle in warps that still run.  Here a block
// of kTeamWarps warps takes one pencil of one sweep for kTeamWarps sources
// (warp w: source group * kTeamWarps + w) and steps them together.  Per step:
//   A  each lane reads its inputs (as above), forms the 1D candidates and the
//      plane guards, and queues one job per plane whose guard holds;
//   B  the block evaluates the queued plane operators 32 to a warp instruction;
//   C  each lane takes its plane results, tests the 3D guard and queues a job;
//   D  the block evaluates the queued 3D operators;
//   E  each lane forms the minimum and the branch record and writes back.
// (Evaluating the rare 3D operator in place, or queueing it before the plane
// results are known, saves two barriers per step but measured slower.)
// Operators and their operands are the same as in node_update3d, so results
// are bit-identical; only which lane evaluates an operator changes.
#ifndef FTEIK_TEAM_WARPS
#define FTEIK_TEAM_WARPS 4
#endif
constexpr int kTeamWarps = FTEIK_TEAM_WARPS;
// Resident team blocks per SM the registers are budgeted for.
#ifndef FTEIK_TEAM_MIN_BLOCKS
#define FTEIK_TEAM_MIN_BLOCKS 7
#endif

// Job q of a block's queue, whose warps queued n[0], n[1], ... jobs in
// turn: the warp w that queued it and its index l in that warp's list.
__device__ __forceinline__ void team_job(const int (&pre)[kTeamWarps + 1], int q, int& w,
                                         int& l) {
  w = 0;
  int base = 0;
#pragma unroll
  for (int x = 1; x < kTeamWarps; ++x)
    if (q >= pre[x]) {
      w = x;
      base = pre[x];
    }
  l = q - base;
}

struct TeamShared {
  // The plane jobs (written in stage A, read in stage B) and the 3D jobs
  // (written in stage C, read in stage D) share their memory: a barrier
  // separates their uses, and the smaller footprint leaves more of the SM's
  // memory to L1.
  union {
    struct {
      // plane jobs, warp w's in [w][0, n2[w]): plane, lane and inputs (u, w, x, q4)
      double ju[kTeamWarps][96], jw[kTeamWarps][96], jx[kTeamWarps][96], jq[kTeamWarps][96];
      int jid[kTeamWarps][96];  // plane * 32 + lane
    };
    struct {
      // 3D jobs: lane and inputs (tv, te, tn, tev, ten, tnv, tnve, t2)
      double kin[8][kTeamWarps][32];
      int kid[kTeamWarps][32];
    };
  };
  double r2[kTeamWarps][3][32];
  double r3[kTeamWarps][32];
  int n2[kTeamWarps], n3[kTeamWarps];
  unsigned ticket;
};

template <bool GRAD, bool COEF, int PW>
__global__ void __launch_bounds__(kTeamWarps * 32, FTEIK_TEAM_MIN_BLOCKS)
    sweep3d_team_kernel(const __grid_constant__ Sweep3Args A) {
  constexpr int PJW = PW, PKW = 32 / PW, LAG = PJW + PKW - 2;
  __shared__ TeamShared sh;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int lj = lane / PKW, lk = lane % PKW;
  const unsigned lt_mask = (1u << lane) - 1u;
  const unsigned per_epoch = (unsigned)A.npencils * A.ngroups;
  const unsigned total_items = (unsigned)A.nepochs * per_epoch;
  const unsigned cmask = (unsigned)A.chunk - 1u;
  const Ops3& o = A.o;
  const int NXY = A.NX * A.NY;  // nodes < 2^31 (checked by the host)
  const int T = A.total_steps;

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sh.ticket = atomicAdd(A.ticket, 1u);
    __syncthreads();
    const unsigned t = sh.ticket;
    if (t >= total_items) break;
    const int e = (int)(t / per_epoch);
    const unsigned rem = t - (unsigned)e * per_epoch;
    const int p = (int)(rem / A.ngroups);
    const int src = (int)(rem - (unsigned)p * A.ngroups) * kTeamWarps + warp;
    bool active = src < A.nsrc;
    const int dir = e & 7;
    const int sz = dir < 4 ? 1 : -1, sx = (dir & 1) ? -1 : 1, sy = (dir & 2) ? -1 : 1;
    const int JL = A.order[p] >> 16, KL = A.order[p] & 0xffff;
    const int J = sx > 0 ? JL : A.PJ - 1 - JL;
    const int K = sy > 0 ? KL : A.PK - 1 - KL;
    const int src_c = active ? src : 0;
    unsigned* prog = A.progress + (long long)src_c * A.npencils;
    unsigned* my_prog = prog + J * A.PK + K;
    const unsigned base = (unsigned)e * A.stride;

    // Dependencies on the previous sweep (see sweep3d_kernel).
    if (active) {
      bool ok = true;
      if (lane == 0 && e > 0) {
        const int pd = (e - 1) & 7;
        const int psx = (pd & 1) ? -1 : 1, psy = (pd & 2) ? -1 : 1;
        const unsigned done = base - A.stride + (unsigned)T;
        ok = wait_geq(my_prog, done, A.status, A.spin_limit);
        const int J2 = J + psx, K2 = K + psy;
        const bool hj = J2 >= 0 && J2 < A.PJ, hk = K2 >= 0 && K2 < A.PK;
        if (ok && hj) ok = wait_geq(prog + J2 * A.PK + K, done, A.status, A.spin_limit);
        if (ok && hk) ok = wait_geq(prog + J * A.PK + K2, done, A.status, A.spin_limit);
        if (ok && hj && hk) ok = wait_geq(prog + J2 * A.PK + K2, done, A.status, A.spin_limit);
      }
      active = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    }

    const int Ju = J - sx, Ku = K - sy;
    const bool hJu = Ju >= 0 && Ju < A.PJ, hKu = Ku >= 0 && Ku < A.PK;
    const unsigned* prog_j = prog + Ju * A.PK + K;
    const unsigned* prog_k = prog + J * A.PK + Ku;
    const unsigned* prog_jk = prog + Ju * A.PK + Ku;
    const int j = sx > 0 ? J * PJW + lj : J * PJW + (PJW - 1) - lj;
    const int k = sy > 0 ? K * PKW + lk : K * PKW + (PKW - 1) - lk;
    const bool in_grid = j < A.NX && k < A.NY;
    const bool frozen_jk = (j == (sx > 0 ? 0 : A.NX - 1)) || (k == (sy > 0 ? 0 : A.NY - 1));
    const int j1 = sx > 0 ? j - 1 : j, k1 = sy > 0 ? k - 1 : k;
    const int jk = j * A.NY + k;
    const int j1k = j1 * A.NY + k, jk1 = j * A.NY + k1;
    const int j1k1 = j1 * A.NY + k1;
    const int jm = imax(j - 1, 0), jp = imin(j, A.NX - 2);
    const int km = imax(k - 1, 0), kp = imin(k, A.NY - 2);
    const int NYc = A.ny, NXYc = A.nx * A.ny;
    const int ju = (sx > 0 ? jm : jp) * NYc, jo = (sx > 0 ? jp : jm) * NYc;
    const int ku = sy > 0 ? km : kp, ko = sy > 0 ? kp : km;
    double* tts = A.tt + (long long)src_c * A.nodes;
    uint8_t* recs = GRAD ? A.rec + (long long)src_c * A.nodes : nullptr;
    const int dj = sx * A.NY, dk = sy;
    const int di = sz * NXY;
    const bool may_skip = *A.no_skip == 0;
    const long long big_bits = __double_as_longlong(kBig);

    double r1 = 0.0, r2v = 0.0, r3v = 0.0;
    for (int s = 0; s < T; ++s) {
      if (active && ((unsigned)s & cmask) == 0) {
        const int last = imin(s + (int)cmask, T - 1);
        bool w = true;
        if (lane == 0) {
          if (hJu) w = wait_geq(prog_j, base + (unsigned)imin(last + PJW, T), A.status, A.spin_limit);
          if (w && hKu)
            w = wait_geq(prog_k, base + (unsigned)imin(last + PKW, T), A.status, A.spin_limit);
          if (w && hJu && hKu)
            w = wait_geq(prog_jk, base + (unsigned)imin(last + LAG + 1, T), A.status,
                         A.spin_limit);
          if (w) __threadfence();
        }
        active = __shfl_sync(0xffffffffu, w ? 1 : 0, 0) != 0;
      }
      // ---- stage A: inputs, 1D candidates, guards, plane jobs ----
      const double uj_1 = __shfl_up_sync(0xffffffffu, r1, PKW);
      const double uj_2 = __shfl_up_sync(0xffffffffu, r2v, PKW);
      const double uk_1 = __shfl_up_sync(0xffffffffu, r1, 1);
      const double uk_2 = __shfl_up_sync(0xffffffffu, r2v, 1);
      const double ujk_2 = __shfl_up_sync(0xffffffffu, r2v, PKW + 1);
      const double ujk_3 = __shfl_up_sync(0xffffffffu, r3v, PKW + 1);
      const int r = s - lj - lk;
      const bool act = active && in_grid && r >= 0 && r < A.NZ;
      const int i = sz > 0 ? r : A.NZ - 1 - r;
      const int n = i * NXY + jk;
      const double t0 = act ? ld_cg(tts + n) : 0.0;
      double res = t0;
      bool go = act && r != 0 && !frozen_jk;
      double tv = 0.0, te = 0.0, tn = 0.0, tev = 0.0, tnv = 0.0, ten = 0.0, tnve = 0.0;
      double t1d1 = kBig, t1d2 = kBig, t1d3 = kBig;
      bool czx = false, czy = false, cxy = false;
      const int i0 = i * NXY;
      const int i1 = (sz > 0 ? i - 1 : i) * NXY;
      const CoefArraysT<int> ca{A.C,      i1 + jk,  i0 + j1k,  i0 + jk1,
                                i1 + j1k, i1 + jk1, i0 + j1k1, i1 + j1k1};
      CoefCells cc{{}, o};
      double q_zx = 0.0, q_zy = 0.0, q_xy = 0.0;
      if (go) {
        tv = r1;
        te = lj > 0 ? uj_1 : ld_cg(tts + n - dj);
        tn = lk > 0 ? uk_1 : ld_cg(tts + n - dk);
        tev = lj > 0 ? uj_2 : ld_cg(tts + n - di - dj);
        tnv = lk > 0 ? uk_2 : ld_cg(tts + n - di - dk);
        ten = (lj > 0 && lk > 0) ? ujk_2 : ld_cg(tts + n - dj - dk);
        tnve = (lj > 0 && lk > 0) ? ujk_3 : ld_cg(tts + n - di - dj - dk);
        if (may_skip) {
          const long long b = __double_as_longlong(t0);
          go = !(b == big_bits && __double_as_longlong(tv) == b &&
                 __double_as_longlong(te) == b && __double_as_longlong(tn) == b &&
                 __double_as_longlong(tev) == b && __double_as_longlong(tnv) == b &&
                 __double_as_longlong(ten) == b && __double_as_longlong(tnve) == b);
        }
      }
      // the 1D candidates' spacing-times-slowness terms (t1d1 = tv + z1 ...)
      double z1 = 0.0, x1 = 0.0, y1 = 0.0;
      int mh = 0;  // hi_max8 of the node's values, for the bound tests
      if (go) {
        if (COEF) {
          z1 = ca.z1();
          x1 = ca.x1();
          y1 = ca.y1();
        } else {
          const int im = imax(i - 1, 0), ip = imin(i, A.NZ - 2);
          const long long iu = (sz > 0 ? im : ip) * NXYc, io = (sz > 0 ? ip : im) * NXYc;
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
              for (int c = 0; c < 2; ++c)
                cc.U[a][b][c] = __ldg(A.slow + (a ? io : iu) + (b ? jo : ju) + (c ? ko : ku));
          z1 = cc.z1();
          x1 = cc.x1();
          y1 = cc.y1();
        }
        if (A.keep_test) {
          mh = hi_max8(t0, tv, te, tn, tev, ten, tnv, tnve);
          go = !keeps_t0(t0, mh, z1, x1, y1, tv, te, tn, tev, ten, tnv, tnve);
        }
      }
      unsigned dead = 0u;  // operators that provably cannot beat t0 (dead_operators)
      // A warp whose nodes all keep t0 runs no FP64 instruction in this stage.
      if (__any_sync(0xffffffffu, go)) {
        double a_zx = 0.0, a_zy = 0.0, a_xy = 0.0;
        int gzx = 0, gzy = 0, gxy = 0;
        if (go) {
          t1d1 = tv + z1;
          t1d2 = te + x1;
          t1d3 = tn + y1;
          if (COEF) {
            a_zx = ca.zxa();
            a_zy = ca.zya();
            a_xy = ca.xya();
            gzx = plane_guard_bound(tv, te, a_zx, ca.zxb());
            gzy = plane_guard_bound(tv, tn, a_zy, ca.zyb());
            gxy = plane_guard_bound(te, tn, a_xy, ca.xyb());
          } else {
            a_zx = cc.zxa();
            a_zy = cc.zya();
            a_xy = cc.xya();
            gzx = plane_guard_bound(tv, te, a_zx, cc.zxb());
            gzy = plane_guard_bound(tv, tn, a_zy, cc.zyb());
            gxy = plane_guard_bound(te, tn, a_xy, cc.xyb());
          }
        }
        // the FP64 guard where the floats cannot decide (rare)
        if (__any_sync(0xffffffffu, (gzx | gzy | gxy) < 0)) {
          if (COEF) {
            if (gzx < 0) gzx = plane_guard(tv, te, a_zx, ca.zxb());
            if (gzy < 0) gzy = plane_guard(tv, tn, a_zy, ca.zyb());
            if (gxy < 0) gxy = plane_guard(te, tn, a_xy, ca.xyb());
          } else {
            if (gzx < 0) gzx = plane_guard(tv, te, a_zx, cc.zxb());
            if (gzy < 0) gzy = plane_guard(tv, tn, a_zy, cc.zyb());
            if (gxy < 0) gxy = plane_guard(te, tn, a_xy, cc.xyb());
          }
        }
        if (go) {
          czx = gzx > 0;
          czy = gzy > 0;
          cxy = gxy > 0;
          if (A.keep_test) {
            dead = dead_operators(t0, mh, dmin(dmin(t1d1, t1d2), t1d3), tv, te, tn, tev, ten,
                                  tnv, tnve, a_zx, a_zy, a_xy);
            czx = czx && !(dead & 1u);
            czy = czy && !(dead & 2u);
            cxy = cxy && !(dead & 4u);
          }
          if (COEF) {
            if (czx) q_zx = ca.zxq();
            if (czy) q_zy = ca.zyq();
            if (cxy) q_xy = ca.xyq();
          } else {
            if (czx) q_zx = cc.zxq();
            if (czy) q_zy = cc.zyq();
            if (cxy) q_xy = cc.xyq();
          }
        }
      }
      {
        const unsigned m0 = __ballot_sync(0xffffffffu, czx);
        const unsigned m1 = __ballot_sync(0xffffffffu, czy);
        const unsigned m2 = __ballot_sync(0xffffffffu, cxy);
        const int b1 = __popc(m0), b2 = b1 + __popc(m1);
        if (czx) {
          const int q = __popc(m0 & lt_mask);
          sh.ju[warp][q] = tv; sh.jw[warp][q] = te; sh.jx[warp][q] = tev; sh.jq[warp][q] = q_zx;
          sh.jid[warp][q] = lane;
        }
        if (czy) {
          const int q = b1 + __popc(m1 & lt_mask);
          sh.ju[warp][q] = tv; sh.jw[warp][q] = tn; sh.jx[warp][q] = tnv; sh.jq[warp][q] = q_zy;
          sh.jid[warp][q] = 32 + lane;
        }
        if (cxy) {
          const int q = b2 + __popc(m2 & lt_mask);
          sh.ju[warp][q] = te; sh.jw[warp][q] = tn; sh.jx[warp][q] = ten; sh.jq[warp][q] = q_xy;
          sh.jid[warp][q] = 64 + lane;
        }
        if (lane == 0) sh.n2[warp] = b2 + __popc(m2);
      }
      __syncthreads();
      // ---- stage B: the queued plane operators, 32 jobs per warp instruction ----
      {
        int pre[kTeamWarps + 1];
        pre[0] = 0;
#pragma unroll
        for (int x = 0; x < kTeamWarps; ++x) pre[x + 1] = pre[x] + sh.n2[x];
        const int c3 = pre[kTeamWarps];
        for (int q = warp * 32 + lane; q - lane < c3; q += kTeamWarps * 32) {
          if (q < c3) {
            int w, l;
            team_job(pre, q, w, l);
            const int id = sh.jid[w][l];
            sh.r2[w][id >> 5][id & 31] =
                plane3(id >> 5, sh.ju[w][l], sh.jw[w][l], sh.jx[w][l], sh.jq[w][l], o);
          }
        }
      }
      __syncthreads();
      // ---- stage C: plane results, 3D guard, 3D jobs ----
      const double t2d1 = czx ? sh.r2[warp][0][lane] : kBig;
      const double t2d2 = czy ? sh.r2[warp][1][lane] : kBig;
      const double t2d3 = cxy ? sh.r2[warp][2][lane] : kBig;
      const bool g3 = go && !(dead & 8u) &&
                      dlt(dmax(dmax(tv, te), tn),
                          dmin(dmin(dmin(t1d1, t1d2), t1d3), dmin(dmin(t2d1, t2d2), t2d3)));
      {
        const unsigned m3 = __ballot_sync(0xffffffffu, g3);
        if (g3) {
          const int q = __popc(m3 & lt_mask);
          sh.kin[0][warp][q] = tv;
          sh.kin[1][warp][q] = te;
          sh.kin[2][warp][q] = tn;
          sh.kin[3][warp][q] = tev;
          sh.kin[4][warp][q] = ten;
          sh.kin[5][warp][q] = tnv;
          sh.kin[6][warp][q] = tnve;
          sh.kin[7][warp][q] = COEF ? ca.t3() : cc.t3();
          sh.kid[warp][q] = lane;
        }
        if (lane == 0) sh.n3[warp] = __popc(m3);
      }
      __syncthreads();
      // ---- stage D: 3D operators ----
      {
        int pre[kTeamWarps + 1];
        pre[0] = 0;
#pragma unroll
        for (int x = 0; x < kTeamWarps; ++x) pre[x + 1] = pre[x] + sh.n3[x];
        const int c3 = pre[kTeamWarps];
        for (int q = warp * 32 + lane; q - lane < c3; q += kTeamWarps * 32) {
          if (q < c3) {
            int w, l;
            team_job(pre, q, w, l);
            sh.r3[w][sh.kid[w][l]] =
                op3d(sh.kin[0][w][l], sh.kin[1][w][l], sh.kin[2][w][l], sh.kin[3][w][l],
                     sh.kin[4][w][l], sh.kin[5][w][l], sh.kin[6][w][l], sh.kin[7][w][l], o);
          }
        }
      }
      __syncthreads();
      // ---- stage E: minimum, branch record, write-back ----
      if (go) {
        const double t3d = g3 ? sh.r3[warp][lane] : kBig;
        uint8_t code = 0;
        res = finish3d<GRAD>(t0, t1d1, t1d2, t1d3, t2d1, t2d2, t2d3, t3d, sz, sx, sy, code);
        if (!deq(res, t0)) {
          tts[n] = res;
          if (GRAD) recs[n] = code;
          if (A.tape.code)
            tape_record(A.tape, A.status, (long long)src * A.nodes + n, e, code, t0);
        }
      }
      r3v = r2v;
      r2v = r1;
      r1 = res;
      if (active && (((unsigned)(s + 1) & cmask) == 0 || s + 1 == T)) {
        __syncwarp();
        if (lane == 0) {
          __threadfence();
          st_release(my_prog, base + (unsigned)(s + 1));
        }
      }
    }
    // Completion (also after an aborted wait, so that no other warp blocks).
    __syncwarp();
    if (src < A.nsrc && lane == 0) {
      __threadfence();
      st_release(my_prog, base + (unsigned)T);
    }
  }
}

// Fill every node with Big and every branch record with "no sign".
__global__ void fill3d_kernel(double* tt, uint8_t* rec, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    tt[q] = kBig;
    if (rec) rec[q] = 13;
  }
}

// Operator coefficients (see Coef3), one thread per node-shaped index.
// Also checks that min(slowness) * min(spacing) >= 1e-9: then a Big-valued
// neighbourhood provably stays Big (every operator exceeds Big by at least
// about slowness * spacing / 2, far above the rounding of Big), which makes
// the sweep's skip of such nodes exact; otherwise the skip is disabled.
__device__ __forceinline__ void coef3d_node(long long q, const double* slow, int nz, int nx,
                                            int ny, const Ops3& o, const Coef3& C, bool write,
                                            int* no_skip) {
  {
    const int NX = nx + 1, NY = ny + 1;
    const double hmin = fmin(o.dz, fmin(o.dx, o.dy));
    const int i = (int)(q / ((long long)NX * NY));
    const int j = (int)((q / NY) % NX);
    const int k = (int)(q % NY);
    const int im = imax(i - 1, 0), ip = imin(i, nz - 1);
    const int jm = imax(j - 1, 0), jp = imin(j, nx - 1);
    const int km = imax(k - 1, 0), kp = imin(k, ny - 1);
#define S(a, b, c) __ldg(slow + ((long long)(a)*nx + (b)) * ny + (c))
    double v;
    if (!write) {
      if (i < nz && j < nx && k < ny && !(S(i, j, k) * hmin >= 1e-9)) atomicOr(no_skip, 1);
      return;
    }
    if (i < nz) {
      v = pmin(pmin(S(i, jm, km), S(i, jm, kp)), pmin(S(i, jp, km), S(i, jp, kp)));
      C.z1[q] = o.dz * v;
    }
    if (j < nx) {
      v = pmin(pmin(S(im, j, km), S(ip, j, km)), pmin(S(im, j, kp), S(ip, j, kp)));
      C.x1[q] = o.dx * v;
    }
    if (k < ny) {
      v = pmin(pmin(S(im, jm, k), S(im, jp, k)), pmin(S(ip, jm, k), S(ip, jp, k)));
      C.y1[q] = o.dy * v;
    }
    if (i < nz && j < nx) {
      v = pmin(S(i, j, km), S(i, j, kp));
      C.zxa[q] = o.dx * v;
      C.zxb[q] = o.dz * v;
      C.zxq[q] = times4(v * v) * o.szx;
    }
    if (i < nz && k < ny) {
      v = pmin(S(i, jm, k), S(i, jp, k));
      C.zya[q] = o.dy * v;
      C.zyb[q] = o.dz * v;
      C.zyq[q] = times4(v * v) * o.szy;
    }
    if (j < nx && k < ny) {
      v = pmin(S(im, j, k), S(ip, j, k));
      C.xya[q] = o.dy * v;
      C.xyb[q] = o.dx * v;
      C.xyq[q] = times4(v * v) * o.sxy;
    }
    if (i < nz && j < nx && k < ny) {
      v = S(i, j, k);
      C.t3[q] = v * v * o.dsum * 9.0;
      if (!(v * hmin >= 1e-9)) atomicOr(no_skip, 1);
    }
#undef S
  }
}

__global__ void coef3d_kernel(const double* slow, int nz, int nx, int ny, Ops3 o, Coef3 C,
                              bool write, int* no_skip) {
  const long long n_nodes = (long long)(nz + 1) * (nx + 1) * (ny + 1);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n_nodes;
       q += (long long)gridDim.x * blockDim.x)
    coef3d_node(q, slow, nz, nx, ny, o, C, write, no_skip);
}

// The same for every model of a batch: blockIdx.y = model.
__global__ void coef3d_batch_kernel(const Model3* models, bool write) {
  const Model3& M = models[blockIdx.y];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < M.nodes;
       q += (long long)gridDim.x * blockDim.x)
    coef3d_node(q, M.slow, M.nz, M.nx, M.ny, M.o, M.C, write, (int*)M.no_skip);
}

// Source set-up, _fteik3d.py:409-456.
__device__ __forceinline__ Source3 init3d_source(const double* slow, const double* src, int nz,
                                                 int nx, int ny, const Ops3& o, double* t) {
  Source3 p;
  double zsa = src[0] / o.dz, xsa = src[1] / o.dx, ysa = src[2] / o.dy;
  zsa = zsa >= nz ? zsa - kEps : zsa;
  xsa = xsa >= nx ? xsa - kEps : xsa;
  ysa = ysa >= ny ? ysa - kEps : ysa;
  p.zsa = zsa;
  p.xsa = xsa;
  p.ysa = ysa;
  p.zsi = imin((int)zsa, nz - 1);
  p.xsi = imin((int)xsa, nx - 1);
  p.ysi = imin((int)ysa, ny - 1);
  p.pad = 0;
  p.vzero = slow[((long long)p.zsi * nx + p.xsi) * ny + p.ysi];
  const int NX = nx + 1, NY = ny + 1;
  for (int q = 0; q < 8; ++q) {
    const int i = p.zsi + (q & 1), j = p.xsi + ((q >> 1) & 1), k = p.ysi + ((q >> 2) & 1);
    double tzc, txc, tyc;
    t[((long long)i * NX + j) * NY + k] = t_anad3(i, j, k, o, p, tzc, txc, tyc);
  }
  return p;
}

// One thread per source.
__global__ void init3d_kernel(const double* slow, const double* src, int nsrc, int nz, int nx,
                              int ny, Ops3 o, double* tt, long long nodes, Source3* params,
                              double* vzero_out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsrc) return;
  const Source3 p = init3d_source(slow, src + 3 * s, nz, nx, ny, o, tt + (long long)s * nodes);
  params[s] = p;
  vzero_out[s] = p.vzero;
}

// One thread per job (model, source) of a batch.
__global__ void init3d_batch_kernel(const Model3* models, const Job3* jobs, int njobs,
                                    const double* src, Source3* params, double* vzero_out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= njobs) return;
  const Job3 jb = jobs[q];
  const Model3& M = models[jb.model];
  const Source3 p = init3d_source(M.slow, src + 3 * q, M.nz, M.nx, M.ny, M.o, jb.tt);
  params[q] = p;
  vzero_out[q] = p.vzero;
}

// The adjoint's tape keeps each source's set-up and the initial values of
// the 8 nodes around it (the values their first change replaces): one thread
// per node.
__global__ void tape_init_kernel(const double* tt, const Source3* params, int nsrc,
                                 long long nodes, int NX, int NY, Tape3 tape) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nsrc * 8) return;
  const int s = q >> 3, c = q & 7;
  const Source3 p = params[s];
  if (c == 0) tape.params[s] = p;
  const int i = p.zsi + (c & 1), j = p.xsi + ((c >> 1) & 1), k = p.ysi + ((c >> 2) & 1);
  tape.init8[q] = tt[(long long)s * nodes + ((long long)i * NX + j) * NY + k];
}

// Fill every node of every job with Big (and its record with "no sign"):
// blockIdx.y = job.
__global__ void fill3d_batch_kernel(const Model3* models, const Job3* jobs) {
  const Job3 jb = jobs[blockIdx.y];
  const long long n = models[jb.model].nodes;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    jb.tt[q] = kBig;
    if (jb.rec) jb.rec[q] = 13;
  }
}

// Gradient post-pass, _fteik3d.py:464-488, for node n = (i, j, k).  The 8
// nodes around the source start from the analytic derivatives they were
// initialised with (_fteik3d.py:453-456); every other node starts from zero.
// The reference's `sgn * (t - t_upwind)` with sgn = +-1 is the difference or
// its negation (the same bits), and `gn > 0` holds exactly when gn's bit
// pattern is positive and not NaN's (gn is a square root).
__device__ __forceinline__ void grad3d_node_at(const double* tt, const uint8_t* rec, long long n,
                                               int i, int j, int k, const Source3& p, int NX,
                                               int NY, const Ops3& o, double* g) {
  const long long NXY = (long long)NX * NY;
  double g0 = 0.0, g1 = 0.0, g2 = 0.0;
  if ((unsigned)(i - p.zsi) <= 1u && (unsigned)(j - p.xsi) <= 1u && (unsigned)(k - p.ysi) <= 1u)
    t_anad3(i, j, k, o, p, g0, g1, g2);
  const int code = rec[n];
  const int cz = code / 9 - 1, cx = (code / 3) % 3 - 1, cy = code % 3 - 1;
  const double tq = tt[n];
  if (cz != 0) {
    const double d = tq - tt[n - cz * NXY];
    g0 = div_by(dflip(d, cz < 0), o.rdz);
  }
  if (cx != 0) {
    const double d = tq - tt[n - (long long)cx * NY];
    g1 = div_by(dflip(d, cx < 0), o.rdx);
  }
  if (cy != 0) {
    const double d = tq - tt[n - cy];
    g2 = div_by(dflip(d, cy < 0), o.rdy);
  }
  const double gn = sqrt_rn(g0 * g0 + g1 * g1 + g2 * g2);
  const long long gb = __double_as_longlong(gn);
  if (gb > 0 && gb <= 0x7ff0000000000000LL) {
    // g /= gn, one correctly rounded quotient per component
    const SharedRecip rn = shared_recip(gn);
    g0 = div_shared(g0, rn);
    g1 = div_shared(g1, rn);
    g2 = div_shared(g2, rn);
  }
  g[3 * n] = g0;
  g[3 * n + 1] = g1;
  g[3 * n + 2] = g2;
}

// One thread per node (grid-stride).  The kernel is bound by its FP64 work
// (three constant divisions, a square root, a reciprocal and three
// corrected quotients per node); the index arithmetic runs beside it on the
// integer pipe.
__device__ __forceinline__ void grad3d_node(const double* tt, const uint8_t* rec, long long n,
                                            const Source3& p, int NX, int NY, const Ops3& o,
                                            double* g) {
  const long long NXY = (long long)NX * NY;
  const int i = (int)(n / NXY);
  const int j = (int)((n - (long long)i * NXY) / NY);
  const int k = (int)(n - (long long)i * NXY - (long long)j * NY);
  grad3d_node_at(tt, rec, n, i, j, k, p, NX, NY, o, g);
}

__global__ void grad3d_kernel(const double* tt, const uint8_t* rec, const Source3* params,
                              int nsrc, int NZ, int NX, int NY, Ops3 o, double* ttgrad) {
  const long long nodes = (long long)NZ * NX * NY;
  const long long total = nodes * nsrc;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(q / nodes);
    const long long off = (long long)s * nodes;
    grad3d_node(tt + off, rec + off, q - off, params[s], NX, NY, o, ttgrad + 3 * off);
  }
}

// Gradients of every job of a batch: blockIdx.y = job; grads[job] is where
// that source's [nodes][3] gradients go.
__global__ void grad3d_batch_kernel(const Model3* models, const Job3* jobs,
                                    const Source3* params, double* const* grads) {
  const Job3 jb = jobs[blockIdx.y];
  const Model3& M = models[jb.model];
  const Source3 p = params[blockIdx.y];
  double* g = grads[blockIdx.y];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < M.nodes;
       q += (long long)gridDim.x * blockDim.x)
    grad3d_node(jb.tt, jb.rec, q, p, M.NX, M.NY, M.o, g);
}

// Work order of the pencils inside one sweep: by diagonal JL + KL (in the
// sweep's own upwind-first coordinates), so every dependency of an item has a
// smaller ticket.  Entry = JL << 16 | KL.
__global__ void pencil_order_kernel(int PJ, int PK, int* order) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= PJ * PK) return;
  const int JL = q / PK, KL = q % PK;
  const int d = JL + KL;
  int before = 0;
  for (int dd = 0; dd < d; ++dd) before += imin(dd, PJ - 1) - imax(0, dd - PK + 1) + 1;
  order[before + JL - imax(0, d - PK + 1)] = (JL << 16) | KL;
}

// ---------------------------------------------------------------- host side --

// Launch shape of the sweep kernel: pencil width (2, 4, 8), steps between
// progress publications (power of 2), coefficient source (1 arrays, 0 cells),
// and whether blocks of kTeamWarps sources step together with compacted
// operators (the team kernel; single-model solves of 4+ sources).
struct Tune3 {
  int pencil, chunk, coef, team;
};

static const void* team_kernel(int grad, bool coef, int pencil) {
#define FTEIK_T(G, C, P) (const void*)sweep3d_team_kernel<G, C, P>
#define FTEIK_TP(G, C) \
  (pencil == 2 ? FTEIK_T(G, C, 2) : pencil == 8 ? FTEIK_T(G, C, 8) : FTEIK_T(G, C, 4))
  if (grad != 0) return coef ? FTEIK_TP(true, true) : FTEIK_TP(true, false);
  return coef ? FTEIK_TP(false, true) : FTEIK_TP(false, false);
#undef FTEIK_TP
#undef FTEIK_T
}

static const void* sweep_kernel(int grad, bool coef, int pencil, bool multi) {
#define FTEIK_K(G, C, P, M) (const void*)sweep3d_kernel<G, C, P, M>
#define FTEIK_KP(G, C, M) \
  (pencil == 2 ? FTEIK_K(G, C, 2, M) : pencil == 8 ? FTEIK_K(G, C, 8, M) : FTEIK_K(G, C, 4, M))
  const bool g = grad != 0;  // 1: gradients, 2: branch record for the tape
  if (multi) {
    if (g) return coef ? FTEIK_KP(true, true, true) : FTEIK_KP(true, false, true);
    return coef ? FTEIK_KP(false, true, true) : FTEIK_KP(false, false, true);
  }
  if (g) return coef ? FTEIK_KP(true, true, false) : FTEIK_KP(true, false, false);
  return coef ? FTEIK_KP(false, true, false) : FTEIK_KP(false, false, false);
#undef FTEIK_KP
#undef FTEIK_K
}

// Launch shapes measured by the autotuner, per problem signature.
static std::mutex g_tune_mu;
static std::map<std::vector<long long>, Tune3> g_tuned;

static bool tuned_lookup(const std::vector<long long>& key, Tune3* t) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tuned.find(key);
  if (it == g_tuned.end()) return false;
  *t = it->second;
  return true;
}

static void tuned_store(const std::vector<long long>& key, const Tune3& t) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned[key] = t;
}

// Default shape for `jobs` (model, source) pairs in flight, of which
// `coef_sources` share one model's coefficients, with `items` (source,
// pencil) work items per sweep (0: not a single-model solve).  Measured on
// GB300 (sweep kernel, nsweep 2):
//  * 1-2 sources are bound by the latency of the pencil wavefront;
//    publishing progress every step (chunk 1) lets downwind pencils start
//    soonest (17% faster than chunk 4 on 128x256x256);
//  * up to ~100K items per sweep one warp per pencil wins (64 sources on
//    96x128x128: 182 ms against 193 ms for the team kernel);
//  * above that the team kernel wins (64 sources on 128x256x256: 989 against
//    1067 ms), and from ~400K items it is best publishing every 16 steps
//    (256 sources: 3734 ms against 3815 ms at chunk 4 and 4120 ms one warp
//    per pencil).
static Tune3 default_tune(int jobs, int coef_sources, long long items = 0) {
  const int team = items >= 100000 ? 1 : 0;
  const int chunk = jobs <= 2 ? 1 : jobs <= 8 ? 2 : (team && items >= 400000) ? 16 : kDefaultChunk;
  return Tune3{kDefaultPencil, chunk, coef_sources >= kCoefMinSources ? 1 : 0, team};
}

// The shape a solve runs with: explicit options first, then a shape the
// autotuner measured for this signature, then the defaults.
static Tune3 resolve_tune(const std::vector<long long>& key, int jobs, int coef_sources,
                          long long items = 0) {
  Tune3 t = default_tune(jobs, coef_sources, items);
  Tune3 m;
  if (tuned_lookup(key, &m)) t = m;
  const long long op = option_value(kOptSweepPencil), oc = option_value(kOptSweepChunk),
                  of = option_value(kOptSweepCoef);
  const long long ot = option_value(kOptSweepTeam);
  if (op > 0) t.pencil = (int)op;
  if (oc > 0) t.chunk = (int)oc;
  if (of >= 0) t.coef = (int)of;
  if (ot >= 0) t.team = (int)ot;
  return t;
}

static std::vector<long long> single_key(int nz, int nx, int ny, int nsrc, int grad) {
  return {0, nz, nx, ny, nsrc, grad == 1};
}

// Persistent launch of the sweep kernel over `items` work items.
static int launch_sweep(const void* kern, const Sweep3Args& A, long long items, cudaStream_t st) {
  int blocks = resident_blocks(kern, kWarpsPerBlock * 32);
  const long long need = (items + kWarpsPerBlock - 1) / kWarpsPerBlock;
  if (need < blocks) blocks = (int)need;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  timing_events(&ev0, &ev1);
  if (ev0) FTEIK_CHECK(cudaEventRecord(ev0, st));
  void* args[] = {(void*)&A};
  FTEIK_CHECK(cudaLaunchKernel(kern, dim3(blocks), dim3(kWarpsPerBlock * 32), args, 0, st));
  if (ev1) FTEIK_CHECK(cudaEventRecord(ev1, st));
  return kOk;
}

// The unchanged-node test (keeps_t0) holds for equal spacings; the option
// "sweep_keep_test" = 0 turns it off.
static int keep_test_enabled(double dz, double dx, double dy) {
  return dz == dx && dx == dy && option_value(kOptKeepTest) != 0 ? 1 : 0;
}

// Name of the sweep kernel the last 3D solve launched (measurement reports).
static const char* g_last_sweep_kernel = "none";

// Persistent launch of the team kernel: one block per item in flight.
static int launch_team(const void* kern, const Sweep3Args& A, long long items, cudaStream_t st) {
  int blocks = resident_blocks(kern, kTeamWarps * 32);
  if (items < blocks) blocks = (int)items;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  timing_events(&ev0, &ev1);
  if (ev0) FTEIK_CHECK(cudaEventRecord(ev0, st));
  void* args[] = {(void*)&A};
  FTEIK_CHECK(cudaLaunchKernel(kern, dim3(blocks), dim3(kTeamWarps * 32), args, 0, st));
  if (ev1) FTEIK_CHECK(cudaEventRecord(ev1, st));
  return kOk;
}

static void sweep_args_defaults(Sweep3Args& A) {
  std::memset((void*)&A, 0, sizeof(A));
}

}  // namespace fteik

using namespace fteik;

extern "C" size_t fteik3d_workspace_bytes(int nz, int nx, int ny, int nsrc, int grad) {
  if (nz < 1 || nx < 1 || ny < 1 || nsrc < 1) return 0;
  return layout3(nz, nx, ny, nsrc, grad).total;
}

static int solve3d_impl(const double* slow, int nz, int nx, int ny, double dz, double dx,
                        double dy, const double* sources, int nsrc, int nsweep, int grad,
                        double* tt, double* ttgrad, double* vzero, void* workspace,
                        size_t workspace_bytes, const Tape3* tape, long long spin_limit,
                        void* stream, const Tune3* force = nullptr) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nz < 2 || nx < 2 || ny < 2 || nsrc < 1 || nsweep < 0 || !slow || !sources || !tt ||
      !vzero || !workspace || grad < 0 || grad > 2 || (grad == 1 && !ttgrad))
    return kInvalidArgument;
  if (!(dz > 1e-100 && dz < 1e100 && dx > 1e-100 && dx < 1e100 && dy > 1e-100 && dy < 1e100))
    return kInvalidArgument;
  const Layout3 L = layout3(nz, nx, ny, nsrc, grad);
  if (workspace_bytes < L.total) return kWorkspaceTooSmall;
  // Source bounds, _fteik3d.py:403-407.
  for (int s = 0; s < nsrc; ++s) {
    const double z = sources[3 * s], x = sources[3 * s + 1], y = sources[3 * s + 2];
    const bool ok = (0.0 <= z && z <= dz * nz) && (0.0 <= x && x <= dx * nx) &&
                    (0.0 <= y && y <= dy * ny);
    if (!ok) return kSourceOutOfBound;
  }
  const long long items_default =
      (long long)nsrc * pencils_of(nx + 1, ny + 1, kDefaultPencil);
  const Tune3 tune = force ? *force
                           : resolve_tune(single_key(nz, nx, ny, nsrc, grad), nsrc, nsrc,
                                          items_default);
  const int pw = tune.pencil, pk = 32 / pw;
  const int NZ = nz + 1, NX = nx + 1, NY = ny + 1;
  const int PJ = (NX + pw - 1) / pw, PK = (NY + pk - 1) / pk;
  const long long nodes = (long long)NZ * NX * NY;
  const int T = NZ + pw + pk - 2;
  const unsigned long long stride = (unsigned long long)T + 1;
  const unsigned long long nepochs = 8ull * nsweep;
  if (nepochs * stride >= (1ull << 31) || nepochs * PJ * PK * (unsigned long long)nsrc >= (1ull << 31) ||
      PJ >= (1 << 15) || PK >= (1 << 16))
    return kInvalidArgument;
  // the sweep kernels index a model's nodes with 32-bit integers
  if (nodes >= (1LL << 31)) {
    set_last_error("a 3D model may hold at most 2^31 - 1 nodes ((nz+1)(nx+1)(ny+1) = %lld)", nodes);
    return kInvalidArgument;
  }

  char* ws = (char*)workspace;
  const Ops3 o = make_ops3(dz, dx, dy);
  Source3* params = (Source3*)(ws + L.params);
  double* src_dev = (double*)(ws + L.src);
  int* order = (int*)(ws + L.order);
  unsigned* progress = (unsigned*)(ws + L.progress);
  uint8_t* rec = grad ? (uint8_t*)(ws + L.rec) : nullptr;
  int* status = (int*)(ws + L.status);
  unsigned* ticket = (unsigned*)(ws + L.status + 4);
  int* no_skip = (int*)(ws + L.status + 8);
  Coef3 C;
  {
    double* c = (double*)(ws + L.coef);
    double** fields[kNumCoef] = {&C.z1,  &C.x1,  &C.y1,  &C.zxa, &C.zxb, &C.zxq, &C.zya,
                                 &C.zyb, &C.zyq, &C.xya, &C.xyb, &C.xyq, &C.t3};
    for (int f = 0; f < kNumCoef; ++f) *fields[f] = c + (size_t)f * nodes;
  }

  FTEIK_CHECK(cudaMemsetAsync(ws + L.status, 0, 16, st));
  FTEIK_CHECK(cudaMemsetAsync(progress, 0, sizeof(unsigned) * (size_t)PJ * PK * nsrc, st));
  FTEIK_CHECK(cudaMemcpyAsync(src_dev, sources, sizeof(double) * 3 * (size_t)nsrc,
                              cudaMemcpyHostToDevice, st));
  pencil_order_kernel<<<(PJ * PK + 127) / 128, 128, 0, st>>>(PJ, PK, order);
  // Coefficient arrays pay off when enough sources share them (they stay in
  // L2 across the sources of a pencil); a few sources read the slowness cells.
  const bool use_coef = tune.coef != 0;
  coef3d_kernel<<<grid_for(nodes, 256), 256, 0, st>>>(slow, nz, nx, ny, o, C, use_coef, no_skip);
  const long long ntot = nodes * nsrc;
  fill3d_kernel<<<grid_for(ntot, 256), 256, 0, st>>>(tt, rec, ntot);
  init3d_kernel<<<(nsrc + 63) / 64, 64, 0, st>>>(slow, src_dev, nsrc, nz, nx, ny, o, tt, nodes,
                                                 params, vzero);
  if (tape)
    tape_init_kernel<<<(nsrc * 8 + 127) / 128, 128, 0, st>>>(tt, params, nsrc, nodes, NX, NY,
                                                             *tape);
  FTEIK_CHECK(cudaGetLastError());
  if (nsweep > 0) {
    Sweep3Args A;
    sweep_args_defaults(A);
    A.tt = tt;
    A.rec = rec;
    A.C = C;
    A.slow = slow;
    A.no_skip = no_skip;
    if (tape) A.tape = *tape;
    A.progress = progress;
    A.ticket = ticket;
    A.status = status;
    A.order = order;
    A.nz = nz;
    A.nx = nx;
    A.ny = ny;
    A.NZ = NZ;
    A.NX = NX;
    A.NY = NY;
    A.nodes = nodes;
    A.nsrc = nsrc;
    A.nepochs = (int)nepochs;
    A.npencils = PJ * PK;
    A.PJ = PJ;
    A.PK = PK;
    A.total_steps = T;
    A.stride = (unsigned)stride;
    A.chunk = tune.chunk;
    A.spin_limit = spin_limit > 0 ? spin_limit : (1LL << 25);
    A.keep_test = keep_test_enabled(dz, dx, dy);
    A.o = o;
    int rc;
    if (tune.team) {
      A.ngroups = (nsrc + kTeamWarps - 1) / kTeamWarps;
      g_last_sweep_kernel = "sweep3d_team_kernel";
      rc = launch_team(team_kernel(grad, use_coef, pw), A,
                       (long long)nepochs * PJ * PK * A.ngroups, st);
    } else {
      g_last_sweep_kernel = "sweep3d_kernel";
      rc = launch_sweep(sweep_kernel(grad, use_coef, pw, false), A,
                        (long long)nepochs * PJ * PK * nsrc, st);
    }
    if (rc != kOk) return rc;
  }
  if (grad == 1) {
    grad3d_kernel<<<grid_for(ntot, 256), 256, 0, st>>>(tt, rec, params, nsrc, NZ, NX, NY, o,
                                                       ttgrad);
    FTEIK_CHECK(cudaGetLastError());
  }
  return kOk;
}

extern "C" int fteik3d_solve_async(const double* slow, int nz, int nx, int ny, double dz,
                                   double dx, double dy, const double* sources, int nsrc,
                                   int nsweep, int grad, double* tt, double* ttgrad,
                                   double* vzero, void* workspace, size_t workspace_bytes,
                                   long long spin_limit, void* stream) {
  return solve3d_impl(slow, nz, nx, ny, dz, dx, dy, sources, nsrc, nsweep, grad, tt, ttgrad,
                      vzero, workspace, workspace_bytes, nullptr, spin_limit, stream);
}

extern "C" size_t fteik3d_tape_bytes(int nz, int nx, int ny, int nsrc, int nsweep,
                                     int history) {
  if (nz < 1 || nx < 1 || ny < 1 || nsrc < 1 || nsweep < 0 || 8 * nsweep > kTapeMaxEpochs ||
      history < 0 || (nsweep > 0 && history > 8 * nsweep - 1) || (nsweep == 0 && history != 0))
    return 0;
  return tape_layout(nz, nx, ny, nsrc, nsweep, history).total;
}

extern "C" int fteik3d_solve_tape(const double* slow, int nz, int nx, int ny, double dz,
                                  double dx, double dy, const double* sources, int nsrc,
                                  int nsweep, double* tt, double* vzero, void* workspace,
                                  size_t workspace_bytes, int history, void* tape,
                                  size_t tape_bytes, long long spin_limit, void* stream) {
  const size_t need = fteik3d_tape_bytes(nz, nx, ny, nsrc, nsweep, history);
  if (!tape || need == 0) return kInvalidArgument;
  if (tape_bytes < need) return kWorkspaceTooSmall;
  const TapeLayout L = tape_layout(nz, nx, ny, nsrc, nsweep, history);
  const Tape3 T = tape_at(tape, L, nsweep, history);
  cudaStream_t st = (cudaStream_t)stream;
  // code 255 marks "unchanged in this sweep"; key 0 marks an empty table slot
  if (L.hist > L.code) FTEIK_CHECK(cudaMemsetAsync(T.code, 0xff, L.hist - L.code, st));
  FTEIK_CHECK(cudaMemsetAsync(T.key, 0, L.val - L.key, st));
  int rc = solve3d_impl(slow, nz, nx, ny, dz, dx, dy, sources, nsrc, nsweep, 2, tt, nullptr,
                        vzero, workspace, workspace_bytes, &T, spin_limit, stream);
  if (rc != kOk) return rc;
  return fteik_workspace_status(workspace, stream);
}

extern "C" int fteik3d_solve(const double* slow, int nz, int nx, int ny, double dz, double dx,
                             double dy, const double* sources, int nsrc, int nsweep, int grad,
                             double* tt, double* ttgrad, double* vzero, void* workspace,
                             size_t workspace_bytes, long long spin_limit, void* stream) {
  int rc = fteik3d_solve_async(slow, nz, nx, ny, dz, dx, dy, sources, nsrc, nsweep, grad, tt,
                               ttgrad, vzero, workspace, workspace_bytes, spin_limit, stream);
  if (rc != kOk) return rc;
  return fteik_workspace_status(workspace, stream);
}

// ------------------------------------------------------------ batch of models --

namespace {

struct Batch3Layout {
  size_t status, models, jobs, items, params, src, grads, progress, noskip, coef, rec, total;
  long long njobs, items_max, progress_len, coef_nodes, rec_nodes;
};

Batch3Layout batch_layout(int nmodel, const int* dims, const int* nsrc, int grad) {
  Batch3Layout L{};
  L.njobs = 0;
  L.items_max = 0;
  L.progress_len = 0;
  L.coef_nodes = 0;
  L.rec_nodes = 0;
  for (int m = 0; m < nmodel; ++m) {
    const long long NZ = dims[3 * m] + 1, NX = dims[3 * m + 1] + 1, NY = dims[3 * m + 2] + 1;
    const long long np = max_pencils((int)NX, (int)NY);
    L.njobs += nsrc[m];
    L.items_max += np * nsrc[m];
    L.progress_len += np * nsrc[m];
    L.coef_nodes += NZ * NX * NY;
    L.rec_nodes += NZ * NX * NY * nsrc[m];
  }
  size_t off = 0;
  L.status = off;
  off = align_up(off + 16);
  L.models = off;
  off = align_up(off + sizeof(Model3) * (size_t)nmodel);
  L.jobs = off;
  off = align_up(off + sizeof(Job3) * (size_t)L.njobs);
  L.items = off;
  off = align_up(off + sizeof(int2) * (size_t)L.items_max);
  L.params = off;
  off = align_up(off + sizeof(Source3) * (size_t)L.njobs);
  L.src = off;
  off = align_up(off + sizeof(double) * 3 * (size_t)L.njobs);
  L.grads = off;
  off = align_up(off + sizeof(double*) * (size_t)L.njobs);
  L.progress = off;
  off = align_up(off + sizeof(unsigned) * (size_t)L.progress_len);
  L.noskip = off;
  off = align_up(off + sizeof(int) * (size_t)nmodel);
  L.coef = off;
  off = align_up(off + sizeof(double) * kNumCoef * (size_t)L.coef_nodes);
  L.rec = off;
  if (grad) off = align_up(off + (size_t)L.rec_nodes);
  L.total = off;
  return L;
}

std::vector<long long> batch_key(int nmodel, const int* dims, const int* nsrc, int grad) {
  std::vector<long long> k{1, nmodel, grad == 1};
  for (int m = 0; m < nmodel; ++m) {
    k.push_back(dims[3 * m]);
    k.push_back(dims[3 * m + 1]);
    k.push_back(dims[3 * m + 2]);
    k.push_back(nsrc[m]);
  }
  return k;
}

}  // namespace

extern "C" size_t fteik3d_batch_workspace_bytes(int nmodel, const int* dims, const int* nsrc,
                                                int grad) {
  if (nmodel < 1 || !dims || !nsrc) return 0;
  for (int m = 0; m < nmodel; ++m)
    if (dims[3 * m] < 1 || dims[3 * m + 1] < 1 || dims[3 * m + 2] < 1 || nsrc[m] < 1) return 0;
  return batch_layout(nmodel, dims, nsrc, grad ? 1 : 0).total;
}

static int solve_batch_impl(int nmodel, const double* const* slow, const int* dims,
                            const double* spacing, const double* sources, const int* nsrc,
                            int nsweep, int grad, double* const* tt, double* const* ttgrad,
                            double* vzero, void* workspace, size_t workspace_bytes,
                            long long spin_limit, void* stream, const Tune3* force) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nmodel < 1 || !slow || !dims || !spacing || !sources || !nsrc || nsweep < 0 || !tt ||
      !vzero || !workspace || grad < 0 || grad > 1 || (grad == 1 && !ttgrad))
    return kInvalidArgument;
  long long total_src = 0;
  for (int m = 0; m < nmodel; ++m) {
    const double dz = spacing[3 * m], dx = spacing[3 * m + 1], dy = spacing[3 * m + 2];
    if (dims[3 * m] < 2 || dims[3 * m + 1] < 2 || dims[3 * m + 2] < 2 || nsrc[m] < 1 ||
        !slow[m] || !tt[m] || (grad == 1 && !ttgrad[m]))
      return kInvalidArgument;
    if (!(dz > 1e-100 && dz < 1e100 && dx > 1e-100 && dx < 1e100 && dy > 1e-100 && dy < 1e100))
      return kInvalidArgument;
    for (int s = 0; s < nsrc[m]; ++s) {
      const double* p = sources + 3 * (total_src + s);
      const bool ok = (0.0 <= p[0] && p[0] <= dz * dims[3 * m]) &&
                      (0.0 <= p[1] && p[1] <= dx * dims[3 * m + 1]) &&
                      (0.0 <= p[2] && p[2] <= dy * dims[3 * m + 2]);
      if (!ok) return kSourceOutOfBound;
    }
    total_src += nsrc[m];
  }
  const Batch3Layout L = batch_layout(nmodel, dims, nsrc, grad);
  if (workspace_bytes < L.total) return kWorkspaceTooSmall;
  const Tune3 tune = force ? *force
                          : resolve_tune(batch_key(nmodel, dims, nsrc, grad), (int)total_src,
                                         (int)(total_src / nmodel));
  const int pw = tune.pencil, pk = 32 / pw;
  char* ws = (char*)workspace;

  // Host tables: models, jobs, and one sweep's work items ordered by pencil
  // diagonal, then job, so that every model's wavefront advances together
  // and every dependency of an item has a smaller ticket.
  std::vector<Model3> models(nmodel);
  std::vector<Job3> jobs((size_t)L.njobs);
  std::vector<double*> grads((size_t)L.njobs, nullptr);
  double* coef = (double*)(ws + L.coef);
  uint8_t* rec = grad ? (uint8_t*)(ws + L.rec) : nullptr;
  unsigned* progress = (unsigned*)(ws + L.progress);
  int* noskip = (int*)(ws + L.noskip);
  long long epochs_steps_max = 0;
  int max_diag = 0;
  {
    long long job = 0, poff = 0;
    for (int m = 0; m < nmodel; ++m) {
      Model3& M = models[m];
      std::memset((void*)&M, 0, sizeof(M));
      M.nz = dims[3 * m];
      M.nx = dims[3 * m + 1];
      M.ny = dims[3 * m + 2];
      M.NZ = M.nz + 1;
      M.NX = M.nx + 1;
      M.NY = M.ny + 1;
      M.nodes = (long long)M.NZ * M.NX * M.NY;
      M.o = make_ops3(spacing[3 * m], spacing[3 * m + 1], spacing[3 * m + 2]);
      M.slow = slow[m];
      M.no_skip = noskip + m;
      M.keep_test = keep_test_enabled(spacing[3 * m], spacing[3 * m + 1], spacing[3 * m + 2]);
      M.PJ = (M.NX + pw - 1) / pw;
      M.PK = (M.NY + pk - 1) / pk;
      M.T = M.NZ + pw + pk - 2;
      M.stride = (unsigned)M.T + 1;
      double** fields[kNumCoef] = {&M.C.z1,  &M.C.x1,  &M.C.y1,  &M.C.zxa, &M.C.zxb,
                                   &M.C.zxq, &M.C.zya, &M.C.zyb, &M.C.zyq, &M.C.xya,
                                   &M.C.xyb, &M.C.xyq, &M.C.t3};
      for (int f = 0; f < kNumCoef; ++f) *fields[f] = coef + (size_t)f * M.nodes;
      coef += (size_t)kNumCoef * M.nodes;
      epochs_steps_max = std::max(epochs_steps_max, (long long)M.stride);
      max_diag = std::max(max_diag, M.PJ + M.PK - 1);
      if (M.PJ >= (1 << 15) || M.PK >= (1 << 16) || M.nodes >= (1LL << 31)) return kInvalidArgument;
      for (int s = 0; s < nsrc[m]; ++s, ++job) {
        Job3& J = jobs[(size_t)job];
        J.model = m;
        J.pad = 0;
        J.tt = tt[m] + (size_t)s * M.nodes;
        J.rec = rec;
        if (rec) rec += M.nodes;
        J.prog = progress + poff;
        poff += (long long)M.PJ * M.PK;
        if (grad == 1) grads[(size_t)job] = ttgrad[m] + (size_t)3 * s * M.nodes;
      }
    }
  }
  std::vector<int2> items;
  items.reserve((size_t)L.items_max);
  for (int d = 0; d < max_diag; ++d)
    for (long long q = 0; q < L.njobs; ++q) {
      const Model3& M = models[jobs[(size_t)q].model];
      for (int JL = std::max(0, d - M.PK + 1); JL <= std::min(d, M.PJ - 1); ++JL)
        items.push_back(make_int2((int)q, (JL << 16) | (d - JL)));
    }
  const unsigned long long nepochs = 8ull * nsweep;
  if (nepochs * epochs_steps_max >= (1ull << 31) || nepochs * items.size() >= (1ull << 31))
    return kInvalidArgument;

  Model3* d_models = (Model3*)(ws + L.models);
  Job3* d_jobs = (Job3*)(ws + L.jobs);
  int2* d_items = (int2*)(ws + L.items);
  Source3* params = (Source3*)(ws + L.params);
  double* src_dev = (double*)(ws + L.src);
  double** d_grads = (double**)(ws + L.grads);
  FTEIK_CHECK(cudaMemsetAsync(ws + L.status, 0, 16, st));
  FTEIK_CHECK(cudaMemsetAsync(noskip, 0, sizeof(int) * (size_t)nmodel, st));
  FTEIK_CHECK(cudaMemsetAsync(progress, 0, sizeof(unsigned) * (size_t)L.progress_len, st));
  FTEIK_CHECK(cudaMemcpyAsync(d_models, models.data(), sizeof(Model3) * models.size(),
                              cudaMemcpyHostToDevice, st));
  FTEIK_CHECK(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(Job3) * jobs.size(),
                              cudaMemcpyHostToDevice, st));
  FTEIK_CHECK(cudaMemcpyAsync(d_items, items.data(), sizeof(int2) * items.size(),
                              cudaMemcpyHostToDevice, st));
  FTEIK_CHECK(cudaMemcpyAsync(src_dev, sources, sizeof(double) * 3 * (size_t)L.njobs,
                              cudaMemcpyHostToDevice, st));
  if (grad == 1)
    FTEIK_CHECK(cudaMemcpyAsync(d_grads, grads.data(), sizeof(double*) * grads.size(),
                                cudaMemcpyHostToDevice, st));
  // The pageable copies above return once the host tables are staged; wait
  // for them before the vectors go out of scope.
  FTEIK_CHECK(cudaStreamSynchronize(st));
  const bool use_coef = tune.coef != 0;
  long long max_nodes = 0;
  for (const Model3& M : models) max_nodes = std::max(max_nodes, M.nodes);
  const int bx = std::max(1, std::min(grid_for(max_nodes, 256), 4096));
  coef3d_batch_kernel<<<dim3(bx, nmodel), 256, 0, st>>>(d_models, use_coef);
  fill3d_batch_kernel<<<dim3(bx, (unsigned)L.njobs), 256, 0, st>>>(d_models, d_jobs);
  init3d_batch_kernel<<<(unsigned)((L.njobs + 63) / 64), 64, 0, st>>>(
      d_models, d_jobs, (int)L.njobs, src_dev, params, vzero);
  FTEIK_CHECK(cudaGetLastError());
  if (nsweep > 0) {
    Sweep3Args A;
    sweep_args_defaults(A);
    A.models = d_models;
    A.jobs = d_jobs;
    A.items = d_items;
    A.items_per_epoch = (unsigned)items.size();
    A.ticket = (unsigned*)(ws + L.status + 4);
    A.status = (int*)(ws + L.status);
    A.nepochs = (int)nepochs;
    A.chunk = tune.chunk;
    A.spin_limit = spin_limit > 0 ? spin_limit : (1LL << 25);
    g_last_sweep_kernel = "sweep3d_kernel (models)";
    const int rc = launch_sweep(sweep_kernel(grad, use_coef, pw, true), A,
                                (long long)nepochs * (long long)items.size(), st);
    if (rc != kOk) return rc;
  }
  if (grad == 1) {
    grad3d_batch_kernel<<<dim3(bx, (unsigned)L.njobs), 256, 0, st>>>(d_models, d_jobs, params,
                                                                     d_grads);
    FTEIK_CHECK(cudaGetLastError());
  }
  return fteik_workspace_status(workspace, stream);
}

extern "C" int fteik3d_solve_batch(int nmodel, const double* const* slow, const int* dims,
                                   const double* spacing, const double* sources, const int* nsrc,
                                   int nsweep, int grad, double* const* tt,
                                   double* const* ttgrad, double* vzero, void* workspace,
                                   size_t workspace_bytes, long long spin_limit, void* stream) {
  return solve_batch_impl(nmodel, slow, dims, spacing, sources, nsrc, nsweep, grad, tt, ttgrad,
                          vzero, workspace, workspace_bytes, spin_limit, stream, nullptr);
}

// ------------------------------------------------------------------ autotuner --

namespace {

// Coordinate search over the launch shape: chunk, then pencil width, then
// coefficient source, each timed (sweep kernel only, CUDA events on the
// stream) with one sweep per direction, the best of `reps` runs.
template <class Run>
int tune_search(Run run, int jobs, int coef_sources, long long items, int reps, bool allow_team,
                Tune3* best, float* best_ms) {
  Tune3 cur = default_tune(jobs, coef_sources, items);
  if (!allow_team) cur.team = 0;
  float cur_ms = 0.f;
  auto time_of = [&](const Tune3& t, float* ms) -> int {
    float b = 3.4e38f;
    for (int r = 0; r < reps; ++r) {
      float x = 0.f;
      const int rc = run(t, &x);
      if (rc != kOk) return rc;
      b = std::min(b, x);
    }
    *ms = b;
    return kOk;
  };
  int rc = run(cur, &cur_ms);  // warm-up (first-touch, module load)
  if (rc != kOk) return rc;
  rc = time_of(cur, &cur_ms);
  if (rc != kOk) return rc;
  const int chunks[] = {1, 2, 4, 8, 16, 32};
  const int pencils[] = {2, 4, 8};
  for (int pass = 0; pass < 4; ++pass) {
    Tune3 base = cur;
    const int n = pass == 0 ? 2 : pass == 1 ? 6 : pass == 2 ? 3 : 2;
    if (pass == 0 && !allow_team) continue;
    for (int q = 0; q < n; ++q) {
      Tune3 t = base;
      if (pass == 0) t.team = q;
      if (pass == 1) t.chunk = chunks[q];
      if (pass == 2) t.pencil = pencils[q];
      if (pass == 3) t.coef = q;
      if (t.chunk == cur.chunk && t.pencil == cur.pencil && t.coef == cur.coef &&
          t.team == cur.team)
        continue;
      float ms = 0.f;
      rc = time_of(t, &ms);
      if (rc != kOk) return rc;
      if (ms < cur_ms) {
        cur = t;
        cur_ms = ms;
      }
    }
  }
  *best = cur;
  *best_ms = cur_ms;
  return kOk;
}

// Times one call of `solve` (a launch that records the timing events).
template <class Solve>
int timed(Solve solve, float* ms) {
  int rc = fteik_kernel_timing(1);
  if (rc != kOk) return rc;
  rc = solve();
  if (rc != kOk) return rc;
  return fteik_last_sweep_ms(ms);
}

}  // namespace

extern "C" int fteik3d_autotune(const double* slow, int nz, int nx, int ny, double dz, double dx,
                                double dy, const double* sources, int nsrc, int grad, double* tt,
                                double* ttgrad, double* vzero, void* workspace,
                                size_t workspace_bytes, long long spin_limit, int* shape,
                                float* best_ms, void* stream) {
  if (grad < 0 || grad > 1) return kInvalidArgument;
  auto run = [&](const Tune3& t, float* ms) {
    return timed(
        [&]() {
          int rc = solve3d_impl(slow, nz, nx, ny, dz, dx, dy, sources, nsrc, 1, grad, tt, ttgrad,
                                vzero, workspace, workspace_bytes, nullptr, spin_limit, stream,
                                &t);
          if (rc != kOk) return rc;
          return fteik_workspace_status(workspace, stream);
        },
        ms);
  };
  Tune3 best;
  float ms = 0.f;
  const bool timing_was_on = kernel_timing_on();
  const int rc = tune_search(run, nsrc, nsrc,
                             (long long)nsrc * pencils_of(nx + 1, ny + 1, kDefaultPencil), 2,
                             true, &best, &ms);
  fteik_kernel_timing(timing_was_on ? 1 : 0);
  if (rc != kOk) return rc;
  tuned_store(single_key(nz, nx, ny, nsrc, grad), best);
  if (shape) {
    shape[0] = best.pencil;
    shape[1] = best.chunk;
    shape[2] = best.coef;
    shape[3] = best.team;
  }
  if (best_ms) *best_ms = ms;
  return kOk;
}

extern "C" int fteik3d_batch_autotune(int nmodel, const double* const* slow, const int* dims,
                                      const double* spacing, const double* sources,
                                      const int* nsrc, int grad, double* const* tt,
                                      double* const* ttgrad, double* vzero, void* workspace,
                                      size_t workspace_bytes, long long spin_limit, int* shape,
                                      float* best_ms, void* stream) {
  if (nmodel < 1 || !nsrc || grad < 0 || grad > 1) return kInvalidArgument;
  long long total = 0;
  for (int m = 0; m < nmodel; ++m) total += nsrc[m];
  auto run = [&](const Tune3& t, float* ms) {
    return timed(
        [&]() {
          return solve_batch_impl(nmodel, slow, dims, spacing, sources, nsrc, 1, grad, tt,
                                  ttgrad, vzero, workspace, workspace_bytes, spin_limit, stream,
                                  &t);
        },
        ms);
  };
  Tune3 best;
  float ms = 0.f;
  const bool timing_was_on = kernel_timing_on();
  const int rc = tune_search(run, (int)total, (int)(total / nmodel), 0, 1, false, &best, &ms);
  fteik_kernel_timing(timing_was_on ? 1 : 0);
  if (rc != kOk) return rc;
  tuned_store(batch_key(nmodel, dims, nsrc, grad), best);
  if (shape) {
    shape[0] = best.pencil;
    shape[1] = best.chunk;
    shape[2] = best.coef;
    shape[3] = 0;
  }
  if (best_ms) *best_ms = ms;
  return kOk;
}

extern "C" const char* fteik_last_sweep_kernel(void) { return g_last_sweep_kernel; }

extern "C" int fteik_clear_tuning(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned.clear();
  return kOk;
}
