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
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "fteik_gb300.h"
#include "runtime.h"
#include "solve3d.cuh"

namespace fteik {

constexpr int kLag = kPJ + kPK - 2;
constexpr int kWarpsPerBlock = 4;
// Batches of at least this many sources read precomputed coefficient arrays.
constexpr int kCoefMinSources = 4;


// Plane operator of _fteik3d.py:113-117 (and its ZY / XY twins):
//   ((p*cp + q*cq) + sqrt(q4 - prod*(ta-tb)^2)) / sum,  q4 = 4*v^2*sum
__device__ __forceinline__ double plane_op(double p, double cp, double q, double cq, double d,
                                           double q4, double prod, const Recip& r) {
  double num = p * cp + q * cq;
  double rad = q4 - prod * (d * d);
  return div_by(num + sqrt(rad), r);
}


// Where the update gets its coefficients from.  Both give the same values:
//  * CoefArrays reads the precomputed arrays (one read each; pays off when
//    many sources share them, as they then stay in L2);
//  * CoefCells derives them from the 8 slowness cells around the node,
//    U[a][b][c] indexed upwind-first (a = 0 is the reference's cell row i1 =
//    i - sgnvz, a = 1 the other row of the pair {max(i-1,0), min(i,nz-2)};
//    b, c likewise along j, k), which stay in L2 for any number of sources.
struct CoefArrays {
  const Coef3& C;
  long long oz1, ox1, oy1, ozx, ozy, oxy, ot3;
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
template <bool GRAD, class CP>
__device__ __forceinline__ double node_update3d(double tv, double te, double tn, double tev,
                                                double ten, double tnv, double tnve, double t0,
                                                const CP& c, const Ops3& o, int sz, int sx,
                                                int sy, uint8_t& code) {
  // 1D operators, _fteik3d.py:76-104
  const double t1d1 = tv + c.z1();
  const double t1d2 = te + c.x1();
  const double t1d3 = tn + c.y1();
  const double t1d = dmin(dmin(t1d1, t1d2), t1d3);

  // 2D operators, _fteik3d.py:106-143
  double t2d1 = kBig;
  if (dlt(tv, te + c.zxa()) && dlt(te, tv + c.zxb())) {
    double ta = tev + te - tv;
    double tb = tev - te + tv;
    t2d1 = plane_op(tb, o.dz2i, ta, o.dx2i, ta - tb, c.zxq(), o.dz2dx2, o.rzx);
  }
  double t2d2 = kBig;
  if (dlt(tv, tn + c.zya()) && dlt(tn, tv + c.zyb())) {
    double ta = tv - tn + tnv;
    double tb = tn - tv + tnv;
    t2d2 = plane_op(ta, o.dz2i, tb, o.dy2i, ta - tb, c.zyq(), o.dz2dy2, o.rzy);
  }
  double t2d3 = kBig;
  if (dlt(te, tn + c.xya()) && dlt(tn, te + c.xyb())) {
    double ta = te - tn + ten;
    double tb = tn - te + ten;
    t2d3 = plane_op(ta, o.dx2i, tb, o.dy2i, ta - tb, c.xyq(), o.dx2dy2, o.rxy);
  }
  const double t2d = dmin(dmin(t2d1, t2d2), t2d3);

  // 3D operator, _fteik3d.py:145-159
  double t3d = kBig;
  if (dlt(dmax(dmax(tv, te), tn), dmin(t1d, t2d))) {
    const double htn = half(tn), hten = half(ten), htv = half(tv), htev = half(tev);
    const double htnv = half(tnv), hte = half(te);
    double ta = te - htn + hten - htv + htev - tnv + tnve;
    double tb = tv - htn + htnv - hte + htev - ten + tnve;
    double tc = tn - hte + hten - htv + htnv - tev + tnve;
    double t2 = c.t3();
    double dab = ta - tb, dbc = tb - tc, dac = ta - tc;
    double t3 = o.dz2dx2 * (dab * dab);
    t3 += o.dz2dy2 * (dbc * dbc);
    t3 += o.dx2dy2 * (dac * dac);
    if (dle(t3, t2)) {
      double t1 = tb * o.dz2i + ta * o.dx2i + tc * o.dy2i;
      t3d = div_by(t1 + sqrt(t2 - t3), o.rsum);
    }
  }

  // _fteik3d.py:161-200
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

struct Sweep3Args {
  double* tt;
  uint8_t* rec;
  Coef3 C;              // precomputed coefficients (COEF variant)
  const double* slow;   // slowness cells (cell variant)
  const int* no_skip;  // set by coef3d_kernel when the all-Big skip is not exact
  uint8_t* tape_code;   // optional: per sweep, the operator code of every change
  double* tape_old;     // optional: per sweep, the value each change replaced
  unsigned* progress;
  unsigned* ticket;
  int* status;
  const int* order;
  int nz, nx, ny;  // cells
  int NZ, NX, NY;  // nodes
  long long nodes;
  int nsrc, nepochs, npencils, PJ, PK, total_steps;
  unsigned stride;
  long long spin_limit;
  Ops3 o;
};

// Lane-0 bounded wait until *p >= target.  Gives up (and flags the status)
// after spin_limit polls, or as soon as another warp has flagged a failure.
__device__ __forceinline__ bool wait_geq(const unsigned* p, unsigned target, int* status,
                                         long long spin_limit) {
  if (ld_acquire(p) >= target) return true;
  for (long long it = 0;; ++it) {
    __nanosleep(it < 8 ? 64 : 512);
    if (ld_acquire(p) >= target) return true;
    if (it >= spin_limit) {
      atomicCAS(status, 0, (int)kDeviceWaitTimeout);
      return false;
    }
    if ((it & 15) == 15 && *((volatile int*)status) != 0) return false;
  }
}

template <bool GRAD, bool COEF>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    sweep3d_kernel(const Sweep3Args A) {
  const int lane = threadIdx.x & 31;
  const int lj = lane >> 3, lk = lane & 7;
  const Ops3& o = A.o;
  const long long NXY = (long long)A.NX * A.NY;
  const unsigned total_items = (unsigned)A.nepochs * A.npencils * A.nsrc;
  const int T = A.total_steps;

  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(A.ticket, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= total_items) break;
    const int e = (int)(t / ((unsigned)A.npencils * A.nsrc));
    const unsigned rem = t - (unsigned)e * A.npencils * A.nsrc;
    const int p = (int)(rem / A.nsrc);
    const int src = (int)(rem - (unsigned)p * A.nsrc);
    const int dir = e & 7;
    const int sz = dir < 4 ? 1 : -1, sx = (dir & 1) ? -1 : 1, sy = (dir & 2) ? -1 : 1;
    const int JL = A.order[p] >> 16, KL = A.order[p] & 0xffff;
    const int J = sx > 0 ? JL : A.PJ - 1 - JL;
    const int K = sy > 0 ? KL : A.PK - 1 - KL;
    unsigned* prog = A.progress + (long long)src * A.npencils;
    unsigned* my_prog = prog + J * A.PK + K;
    const unsigned base = (unsigned)e * A.stride;

    // Dependencies on the previous sweep: this pencil, and the pencils that
    // read it (its downwind neighbours in the previous direction).
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
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    if (!ok) {
      __syncwarp();
      if (lane == 0) st_release(my_prog, base + (unsigned)T);
      continue;
    }

    // Upwind pencils of this sweep.
    const int Ju = J - sx, Ku = K - sy;
    const bool hJu = Ju >= 0 && Ju < A.PJ, hKu = Ku >= 0 && Ku < A.PK;
    const unsigned* prog_j = prog + Ju * A.PK + K;
    const unsigned* prog_k = prog + J * A.PK + Ku;
    const unsigned* prog_jk = prog + Ju * A.PK + Ku;

    const int j = sx > 0 ? J * kPJ + lj : J * kPJ + (kPJ - 1) - lj;
    const int k = sy > 0 ? K * kPK + lk : K * kPK + (kPK - 1) - lk;
    const bool in_grid = j < A.NX && k < A.NY;
    const bool frozen_jk = (j == (sx > 0 ? 0 : A.NX - 1)) || (k == (sy > 0 ? 0 : A.NY - 1));
    // Offsets of the coefficient reads that depend on the column only (see
    // Coef3): j1, k1 are the upwind cell indices of the reference.
    const int j1 = sx > 0 ? j - 1 : j, k1 = sy > 0 ? k - 1 : k;
    const long long jk = (long long)j * A.NY + k;
    const long long j1k = (long long)j1 * A.NY + k, jk1 = (long long)j * A.NY + k1;
    const long long j1k1 = (long long)j1 * A.NY + k1;
    // Slowness cell offsets around the column, upwind cell first (CoefCells).
    const int jm = imax(j - 1, 0), jp = imin(j, A.NX - 2);
    const int km = imax(k - 1, 0), kp = imin(k, A.NY - 2);
    const long long NYc = A.ny, NXYc = (long long)A.nx * A.ny;
    const long long ju = (sx > 0 ? jm : jp) * NYc, jo = (sx > 0 ? jp : jm) * NYc;
    const long long ku = sy > 0 ? km : kp, ko = sy > 0 ? kp : km;
    double* tts = A.tt + (long long)src * A.nodes;
    uint8_t* recs = GRAD ? A.rec + (long long)src * A.nodes : nullptr;
    const long long dj = (long long)sx * A.NY, dk = sy;
    const long long di = (long long)sz * NXY;
    const bool may_skip = *A.no_skip == 0;
    const long long big_bits = __double_as_longlong(kBig);

    double r1 = 0.0, r2 = 0.0, r3 = 0.0;
    constexpr int kChunk = 4;
    for (int s = 0; s < T; ++s) {
      if ((s % kChunk) == 0) {
        // Upwind data needed by the steps s .. s+kChunk-1 of this chunk.
        const int last = imin(s + kChunk - 1, T - 1);
        bool w = true;
        if (lane == 0) {
          if (hJu) w = wait_geq(prog_j, base + (unsigned)imin(last + kPJ, T), A.status, A.spin_limit);
          if (w && hKu)
            w = wait_geq(prog_k, base + (unsigned)imin(last + kPK, T), A.status, A.spin_limit);
          if (w && hJu && hKu)
            w = wait_geq(prog_jk, base + (unsigned)imin(last + kLag + 1, T), A.status,
                         A.spin_limit);
          if (w) __threadfence();
        }
        w = __shfl_sync(0xffffffffu, w ? 1 : 0, 0) != 0;
        __syncwarp();
        if (!w) break;
      }
      const double u8_1 = __shfl_up_sync(0xffffffffu, r1, 8);
      const double u8_2 = __shfl_up_sync(0xffffffffu, r2, 8);
      const double u1_1 = __shfl_up_sync(0xffffffffu, r1, 1);
      const double u1_2 = __shfl_up_sync(0xffffffffu, r2, 1);
      const double u9_2 = __shfl_up_sync(0xffffffffu, r2, 9);
      const double u9_3 = __shfl_up_sync(0xffffffffu, r3, 9);
      const int r = s - lj - lk;
      const bool act = in_grid && r >= 0 && r < A.NZ;
      const int i = sz > 0 ? r : A.NZ - 1 - r;
      const long long n = (long long)i * NXY + jk;
      const double t0 = act ? ld_cg(tts + n) : 0.0;
      double res = t0;
      bool upd = act && r != 0 && !frozen_jk;
      double tv = 0.0, te = 0.0, tn = 0.0, tev = 0.0, tnv = 0.0, ten = 0.0, tnve = 0.0;
      if (upd) {
        tv = r1;
        te = lj > 0 ? u8_1 : ld_cg(tts + n - dj);
        tn = lk > 0 ? u1_1 : ld_cg(tts + n - dk);
        tev = lj > 0 ? u8_2 : ld_cg(tts + n - di - dj);
        tnv = lk > 0 ? u1_2 : ld_cg(tts + n - di - dk);
        ten = (lj > 0 && lk > 0) ? u9_2 : ld_cg(tts + n - dj - dk);
        tnve = (lj > 0 && lk > 0) ? u9_3 : ld_cg(tts + n - di - dj - dk);
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
        if (upd) {
          uint8_t code = 0;
          if (COEF) {
            const long long i0 = (long long)i * NXY;
            const long long i1 = (long long)(sz > 0 ? i - 1 : i) * NXY;
            const CoefArrays cp{A.C,      i1 + jk,   i0 + j1k,   i0 + jk1,
                                i1 + j1k, i1 + jk1, i0 + j1k1, i1 + j1k1};
            res = node_update3d<GRAD>(tv, te, tn, tev, ten, tnv, tnve, t0, cp, o, sz, sx, sy,
                                      code);
          } else {
            const int im = imax(i - 1, 0), ip = imin(i, A.NZ - 2);
            const long long iu = (sz > 0 ? im : ip) * NXYc, io = (sz > 0 ? ip : im) * NXYc;
            CoefCells cp{{}, o};
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
              for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int c = 0; c < 2; ++c)
                  cp.U[a][b][c] = __ldg(A.slow + (a ? io : iu) + (b ? jo : ju) + (c ? ko : ku));
            res = node_update3d<GRAD>(tv, te, tn, tev, ten, tnv, tnve, t0, cp, o, sz, sx, sy,
                                      code);
          }
          if (!deq(res, t0)) {
            tts[n] = res;
            if (GRAD) recs[n] = code;
            if (A.tape_code) {
              const long long tq = ((long long)e * A.nsrc + src) * A.nodes + n;
              A.tape_code[tq] = code;
              A.tape_old[tq] = t0;
            }
          }
        }
      }
      r3 = r2;
      r2 = r1;
      r1 = res;
      if (((s + 1) % kChunk) == 0 || s + 1 == T) {
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
__global__ void coef3d_kernel(const double* slow, int nz, int nx, int ny, Ops3 o, Coef3 C,
                              bool write, int* no_skip) {
  const int NX = nx + 1, NY = ny + 1;
  const long long n_nodes = (long long)(nz + 1) * NX * NY;
  const double hmin = fmin(o.dz, fmin(o.dx, o.dy));
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n_nodes;
       q += (long long)gridDim.x * blockDim.x) {
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
      continue;
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

// Source set-up, _fteik3d.py:409-456: one thread per source.
__global__ void init3d_kernel(const double* slow, const double* src, int nsrc, int nz, int nx,
                              int ny, Ops3 o, double* tt, long long nodes, Source3* params,
                              double* vzero_out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsrc) return;
  Source3 p;
  double zsa = src[3 * s] / o.dz, xsa = src[3 * s + 1] / o.dx, ysa = src[3 * s + 2] / o.dy;
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
  params[s] = p;
  vzero_out[s] = p.vzero;
  const int NX = nx + 1, NY = ny + 1;
  double* t = tt + (long long)s * nodes;
  for (int q = 0; q < 8; ++q) {
    const int i = p.zsi + (q & 1), j = p.xsi + ((q >> 1) & 1), k = p.ysi + ((q >> 2) & 1);
    double tzc, txc, tyc;
    t[((long long)i * NX + j) * NY + k] = t_anad3(i, j, k, o, p, tzc, txc, tyc);
  }
}

// Gradient post-pass, _fteik3d.py:464-488.  The 8 nodes around the source
// start from the analytic derivatives they were initialised with
// (_fteik3d.py:453-456); every other node starts from zero.
__global__ void grad3d_kernel(const double* tt, const uint8_t* rec, const Source3* params,
                              int nsrc, int NZ, int NX, int NY, Ops3 o, double* ttgrad) {
  const long long nodes = (long long)NZ * NX * NY;
  const long long total = nodes * nsrc;
  const long long NXY = (long long)NX * NY;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(q / nodes);
    const long long n = q - (long long)s * nodes;
    const int i = (int)(n / NXY);
    const int j = (int)((n - (long long)i * NXY) / NY);
    const int k = (int)(n - (long long)i * NXY - (long long)j * NY);
    const Source3 p = params[s];
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    if ((unsigned)(i - p.zsi) <= 1u && (unsigned)(j - p.xsi) <= 1u && (unsigned)(k - p.ysi) <= 1u)
      t_anad3(i, j, k, o, p, g0, g1, g2);
    const int code = rec[q];
    const int cz = code / 9 - 1, cx = (code / 3) % 3 - 1, cy = code % 3 - 1;
    const double tq = tt[q];
    if (cz != 0) g0 = div_by((double)cz * (tq - tt[q - cz * NXY]), o.rdz);
    if (cx != 0) g1 = div_by((double)cx * (tq - tt[q - (long long)cx * NY]), o.rdx);
    if (cy != 0) g2 = div_by((double)cy * (tq - tt[q - cy]), o.rdy);
    const double gn = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
    if (gn > 0.0) {
      g0 /= gn;
      g1 /= gn;
      g2 /= gn;
    }
    ttgrad[3 * q] = g0;
    ttgrad[3 * q + 1] = g1;
    ttgrad[3 * q + 2] = g2;
  }
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


}  // namespace fteik

using namespace fteik;

extern "C" size_t fteik3d_workspace_bytes(int nz, int nx, int ny, int nsrc, int grad) {
  if (nz < 1 || nx < 1 || ny < 1 || nsrc < 1) return 0;
  return layout3(nz, nx, ny, nsrc, grad).total;
}

static int solve3d_impl(const double* slow, int nz, int nx, int ny, double dz, double dx,
                        double dy, const double* sources, int nsrc, int nsweep, int grad,
                        double* tt, double* ttgrad, double* vzero, void* workspace,
                        size_t workspace_bytes, uint8_t* tape_code, double* tape_old,
                        long long spin_limit, void* stream) {
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
  const int NZ = nz + 1, NX = nx + 1, NY = ny + 1;
  const int PJ = (NX + kPJ - 1) / kPJ, PK = (NY + kPK - 1) / kPK;
  const long long nodes = (long long)NZ * NX * NY;
  const int T = NZ + kLag;
  const unsigned long long stride = (unsigned long long)T + 1;
  const unsigned long long nepochs = 8ull * nsweep;
  if (nepochs * stride >= (1ull << 31) || nepochs * PJ * PK * (unsigned long long)nsrc >= (1ull << 31) ||
      PJ >= (1 << 15) || PK >= (1 << 16))
    return kInvalidArgument;

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
  const long long opt_coef = option_value(kOptSweepCoef);
  const bool use_coef = opt_coef < 0 ? nsrc >= kCoefMinSources : opt_coef != 0;
  coef3d_kernel<<<grid_for(nodes, 256), 256, 0, st>>>(slow, nz, nx, ny, o, C, use_coef, no_skip);
  const long long ntot = nodes * nsrc;
  fill3d_kernel<<<grid_for(ntot, 256), 256, 0, st>>>(tt, rec, ntot);
  init3d_kernel<<<(nsrc + 63) / 64, 64, 0, st>>>(slow, src_dev, nsrc, nz, nx, ny, o, tt, nodes,
                                                 params, vzero);
  FTEIK_CHECK(cudaGetLastError());
  if (nsweep > 0) {
    Sweep3Args A;
    A.tt = tt;
    A.rec = rec;
    A.C = C;
    A.slow = slow;
    A.no_skip = no_skip;
    A.tape_code = tape_code;
    A.tape_old = tape_old;
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
    A.spin_limit = spin_limit > 0 ? spin_limit : (1LL << 25);
    A.o = o;
    const long long items = (long long)nepochs * PJ * PK * nsrc;
    const void* kern = grad ? (use_coef ? (const void*)sweep3d_kernel<true, true>
                                        : (const void*)sweep3d_kernel<true, false>)
                            : (use_coef ? (const void*)sweep3d_kernel<false, true>
                                        : (const void*)sweep3d_kernel<false, false>);
    int blocks = resident_blocks(kern, kWarpsPerBlock * 32);
    const long long need = (items + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (need < blocks) blocks = (int)need;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    timing_events(&ev0, &ev1);
    if (ev0) FTEIK_CHECK(cudaEventRecord(ev0, st));
    void* args[] = {(void*)&A};
    FTEIK_CHECK(cudaLaunchKernel(kern, dim3(blocks), dim3(kWarpsPerBlock * 32), args, 0, st));
    if (ev1) FTEIK_CHECK(cudaEventRecord(ev1, st));
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
                      vzero, workspace, workspace_bytes, nullptr, nullptr, spin_limit, stream);
}

extern "C" size_t fteik3d_tape_bytes(int nz, int nx, int ny, int nsrc, int nsweep) {
  if (nz < 1 || nx < 1 || ny < 1 || nsrc < 1 || nsweep < 0) return 0;
  const size_t n = (size_t)(nz + 1) * (nx + 1) * (ny + 1) * nsrc * 8 * (size_t)nsweep;
  return n == 0 ? 256 : align_up(n) + align_up(8 * n);  // nsweep 0: a token buffer
}

extern "C" int fteik3d_solve_tape(const double* slow, int nz, int nx, int ny, double dz,
                                  double dx, double dy, const double* sources, int nsrc,
                                  int nsweep, double* tt, double* vzero, void* workspace,
                                  size_t workspace_bytes, void* tape, size_t tape_bytes,
                                  long long spin_limit, void* stream) {
  const size_t need = fteik3d_tape_bytes(nz, nx, ny, nsrc, nsweep);
  if (!tape || need == 0) return kInvalidArgument;
  if (tape_bytes < need) return kWorkspaceTooSmall;
  const size_t n = (size_t)(nz + 1) * (nx + 1) * (ny + 1) * nsrc * 8 * (size_t)nsweep;
  uint8_t* code = (uint8_t*)tape;
  double* old = (double*)((char*)tape + align_up(n));
  // 255 marks "unchanged in this sweep"
  FTEIK_CHECK(cudaMemsetAsync(code, 0xff, n, (cudaStream_t)stream));
  int rc = solve3d_impl(slow, nz, nx, ny, dz, dx, dy, sources, nsrc, nsweep, 2, tt, nullptr,
                        vzero, workspace, workspace_bytes, code, old, spin_limit, stream);
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
