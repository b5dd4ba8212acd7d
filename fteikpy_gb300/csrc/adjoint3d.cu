// Adjoint of the 3D solve: d(loss)/d(slowness) for a loss on the traveltimes
// interpolated at receivers.  The reference has no derivative; this is the
// differentiation the GPU path adds for tomography.
//
// It is the exact reverse-mode derivative of the sweeps the reference runs,
// not of an idealised fixed point: FTeik's rotated 2D/3D stencils have
// negative partials, so after the last sweep some nodes still hold values
// computed from older neighbour values, and a fixed-point adjoint would not
// match finite differences of the solver.  The forward solve therefore keeps a
// tape (fteik3d_solve_tape): for every sweep, the code of the operator that
// changed each node (the reference's ttsgn, _fteik3d.py:166-200) and the value
// it replaced.  Going back through the sweeps, each undone against its own
// direction (so that a node comes after every node that read it), a node
// first collects the adjoint its readers of that sweep sent it, then, if
// the sweep changed it, recomputes its operator's partials from the values it
// read (_fteik3d.py:76-159; no saved intermediates), sends the adjoint on to
// those inputs, books the slowness term, and restores its previous value.
// Every transfer is a pull or a per-node accumulation, so the result is the
// same from run to run.
#include <algorithm>
#include <climits>
#include <cstdint>

#include "common.cuh"
#include "fteik_gb300.h"
#include "interp.cuh"
#include "runtime.h"
#include "solve3d.cuh"

namespace fteik {

constexpr int kSlots = 7;  // input slot (bz,bx,by) = bz*4 + bx*2 + by - 1

struct RevArgs {
  const double* slow;
  const Source3* params;
  double* tt;            // [nsrc][nodes] traveltimes, rolled back sweep by sweep
  double* lam;           // [nsrc][nodes] adjoint of each node's current value
  double* contrib;       // [nsrc][nodes][7] adjoint a changed node sends to each input
  double* g8;            // [nsrc][nodes][8] dL/ds per node, by surrounding cell
  Tape3 tape;            // the forward's record of every change (see Tape3)
  int nz, nx, ny, NZ, NX, NY;
  long long nodes;
  int nsrc;
  Ops3 o;
};

__device__ __forceinline__ void decode(int code, int& az, int& ax, int& ay) {
  az = code / 9 - 1;
  ax = (code / 3) % 3 - 1;
  ay = code % 3 - 1;
}

// The cells around node (i, j, k) are named by their slot a*4 + b*2 + c:
// a = 0 for the cell row max(i-1, 0), 1 for min(i, nz-1), and b, c likewise
// along j and k; where the two rows coincide (the model's edges) the one cell
// is slot a = 0.  CellFrame holds, per axis, the linear offsets of the two
// rows and whether they differ.
struct CellFrame {
  long long z0, z1, x0, x1, y0, y1;  // row offsets into slow: z * nx * ny, x * ny, y
  int za, xa, ya;                    // 1 if the second row is a different cell
};

__device__ __forceinline__ long long cell_at(const CellFrame& F, int slot) {
  return ((slot & 4) ? F.z1 : F.z0) + ((slot & 2) ? F.x1 : F.x0) + ((slot & 1) ? F.y1 : F.y0);
}

// The distinct cells of the list whose slowness is minimal, as a bit mask
// of slots (duplicate slots from collapsed rows are one cell, not a tie).
// Slowness is positive, so its bit patterns order like its values.
template <int N>
__device__ __forceinline__ unsigned min_slots(const double* slow, const CellFrame& F,
                                              const int (&slots)[N], double& vmin) {
  long long bits[N];
  long long bv = LLONG_MAX;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    bits[q] = __double_as_longlong(__ldg(slow + cell_at(F, slots[q])));
    bv = bits[q] < bv ? bits[q] : bv;
  }
  unsigned mask = 0;
#pragma unroll
  for (int q = 0; q < N; ++q)
    if (bits[q] == bv) mask |= 1u << slots[q];
  vmin = __longlong_as_double(bv);
  return mask;
}

// Partials of the operator that produced t_n (signs az, ax, ay from the
// branch record) with respect to its inputs (slot (bz,bx,by) = input at
// n - (bz*az, bx*ax, by*ay)) and to the slowness it used, evaluated at the
// input values in t: the derivatives of _fteik3d.py:76-159.  The 1D and 2D
// operators use the minimum slowness of 4 or 2 cells.  Where several cells
// share that minimum the solver has no derivative: lowering one of them moves
// the result, raising it does not.  Each tied cell then gets half the
// partial, the mean of its two one-sided derivatives, which is what a central
// difference on that cell measures.  The cells come back as a bit mask of
// slots, with the partial ps for each.
//
// These partials need not reproduce any rounding of the reference, so they
// use the per-launch reciprocals of the operators' denominators and one
// reciprocal square root per operator instead of divisions.
__device__ void linearize(int az, int ax, int ay, int i, int j, int k, long long n,
                          const double* t, const double* slow, const CellFrame& F, int NX_,
                          int NY_, const Ops3& o, double (&w)[kSlots], double& ps,
                          unsigned& cells) {
  const long long NXY = (long long)NX_ * NY_;
#pragma unroll
  for (int e = 0; e < kSlots; ++e) w[e] = 0.0;
  ps = 0.0;
  double v;
  // upwind row of each axis: the reference's i1 = i - 1 (sign +) or i (sign -)
  const int a1 = az > 0 ? 0 : F.za, b1 = ax > 0 ? 0 : F.xa, c1 = ay > 0 ? 0 : F.ya;
#define T(bz, bx, by) \
  __ldcg(t + n - (long long)(bz) * az * NXY - (long long)(bx) * ax * NY_ - (by) * ay)
  const int nnz = (az != 0) + (ax != 0) + (ay != 0);
  if (nnz == 1) {
    int sl[4];
    if (az != 0) {
      sl[0] = a1 * 4; sl[1] = a1 * 4 + F.ya; sl[2] = a1 * 4 + F.xa * 2; sl[3] = sl[2] + F.ya;
      w[3] = 1.0;
      ps = o.dz;
    } else if (ax != 0) {
      sl[0] = b1 * 2; sl[1] = F.za * 4 + b1 * 2; sl[2] = b1 * 2 + F.ya; sl[3] = sl[1] + F.ya;
      w[1] = 1.0;
      ps = o.dx;
    } else {
      sl[0] = c1; sl[1] = F.xa * 2 + c1; sl[2] = F.za * 4 + c1; sl[3] = sl[2] + F.xa * 2;
      w[0] = 1.0;
      ps = o.dy;
    }
    cells = min_slots(slow, F, sl, v);
  } else if (nnz == 2) {
    // plane operators, _fteik3d.py:106-143
    double c1v, c2v, iS, ta, tb;
    int sl[2];
    if (ay == 0) {  // ZX: inputs tv (slot 3), te (1), tev (5)
      const double tv = T(1, 0, 0), te = T(0, 1, 0), tev = T(1, 1, 0);
      ta = tev + te - tv;
      tb = tev - te + tv;
      c1v = o.dz2i; c2v = o.dx2i; iS = o.rzx.hi;  // num = tb*c1 + ta*c2
      sl[0] = a1 * 4 + b1 * 2; sl[1] = sl[0] + F.ya;
    } else if (ax == 0) {  // ZY: inputs tv (3), tn (0), tnv (4)
      const double tv = T(1, 0, 0), tn = T(0, 0, 1), tnv = T(1, 0, 1);
      ta = tv - tn + tnv;
      tb = tn - tv + tnv;
      c1v = o.dz2i; c2v = o.dy2i; iS = o.rzy.hi;  // num = ta*c1 + tb*c2
      sl[0] = a1 * 4 + c1; sl[1] = sl[0] + F.xa * 2;
    } else {  // XY: inputs te (1), tn (0), ten (2)
      const double te = T(0, 1, 0), tn = T(0, 0, 1), ten = T(0, 1, 1);
      ta = te - tn + ten;
      tb = tn - te + ten;
      c1v = o.dx2i; c2v = o.dy2i; iS = o.rxy.hi;  // num = ta*c1 + tb*c2
      sl[0] = b1 * 2 + c1; sl[1] = sl[0] + F.za * 4;
    }
    cells = min_slots(slow, F, sl, v);
    const double S = c1v + c2v, d = ta - tb, p12 = c1v * c2v;
    const double Q = 4.0 * v * v * S - p12 * d * d;
    // t = (num + R) / S with R = sqrt(Q); only 1/R enters the partials
    const double iR = Q > 0.0 ? rsqrt(Q) : 0.0;
    const double r = p12 * d * iR;
    // partials of t with respect to ta and tb
    double dta, dtb;
    if (ay == 0) {  // num = tb*dz2i + ta*dx2i
      dta = (c2v - r) * iS;
      dtb = (c1v + r) * iS;
    } else {  // num = ta*c1 + tb*c2
      dta = (c1v - r) * iS;
      dtb = (c2v + r) * iS;
    }
    // ta = x12 + x2 - x1 (ZX: tev + te - tv) or x1 - x2 + x12 (ZY, XY)
    if (ay == 0) {
      w[3] = dtb - dta;  // tv
      w[1] = dta - dtb;  // te
      w[5] = dta + dtb;  // tev
    } else if (ax == 0) {
      w[3] = dta - dtb;  // tv
      w[0] = dtb - dta;  // tn
      w[4] = dta + dtb;  // tnv
    } else {
      w[1] = dta - dtb;  // te
      w[0] = dtb - dta;  // tn
      w[2] = dta + dtb;  // ten
    }
    ps = 4.0 * v * iR;  // dt/dv = (dR/dv) / S, dR/dv = 4 v S / R
  } else {
    // 3D operator, _fteik3d.py:145-159
    const double tv = T(1, 0, 0), te = T(0, 1, 0), tn = T(0, 0, 1), tev = T(1, 1, 0);
    const double ten = T(0, 1, 1), tnv = T(1, 0, 1), tnve = T(1, 1, 1);
    const double ta = te - 0.5 * tn + 0.5 * ten - 0.5 * tv + 0.5 * tev - tnv + tnve;
    const double tb = tv - 0.5 * tn + 0.5 * tnv - 0.5 * te + 0.5 * tev - ten + tnve;
    const double tc = tn - 0.5 * te + 0.5 * ten - 0.5 * tv + 0.5 * tnv - tev + tnve;
    const int sl = a1 * 4 + b1 * 2 + c1;
    cells = 1u << sl;
    v = __ldg(slow + cell_at(F, sl));
    const double dab = ta - tb, dbc = tb - tc, dac = ta - tc;
    const double t2 = v * v * o.dsum * 9.0;
    const double t3 = o.dz2dx2 * dab * dab + o.dz2dy2 * dbc * dbc + o.dx2dy2 * dac * dac;
    const double iw = t2 > t3 ? rsqrt(t2 - t3) : 0.0;  // 1 / W, W = sqrt(t2 - t3)
    const double isum = o.rsum.hi;
    const double dta = (o.dx2i - (o.dz2dx2 * dab + o.dx2dy2 * dac) * iw) * isum;
    const double dtb = (o.dz2i - (o.dz2dy2 * dbc - o.dz2dx2 * dab) * iw) * isum;
    const double dtc = (o.dy2i + (o.dz2dy2 * dbc + o.dx2dy2 * dac) * iw) * isum;
    // d(ta, tb, tc) / d(tv, te, tn, tev, ten, tnv, tnve)
    const double hta = 0.5 * dta, htb = 0.5 * dtb, htc = 0.5 * dtc;
    w[3] = dtb - hta - htc;  // tv
    w[1] = dta - htb - htc;  // te
    w[0] = dtc - hta - htb;  // tn
    w[5] = hta + htb - dtc;  // tev
    w[2] = hta + htc - dtb;  // ten
    w[4] = htb + htc - dta;  // tnv
    w[6] = dta + dtb + dtc;  // tnve
    ps = 9.0 * v * iw;
  }
  if (__popc(cells) > 1) ps *= 0.5;
#undef T
}

// Slot of cell (ci, cj, ck) among the 8 cells around node (i, j, k)
// (a = 0 for the cell row max(i-1, 0), 1 for min(i, nz-1); equal rows use 0).
__device__ __forceinline__ int cell_slot(int i, int j, int k, int ci, int cj, int ck) {
  const int a = ci == imax(i - 1, 0) ? 0 : 1;
  const int b = cj == imax(j - 1, 0) ? 0 : 1;
  const int c = ck == imax(k - 1, 0) ? 0 : 1;
  return a * 4 + b * 2 + c;
}

// The reverse pass.  Undoing sweep e (signs sz, sx, sy) must visit a node
// after every node that read it in that sweep (its downwind neighbours n +
// (bz*sz, bx*sx, by*sy)), so it is itself a directional sweep, against the
// direction of e, and runs in the forward kernel's schedule with the signs
// reversed: one warp owns one pencil of 4 x 8 node columns, lane (lj, lk)
// handles row r = s - lj - lk at step s, and the pencils of all sources and
// all sweeps run in one persistent launch, taking work items from a ticket
// counter and waiting (bounded) on per-pencil progress counters.
//
// Each node n first pulls what its readers of the sweep sent it.  The reader
// across input slot (bz, bx, by) lies in lane (lj - bx, lk - by) and was
// visited bz + bx + by steps earlier, so inside a pencil the contribution
// arrives by a warp shuffle from a short per-slot history kept in registers;
// a reader in a neighbouring pencil left it in `contrib` (the lanes on a
// pencil's far faces write the slots their neighbours consume).  A reader
// that did not change in the sweep, or whose operator does not use the slot,
// sends -0.0, which leaves the sum bit for bit unchanged.  Then, if the sweep
// changed n, it recomputes its operator's partials from the values it read
// (its upwind neighbours, not yet restored: they come later in this order),
// forms what it sends to each input, books the slowness term and restores
// its previous value.
constexpr int kRevPW = 4;     // pencil width along j (the pencil is 4 x 8 columns)
constexpr int kRevWarps = 4;  // warps per block

struct RevSched {
  unsigned* progress;  // [nsrc][PJ*PK]
  unsigned* ticket;
  int* status;
  int PJ, PK, T, nepochs, chunk;
  unsigned stride;  // progress counter range of one reverse sweep (>= T)
  long long spin_limit;
};

// The p-th pencil in order of its diagonal JL + KL (then JL): every pencil a
// pencil depends on in the same sweep comes first.
__device__ __forceinline__ void pencil_at(int p, int PJ, int PK, int& JL, int& KL) {
  for (int d = 0;; ++d) {
    const int lo = imax(0, d - PK + 1), hi = imin(d, PJ - 1);
    const int cnt = hi - lo + 1;
    if (p < cnt) {
      JL = lo + p;
      KL = d - JL;
      return;
    }
    p -= cnt;
  }
}

// The value that the change of node n = (i, j, k) of source src in sweep e
// replaced (see Tape3): its initial value for a first change (Big, or the
// analytic value kept for the 8 nodes around the source), else the history
// slot or the overflow table.  Flags FTEIK_TAPE_OVERFLOW if the table lacks
// the entry (which a solve that reported no overflow never leaves).
__device__ __forceinline__ double tape_replaced(const Tape3& P, int src, long long sn,
                                                const uint8_t* rec, int e, int i, int j, int k,
                                                int zsi, int xsi, int ysi, int* status) {
  const int m = tape_changes_before(rec, e) + 1;
  if (m == 1) {
    const int a = i - zsi, b = j - xsi, c = k - ysi;
    if ((unsigned)a <= 1u && (unsigned)b <= 1u && (unsigned)c <= 1u)
      return __ldg(P.init8 + src * 8 + a + 2 * b + 4 * c);
    return kBig;
  }
  if (m - 2 < P.H) return __ldg(P.hist + sn * P.H + (m - 2));
  const unsigned long long key = tape_key(sn + P.sn0, m);
  unsigned long long h = tape_slot(key, P.mask);
  for (int q = 0; q < kTapeProbes; ++q) {
    const unsigned long long kq = __ldg(P.key + h);
    if (kq == key) return __ldg(P.val + h);
    if (kq == 0ull) break;
    h = (h + 1) & P.mask;
  }
  atomicCAS(status, 0, (int)kTapeOverflow);
  return kBig;
}

// Whether the operator with signs (az, ax, ay) reads input slot (bz, bx, by).
__device__ __forceinline__ bool uses_slot(int az, int ax, int ay, int bz, int bx, int by) {
  return !((bz && !az) || (bx && !ax) || (by && !ay));
}

template <int PW>
__global__ void __launch_bounds__(kRevWarps * 32)
    adj_sweep_kernel(const __grid_constant__ RevArgs A, const __grid_constant__ RevSched S) {
  constexpr int PJW = PW, PKW = 32 / PW, LAG = PJW + PKW - 2;
  const int lane = threadIdx.x & 31;
  const int lj = lane / PKW, lk = lane % PKW;
  const unsigned npen = (unsigned)S.PJ * S.PK;
  const unsigned per_epoch = npen * (unsigned)A.nsrc;
  const unsigned total_items = (unsigned)S.nepochs * per_epoch;
  const unsigned cmask = (unsigned)S.chunk - 1u;
  const long long NXY = (long long)A.NX * A.NY;
  const double nz0 = -0.0;

  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(S.ticket, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= total_items) break;
    const int er = (int)(t / per_epoch);  // sweeps are undone last first
    const int e = S.nepochs - 1 - er;
    const unsigned rem = t - (unsigned)er * per_epoch;
    const int p = (int)(rem / (unsigned)A.nsrc);
    const int src = (int)(rem - (unsigned)p * A.nsrc);
    int JL, KL;
    pencil_at(p, S.PJ, S.PK, JL, KL);
    const int dir = e & 7;
    const int sz = dir < 4 ? 1 : -1, sx = (dir & 1) ? -1 : 1, sy = (dir & 2) ? -1 : 1;
    const int rz = -sz, rx = -sx, ry = -sy;  // direction of the reverse pass
    const int J = rx > 0 ? JL : S.PJ - 1 - JL;
    const int K = ry > 0 ? KL : S.PK - 1 - KL;
    unsigned* prog = S.progress + (long long)src * npen;
    unsigned* my_prog = prog + J * S.PK + K;
    const unsigned base = (unsigned)er * S.stride;

    // The previous reverse sweep must be done on this pencil and its 8
    // neighbours: their nodes are restored to the values this sweep's
    // operators read, and their readers have consumed the contributions this
    // pencil is about to overwrite.
    bool ok = true;
    if (lane == 0 && er > 0) {
      const unsigned done = base - S.stride + (unsigned)S.T;
      for (int dj = -1; dj <= 1 && ok; ++dj)
        for (int dk = -1; dk <= 1 && ok; ++dk) {
          const int J2 = J + dj, K2 = K + dk;
          if (J2 < 0 || J2 >= S.PJ || K2 < 0 || K2 >= S.PK) continue;
          ok = wait_geq(prog + J2 * S.PK + K2, done, S.status, S.spin_limit);
        }
      if (ok) __threadfence();
    }
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    if (!ok) {
      __syncwarp();
      if (lane == 0) st_release(my_prog, base + (unsigned)S.T);
      continue;
    }

    // Pencils upstream in the reverse direction hold the readers across the
    // pencil's near faces.
    const int Ju = J - rx, Ku = K - ry;
    const bool hJu = Ju >= 0 && Ju < S.PJ, hKu = Ku >= 0 && Ku < S.PK;
    const unsigned* prog_j = prog + Ju * S.PK + K;
    const unsigned* prog_k = prog + J * S.PK + Ku;
    const unsigned* prog_jk = prog + Ju * S.PK + Ku;

    const int j = rx > 0 ? J * PJW + lj : J * PJW + (PJW - 1) - lj;
    const int k = ry > 0 ? K * PKW + lk : K * PKW + (PKW - 1) - lk;
    const bool in_grid = j < A.NX && k < A.NY;
    // readers along j and k exist (the reader along i exists from row 1 on)
    const bool jin = j + sx >= 0 && j + sx < A.NX, kin = k + sy >= 0 && k + sy < A.NY;
    const long long di = (long long)sz * NXY, dj = (long long)sx * A.NY, dk = sy;
    const long long jk = (long long)j * A.NY + k;
    const long long sbase = (long long)src * A.nodes;
    double* lam_s = A.lam + sbase;
    double* tt_s = A.tt + sbase;
    double* con_s = A.contrib + sbase * kSlots;
    double* g8_s = A.g8 + sbase * 8;
    const int zsi = A.params[src].zsi, xsi = A.params[src].xsi, ysi = A.params[src].ysi;
    const bool face_j = lj == PJW - 1, face_k = lk == PKW - 1;
    // the cells around this column (rows along i are set per node)
    const long long nxy_c = (long long)A.nx * A.ny;
    CellFrame F;
    F.x0 = (long long)imax(j - 1, 0) * A.ny;
    F.x1 = (long long)imin(j, A.nx - 1) * A.ny;
    F.xa = F.x1 != F.x0;
    F.y0 = imax(k - 1, 0);
    F.y1 = imin(k, A.ny - 1);
    F.ya = F.y1 != F.y0;

    // What this lane sent across each slot 1, 2 and 3 steps ago.
    double h0 = nz0, h1 = nz0, h3 = nz0;                         // slots 0, 1, 3
    double h2a = nz0, h2b = nz0, h4a = nz0, h4b = nz0, h5a = nz0, h5b = nz0;  // 2, 4, 5
    double h6a = nz0, h6b = nz0, h6c = nz0;                      // slot 6
    for (int s = 0; s < S.T; ++s) {
      if (((unsigned)s & cmask) == 0) {
        const int last = imin(s + (int)cmask, S.T - 1);
        bool w = true;
        if (lane == 0) {
          if (hJu) w = wait_geq(prog_j, base + (unsigned)imin(last + PJW, S.T), S.status, S.spin_limit);
          if (w && hKu)
            w = wait_geq(prog_k, base + (unsigned)imin(last + PKW, S.T), S.status, S.spin_limit);
          if (w && hJu && hKu)
            w = wait_geq(prog_jk, base + (unsigned)imin(last + LAG + 1, S.T), S.status,
                         S.spin_limit);
          if (w) __threadfence();
        }
        w = __shfl_sync(0xffffffffu, w ? 1 : 0, 0) != 0;
        __syncwarp();
        if (!w) break;
      }
      // Contributions from readers in this pencil (lane (lj-bx, lk-by),
      // bz+bx+by steps ago); lanes on the near faces replace them below.
      double p0 = __shfl_up_sync(0xffffffffu, h0, 1);
      double p1 = __shfl_up_sync(0xffffffffu, h1, PKW);
      double p2 = __shfl_up_sync(0xffffffffu, h2b, PKW + 1);
      const double p3 = h3;
      double p4 = __shfl_up_sync(0xffffffffu, h4b, 1);
      double p5 = __shfl_up_sync(0xffffffffu, h5b, PKW);
      double p6 = __shfl_up_sync(0xffffffffu, h6c, PKW + 1);
      const int r = s - lj - lk;
      const bool act = in_grid && r >= 0 && r < A.NZ;
      double c[kSlots];
#pragma unroll
      for (int q = 0; q < kSlots; ++q) c[q] = nz0;
      if (act) {
        const int i = rz > 0 ? r : A.NZ - 1 - r;
        const long long n = (long long)i * NXY + jk;
        const uint8_t* rec = A.tape.code + (sbase + n) * A.tape.E;
        const int code = __ldg(rec + e);
        const double lam0 = __ldcg(lam_s + n);
        const bool iin = r > 0;
        if (lj == 0) {
          p1 = jin ? __ldcg(con_s + (n + dj) * kSlots + 1) : nz0;
          p5 = jin && iin ? __ldcg(con_s + (n + di + dj) * kSlots + 5) : nz0;
        }
        if (lk == 0) {
          p0 = kin ? __ldcg(con_s + (n + dk) * kSlots + 0) : nz0;
          p4 = kin && iin ? __ldcg(con_s + (n + di + dk) * kSlots + 4) : nz0;
        }
        if (lj == 0 || lk == 0) {
          p2 = jin && kin ? __ldcg(con_s + (n + dj + dk) * kSlots + 2) : nz0;
          p6 = jin && kin && iin ? __ldcg(con_s + (n + di + dj + dk) * kSlots + 6) : nz0;
        }
        double lam = lam0 + p0;
        lam = lam + p1;
        lam = lam + p2;
        lam = lam + p3;
        lam = lam + p4;
        lam = lam + p5;
        lam = lam + p6;
        if (code == 255) {
          if (__double_as_longlong(lam) != __double_as_longlong(lam0)) lam_s[n] = lam;
        } else {
          int az, ax, ay;
          decode(code, az, ax, ay);
          F.z0 = (long long)imax(i - 1, 0) * nxy_c;
          F.z1 = (long long)imin(i, A.nz - 1) * nxy_c;
          F.za = F.z1 != F.z0;
          double w[kSlots], ps;
          unsigned cells;
          linearize(az, ax, ay, i, j, k, n, tt_s, A.slow, F, A.NX, A.NY, A.o, w, ps, cells);
#pragma unroll
          for (int q = 0; q < kSlots; ++q) {
            const int bz = (q + 1) >> 2, bx = ((q + 1) >> 1) & 1, by = (q + 1) & 1;
            if (uses_slot(az, ax, ay, bz, bx, by)) c[q] = lam * w[q];
          }
          for (unsigned m = cells; m; m &= m - 1) {
            double* g = g8_s + n * 8 + (__ffs(m) - 1);
            *g = __ldcg(g) + lam * ps;
          }
          lam_s[n] = 0.0;
          tt_s[n] = tape_replaced(A.tape, src, sbase + n, rec, e, i, j, k, zsi, xsi, ysi,
                                  S.status);
        }
        // Slots read by the readers' pencils across the far faces.
        double* co = con_s + n * kSlots;
        if (face_j) {
          co[1] = c[1];
          co[5] = c[5];
        }
        if (face_k) {
          co[0] = c[0];
          co[4] = c[4];
        }
        if (face_j || face_k) {
          co[2] = c[2];
          co[6] = c[6];
        }
      }
      h0 = c[0];
      h1 = c[1];
      h3 = c[3];
      h2b = h2a; h2a = c[2];
      h4b = h4a; h4a = c[4];
      h5b = h5a; h5a = c[5];
      h6c = h6b; h6b = h6a; h6a = c[6];
      if (((unsigned)(s + 1) & cmask) == 0 || s + 1 == S.T) {
        __syncwarp();
        if (lane == 0) {
          __threadfence();
          st_release(my_prog, base + (unsigned)(s + 1));
        }
      }
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      st_release(my_prog, base + (unsigned)S.T);
    }
  }
}

// After the first sweep has been undone every node holds its initial value:
// around the source t = vzero * distance (_fteik3d.py:440-451), which depends
// on the source cell's slowness; every other node holds Big.
__global__ void adj_initial_kernel(const RevArgs A) {
  const long long total = (long long)A.nsrc * 8;
  const long long NXY = (long long)A.NX * A.NY;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int src = (int)(q / 8), e = (int)(q % 8);
    const Source3 p = A.params[src];
    const int i = p.zsi + (e & 1), j = p.xsi + ((e >> 1) & 1), k = p.ysi + (e >> 2);
    const long long n = (long long)i * NXY + (long long)j * A.NY + k;
    const long long base = (long long)src * A.nodes;
    const double a = A.o.dz * ((double)i - p.zsa), b = A.o.dx * ((double)j - p.xsa),
                 c = A.o.dy * ((double)k - p.ysa);
    A.g8[(base + n) * 8 + cell_slot(i, j, k, p.zsi, p.xsi, p.ysi)] +=
        A.lam[base + n] * sqrt(a * a + b * b + c * c);
  }
}

// Receivers: the traveltime at a receiver is _vinterp3d of the final grid; its
// partials with respect to the 8 corner traveltimes seed the adjoint, and the
// source-cell cases T = vzero * distance feed the source cell.  One thread per
// source walks its receivers in order, so the sums are reproducible.
__global__ void adj_seed_kernel(const RevArgs A, const double* ax0, const double* ax1,
                                const double* ax2, const double* sources, const double* recv,
                                int nrec, const double* gT, double* vzg) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= A.nsrc) return;
  const int nx = A.NZ, ny = A.NX, nz = A.NY;  // axis lengths in _vinterp3d's naming
  const double xs = sources[3 * s], ys = sources[3 * s + 1], zs = sources[3 * s + 2];
  const int xsi = search_right_m1(ax0, nx, xs), ysi = search_right_m1(ax1, ny, ys),
            zsi = search_right_m1(ax2, nz, zs);
  const double* t = A.tt + (long long)s * A.nodes;
  double* lam = A.lam + (long long)s * A.nodes;
  double vz_acc = 0.0;
  for (int r = 0; r < nrec; ++r) {
    const double g = gT[(long long)s * nrec + r];
    if (g == 0.0) continue;
    const double xq = recv[3 * r], yq = recv[3 * r + 1], zq = recv[3 * r + 2];
    if (!inside3(ax0, nx, ax1, ny, ax2, nz, xq, yq, zq)) continue;
    const Cell3 c = locate3(ax0, nx, ax1, ny, ax2, nz, xq, yq, zq);
    const double D = dist3(xs, ys, zs, xq, yq, zq);
    if (xsi == c.i1 && ysi == c.j1 && zsi == c.k1) {
      vz_acc += g * D;
      continue;
    }
    double v[8];
    corners3(t, 1, c, ny, nz, v);
    bool all_nonzero = true;
    for (int e = 0; e < 8; ++e) all_nonzero = all_nonzero && (v[e] != 0.0);
    if (!all_nonzero) {
      vz_acc += g * D;
      continue;
    }
    double d[8], w[8];
    d[0] = dist3(xs, ys, zs, c.x1, c.y1, c.z1);
    d[1] = c.ei ? 0.0 : dist3(xs, ys, zs, c.x2, c.y1, c.z1);
    d[2] = c.ej ? 0.0 : dist3(xs, ys, zs, c.x1, c.y2, c.z1);
    d[3] = (c.ei || c.ej) ? 0.0 : dist3(xs, ys, zs, c.x2, c.y2, c.z1);
    d[4] = c.ek ? 0.0 : dist3(xs, ys, zs, c.x1, c.y1, c.z2);
    d[5] = (c.ei || c.ek) ? 0.0 : dist3(xs, ys, zs, c.x2, c.y1, c.z2);
    d[6] = (c.ej || c.ek) ? 0.0 : dist3(xs, ys, zs, c.x1, c.y2, c.z2);
    d[7] = (c.ei || c.ej || c.ek) ? 0.0 : dist3(xs, ys, zs, c.x2, c.y2, c.z2);
    weights3(c, xq, yq, zq, w);
    const double W = fabs((c.x2 - c.x1) * (c.y2 - c.y1) * (c.z2 - c.z1));
    double vq = d[0] / v[0] * w[0];
    for (int e = 1; e < 8; ++e) vq += d[e] / v[e] * w[e];
    vq /= W;
    // T = D / vq, dvq/dv_e = -d_e w_e / (W v_e^2)
    const double f = g * D / (vq * vq * W);
    const long long b = ((long long)c.i1 * ny + c.j1) * nz + c.k1;
    const long long off[8] = {0, (long long)ny * nz, nz, (long long)ny * nz + nz,
                              1, (long long)ny * nz + 1, nz + 1, (long long)ny * nz + nz + 1};
    for (int e = 0; e < 8; ++e) {
      if (d[e] == 0.0) continue;  // a corner past the last node (value 1.0, weight 0)
      lam[b + off[e]] += f * d[e] * w[e] / (v[e] * v[e]);
    }
  }
  vzg[s] = vz_acc;
}

// dL/ds per cell: the terms its 8 corner nodes booked for it, summed over the
// sources in order, plus the receivers' source-cell terms; with `accumulate`,
// the sum continues from the value already in grad_slow, so a problem split
// into consecutive source chunks sums in exactly the unsplit order.
__global__ void adj_gather_kernel(const RevArgs A, const double* vzg, int accumulate,
                                  double* grad_slow) {
  const long long ncell = (long long)A.nz * A.nx * A.ny;
  const long long NXY = (long long)A.NX * A.NY;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(c / ((long long)A.nx * A.ny));
    const int cj = (int)((c / A.ny) % A.nx), ck = (int)(c % A.ny);
    double g = accumulate ? grad_slow[c] : 0.0;
    for (int s = 0; s < A.nsrc; ++s) {
      const long long base = (long long)s * A.nodes;
      for (int e = 0; e < 8; ++e) {
        const int i = ci + (e & 1), j = cj + ((e >> 1) & 1), k = ck + (e >> 2);
        const long long n = (long long)i * NXY + (long long)j * A.NY + k;
        g += A.g8[(base + n) * 8 + cell_slot(i, j, k, ci, cj, ck)];
      }
      const Source3 p = A.params[s];
      if (ci == p.zsi && cj == p.xsi && ck == p.ysi) g += vzg[s];
    }
    grad_slow[c] = g;
  }
}

struct AdjLayout {
  size_t tt, lam, contrib, g8, vzg, sync, total;
  int PJ, PK;
};

static AdjLayout adj_layout(int nz, int nx, int ny, int nsrc) {
  const size_t N = (size_t)(nz + 1) * (nx + 1) * (ny + 1) * nsrc;
  AdjLayout L;
  L.PJ = (nx + 1 + kRevPW - 1) / kRevPW;
  L.PK = (ny + 1 + 32 / kRevPW - 1) / (32 / kRevPW);
  size_t off = 0;
  L.tt = off;
  off = align_up(off + 8 * N);
  L.lam = off;
  off = align_up(off + 8 * N);
  L.contrib = off;
  off = align_up(off + 8 * kSlots * N);
  L.g8 = off;
  off = align_up(off + 8 * 8 * N);
  L.vzg = off;
  off = align_up(off + 8 * (size_t)nsrc);
  L.sync = off;  // int status, unsigned ticket, then the progress counters
  off = align_up(off + 8 + 4 * (size_t)L.PJ * L.PK * nsrc);
  L.total = off;
  return L;
}

}  // namespace fteik

using namespace fteik;

extern "C" size_t fteik3d_adjoint_workspace_bytes(int nz, int nx, int ny, int nsrc) {
  if (nz < 1 || nx < 1 || ny < 1 || nsrc < 1) return 0;
  return adj_layout(nz, nx, ny, nsrc).total;
}

extern "C" int fteik3d_adjoint(const double* slow, int nz, int nx, int ny, double dz, double dx,
                               double dy, int nsrc, int nsweep, const double* tt, int history,
                               const void* tape, size_t tape_bytes,
                               const double* ax0, const double* ax1, const double* ax2,
                               const double* sources, const double* receivers, int nrec,
                               const double* grad_tt_rec, int accumulate, double* grad_slow,
                               void* workspace, size_t workspace_bytes, long long spin_limit,
                               void* stream) {
  return fteik3d_adjoint_part(slow, nz, nx, ny, dz, dx, dy, nsrc, 0, nsrc, nsweep, tt, history,
                              tape, tape_bytes, ax0, ax1, ax2, sources, receivers, nrec,
                              grad_tt_rec, accumulate, grad_slow, workspace, workspace_bytes,
                              spin_limit, stream);
}

extern "C" int fteik3d_adjoint_part(const double* slow, int nz, int nx, int ny, double dz,
                                    double dx, double dy, int nsrc_tape, int src0, int nsrc,
                                    int nsweep, const double* tt_all, int history,
                                    const void* tape, size_t tape_bytes, const double* ax0,
                                    const double* ax1, const double* ax2,
                                    const double* sources_all, const double* receivers, int nrec,
                                    const double* grad_tt_rec_all, int accumulate,
                                    double* grad_slow, void* workspace, size_t workspace_bytes,
                                    long long spin_limit, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nz < 2 || nx < 2 || ny < 2 || nsrc < 1 || src0 < 0 || nsrc_tape < src0 + nsrc ||
      nsweep < 0 || nrec < 0 || !slow || !tt_all || !tape || !ax0 || !ax1 || !ax2 ||
      !sources_all || (nrec > 0 && (!receivers || !grad_tt_rec_all)) || !grad_slow || !workspace)
    return kInvalidArgument;
  const size_t tape_need = fteik3d_tape_bytes(nz, nx, ny, nsrc_tape, nsweep, history);
  if (tape_need == 0) return kInvalidArgument;
  if (tape_bytes < tape_need) return kWorkspaceTooSmall;
  const long long nodes = (long long)(nz + 1) * (nx + 1) * (ny + 1);
  // this part's sources: src0 .. src0 + nsrc - 1 of the solve
  const double* tt = tt_all + src0 * nodes;
  const double* sources = sources_all + 3LL * src0;
  const double* grad_tt_rec = nrec > 0 ? grad_tt_rec_all + (long long)nrec * src0 : nullptr;
  const AdjLayout L = adj_layout(nz, nx, ny, nsrc);
  if (workspace_bytes < L.total) return kWorkspaceTooSmall;
  char* ws = (char*)workspace;
  RevArgs A;
  A.slow = slow;
  A.tt = (double*)(ws + L.tt);
  A.lam = (double*)(ws + L.lam);
  A.contrib = (double*)(ws + L.contrib);
  A.g8 = (double*)(ws + L.g8);
  A.nz = nz;
  A.nx = nx;
  A.ny = ny;
  A.NZ = nz + 1;
  A.NX = nx + 1;
  A.NY = ny + 1;
  A.nodes = (long long)A.NZ * A.NX * A.NY;
  A.nsrc = nsrc;
  A.o = make_ops3(dz, dx, dy);
  const long long N = A.nodes * nsrc;
  A.tape = tape_at(const_cast<void*>(tape), tape_layout(nz, nx, ny, nsrc_tape, nsweep, history),
                   nsweep, history);
  A.tape.code += src0 * nodes * A.tape.E;
  A.tape.hist += src0 * nodes * A.tape.H;
  A.tape.init8 += 8LL * src0;
  A.tape.params += src0;
  A.tape.sn0 = src0 * nodes;
  A.params = A.tape.params;
  double* vzg = (double*)(ws + L.vzg);

  FTEIK_CHECK(cudaMemcpyAsync(A.tt, tt, 8 * (size_t)N, cudaMemcpyDeviceToDevice, st));
  FTEIK_CHECK(cudaMemsetAsync(A.lam, 0, 8 * (size_t)N, st));
  FTEIK_CHECK(cudaMemsetAsync(A.g8, 0, 64 * (size_t)N, st));
  adj_seed_kernel<<<(nsrc + 63) / 64, 64, 0, st>>>(A, ax0, ax1, ax2, sources, receivers, nrec,
                                                   grad_tt_rec, vzg);
  FTEIK_CHECK(cudaGetLastError());
  const int nepochs = 8 * nsweep;
  int* status = (int*)(ws + L.sync);
  if (nepochs > 0) {
    RevSched R;
    R.status = status;
    R.ticket = (unsigned*)(ws + L.sync + 4);
    R.progress = (unsigned*)(ws + L.sync + 8);
    R.PJ = L.PJ;
    R.PK = L.PK;
    R.T = A.NZ + kRevPW + 32 / kRevPW - 2;
    R.nepochs = nepochs;
    const long long chunk = option_value(kOptAdjointChunk);
    R.chunk = chunk > 0 ? (int)chunk : 4;  // 4 measured best on 96x128x128, 64 sources
    R.stride = (unsigned)R.T;
    R.spin_limit = spin_limit > 0 ? spin_limit : (1LL << 25);
    FTEIK_CHECK(
        cudaMemsetAsync(ws + L.sync, 0, 8 + 4 * (size_t)L.PJ * L.PK * nsrc, st));
    // persistent: as many blocks as are resident at once, so every ticket
    // holder runs and each wait is on an item that is already running
    const int threads = kRevWarps * 32;
    const int blocks = resident_blocks((const void*)adj_sweep_kernel<kRevPW>, threads);
    adj_sweep_kernel<kRevPW><<<blocks, threads, 0, st>>>(A, R);
  }
  FTEIK_CHECK(cudaGetLastError());
  adj_initial_kernel<<<(nsrc * 8 + 127) / 128, 128, 0, st>>>(A);
  adj_gather_kernel<<<grid_for((long long)nz * nx * ny, 256), 256, 0, st>>>(A, vzg, accumulate,
                                                                           grad_slow);
  FTEIK_CHECK(cudaGetLastError());
  FTEIK_CHECK(cudaStreamSynchronize(st));
  if (nepochs > 0) {
    int dev_status = 0;
    FTEIK_CHECK(cudaMemcpy(&dev_status, status, sizeof(int), cudaMemcpyDeviceToHost));
    if (dev_status != 0) return dev_status;
  }
  return kOk;
}
