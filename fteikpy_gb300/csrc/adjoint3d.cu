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
// it replaced.  Going back through the sweeps in reverse hyperplane order, a
// node first collects the adjoint its readers of that sweep sent it, then, if
// the sweep changed it, recomputes its operator's partials from the values it
// read (_fteik3d.py:76-159; no saved intermediates), sends the adjoint on to
// those inputs, books the slowness term, and restores its previous value.
// Every transfer is a pull or a per-node accumulation, so the result is the
// same from run to run.
#include <algorithm>
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
  const uint8_t* tcode;  // [nepochs][nsrc][nodes] operator code of each change (255: none)
  const double* told;    // [nepochs][nsrc][nodes] value each change replaced
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

// The distinct cells of the list whose slowness is minimal.  Boundary clamps
// can list a cell twice; that is one cell, not a tie.
__device__ __forceinline__ int min_cells(const double* slow, const int* cells, int n,
                                         int (&out)[4], double& vmin) {
  double bv = __ldg(slow + cells[0]);
  for (int q = 1; q < n; ++q) bv = fmin(bv, __ldg(slow + cells[q]));
  int m = 0;
  for (int q = 0; q < n; ++q) {
    if (__ldg(slow + cells[q]) != bv) continue;
    bool seen = false;
    for (int r = 0; r < m; ++r) seen = seen || out[r] == cells[q];
    if (!seen) out[m++] = cells[q];
  }
  vmin = bv;
  return m;
}

// Partials of the operator that produced t_n (signs az, ax, ay from the
// branch record) with respect to its inputs (slot (bz,bx,by) = input at
// n - (bz*az, bx*ax, by*ay)) and to the slowness it used, evaluated at the
// input values in t.  Recomputed from the traveltimes, _fteik3d.py:76-159.
// The 1D and 2D operators use the minimum slowness of 4 or 2 cells.  Where
// several cells share that minimum the solver has no derivative: lowering one
// of them moves the result, raising it does not.  Each tied cell then gets
// half the partial, the mean of its two one-sided derivatives, which is what
// a central difference on that cell measures.  The cells are returned in
// cells[0..ncell) with the partial ps for each.
__device__ void linearize(int az, int ax, int ay, int i, int j, int k, long long n,
                          const double* t, const double* slow, int nz_, int nx_, int ny_,
                          int NX_, int NY_, const Ops3& o, double (&w)[kSlots], double& ps,
                          int (&cell)[4], int& ncell) {
  struct Dims { int nz, nx, ny, NX, NY; } A{nz_, nx_, ny_, NX_, NY_};
  const long long NXY = (long long)NX_ * NY_;
#pragma unroll
  for (int e = 0; e < kSlots; ++e) w[e] = 0.0;
  ps = 0.0;
  ncell = 0;
  double v;
  const int im = imax(i - 1, 0), ip = imin(i, A.nz - 1);
  const int jm = imax(j - 1, 0), jp = imin(j, A.nx - 1);
  const int km = imax(k - 1, 0), kp = imin(k, A.ny - 1);
  const int i1 = az > 0 ? i - 1 : i, j1 = ax > 0 ? j - 1 : j, k1 = ay > 0 ? k - 1 : k;
#define C(a, b, c) (((a)*A.nx + (b)) * A.ny + (c))
#define T(bz, bx, by) __ldcg(t + n - (long long)(bz) * az * NXY - (long long)(bx) * ax * A.NY - (by) * ay)
  const int nnz = (az != 0) + (ax != 0) + (ay != 0);
  if (nnz == 1) {
    int cells[4];
    if (az != 0) {
      cells[0] = C(i1, jm, km); cells[1] = C(i1, jm, kp); cells[2] = C(i1, jp, km); cells[3] = C(i1, jp, kp);
      w[3] = 1.0;
      ps = o.dz;
    } else if (ax != 0) {
      cells[0] = C(im, j1, km); cells[1] = C(ip, j1, km); cells[2] = C(im, j1, kp); cells[3] = C(ip, j1, kp);
      w[1] = 1.0;
      ps = o.dx;
    } else {
      cells[0] = C(im, jm, k1); cells[1] = C(im, jp, k1); cells[2] = C(ip, jm, k1); cells[3] = C(ip, jp, k1);
      w[0] = 1.0;
      ps = o.dy;
    }
    ncell = min_cells(slow, cells, 4, cell, v);
  } else if (nnz == 2) {
    // plane operators, _fteik3d.py:106-143
    double c1, c2, ta, tb;
    int cells[2], s1, s2, s12;
    if (ay == 0) {  // ZX: inputs tv (slot 3), te (1), tev (5)
      const double tv = T(1, 0, 0), te = T(0, 1, 0), tev = T(1, 1, 0);
      ta = tev + te - tv;
      tb = tev - te + tv;
      c1 = o.dz2i; c2 = o.dx2i;  // num = tb*c1 + ta*c2
      s1 = 3; s2 = 1; s12 = 5;
      cells[0] = C(i1, j1, km); cells[1] = C(i1, j1, kp);
    } else if (ax == 0) {  // ZY: inputs tv (3), tn (0), tnv (4)
      const double tv = T(1, 0, 0), tn = T(0, 0, 1), tnv = T(1, 0, 1);
      ta = tv - tn + tnv;
      tb = tn - tv + tnv;
      c1 = o.dz2i; c2 = o.dy2i;  // num = ta*c1 + tb*c2
      s1 = 3; s2 = 0; s12 = 4;
      cells[0] = C(i1, jm, k1); cells[1] = C(i1, jp, k1);
    } else {  // XY: inputs te (1), tn (0), ten (2)
      const double te = T(0, 1, 0), tn = T(0, 0, 1), ten = T(0, 1, 1);
      ta = te - tn + ten;
      tb = tn - te + ten;
      c1 = o.dx2i; c2 = o.dy2i;  // num = ta*c1 + tb*c2
      s1 = 1; s2 = 0; s12 = 2;
      cells[0] = C(im, j1, k1); cells[1] = C(ip, j1, k1);
    }
    ncell = min_cells(slow, cells, 2, cell, v);
    const double S = c1 + c2, d = ta - tb;
    const double Q = 4.0 * v * v * S - c1 * c2 * d * d;
    const double R = Q > 0.0 ? sqrt(Q) : 0.0;
    const double r = R > 0.0 ? c1 * c2 * d / R : 0.0;
    // partials of t with respect to ta and tb
    double dta, dtb;
    if (ay == 0) {  // num = tb*dz2i + ta*dx2i
      dta = (c2 - r) / S;
      dtb = (c1 + r) / S;
    } else {  // num = ta*c1 + tb*c2
      dta = (c1 - r) / S;
      dtb = (c2 + r) / S;
    }
    // ta = x12 + x2 - x1 (ZX: tev + te - tv) or x1 - x2 + x12 (ZY, XY)
    if (ay == 0) {
      w[s1] = -dta + dtb;  // tv
      w[s2] = dta - dtb;   // te
    } else {
      w[s1] = dta - dtb;   // tv (ZY) / te (XY)
      w[s2] = -dta + dtb;  // tn
    }
    w[s12] = dta + dtb;
    ps = R > 0.0 ? 4.0 * v / R : 0.0;  // dt/dv = (dR/dv) / S, dR/dv = 4 v S / R
  } else {
    // 3D operator, _fteik3d.py:145-159
    const double tv = T(1, 0, 0), te = T(0, 1, 0), tn = T(0, 0, 1), tev = T(1, 1, 0);
    const double ten = T(0, 1, 1), tnv = T(1, 0, 1), tnve = T(1, 1, 1);
    const double ta = te - 0.5 * tn + 0.5 * ten - 0.5 * tv + 0.5 * tev - tnv + tnve;
    const double tb = tv - 0.5 * tn + 0.5 * tnv - 0.5 * te + 0.5 * tev - ten + tnve;
    const double tc = tn - 0.5 * te + 0.5 * ten - 0.5 * tv + 0.5 * tnv - tev + tnve;
    cell[0] = C(i1, j1, k1);
    ncell = 1;
    v = __ldg(slow + cell[0]);
    const double t2 = v * v * o.dsum * 9.0;
    const double t3 = o.dz2dx2 * (ta - tb) * (ta - tb) + o.dz2dy2 * (tb - tc) * (tb - tc) +
                      o.dx2dy2 * (ta - tc) * (ta - tc);
    const double W = t2 > t3 ? sqrt(t2 - t3) : 0.0;
    const double iw = W > 0.0 ? 1.0 / W : 0.0;
    const double dta = (o.dx2i - (o.dz2dx2 * (ta - tb) + o.dx2dy2 * (ta - tc)) * iw) / o.dsum;
    const double dtb = (o.dz2i - (-o.dz2dx2 * (ta - tb) + o.dz2dy2 * (tb - tc)) * iw) / o.dsum;
    const double dtc = (o.dy2i - (-o.dz2dy2 * (tb - tc) - o.dx2dy2 * (ta - tc)) * iw) / o.dsum;
    // d(ta, tb, tc) / d(tv, te, tn, tev, ten, tnv, tnve)
    w[3] = -0.5 * dta + dtb - 0.5 * dtc;        // tv
    w[1] = dta - 0.5 * dtb - 0.5 * dtc;         // te
    w[0] = -0.5 * dta - 0.5 * dtb + dtc;        // tn
    w[5] = 0.5 * dta + 0.5 * dtb - dtc;         // tev
    w[2] = 0.5 * dta - dtb + 0.5 * dtc;         // ten
    w[4] = -dta + 0.5 * dtb + 0.5 * dtc;        // tnv
    w[6] = dta + dtb + dtc;                     // tnve
    ps = 9.0 * v * iw;
  }
  if (ncell > 1) ps *= 0.5;
#undef T
#undef C
}

// Slot of cell (ci, cj, ck) among the 8 cells around node (i, j, k)
// (a = 0 for the cell row max(i-1, 0), 1 for min(i, nz-1); equal rows use 0).
__device__ __forceinline__ int cell_slot(int i, int j, int k, int ci, int cj, int ck) {
  const int a = ci == imax(i - 1, 0) ? 0 : 1;
  const int b = cj == imax(j - 1, 0) ? 0 : 1;
  const int c = ck == imax(k - 1, 0) ? 0 : 1;
  return a * 4 + b * 2 + c;
}

// One node of one sweep, in reverse.  In sweep e (signs sz, sx, sy) the node
// at local coordinates (ii, jj, kk) was updated after every node of a smaller
// ii + jj + kk; going back, its hyperplane runs after the planes above it.
// The node first collects what its readers of this sweep sent it (they lie
// downwind, on planes already done), then, if this sweep changed it,
// linearises the operator at the values it read, sends the adjoint on to its
// inputs, books the slowness term and restores its previous value.  Arrays
// other threads write are read through L2 (ld.global.cg).
__device__ __forceinline__ void reverse_node(const RevArgs& A, int e, int src, int ii, int jj,
                                             int kk) {
  const int dir = e & 7;
  const int sz = dir < 4 ? 1 : -1, sx = (dir & 1) ? -1 : 1, sy = (dir & 2) ? -1 : 1;
  const long long NXY = (long long)A.NX * A.NY;
  const int i = sz > 0 ? ii : A.NZ - 1 - ii;
  const int j = sx > 0 ? jj : A.NX - 1 - jj;
  const int k = sy > 0 ? kk : A.NY - 1 - kk;
  const long long n = (long long)i * NXY + (long long)j * A.NY + k;
  const long long base = (long long)src * A.nodes;
  const long long tbase = ((long long)e * A.nsrc + src) * A.nodes;
  // All reads are issued before any is used, so their latencies overlap.
  const int code = __ldg(A.tcode + tbase + n);
  const double lam0 = __ldcg(A.lam + base + n);
  long long m[kSlots];
  int dcode[kSlots];
#pragma unroll
  for (int slot = 0; slot < kSlots; ++slot) {
    const int bz = (slot + 1) >> 2, bx = ((slot + 1) >> 1) & 1, by = (slot + 1) & 1;
    const int mi = i + bz * sz, mj = j + bx * sx, mk = k + by * sy;
    const bool in = mi >= 0 && mi < A.NZ && mj >= 0 && mj < A.NX && mk >= 0 && mk < A.NY;
    m[slot] = (long long)mi * NXY + (long long)mj * A.NY + mk;
    dcode[slot] = in ? (int)__ldg(A.tcode + tbase + m[slot]) : 255;
  }
  double part[kSlots];
#pragma unroll
  for (int slot = 0; slot < kSlots; ++slot) {
    const int bz = (slot + 1) >> 2, bx = ((slot + 1) >> 1) & 1, by = (slot + 1) & 1;
    part[slot] = 0.0;
    if (dcode[slot] == 255) continue;
    int az, ax, ay;
    decode(dcode[slot], az, ax, ay);
    if ((bz && !az) || (bx && !ax) || (by && !ay)) continue;
    part[slot] = __ldcg(A.contrib + (base + m[slot]) * kSlots + slot);
  }
  double lam = lam0;
  bool pulled = false;
#pragma unroll
  for (int slot = 0; slot < kSlots; ++slot) {
    if (dcode[slot] == 255) continue;
    lam += part[slot];
    pulled = true;
  }
  if (code == 255) {
    if (pulled) A.lam[base + n] = lam;
    return;
  }
  int az, ax, ay;
  decode(code, az, ax, ay);
  double w[kSlots], ps;
  int cell[4], ncell;
  linearize(az, ax, ay, i, j, k, n, A.tt + base, A.slow, A.nz, A.nx, A.ny, A.NX, A.NY, A.o, w, ps,
            cell, ncell);
  double* c = A.contrib + (base + n) * kSlots;
#pragma unroll
  for (int slot = 0; slot < kSlots; ++slot) c[slot] = lam * w[slot];
  for (int q = 0; q < ncell; ++q) {
    const int ci = cell[q] / (A.nx * A.ny), cj = (cell[q] / A.ny) % A.nx, ck = cell[q] % A.ny;
    double* g = A.g8 + (base + n) * 8 + cell_slot(i, j, k, ci, cj, ck);
    *g = __ldcg(g) + lam * ps;
  }
  A.lam[base + n] = 0.0;
  A.tt[base + n] = __ldg(A.told + tbase + n);
}

// Barrier of the `nblocks` blocks of one group of a cooperative launch
// (every block is resident). The last block to arrive resets the count and
// publishes a new generation; the others poll the generation at most
// spin_limit times, then flag FTEIK_DEVICE_WAIT_TIMEOUT and return false, as
// they do once any block has flagged a failure.
struct GridBarrier {
  unsigned count, gen;
};

__device__ bool group_barrier(GridBarrier* b, unsigned nblocks, int* status,
                              long long spin_limit) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g = ld_acquire(&b->gen);
    __threadfence();
    if (atomicAdd(&b->count, 1u) + 1u == nblocks) {
      b->count = 0;
      __threadfence();
      st_release(&b->gen, g + 1u);
    } else {
      for (long long it = 0; ld_acquire(&b->gen) == g; ++it) {
        if (it >= spin_limit) {
          atomicCAS(status, 0, (int)kDeviceWaitTimeout);
          ok = 0;
          break;
        }
        if ((it & 15) == 15 && *((volatile int*)status) != 0) {
          ok = 0;
          break;
        }
        if (it >= 64) __nanosleep(64);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Every sweep in reverse, hyperplane by hyperplane, in one cooperative
// launch. Sources are independent, so the blocks form `ngroups` groups that
// each take every ngroups-th source and meet only at their own barrier: per
// plane, the group's threads share out the plane's nodes (per column jj, the
// band of kk whose ii = h - jj - kk lies in the grid), then wait for each
// other before the plane below.
__global__ void __launch_bounds__(256)
    adj_reverse_kernel(const RevArgs A, int nepochs, int ngroups, GridBarrier* bars,
                       int* status, long long spin_limit) {
  const int hmax = A.NZ + A.NX + A.NY - 3;
  const int g = (int)((long long)blockIdx.x * ngroups / gridDim.x);
  const int b0 = (int)(((long long)g * gridDim.x + ngroups - 1) / ngroups);
  const int b1 = (int)(((long long)(g + 1) * gridDim.x + ngroups - 1) / ngroups);
  const unsigned nb = (unsigned)(b1 - b0);
  const long long tid = (long long)(blockIdx.x - b0) * blockDim.x + threadIdx.x;
  const long long nthreads = (long long)nb * blockDim.x;
  GridBarrier* bar = bars + g;
  for (int src = g; src < A.nsrc; src += ngroups) {
    for (int e = nepochs - 1; e >= 0; --e) {
      for (int h = hmax; h >= 0; --h) {
        const int jlo = imax(0, h - (A.NZ - 1) - (A.NY - 1)), jhi = imin(A.NX - 1, h);
        const int W = imin(imin(A.NZ, A.NY), h + 1);
        const long long total = (long long)(jhi - jlo + 1) * W;
        for (long long q = tid; q < total; q += nthreads) {
          const int jj = jlo + (int)(q / W);
          const int kk = imax(0, h - jj - (A.NZ - 1)) + (int)(q % W);
          if (kk > imin(A.NY - 1, h - jj)) continue;
          reverse_node(A, e, src, h - jj - kk, jj, kk);
        }
        if (!group_barrier(bar, nb, status, spin_limit)) return;
      }
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
// sources in order, plus the receivers' source-cell terms.
__global__ void adj_gather_kernel(const RevArgs A, const double* vzg, double* grad_slow) {
  const long long ncell = (long long)A.nz * A.nx * A.ny;
  const long long NXY = (long long)A.NX * A.NY;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(c / ((long long)A.nx * A.ny));
    const int cj = (int)((c / A.ny) % A.nx), ck = (int)(c % A.ny);
    double g = 0.0;
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
};

static AdjLayout adj_layout(int nz, int nx, int ny, int nsrc) {
  const size_t N = (size_t)(nz + 1) * (nx + 1) * (ny + 1) * nsrc;
  AdjLayout L;
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
  L.sync = off;  // int status, then one barrier per source group
  off = align_up(off + 8 + 8 * (size_t)nsrc);
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
                               double dy, int nsrc, int nsweep, const double* tt,
                               const void* solve_workspace, size_t solve_workspace_bytes,
                               const void* tape, size_t tape_bytes, const double* ax0,
                               const double* ax1, const double* ax2, const double* sources,
                               const double* receivers, int nrec, const double* grad_tt_rec,
                               double* grad_slow, void* workspace, size_t workspace_bytes,
                               long long spin_limit, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nz < 2 || nx < 2 || ny < 2 || nsrc < 1 || nsweep < 0 || nrec < 0 || !slow || !tt ||
      !solve_workspace || !tape || !ax0 || !ax1 || !ax2 || !sources ||
      (nrec > 0 && (!receivers || !grad_tt_rec)) || !grad_slow || !workspace)
    return kInvalidArgument;
  const Layout3 S = layout3(nz, nx, ny, nsrc, 2);
  if (solve_workspace_bytes < S.total) return kWorkspaceTooSmall;
  if (tape_bytes < fteik3d_tape_bytes(nz, nx, ny, nsrc, nsweep)) return kWorkspaceTooSmall;
  const AdjLayout L = adj_layout(nz, nx, ny, nsrc);
  if (workspace_bytes < L.total) return kWorkspaceTooSmall;
  const char* sw = (const char*)solve_workspace;
  char* ws = (char*)workspace;
  RevArgs A;
  A.slow = slow;
  A.params = (const Source3*)(sw + S.params);
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
  const size_t ntape = (size_t)N * 8 * (size_t)nsweep;
  A.tcode = (const uint8_t*)tape;
  A.told = (const double*)((const char*)tape + align_up(ntape));
  double* vzg = (double*)(ws + L.vzg);

  FTEIK_CHECK(cudaMemcpyAsync(A.tt, tt, 8 * (size_t)N, cudaMemcpyDeviceToDevice, st));
  FTEIK_CHECK(cudaMemsetAsync(A.lam, 0, 8 * (size_t)N, st));
  FTEIK_CHECK(cudaMemsetAsync(A.g8, 0, 64 * (size_t)N, st));
  adj_seed_kernel<<<(nsrc + 63) / 64, 64, 0, st>>>(A, ax0, ax1, ax2, sources, receivers, nrec,
                                                   grad_tt_rec, vzg);
  FTEIK_CHECK(cudaGetLastError());
  int nepochs = 8 * nsweep;
  if (nepochs > 0) {
    int* status = (int*)(ws + L.sync);
    GridBarrier* bars = (GridBarrier*)(ws + L.sync + 8);
    FTEIK_CHECK(cudaMemsetAsync(ws + L.sync, 0, 8 + sizeof(GridBarrier) * (size_t)nsrc, st));
    const void* kern = (const void*)adj_reverse_kernel;
    const int blocks = resident_blocks(kern, 256);
    // one group of blocks per source while there are blocks enough
    int ngroups = std::min(nsrc, blocks);
    long long limit = spin_limit > 0 ? spin_limit : (1LL << 25);
    void* args[] = {(void*)&A,    (void*)&nepochs, (void*)&ngroups,
                    (void*)&bars, (void*)&status,  (void*)&limit};
    FTEIK_CHECK(cudaLaunchCooperativeKernel(kern, dim3(blocks), dim3(256), args, 0, st));
  }
  FTEIK_CHECK(cudaGetLastError());
  adj_initial_kernel<<<(nsrc * 8 + 127) / 128, 128, 0, st>>>(A);
  adj_gather_kernel<<<grid_for((long long)nz * nx * ny, 256), 256, 0, st>>>(A, vzg, grad_slow);
  FTEIK_CHECK(cudaGetLastError());
  FTEIK_CHECK(cudaStreamSynchronize(st));
  if (nepochs > 0) {
    int dev_status = 0;
    FTEIK_CHECK(cudaMemcpy(&dev_status, ws + L.sync, sizeof(int), cudaMemcpyDeviceToHost));
    if (dev_status != 0) return dev_status;
  }
  return kOk;
}
