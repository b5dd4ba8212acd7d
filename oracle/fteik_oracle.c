/*
 * CPU restatement of fteikpy's traveltime path: the oracle.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker for the CUDA kernels of
 * fteikpy_gb300 and the CPU baseline timed beside them; the product never
 * links, loads or calls it. Only tests/, __graft_entry__.smoke() and the CPU
 * legs of bench.py use it.
 *
 * It restates, function by function, the numba kernels of fteikpy v2.4.0
 * (file:line cited at each function) with the floating-point semantics the
 * reference's numba build resolves to: `x ** 2.0` is `x * x`, `x ** 0.5` is a
 * correctly rounded `sqrt`, divisions are IEEE divisions, no fused
 * multiply-add (compile with -ffp-contract=off), and Python's `min`/`max`
 * built-ins keep the first argument unless a later one compares strictly
 * smaller/larger.  Division by zero follows IEEE (the reference in its
 * pure-Python mode follows numpy scalars, which do the same).
 *
 * Parity is pinned against the reference itself: tests/golden/*.npz were
 * produced by importing the reference (tests/golden/make_golden.py), and the
 * reference's own golden sums (tests/test_eikonal*.py and friends) are checked
 * in tests/test_oracle.py.
 *
 * Array layouts are the reference's C-order layouts: velocity/slowness cells
 * [nz][nx](ny), traveltime nodes [nz+1][nx+1](ny+1), gradient nodes
 * [..][ndim].  All sizes passed in are CELL counts unless named otherwise.
 *
 * Build: see oracle/build_oracle.sh (gcc -O2 -ffp-contract=off -fopenmp).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define BIG 1.0e5
#define EPS 1.0e-15
#define EPSIN 5

/* Status codes shared with the product C-ABI. */
#define ST_OK 0
#define ST_SOURCE_OOB 1
#define ST_ENDPOINT_OOB 2
#define ST_MAX_STEP 3

/* Python min/max built-ins: keep the running value unless strictly beaten. */
static inline double pmin2(double a, double b) { return (b < a) ? b : a; }
static inline double pmax2(double a, double b) { return (b > a) ? b : a; }
static inline double pmin3(double a, double b, double c) { return pmin2(pmin2(a, b), c); }
static inline double pmin4(double a, double b, double c, double d) {
  return pmin2(pmin2(pmin2(a, b), c), d);
}
static inline double pmax3(double a, double b, double c) { return pmax2(pmax2(a, b), c); }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

/* np.searchsorted(a, v, side="right") - 1 for an ascending array. */
static int search_right_m1(const double* a, int n, double v) {
  int lo = 0, hi = n; /* first index with a[idx] > v */
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] <= v)
      lo = mid + 1;
    else
      hi = mid;
  }
  /* numpy places NaN after every number */
  if (v != v) lo = n;
  return lo - 1;
}

/* ------------------------------------------------------------------------ */
/* 3D solver: fteikpy/_fteik/_fteik3d.py                                    */
/* ------------------------------------------------------------------------ */

/* t_ana, _fteik3d.py:10-17 */
static double t_ana3(int i, int j, int k, double dz, double dx, double dy, double zsa,
                     double xsa, double ysa, double vzero) {
  double a = dz * ((double)i - zsa);
  double b = dx * ((double)j - xsa);
  double c = dy * ((double)k - ysa);
  return vzero * sqrt(a * a + b * b + c * c);
}

/* t_anad, _fteik3d.py:20-35 */
static double t_anad3(int i, int j, int k, double dz, double dx, double dy, double zsa,
                      double xsa, double ysa, double vzero, double* tzc, double* txc,
                      double* tyc) {
  double t = t_ana3(i, j, k, dz, dx, dy, zsa, xsa, ysa, vzero);
  if (t > 0.0) {
    double tmp = vzero * vzero / t;
    *tzc = ((double)i - zsa) * dz * tmp;
    *txc = ((double)j - xsa) * dx * tmp;
    *tyc = ((double)k - ysa) * dy * tmp;
  } else {
    *tzc = 0.0;
    *txc = 0.0;
    *tyc = 0.0;
  }
  return t;
}

typedef struct {
  double dz, dx, dy, dz2i, dx2i, dy2i, dz2dx2, dz2dy2, dx2dy2, dsum;
} dargs3_t;

/* Optional instrumentation of the 3D node updates, for choosing the cells of
 * the adjoint's finite-difference check (not part of the reference): per
 * solve, a digest of every discrete decision (which candidate each update
 * keeps, and which slowness cells attain the minimum its operator takes), and
 * a flag on every cell that a kept operator's minimum takes within a relative
 * `margin` of another cell (a tie: there the solve has only one-sided
 * derivatives in that cell).  Set per thread while a solve runs. */
typedef struct {
  unsigned long long digest;
  uint8_t* tied; /* [cells], or NULL */
  double margin;
} probe3_t;
static _Thread_local probe3_t* g_probe3 = NULL;

static void probe3_update(probe3_t* p, const double* slow, int winner, int i1, int j1, int k1,
                          int im, int ip, int jm, int jp, int km, int kp, int nx, int ny) {
  /* the cells of the winner's slowness minimum (_fteik3d.py:78-101,108,121,134,148) */
  int c[4][3], nc = 0;
#define PUT(a, b, d) (c[nc][0] = (a), c[nc][1] = (b), c[nc][2] = (d), ++nc)
  switch (winner) {
    case 1: PUT(i1, jm, km); PUT(i1, jm, kp); PUT(i1, jp, km); PUT(i1, jp, kp); break;
    case 2: PUT(im, j1, km); PUT(ip, j1, km); PUT(im, j1, kp); PUT(ip, j1, kp); break;
    case 3: PUT(im, jm, k1); PUT(im, jp, k1); PUT(ip, jm, k1); PUT(ip, jp, k1); break;
    case 4: PUT(i1, j1, km); PUT(i1, j1, kp); break;
    case 5: PUT(i1, jm, k1); PUT(i1, jp, k1); break;
    case 6: PUT(im, j1, k1); PUT(ip, j1, k1); break;
    case 7: PUT(i1, j1, k1); break;
    default: break;
  }
#undef PUT
  const long SXY = (long)(nx - 1) * (ny - 1);
  const int SY = ny - 1;
  long idx[4];
  double v[4], vmin = 0.0;
  for (int q = 0; q < nc; ++q) {
    idx[q] = (long)c[q][0] * SXY + (long)c[q][1] * SY + c[q][2];
    v[q] = slow[idx[q]];
    vmin = (q == 0 || v[q] < vmin) ? v[q] : vmin;
  }
  unsigned mask = 0;
  int near = 0;
  for (int q = 0; q < nc; ++q) {
    if (v[q] == vmin) mask |= 1u << q;
    int dup = 0;
    for (int r = 0; r < q; ++r) dup |= idx[r] == idx[q];
    if (!dup && v[q] <= vmin * (1.0 + p->margin)) ++near;
  }
  p->digest = (p->digest ^ (unsigned long long)(winner | (mask << 4))) * 0x100000001b3ull;
  if (near > 1 && p->tied)
    for (int q = 0; q < nc; ++q)
      if (v[q] <= vmin * (1.0 + p->margin)) {
#pragma omp atomic write
        p->tied[idx[q]] = 1;
      }
}

/* sweep (one node update), _fteik3d.py:38-200.  nz, nx, ny are NODE counts. */
static void sweep3_node(double* tt, int8_t* sgn, const double* slow, const dargs3_t* d, int i,
                        int j, int k, int sgnvz, int sgnvx, int sgnvy, int sgntz, int sgntx,
                        int sgnty, int nz, int nx, int ny, int grad) {
  const long NXY = (long)nx * ny;
  const long SXY = (long)(nx - 1) * (ny - 1);
  const int SY = ny - 1;
#define TT(a, b, c) tt[(long)(a)*NXY + (long)(b)*ny + (c)]
#define SL(a, b, c) slow[(long)(a)*SXY + (long)(b)*SY + (c)]
  int i1 = i - sgnvz, j1 = j - sgnvx, k1 = k - sgnvy;
  double tv = TT(i - sgntz, j, k);
  double te = TT(i, j - sgntx, k);
  double tn = TT(i, j, k - sgnty);
  double tev = TT(i - sgntz, j - sgntx, k);
  double ten = TT(i, j - sgntx, k - sgnty);
  double tnv = TT(i - sgntz, j, k - sgnty);
  double tnve = TT(i - sgntz, j - sgntx, k - sgnty);
  int im = imax(i - 1, 0), ip = imin(i, nz - 2);
  int jm = imax(j - 1, 0), jp = imin(j, nx - 2);
  int km = imax(k - 1, 0), kp = imin(k, ny - 2);

  /* 1D operators, _fteik3d.py:76-104 */
  double vref = pmin4(SL(i1, jm, km), SL(i1, jm, kp), SL(i1, jp, km), SL(i1, jp, kp));
  double t1d1 = tv + d->dz * vref;
  vref = pmin4(SL(im, j1, km), SL(ip, j1, km), SL(im, j1, kp), SL(ip, j1, kp));
  double t1d2 = te + d->dx * vref;
  vref = pmin4(SL(im, jm, k1), SL(im, jp, k1), SL(ip, jm, k1), SL(ip, jp, k1));
  double t1d3 = tn + d->dy * vref;
  double t1d = pmin3(t1d1, t1d2, t1d3);

  /* 2D operators, _fteik3d.py:106-143 */
  double t2d1 = BIG;
  vref = pmin2(SL(i1, j1, km), SL(i1, j1, kp));
  if (tv < te + d->dx * vref && te < tv + d->dz * vref) {
    double ta = tev + te - tv;
    double tb = tev - te + tv;
    double dd = ta - tb;
    t2d1 = ((tb * d->dz2i + ta * d->dx2i) +
            sqrt(4.0 * (vref * vref) * (d->dz2i + d->dx2i) - d->dz2i * d->dx2i * (dd * dd))) /
           (d->dz2i + d->dx2i);
  }
  double t2d2 = BIG;
  vref = pmin2(SL(i1, jm, k1), SL(i1, jp, k1));
  if (tv < tn + d->dy * vref && tn < tv + d->dz * vref) {
    double ta = tv - tn + tnv;
    double tb = tn - tv + tnv;
    double dd = ta - tb;
    t2d2 = ((ta * d->dz2i + tb * d->dy2i) +
            sqrt(4.0 * (vref * vref) * (d->dz2i + d->dy2i) - d->dz2i * d->dy2i * (dd * dd))) /
           (d->dz2i + d->dy2i);
  }
  double t2d3 = BIG;
  vref = pmin2(SL(im, j1, k1), SL(ip, j1, k1));
  if (te < tn + d->dy * vref && tn < te + d->dx * vref) {
    double ta = te - tn + ten;
    double tb = tn - te + ten;
    double dd = ta - tb;
    t2d3 = ((ta * d->dx2i + tb * d->dy2i) +
            sqrt(4.0 * (vref * vref) * (d->dx2i + d->dy2i) - d->dx2i * d->dy2i * (dd * dd))) /
           (d->dx2i + d->dy2i);
  }
  double t2d = pmin3(t2d1, t2d2, t2d3);

  /* 3D operator, _fteik3d.py:145-159 */
  double t3d = BIG;
  if (pmin2(t1d, t2d) > pmax3(tv, te, tn)) {
    vref = SL(i1, j1, k1);
    double ta = te - 0.5 * tn + 0.5 * ten - 0.5 * tv + 0.5 * tev - tnv + tnve;
    double tb = tv - 0.5 * tn + 0.5 * tnv - 0.5 * te + 0.5 * tev - ten + tnve;
    double tc = tn - 0.5 * te + 0.5 * ten - 0.5 * tv + 0.5 * tnv - tev + tnve;
    double t2 = vref * vref * d->dsum * 9.0;
    double ab = ta - tb, bc = tb - tc, ac = ta - tc;
    double t3 = d->dz2dx2 * (ab * ab);
    t3 += d->dz2dy2 * (bc * bc);
    t3 += d->dx2dy2 * (ac * ac);
    if (t2 >= t3) {
      double t1 = tb * d->dz2i + ta * d->dx2i + tc * d->dy2i;
      t3d = (t1 + sqrt(t2 - t3)) / d->dsum;
    }
  }

  /* _fteik3d.py:161-200 */
  double t0 = TT(i, j, k);
  double tnew = pmin4(t0, t1d, t2d, t3d);
  TT(i, j, k) = tnew;
  if (g_probe3) {
    int w = tnew == t0 ? 0 : tnew == t1d1 ? 1 : tnew == t1d2 ? 2 : tnew == t1d3 ? 3
            : tnew == t2d1 ? 4 : tnew == t2d2 ? 5 : tnew == t2d3 ? 6 : 7;
    probe3_update(g_probe3, slow, w, i1, j1, k1, im, ip, jm, jp, km, kp, nx, ny);
  }
  if (grad && tnew != t0) {
    long n = ((long)i * NXY + (long)j * ny + k) * 3;
    int a, b, c;
    if (tnew == t1d1) {
      a = sgntz; b = 0; c = 0;
    } else if (tnew == t1d2) {
      a = 0; b = sgntx; c = 0;
    } else if (tnew == t1d3) {
      a = 0; b = 0; c = sgnty;
    } else if (tnew == t2d1) {
      a = sgntz; b = sgntx; c = 0;
    } else if (tnew == t2d2) {
      a = sgntz; b = 0; c = sgnty;
    } else if (tnew == t2d3) {
      a = 0; b = sgntx; c = sgnty;
    } else {
      a = sgntz; b = sgntx; c = sgnty;
    }
    sgn[n] = (int8_t)a;
    sgn[n + 1] = (int8_t)b;
    sgn[n + 2] = (int8_t)c;
  }
#undef TT
#undef SL
}

/* sweep3d, _fteik3d.py:203-391: the 8 directional sweeps in reference order. */
static void sweep3d(double* tt, int8_t* sgn, const double* slow, double dz, double dx, double dy,
                    int nz, int nx, int ny, int grad) {
  dargs3_t d;
  d.dz = dz; d.dx = dx; d.dy = dy;
  d.dz2i = 1.0 / dz / dz;
  d.dx2i = 1.0 / dx / dx;
  d.dy2i = 1.0 / dy / dy;
  d.dz2dx2 = d.dz2i * d.dx2i;
  d.dz2dy2 = d.dz2i * d.dy2i;
  d.dx2dy2 = d.dx2i * d.dy2i;
  d.dsum = d.dz2i + d.dx2i + d.dy2i;
  /* (sgntz, sgntx, sgnty) of the 8 sweeps, in order */
  static const int S[8][3] = {{1, 1, 1},   {1, -1, 1},  {1, 1, -1},  {1, -1, -1},
                              {-1, 1, 1},  {-1, -1, 1}, {-1, 1, -1}, {-1, -1, -1}};
  for (int s = 0; s < 8; ++s) {
    int tz = S[s][0], tx = S[s][1], ty = S[s][2];
    int vz = tz > 0, vx = tx > 0, vy = ty > 0;
    int k0 = ty > 0 ? 1 : ny - 2, k1 = ty > 0 ? ny : -1;
    int j0 = tx > 0 ? 1 : nx - 2, j1 = tx > 0 ? nx : -1;
    int i0 = tz > 0 ? 1 : nz - 2, i1 = tz > 0 ? nz : -1;
    for (int k = k0; k != k1; k += ty)
      for (int j = j0; j != j1; j += tx)
        for (int i = i0; i != i1; i += tz)
          sweep3_node(tt, sgn, slow, &d, i, j, k, vz, vx, vy, tz, tx, ty, nz, nx, ny, grad);
  }
}

/* fteik3d, _fteik3d.py:394-490.  slow is [nz][nx][ny] cells; tt is
 * [nz+1][nx+1][ny+1]; ttgrad (may be NULL when grad == 0) is [...][3]. */
static int8_t* g_sgn_out = NULL; /* when set, receives the branch record of the next solve */

int oracle_fteik3d(const double* slow, int nz, int nx, int ny, double dz, double dx, double dy,
                   double zsrc, double xsrc, double ysrc, int nsweep, int grad, double* tt,
                   double* ttgrad, double* vzero_out) {
  int condz = 0.0 <= zsrc && zsrc <= dz * nz;
  int condx = 0.0 <= xsrc && xsrc <= dx * nx;
  int condy = 0.0 <= ysrc && ysrc <= dy * ny;
  if (!(condz && condx && condy)) return ST_SOURCE_OOB;

  double zsa = zsrc / dz, xsa = xsrc / dx, ysa = ysrc / dy;
  zsa = zsa >= nz ? zsa - EPS : zsa;
  xsa = xsa >= nx ? xsa - EPS : xsa;
  ysa = ysa >= ny ? ysa - EPS : ysa;
  int zsi = imin((int)zsa, nz - 1);
  int xsi = imin((int)xsa, nx - 1);
  int ysi = imin((int)ysa, ny - 1);
  double vzero = slow[((long)zsi * nx + xsi) * ny + ysi];

  int NZ = nz + 1, NX = nx + 1, NY = ny + 1;
  long nn = (long)NZ * NX * NY;
  for (long n = 0; n < nn; ++n) tt[n] = BIG;
  int8_t* sgn = NULL;
  if (grad) {
    sgn = (int8_t*)calloc((size_t)nn * 3, 1);
    memset(ttgrad, 0, sizeof(double) * (size_t)nn * 3);
  }
  static const int OFF[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  for (int q = 0; q < 8; ++q) {
    int i = zsi + OFF[q][0], j = xsi + OFF[q][1], k = ysi + OFF[q][2];
    double tzc, txc, tyc;
    long n = ((long)i * NX + j) * NY + k;
    tt[n] = t_anad3(i, j, k, dz, dx, dy, zsa, xsa, ysa, vzero, &tzc, &txc, &tyc);
    if (grad) {
      ttgrad[n * 3] = tzc;
      ttgrad[n * 3 + 1] = txc;
      ttgrad[n * 3 + 2] = tyc;
    }
  }
  for (int s = 0; s < nsweep; ++s) sweep3d(tt, sgn, slow, dz, dx, dy, NZ, NX, NY, grad);

  if (grad) { /* _fteik3d.py:464-488 */
    for (int i = 0; i < NZ; ++i)
      for (int j = 0; j < NX; ++j)
        for (int k = 0; k < NY; ++k) {
          long n = ((long)i * NX + j) * NY + k;
          double* g = ttgrad + n * 3;
          int sz = sgn[n * 3], sx = sgn[n * 3 + 1], sy = sgn[n * 3 + 2];
          if (sz != 0) g[0] = (double)sz * (tt[n] - tt[n - (long)sz * NX * NY]) / dz;
          if (sx != 0) g[1] = (double)sx * (tt[n] - tt[n - (long)sx * NY]) / dx;
          if (sy != 0) g[2] = (double)sy * (tt[n] - tt[n - sy]) / dy;
          double gn = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
          if (gn > 0.0) {
            g[0] /= gn;
            g[1] /= gn;
            g[2] /= gn;
          }
        }
    if (g_sgn_out) memcpy(g_sgn_out, sgn, (size_t)nn * 3);
    free(sgn);
  }
  *vzero_out = vzero;
  return ST_OK;
}

/* One solve (with gradients) that also returns the branch record, the
 * reference's ttsgn (_fteik3d.py:431-437), as int8 [nodes][3]. */
int oracle_fteik3d_record(const double* slow, int nz, int nx, int ny, double dz, double dx,
                          double dy, double zsrc, double xsrc, double ysrc, int nsweep,
                          double* tt, double* ttgrad, double* vzero, int8_t* sgn) {
  g_sgn_out = sgn;
  int st = oracle_fteik3d(slow, nz, nx, ny, dz, dx, dy, zsrc, xsrc, ysrc, nsweep, 1, tt, ttgrad,
                          vzero);
  g_sgn_out = NULL;
  return st;
}

/* fteik3d_vectorized, _fteik3d.py:493-513: one solve per source, in
 * parallel over sources.  tt is [nsrc][nodes], ttgrad [nsrc][nodes][3]. */
int oracle_fteik3d_many(const double* slow, int nz, int nx, int ny, double dz, double dx,
                        double dy, const double* src, int nsrc, int nsweep, int grad, double* tt,
                        double* ttgrad, double* vzero, int nthreads) {
  long nn = (long)(nz + 1) * (nx + 1) * (ny + 1);
  int status = ST_OK;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) if (nthreads > 1)
  for (int s = 0; s < nsrc; ++s) {
    int st = oracle_fteik3d(slow, nz, nx, ny, dz, dx, dy, src[3 * s], src[3 * s + 1],
                            src[3 * s + 2], nsweep, grad, tt + s * nn,
                            grad ? ttgrad + s * nn * 3 : NULL, vzero + s);
    if (st != ST_OK) {
#pragma omp critical
      status = st;
    }
  }
  return status;
}

/* oracle_fteik3d_many with the instrumentation above: digests[nsrc] of each
 * solve's decisions, and tied[cells] set on every cell that some source's
 * kept operator takes within `margin` of a tie (NULL: not wanted). */
int oracle_fteik3d_probe(const double* slow, int nz, int nx, int ny, double dz, double dx,
                         double dy, const double* src, int nsrc, int nsweep, double margin,
                         double* tt, double* vzero, unsigned long long* digests, uint8_t* tied,
                         int nthreads) {
  long nn = (long)(nz + 1) * (nx + 1) * (ny + 1);
  int status = ST_OK;
  if (tied) memset(tied, 0, (size_t)nz * nx * ny);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) if (nthreads > 1)
  for (int s = 0; s < nsrc; ++s) {
    probe3_t p = {0xcbf29ce484222325ull, tied, margin};
    g_probe3 = &p;
    int st = oracle_fteik3d(slow, nz, nx, ny, dz, dx, dy, src[3 * s], src[3 * s + 1],
                            src[3 * s + 2], nsweep, 0, tt + s * nn, NULL, vzero + s);
    g_probe3 = NULL;
    digests[s] = p.digest;
    if (st != ST_OK) {
#pragma omp critical
      status = st;
    }
  }
  return status;
}

/* ------------------------------------------------------------------------ */
/* 2D solver: fteikpy/_fteik/_fteik2d.py                                    */
/* ------------------------------------------------------------------------ */

/* t_ana, _fteik2d.py:11-14 */
static double t_ana2(int i, int j, double dz, double dx, double zsa, double xsa, double vzero) {
  double a = dz * ((double)i - zsa);
  double b = dx * ((double)j - xsa);
  return vzero * sqrt(a * a + b * b);
}

/* t_anad, _fteik2d.py:17-30 */
static double t_anad2(int i, int j, double dz, double dx, double zsa, double xsa, double vzero,
                      double* tzc, double* txc) {
  double t = t_ana2(i, j, dz, dx, zsa, xsa, vzero);
  if (t > 0.0) {
    double tmp = vzero * vzero / t;
    *tzc = ((double)i - zsa) * dz * tmp;
    *txc = ((double)j - xsa) * dx * tmp;
  } else {
    *tzc = 0.0;
    *txc = 0.0;
  }
  return t;
}

/* delta, _fteik2d.py:33-67 */
static double delta2(double t1, double tauv, double taue, double tauev, double t0c, double tzc,
                     double txc, double dzi, double dxi, double dz2i, double dx2i, double vzero,
                     double vref, int sgntz, int sgntx) {
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

typedef struct {
  double dz, dx, dzi, dxi, dz2i, dx2i;
  double zsi, xsi, zsa, xsa, vzero;
} dargs2_t;

/* sweep (one node update), _fteik2d.py:70-187.  nz, nx are NODE counts. */
static void sweep2_node(double* tt, int8_t* sgn, const double* slow, const dargs2_t* d, int i,
                        int j, int sgnvz, int sgnvx, int sgntz, int sgntx, int nz, int nx,
                        int grad) {
#define TT(a, b) tt[(long)(a)*nx + (b)]
#define SL(a, b) slow[(long)(a) * (nx - 1) + (b)]
  int i1 = i - sgnvz, j1 = j - sgnvx;
  double tv = TT(i - sgntz, j);
  double te = TT(i, j - sgntx);
  double tev = TT(i - sgntz, j - sgntx);
  double dz = d->dz, dx = d->dx, dz2i = d->dz2i, dx2i = d->dx2i;

  double vref = pmin2(SL(i1, imax(j - 1, 0)), SL(i1, imin(j, nx - 2)));
  double t1d1 = tv + dz * vref;
  vref = pmin2(SL(imax(i - 1, 0), j1), SL(imin(i, nz - 2), j1));
  double t1d2 = te + dx * vref;
  double t1d = pmin2(t1d1, t1d2);

  double t2d = BIG;
  vref = SL(i1, j1);
  if (fabs((double)i - d->zsi) > EPSIN || fabs((double)j - d->xsi) > EPSIN) {
    if (tv <= te + dx * vref && te <= tv + dz * vref && te >= tev && tv >= tev) {
      double ta = tev + te - tv;
      double tb = tev - te + tv;
      double dd = ta - tb;
      t2d = ((tb * dz2i + ta * dx2i) +
             sqrt(4.0 * (vref * vref) * (dz2i + dx2i) - dz2i * dx2i * (dd * dd))) /
            (dz2i + dx2i);
    } else if (te - tev <= (dz * dz) * vref / sqrt(dx * dx + dz * dz) && te - tev > 0.0) {
      double q = (te - tev) / dz;
      t2d = te + dx * sqrt(vref * vref - q * q);
    } else if (tv - tev <= (dx * dx) * vref / sqrt(dx * dx + dz * dz) && tv - tev > 0.0) {
      double q = (tv - tev) / dx;
      t2d = tv + dz * sqrt(vref * vref - q * q);
    }
  } else {
    if (tv < te + dx * vref && te < tv + dz * vref && te >= tev && tv >= tev) {
      double tzc, txc;
      double t0c = t_anad2(i, j, dz, dx, d->zsa, d->xsa, d->vzero, &tzc, &txc);
      double tauv = tv - t_ana2(i - sgntz, j, dz, dx, d->zsa, d->xsa, d->vzero);
      double taue = te - t_ana2(i, j - sgntx, dz, dx, d->zsa, d->xsa, d->vzero);
      double tauev = tev - t_ana2(i - sgntz, j - sgntx, dz, dx, d->zsa, d->xsa, d->vzero);
      t2d = delta2(t2d, tauv, taue, tauev, t0c, tzc, txc, d->dzi, d->dxi, dz2i, dx2i, d->vzero,
                   vref, sgntz, sgntx);
      if (t2d < tv || t2d < te) t2d = BIG;
    }
  }
  double t0 = TT(i, j);
  double tnew = pmin3(t0, t1d, t2d);
  TT(i, j) = tnew;
  if (grad && tnew != t0) {
    long n = ((long)i * nx + j) * 2;
    if (tnew == t1d1) {
      sgn[n] = (int8_t)sgntz; sgn[n + 1] = 0;
    } else if (tnew == t1d2) {
      sgn[n] = 0; sgn[n + 1] = (int8_t)sgntx;
    } else {
      sgn[n] = (int8_t)sgntz; sgn[n + 1] = (int8_t)sgntx;
    }
  }
#undef TT
#undef SL
}

/* sweep2d, _fteik2d.py:190-287: interleaved column sweeps. */
static void sweep2d(double* tt, int8_t* sgn, const double* slow, dargs2_t* d, int nz, int nx,
                    int grad) {
  d->dzi = 1.0 / d->dz;
  d->dxi = 1.0 / d->dx;
  d->dz2i = d->dzi / d->dz;
  d->dx2i = d->dxi / d->dx;
  for (int j = 1; j < nx; ++j) {
    for (int i = 1; i < nz; ++i) sweep2_node(tt, sgn, slow, d, i, j, 1, 1, 1, 1, nz, nx, grad);
    for (int i = nz - 2; i >= 0; --i)
      sweep2_node(tt, sgn, slow, d, i, j, 0, 1, -1, 1, nz, nx, grad);
  }
  for (int j = nx - 2; j >= 0; --j) {
    for (int i = 1; i < nz; ++i) sweep2_node(tt, sgn, slow, d, i, j, 1, 0, 1, -1, nz, nx, grad);
    for (int i = nz - 2; i >= 0; --i)
      sweep2_node(tt, sgn, slow, d, i, j, 0, 0, -1, -1, nz, nx, grad);
  }
}

/* fteik2d, _fteik2d.py:290-641. */
int oracle_fteik2d(const double* slow, int nz, int nx, double dz, double dx, double zsrc,
                   double xsrc, int nsweep, int grad, double* tt, double* ttgrad,
                   double* vzero_out) {
  int condz = 0.0 <= zsrc && zsrc <= dz * nz;
  int condx = 0.0 <= xsrc && xsrc <= dx * nx;
  if (!(condz && condx)) return ST_SOURCE_OOB;

  double zsa = zsrc / dz, xsa = xsrc / dx;
  zsa = zsa >= nz ? zsa - EPS : zsa;
  xsa = xsa >= nx ? xsa - EPS : xsa;
  int zsi = imin((int)zsa, nz - 1);
  int xsi = imin((int)xsa, nx - 1);
  double vzero = slow[(long)zsi * nx + xsi];

  int NZ = nz + 1, NX = nx + 1;
  long nn = (long)NZ * NX;
  for (long n = 0; n < nn; ++n) tt[n] = BIG;
  int8_t* sgn = NULL;
  if (grad) {
    sgn = (int8_t*)calloc((size_t)nn * 2, 1);
    memset(ttgrad, 0, sizeof(double) * (size_t)nn * 2);
  }
#define TT(a, b) tt[(long)(a)*NX + (b)]
#define SL(a, b) slow[(long)(a)*nx + (b)]
#define SGN(a, b, c) sgn[((long)(a)*NX + (b)) * 2 + (c)]

  /* source classification, _fteik2d.py:328-352 */
  double dzu = fabs(zsa - (double)zsi);
  double dzd = 1.0 - dzu;
  double dxw = fabs(xsa - (double)xsi);
  double dxe = 1.0 - dxw;
  double dzv_min = pmin2(dzu, dzd);
  double dzh_min = pmin2(dxw, dxe);
  int iflag;
  if (dzv_min < EPS && dzh_min < EPS) {
    zsa = rint(zsa);
    xsa = rint(xsa);
    iflag = 1;
  } else if (dzv_min > EPS || dzh_min > EPS) {
    zsa = dzv_min < EPS ? rint(zsa) : zsa;
    xsa = dzh_min < EPS ? rint(xsa) : xsa;
    iflag = 2;
  } else {
    zsa = rint(zsa);
    xsa = rint(xsa);
    iflag = 3;
  }

  if (iflag == 2) { /* _fteik2d.py:355-614 */
    int ntd = NZ > NX ? NZ : NX;
    double* td = (double*)malloc(sizeof(double) * (size_t)ntd);
    for (int q = 0; q < ntd; ++q) td[q] = BIG;
    dzu = fabs(zsa - (double)zsi);
    dzd = 1.0 - dzu;
    dxw = fabs(xsa - (double)xsi);
    dxe = 1.0 - dxw;
    static const int OFF[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
    for (int q = 0; q < 4; ++q) {
      int i = zsi + OFF[q][0], j = xsi + OFF[q][1];
      double tzc, txc;
      TT(i, j) = t_anad2(i, j, dz, dx, zsa, xsa, vzero, &tzc, &txc);
      if (grad) {
        ttgrad[((long)i * NX + j) * 2] = tzc;
        ttgrad[((long)i * NX + j) * 2 + 1] = txc;
      }
    }
    double dxi = 1.0 / dx;
    double dx2i = dxi / dx;
    double dzi, dz2i, tzc, txc, t0c, vref, tauv, tauev, taue;
    td[xsi + 1] = vzero * dxe * dx;
    for (int j = xsi + 2; j < NX; ++j) {
      vref = SL(zsi, j - 1);
      td[j] = td[j - 1] + dx * vref;
      tauv = td[j] - vzero * fabs((double)j - xsa) * dx;
      tauev = td[j - 1] - vzero * fabs((double)j - xsa - 1.0) * dx;
      dzi = 1.0 / dzd;
      dz2i = dz / dzd / dzd;
      taue = TT(zsi + 1, j - 1) - t_ana2(zsi + 1, j - 1, dz, dx, zsa, xsa, vzero);
      t0c = t_anad2(zsi + 1, j, dz, dx, zsa, xsa, vzero, &tzc, &txc);
      TT(zsi + 1, j) = delta2(TT(zsi + 1, j), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i,
                              dx2i, vzero, vref, 1, 1);
      if (grad) { SGN(zsi + 1, j, 0) = 1; SGN(zsi + 1, j, 1) = 1; }
      if (dzu > 0.0) {
        dzi = 1.0 / dzu;
        dz2i = dz / dzu / dzu;
        taue = TT(zsi, j - 1) - t_ana2(zsi, j - 1, dz, dx, zsa, xsa, vzero);
        t0c = t_anad2(zsi, j, dz, dx, zsa, xsa, vzero, &tzc, &txc);
        TT(zsi, j) = delta2(TT(zsi, j), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i, dx2i,
                            vzero, vref, -1, 1);
        if (grad) { SGN(zsi, j, 0) = -1; SGN(zsi, j, 1) = 1; }
      }
    }
    td[xsi] = vzero * dxw * dx;
    for (int j = xsi - 1; j >= 0; --j) {
      vref = SL(zsi, j);
      td[j] = td[j + 1] + dx * vref;
      tauv = td[j] - vzero * fabs((double)j - xsa) * dx;
      tauev = td[j + 1] - vzero * fabs((double)j - xsa + 1.0) * dx;
      dzi = 1.0 / dzd;
      dz2i = dz / dzd / dzd;
      taue = TT(zsi + 1, j + 1) - t_ana2(zsi + 1, j + 1, dz, dx, zsa, xsa, vzero);
      t0c = t_anad2(zsi + 1, j, dz, dx, zsa, xsa, vzero, &tzc, &txc);
      TT(zsi + 1, j) = delta2(TT(zsi + 1, j), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i,
                              dx2i, vzero, vref, 1, -1);
      if (grad) { SGN(zsi + 1, j, 0) = 1; SGN(zsi + 1, j, 1) = -1; }
      if (dzu > 0.0) {
        dzi = 1.0 / dzu;
        dz2i = dz / dzu / dzu;
        /* the reference reads row zsi + 1 here (_fteik2d.py:472-474) */
        taue = TT(zsi + 1, j + 1) - t_ana2(zsi + 1, j + 1, dz, dx, zsa, xsa, vzero);
        t0c = t_anad2(zsi, j, dz, dx, zsa, xsa, vzero, &tzc, &txc);
        TT(zsi, j) = delta2(TT(zsi, j), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i, dx2i,
                            vzero, vref, -1, -1);
        if (grad) { SGN(zsi, j, 0) = -1; SGN(zsi, j, 1) = -1; }
      }
    }
    dzi = 1.0 / dz;
    dz2i = dzi / dz;
    for (int q = 0; q < ntd; ++q) td[q] = BIG;
    td[zsi + 1] = vzero * dzd * dz;
    for (int i = zsi + 2; i < NZ; ++i) {
      vref = SL(i - 1, xsi);
      td[i] = td[i - 1] + dz * vref;
      taue = td[i] - vzero * fabs((double)i - zsa) * dz;
      tauev = td[i - 1] - vzero * fabs((double)i - zsa - 1.0) * dz;
      dxi = 1.0 / dxe;
      dx2i = dx / dxe / dxe;
      tauv = TT(i - 1, xsi + 1) - t_ana2(i - 1, xsi + 1, dz, dx, zsa, xsa, vzero);
      t0c = t_anad2(i, xsi + 1, dz, dx, zsa, xsa, vzero, &tzc, &txc);
      TT(i, xsi + 1) = delta2(TT(i, xsi + 1), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i,
                              dx2i, vzero, vref, 1, 1);
      if (grad) { SGN(i, xsi + 1, 0) = 1; SGN(i, xsi + 1, 1) = 1; }
      if (dxw > 0.0) {
        dxi = 1.0 / dxw;
        dx2i = dx / dxw / dxw;
        tauv = TT(i - 1, xsi) - t_ana2(i - 1, xsi, dz, dx, zsa, xsa, vzero);
        t0c = t_anad2(i, xsi, dz, dx, zsa, xsa, vzero, &tzc, &txc);
        TT(i, xsi) = delta2(TT(i, xsi), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i, dx2i,
                            vzero, vref, 1, -1);
        if (grad) { SGN(i, xsi, 0) = 1; SGN(i, xsi, 1) = -1; }
      }
    }
    td[zsi] = vzero * dzu * dz;
    for (int i = zsi - 1; i >= 0; --i) {
      vref = SL(i, xsi);
      td[i] = td[i + 1] + dz * vref;
      taue = td[i] - vzero * fabs((double)i - zsa) * dz;
      tauev = td[i + 1] - vzero * fabs((double)i - zsa + 1.0) * dz;
      dxi = 1.0 / dxe;
      dx2i = dx / dxe / dxe;
      tauv = TT(i + 1, xsi + 1) - t_ana2(i + 1, xsi + 1, dz, dx, zsa, xsa, vzero);
      t0c = t_anad2(i, xsi + 1, dz, dx, zsa, xsa, vzero, &tzc, &txc);
      TT(i, xsi + 1) = delta2(TT(i, xsi + 1), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i,
                              dx2i, vzero, vref, -1, 1);
      if (grad) { SGN(i, xsi + 1, 0) = -1; SGN(i, xsi + 1, 1) = 1; }
      if (dxw > 0.0) {
        dxi = 1.0 / dxw;
        dx2i = dx / dxw / dxw;
        tauv = TT(i + 1, xsi) - t_ana2(i + 1, xsi, dz, dx, zsa, xsa, vzero);
        t0c = t_anad2(i, xsi, dz, dx, zsa, xsa, vzero, &tzc, &txc);
        TT(i, xsi) = delta2(TT(i, xsi), tauv, taue, tauev, t0c, tzc, txc, dzi, dxi, dz2i, dx2i,
                            vzero, vref, -1, -1);
        if (grad) { SGN(i, xsi, 0) = -1; SGN(i, xsi, 1) = -1; }
      }
    }
    free(td);
  } else {
    TT((int)zsa, (int)xsa) = 0.0; /* _fteik2d.py:616-617 */
  }

  dargs2_t d;
  d.dz = dz; d.dx = dx;
  d.zsi = (double)zsi; d.xsi = (double)xsi;
  d.zsa = zsa; d.xsa = xsa; d.vzero = vzero;
  for (int s = 0; s < nsweep; ++s) sweep2d(tt, sgn, slow, &d, NZ, NX, grad);

  if (grad) { /* _fteik2d.py:623-639 */
    for (int i = 0; i < NZ; ++i)
      for (int j = 0; j < NX; ++j) {
        long n = (long)i * NX + j;
        double* g = ttgrad + n * 2;
        int sz = sgn[n * 2], sx = sgn[n * 2 + 1];
        if (sz != 0) g[0] = (double)sz * (tt[n] - tt[n - (long)sz * NX]) / dz;
        if (sx != 0) g[1] = (double)sx * (tt[n] - tt[n - sx]) / dx;
        double gn = sqrt(g[0] * g[0] + g[1] * g[1]);
        if (gn > 0.0) {
          g[0] /= gn;
          g[1] /= gn;
        }
      }
    free(sgn);
  }
#undef TT
#undef SL
#undef SGN
  *vzero_out = vzero;
  return ST_OK;
}

/* fteik2d_vectorized, _fteik2d.py:644-664 */
int oracle_fteik2d_many(const double* slow, int nz, int nx, double dz, double dx,
                        const double* src, int nsrc, int nsweep, int grad, double* tt,
                        double* ttgrad, double* vzero, int nthreads) {
  long nn = (long)(nz + 1) * (nx + 1);
  int status = ST_OK;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) if (nthreads > 1)
  for (int s = 0; s < nsrc; ++s) {
    int st = oracle_fteik2d(slow, nz, nx, dz, dx, src[2 * s], src[2 * s + 1], nsweep, grad,
                            tt + s * nn, grad ? ttgrad + s * nn * 2 : NULL, vzero + s);
    if (st != ST_OK) {
#pragma omp critical
      status = st;
    }
  }
  return status;
}

/* ------------------------------------------------------------------------ */
/* Interpolation: fteikpy/_interp/*.py                                      */
/* The axis arrays (x, y, z) are positional, as in the reference: for the   */
/* grids they are (zaxis, xaxis, yaxis). v is read with element stride vs   */
/* so that a gradient component of a [..][3] array can be read in place.    */
/* ------------------------------------------------------------------------ */

/* _interp3d, _interp3d.py:7-174 */
static double interp3_point(const double* x, int nx, const double* y, int ny, const double* z,
                            int nz, const double* v, long vs, double xq, double yq, double zq,
                            double fval) {
  int condx = x[0] <= xq && xq <= x[nx - 1];
  int condy = y[0] <= yq && yq <= y[ny - 1];
  int condz = z[0] <= zq && zq <= z[nz - 1];
  if (!(condx && condy && condz)) return fval;
  int lx = nx - 1, ly = ny - 1, lz = nz - 1;
  int i1 = search_right_m1(x, nx, xq), j1 = search_right_m1(y, ny, yq),
      k1 = search_right_m1(z, nz, zq);
  int i2 = i1 + 1, j2 = j1 + 1, k2 = k1 + 1;
  int ei = i1 == lx, ej = j1 == ly, ek = k1 == lz;
#define V(a, b, c) v[(((long)(a)*ny + (b)) * nz + (c)) * vs]
  double x1 = x[i1], y1 = y[j1], z1 = z[k1];
  double x2 = ei ? 2.0 * x1 - x[nx - 2] : x[i2];
  double y2 = ej ? 2.0 * y1 - y[ny - 2] : y[j2];
  double z2 = ek ? 2.0 * z1 - z[nz - 2] : z[k2];
  double v111 = V(i1, j1, k1);
  double v211 = ei ? 1.0 : V(i2, j1, k1);
  double v121 = ej ? 1.0 : V(i1, j2, k1);
  double v221 = (ei || ej) ? 1.0 : V(i2, j2, k1);
  double v112 = ek ? 1.0 : V(i1, j1, k2);
  double v212 = (ei || ek) ? 1.0 : V(i2, j1, k2);
  double v122 = (ej || ek) ? 1.0 : V(i1, j2, k2);
  double v222 = (ei || ej || ek) ? 1.0 : V(i2, j2, k2);
#undef V
  double vq = v111 * fabs((x2 - xq) * (y2 - yq) * (z2 - zq));
  vq += v211 * fabs((x1 - xq) * (y2 - yq) * (z2 - zq));
  vq += v121 * fabs((x2 - xq) * (y1 - yq) * (z2 - zq));
  vq += v221 * fabs((x1 - xq) * (y1 - yq) * (z2 - zq));
  vq += v112 * fabs((x2 - xq) * (y2 - yq) * (z1 - zq));
  vq += v212 * fabs((x1 - xq) * (y2 - yq) * (z1 - zq));
  vq += v122 * fabs((x2 - xq) * (y1 - yq) * (z1 - zq));
  vq += v222 * fabs((x1 - xq) * (y1 - yq) * (z1 - zq));
  vq /= fabs((x2 - x1) * (y2 - y1) * (z2 - z1));
  return vq;
}

/* _interp2d, _interp2d.py:7-74 */
static double interp2_point(const double* x, int nx, const double* y, int ny, const double* v,
                            long vs, double xq, double yq, double fval) {
  int condx = x[0] <= xq && xq <= x[nx - 1];
  int condy = y[0] <= yq && yq <= y[ny - 1];
  if (!(condx && condy)) return fval;
  int i1 = search_right_m1(x, nx, xq), j1 = search_right_m1(y, ny, yq);
  int i2 = i1 + 1, j2 = j1 + 1;
  int ei = i1 == nx - 1, ej = j1 == ny - 1;
#define V(a, b) v[((long)(a)*ny + (b)) * vs]
  double x1 = x[i1], y1 = y[j1];
  double x2 = ei ? 2.0 * x1 - x[nx - 2] : x[i2];
  double y2 = ej ? 2.0 * y1 - y[ny - 2] : y[j2];
  double v11 = V(i1, j1);
  double v21 = ei ? 1.0 : V(i2, j1);
  double v12 = ej ? 1.0 : V(i1, j2);
  double v22 = (ei || ej) ? 1.0 : V(i2, j2);
#undef V
  double vq = v11 * fabs((x2 - xq) * (y2 - yq));
  vq += v21 * fabs((x1 - xq) * (y2 - yq));
  vq += v12 * fabs((x2 - xq) * (y1 - yq));
  vq += v22 * fabs((x1 - xq) * (y1 - yq));
  vq /= fabs((x2 - x1) * (y2 - y1));
  return vq;
}

static inline double dist3(double x1, double y1, double z1, double x2, double y2, double z2) {
  double a = x1 - x2, b = y1 - y2, c = z1 - z2;
  return sqrt(a * a + b * b + c * c);
}
static inline double dist2(double x1, double y1, double x2, double y2) {
  double a = x1 - x2, b = y1 - y2;
  return sqrt(a * a + b * b);
}

/* _vinterp3d, _vinterp3d.py:7-264 */
static double vinterp3_point(const double* x, int nx, const double* y, int ny, const double* z,
                             int nz, const double* v, double xq, double yq, double zq,
                             double xs, double ys, double zs, double vzero, double fval) {
  int condx = x[0] <= xq && xq <= x[nx - 1];
  int condy = y[0] <= yq && yq <= y[ny - 1];
  int condz = z[0] <= zq && zq <= z[nz - 1];
  if (!(condx && condy && condz)) return fval;
  int xsi = search_right_m1(x, nx, xs), ysi = search_right_m1(y, ny, ys),
      zsi = search_right_m1(z, nz, zs);
  int i1 = search_right_m1(x, nx, xq), j1 = search_right_m1(y, ny, yq),
      k1 = search_right_m1(z, nz, zq);
  if (xsi == i1 && ysi == j1 && zsi == k1) return vzero * dist3(xs, ys, zs, xq, yq, zq);
  int i2 = i1 + 1, j2 = j1 + 1, k2 = k1 + 1;
  int ei = i1 == nx - 1, ej = j1 == ny - 1, ek = k1 == nz - 1;
#define V(a, b, c) v[((long)(a)*ny + (b)) * nz + (c)]
  double x1 = x[i1], y1 = y[j1], z1 = z[k1];
  double x2 = ei ? 2.0 * x1 - x[nx - 2] : x[i2];
  double y2 = ej ? 2.0 * y1 - y[ny - 2] : y[j2];
  double z2 = ek ? 2.0 * z1 - z[nz - 2] : z[k2];
  double d111 = dist3(xs, ys, zs, x1, y1, z1);
  double d211 = ei ? 0.0 : dist3(xs, ys, zs, x2, y1, z1);
  double d121 = ej ? 0.0 : dist3(xs, ys, zs, x1, y2, z1);
  double d221 = (ei || ej) ? 0.0 : dist3(xs, ys, zs, x2, y2, z1);
  double d112 = ek ? 0.0 : dist3(xs, ys, zs, x1, y1, z2);
  double d212 = (ei || ek) ? 0.0 : dist3(xs, ys, zs, x2, y1, z2);
  double d122 = (ej || ek) ? 0.0 : dist3(xs, ys, zs, x1, y2, z2);
  double d222 = (ei || ej || ek) ? 0.0 : dist3(xs, ys, zs, x2, y2, z2);
  double v111 = V(i1, j1, k1);
  double v211 = ei ? 1.0 : V(i2, j1, k1);
  double v121 = ej ? 1.0 : V(i1, j2, k1);
  double v221 = (ei || ej) ? 1.0 : V(i2, j2, k1);
  double v112 = ek ? 1.0 : V(i1, j1, k2);
  double v212 = (ei || ek) ? 1.0 : V(i2, j1, k2);
  double v122 = (ej || ek) ? 1.0 : V(i1, j2, k2);
  double v222 = (ei || ej || ek) ? 1.0 : V(i2, j2, k2);
#undef V
  if (!(v111 != 0.0 && v211 != 0.0 && v121 != 0.0 && v221 != 0.0 && v112 != 0.0 &&
        v212 != 0.0 && v122 != 0.0 && v222 != 0.0))
    return vzero * dist3(xs, ys, zs, xq, yq, zq);
  double vq = d111 / v111 * fabs((x2 - xq) * (y2 - yq) * (z2 - zq));
  vq += d211 / v211 * fabs((x1 - xq) * (y2 - yq) * (z2 - zq));
  vq += d121 / v121 * fabs((x2 - xq) * (y1 - yq) * (z2 - zq));
  vq += d221 / v221 * fabs((x1 - xq) * (y1 - yq) * (z2 - zq));
  vq += d112 / v112 * fabs((x2 - xq) * (y2 - yq) * (z1 - zq));
  vq += d212 / v212 * fabs((x1 - xq) * (y2 - yq) * (z1 - zq));
  vq += d122 / v122 * fabs((x2 - xq) * (y1 - yq) * (z1 - zq));
  vq += d222 / v222 * fabs((x1 - xq) * (y1 - yq) * (z1 - zq));
  vq /= fabs((x2 - x1) * (y2 - y1) * (z2 - z1));
  return dist3(xs, ys, zs, xq, yq, zq) / vq;
}

/* _vinterp2d, _vinterp2d.py:7-108 */
static double vinterp2_point(const double* x, int nx, const double* y, int ny, const double* v,
                             double xq, double yq, double xs, double ys, double vzero,
                             double fval) {
  int condx = x[0] <= xq && xq <= x[nx - 1];
  int condy = y[0] <= yq && yq <= y[ny - 1];
  if (!(condx && condy)) return fval;
  int xsi = search_right_m1(x, nx, xs), ysi = search_right_m1(y, ny, ys);
  int i1 = search_right_m1(x, nx, xq), j1 = search_right_m1(y, ny, yq);
  if (xsi == i1 && ysi == j1) return vzero * dist2(xs, ys, xq, yq);
  int i2 = i1 + 1, j2 = j1 + 1;
  int ei = i1 == nx - 1, ej = j1 == ny - 1;
#define V(a, b) v[(long)(a)*ny + (b)]
  double x1 = x[i1], y1 = y[j1];
  double x2 = ei ? 2.0 * x1 - x[nx - 2] : x[i2];
  double y2 = ej ? 2.0 * y1 - y[ny - 2] : y[j2];
  double d11 = dist2(xs, ys, x1, y1);
  double d21 = ei ? 0.0 : dist2(xs, ys, x2, y1);
  double d12 = ej ? 0.0 : dist2(xs, ys, x1, y2);
  double d22 = (ei || ej) ? 0.0 : dist2(xs, ys, x2, y2);
  double v11 = V(i1, j1);
  double v21 = ei ? 1.0 : V(i2, j1);
  double v12 = ej ? 1.0 : V(i1, j2);
  double v22 = (ei || ej) ? 1.0 : V(i2, j2);
#undef V
  if (!(v11 != 0.0 && v21 != 0.0 && v12 != 0.0 && v22 != 0.0))
    return vzero * dist2(xs, ys, xq, yq);
  double vq = d11 / v11 * fabs((x2 - xq) * (y2 - yq));
  vq += d21 / v21 * fabs((x1 - xq) * (y2 - yq));
  vq += d12 / v12 * fabs((x2 - xq) * (y1 - yq));
  vq += d22 / v22 * fabs((x1 - xq) * (y1 - yq));
  vq /= fabs((x2 - x1) * (y2 - y1));
  return dist2(xs, ys, xq, yq) / vq;
}

void oracle_interp3d(const double* x, int nx, const double* y, int ny, const double* z, int nz,
                     const double* v, long vs, const double* q, int nq, double fval,
                     double* out) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < nq; ++p)
    out[p] = interp3_point(x, nx, y, ny, z, nz, v, vs, q[3 * p], q[3 * p + 1], q[3 * p + 2],
                           fval);
}

void oracle_interp2d(const double* x, int nx, const double* y, int ny, const double* v, long vs,
                     const double* q, int nq, double fval, double* out) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < nq; ++p)
    out[p] = interp2_point(x, nx, y, ny, v, vs, q[2 * p], q[2 * p + 1], fval);
}

void oracle_vinterp3d(const double* x, int nx, const double* y, int ny, const double* z, int nz,
                      const double* v, const double* q, int nq, const double* src, double vzero,
                      double fval, double* out) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < nq; ++p)
    out[p] = vinterp3_point(x, nx, y, ny, z, nz, v, q[3 * p], q[3 * p + 1], q[3 * p + 2],
                            src[0], src[1], src[2], vzero, fval);
}

void oracle_vinterp2d(const double* x, int nx, const double* y, int ny, const double* v,
                      const double* q, int nq, const double* src, double vzero, double fval,
                      double* out) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < nq; ++p)
    out[p] = vinterp2_point(x, nx, y, ny, v, q[2 * p], q[2 * p + 1], src[0], src[1], vzero,
                            fval);
}

/* ------------------------------------------------------------------------ */
/* Ray tracing: fteikpy/_fteik/_ray3d.py, _ray2d.py, _common.py            */
/* ------------------------------------------------------------------------ */

/* numpy's ndarray.min(): NaN if any element is NaN. */
static double np_min(const double* a, int n) {
  double m = a[0];
  for (int q = 0; q < n; ++q) {
    if (a[q] != a[q]) return a[q];
    if (a[q] < m) m = a[q];
  }
  return m;
}

/* shrink, _fteik/_common.py:4-28 */
static double shrink(const double* pcur, const double* delta, const double* lower,
                     const double* upper, int nd) {
  double bl[3], bu[3];
  int nl = 0, nu = 0;
  for (int q = 0; q < nd; ++q) {
    double tmp = pcur[q] - delta[q];
    if (tmp < lower[q]) bl[nl++] = (pcur[q] - lower[q]) / delta[q];
    if (tmp > upper[q]) bu[nu++] = (pcur[q] - upper[q]) / delta[q];
  }
  if (nl && nu) return pmin2(np_min(bl, nl), np_min(bu, nu));
  if (nl) return np_min(bl, nl);
  if (nu) return np_min(bu, nu);
  return 1.0;
}

/* _ray3d / _ray2d, _ray3d.py:9-120 and _ray2d.py:9-91, written once for
 * nd = 2 or 3.  ax[d] / n[d] are the node axes (z, x[, y]); grad points to the
 * gradient array [..][nd] (component c read with stride nd).  The ray is
 * written receiver-first into ray[max_step][nd]; *count receives the index of
 * the last point (the source), as the reference returns.  One intentional
 * difference: the reference reads one element past the end of an axis when a
 * honor_grid step lands exactly on the last node (_ray3d.py:96-98); here the
 * index is clamped to the last node instead. */
static int ray_one(int nd, const double* const* ax, const int* n, const double* grad,
                   const double* end, const double* src, double stepsize, int max_step,
                   int honor_grid, double* ray, int* count_out) {
  for (int q = 0; q < nd; ++q)
    if (!(ax[q][0] <= end[q] && end[q] <= ax[q][n[q] - 1])) return ST_ENDPOINT_OOB;
  double lower[3], upper[3];
  int isrc[3], cell[3];
  if (honor_grid) {
    for (int q = 0; q < nd; ++q) {
      int i = search_right_m1(ax[q], n[q], end[q]);
      lower[q] = end[q] == ax[q][i] ? ax[q][imax(i - 1, 0)] : ax[q][i];
      upper[q] = ax[q][imin(i + 1, n[q] - 1)];
      isrc[q] = search_right_m1(ax[q], n[q], src[q]);
    }
  }
  int count = 1;
  double pcur[3], delta[3];
  for (int q = 0; q < nd; ++q) {
    pcur[q] = end[q];
    ray[q] = pcur[q];
  }
  for (;;) {
    double dd = nd == 3 ? dist3(src[0], src[1], src[2], pcur[0], pcur[1], pcur[2])
                        : dist2(src[0], src[1], pcur[0], pcur[1]);
    if (!(dd >= stepsize)) break;
    double g[3], gn;
    if (nd == 3) {
      for (int c = 0; c < 3; ++c)
        g[c] = interp3_point(ax[0], n[0], ax[1], n[1], ax[2], n[2], grad + c, 3, pcur[0],
                             pcur[1], pcur[2], NAN);
      gn = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    } else {
      for (int c = 0; c < 2; ++c)
        g[c] = interp2_point(ax[0], n[0], ax[1], n[1], grad + c, 2, pcur[0], pcur[1], NAN);
      gn = sqrt(g[0] * g[0] + g[1] * g[1]);
    }
    double gni;
    if (gn > 0.0)
      gni = 1.0 / gn;
    else
      break;
    for (int q = 0; q < nd; ++q) delta[q] = stepsize * g[q] * gni;
    if (honor_grid) {
      double fac = shrink(pcur, delta, lower, upper, nd);
      for (int q = 0; q < nd; ++q) {
        pcur[q] -= fac * delta[q];
        pcur[q] = pmin2(pmax2(pcur[q], ax[q][0]), ax[q][n[q] - 1]);
      }
      if (fac < 1.0) {
        for (int q = 0; q < nd; ++q) {
          if (fabs(pcur[q] - lower[q]) < 1.0e-8)
            pcur[q] = lower[q];
          else if (fabs(pcur[q] - upper[q]) < 1.0e-8)
            pcur[q] = upper[q];
        }
        int hit = 1;
        for (int q = 0; q < nd; ++q) {
          int i = search_right_m1(ax[q], n[q], pcur[q]);
          cell[q] = i;
          lower[q] = pcur[q] == ax[q][i] ? ax[q][imax(i - 1, 0)] : ax[q][i];
          upper[q] = ax[q][imin(i + 1, n[q] - 1)];
          hit = hit && (i == isrc[q]);
        }
        for (int q = 0; q < nd; ++q) ray[count * nd + q] = pcur[q];
        count += 1;
        if (hit) break;
      }
    } else {
      for (int q = 0; q < nd; ++q) {
        pcur[q] -= delta[q];
        pcur[q] = pmin2(pmax2(pcur[q], ax[q][0]), ax[q][n[q] - 1]);
      }
      for (int q = 0; q < nd; ++q) ray[count * nd + q] = pcur[q];
      count += 1;
    }
    if (count >= max_step) return ST_MAX_STEP;
  }
  for (int q = 0; q < nd; ++q) ray[count * nd + q] = src[q];
  *count_out = count;
  return ST_OK;
}

/* _ray3d_vectorized, _ray3d.py:123-164.  rays is [nrays][max_step][3];
 * status[r] receives the per-ray status code. */
void oracle_ray3d(const double* z, int nz, const double* x, int nx, const double* y, int ny,
                  const double* grad, const double* ends, int nrays, const double* src,
                  double stepsize, int max_step, int honor_grid, double* rays, int* counts,
                  int* status) {
  const double* ax[3] = {z, x, y};
  int n[3] = {nz, nx, ny};
#pragma omp parallel for schedule(dynamic, 4)
  for (int r = 0; r < nrays; ++r) {
    counts[r] = 0;
    status[r] = ray_one(3, ax, n, grad, ends + 3 * r, src, stepsize, max_step, honor_grid,
                        rays + (long)r * max_step * 3, counts + r);
  }
}

/* _ray2d_vectorized, _ray2d.py:94-117 */
void oracle_ray2d(const double* z, int nz, const double* x, int nx, const double* grad,
                  const double* ends, int nrays, const double* src, double stepsize,
                  int max_step, int honor_grid, double* rays, int* counts, int* status) {
  const double* ax[3] = {z, x, NULL};
  int n[3] = {nz, nx, 0};
#pragma omp parallel for schedule(dynamic, 4)
  for (int r = 0; r < nrays; ++r) {
    counts[r] = 0;
    status[r] = ray_one(2, ax, n, grad, ends + 2 * r, src, stepsize, max_step, honor_grid,
                        rays + (long)r * max_step * 2, counts + r);
  }
}

/* ------------------------------------------------------------------------ */
/* Adjoint of the 3D solve (no counterpart in the reference)                */
/* ------------------------------------------------------------------------ */
/*
 * d(loss)/d(slowness) for a loss on the traveltimes _vinterp3d gives at
 * receivers, as the plain sequential reverse-mode derivative of
 * oracle_fteik3d: the forward runs the reference's sweep loops unchanged and
 * tapes, per directional sweep, every node that changed (the branch code of
 * the winning operator, _fteik3d.py:166-200, and the value it replaced); the
 * reverse pass walks each sweep's loop nest backwards and pushes the adjoint
 * of every changed node to the inputs of its operator.
 *
 * Where the operator's slowness is a minimum over 2 or 4 cells and several
 * distinct cells share it, each of them gets half the partial (the mean of
 * the two one-sided derivatives, i.e. what a central difference measures).
 *
 * The checker for fteik3d_adjoint; finite differences of oracle_fteik3d pin it.
 */

/* partials of the operator coded (a, b, c) at node (i, j, k) in the current
 * traveltimes; w[] indexed like the reference's neighbour names. */
enum { W_TV, W_TE, W_TN, W_TEV, W_TEN, W_TNV, W_TNVE, W_N };

static int distinct_min_cells(const double* slow, const long* c, int n, long* out, double* vmin) {
  double m = slow[c[0]];
  for (int q = 1; q < n; ++q)
    if (slow[c[q]] < m) m = slow[c[q]];
  int k = 0;
  for (int q = 0; q < n; ++q) {
    if (slow[c[q]] != m) continue;
    int dup = 0;
    for (int r = 0; r < k; ++r) dup |= out[r] == c[q];
    if (!dup) out[k++] = c[q];
  }
  *vmin = m;
  return k;
}

static void adj_push(double* tt, double* lam, double* gs, const double* slow, const dargs3_t* d,
                     int i, int j, int k, int a, int b, int c, int nz, int nx, int ny,
                     double lam_n) {
  /* nz, nx, ny are NODE counts here, as in sweep3_node */
  const long NXY = (long)nx * ny, SXY = (long)(nx - 1) * (ny - 1);
  const int SY = ny - 1;
#define IDX(p, q, r) ((long)(p)*NXY + (long)(q)*ny + (r))
#define CEL(p, q, r) ((long)(p)*SXY + (long)(q)*SY + (r))
  int tz = a, tx = b, ty = c; /* the sweep's signs where the operator uses an axis */
  long nv = IDX(i - tz, j, k), ne = IDX(i, j - tx, k), nn = IDX(i, j, k - ty);
  long nev = IDX(i - tz, j - tx, k), nen = IDX(i, j - tx, k - ty);
  long nnv = IDX(i - tz, j, k - ty), nnve = IDX(i - tz, j - tx, k - ty);
  int i1 = i - (tz > 0), j1 = j - (tx > 0), k1 = k - (ty > 0);
  int im = imax(i - 1, 0), ip = imin(i, nz - 2);
  int jm = imax(j - 1, 0), jp = imin(j, nx - 2);
  int km = imax(k - 1, 0), kp = imin(k, ny - 2);
  double w[W_N] = {0, 0, 0, 0, 0, 0, 0};
  long cand[4], cells[4];
  int ncell = 0;
  double ps = 0.0, v;
  int nnz = (a != 0) + (b != 0) + (c != 0);
  if (nnz == 1) {
    if (a) {
      cand[0] = CEL(i1, jm, km); cand[1] = CEL(i1, jm, kp);
      cand[2] = CEL(i1, jp, km); cand[3] = CEL(i1, jp, kp);
      w[W_TV] = 1.0; ps = d->dz;
    } else if (b) {
      cand[0] = CEL(im, j1, km); cand[1] = CEL(ip, j1, km);
      cand[2] = CEL(im, j1, kp); cand[3] = CEL(ip, j1, kp);
      w[W_TE] = 1.0; ps = d->dx;
    } else {
      cand[0] = CEL(im, jm, k1); cand[1] = CEL(im, jp, k1);
      cand[2] = CEL(ip, jm, k1); cand[3] = CEL(ip, jp, k1);
      w[W_TN] = 1.0; ps = d->dy;
    }
    ncell = distinct_min_cells(slow, cand, 4, cells, &v);
  } else if (nnz == 2) {
    /* t = (p1 * x + p2 * y + sqrt(4 v^2 (p1 + p2) - p1 p2 (x - y)^2)) / (p1 + p2)
     * with x, y the two combinations below and p1, p2 their weights */
    double p1, p2, x, y;
    int u1, u2, u12; /* inputs: x = u12 + u1 - u2 ... spelled out per plane */
    if (!c) { /* ZX: x = tb = tev - te + tv (weight dz2i), y = ta = tev + te - tv (dx2i) */
      cand[0] = CEL(i1, j1, km); cand[1] = CEL(i1, j1, kp);
      p1 = d->dz2i; p2 = d->dx2i;
      x = tt[nev] - tt[ne] + tt[nv]; y = tt[nev] + tt[ne] - tt[nv];
      u1 = W_TV; u2 = W_TE; u12 = W_TEV;
    } else if (!b) { /* ZY: x = ta = tv - tn + tnv (dz2i), y = tb = tn - tv + tnv (dy2i) */
      cand[0] = CEL(i1, jm, k1); cand[1] = CEL(i1, jp, k1);
      p1 = d->dz2i; p2 = d->dy2i;
      x = tt[nv] - tt[nn] + tt[nnv]; y = tt[nn] - tt[nv] + tt[nnv];
      u1 = W_TV; u2 = W_TN; u12 = W_TNV;
    } else { /* XY: x = ta = te - tn + ten (dx2i), y = tb = tn - te + ten (dy2i) */
      cand[0] = CEL(im, j1, k1); cand[1] = CEL(ip, j1, k1);
      p1 = d->dx2i; p2 = d->dy2i;
      x = tt[ne] - tt[nn] + tt[nen]; y = tt[nn] - tt[ne] + tt[nen];
      u1 = W_TE; u2 = W_TN; u12 = W_TEN;
    }
    ncell = distinct_min_cells(slow, cand, 2, cells, &v);
    double P = p1 + p2, dxy = x - y;
    double R = sqrt(4.0 * v * v * P - p1 * p2 * dxy * dxy);
    double dx_ = (p1 - p1 * p2 * dxy / R) / P; /* dt/dx */
    double dy_ = (p2 + p1 * p2 * dxy / R) / P; /* dt/dy */
    /* x = u1-ish: in every plane x = +u1 - u2 + u12, y = -u1 + u2 + u12 */
    w[u1] = dx_ - dy_;
    w[u2] = -dx_ + dy_;
    w[u12] = dx_ + dy_;
    ps = 4.0 * v / R;
  } else {
    double tv = tt[nv], te = tt[ne], tn = tt[nn], tev = tt[nev], ten = tt[nen], tnv = tt[nnv],
           tnve = tt[nnve];
    double ta = te - 0.5 * tn + 0.5 * ten - 0.5 * tv + 0.5 * tev - tnv + tnve;
    double tb = tv - 0.5 * tn + 0.5 * tnv - 0.5 * te + 0.5 * tev - ten + tnve;
    double tc = tn - 0.5 * te + 0.5 * ten - 0.5 * tv + 0.5 * tnv - tev + tnve;
    cells[0] = CEL(i1, j1, k1);
    ncell = 1;
    v = slow[cells[0]];
    double Wr = sqrt(v * v * d->dsum * 9.0 - d->dz2dx2 * (ta - tb) * (ta - tb) -
                     d->dz2dy2 * (tb - tc) * (tb - tc) - d->dx2dy2 * (ta - tc) * (ta - tc));
    /* t = (dz2i tb + dx2i ta + dy2i tc + Wr) / dsum */
    double ga = (d->dx2i - (d->dz2dx2 * (ta - tb) + d->dx2dy2 * (ta - tc)) / Wr) / d->dsum;
    double gb = (d->dz2i - (d->dz2dy2 * (tb - tc) - d->dz2dx2 * (ta - tb)) / Wr) / d->dsum;
    double gc = (d->dy2i + (d->dz2dy2 * (tb - tc) + d->dx2dy2 * (ta - tc)) / Wr) / d->dsum;
    /* coefficients of (tv, te, tn, tev, ten, tnv, tnve) in ta, tb, tc */
    static const double A[3][7] = {{-0.5, 1.0, -0.5, 0.5, 0.5, -1.0, 1.0},
                                   {1.0, -0.5, -0.5, 0.5, -1.0, 0.5, 1.0},
                                   {-0.5, -0.5, 1.0, -1.0, 0.5, 0.5, 1.0}};
    for (int q = 0; q < 7; ++q) w[q] = ga * A[0][q] + gb * A[1][q] + gc * A[2][q];
    ps = 9.0 * v / Wr;
  }
  const long in[W_N] = {nv, ne, nn, nev, nen, nnv, nnve};
  for (int q = 0; q < W_N; ++q)
    if (w[q] != 0.0) lam[in[q]] += lam_n * w[q];
  if (ncell > 1) ps *= 0.5;
  for (int q = 0; q < ncell; ++q) gs[cells[q]] += lam_n * ps;
#undef IDX
#undef CEL
}

/* Partials of _vinterp3d's value at one receiver with respect to the node
 * traveltimes (added into lam, scaled by g) and to vzero (returned). */
static double vinterp3_adjoint(const double* x, int nx, const double* y, int ny, const double* z,
                               int nz, const double* v, double* lam, double xq, double yq,
                               double zq, double xs, double ys, double zs, double g) {
  int condx = x[0] <= xq && xq <= x[nx - 1];
  int condy = y[0] <= yq && yq <= y[ny - 1];
  int condz = z[0] <= zq && zq <= z[nz - 1];
  if (!(condx && condy && condz)) return 0.0;
  int xsi = search_right_m1(x, nx, xs), ysi = search_right_m1(y, ny, ys),
      zsi = search_right_m1(z, nz, zs);
  int i1 = search_right_m1(x, nx, xq), j1 = search_right_m1(y, ny, yq),
      k1 = search_right_m1(z, nz, zq);
  double D = dist3(xs, ys, zs, xq, yq, zq);
  if (xsi == i1 && ysi == j1 && zsi == k1) return g * D;
  int ei = i1 == nx - 1, ej = j1 == ny - 1, ek = k1 == nz - 1;
  double xx[2] = {x[i1], ei ? 2.0 * x[i1] - x[nx - 2] : x[i1 + 1]};
  double yy[2] = {y[j1], ej ? 2.0 * y[j1] - y[ny - 2] : y[j1 + 1]};
  double zz[2] = {z[k1], ek ? 2.0 * z[k1] - z[nz - 2] : z[k1 + 1]};
  double dd[8], vv[8], ww[8];
  long id[8];
  for (int q = 0; q < 8; ++q) {
    int a = q & 1, b = (q >> 1) & 1, c = q >> 2; /* corner (x, y, z) offsets */
    int past = (a && ei) || (b && ej) || (c && ek);
    id[q] = past ? -1 : ((long)(i1 + a) * ny + (j1 + b)) * nz + (k1 + c);
    dd[q] = past ? 0.0 : dist3(xs, ys, zs, xx[a], yy[b], zz[c]);
    vv[q] = past ? 1.0 : v[id[q]];
    ww[q] = fabs((xx[1 - a] - xq) * (yy[1 - b] - yq) * (zz[1 - c] - zq));
  }
  for (int q = 0; q < 8; ++q)
    if (vv[q] == 0.0) return g * D;
  double W = fabs((xx[1] - xx[0]) * (yy[1] - yy[0]) * (zz[1] - zz[0]));
  double vq = 0.0;
  for (int q = 0; q < 8; ++q) vq += dd[q] / vv[q] * ww[q];
  vq /= W;
  /* T = D / vq; dT/dv_q = D / vq^2 * dd_q ww_q / (W v_q^2) */
  for (int q = 0; q < 8; ++q)
    if (id[q] >= 0) lam[id[q]] += g * D / (vq * vq) * dd[q] * ww[q] / (W * vv[q] * vv[q]);
  return 0.0;
}

/* One source: forward with tape, then the reverse pass.  gs (cells) receives
 * this source's d(loss)/d(slowness). */
static int adjoint3d_one(const double* slow, int nz, int nx, int ny, double dz, double dx,
                         double dy, const double* src, int nsweep, const double* ax0,
                         const double* ax1, const double* ax2, const double* rec, int nrec,
                         const double* grec, double* gs) {
  int NZ = nz + 1, NX = nx + 1, NY = ny + 1;
  long nn = (long)NZ * NX * NY;
  int nep = 8 * nsweep;
  double* tt = (double*)malloc(sizeof(double) * nn);
  double* tg = (double*)malloc(sizeof(double) * nn * 3);
  double* lam = (double*)calloc((size_t)nn, sizeof(double));
  double* old = (double*)malloc(sizeof(double) * nn * (nep ? nep : 1));
  uint8_t* code = (uint8_t*)malloc((size_t)nn * (nep ? nep : 1));
  int8_t* sgn = (int8_t*)calloc((size_t)nn * 3, 1);
  double vz;
  /* initial state: a 0-sweep solve */
  int st = oracle_fteik3d(slow, nz, nx, ny, dz, dx, dy, src[0], src[1], src[2], 0, 0, tt, NULL,
                          &vz);
  if (st != ST_OK) goto done;
  memset(code, 255, (size_t)nn * (nep ? nep : 1));
  dargs3_t d;
  d.dz = dz; d.dx = dx; d.dy = dy;
  d.dz2i = 1.0 / dz / dz; d.dx2i = 1.0 / dx / dx; d.dy2i = 1.0 / dy / dy;
  d.dz2dx2 = d.dz2i * d.dx2i; d.dz2dy2 = d.dz2i * d.dy2i; d.dx2dy2 = d.dx2i * d.dy2i;
  d.dsum = d.dz2i + d.dx2i + d.dy2i;
  static const int S[8][3] = {{1, 1, 1},   {1, -1, 1},  {1, 1, -1},  {1, -1, -1},
                              {-1, 1, 1},  {-1, -1, 1}, {-1, 1, -1}, {-1, -1, -1}};
  for (int e = 0; e < nep; ++e) {
    int tz = S[e & 7][0], tx = S[e & 7][1], ty = S[e & 7][2];
    int k0 = ty > 0 ? 1 : NY - 2, k1 = ty > 0 ? NY : -1;
    int j0 = tx > 0 ? 1 : NX - 2, j1 = tx > 0 ? NX : -1;
    int i0 = tz > 0 ? 1 : NZ - 2, i1 = tz > 0 ? NZ : -1;
    for (int k = k0; k != k1; k += ty)
      for (int j = j0; j != j1; j += tx)
        for (int i = i0; i != i1; i += tz) {
          long n = ((long)i * NX + j) * NY + k;
          double t0 = tt[n];
          sweep3_node(tt, sgn, slow, &d, i, j, k, tz > 0, tx > 0, ty > 0, tz, tx, ty, NZ, NX, NY,
                      1);
          if (tt[n] != t0) {
            code[e * nn + n] = (uint8_t)((sgn[3 * n] + 1) * 9 + (sgn[3 * n + 1] + 1) * 3 +
                                         (sgn[3 * n + 2] + 1));
            old[e * nn + n] = t0;
          }
        }
  }
  /* seed: receivers (axes in _vinterp3d's naming: x = z axis, y = x, z = y) */
  double gvz = 0.0;
  for (int r = 0; r < nrec; ++r)
    gvz += vinterp3_adjoint(ax0, NZ, ax1, NX, ax2, NY, tt, lam, rec[3 * r], rec[3 * r + 1],
                            rec[3 * r + 2], src[0], src[1], src[2], grec[r]);
  for (int e = nep - 1; e >= 0; --e) {
    int tz = S[e & 7][0], tx = S[e & 7][1], ty = S[e & 7][2];
    /* the forward loops backwards: from the last index down to the first */
    for (int k = (ty > 0 ? NY - 1 : 0); k != (ty > 0 ? 0 : NY - 1); k -= ty)
      for (int j = (tx > 0 ? NX - 1 : 0); j != (tx > 0 ? 0 : NX - 1); j -= tx)
        for (int i = (tz > 0 ? NZ - 1 : 0); i != (tz > 0 ? 0 : NZ - 1); i -= tz) {
          long n = ((long)i * NX + j) * NY + k;
          int cd = code[e * nn + n];
          if (cd == 255) continue;
          double l = lam[n];
          lam[n] = 0.0;
          adj_push(tt, lam, gs, slow, &d, i, j, k, cd / 9 - 1, (cd / 3) % 3 - 1, cd % 3 - 1, NZ,
                   NX, NY, l);
          tt[n] = old[e * nn + n];
        }
  }
  /* initial nodes: t = vzero * distance; vzero is the source cell's slowness */
  {
    double zsa = src[0] / dz, xsa = src[1] / dx, ysa = src[2] / dy;
    zsa = zsa >= nz ? zsa - EPS : zsa;
    xsa = xsa >= nx ? xsa - EPS : xsa;
    ysa = ysa >= ny ? ysa - EPS : ysa;
    int zsi = imin((int)zsa, nz - 1), xsi = imin((int)xsa, nx - 1), ysi = imin((int)ysa, ny - 1);
    long sc = ((long)zsi * nx + xsi) * ny + ysi;
    for (int q = 0; q < 8; ++q) {
      int i = zsi + (q & 1), j = xsi + ((q >> 1) & 1), k = ysi + (q >> 2);
      long n = ((long)i * NX + j) * NY + k;
      double a = dz * (i - zsa), b = dx * (j - xsa), c = dy * (k - ysa);
      gs[sc] += lam[n] * sqrt(a * a + b * b + c * c);
    }
    gs[sc] += gvz;
  }
done:
  free(tt); free(tg); free(lam); free(old); free(code); free(sgn);
  return st;
}

/* d(loss)/d(slowness) [nz][nx][ny] summed over sources; grec is
 * [nsrc][nrec] d(loss)/d(traveltime at receiver). */
int oracle_adjoint3d(const double* slow, int nz, int nx, int ny, double dz, double dx, double dy,
                     const double* src, int nsrc, int nsweep, const double* rec, int nrec,
                     const double* grec, double* grad_slow, int nthreads) {
  long nc = (long)nz * nx * ny;
  int NZ = nz + 1, NX = nx + 1, NY = ny + 1;
  double* ax0 = (double*)malloc(sizeof(double) * NZ);
  double* ax1 = (double*)malloc(sizeof(double) * NX);
  double* ax2 = (double*)malloc(sizeof(double) * NY);
  for (int q = 0; q < NZ; ++q) ax0[q] = dz * q;
  for (int q = 0; q < NX; ++q) ax1[q] = dx * q;
  for (int q = 0; q < NY; ++q) ax2[q] = dy * q;
  double* per = (double*)calloc((size_t)nc * nsrc, sizeof(double));
  int status = ST_OK;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) if (nthreads > 1)
  for (int s = 0; s < nsrc; ++s) {
    int st = adjoint3d_one(slow, nz, nx, ny, dz, dx, dy, src + 3 * s, nsweep, ax0, ax1, ax2, rec,
                           nrec, grec + (long)s * nrec, per + (long)s * nc);
    if (st != ST_OK) {
#pragma omp critical
      status = st;
    }
  }
  for (long c = 0; c < nc; ++c) {
    double g = 0.0;
    for (int s = 0; s < nsrc; ++s) g += per[(long)s * nc + c];
    grad_slow[c] = g;
  }
  free(per); free(ax0); free(ax1); free(ax2);
  return status;
}
