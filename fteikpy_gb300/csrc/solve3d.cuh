// Definitions shared by the 3D solve (fteik3d.cu) and its adjoint
// (adjoint3d.cu): per-solve constants, per-source set-up, the coefficient
// arrays and the workspace layout.
#pragma once
#include <cstdint>

#include "common.cuh"

namespace fteik {

// A pencil is PW x 32/PW node columns (x by y), one per warp lane.
constexpr int kDefaultPencil = 4;
constexpr int kDefaultChunk = 4;

inline int pencils_of(int NX, int NY, int pw) {
  const int pk = 32 / pw;
  return ((NX + pw - 1) / pw) * ((NY + pk - 1) / pk);
}
// Pencil count of the largest of the supported shapes (2, 4 or 8 wide).
inline int max_pencils(int NX, int NY) {
  int m = pencils_of(NX, NY, 2);
  if (pencils_of(NX, NY, 4) > m) m = pencils_of(NX, NY, 4);
  if (pencils_of(NX, NY, 8) > m) m = pencils_of(NX, NY, 8);
  return m;
}

struct Ops3 {
  double dz, dx, dy, dz2i, dx2i, dy2i, dz2dx2, dz2dy2, dx2dy2, dsum;
  double szx, szy, sxy;  // dz2i + dx2i, dz2i + dy2i, dx2i + dy2i
  Recip rzx, rzy, rxy, rsum;
  Recip rdz, rdx, rdy;  // for the gradient post-pass
};

// Per-sweep constants, _fteik3d.py:208-215.
inline Ops3 make_ops3(double dz, double dx, double dy) {
  Ops3 o;
  o.dz = dz;
  o.dx = dx;
  o.dy = dy;
  o.dz2i = 1.0 / dz / dz;
  o.dx2i = 1.0 / dx / dx;
  o.dy2i = 1.0 / dy / dy;
  o.dz2dx2 = o.dz2i * o.dx2i;
  o.dz2dy2 = o.dz2i * o.dy2i;
  o.dx2dy2 = o.dx2i * o.dy2i;
  o.dsum = o.dz2i + o.dx2i + o.dy2i;
  o.szx = o.dz2i + o.dx2i;
  o.szy = o.dz2i + o.dy2i;
  o.sxy = o.dx2i + o.dy2i;
  o.rzx = make_recip(o.szx);
  o.rzy = make_recip(o.szy);
  o.rxy = make_recip(o.sxy);
  o.rsum = make_recip(o.dsum);
  o.rdz = make_recip(dz);
  o.rdx = make_recip(dx);
  o.rdy = make_recip(dy);
  return o;
}

struct Source3 {
  double zsa, xsa, ysa, vzero;
  int zsi, xsi, ysi, pad;
};

// t_ana / t_anad, _fteik3d.py:10-35.
__device__ __forceinline__ double t_ana3(int i, int j, int k, const Ops3& o, const Source3& s) {
  double a = o.dz * ((double)i - s.zsa);
  double b = o.dx * ((double)j - s.xsa);
  double c = o.dy * ((double)k - s.ysa);
  return s.vzero * sqrt(a * a + b * b + c * c);
}
__device__ __forceinline__ double t_anad3(int i, int j, int k, const Ops3& o, const Source3& s,
                                          double& tzc, double& txc, double& tyc) {
  double t = t_ana3(i, j, k, o, s);
  if (t > 0.0) {
    double tmp = s.vzero * s.vzero / t;
    tzc = ((double)i - s.zsa) * o.dz * tmp;
    txc = ((double)j - s.xsa) * o.dx * tmp;
    tyc = ((double)k - s.ysa) * o.dy * tmp;
  } else {
    tzc = txc = tyc = 0.0;
  }
  return t;
}

// Slowness-only operator coefficients, the same for every source and sweep,
// computed once per solve by coef3d_kernel.  Node-shaped arrays with node
// strides; the index in brackets is where the update reads them, with
// (i1, j1, k1) the reference's upwind cell (i - sgnvz, ...):
//   z1[i1][j][k]   = dz * min of the 4 cells of row i1 around column (j, k)
//   x1[i][j1][k], y1[i][j][k1]: the same along x and y      (_fteik3d.py:76-102)
//   zx?[i1][j1][k] from v = min(s[i1,j1,max(k-1,0)], s[i1,j1,min(k,ny-2)]):
//        a = dx*v, b = dz*v, q = 4*v^2*(dz2i+dx2i)           (_fteik3d.py:109-117)
//   zy?[i1][j][k1], xy?[i][j1][k1]: the ZY and XY planes     (_fteik3d.py:121-141)
//   t3[i1][j1][k1] = s^2 * dsum * 9                          (_fteik3d.py:148,153)
struct Coef3 {
  double *z1, *x1, *y1, *zxa, *zxb, *zxq, *zya, *zyb, *zyq, *xya, *xyb, *xyq, *t3;
};
constexpr int kNumCoef = 13;

struct Layout3 {
  size_t status, params, src, order, progress, coef, rec, total;
};

inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

inline Layout3 layout3(int nz, int nx, int ny, int nsrc, int grad) {
  const size_t npen = (size_t)max_pencils(nx + 1, ny + 1);
  const size_t nodes = (size_t)(nz + 1) * (nx + 1) * (ny + 1);
  Layout3 L;
  size_t off = 0;
  L.status = off;  // int status; unsigned ticket; int no_skip
  off = align_up(off + 16);
  L.params = off;
  off = align_up(off + sizeof(Source3) * (size_t)nsrc);
  L.src = off;
  off = align_up(off + sizeof(double) * 3 * (size_t)nsrc);
  L.order = off;
  off = align_up(off + sizeof(int) * npen);
  L.progress = off;
  off = align_up(off + sizeof(unsigned) * npen * nsrc);
  L.coef = off;
  off = align_up(off + sizeof(double) * nodes * kNumCoef);
  L.rec = off;
  if (grad) off = align_up(off + nodes * (size_t)nsrc);
  L.total = off;
  return L;
}

}  // namespace fteik
