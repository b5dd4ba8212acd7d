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
  return s.vzero * sqrt_rn(a * a + b * b + c * c);
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

// ---- the adjoint's tape ------------------------------------------------------
//
// What the reverse pass needs from the forward sweeps, per source and node:
// in which sweeps the node changed, with the code of the operator that
// changed it (the reference's ttsgn triple, _fteik3d.py:166-200), and the
// value each change replaced.  Most nodes change two or three times in all
// (about 95% on layered and gradient models at nsweep 2), so the replaced
// values are kept compactly:
//   code [nsrc][nodes][E]  E = 8 * nsweep bytes per node, 255 = unchanged in
//                          that sweep; the count of changes before sweep e is
//                          the count of codes != 255 at sweeps < e
//   hist [nsrc][nodes][H]  the value replaced by the node's 2nd .. (H+1)-th
//                          change (its first change replaces the initial
//                          value: Big, or the analytic value of the 8 nodes
//                          around the source, kept in init8)
//   table                  later changes (rare): an open-addressing table of
//                          (source node, change number) -> replaced value,
//                          capacity a power of 2 >= nodes * nsrc / 4; when a
//                          probe sequence runs past kTapeProbes the solve
//                          reports FTEIK_TAPE_OVERFLOW (the caller retries
//                          with a larger H; H = E - 1 never needs the table)
//   init8 [nsrc][8]        the initial values of the nodes around the source
//   params [nsrc]          each source's set-up (Source3), for the adjoint
constexpr int kTapeProbes = 64;
constexpr int kTapeMaxEpochs = 4095;  // change numbers fit in the key's 12 bits

struct Tape3 {
  uint8_t* code;
  double* hist;
  unsigned long long* key;  // 0: empty slot, else ((source node) << 12 | change) + 1
  double* val;
  double* init8;
  Source3* params;
  unsigned long long mask;  // table capacity - 1
  int E, H;
  // Added to a source-node index before it forms a table key: a tape viewed
  // from its source src0 on (code, hist, init8 and params shifted by src0)
  // has sn0 = src0 * nodes, so its keys stay those the solve wrote.
  long long sn0;
};

struct TapeLayout {
  size_t code, hist, key, val, init8, params, total;
  unsigned long long cap;
};

inline TapeLayout tape_layout(int nz, int nx, int ny, int nsrc, int nsweep, int history) {
  const size_t N = (size_t)(nz + 1) * (nx + 1) * (ny + 1) * (size_t)nsrc;
  const size_t E = 8 * (size_t)nsweep;
  TapeLayout L;
  unsigned long long cap = 4096;
  while (cap < N / 4) cap <<= 1;
  L.cap = cap;
  size_t off = 0;
  L.code = off;
  off = align_up(off + N * E);
  L.hist = off;
  off = align_up(off + N * (size_t)history * 8);
  L.key = off;
  off = align_up(off + cap * 8);
  L.val = off;
  off = align_up(off + cap * 8);
  L.init8 = off;
  off = align_up(off + (size_t)nsrc * 64);
  L.params = off;
  off = align_up(off + (size_t)nsrc * sizeof(Source3));
  L.total = off;
  return L;
}

inline Tape3 tape_at(void* base, const TapeLayout& L, int nsweep, int history) {
  char* b = (char*)base;
  Tape3 t;
  t.code = (uint8_t*)(b + L.code);
  t.hist = (double*)(b + L.hist);
  t.key = (unsigned long long*)(b + L.key);
  t.val = (double*)(b + L.val);
  t.init8 = (double*)(b + L.init8);
  t.params = (Source3*)(b + L.params);
  t.mask = L.cap - 1;
  t.E = 8 * nsweep;
  t.H = history;
  t.sn0 = 0;
  return t;
}

__device__ __forceinline__ unsigned long long tape_key(long long sn, int m) {
  return (((unsigned long long)sn << 12) | (unsigned)m) + 1ull;
}
// First probe slot of a key: MurmurHash3's 64-bit finaliser (fmix64, public
// domain), so neighbouring nodes spread over the whole table.
__device__ __forceinline__ unsigned long long tape_slot(unsigned long long key,
                                                        unsigned long long mask) {
  unsigned long long h = key;
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h & mask;
}

// Number of sweeps before sweep e (e < E) in which the node with this code
// record changed.  E is a multiple of 8 and rec is 8-byte aligned.
__device__ __forceinline__ int tape_changes_before(const uint8_t* rec, int e) {
  int m = 0;
  for (int w = 0; w * 8 < e; ++w) {
    const unsigned long long x = __ldcg((const unsigned long long*)rec + w);
    const int nb = e - w * 8 < 8 ? e - w * 8 : 8;
#pragma unroll
    for (int b = 0; b < 8; ++b)
      if (b < nb) m += ((x >> (8 * b)) & 0xffull) != 0xffull;
  }
  return m;
}

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
