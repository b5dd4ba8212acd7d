// Device helpers shared by the fteik_gb300 kernels (sm_103a, FP64).
//
// The kernels reproduce fteikpy's numba arithmetic operation by operation:
// `x ** 2.0` is x*x, `x ** 0.5` is the correctly rounded sqrt, every other
// operation is a single IEEE double operation in the reference's evaluation
// order, and every file that computes the reference's results is compiled
// with --fmad=false so nothing is contracted (only the adjoint's partials,
// which have no bitwise counterpart, may contract).  On GB300 the FP64 pipe is the bottleneck (about 1.2 TFLOP/s), so
// work that can leave it without changing a single result bit does:
//
//  * comparisons, min and max of doubles run on the integer pipe through an
//    order-preserving integer key of the bit pattern (exact for all non-NaN
//    values; -0.0 never arises in these kernels);
//  * tests that only bound a result (whether a node keeps its value, which
//    operators cannot win, most plane guards) are decided with float bounds
//    of the doubles on the integer and FP32 pipes (f_below / f_above), and
//    fall back to FP64 only where those cannot decide;
//  * multiplication by 0.5 or 4.0 (exact scalings) edits the exponent field;
//  * division by a per-launch constant c uses a double-double reciprocal of c
//    and one Markstein correction step: with y = RN(1/c), a quotient q within
//    one ulp of a/c (from the double-double product) and the exact remainder
//    r = a - c*q (one FMA), RN(q + r*y) is the correctly rounded a/c
//    (P. Markstein's correction theorem, IBM J. Res. Dev. 34(1), 1990; the
//    division chapter of Muller et al., Handbook of Floating-Point
//    Arithmetic). The bitwise tests against the oracle, which divides with
//    IEEE `/`, check it on every solve.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fteik {

constexpr double kBig = 1.0e5;   // fteikpy/_fteik/_fteik3d.py:6, _fteik2d.py:6
constexpr double kEps = 1.0e-15; // fteikpy/_fteik/_fteik3d.py:7, _fteik2d.py:7
constexpr int kEpsin = 5;        // fteikpy/_fteik/_fteik2d.py:8

// Status codes returned by every C-ABI entry point.
enum Status : int {
  kOk = 0,
  kSourceOutOfBound = 1,
  kEndPointOutOfBound = 2,
  kMaxStepReached = 3,
  kDeviceWaitTimeout = 4,
  kInvalidArgument = 5,
  kCudaError = 6,
  kWorkspaceTooSmall = 7,
  kTapeOverflow = 8,
};

// ---- integer-pipe comparisons -------------------------------------------------

// Order-preserving key: key(a) < key(b) <=> a < b for non-NaN doubles (with
// -0.0 ordered before +0.0, which never arises here).
__device__ __forceinline__ long long okey(double x) {
  long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool dlt(double a, double b) { return okey(a) < okey(b); }
__device__ __forceinline__ bool dle(double a, double b) { return okey(a) <= okey(b); }
// Python min/max built-ins: keep the first argument unless strictly beaten.
__device__ __forceinline__ double dmin(double a, double b) { return okey(b) < okey(a) ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return okey(b) > okey(a) ? b : a; }
// Min of two positive doubles (slowness): the raw bit patterns order like the values.
__device__ __forceinline__ double pmin(double a, double b) {
  long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  return __longlong_as_double(y < x ? y : x);
}
__device__ __forceinline__ bool deq(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}

// ---- float bounds of non-negative doubles --------------------------------------
//
// A bound test such as "RN(x + y) <= RN(u + v)" needs no FP64 addition when it
// can be decided with floats rounded the safe way: f_below(x) <= x <=
// f_above(x) for every finite x >= 0, and __fadd_rd / __fadd_ru round a float
// sum down / up, so f_above-sums <= f_below-sums implies the real sums are
// ordered, and RN keeps that order.  Both bounds are built on the integer
// pipe from x's high word: its top 20 significand bits (truncated, i.e.
// rounded down, or plus one unit, which is strictly above x), re-biased from
// double's exponent (1023) to float's (127).  Below float's normal range
// f_below is 0 (or a float that is still below x) and f_above the least
// normal float; above it f_below is the largest finite float and f_above +inf.
// The callers pass traveltimes and spacing-times-slowness factors, which are
// >= 0; for a negative x (or -0.0) f_below is -inf and f_above 0, so the
// bounds hold for every non-NaN x.
__device__ __forceinline__ float f_below(double x) {
  const int hi = __double2hiint(x);
  const int d = (int)((unsigned)hi - (896u << 20));  // wraps only for hi < 0
  const float f = __int_as_float(min(max(d, 0), (255 << 20) - 1) << 3);
  return hi < 0 ? -__int_as_float(0x7f800000) : f;
}
__device__ __forceinline__ float f_above(double x) {
  const int hi = __double2hiint(x);
  const int d = (int)((unsigned)hi - (896u << 20)) + 1;
  const float f = __int_as_float(min(max(d, 1 << 20), 255 << 20) << 3);
  return hi < 0 ? 0.0f : f;
}

// ---- exact power-of-two scalings ---------------------------------------------

// 0.5 * x, exact for zero and for |x| >= 2^-1021 (the callers' precondition,
// checked on the host from the model's scales).
__device__ __forceinline__ double half(double x) {
  long long b = __double_as_longlong(x);
  return (b & 0x7ff0000000000000LL) ? __longlong_as_double(b - (1LL << 52)) : x;
}
// 4.0 * x, exact for zero and for normal x below 2^1021.
__device__ __forceinline__ double times4(double x) {
  long long b = __double_as_longlong(x);
  return (b & 0x7ff0000000000000LL) ? __longlong_as_double(b + (2LL << 52)) : x;
}

// ---- correctly rounded division by a per-launch constant -----------------------

struct Recip {
  double c, hi, lo;  // c, RN(1/c), (1 - c*hi)/c
};
__host__ __device__ inline Recip make_recip(double c) {
  Recip r;
  r.c = c;
  r.hi = 1.0 / c;
#ifdef __CUDA_ARCH__
  r.lo = __fma_rn(-c, r.hi, 1.0) / c;
#else
  r.lo = __builtin_fma(-c, r.hi, 1.0) / c;
#endif
  return r;
}
// RN(x / c) for finite x (no overflow/underflow), as IEEE division returns.
__device__ __forceinline__ double div_by(double x, const Recip& r) {
  double q = __fma_rn(x, r.hi, __dmul_rn(x, r.lo));  // faithful quotient
  double rem = __fma_rn(-q, r.c, x);                 // exact remainder
  return __fma_rn(rem, r.hi, q);                     // Markstein correction
}

// RN(a / b) for several numerators sharing one divisor b: y = RN(1/b) and
// lo = RN((1 - b*y) * y) make y + lo a reciprocal of b accurate to about
// 2^-104, so q = a*y + a*lo (one FMA) is faithful, and the same Markstein
// correction as div_by rounds it correctly.  Numerators that are zero (the
// quotient keeps their sign), non-finite, or so small that the quotient
// could leave the normal range take the IEEE division.
struct SharedRecip {
  double b, y, lo;
};
__device__ __forceinline__ SharedRecip shared_recip(double b) {
  SharedRecip r;
  r.b = b;
  r.y = 1.0 / b;
  r.lo = __dmul_rn(__fma_rn(-b, r.y, 1.0), r.y);
  return r;
}
__device__ __forceinline__ double div_shared(double a, const SharedRecip& r) {
  const long long ba = __double_as_longlong(a) & 0x7fffffffffffffffLL;
  const int ea = (int)(ba >> 52), eb = (int)((__double_as_longlong(r.b) >> 52) & 0x7ff);
  if (ba == 0) return a;
  if (ea == 0x7ff || ea - eb < -900 || eb < 64 || eb > 1983) return a / r.b;
  const double q = __fma_rn(a, r.y, __dmul_rn(a, r.lo));
  const double rem = __fma_rn(-q, r.b, a);
  return __fma_rn(rem, r.y, q);
}

// ---- misc ------------------------------------------------------------------------

__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }
__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }

// L2-coherent loads/stores for data exchanged between warps of a running kernel.
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
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

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

}  // namespace fteik
