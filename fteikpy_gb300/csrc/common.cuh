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
//  * division by a constant c > 0 (or a divisor shared by several quotients)
//    multiplies by y = RN(1/c) and settles the last bit with Tuckerman's
//    rounding test on the FMA remainder (div_tk, two FP64 instructions), or
//    corrects a double-double quotient (div_dd, four, fewer registers);
//  * the square root takes a float seed, a fixed-point Newton step on the
//    integer pipe, one coupled FP64 Newton step and the same rounding test
//    (sqrt_rn, four FP64 instructions).
// Both return IEEE's correctly rounded result, bit for bit; the bitwise tests
// against the oracle, which uses IEEE `/` and sqrt, check them on every solve.
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
// -x, or x with its sign flipped when `flip`, on the integer pipe (an FP64
// negation that is not folded into its consumer takes an FP64 instruction).
__device__ __forceinline__ double dneg(double x) {
  return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}
__device__ __forceinline__ double dflip(double x, bool flip) {
  return __hiloint2double(__double2hiint(x) ^ (flip ? (int)0x80000000 : 0), __double2loint(x));
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

// ---- correctly rounded square root with four FP64 instructions ------------------
//
// sqrt_rn(x) returns the same bits as IEEE sqrt (RN(sqrt(x))), which the
// reference's `x ** 0.5` is, with most of the work off the FP64 pipe:
//  1. x = x' 2^(2k) with x' in [1, 4) (exponent arithmetic), so sqrt(x) =
//     sqrt(x') 2^k exactly.
//  2. y0 = rsqrtf of x' rounded down to float (a relative error of at most
//     about 2^-21.7: 2^-24 from the truncation, and rsqrtf's documented
//     2 ulp).
//  3. One Newton step for 1/sqrt(x'), y1 = y0 (3 - x' y0^2) / 2, in 32- and
//     64-bit fixed point on the integer pipe: a relative error e1 below
//     about 2^-28 (the truncations; the step's own term 1.5 e0^2 is ~2^-42).
//  4. One step of the coupled Newton iteration for sqrt and 1/(2 sqrt)
//     (P. Markstein, IBM J. Res. Dev. 34(1), 1990): g = RN(x' y1),
//     h = y1 / 2, r = RN(0.5 - g h), g1 = RN(g + g r).  As g and h come from
//     the same y1, g (1 + r) = sqrt(x') (1 + eta/2 - 1.5 e1^2 + ...) with
//     |eta| <= 2^-53 the rounding of g: before its own rounding g1 is within
//     0.5 + 0.14 ulp of sqrt(x') (ulp = 2^-52, sqrt(x') < 2), so
//     |g1 - sqrt(x')| < 1.2 ulp.
//  5. Tuckerman's rounding test: with ulp = 2^-52 (g1 in [1, 2)) every
//     quantity below is a multiple of ulp^2, so sqrt(x') > g1 + ulp/2 exactly
//     when d = x' - g1^2 > g1 ulp, and sqrt(x') < g1 - ulp/2 exactly when
//     d <= -g1 ulp (sqrt is never exactly a midpoint).  d = RN(x' - g1^2) is
//     one FMA (computed as its negation, RN(g1^2 - x'), so that no operand
//     needs an FP64 negation); comparing it with the double u = g1 ulp decides every case
//     except RN(d) = +-u, where d itself might differ from RN(d).  As g1 is
//     within 1.5 ulp, the result is g1 - ulp, g1 or g1 + ulp.
// Zero, subnormal, negative, infinite or NaN inputs, a g1 outside [1, 2) and
// the RN(d) = +-u case take CUDA's sqrt instead (rare: the last two need
// x' within an ulp or so of 1 or 4, or sqrt(x') within ~2^-104 of a
// midpoint).  The kernels' tests compare every result bitwise with the
// oracle's IEEE sqrt, and a dedicated test compares sqrt_rn with CUDA's sqrt
// on many millions of inputs, including squares and near-midpoint cases.
__device__ __forceinline__ double sqrt_fallback(double x) { return sqrt(x); }

__device__ __forceinline__ double sqrt_rn(double x) {
  const int hx = __double2hiint(x);
  const unsigned lx = (unsigned)__double2loint(x);
  const int ex = hx >> 20;  // biased exponent; negative x gives ex < 0
  const int k = (ex - 1023) >> 1;
  const int s = (ex - 1023) & 1;  // x' = x 2^-2k in [1, 2) (s = 0) or [2, 4) (s = 1)
  const unsigned mant = (unsigned)hx & 0xfffffu;
  // x' in fixed point with 30 fraction bits (truncated), and as a float
  // rounded down
  const unsigned M = mant | 0x100000u;
  const unsigned X = (M << (10 + s)) | (lx >> (22 - s));
  const float xf = __int_as_float(((127 + s) << 23) | (int)((mant << 3) | (lx >> 29)));
  const float y0 = rsqrtf(xf);  // in (0.5, 1]
  // y0 in fixed point with 31 fraction bits (exact: y0 has 24 bits)
  const int fy = __float_as_int(y0);
  const unsigned Y = ((unsigned)(fy & 0x7fffff) | 0x800000u) << ((fy >> 23) - 119);
  // y1 = y0 (3 - x' y0^2) / 2
  const unsigned P = (unsigned)(((unsigned long long)Y * Y) >> 31);  // y0^2 2^31
  const unsigned long long Q = (unsigned long long)X * P;             // x' y0^2 2^61
  const unsigned E = (unsigned)(((3ull << 61) - Q) >> 31);            // (3 - x' y0^2) 2^30
  const unsigned R = (unsigned)(((unsigned long long)Y * E) >> 32);   // y1 2^30
  // y1 as a double: R in (2^29, 2^30 (1 + 2^-28)), leading bit 29 or 30
  const int lz = __clz((int)R);
  const unsigned frac = (R << lz) << 1;  // the bits after the leading one
  const double y = __hiloint2double(((1024 - lz) << 20) | (int)(frac >> 12), (int)(frac << 20));
  // x' and -x', and -y/2, built from bit patterns: an FP64 negation that
  // the compiler does not fold into an FMA costs a whole FP64 instruction
  const int hxs = ((1023 + s) << 20) | (int)mant;
  const double xs = __hiloint2double(hxs, (int)lx);
  const double nxs = __hiloint2double(hxs | (int)0x80000000, (int)lx);
  const double g = __dmul_rn(xs, y);
  const double nh = __hiloint2double((__double2hiint(y) - (1 << 20)) | (int)0x80000000,
                                     __double2loint(y));  // -y/2
  const double r = __fma_rn(g, nh, 0.5);
  const double g1 = __fma_rn(g, r, g);
  const double nd = __fma_rn(g1, g1, nxs);  // RN(g1^2 - x') = -RN(x' - g1^2)
  const int hg = __double2hiint(g1);
  // |d| against u = g1 2^-52 > 0 by bit patterns, d's sign giving the
  // direction.  Both patterns are assembled from 32-bit words: a 64-bit mask
  // of the sign bit is compiled as an FP64 absolute value (an FP64
  // instruction).
  const long long bu = ((long long)(hg - (52 << 20)) << 32) | (unsigned)__double2loint(g1);
  const int hd = __double2hiint(nd);
  const long long ad = ((long long)(hd & 0x7fffffff) << 32) | (unsigned)__double2loint(nd);
  const bool ok = ex > 0 && ex < 2047 && (hg >> 20) == 1023 && ad != bu;
  if (!ok) return sqrt_fallback(x);
  const long long gb = __double_as_longlong(g1) + (ad > bu ? (hd < 0 ? 1 : -1) : 0);
  return __longlong_as_double(gb + ((long long)k << 52));
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

// ---- correctly rounded division with two FP64 instructions ------------------------
//
// div_tk(x, c, nc, y) = RN(x / c) for c > 0 given nc = -c and y = RN(1/c), by Tuckerman's
// rounding test (as sqrt_rn above):
//  * q0 = RN(x y) is within 1.5 ulp of x/c: x y = (x/c)(1 + e) with
//    |e| < 2^-53, so |x y - x/c| < ulp(q0) (at most a hair more where x/c
//    crosses a power of two above q0, which leaves q0 + ulp the right
//    result), plus half an ulp for the rounding.  RN(x/c) is therefore
//    q0 - ulp, q0 or q0 + ulp in value.
//  * x/c > q0 + ulp/2 exactly when the remainder x - c q0 > c ulp/2, and
//    x/c < q0 - ulp/2 exactly when it is < -c ulp/2; a quotient of two
//    doubles is never a midpoint (its odd part would exceed 2^53).
//    rem = RN(x - c q0) is one FMA and c ulp/2 a double (c scaled by a
//    power of two), and RN keeps the order of each comparison, so they
//    decide every case but RN(rem) = +-c ulp/2.
// That case, a q0 that is zero, subnormal, infinite, NaN or a power of two
// (its lower neighbour is half an ulp away), and a c ulp/2 outside the
// normal range take the IEEE division.  The bitwise tests against the
// oracle, which divides with IEEE `/`, check it on every solve, and a
// dedicated test compares it with IEEE division on many millions of inputs.
// The rounding test on a quotient q0 within 1.5 ulp of x / c (c > 0, nc = -c):
// returns RN(x / c) through `bits`, or false where IEEE division must decide.
__device__ __forceinline__ bool tk_round(double x, double q0, double c, double nc,
                                         long long& bits) {
  const double rem = __fma_rn(q0, nc, x);  // x - c q0 (nc = -c: no FP64 negation)
  const long long bq = __double_as_longlong(q0);
  const int eq = (int)((bq >> 52) & 0x7ff);
  const int hc = __double2hiint(c);
  const int eh = ((hc >> 20) & 0x7ff) + eq - 1076;  // exponent field of c ulp(q0) / 2
  // c ulp(q0) / 2 (a power-of-two scaling of c), and |rem| against it by bit
  // patterns, rem's sign giving the direction; both assembled from 32-bit
  // words (a 64-bit mask of the sign bit is compiled as an FP64 absolute
  // value)
  const long long bh = ((long long)(hc + (eq - 1076) * (1 << 20)) << 32) |
                       (unsigned)__double2loint(c);
  const int hr = __double2hiint(rem);
  const long long ar = ((long long)(hr & 0x7fffffff) << 32) | (unsigned)__double2loint(rem);
  // one ulp away from zero when rem and q0 have the same sign, towards it
  // otherwise
  bits = bq + (ar > bh ? (((hr ^ (int)(bq >> 32)) < 0) ? -1 : 1) : 0);
  return eq > 0 && eq < 2047 && (bq & 0xfffffffffffffLL) != 0 && eh > 0 && eh < 2047 &&
         ar != bh;
}

__device__ __forceinline__ double div_tk(double x, double c, double nc, double y) {
  long long bits;
  if (!tk_round(x, __dmul_rn(x, y), c, nc, bits)) return x / c;
  return __longlong_as_double(bits);
}

// RN(1 / b) for b > 0 (the IEEE reciprocal) with three FP64 instructions:
// b = b' 2^(e-1023) with b' in [1, 2); a float seed y0 = RN_f(1 / b') from
// b' rounded down to float (relative error below 2^-22); one Newton step
// y1 = y0 (2 - b' y0) in fixed point on the integer pipe (below about
// 2^-28); one in FP64, y2 = y1 + y1 (1 - b' y1) (two FMAs; within
// 0.5 ulp + 2^-55 of 1/b'); then the rounding test above with x = 1 (one
// FMA), and the exact scaling by 2^(1023-e).  Zero, subnormal, negative,
// infinite or NaN b, a b whose reciprocal leaves the normal range, and the
// test's undecided cases take IEEE division.
__device__ __forceinline__ double recip_rn(double b) {
  const int hb = __double2hiint(b);
  const unsigned lb = (unsigned)__double2loint(b);
  const int eb = hb >> 20;  // negative b gives eb < 0
  const unsigned mant = (unsigned)hb & 0xfffffu;
  const int hbs = (1023 << 20) | (int)mant;
  const double bs = __hiloint2double(hbs, (int)lb);
  const double nbs = __hiloint2double(hbs | (int)0x80000000, (int)lb);
  const float y0 = __frcp_rn(__int_as_float((127 << 23) | (int)((mant << 3) | (lb >> 29))));
  // y0 in fixed point with 31 fraction bits (exact: y0 has 24 bits, in (0.5, 1])
  const int fy = __float_as_int(y0);
  const unsigned Y = ((unsigned)(fy & 0x7fffff) | 0x800000u) << ((fy >> 23) - 119);
  const unsigned B = 0x80000000u | (mant << 11) | (lb >> 21);          // b' 2^31
  const unsigned long long T = (unsigned long long)B * Y;               // b' y0 2^62
  const unsigned E = (unsigned)(((2ull << 62) - T) >> 31);              // (2 - b' y0) 2^31
  const unsigned R = (unsigned)(((unsigned long long)Y * E) >> 32);     // y1 2^30
  const int lz = __clz((int)R);
  const unsigned frac = (R << lz) << 1;
  const double y1 = __hiloint2double(((1024 - lz) << 20) | (int)(frac >> 12), (int)(frac << 20));
  const double e = __fma_rn(nbs, y1, 1.0);
  const double y2 = __fma_rn(y1, e, y1);
  long long bits;
  if (!tk_round(1.0, y2, bs, nbs, bits) || eb < 1 || eb > 2043) return 1.0 / b;
  return __longlong_as_double(bits + (long long)(1023 - eb) * (1LL << 52));
}

// ---- division by a per-launch constant --------------------------------------------

// Two ways to divide by a constant c > 0, both giving IEEE's RN(x / c):
//  * div_by: div_tk above, two FP64 instructions;
//  * div_dd: a double-double reciprocal hi + lo of c makes q = x hi + x lo
//    (one FMA) faithful, and one Markstein correction with the exact
//    remainder rounds it correctly (P. Markstein, IBM J. Res. Dev. 34(1),
//    1990): four FP64 instructions, but fewer live registers, which is what
//    the team sweep kernel's operators need (measured faster there).
struct Recip {
  double c, nc, hi, lo;  // c > 0, -c, RN(1/c), (1 - c*hi)/c
};
__host__ __device__ inline Recip make_recip(double c) {
  Recip r;
  r.c = c;
  r.nc = -c;
  r.hi = 1.0 / c;
#ifdef __CUDA_ARCH__
  r.lo = __fma_rn(-c, r.hi, 1.0) / c;
#else
  r.lo = __builtin_fma(-c, r.hi, 1.0) / c;
#endif
  return r;
}
__device__ __forceinline__ double div_dd(double x, const Recip& r) {
  double q = __fma_rn(x, r.hi, __dmul_rn(x, r.lo));
  double rem = __fma_rn(q, r.nc, x);
  return __fma_rn(rem, r.hi, q);
}
__device__ __forceinline__ double div_by(double x, const Recip& r) {
  return div_tk(x, r.c, r.nc, r.hi);
}

// RN(a / b) for several numerators sharing one divisor b > 0: the reciprocal
// is taken once.
struct SharedRecip {
  double b, nb, y;
};
__device__ __forceinline__ SharedRecip shared_recip(double b) {
  SharedRecip r;
  r.b = b;
  r.nb = dneg(b);
  r.y = recip_rn(b);
  return r;
}
__device__ __forceinline__ double div_shared(double a, const SharedRecip& r) {
  return div_tk(a, r.b, r.nb, r.y);
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
