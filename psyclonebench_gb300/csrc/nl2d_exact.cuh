// Exact FP64 building blocks for the fused NEMOLite2D step.
//
// On GB300 the FP64 pipe issues 2 thread-operations per clock per SM, ~60x
// fewer than the integer and FP32 pipes, and an IEEE FP64 divide costs ~15
// FP64 instructions.  Each helper below returns the SAME bits as the plain
// IEEE expression it replaces, for every input, but spends fewer FP64
// instructions:
//
//  * div_rn(x, d, r): x / d rounded to nearest for a divisor d > 0 whose
//    reciprocal r = RN(1/d) was computed beforehand.  q0 = RN(x * r) is
//    within 1.5 ulp of x / d; one exact FMA remainder e0 = q0 * d - x,
//    compared as an integer with half an ulp of q0 times d, picks the
//    correctly rounded quotient among q0 and its two neighbours.  1 DMUL +
//    1 DFMA.  When q0 is a power of two (the spacing changes below it) the
//    quotient takes Markstein's two refinements instead (Markstein,
//    "Computation of elementary functions on the IBM RISC System/6000
//    processor", IBM J. Res. Dev. 34(1), 1990; Muller et al., Handbook of
//    Floating-Point Arithmetic, 2nd ed., Sec. 4.7), 1 DMUL + 4 DFMA.
//    x = +-0 returns x.  Dividends whose magnitude is tiny (below 2^-899,
//    other than zero), huge (2^900 and above) or not finite use the IEEE
//    divide, so no intermediate underflows or overflows; divisors are
//    checked on the host to lie in [2^-100, 2^100].
//  * half(x): 0.5 * x.  For normal x with a biased exponent >= 2 this is
//    exact, i.e. the exponent minus one, done in integer arithmetic; zero
//    keeps its bits; subnormal, smallest-normal and non-finite x use DMUL.
//  * upwind(w, p, q): (0.5 - copysign(0.5, w)) * p + (0.5 + copysign(0.5, w)) * q,
//    the first-order upwind pick of momentum_{u,v}_kern.c.  One weight is
//    1 and the other +0, so the value is the picked operand plus a zero
//    carrying the sign of the other operand; that is the picked operand,
//    or a zero whose sign is the AND of both signs.  Integer select; a
//    non-finite partner takes the IEEE expression.
#pragma once
#include <cuda_runtime.h>

namespace nl2d {

// A double's bit pattern and back.  Moved through inline PTX so the
// compiler treats the integer work on the bits as integer work: through a
// plain bitcast it may rewrite bits(x) & 0x7fff... as fabs(x), a sign-bit
// merge as copysign and a zero test as an FP64 compare, and on GB300 those
// run on the FP64 pipe the helpers are there to spare.  (The move itself
// costs nothing: both sides live in the same 64-bit register pair.)
__device__ __forceinline__ long long bits(double x) {
  long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}
__device__ __forceinline__ double from_bits(long long b) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(b));
  return x;
}
// The IEEE expressions the helpers fall back to, kept out of line: inlined,
// the compiler may predicate them and issue their FP64 instructions on every
// call, taken or not; as calls behind a branch they cost nothing when not
// taken.
static __device__ __noinline__ double div_ieee(double x, double d) { return x / d; }
static __device__ __noinline__ double half_ieee(double x) { return 0.5 * x; }
static __device__ __noinline__ double pick_ieee(double a, double z) { return a + 0.0 * z; }

// Markstein's two refinements: a faithful quotient, then the correctly
// rounded one.  Out of line: taken only when x * r lands on a power of two.
static __device__ __noinline__ double div_markstein(double x, double d, double r) {
  const double q0 = x * r;
  const double e0 = fma(q0, d, -x);
  const double q1 = fma(-e0, r, q0);
  const double e1 = fma(q1, d, -x);
  return fma(-e1, r, q1);
}

__device__ __forceinline__ double div_rn(double x, double d, double r) {
  const long long xb = bits(x);
  if ((xb & 0x7fffffffffffffffLL) == 0) return x;  // +-0 / d keeps the sign for d > 0
  const int ex = (int)((xb >> 52) & 0x7ff);
  if (ex < 124 || ex > 1922) return div_ieee(x, d);
  const double q0 = x * r;
  const long long qb = bits(q0);
  if ((qb & 0xfffffffffffffLL) == 0) return div_markstein(x, d, r);
  // q0 is not a power of two, so q = x / d lies in q0's binade and within
  // 1.5 ulp of it: RN(q) is q0 - ulp, q0 or q0 + ulp.  The remainder
  // e0 = q0 * d - x = d * (q0 - q) is exact wherever it decides (|e0| <
  // 2^53 units of its grid), and RN(q) moves off q0 exactly when |e0| >
  // h = d * ulp(q0) / 2 (a quotient is never a midpoint).  h is d with
  // its exponent shifted, compared as a bit pattern.
  const double e0 = fma(q0, d, -x);
  const long long eb = bits(e0);
  const int eq = (int)((qb >> 52) & 0x7ff);
  const long long hb = bits(d) + ((long long)(eq - 1076) << 52);
  long long k = 0;  // +1: one ulp up in value, -1: one ulp down
  if ((eb & 0x7fffffffffffffffLL) > hb) k = (eb < 0) ? 1 : -1;
  return from_bits(qb + (qb < 0 ? -k : k));
}

__device__ __forceinline__ double half(double x) {
  const long long b = bits(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex >= 2 && ex <= 2046) return from_bits(b - (1LL << 52));
  if ((b & 0x7fffffffffffffffLL) == 0) return x;
  return half_ieee(x);
}

// a + (+0 * z): the operand with weight 1 plus the zero-weighted partner.
__device__ __forceinline__ double pick(double a, double z) {
  const long long ab = bits(a), zb = bits(z);
  if (((zb >> 52) & 0x7ff) == 0x7ff) return pick_ieee(a, z);
  if ((ab & 0x7fffffffffffffffLL) != 0) return a;
  return from_bits(ab & (zb | 0x7fffffffffffffffLL));
}

__device__ __forceinline__ double upwind(double w, double p, double q) {
  return (bits(w) < 0) ? pick(p, q) : pick(q, p);
}

}  // namespace nl2d
