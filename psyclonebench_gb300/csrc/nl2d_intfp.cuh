// IEEE binary64 addition and multiplication on the integer pipes.
//
// The FP64 pipe of GB300 issues ~1.8 operations per clock per SM and the
// integer pipes ~60 each, so an exact add or multiply in integer arithmetic
// (a few dozen instructions) looked like a way to move work off the FP64
// pipe of the FP64-bound kernels.  It is exact (nl2d_selftest_intfp: no
// mismatch on 2^28 adversarial pairs) and in isolation it adds throughput
// (the pipe-rate probe: dadd_i 0.86 and dmul_i 1.23 operations per clock
// per SM next to the FP64 pipe's 1.8), but inside the kernels it loses:
// moving the fused step's phase-1 multiplications here took a 4096^2 step
// from 6.66 to 7.12 ms, and the tracer's flux multiplications from 2.15 to
// 2.64 ms per iteration.  The step kernels therefore do not use it; the
// self-test and the probe keep the measurement reproducible.
#pragma once
#include <cuda_runtime.h>

#include "nl2d_exact.cuh"

// dadd_i / dmul_i return the bits of a + b / a * b rounded to nearest even,
// for every input: normal operands and zeros take the integer path (a 53-bit
// significand with 10 guard bits and a sticky bit, the textbook soft-float
// construction); subnormal, infinite and NaN operands, and results that
// overflow or fall below the normal range, take the IEEE operation out of
// line.
namespace nl2d {
static __device__ __noinline__ double dadd_ieee(double a, double b) { return a + b; }
static __device__ __noinline__ double dmul_ieee(double a, double b) { return a * b; }

constexpr unsigned long long kI_SIGN = 0x8000000000000000ULL;
constexpr unsigned long long kI_MAG = 0x7fffffffffffffffULL;
constexpr unsigned long long kI_FRAC = 0x000fffffffffffffULL;
constexpr unsigned long long kI_HID = 0x0010000000000000ULL;

// r holds the significand with its leading one at bit 62 and guard / sticky
// bits below bit 10; e the biased exponent.  Round to nearest even and pack,
// or 0 for "out of range" (the caller falls back): a result below the normal
// range rounds at a fixed position, not at 53 bits, so it is left to the
// IEEE operation whatever its rounding would give.
__device__ __forceinline__ unsigned long long round_pack(unsigned long long sign,
                                                         unsigned long long r, int e) {
  if (e <= 0 || e >= 2047) return 0;
  unsigned long long q = r >> 10;
  const unsigned rem = (unsigned)(r & 0x3ff);
  if (rem > 0x200u || (rem == 0x200u && (q & 1ull))) {
    q += 1;
    if (q >> 53) {
      q >>= 1;
      e += 1;
    }
  }
  if (e <= 0 || e >= 2047) return 0;
  return sign | ((unsigned long long)e << 52) | (q & kI_FRAC);
}

__device__ __forceinline__ double dadd_i(double a, double b) {
  unsigned long long ua = (unsigned long long)bits(a), ub = (unsigned long long)bits(b);
  unsigned long long ma = ua & kI_MAG, mb = ub & kI_MAG;
  int ea = (int)(ma >> 52), eb = (int)(mb >> 52);
  if (mb == 0 && ea != 2047) {  // b = +-0, a finite: a, or a signed zero
    if (ma != 0) return a;
    return from_bits((long long)(ua & ub & kI_SIGN));
  }
  if (ma == 0 && eb != 2047) return b;  // a = +-0, b finite and not zero
  if (ea == 0 || eb == 0 || ea == 2047 || eb == 2047) return dadd_ieee(a, b);
  if (ma < mb) {  // |a| >= |b| from here
    unsigned long long t = ua; ua = ub; ub = t;
    t = ma; ma = mb; mb = t;
    int te = ea; ea = eb; eb = te;
  }
  const unsigned long long fa = ((ma & kI_FRAC) | kI_HID) << 10;
  unsigned long long fb = ((mb & kI_FRAC) | kI_HID) << 10;
  const int d = ea - eb;
  if (d >= 63) fb = 1;  // only a sticky bit is left
  else if (d > 0) fb = (fb >> d) | ((fb << (64 - d)) != 0 ? 1ull : 0ull);
  unsigned long long r;
  int e = ea;
  if ((long long)(ua ^ ub) >= 0) {  // same sign
    r = fa + fb;
    if (r >> 63) {
      r = (r >> 1) | (r & 1ull);
      e += 1;
    }
  } else {
    r = fa - fb;
    if (r == 0) return 0.0;  // x - x = +0 when rounding to nearest
    const int lz = __clzll((long long)r) - 1;
    r <<= lz;
    e -= lz;
  }
  const unsigned long long p = round_pack(ua & kI_SIGN, r, e);
  return p ? from_bits((long long)p) : dadd_ieee(a, b);
}

__device__ __forceinline__ double dmul_i(double a, double b) {
  const unsigned long long ua = (unsigned long long)bits(a), ub = (unsigned long long)bits(b);
  const unsigned long long ma = ua & kI_MAG, mb = ub & kI_MAG;
  const int ea = (int)(ma >> 52), eb = (int)(mb >> 52);
  const unsigned long long sign = (ua ^ ub) & kI_SIGN;
  if ((ma == 0 && eb != 2047) || (mb == 0 && ea != 2047))
    return from_bits((long long)sign);  // a zero times a finite value
  if (ea == 0 || eb == 0 || ea == 2047 || eb == 2047) return dmul_ieee(a, b);
  const unsigned long long fa = ((ma & kI_FRAC) | kI_HID) << 11;
  const unsigned long long fb = ((mb & kI_FRAC) | kI_HID) << 11;
  const unsigned long long hi = __umul64hi(fa, fb);  // the product's top 64 of 128 bits
  const unsigned long long sticky = (fa * fb) != 0 ? 1ull : 0ull;
  int e = ea + eb - 1023;
  unsigned long long r;
  if (hi >> 63) {
    r = (hi >> 1) | (hi & 1ull) | sticky;
    e += 1;
  } else {
    r = hi | sticky;
  }
  const unsigned long long p = round_pack(sign, r, e);
  return p ? from_bits((long long)p) : dmul_ieee(a, b);
}
}  // namespace nl2d
