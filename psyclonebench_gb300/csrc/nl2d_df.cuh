// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi) / 2, carrying about 48 significant bits
// (relative rounding error near 2^-47 per operation instead of FP64's
// 2^-53), computed on the FP32 pipe.  The error-free building blocks are
// the published ones: Knuth's TwoSum (The Art of Computer Programming,
// vol. 2, 4.2.2), Dekker's Fast2Sum and an FMA-based exact product (Dekker
// 1971, "A floating-point technique for extending the available
// precision"; Muller et al., Handbook of Floating-Point Arithmetic, ch. 4).
// Every operation is an explicit round-to-nearest intrinsic, so no compiler
// contraction or reassociation can change them.
#pragma once
#include <cuda_runtime.h>

namespace nl2d {
namespace dfk {

struct df {
  float hi, lo;
};

// a + b exactly as s + e (Knuth's TwoSum, no condition on the operands)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// a + b exactly as s + e when |a| >= |b| or a == 0 (Dekker's Fast2Sum)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df dadd(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s, e);
}

__device__ __forceinline__ df dneg(df a) { return df{-a.hi, -a.lo}; }

__device__ __forceinline__ df dsub(df a, df b) { return dadd(a, dneg(b)); }

// a * b: the exact product of the high parts by FMA, plus the cross terms
__device__ __forceinline__ df dmul(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// a * b left unnormalised: the product of the high parts, its exact error
// by FMA and all three cross terms (lo * lo too, so that chains of such
// products lose nothing), without the closing Fast2Sum: 5 instructions
// instead of 7.  |lo| stays within a few 2^-24 |hi|, which every consumer
// takes: dadd and the sums below renormalise, dmul / dmul_u add the cross
// terms in FP32 (relative error 2^-24 of a term below 2^-21 of the product),
// the upwind sign test reads hi's sign (unchanged while |lo| < |hi|) and
// join_bits adds the two halves exactly before rounding.
__device__ __forceinline__ df dmul_u(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(a.lo, b.lo, e);
  return df{p, e};
}

// a + b + c and a + b + c + d in one pass, the cascade of Ogita, Rump and
// Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005,
// Sum2): the high parts summed by TwoSum, their rounding errors and the low
// parts gathered in one FP32 accumulator, one Fast2Sum at the end (19 and
// 27 instructions against 22 and 33 for chained dadd).
__device__ __forceinline__ df dsum3(df a, df b, df c) {
  float s, e1, e2;
  two_sum(a.hi, b.hi, s, e1);
  two_sum(s, c.hi, s, e2);
  const float t = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), __fadd_rn(a.lo, b.lo)), c.lo);
  return fast_two_sum(s, t);
}

__device__ __forceinline__ df dsum4(df a, df b, df c, df d) {
  float s, e1, e2, e3;
  two_sum(a.hi, b.hi, s, e1);
  two_sum(s, c.hi, s, e2);
  two_sum(s, d.hi, s, e3);
  const float t = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), __fadd_rn(e3, __fadd_rn(a.lo, b.lo))),
                            __fadd_rn(c.lo, d.lo));
  return fast_two_sum(s, t);
}

// a * c for an FP32 c (exactly representable constants such as 0.5)
__device__ __forceinline__ df dmulf(df a, float c) {
  const float p = __fmul_rn(a.hi, c);
  float e = __fmaf_rn(a.hi, c, -p);
  e = __fmaf_rn(a.lo, c, e);
  return fast_two_sum(p, e);
}

// exact multiplication by a power of two
__device__ __forceinline__ df dhalf(df a) { return df{0.5f * a.hi, 0.5f * a.lo}; }

__host__ __device__ inline df from_double(double x) {
  const float hi = (float)x;
  return df{hi, (float)(x - (double)hi)};
}

__device__ __forceinline__ double to_double(df a) { return (double)a.hi + (double)a.lo; }

// The same two conversions without the FP64 pipe, for kernels that convert
// every value they load and store: on GB300 the FP64 pipe issues about 1.7
// operations per clock per SM, the integer and FP32 pipes over 60 each, and
// the hardware conversions between FP64 and FP32 run on the FP64 pipe.
//
// split_bits(x): hi is x truncated to 24 significant bits, built from the
// bit pattern (exponent rebiased from 1023 to 127, the top 23 mantissa bits
// kept); lo is the next 29 bits rounded to 23 and made a float exactly (the
// 2^23 exponent trick: the float with bits 0x4B000000 + m is 2^23 + m for
// m <= 2^23) and scaled by a power of two; Fast2Sum normalises the pair.
// 47 of the 53 significant bits are kept (relative error below 2^-46).  Out
// of range, without branches: |x| < 2^-80 keeps hi only (lo would leave the
// FP32 normal range), |x| < 2^-126 gives a signed zero, |x| >= 2^127 an
// infinity (so that hi + lo cannot round past the largest float) and a NaN
// a NaN.
__device__ __forceinline__ df split_bits(double x) {
  unsigned lw, hw;
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lw), "=r"(hw) : "d"(x));
  const unsigned sign = hw & 0x80000000u;
  const unsigned e = (hw >> 20) & 0x7ffu;
  // bits 31..23 of the funnel shift are e mod 512; subtracting 384 << 23
  // leaves e - 896 there for 897 <= e <= 1149
  const unsigned hb_n = (__funnelshift_l(lw, hw, 3) - 0xC0000000u) | sign;
  const bool nan = e == 0x7ffu && ((hw & 0xfffffu) | lw) != 0u;
  const unsigned hb = e - 897u <= 1149u - 897u ? hb_n
                      : e > 1149u ? (sign | 0x7f800000u | (nan ? 0x400000u : 0u))
                                  : sign;
  const unsigned r23 = ((lw & 0x1fffffffu) + 32u) >> 6;  // 0 .. 2^23
  const float m = __fsub_rn(__uint_as_float(0x4B000000u + r23), 8388608.0f);
  const float scale = __uint_as_float((e - 942u) << 23);  // 2^(e - 1069)
  const float lo_n = __uint_as_float(__float_as_uint(__fmul_rn(m, scale)) | sign);
  const float lo = e - 943u <= 1149u - 943u ? lo_n : __uint_as_float(sign);
  return fast_two_sum(__uint_as_float(hb), lo);
}

// f widened exactly to FP64 from its bit pattern (exponent rebiased from
// 127 to 1023, mantissa moved up 29 bits); zeros and subnormals give a
// signed zero, infinities and NaN the same in FP64.
__device__ __forceinline__ double widen_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned sign = b & 0x80000000u;
  const unsigned ef = (b >> 23) & 0xffu;
  const unsigned hw_n = sign | (((b >> 3) & 0x0fffffffu) + (896u << 20));
  const unsigned hw = ef - 1u <= 253u ? hw_n
                      : ef == 0u ? sign
                                 : (sign | 0x7ff00000u | ((b & 0x7fffffu) ? 0x80000u : 0u));
  const unsigned lw = ef - 1u <= 253u ? b << 29 : 0u;
  double x;
  asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lw), "r"(hw));
  return x;
}

// hi + lo rounded to FP64: one FP64 add.
__device__ __forceinline__ double join_bits(df a) {
  return __dadd_rn(widen_bits(a.hi), widen_bits(a.lo));
}

// The sign test of an upwind switch: the sign of the value, which is the
// sign of hi for a normalised pair.
__device__ __forceinline__ bool dneg_sign(df a) { return a.hi < 0.f; }

}  // namespace dfk
}  // namespace nl2d
