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

// The sign test of an upwind switch: the sign of the value, which is the
// sign of hi for a normalised pair.
__device__ __forceinline__ bool dneg_sign(df a) { return a.hi < 0.f; }

}  // namespace dfk
}  // namespace nl2d
