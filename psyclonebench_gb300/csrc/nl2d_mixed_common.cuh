// What the mixed-precision NEMOLite2D step's device code shares
// (nl2d_mixed_march.cuh): its step constants, the upwind weights and the
// compensated FP32 update of the sea-surface height.
#pragma once
#include "nl2d_internal.h"

namespace nl2d {
namespace mixk {  // separate names: the FP64 tile header uses the same ones
namespace {

// The step's constants in FP32, from the domain's uniform metrics and the
// run's scalars (make_mix_const).
struct MixConst {
  float area_t, area_u, area_v, dx_u, dx_v, dx_t, dy_u, dy_v, dy_t;
  float r_area_t, r_area_u, r_area_v, r_dx_t, r_dy_t, r_dxv2, r_dyu2, r_fric;
  float dxv2, dyu2, cor_u, cor_v, g, rdt, visc;
};

// The upwind weights 0.5 - SIGN(0.5, w) and 0.5 + SIGN(0.5, w) of the
// momentum kernels' advection terms.
__device__ __forceinline__ float wlo(float x) { return 0.5f - copysignf(0.5f, x); }
__device__ __forceinline__ float whi(float x) { return 0.5f + copysignf(0.5f, x); }

// hi + lo + delta as a new (hi, lo) pair: TwoSum, then Fast2Sum.
__device__ __forceinline__ float2 dd_add(float2 a, float delta) {
  const float s = __fadd_rn(a.x, delta);
  const float bb = __fsub_rn(s, a.x);
  const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(delta, bb));
  const float lo = __fadd_rn(a.y, err);
  const float hi = __fadd_rn(s, lo);
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

inline MixConst make_mix_const(const Scalars& s, const UniformMetrics& um) {
  MixConst k;
  k.area_t = (float)um.area_t, k.area_u = (float)um.area_u, k.area_v = (float)um.area_v;
  k.dx_u = (float)um.dx_u, k.dx_v = (float)um.dx_v, k.dx_t = (float)um.dx_t;
  k.dy_u = (float)um.dy_u, k.dy_v = (float)um.dy_v, k.dy_t = (float)um.dy_t;
  k.dxv2 = (float)(um.dx_v + um.dx_v);
  k.dyu2 = (float)(um.dy_u + um.dy_u);
  k.r_area_t = (float)(1.0 / um.area_t), k.r_area_u = (float)(1.0 / um.area_u);
  k.r_area_v = (float)(1.0 / um.area_v);
  k.r_dx_t = (float)(1.0 / um.dx_t), k.r_dy_t = (float)(1.0 / um.dy_t);
  k.r_dxv2 = (float)(1.0 / (um.dx_v + um.dx_v)), k.r_dyu2 = (float)(1.0 / (um.dy_u + um.dy_u));
  k.r_fric = (float)(1.0 / (1.0 + s.cbfr * s.rdt));
  k.cor_u = (float)(2. * s.omega * um.sin_u), k.cor_v = (float)(2. * s.omega * um.sin_v);
  k.g = (float)s.g, k.rdt = (float)s.rdt, k.visc = (float)s.visc;
  return k;
}

}  // namespace
}  // namespace mixk
}  // namespace nl2d
