// Device code of one tile of the mixed-precision NEMOLite2D step, shared by
// the single-domain kernel (nl2d_mixed.cu) and the ensemble's persistent
// kernel (nl2d_ensemble.cu).  See nl2d_mixed.cu for the arithmetic.
#pragma once
#include "nl2d_internal.h"

namespace nl2d {
namespace mixk {  // separate names: the FP64 tile header uses the same ones
namespace {


constexpr int TX = 32, TY = 8, HALO = 2;
constexpr int SX = TX + 2 * HALO, SY = TY + 2 * HALO, S0 = SX * SY;
constexpr int P1X = TX + 2, P1Y = TY + 2, S1 = P1X * P1Y;

struct MixConst {
  float area_t, area_u, area_v, dx_u, dx_v, dx_t, dy_u, dy_v, dy_t;
  float r_area_t, r_area_u, r_area_v, r_dx_t, r_dy_t, r_dxv2, r_dyu2, r_fric;
  float dxv2, dyu2, cor_u, cor_v, g, rdt, visc;
};

struct MCtx {
  const float *un, *vn, *ht, *hu, *hv, *sn;  // sn: shared, hi parts (halo 2)
  const float *rhu, *rhv;                     // 1 / (hu + ssha_u), 1 / (hv + ssha_v)
  const float *su, *sv;                       // shared sshn_u / sshn_v (halo 2)
  const int* m;                               // shared mask (halo 2)
  const double *ua_arr, *va_arr;              // FP64 reference arrays (static here)
  int W, i0, j0;
  Dims d;
  MixConst k;
  __device__ __forceinline__ int slot(int i, int j) const {
    return (j - j0 + HALO) * SX + (i - i0 + HALO);
  }
  __device__ __forceinline__ bool in_copy(int i, int j) const {
    return i >= d.xs - 1 && i <= d.xe + 1 && j >= d.ys - 1 && j <= d.ye;
  }
};

__device__ __forceinline__ float wlo(float x) { return 0.5f - copysignf(0.5f, x); }
__device__ __forceinline__ float whi(float x) { return 0.5f + copysignf(0.5f, x); }

// momentum_u_kern.c:150-262 in FP32.  Global arrays are indexed by cell,
// the shared tiles by slot.
__device__ bool mom_u32(const MCtx& x, int i, int j, float& out) {
  const int W = x.W, c = j * W + i, e = c + 1, wst = c - 1, s = c - W, n = c + W,
            se = s + 1;
  const int t = x.slot(i, j), te = t + 1, ts = t - SX, tn = t + SX, tse = ts + 1,
            tne = tn + 1;
  const int* m = x.m;
  if (m[t] + m[te] <= 0) return false;
  if (m[t] <= 0 || m[te] <= 0) return false;
  const float *un = x.un, *vn = x.vn, *hu = x.hu, *hv = x.hv, *ht = x.ht, *sn = x.sn,
              *su = x.su, *sv = x.sv;
  const MixConst& k = x.k;
  const float u_e = 0.5f * (un[c] + un[e]) * k.dy_t;
  const float depe = ht[e] + sn[te];
  const float u_w = 0.5f * (un[c] + un[wst]) * k.dy_t;
  const float depw = ht[c] + sn[t];
  const float v_sc = 0.5f * (vn[s] + vn[se]);
  const float v_s = 0.5f * v_sc * k.dxv2;
  const float deps = 0.5f * (hv[s] + sv[ts] + hv[se] + sv[tse]);
  const float v_nc = 0.5f * (vn[c] + vn[e]);
  const float v_n = 0.5f * v_nc * k.dxv2;
  const float depn = 0.5f * (hv[c] + sv[t] + hv[e] + sv[te]);
  const float uu_w = wlo(u_w) * un[c] + whi(u_w) * un[wst];
  const float uu_e = whi(u_e) * un[c] + wlo(u_e) * un[e];
  const bool south_dry = m[ts] <= 0 || m[tse] <= 0;
  const bool north_dry = m[tn] <= 0 || m[tne] <= 0;
  const float uu_s = south_dry ? wlo(v_s) * un[c] : wlo(v_s) * un[c] + whi(v_s) * un[s];
  const float uu_n = north_dry ? whi(v_n) * un[c] : whi(v_n) * un[c] + wlo(v_n) * un[n];
  const float adv = uu_w * u_w * depw - uu_e * u_e * depe + uu_s * v_s * deps -
                    uu_n * v_n * depn;
  const float dudx_e = (un[e] - un[c]) * k.r_dx_t * depe;
  const float dudx_w = (un[c] - un[wst]) * k.r_dx_t * depw;
  const float Hu = hu[c] + su[t];
  const float dudy_s =
      south_dry ? 0.f : (un[c] - un[s]) * k.r_dyu2 * (Hu + hu[s] + su[ts]);
  const float dudy_n =
      north_dry ? 0.f : (un[n] - un[c]) * k.r_dyu2 * (Hu + hu[n] + su[tn]);
  const float vis =
      k.visc * ((dudx_e - dudx_w) * k.dy_u + (dudy_n - dudy_s) * k.dx_u * 0.5f);
  const float cor = 0.5f * (k.cor_u * (v_sc + v_nc)) * k.area_u * Hu;
  const float hpg = -k.g * Hu * k.dy_u * (sn[te] - sn[t]);
  out = (un[c] * Hu + k.rdt * (adv + vis + cor + hpg) * k.r_area_u) * x.rhu[c] * k.r_fric;
  return true;
}

// momentum_v_kern.c:125-241 in FP32.
__device__ bool mom_v32(const MCtx& x, int i, int j, float& out) {
  const int W = x.W, c = j * W + i, e = c + 1, wst = c - 1, s = c - W, n = c + W,
            nw = n - 1;
  const int t = x.slot(i, j), te = t + 1, tw = t - 1, tn = t + SX, tnw = tn - 1,
            tne = tn + 1;
  const int* m = x.m;
  if (m[t] + m[te] <= 0) return false;
  if (m[t] <= 0 || m[tn] <= 0) return false;
  const float *un = x.un, *vn = x.vn, *hu = x.hu, *hv = x.hv, *ht = x.ht, *sn = x.sn,
              *su = x.su, *sv = x.sv;
  const MixConst& k = x.k;
  const float v_n = 0.5f * (vn[c] + vn[n]) * k.dx_t;
  const float depn = ht[n] + sn[tn];
  const float v_s = 0.5f * (vn[c] + vn[s]) * k.dx_t;
  const float deps = ht[c] + sn[t];
  const float u_wc = 0.5f * (un[wst] + un[nw]);
  const float u_w = 0.5f * u_wc * k.dyu2;
  const float depw = 0.5f * (hu[wst] + su[tw] + hu[nw] + su[tnw]);
  const float u_ec = 0.5f * (un[c] + un[n]);
  const float u_e = 0.5f * u_ec * k.dyu2;
  const float depe = 0.5f * (hu[c] + su[t] + hu[n] + su[tn]);
  const float vv_s = wlo(v_s) * vn[c] + whi(v_s) * vn[s];
  const float vv_n = whi(v_n) * vn[c] + wlo(v_n) * vn[n];
  const bool west_dry = m[tw] <= 0 || m[tnw] <= 0;
  const bool east_dry = m[te] <= 0 || m[tne] <= 0;
  const float vv_w = west_dry ? wlo(u_w) * vn[c] : wlo(u_w) * vn[c] + whi(u_w) * vn[wst];
  const float vv_e = east_dry ? whi(u_e) * vn[c] : whi(u_e) * vn[c] + wlo(u_e) * vn[e];
  const float adv = vv_w * u_w * depw - vv_e * u_e * depe + vv_s * v_s * deps -
                    vv_n * v_n * depn;
  const float dvdy_n = (vn[n] - vn[c]) * k.r_dy_t * depn;
  const float dvdy_s = (vn[c] - vn[s]) * k.r_dy_t * deps;
  const float Hv = hv[c] + sv[t];
  const float dvdx_w =
      west_dry ? 0.f : (vn[c] - vn[wst]) * k.r_dxv2 * (Hv + hv[wst] + sv[tw]);
  const float dvdx_e =
      east_dry ? 0.f : (vn[e] - vn[c]) * k.r_dxv2 * (Hv + hv[e] + sv[te]);
  const float vis =
      k.visc * ((dvdy_n - dvdy_s) * k.dx_v + (dvdx_e - dvdx_w) * k.dy_v * 0.5f);
  const float cor = -0.5f * (k.cor_v * (u_ec + u_wc)) * k.area_v * Hv;
  const float hpg = -k.g * Hv * k.dx_v * (sn[tn] - sn[t]);
  out = (vn[c] * Hv + k.rdt * (adv + vis + cor + hpg) * k.r_area_v) * x.rhv[c] * k.r_fric;
  return true;
}

__device__ float ua_pre(const MCtx& x, int i, int j) {
  const int c = j * x.W + i;
  float ua = x.in_copy(i, j) ? x.un[c] : (float)x.ua_arr[c];
  if (i >= x.d.xs && i <= x.d.xe - 1 && j >= x.d.ys && j <= x.d.ye) {
    float v;
    if (mom_u32(x, i, j, v)) ua = v;
  }
  const int t = x.slot(i, j);
  if (i >= x.d.xs - 1 && i <= x.d.xe && j >= x.d.ys - 1 && j <= x.d.ye + 1 &&
      x.m[t] * x.m[t + 1] == 0)
    ua = 0.f;
  return ua;
}

__device__ float va_pre(const MCtx& x, int i, int j) {
  const int c = j * x.W + i;
  float va = x.in_copy(i, j) ? x.vn[c] : (float)x.va_arr[c];
  if (i >= x.d.xs && i <= x.d.xe && j >= x.d.ys && j <= x.d.ye - 1) {
    float v;
    if (mom_v32(x, i, j, v)) va = v;
  }
  const int t = x.slot(i, j);
  if (i >= x.d.xs - 1 && i <= x.d.xe + 1 && j >= x.d.ys - 1 && j <= x.d.ye &&
      x.m[t] * x.m[t + SX] == 0)
    va = 0.f;
  return va;
}

// hi + lo + delta as a new (hi, lo) pair: TwoSum, then Fast2Sum.
__device__ __forceinline__ float2 dd_add(float2 a, float delta) {
  const float s = __fadd_rn(a.x, delta);
  const float bb = __fsub_rn(s, a.x);
  const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(delta, bb));
  const float lo = __fadd_rn(a.y, err);
  const float hi = __fadd_rn(s, lo);
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// One TX x TY tile of the mixed step of one domain (cells [i0, i0+TX) x
// [j0, j0+TY) of its copy region); `tide` is this step's bc_ssh value.
__device__ __forceinline__ void mixed_tile(const MixedFields& mf, const MixedState& ms,
                                           const Fields& f, const Dims& d, const MixConst& k,
                                           double tide, int i0, int j0) {
  __shared__ float s_sn[S0], s_su[S0], s_sv[S0];
  __shared__ float s_un[S0], s_vn[S0], s_hu[S0], s_hv[S0], s_Hu[S0], s_Hv[S0];
  __shared__ int s_m[S0];
  // terms shared by neighbouring updates (halo 1), as in the FP64 step
  __shared__ float b_flxu[S1], b_flxv[S1], b_gx[S1], b_gy[S1], b_fxu[S1], b_fyv[S1];
  __shared__ float b_vsc[S1], b_fyu[S1], b_qy[S1], b_uwc[S1], b_fxv[S1], b_qx[S1];
  const int W = d.width, H = d.height;
  const float2* __restrict__ sn2 = ms.sn_in;
  const int tid = threadIdx.y * TX + threadIdx.x;

  for (int t = tid; t < S0; t += TX * TY) {
    const int i = i0 - HALO + t % SX, j = j0 - HALO + t / SX;
    float vsn = 0.f, su = 0.f, sv = 0.f, vun = 0.f, vvn = 0.f, vhu = 0.f, vhv = 0.f;
    int mm = 0;
    if (i >= 0 && i < W && j >= 0 && j < H) {
      const int c = j * W + i;
      const int* m = f.tmask;
      vsn = sn2[c].x;
      vun = ms.un_in[c];
      vvn = ms.vn_in[c];
      vhu = mf.hu[c];
      vhv = mf.hv[c];
      mm = m[c];
      bool su_static = true, sv_static = true;
      if (j >= d.ys && j <= d.ye && i >= d.xs && i <= d.xe - 1) {
        const int n = c + 1, mn = m[n];
        if (mm + mn > 0) {
          su_static = false;
          if (mm * mn > 0)
            su = 0.5f * (k.area_t * vsn + k.area_t * sn2[n].x) * k.r_area_u;
          else if (mm <= 0)
            su = sn2[n].x;
          else
            su = vsn;
        }
      }
      if (j >= d.ys && j <= d.ye - 1 && i >= d.xs && i <= d.xe) {
        const int n = c + W, mn = m[n];
        if (mm + mn > 0) {
          sv_static = false;
          if (mm * mn > 0)
            sv = 0.5f * (k.area_t * vsn + k.area_t * sn2[n].x) * k.r_area_v;
          else if (mm <= 0)
            sv = sn2[n].x;
          else
            sv = vsn;
        }
      }
      // faces next_ssh{u,v} never updates keep their stored value
      if (su_static) su = (float)f.sshn_u[c];
      if (sv_static) sv = (float)f.sshn_v[c];
    }
    s_sn[t] = vsn;
    s_su[t] = su;
    s_sv[t] = sv;
    s_un[t] = vun;
    s_vn[t] = vvn;
    s_hu[t] = vhu;
    s_hv[t] = vhv;
    s_Hu[t] = vhu + su;
    s_Hv[t] = vhv + sv;
    s_m[t] = mm;
  }
  __syncthreads();

  for (int t = tid; t < S1; t += TX * TY) {
    const int ti = t % P1X, tj = t / P1X;
    const int i = i0 - 1 + ti, j = j0 - 1 + tj;
    const int q = (tj + 1) * SX + (ti + 1);
    const int qw = q - 1, qs = q - SX, qse = qs + 1, qwn = qw + SX;
    const float ht = (i >= 0 && i < W && j >= 0 && j < H) ? mf.ht[j * W + i] : 0.f;
    const float D = ht + s_sn[q];
    const float u_c = s_un[q], u_w = s_un[qw], u_s = s_un[qs], u_wn = s_un[qwn];
    const float v_c = s_vn[q], v_w = s_vn[qw], v_s = s_vn[qs], v_se = s_vn[qse];
    b_flxu[t] = s_Hu[q] * u_c;
    b_flxv[t] = s_Hv[q] * v_c;
    b_gx[t] = (u_c - u_w) * k.r_dx_t * D;
    b_gy[t] = (v_c - v_s) * k.r_dy_t * D;
    const float U = 0.5f * (u_c + u_w) * k.dy_t;
    b_fxu[t] = (U < 0.f ? u_c : u_w) * U * D;
    const float V = 0.5f * (v_c + v_s) * k.dx_t;
    b_fyv[t] = (V < 0.f ? v_c : v_s) * V * D;
    const float vsc = 0.5f * (v_s + v_se);
    b_vsc[t] = vsc;
    const float Vs = 0.5f * vsc * k.dxv2;
    const float deps = 0.5f * (s_Hv[qs] + s_hv[qse] + s_sv[qse]);
    b_fyu[t] = (Vs < 0.f ? u_c : u_s) * Vs * deps;
    b_qy[t] = (u_c - u_s) * k.r_dyu2;
    const float uwc = 0.5f * (u_w + u_wn);
    b_uwc[t] = uwc;
    const float Uw = 0.5f * uwc * k.dyu2;
    const float depw = 0.5f * (s_Hu[qw] + s_hu[qwn] + s_su[qwn]);
    b_fxv[t] = (Uw < 0.f ? v_c : v_w) * Uw * depw;
    b_qx[t] = (v_c - v_w) * k.r_dxv2;
  }
  __syncthreads();

  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  if (i > d.xe + 1 || j > d.ye) return;
  const int c = j * W + i;
  MCtx x;
  x.un = ms.un_in;
  x.vn = ms.vn_in;
  x.ht = mf.ht;
  x.hu = mf.hu;
  x.hv = mf.hv;
  x.sn = s_sn;
  x.su = s_su;
  x.sv = s_sv;
  x.m = s_m;
  x.rhu = mf.rhu;
  x.rhv = mf.rhv;
  x.ua_arr = f.ua;
  x.va_arr = f.va;
  x.W = W;
  x.i0 = i0;
  x.j0 = j0;
  x.d = d;
  x.k = k;
  const int t = x.slot(i, j);
  const int* m = s_m;

  bool regular = i >= d.xs && i <= d.xe - 1 && j >= d.ys && j <= d.ye - 1;
  if (regular) {
#pragma unroll
    for (int dj = -1; dj <= 1; dj++)
#pragma unroll
      for (int di = -1; di <= 1; di++) regular &= m[t + dj * SX + di] > 0;
  }
  if (regular) {
    // Wet cell with a wet 3x3 neighbourhood: no boundary condition applies.
    const int r = (threadIdx.y + 1) * P1X + (threadIdx.x + 1);
    const float snc = s_sn[t], Hu = s_Hu[t], Hv = s_Hv[t];
    const float div = ((b_flxu[r - 1] - b_flxu[r]) + b_flxv[r - P1X]) - b_flxv[r];
    ms.sn_out[c] = dd_add(sn2[c], div * k.rdt * k.r_area_t);
    {
      const float adv = ((b_fxu[r] - b_fxu[r + 1]) + b_fyu[r]) - b_fyu[r + P1X];
      const float dudy_s = b_qy[r] * (Hu + s_hu[t - SX] + s_su[t - SX]);
      const float dudy_n = b_qy[r + P1X] * (Hu + s_hu[t + SX] + s_su[t + SX]);
      const float vis =
          k.visc * ((b_gx[r + 1] - b_gx[r]) * k.dy_u + 0.5f * (dudy_n - dudy_s) * k.dx_u);
      const float cor = 0.5f * (k.cor_u * (b_vsc[r] + b_vsc[r + P1X])) * k.area_u * Hu;
      const float hpg = -k.g * Hu * k.dy_u * (s_sn[t + 1] - snc);
      ms.un_out[c] = (s_un[t] * Hu + k.rdt * (adv + vis + cor + hpg) * k.r_area_u) *
                     mf.rhu[c] * k.r_fric;
    }
    {
      const float adv = ((b_fxv[r] - b_fxv[r + 1]) + b_fyv[r]) - b_fyv[r + P1X];
      const float dvdx_w = b_qx[r] * (Hv + s_hv[t - 1] + s_sv[t - 1]);
      const float dvdx_e = b_qx[r + 1] * (Hv + s_hv[t + 1] + s_sv[t + 1]);
      const float vis =
          k.visc * ((b_gy[r + P1X] - b_gy[r]) * k.dx_v + 0.5f * (dvdx_e - dvdx_w) * k.dy_v);
      const float cor = -0.5f * (k.cor_v * (b_uwc[r + 1] + b_uwc[r])) * k.area_v * Hv;
      const float hpg = -k.g * Hv * k.dx_v * (s_sn[t + SX] - snc);
      ms.vn_out[c] = (s_vn[t] * Hv + k.rdt * (adv + vis + cor + hpg) * k.r_area_v) *
                     mf.rhv[c] * k.r_fric;
    }
    return;
  }

  // ssh: continuity (FP32 flux divergence) + compensated update, bc_ssh
  float2 ssh = sn2[c];
  if (i >= d.xs && i <= d.xe && j >= d.ys && j <= d.ye) {
    const float r1 = (s_su[t] + mf.hu[c]) * x.un[c];
    const float r2 = (s_su[t - 1] + mf.hu[c - 1]) * x.un[c - 1];
    const float r3 = (s_sv[t] + mf.hv[c]) * x.vn[c];
    const float r4 = (s_sv[t - SX] + mf.hv[c - W]) * x.vn[c - W];
    ssh = dd_add(ssh, (r2 - r1 + r4 - r3) * k.rdt * k.r_area_t);
    if (m[t] > 0 && (m[t - SX] < 0 || m[t + SX] < 0 || m[t + 1] < 0 || m[t - 1] < 0)) {
      const double tv = tide;
      const float hi = (float)tv;
      ssh = make_float2(hi, (float)(tv - (double)hi));
    }
  }
  ms.sn_out[c] = ssh;

  float ua = x.un[c];
  if (i <= d.xe) {
    ua = ua_pre(x, i, j);
    if (m[t] + m[t + 1] > -1) {
      if (m[t] < 0)
        ua = ua_pre(x, i + 1, j) + sqrtf(k.g / mf.hu[c]) * (s_su[t] - s_su[t + 1]);
      else if (m[t + 1] < 0 && i >= 1)
        ua = ua_pre(x, i - 1, j) + sqrtf(k.g / mf.hu[c]) * (s_su[t] - s_su[t - 1]);
    }
  }
  ms.un_out[c] = ua;

  float va = va_pre(x, i, j);
  if (m[t] + m[t + SX] > -1) {
    if (m[t] < 0)
      va = va_pre(x, i, j + 1) + sqrtf(k.g / mf.hv[c]) * (s_sv[t] - s_sv[t + SX]);
    else if (m[t + SX] < 0 && j >= 1)
      va = va_pre(x, i, j - 1) + sqrtf(k.g / mf.hv[c]) * (s_sv[t] - s_sv[t - SX]);
  }
  ms.vn_out[c] = va;
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
