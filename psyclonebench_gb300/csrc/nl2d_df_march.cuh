// The double-float column march of one warp (the FP64-equivalent form's
// interior cells): device code shared by the single-domain kernel
// (nl2d_df.cu) and the ensemble's step (nl2d_ensemble.cu).  The arithmetic
// is nl2d_df.cuh's; what the march computes and where is described in
// nl2d_df.cu.
#pragma once
#include "nl2d_df.cuh"
#include "nl2d_internal.h"

namespace nl2d {
namespace dfm {
using namespace dfk;

constexpr int MW = kDfMarchCols;
constexpr int WARPS = 4;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ df shd(df x) {
  return df{__shfl_down_sync(FULL, x.hi, 1), __shfl_down_sync(FULL, x.lo, 1)};
}
__device__ __forceinline__ df shu(df x) {
  return df{__shfl_up_sync(FULL, x.hi, 1), __shfl_up_sync(FULL, x.lo, 1)};
}
__device__ __forceinline__ df sel_lt0(df w, df a, df b) { return dneg_sign(w) ? a : b; }

struct MRow {
  df u, v, hu, hv, su, sv, sn, D;  // D = ht + sn
};
struct MRaw {
  double sn, u, v;
  float2 ht, hu, hv;
};
struct MTerm {
  df Hu, Hv, fu, fv, gu, gv, fxu, fxv, fyu, fyv, qu, qv, vws, uws;
};
struct MOut {
  df rhu, rhv;
  unsigned char reg;
};

__device__ __forceinline__ df pair(float2 a) { return df{a.x, a.y}; }

__device__ __forceinline__ MRaw load_raw(const FusedState& fs, const DfFields& ff, int i, int j,
                                         int W, int H) {
  MRaw r;
  const bool ok = i >= 0 && i < W && j >= 0 && j < H;
  const size_t c = ok ? (size_t)j * W + i : 0;
  r.sn = ok ? __ldg(fs.sshn_in + c) : 0.0;
  r.u = ok ? __ldg(fs.un_in + c) : 0.0;
  r.v = ok ? __ldg(fs.vn_in + c) : 0.0;
  const float2 z = make_float2(0.f, 0.f);
  r.ht = ok ? __ldg(ff.ht + c) : z;
  r.hu = ok ? __ldg(ff.hu + c) : z;
  r.hv = ok ? __ldg(ff.hv + c) : z;
  return r;
}

__device__ __forceinline__ MRow finish_row(const MRaw& a, const DfConst& k) {
  MRow r;
  r.sn = split_bits(a.sn);
  r.u = split_bits(a.u);
  r.v = split_bits(a.v);
  r.hu = pair(a.hu);
  r.hv = pair(a.hv);
  r.D = dadd(pair(a.ht), r.sn);
  r.su = dmul_u(dadd(r.sn, shd(r.sn)), k.face_u);
  r.sv = df{0.f, 0.f};
  return r;
}

__device__ __forceinline__ MOut load_out(const DfFields& ff, bool col, int i, int j, int W,
                                         int jend) {
  MOut o{df{0.f, 0.f}, df{0.f, 0.f}, 0};
  if (col && j < jend) {
    const size_t c = (size_t)j * W + i;
    o.reg = __ldg(ff.reg + c);
    o.rhu = pair(__ldg(ff.rhu + c));
    o.rhv = pair(__ldg(ff.rhv + c));
  }
  return o;
}

// The shared terms of row C (P below, N above), as in the mixed march's
// row_terms.
__device__ __forceinline__ MTerm row_terms(const MRow& P, const MRow& C, const MRow& N,
                                           const DfConst& k) {
  MTerm t;
  t.Hu = dadd(C.hu, C.su);
  t.Hv = dadd(C.hv, C.sv);
  t.fu = dmul_u(t.Hu, C.u);
  t.fv = dmul_u(t.Hv, C.v);
  const df uW = shu(C.u), vW = shu(C.v), HuW = shu(t.Hu);
  const df vE_P = shd(P.v), hvE_P = shd(P.hv), svE_P = shd(P.sv);
  const df uW_N = shu(N.u), huW_N = shu(N.hu), suW_N = shu(N.su);
  t.gu = dmul_u(dmul_u(dsub(C.u, uW), k.r_dx), C.D);
  t.gv = dmul_u(dmul_u(dsub(C.v, P.v), k.r_dy), C.D);
  const df sAx = dadd(C.u, uW), sAy = dadd(uW, uW_N);
  const df sBx = dadd(P.v, vE_P), sBy = dadd(C.v, P.v);
  t.vws = sBx;
  t.uws = sAy;
  const df UUx = dmul_u(sAx, k.uu_x), UUy = dmul_u(sAy, k.uu_y);
  const df VVx = dmul_u(sBx, k.vv_x), VVy = dmul_u(sBy, k.vv_y);
  const df depx = dsum3(HuW, huW_N, suW_N);
  const df depy = dsum4(P.hv, P.sv, hvE_P, svE_P);
  t.fxu = dmul_u(dmul_u(sel_lt0(UUx, C.u, uW), UUx), C.D);
  t.fxv = dmul_u(dmul_u(sel_lt0(UUy, C.v, vW), UUy), depx);
  t.fyu = dmul_u(dmul_u(sel_lt0(VVx, C.u, P.u), VVx), depy);
  t.fyv = dmul_u(dmul_u(sel_lt0(VVy, C.v, P.v), VVy), C.D);
  t.qu = dmul_u(dsub(C.u, P.u), k.r_qu);
  t.qv = dmul_u(dsub(C.v, vW), k.r_qv);
  return t;
}

// One warp's strip: columns i0 .. i0 + MW - 1, rows j0 .. j0 + mr - 1 of the
// copy region of the domain whose arrays fs and ff point into.
__device__ __forceinline__ void df_march(const FusedState& fs, const DfFields& ff, const Dims& d,
                                         const DfConst& k, int i0, int j0, int mr) {
  const int lane = threadIdx.x & 31;
  const int W = d.width, H = d.height;
  const int i = i0 - 1 + lane;
  const int jend = min(j0 + mr, d.ye + 1);
  const bool out_col = lane >= 1 && lane <= MW && i <= d.xe + 1;
  MRow P = finish_row(load_raw(fs, ff, i, j0 - 1, W, H), k);
  MRow C = finish_row(load_raw(fs, ff, i, j0, W, H), k);
  MRow N = finish_row(load_raw(fs, ff, i, j0 + 1, W, H), k);
  MRaw R1 = load_raw(fs, ff, i, j0 + 2, W, H);
  MOut O = load_out(ff, out_col, i, j0, W, jend);
  P.sv = dmul_u(dadd(P.sn, C.sn), k.face_v);
  C.sv = dmul_u(dadd(C.sn, N.sn), k.face_v);
  // row j0-1: what the updates of row j0 read from it
  df fv0 = dmul_u(dadd(P.hv, P.sv), P.v), hu0 = P.hu, su0 = P.su;
  MTerm T1 = row_terms(P, C, N, k);  // row j0
  for (int j = j0; j < jend; j++) {
    P = C;                  // row j
    C = N;                  // row j+1
    N = finish_row(R1, k);  // row j+2, loaded an iteration ago
    R1 = load_raw(fs, ff, i, j + 3, W, H);
    const MOut Oc = O;
    O = load_out(ff, out_col, i, j + 1, W, jend);
    C.sv = dmul_u(dadd(C.sn, N.sn), k.face_v);
    const MTerm T2 = row_terms(P, C, N, k);  // row j+1
    // x neighbours of row j's terms (every lane takes part)
    const df fuW = shu(T1.fu), snE = shd(P.sn);
    const df fxuE = shd(T1.fxu), fxvE = shd(T1.fxv), guE = shd(T1.gu), qvE = shd(T1.qv),
             uwsE = shd(T1.uws);
    const df hvW = shu(P.hv), svW = shu(P.sv), hvE = shd(P.hv), svE = shd(P.sv);
    if (out_col && Oc.reg) {
      const size_t c = (size_t)j * W + i;
      const df div = dsum4(fuW, dneg(T1.fu), fv0, dneg(T1.fv));
      const df ssh = dadd(P.sn, dmul_u(div, k.rrat));
      const df advu = dsum4(T1.fxu, dneg(fxuE), T1.fyu, dneg(T2.fyu));
      const df advv = dsum4(T1.fxv, dneg(fxvE), T1.fyv, dneg(T2.fyv));
      const df dSu = dmul_u(T1.qu, dsum3(T1.Hu, hu0, su0));
      const df dSv = dmul_u(T1.qv, dsum3(T1.Hv, hvW, svW));
      const df dNu = dmul_u(T2.qu, dsum3(T1.Hu, C.hu, C.su));
      const df dNv = dmul_u(qvE, dsum3(T1.Hv, hvE, svE));
      const df visu = dadd(dmul_u(dsub(dNu, dSu), k.vis2_u), dmul_u(dsub(guE, T1.gu), k.vis1_u));
      const df visv = dadd(dmul_u(dsub(dNv, dSv), k.vis2_v), dmul_u(dsub(T2.gv, T1.gv), k.vis1_v));
      const df coru = dmul_u(dmul_u(dadd(T1.vws, T2.vws), k.cor_u), T1.Hu);
      const df corv = dmul_u(dmul_u(dadd(uwsE, T1.uws), k.cor_v), T1.Hv);
      const df hpgu = dmul_u(dmul_u(T1.Hu, k.hpg_u), dsub(snE, P.sn));
      const df hpgv = dmul_u(dmul_u(T1.Hv, k.hpg_v), dsub(C.sn, P.sn));
      const df tu = dsum4(advu, visu, coru, hpgu);
      const df tv = dsum4(advv, visv, corv, hpgv);
      const df ou = dmul_u(dmul_u(dadd(dmul_u(tu, k.rra_u), dmul_u(P.u, T1.Hu)), Oc.rhu), k.r_fric);
      const df ov = dmul_u(dmul_u(dadd(dmul_u(tv, k.rra_v), dmul_u(P.v, T1.Hv)), Oc.rhv), k.r_fric);
      fs.sshn_out[c] = join_bits(ssh);
      fs.un_out[c] = join_bits(ou);
      fs.vn_out[c] = join_bits(ov);
    }
    fv0 = T1.fv;
    hu0 = P.hu;
    su0 = P.su;
    T1 = T2;
  }
}

}  // namespace dfm
}  // namespace nl2d
