// The mixed-precision step as a column march (device code of the single
// domain's and the ensemble's kernels).
//
// One warp owns MW = 30 consecutive columns (one lane per column, plus one
// halo lane on each side) and marches down a strip of MR rows.  Each lane
// keeps rows j-1, j, j+1 of its column in registers, takes its x neighbours
// by warp shuffles, and forms every term that two neighbouring updates
// share once per position.  No shared memory, no block barrier; the
// redundancy is 32/30 in x and (MR+3)/MR in loads along y.  (A shared-memory
// tile form staging a 2-cell halo of every field took 1.7x the cells in
// loads, index arithmetic and terms, ~930 instructions per cell.)
//
// The march writes the REGULAR cells only: xs+1 <= i <= xe-1,
// ys+1 <= j <= ye-1, 3x3 mask neighbourhood wet (the byte flags `reg`).
// For them every sshn_u / sshn_v face the update reads takes next_ssh's
// two-sided formula, and no momentum mask, bc_ssh, solid-wall or Flather
// rule applies: continuity and unmasked momentum in FP32 with the
// compensated ssh.  Every other cell of the copy region (a precomputed
// list, ~0.1 % of a 4096^2 domain) is updated by k_mixed_general with the
// reference's per-point code in FP32 on global memory (general_cell below).
// Both kernels read the same input buffers and write disjoint cells of the
// output buffers.
#pragma once
#include "nl2d_mixed_common.cuh"

namespace nl2d {
namespace mixk {
namespace {

constexpr int MW = 30;  // output columns per warp
constexpr int MR = 64;  // output rows per warp (at most; smaller domains take shorter strips)
constexpr int MARCH_WARPS = 4;
constexpr int PF = 2;  // rows between an L2 prefetch and the row's loads
constexpr unsigned FULL = 0xffffffffu;

// log2 of the element size of the array this lane prefetches in the march
// (the lane id is read again where it is needed, not held in a register)
__device__ __forceinline__ int pf_shift() {
  unsigned l;
  asm("mov.u32 %0, %%laneid;" : "=r"(l));
  return l < 3 ? 3 : (l < 17 ? 2 : 0);
}

__device__ __forceinline__ float shd(float x) { return __shfl_down_sync(FULL, x, 1); }
__device__ __forceinline__ float shu(float x) { return __shfl_up_sync(FULL, x, 1); }

__device__ __forceinline__ float face_ssh(const MixConst& k, float a, float b, float r_area) {
  return 0.5f * (k.area_t * a + k.area_t * b) * r_area;
}

// The u and v halves of the update have the same shape, so they run as
// pairs on the packed FP32 instructions (add / mul / fma .f32x2: one issue
// slot for two operations); a float2 below is always (u side, v side).  The
// shared terms (row_terms) use the same pairs with scalar operations: packed
// there too, the march needed 117 registers instead of 96 (4 blocks of 4
// warps per SM instead of 5) and ran slower (63.8 k against 71.3 k
// Mcell-steps/s at 4096^2; packed in the update only: 74.0 k).
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b in one rounding: (-1) * b + a
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ float2 add2s(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 mul2s(float2 a, float2 b) {
  return make_float2(a.x * b.x, a.y * b.y);
}
__device__ __forceinline__ float2 sub2s(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}

// The march's step constants, pairs as above, with the factors 0.5 of the
// face averages and upwind speeds folded in (powers of two: the same
// values) and the per-step products formed once.
struct MarchConst {
  float2 r_dxy;  // (1/dx_t, 1/dy_t): the x / y gradients
  float2 uu;     // (dy_t / 2, dyu2 / 8): U east-west and the U of the v flux
  float2 vv;     // (dxv2 / 8, dx_t / 2): the V of the u flux and V north-south
  float2 r_q;    // (1/dyu2, 1/dxv2): the cross gradients
  float2 vis1;   // (visc dy_u, visc dx_v)
  float2 vis2;   // (visc dx_u / 2, visc dy_v / 2)
  float2 cor;    // (cor_u area_u / 4, -cor_v area_v / 4)
  float2 hpg;    // (-g dy_u, -g dx_v)
  float2 rra;    // (rdt / area_u, rdt / area_v)
  float face_u, face_v;  // area_t / (2 area_u), area_t / (2 area_v): next_ssh's faces
  float rrat;            // rdt / area_t
  float r_fric;
};

inline MarchConst make_march_const(const MixConst& k) {
  MarchConst c;
  c.r_dxy = make_float2(k.r_dx_t, k.r_dy_t);
  c.uu = make_float2(0.5f * k.dy_t, 0.125f * k.dyu2);
  c.vv = make_float2(0.125f * k.dxv2, 0.5f * k.dx_t);
  c.r_q = make_float2(k.r_dyu2, k.r_dxv2);
  c.vis1 = make_float2(k.visc * k.dy_u, k.visc * k.dx_v);
  c.vis2 = make_float2(0.5f * k.visc * k.dx_u, 0.5f * k.visc * k.dy_v);
  c.cor = make_float2(0.25f * k.cor_u * k.area_u, -0.25f * k.cor_v * k.area_v);
  c.hpg = make_float2(-k.g * k.dy_u, -k.g * k.dx_v);
  c.rra = make_float2(k.rdt * k.r_area_u, k.rdt * k.r_area_v);
  c.face_u = 0.5f * k.area_t * k.r_area_u;
  c.face_v = 0.5f * k.area_t * k.r_area_v;
  c.rrat = k.rdt * k.r_area_t;
  c.r_fric = k.r_fric;
  return c;
}

// One loaded row of one column.
struct MRow {
  float2 uv, hh;  // (u, v), (hu, hv)
  float2 ss;      // (sshn_u of the east face, sshn_v of the north face); the
                  // north face is formed once the next row is loaded
  float sn, lo, ht;
};

// The terms at one position that neighbouring updates share, and the row
// values the update at that position reads.
struct MTerm {
  float2 flx;  // (hu + su) u, (hv + sv) v: the continuity fluxes
  float2 g;    // x gradient of u, y gradient of v, times the depth
  float2 fx;   // advective fluxes of u and of v through the west face
  float2 fy;   // advective fluxes of u and of v through the south face
  float2 q;    // y gradient of u, x gradient of v
  float2 vw;   // the v sum of the u Coriolis term, the u sum of the v one
  float2 H;    // total depths at the u and v faces
  float2 hh, ss, uv;
  float sn, lo;
};

// The values of one row of one column, as loaded.
struct MRaw {
  float2 s, uv, hh;
  float ht;
};

__device__ __forceinline__ MRaw load_raw(const MixedFields& mf, const MixedState& ms, int c) {
  MRaw r;
  r.s = __ldg(ms.sn_in + c);
  r.uv = make_float2(__ldg(ms.un_in + c), __ldg(ms.vn_in + c));
  r.hh = make_float2(__ldg(mf.hu + c), __ldg(mf.hv + c));
  r.ht = __ldg(mf.ht + c);
  return r;
}

// A loaded row and its east face's sshn_u; the east neighbour's ssh comes
// from lane + 1 (lane 31's su is not used).
__device__ __forceinline__ MRow finish_row(const MRaw& a, const MarchConst& c) {
  MRow r;
  r.sn = a.s.x;
  r.lo = a.s.y;
  r.uv = a.uv;
  r.hh = a.hh;
  r.ht = a.ht;
  r.ss = make_float2((r.sn + shd(r.sn)) * c.face_u, 0.f);
  return r;
}

// What the update of output row j reads besides the terms, issued a row
// ahead.
struct MOut {
  float2 rh;  // 1 / (hu + ssha_u), 1 / (hv + ssha_v)
  unsigned char reg;
};

__device__ __forceinline__ MOut load_out(const MixedFields& mf, bool col, int c) {
  MOut o{make_float2(0.f, 0.f), 0};
  if (col) {
    o.reg = __ldg(mf.reg + c);
    o.rh = make_float2(__ldg(mf.rhu + c), __ldg(mf.rhv + c));
  }
  return o;
}

// The shared terms at (i, r) from rows r-1 (P), r (C), r+1 (N): the tile
// form's phase 1, in (scalar) pairs.
__device__ __forceinline__ MTerm row_terms(const MRow& P, const MRow& C, const MRow& N,
                                           const MarchConst& c) {
  MTerm t;
  t.H = add2s(C.hh, C.ss);
  t.flx = mul2s(t.H, C.uv);
  const float uW = shu(C.uv.x), vW = shu(C.uv.y), HuW = shu(t.H.x);
  const float vE_P = shd(P.uv.y), hvE_P = shd(P.hh.y), svE_P = shd(P.ss.y);
  const float uW_N = shu(N.uv.x), huW_N = shu(N.hh.x), suW_N = shu(N.ss.x);
  const float D = C.ht + C.sn;
  t.g = mul2s(mul2s(sub2s(C.uv, make_float2(uW, P.uv.y)), c.r_dxy), make_float2(D, D));
  // (u + u_west, u_west + u_west of the next row), (v_south + v_south-east, v + v_south)
  const float2 sA = add2s(make_float2(C.uv.x, uW), make_float2(uW, uW_N));
  const float2 sB = add2s(make_float2(P.uv.y, C.uv.y), make_float2(vE_P, P.uv.y));
  t.vw = make_float2(sB.x, sA.y);
  const float2 UU = mul2s(sA, c.uu);  // (U, U of the v flux / 2)
  const float2 VV = mul2s(sB, c.vv);  // (V of the u flux / 2, V)
  // depths of the v-flux west face and the u-flux south face, times 2
  const float2 dep = add2s(add2s(make_float2(HuW, P.hh.y + P.ss.y), make_float2(huW_N, hvE_P)),
                          make_float2(suW_N, svE_P));
  const float2 selx = make_float2(UU.x < 0.f ? C.uv.x : uW, UU.y < 0.f ? C.uv.y : vW);
  const float2 sely = make_float2(VV.x < 0.f ? C.uv.x : P.uv.x, VV.y < 0.f ? C.uv.y : P.uv.y);
  t.fx = mul2s(mul2s(selx, UU), make_float2(D, dep.x));
  t.fy = mul2s(mul2s(sely, VV), make_float2(dep.y, D));
  t.q = mul2s(sub2s(C.uv, make_float2(P.uv.x, vW)), c.r_q);
  t.hh = C.hh;
  t.ss = C.ss;
  t.uv = C.uv;
  t.sn = C.sn;
  t.lo = C.lo;
  return t;
}

// One warp: lane L holds column i0-1+L; output rows j0 .. j0+mr-1 of the
// copy region, regular cells only.  `base`: the domain's first element in
// the arrays (an ensemble packs its domains back to back; 0 otherwise).
__device__ __forceinline__ void mixed_march(const MixedFields& mf, const MixedState& ms,
                                            const Dims& d, const MarchConst& k, int i0, int j0,
                                            size_t base, int mr) {
  const int lane = threadIdx.x & 31;
  const int W = d.width, H = d.height;
  const int i = i0 - 1 + lane;
  const int jend = min(j0 + mr, d.ye + 1);
  const bool out_col = lane >= 1 && lane <= MW && i <= d.xe + 1;
  // Element offsets are 32-bit: every array the march reads holds fewer
  // than 2^31 elements (a single domain of 2^31 cells would need 25 FP64
  // arrays of 16 GB; an ensemble packs fewer cells still).  Rows and columns
  // outside the array are clamped onto it: a clamped value only reaches
  // terms of cells the march does not write (it writes regular cells, whose
  // stencil rows j-1 .. j+2 and columns i-1 .. i+1 lie inside the array), so
  // the loads need no bounds test and no select.
  const int cb = (int)base + min(max(i, 0), W - 1);  // this lane's column
  auto at = [cb, W, H](int j) { return cb + min(max(j, 0), H - 1) * W; };
  // The row PF ahead of the loads goes into L2 first, one line per lane:
  // lanes 0-2 the first, middle and last of the warp's columns in the
  // 8-byte ssh pairs, lanes 3-16 the first and last in each of the seven
  // 4-byte arrays, lanes 17-18 in the flag bytes (pf_shift gives each lane's
  // element size), so that the loads PF rows later find their lines there.
  const char* pf = nullptr;
  {
    const int c0 = (int)base + min(max(i0 - 1, 0), W - 1);
    const int c1 = (int)base + min(i0 + MW, W - 1), cm = (int)base + min(i0 + MW / 2, W - 1);
    switch (lane) {
      case 0: pf = (const char*)(ms.sn_in + c0); break;
      case 1: pf = (const char*)(ms.sn_in + cm); break;
      case 2: pf = (const char*)(ms.sn_in + c1); break;
      case 3: case 4: pf = (const char*)(ms.un_in + (lane & 1 ? c0 : c1)); break;
      case 5: case 6: pf = (const char*)(ms.vn_in + (lane & 1 ? c0 : c1)); break;
      case 7: case 8: pf = (const char*)(mf.hu + (lane & 1 ? c0 : c1)); break;
      case 9: case 10: pf = (const char*)(mf.hv + (lane & 1 ? c0 : c1)); break;
      case 11: case 12: pf = (const char*)(mf.ht + (lane & 1 ? c0 : c1)); break;
      case 13: case 14: pf = (const char*)(mf.rhu + (lane & 1 ? c0 : c1)); break;
      case 15: case 16: pf = (const char*)(mf.rhv + (lane & 1 ? c0 : c1)); break;
      case 17: case 18: pf = (const char*)(mf.reg + (lane & 1 ? c0 : c1)); break;
      default: break;
    }
  }
  MRow P = finish_row(load_raw(mf, ms, at(j0 - 1)), k);
  MRow C = finish_row(load_raw(mf, ms, at(j0)), k);
  MRow N = finish_row(load_raw(mf, ms, at(j0 + 1)), k);
  MRaw R1 = load_raw(mf, ms, at(j0 + 2)), R2 = load_raw(mf, ms, at(j0 + 3));
  // rows j0 .. jend lie inside the array (jend <= ye + 1 <= H - 1)
  MOut O = load_out(mf, out_col, cb + j0 * W);
  P.ss.y = (P.sn + C.sn) * k.face_v;
  C.ss.y = (C.sn + N.sn) * k.face_v;
  // row j0-1: what the updates of row j0 read from it
  float flxv0 = (P.hh.y + P.ss.y) * P.uv.y, hu0 = P.hh.x, su0 = P.ss.x;
  MTerm T1 = row_terms(P, C, N, k);  // row j0
  for (int j = j0; j < jend; j++) {
    P = C;  // row j
    C = N;  // row j+1
    N = finish_row(R1, k);  // row j+2, loaded two iterations ago
    R1 = R2;
    R2 = load_raw(mf, ms, at(j + 4));  // in flight for two iterations
    if (pf) {
      const size_t off = (size_t)min(j + 4 + PF, H - 1) * W;
      asm volatile("prefetch.global.L2 [%0];" ::"l"(pf + (off << pf_shift())));
    }
    const MOut Oc = O;
    O = load_out(mf, out_col, cb + (j + 1) * W);
    C.ss.y = (C.sn + N.sn) * k.face_v;
    const MTerm T2 = row_terms(P, C, N, k);  // row j+1
    // x neighbours of row j's terms (every lane takes part)
    const float flxuW = shu(T1.flx.x), snE = shd(T1.sn);
    const float2 fxE = make_float2(shd(T1.fx.x), shd(T1.fx.y));
    const float gxE = shd(T1.g.x), qxE = shd(T1.q.y), uwcE = shd(T1.vw.y);
    const float hvW = shu(T1.hh.y), svW = shu(T1.ss.y), hvE = shd(T1.hh.y), svE = shd(T1.ss.y);
    if (out_col && Oc.reg) {
      const int c = cb + j * W;
      const float div = ((flxuW - T1.flx.x) + flxv0) - T1.flx.y;
      ms.sn_out[c] = dd_add(make_float2(T1.sn, T1.lo), div * k.rrat);
      const float2 Hf = T1.H;
      const float2 adv = sub2(add2(sub2(T1.fx, fxE), T1.fy), T2.fy);
      // (du/dy, dv/dx) times the depth at the south / west and north / east faces
      const float2 dS = mul2(T1.q, add2(add2(Hf, make_float2(hu0, hvW)), make_float2(su0, svW)));
      const float2 dN = mul2(make_float2(T2.q.x, qxE),
                             add2(add2(Hf, make_float2(T2.hh.x, hvE)), make_float2(T2.ss.x, svE)));
      const float2 vis =
          fma2(sub2(dN, dS), k.vis2, mul2(sub2(make_float2(gxE, T2.g.y), T1.g), k.vis1));
      const float2 cor =
          mul2(mul2(add2(make_float2(T1.vw.x, uwcE), make_float2(T2.vw.x, T1.vw.y)), k.cor), Hf);
      const float2 hpg =
          mul2(mul2(Hf, k.hpg), sub2(make_float2(snE, T2.sn), make_float2(T1.sn, T1.sn)));
      const float2 tend = add2(add2(add2(adv, vis), cor), hpg);
      const float2 out = mul2(mul2(fma2(tend, k.rra, mul2(T1.uv, Hf)), Oc.rh),
                              make_float2(k.r_fric, k.r_fric));
      ms.un_out[c] = out.x;
      ms.vn_out[c] = out.y;
    }
    flxv0 = T1.flx.y;
    hu0 = T1.hh.x;
    su0 = T1.ss.x;
    T1 = T2;
  }
}

// ---- the other cells of the copy region, on global memory ----------------

// One domain of a mixed-precision ensemble (device descriptor).
struct EnsDom {
  MixedFields mf;
  MixedState ms[2];
  Fields f;  // FP64 arrays the mixed step reads where no step writes
  Dims d;
  MixConst k;
  size_t off;  // the domain's first element in the packed arrays
};

// Global-memory view of the fields the general code reads: zeros outside the
// array, sshn_u / sshn_v by next_ssh{u,v}'s rules inside it (the stored
// value on faces those kernels never update).  The members refer to a
// domain descriptor held in memory (the ensemble's device array, or a
// single domain's copy in shared memory), so the context passed to the
// out-of-line helpers is five pointers, not a copy of the descriptor.
struct GCtx {
  const MixedFields& mf;
  const MixedState& ms;
  const Fields& f;
  const Dims& d;
  const MixConst& k;
  __device__ __forceinline__ bool in(int i, int j) const {
    return i >= 0 && i < d.width && j >= 0 && j < d.height;
  }
  __device__ __forceinline__ int ix(int i, int j) const { return j * d.width + i; }
  __device__ __forceinline__ int m(int i, int j) const { return in(i, j) ? f.tmask[ix(i, j)] : 0; }
  __device__ __forceinline__ float sn(int i, int j) const {
    return in(i, j) ? ms.sn_in[ix(i, j)].x : 0.f;
  }
  __device__ __forceinline__ float su(int i, int j) const {
    if (!in(i, j)) return 0.f;
    const int mm = m(i, j);
    if (j >= d.ys && j <= d.ye && i >= d.xs && i <= d.xe - 1) {
      const int mn = m(i + 1, j);
      if (mm + mn > 0) {
        if (mm * mn > 0) return face_ssh(k, sn(i, j), sn(i + 1, j), k.r_area_u);
        return mm <= 0 ? sn(i + 1, j) : sn(i, j);
      }
    }
    return (float)f.sshn_u[ix(i, j)];
  }
  __device__ __forceinline__ float sv(int i, int j) const {
    if (!in(i, j)) return 0.f;
    const int mm = m(i, j);
    if (j >= d.ys && j <= d.ye - 1 && i >= d.xs && i <= d.xe) {
      const int mn = m(i, j + 1);
      if (mm + mn > 0) {
        if (mm * mn > 0) return face_ssh(k, sn(i, j), sn(i, j + 1), k.r_area_v);
        return mm <= 0 ? sn(i, j + 1) : sn(i, j);
      }
    }
    return (float)f.sshn_v[ix(i, j)];
  }
  __device__ __forceinline__ bool in_copy(int i, int j) const {
    return i >= d.xs - 1 && i <= d.xe + 1 && j >= d.ys - 1 && j <= d.ye;
  }
};

// momentum_u_kern.c:150-262 in FP32 at (i, j), with the masked branches.
__device__ bool gmom_u(const GCtx& x, int i, int j, float& out) {
  const int W = x.d.width, c = j * W + i, e = c + 1, wst = c - 1, s = c - W, n = c + W,
            se = s + 1;
  if (x.m(i, j) + x.m(i + 1, j) <= 0) return false;
  if (x.m(i, j) <= 0 || x.m(i + 1, j) <= 0) return false;
  const float *un = x.ms.un_in, *vn = x.ms.vn_in, *hu = x.mf.hu, *hv = x.mf.hv, *ht = x.mf.ht;
  const MixConst& k = x.k;
  const float sn_c = x.sn(i, j), sn_e = x.sn(i + 1, j);
  const float u_e = 0.5f * (un[c] + un[e]) * k.dy_t;
  const float depe = ht[e] + sn_e;
  const float u_w = 0.5f * (un[c] + un[wst]) * k.dy_t;
  const float depw = ht[c] + sn_c;
  const float v_sc = 0.5f * (vn[s] + vn[se]);
  const float v_s = 0.5f * v_sc * k.dxv2;
  const float deps = 0.5f * (hv[s] + x.sv(i, j - 1) + hv[se] + x.sv(i + 1, j - 1));
  const float v_nc = 0.5f * (vn[c] + vn[e]);
  const float v_n = 0.5f * v_nc * k.dxv2;
  const float depn = 0.5f * (hv[c] + x.sv(i, j) + hv[e] + x.sv(i + 1, j));
  const float uu_w = wlo(u_w) * un[c] + whi(u_w) * un[wst];
  const float uu_e = whi(u_e) * un[c] + wlo(u_e) * un[e];
  const bool south_dry = x.m(i, j - 1) <= 0 || x.m(i + 1, j - 1) <= 0;
  const bool north_dry = x.m(i, j + 1) <= 0 || x.m(i + 1, j + 1) <= 0;
  const float uu_s = south_dry ? wlo(v_s) * un[c] : wlo(v_s) * un[c] + whi(v_s) * un[s];
  const float uu_n = north_dry ? whi(v_n) * un[c] : whi(v_n) * un[c] + wlo(v_n) * un[n];
  const float adv = uu_w * u_w * depw - uu_e * u_e * depe + uu_s * v_s * deps -
                    uu_n * v_n * depn;
  const float dudx_e = (un[e] - un[c]) * k.r_dx_t * depe;
  const float dudx_w = (un[c] - un[wst]) * k.r_dx_t * depw;
  const float Hu = hu[c] + x.su(i, j);
  const float dudy_s =
      south_dry ? 0.f : (un[c] - un[s]) * k.r_dyu2 * (Hu + hu[s] + x.su(i, j - 1));
  const float dudy_n =
      north_dry ? 0.f : (un[n] - un[c]) * k.r_dyu2 * (Hu + hu[n] + x.su(i, j + 1));
  const float vis =
      k.visc * ((dudx_e - dudx_w) * k.dy_u + (dudy_n - dudy_s) * k.dx_u * 0.5f);
  const float cor = 0.5f * (k.cor_u * (v_sc + v_nc)) * k.area_u * Hu;
  const float hpg = -k.g * Hu * k.dy_u * (sn_e - sn_c);
  out = (un[c] * Hu + k.rdt * (adv + vis + cor + hpg) * k.r_area_u) * x.mf.rhu[c] * k.r_fric;
  return true;
}

// momentum_v_kern.c:125-241 in FP32 at (i, j), with the masked branches
// (its first guard reads the east mask, as the reference kernel does).
__device__ bool gmom_v(const GCtx& x, int i, int j, float& out) {
  const int W = x.d.width, c = j * W + i, e = c + 1, wst = c - 1, s = c - W, n = c + W,
            nw = n - 1;
  if (x.m(i, j) + x.m(i + 1, j) <= 0) return false;
  if (x.m(i, j) <= 0 || x.m(i, j + 1) <= 0) return false;
  const float *un = x.ms.un_in, *vn = x.ms.vn_in, *hu = x.mf.hu, *hv = x.mf.hv, *ht = x.mf.ht;
  const MixConst& k = x.k;
  const float sn_c = x.sn(i, j), sn_n = x.sn(i, j + 1);
  const float v_n = 0.5f * (vn[c] + vn[n]) * k.dx_t;
  const float depn = ht[n] + sn_n;
  const float v_s = 0.5f * (vn[c] + vn[s]) * k.dx_t;
  const float deps = ht[c] + sn_c;
  const float u_wc = 0.5f * (un[wst] + un[nw]);
  const float u_w = 0.5f * u_wc * k.dyu2;
  const float depw = 0.5f * (hu[wst] + x.su(i - 1, j) + hu[nw] + x.su(i - 1, j + 1));
  const float u_ec = 0.5f * (un[c] + un[n]);
  const float u_e = 0.5f * u_ec * k.dyu2;
  const float depe = 0.5f * (hu[c] + x.su(i, j) + hu[n] + x.su(i, j + 1));
  const float vv_s = wlo(v_s) * vn[c] + whi(v_s) * vn[s];
  const float vv_n = whi(v_n) * vn[c] + wlo(v_n) * vn[n];
  const bool west_dry = x.m(i - 1, j) <= 0 || x.m(i - 1, j + 1) <= 0;
  const bool east_dry = x.m(i + 1, j) <= 0 || x.m(i + 1, j + 1) <= 0;
  const float vv_w = west_dry ? wlo(u_w) * vn[c] : wlo(u_w) * vn[c] + whi(u_w) * vn[wst];
  const float vv_e = east_dry ? whi(u_e) * vn[c] : whi(u_e) * vn[c] + wlo(u_e) * vn[e];
  const float adv = vv_w * u_w * depw - vv_e * u_e * depe + vv_s * v_s * deps -
                    vv_n * v_n * depn;
  const float dvdy_n = (vn[n] - vn[c]) * k.r_dy_t * depn;
  const float dvdy_s = (vn[c] - vn[s]) * k.r_dy_t * deps;
  const float Hv = hv[c] + x.sv(i, j);
  const float dvdx_w =
      west_dry ? 0.f : (vn[c] - vn[wst]) * k.r_dxv2 * (Hv + hv[wst] + x.sv(i - 1, j));
  const float dvdx_e =
      east_dry ? 0.f : (vn[e] - vn[c]) * k.r_dxv2 * (Hv + hv[e] + x.sv(i + 1, j));
  const float vis =
      k.visc * ((dvdy_n - dvdy_s) * k.dx_v + (dvdx_e - dvdx_w) * k.dy_v * 0.5f);
  const float cor = -0.5f * (k.cor_v * (u_ec + u_wc)) * k.area_v * Hv;
  const float hpg = -k.g * Hv * k.dx_v * (sn_n - sn_c);
  out = (vn[c] * Hv + k.rdt * (adv + vis + cor + hpg) * k.r_area_v) * x.mf.rhv[c] * k.r_fric;
  return true;
}

// u at face (i, j) before Flather: momentum where it applies, bc_solid_u.
__device__ float gua_pre(const GCtx& x, int i, int j) {
  const int c = x.ix(i, j);
  float ua = x.in_copy(i, j) ? x.ms.un_in[c] : (float)x.f.ua[c];
  if (i >= x.d.xs && i <= x.d.xe - 1 && j >= x.d.ys && j <= x.d.ye) {
    float v;
    if (gmom_u(x, i, j, v)) ua = v;
  }
  if (i >= x.d.xs - 1 && i <= x.d.xe && j >= x.d.ys - 1 && j <= x.d.ye + 1 &&
      x.m(i, j) * x.m(i + 1, j) == 0)
    ua = 0.f;
  return ua;
}

// v at face (i, j) before Flather: momentum where it applies, bc_solid_v.
__device__ float gva_pre(const GCtx& x, int i, int j) {
  const int c = x.ix(i, j);
  float va = x.in_copy(i, j) ? x.ms.vn_in[c] : (float)x.f.va[c];
  if (i >= x.d.xs && i <= x.d.xe && j >= x.d.ys && j <= x.d.ye - 1) {
    float v;
    if (gmom_v(x, i, j, v)) va = v;
  }
  if (i >= x.d.xs - 1 && i <= x.d.xe + 1 && j >= x.d.ys - 1 && j <= x.d.ye &&
      x.m(i, j) * x.m(i, j + 1) == 0)
    va = 0.f;
  return va;
}

// One cell (i, j) of the copy region by the reference's per-point code:
// continuity and bc_ssh, momentum, bc_solid and bc_flather.
__device__ void general_cell(const GCtx& x, int i, int j, double tide) {
  const Dims& d = x.d;
  const MixConst& k = x.k;
  const int W = d.width, c = x.ix(i, j);
  float2 ssh = x.ms.sn_in[c];
  if (i >= d.xs && i <= d.xe && j >= d.ys && j <= d.ye) {
    const float r1 = (x.su(i, j) + x.mf.hu[c]) * x.ms.un_in[c];
    const float r2 = (x.su(i - 1, j) + x.mf.hu[c - 1]) * x.ms.un_in[c - 1];
    const float r3 = (x.sv(i, j) + x.mf.hv[c]) * x.ms.vn_in[c];
    const float r4 = (x.sv(i, j - 1) + x.mf.hv[c - W]) * x.ms.vn_in[c - W];
    ssh = dd_add(ssh, (r2 - r1 + r4 - r3) * k.rdt * k.r_area_t);
    if (x.m(i, j) > 0 && (x.m(i, j - 1) < 0 || x.m(i, j + 1) < 0 || x.m(i + 1, j) < 0 ||
                          x.m(i - 1, j) < 0)) {
      const float hi = (float)tide;
      ssh = make_float2(hi, (float)(tide - (double)hi));
    }
  }
  x.ms.sn_out[c] = ssh;

  float ua = x.ms.un_in[c];
  if (i <= d.xe) {
    ua = gua_pre(x, i, j);
    const int mc = x.m(i, j), me = x.m(i + 1, j);
    if (mc + me > -1) {
      if (mc < 0)
        ua = gua_pre(x, i + 1, j) + sqrtf(k.g / x.mf.hu[c]) * (x.su(i, j) - x.su(i + 1, j));
      else if (me < 0 && i >= 1)
        ua = gua_pre(x, i - 1, j) + sqrtf(k.g / x.mf.hu[c]) * (x.su(i, j) - x.su(i - 1, j));
    }
  }
  x.ms.un_out[c] = ua;

  float va = gva_pre(x, i, j);
  const int mc = x.m(i, j), mn = x.m(i, j + 1);
  if (mc + mn > -1) {
    if (mc < 0)
      va = gva_pre(x, i, j + 1) + sqrtf(k.g / x.mf.hv[c]) * (x.sv(i, j) - x.sv(i, j + 1));
    else if (mn < 0 && j >= 1)
      va = gva_pre(x, i, j - 1) + sqrtf(k.g / x.mf.hv[c]) * (x.sv(i, j) - x.sv(i, j - 1));
  }
  x.ms.vn_out[c] = va;
}

// Whether the march updates cell (i, j): interior away from the edges of
// next_ssh's ranges, 3x3 mask neighbourhood wet.
__device__ __forceinline__ bool march_regular(const Fields& f, const Dims& d, int i, int j) {
  if (i < d.xs + 1 || i > d.xe - 1 || j < d.ys + 1 || j > d.ye - 1) return false;
  const int W = d.width;
#pragma unroll
  for (int dj = -1; dj <= 1; dj++)
#pragma unroll
    for (int di = -1; di <= 1; di++)
      if (f.tmask[(j + dj) * W + (i + di)] <= 0) return false;
  return true;
}

}  // namespace
}  // namespace mixk
}  // namespace nl2d
