// Device code of one tile of the fused FP64 NEMOLite2D step, shared by the
// single-domain kernel (nl2d_fused.cu) and the ensemble's persistent kernel
// (nl2d_ensemble.cu).  See nl2d_fused.cu for what a step computes and why it
// is bit-identical to the reference.
#pragma once
#include "nl2d_exact.cuh"
#include "nl2d_internal.h"

namespace nl2d {
namespace {


// A tile is TX x TY cells, worked on by 256 threads laid out TX x
// (256 / TX); in the last phase each thread updates TY / (256 / TX) cells
// of one column.  Tile<TX, TY> holds a shape's constants; the ensemble
// instantiates several shapes (its autotuner picks one), the single-domain
// kernel uses DefaultTile.  The arithmetic does not depend on the shape.
constexpr int HALO = 2, NTHREADS = 256;

// Step-invariant constants of the fast path, evaluated on the host with the
// operations the reference performs per point (e.g. dx_v[c] + dx_v[e] on a
// uniform grid is one add of two equal values), so they are bit-identical.
struct FastConst {
  double area_t, area_u, area_v, dx_u, dx_v, dx_t, dy_u, dy_v, dy_t;
  double r_area_t, r_area_u, r_area_v, r_dx_t, r_dy_t;  // RN(1/d)
  double dxv2, dyu2, r_dxv2, r_dyu2;                    // dx_v + dx_v, dy_u + dy_u
  double fric, r_fric;                                  // 1.0 + cbfr * rdt
  double cor_u, cor_v;                                  // 2. * omega * sin(gphi * d2r)
  double neg_g, rdt, visc, g;
  int fast_div;  // every constant divisor lies in [2^-100, 2^100]
};

// One domain of an ensemble (device-resident descriptor).
struct EnsDomain {
  Fields f;
  FusedState fs[2];  // [parity]: state buffers read and written at that parity
  Dims d;
  Scalars p;
  UniformMetrics um;
  FastConst k;
};

// Division by a step constant: the Markstein form when the constants allow
// it, otherwise the IEEE divide.  Both give the same bits.
__device__ __forceinline__ double dvc(double x, double d, double r, int fast) {
  return fast ? div_rn(x, d, r) : x / d;
}
// Division by a per-face depth with a precomputed reciprocal; r == 0 marks
// a depth outside [2^-100, 2^100] (IEEE divide).
__device__ __forceinline__ double dvf(double x, double d, double r) {
  return bits(r) != 0 ? div_rn(x, d, r) : x / d;
}

template <int SX>
struct Ctx {
  const double *__restrict__ sn, *__restrict__ un, *__restrict__ vn;
  const double *__restrict__ hu, *__restrict__ hv, *__restrict__ ht;
  const double *__restrict__ ssha_u, *__restrict__ ssha_v;
  const double *__restrict__ r_hu, *__restrict__ r_hv;
  const int* __restrict__ m;
  const double* su_tile;  // shared: sshn_u seen by this step
  const double* sv_tile;  // shared: sshn_v seen by this step
  int W, i0, j0;          // tile origin (cell coordinates of su_tile[0] + HALO)
  Dims d;
  FastConst k;

  // Shared-memory slot of cell (i,j); the caller keeps (i,j) within the
  // tile plus its halo.
  __device__ __forceinline__ int slot(int i, int j) const {
    return (j - j0 + HALO) * SX + (i - i0 + HALO);
  }
  __device__ __forceinline__ bool in_copy(int i, int j) const {
    return i >= d.xs - 1 && i <= d.xe + 1 && j >= d.ys - 1 && j <= d.ye;
  }
  // sshn_u / sshn_v this step sees at face (i,j)
  __device__ __forceinline__ double su(int i, int j) const { return su_tile[slot(i, j)]; }
  __device__ __forceinline__ double sv(int i, int j) const { return sv_tile[slot(i, j)]; }
};

// next_sshu_code / next_sshv_code (time_update_kern.c:90-155) at face
// (i,j) over their loop ranges; faces outside them keep the stored value.
// The tile stages these in shared memory (phase 0 of fused_tile); the
// general pass without a tile computes them where it reads them.
__device__ __forceinline__ bool next_sshu_at(const int* __restrict__ m,
                                             const double* __restrict__ sn, const Dims& d,
                                             const FastConst& k, int i, int j, double& su) {
  if (!(j >= d.ys && j <= d.ye && i >= d.xs && i <= d.xe - 1)) return false;
  const int c = j * d.width + i, n = c + 1, mm = m[c], mn = m[n];
  if (mm + mn <= 0) return false;
  if (mm * mn > 0) {
    double rtmp1 = k.area_t * sn[c] + k.area_t * sn[n];
    su = dvc(half(rtmp1), k.area_u, k.r_area_u, k.fast_div);
  } else if (mm <= 0) {
    su = sn[n];
  } else {
    su = sn[c];
  }
  return true;
}
__device__ __forceinline__ bool next_sshv_at(const int* __restrict__ m,
                                             const double* __restrict__ sn, const Dims& d,
                                             const FastConst& k, int i, int j, double& sv) {
  if (!(j >= d.ys && j <= d.ye - 1 && i >= d.xs && i <= d.xe)) return false;
  const int c = j * d.width + i, n = c + d.width, mm = m[c], mn = m[n];
  if (mm + mn <= 0) return false;
  if (mm * mn > 0) {
    double rtmp1 = k.area_t * sn[c] + k.area_t * sn[n];
    sv = dvc(half(rtmp1), k.area_v, k.r_area_v, k.fast_div);
  } else if (mm <= 0) {
    sv = sn[n];
  } else {
    sv = sn[c];
  }
  return true;
}

// The general pass's context without a tile: every input read from the
// domain's arrays in global memory (the members refer to the domain's
// descriptor, so no thread holds a copy of it), sshn_u / sshn_v computed
// where they are read.  Valid for the faces a copy-region cell's general
// update reads, all of which lie inside the array.
struct GlobalCtx {
  const double* const& sn;  // the state buffers read this step
  const double* const& un;
  const double* const& vn;
  double* const& hu;  // the domain's Fields
  double* const& hv;
  double* const& ht;
  double* const& ssha_u;
  double* const& ssha_v;
  double* const& r_hu;
  double* const& r_hv;
  int* const& m;
  double* const& sshn_u;
  double* const& sshn_v;
  const int& W;
  const Dims& d;
  const FastConst& k;

  __device__ __forceinline__ bool in_copy(int i, int j) const {
    return i >= d.xs - 1 && i <= d.xe + 1 && j >= d.ys - 1 && j <= d.ye;
  }
  __device__ __forceinline__ double su(int i, int j) const {
    double v;
    return next_sshu_at(m, sn, d, k, i, j, v) ? v : sshn_u[j * W + i];
  }
  __device__ __forceinline__ double sv(int i, int j) const {
    double v;
    return next_sshv_at(m, sn, d, k, i, j, v) ? v : sshn_v[j * W + i];
  }
};

// (0.5 - copysign(0.5, w)) * p and (0.5 + copysign(0.5, w)) * p alone (the
// masked upwind forms): p, or +0 * p.
// (the IEEE form for a non-finite p is out of line, as for the helpers of
// nl2d_exact.cuh, so that it is not issued on every call)
static __device__ __noinline__ double zero_times_ieee(double p) { return 0.0 * p; }
__device__ __forceinline__ double zero_times(double p) {
  const long long b = bits(p);
  if (((b >> 52) & 0x7ff) == 0x7ff) return zero_times_ieee(p);
  return from_bits(b & (long long)0x8000000000000000ULL);
}
__device__ __forceinline__ double lo_only(double w, double p) {
  return bits(w) < 0 ? p : zero_times(p);
}
__device__ __forceinline__ double hi_only(double w, double p) {
  return bits(w) < 0 ? zero_times(p) : p;
}

// momentum_u_code (momentum_u_kern.c:150-262) at u face (i,j) in its loop
// range, with the masked (slip-wall) branches; returns false where the
// kernel returns early (ua keeps its value).  Same operations as the
// reference, with the exact helpers for halving, upwind picks and division.
template <class X>
__device__ __forceinline__ bool mom_u(const X& x, int i, int j, double& out) {
  const int W = x.W, c = j * W + i, e = c + 1, wst = c - 1, s = c - W, n = c + W,
            se = s + 1, ne = n + 1;
  const int* m = x.m;
  if (m[c] + m[e] <= 0) return false;
  if (m[c] <= 0 || m[e] <= 0) return false;
  const double *un = x.un, *vn = x.vn, *hu = x.hu, *hv = x.hv, *ht = x.ht, *sn = x.sn;
  const FastConst& k = x.k;
  const double su_c = x.su(i, j), su_s = x.su(i, j - 1), su_n = x.su(i, j + 1);
  const double sv_s = x.sv(i, j - 1), sv_se = x.sv(i + 1, j - 1), sv_c = x.sv(i, j),
               sv_e = x.sv(i + 1, j);

  double u_e = half(un[c] + un[e]) * k.dy_t;
  double depe = ht[e] + sn[e];
  double u_w = half(un[c] + un[wst]) * k.dy_t;
  double depw = ht[c] + sn[c];
  double v_sc = half(vn[s] + vn[se]);
  double v_s = half(v_sc) * k.dxv2;
  double deps = half(hv[s] + sv_s + hv[se] + sv_se);
  double v_nc = half(vn[c] + vn[e]);
  double v_n = half(v_nc) * k.dxv2;
  double depn = half(hv[c] + sv_c + hv[e] + sv_e);

  double uu_w = upwind(u_w, un[c], un[wst]);
  double uu_e = upwind(u_e, un[e], un[c]);
  const bool south_dry = m[s] <= 0 || m[se] <= 0;
  const bool north_dry = m[n] <= 0 || m[ne] <= 0;
  double uu_s = south_dry ? lo_only(v_s, un[c]) : upwind(v_s, un[c], un[s]);
  double uu_n = north_dry ? hi_only(v_n, un[c]) : upwind(v_n, un[n], un[c]);
  double adv = uu_w * u_w * depw - uu_e * u_e * depe + uu_s * v_s * deps -
               uu_n * v_n * depn;

  double dudx_e = dvc(un[e] - un[c], k.dx_t, k.r_dx_t, k.fast_div) * (ht[e] + sn[e]);
  double dudx_w = dvc(un[c] - un[wst], k.dx_t, k.r_dx_t, k.fast_div) * (ht[c] + sn[c]);
  double dudy_s = south_dry ? 0.0
                            : dvc(un[c] - un[s], k.dyu2, k.r_dyu2, k.fast_div) *
                                  (hu[c] + su_c + hu[s] + su_s);
  double dudy_n = north_dry ? 0.0
                            : dvc(un[n] - un[c], k.dyu2, k.r_dyu2, k.fast_div) *
                                  (hu[c] + su_c + hu[n] + su_n);
  double vis = (dudx_e - dudx_w) * k.dy_u + half((dudy_n - dudy_s) * k.dx_u);
  vis = k.visc * vis;
  double cor = half(k.cor_u * (v_sc + v_nc)) * k.area_u * (hu[c] + su_c);
  double hpg = k.neg_g * (hu[c] + su_c) * k.dy_u * (sn[e] - sn[c]);
  const double num =
      un[c] * (hu[c] + su_c) + dvc(k.rdt * (adv + vis + cor + hpg), k.area_u, k.r_area_u,
                                   k.fast_div);
  out = dvc(dvf(num, hu[c] + x.ssha_u[c], x.r_hu[c]), k.fric, k.r_fric, k.fast_div);
  return true;
}

// momentum_v_code (momentum_v_kern.c:125-241) at v face (i,j).
template <class X>
__device__ __forceinline__ bool mom_v(const X& x, int i, int j, double& out) {
  const int W = x.W, c = j * W + i, e = c + 1, wst = c - 1, s = c - W, n = c + W,
            nw = n - 1, ne = n + 1;
  const int* m = x.m;
  if (m[c] + m[e] <= 0) return false;
  if (m[c] <= 0 || m[n] <= 0) return false;
  const double *un = x.un, *vn = x.vn, *hu = x.hu, *hv = x.hv, *ht = x.ht, *sn = x.sn;
  const FastConst& k = x.k;
  const double su_w = x.su(i - 1, j), su_nw = x.su(i - 1, j + 1), su_c = x.su(i, j),
               su_n = x.su(i, j + 1);
  const double sv_c = x.sv(i, j), sv_w = x.sv(i - 1, j), sv_e = x.sv(i + 1, j);

  double v_n = half(vn[c] + vn[n]) * k.dx_t;
  double depn = ht[n] + sn[n];
  double v_s = half(vn[c] + vn[s]) * k.dx_t;
  double deps = ht[c] + sn[c];
  double u_wc = half(un[wst] + un[nw]);
  double u_w = half(u_wc) * k.dyu2;
  double depw = half(hu[wst] + su_w + hu[nw] + su_nw);
  double u_ec = half(un[c] + un[n]);
  double u_e = half(u_ec) * k.dyu2;
  double depe = half(hu[c] + su_c + hu[n] + su_n);

  double vv_s = upwind(v_s, vn[c], vn[s]);
  double vv_n = upwind(v_n, vn[n], vn[c]);
  const bool west_dry = m[wst] <= 0 || m[nw] <= 0;
  const bool east_dry = m[e] <= 0 || m[ne] <= 0;
  double vv_w = west_dry ? lo_only(u_w, vn[c]) : upwind(u_w, vn[c], vn[wst]);
  double vv_e = east_dry ? hi_only(u_e, vn[c]) : upwind(u_e, vn[e], vn[c]);
  double adv = vv_w * u_w * depw - vv_e * u_e * depe + vv_s * v_s * deps -
               vv_n * v_n * depn;

  double dvdy_n = dvc(vn[n] - vn[c], k.dy_t, k.r_dy_t, k.fast_div) * (ht[n] + sn[n]);
  double dvdy_s = dvc(vn[c] - vn[s], k.dy_t, k.r_dy_t, k.fast_div) * (ht[c] + sn[c]);
  double dvdx_w = west_dry ? 0.0
                           : dvc(vn[c] - vn[wst], k.dxv2, k.r_dxv2, k.fast_div) *
                                 (hv[c] + sv_c + hv[wst] + sv_w);
  double dvdx_e = east_dry ? 0.0
                           : dvc(vn[e] - vn[c], k.dxv2, k.r_dxv2, k.fast_div) *
                                 (hv[c] + sv_c + hv[e] + sv_e);
  double vis = (dvdy_n - dvdy_s) * k.dx_v + half((dvdx_e - dvdx_w) * k.dy_v);
  vis = k.visc * vis;
  double cor = -half(k.cor_v * (u_ec + u_wc)) * k.area_v * (hv[c] + sv_c);
  double hpg = k.neg_g * (hv[c] + sv_c) * k.dx_v * (sn[n] - sn[c]);
  const double num =
      vn[c] * (hv[c] + sv_c) + dvc(k.rdt * (adv + vis + cor + hpg), k.area_v, k.r_area_v,
                                   k.fast_div);
  out = dvc(dvf(num, hv[c] + x.ssha_v[c], x.r_hv[c]), k.fric, k.r_fric, k.fast_div);
  return true;
}

// ua at u face (i,j) after momentum_u and bc_solid_u, before Flather: the
// value bc_flather_u reads.  On the copy region the previous step's ua is
// the current un; elsewhere it is the ua array, which no fused step changes.
template <class X>
__device__ __forceinline__ double ua_pre_flather(const X& x, const double* ua_arr,
                                                 int i, int j) {
  const int c = j * x.W + i;
  double ua = x.in_copy(i, j) ? x.un[c] : ua_arr[c];
  if (i >= x.d.xs && i <= x.d.xe - 1 && j >= x.d.ys && j <= x.d.ye) {
    double v;
    if (mom_u(x, i, j, v)) ua = v;
  }
  if (i >= x.d.xs - 1 && i <= x.d.xe && j >= x.d.ys - 1 && j <= x.d.ye + 1 &&
      x.m[c] * x.m[c + 1] == 0)
    ua = 0.0;  // bc_solid_u
  return ua;
}

template <class X>
__device__ __forceinline__ double va_pre_flather(const X& x, const double* va_arr,
                                                 int i, int j) {
  const int c = j * x.W + i;
  double va = x.in_copy(i, j) ? x.vn[c] : va_arr[c];
  if (i >= x.d.xs && i <= x.d.xe && j >= x.d.ys && j <= x.d.ye - 1) {
    double v;
    if (mom_v(x, i, j, v)) va = v;
  }
  if (i >= x.d.xs - 1 && i <= x.d.xe + 1 && j >= x.d.ys - 1 && j <= x.d.ye &&
      x.m[c] * x.m[c + x.W] == 0)
    va = 0.0;  // bc_solid_v
  return va;
}

// A copy-region cell's update by the reference's per-point code, in its
// order: sea-surface height (continuity_kern.c:90-117, then bc_ssh), u at
// the east face (momentum_u, bc_solid_u, bc_flather_u), v at the north face
// (momentum_v, bc_solid_v, bc_flather_v).  x supplies the fields and the
// sshn_u / sshn_v this step sees (a tile's shared memory, or global memory).
template <class X>
__device__ __forceinline__ void general_cell(const X& x, const Fields& f, const FusedState& fs,
                                             const Scalars& p, double tide, int i, int j) {
  const int W = x.W;
  const Dims& d = x.d;
  const FastConst& k = x.k;
  const int* __restrict__ m = x.m;
  const double* __restrict__ sn = x.sn;
  const double* __restrict__ un = x.un;
  const double* __restrict__ vn = x.vn;
  const int c = j * W + i;

  double ssh = sn[c];
  if (i >= d.xs && i <= d.xe && j >= d.ys && j <= d.ye) {
    const int w = c - 1, s = c - W;
    double r1 = (x.su(i, j) + f.hu[c]) * un[c];
    double r2 = (x.su(i - 1, j) + f.hu[w]) * un[w];
    double r3 = (x.sv(i, j) + f.hv[c]) * vn[c];
    double r4 = (x.sv(i, j - 1) + f.hv[s]) * vn[s];
    ssh = sn[c] + dvc((r2 - r1 + r4 - r3) * k.rdt, k.area_t, k.r_area_t, k.fast_div);
    if (m[c] > 0 && (m[c - W] < 0 || m[c + W] < 0 || m[c + 1] < 0 || m[c - 1] < 0))
      ssh = tide;
  }
  fs.sshn_out[c] = ssh;

  double ua = un[c];
  if (i <= d.xe) {  // u whole range [xs-1, xe] x [ys-1, ye+1] (tiling gives the rest)
    ua = ua_pre_flather(x, f.ua, i, j);
    if (m[c] + m[c + 1] > -1) {
      if (m[c] < 0) {
        ua = ua_pre_flather(x, f.ua, i + 1, j) +
             sqrt(p.g / f.hu[c]) * (x.su(i, j) - x.su(i + 1, j));
      } else if (m[c + 1] < 0 && i >= 1) {  // i == 0 would read outside the array
        ua = ua_pre_flather(x, f.ua, i - 1, j) +
             sqrt(p.g / f.hu[c]) * (x.su(i, j) - x.su(i - 1, j));
      }
    }
  }
  fs.un_out[c] = ua;

  // the copy region is exactly the v whole range [xs-1, xe+1] x [ys-1, ye]
  double va = va_pre_flather(x, f.va, i, j);
  if (m[c] + m[c + W] > -1) {
    if (m[c] < 0) {
      va = va_pre_flather(x, f.va, i, j + 1) +
           sqrt(p.g / f.hv[c]) * (x.sv(i, j) - x.sv(i, j + 1));
    } else if (m[c + W] < 0 && j >= 1) {
      va = va_pre_flather(x, f.va, i, j - 1) +
           sqrt(p.g / f.hv[c]) * (x.sv(i, j) - x.sv(i, j - 1));
    }
  }
  fs.vn_out[c] = va;
}

// Shared-memory layout of one tile.  Phase 0 (halo 2) holds the loaded
// fields and the sshn_u / sshn_v values this step sees; phase 1 (halo 1)
// holds the terms that two neighbouring updates share.
enum { A_SN, A_UN, A_VN, A_HU, A_HV, A_SU, A_SV, A_HUS, A_HVS, N_A0 };
enum { B_FLXU, B_FLXV, B_GX, B_GY, B_FXU, B_FYV, B_VSC, B_FYU, B_QY, B_UWC, B_FXV, B_QX, N_B1 };

template <int TX_, int TY_>
struct Tile {
  static constexpr int TX = TX_, TY = TY_;
  static constexpr int RPP = NTHREADS / TX;  // rows per pass of the thread block
  static constexpr int RPT = TY / RPP;       // cells per thread in the update phase
  static_assert(NTHREADS % TX == 0 && TY % RPP == 0 && (RPT == 1 || RPT == 2 || RPT == 4),
                "tile shape");
  static constexpr int SX = TX + 2 * HALO, SY = TY + 2 * HALO;
  static constexpr int S0 = SX * SY;  // phase-0 positions (36 x 20 for 32 x 16)
  static constexpr int P1X = TX + 2, P1Y = TY + 2;
  static constexpr int S1 = P1X * P1Y;  // phase-1 positions (34 x 18 for 32 x 16)
  // + the mask, and the list of the tile's general (non-regular) cells
  static constexpr size_t kSmemBytes =
      sizeof(double) * (N_A0 * S0 + N_B1 * S1) + sizeof(int) * (S0 + TX * TY + 1);
  // two CTAs of 256 threads per SM when their shared memory fits
  static constexpr int kMinBlocks = 2 * kSmemBytes <= 227 * 1024 ? 2 : 1;
};
using DefaultTile = Tile<32, 16>;

// A regular cell's new (sshn_t, un, vn) from the tile's staged fields (a0)
// and shared terms (b1) at its slots q (phase 0) and r (phase 1): continuity
// (continuity_kern.c:90-117) and unmasked momentum
// (momentum_u_kern.c:184-261, momentum_v_kern.c:159-239) in the
// reference's operation order.  sau, rhu, sav, rhv: ssha_u, RN(1 / (hu +
// ssha_u)), ssha_v, RN(1 / (hv + ssha_v)) at the cell.
struct RegOut {
  double ssh, u, v;
};
template <class T>
__device__ __forceinline__ RegOut regular_cell(const double* a0, const double* b1, int q, int r,
                                               double sau, double rhu, double sav, double rhv,
                                               const FastConst& k) {
  constexpr int S0 = T::S0, S1 = T::S1, SX = T::SX, P1X = T::P1X;
#define A(qq, t) a0[(qq) * S0 + (t)]
#define B(qq, t) b1[(qq) * S1 + (t)]
  RegOut o;
  const double snc = A(A_SN, q), Hu = A(A_HUS, q), Hv = A(A_HVS, q);
  const double ssh = (((B(B_FLXU, r - 1) - B(B_FLXU, r)) + B(B_FLXV, r - P1X)) - B(B_FLXV, r)) *
                     k.rdt;
  o.ssh = snc + dvc(ssh, k.area_t, k.r_area_t, k.fast_div);
  {
    const double adv = ((B(B_FXU, r) - B(B_FXU, r + 1)) + B(B_FYU, r)) - B(B_FYU, r + P1X);
    const double dudy_s = B(B_QY, r) * ((Hu + A(A_HU, q - SX)) + A(A_SU, q - SX));
    const double dudy_n = B(B_QY, r + P1X) * ((Hu + A(A_HU, q + SX)) + A(A_SU, q + SX));
    double vis = (B(B_GX, r + 1) - B(B_GX, r)) * k.dy_u + half((dudy_n - dudy_s) * k.dx_u);
    vis = k.visc * vis;
    const double cor = (half(k.cor_u * (B(B_VSC, r) + B(B_VSC, r + P1X))) * k.area_u) * Hu;
    const double hpg = ((k.neg_g * Hu) * k.dy_u) * (A(A_SN, q + 1) - snc);
    const double num =
        A(A_UN, q) * Hu +
        dvc(k.rdt * (((adv + vis) + cor) + hpg), k.area_u, k.r_area_u, k.fast_div);
    const double t1 = dvf(num, A(A_HU, q) + sau, rhu);
    o.u = dvc(t1, k.fric, k.r_fric, k.fast_div);
  }
  {
    const double adv = ((B(B_FXV, r) - B(B_FXV, r + 1)) + B(B_FYV, r)) - B(B_FYV, r + P1X);
    const double dvdx_w = B(B_QX, r) * ((Hv + A(A_HV, q - 1)) + A(A_SV, q - 1));
    const double dvdx_e = B(B_QX, r + 1) * ((Hv + A(A_HV, q + 1)) + A(A_SV, q + 1));
    double vis = (B(B_GY, r + P1X) - B(B_GY, r)) * k.dx_v + half((dvdx_e - dvdx_w) * k.dy_v);
    vis = k.visc * vis;
    const double cor = (-half(k.cor_v * (B(B_UWC, r + 1) + B(B_UWC, r))) * k.area_v) * Hv;
    const double hpg = ((k.neg_g * Hv) * k.dx_v) * (A(A_SN, q + SX) - snc);
    const double num =
        A(A_VN, q) * Hv +
        dvc(k.rdt * (((adv + vis) + cor) + hpg), k.area_v, k.r_area_v, k.fast_div);
    const double t1 = dvf(num, A(A_HV, q) + sav, rhv);
    o.v = dvc(t1, k.fric, k.r_fric, k.fast_div);
  }
#undef A
#undef B
  return o;
}

// One tile of the fused step: cells [i0, i0+TX) x [j0, j0+TY) of the copy
// region of one domain.  `tide` is this step's bc_ssh value.
template <class T>
__device__ __forceinline__ void fused_tile(const Fields& f, const FusedState& fs, const Dims& d,
                                           const Scalars& p, const UniformMetrics& um,
                                           const FastConst& k, double tide, int i0, int j0,
                                           double* smem) {
  constexpr int TX = T::TX, SX = T::SX, S0 = T::S0, S1 = T::S1, P1X = T::P1X;
  constexpr int ROWS_PER_PASS = T::RPP;
  double* a0 = smem;                 // [N_A0][S0]
  double* b1 = smem + N_A0 * S0;     // [N_B1][S1]
  int* mk = (int*)(b1 + N_B1 * S1);  // [S0]
  int* glist = mk + S0;              // [TX * TY] general cells of this tile
  int* gcount = glist + TX * T::TY;
#define A(q, t) a0[(q) * S0 + (t)]
#define B(q, t) b1[(q) * S1 + (t)]

  const int W = d.width, H = d.height;
  const int* __restrict__ m = f.tmask;
  const double* __restrict__ sn = fs.sshn_in;
  const double* __restrict__ un = fs.un_in;
  const double* __restrict__ vn = fs.vn_in;
  const int tid = threadIdx.y * TX + threadIdx.x;

  if (tid == 0) *gcount = 0;
  // ---- phase 0: fields and the sshn_u / sshn_v this step reads ----
  for (int t = tid; t < S0; t += NTHREADS) {
    const int i = i0 - HALO + t % SX, j = j0 - HALO + t / SX;
    double vsn = 0.0, vun = 0.0, vvn = 0.0, vhu = 0.0, vhv = 0.0, su = 0.0, sv = 0.0;
    int mm = 0;
    if (i >= 0 && i < W && j >= 0 && j < H) {
      const int c = j * W + i;
      vsn = sn[c];
      vun = un[c];
      vvn = vn[c];
      vhu = f.hu[c];
      vhv = f.hv[c];
      mm = m[c];
      // next_sshu_code / next_sshv_code (time_update_kern.c:90-155) over
      // their loop ranges; other faces keep the stored value, which is read
      // only for them.
      bool su_stored = true, sv_stored = true;
      if (j >= d.ys && j <= d.ye && i >= d.xs && i <= d.xe - 1) {
        const int n = c + 1, mn = m[n];
        if (mm + mn > 0) {
          su_stored = false;
          if (mm * mn > 0) {
            double rtmp1 = k.area_t * vsn + k.area_t * sn[n];
            su = dvc(half(rtmp1), k.area_u, k.r_area_u, k.fast_div);
          } else if (mm <= 0) {
            su = sn[n];
          } else {
            su = vsn;
          }
        }
      }
      if (j >= d.ys && j <= d.ye - 1 && i >= d.xs && i <= d.xe) {
        const int n = c + W, mn = m[n];
        if (mm + mn > 0) {
          sv_stored = false;
          if (mm * mn > 0) {
            double rtmp1 = k.area_t * vsn + k.area_t * sn[n];
            sv = dvc(half(rtmp1), k.area_v, k.r_area_v, k.fast_div);
          } else if (mm <= 0) {
            sv = sn[n];
          } else {
            sv = vsn;
          }
        }
      }
      if (su_stored) su = f.sshn_u[c];
      if (sv_stored) sv = f.sshn_v[c];
    }
    A(A_SN, t) = vsn;
    A(A_UN, t) = vun;
    A(A_VN, t) = vvn;
    A(A_HU, t) = vhu;
    A(A_HV, t) = vhv;
    A(A_SU, t) = su;
    A(A_SV, t) = sv;
    A(A_HUS, t) = vhu + su;
    A(A_HVS, t) = vhv + sv;
    mk[t] = mm;
  }
  __syncthreads();

  // ---- phase 1: terms shared by neighbouring updates ----
  // Every term is the exact operation sequence of momentum_{u,v}_kern.c /
  // continuity_kern.c for one of the two updates that use it; for the other
  // update the reference evaluates the same operations on the same operands
  // (addition commuted), so the bits agree.
  for (int t = tid; t < S1; t += NTHREADS) {
    const int ti = t % P1X, tj = t / P1X;
    const int i = i0 - 1 + ti, j = j0 - 1 + tj;
    const int q = (tj + 1) * SX + (ti + 1);  // phase-0 slot of (i,j)
    const int qw = q - 1, qs = q - SX, qse = qs + 1, qwn = qw + SX;
    const double ht = (i >= 0 && i < W && j >= 0 && j < H) ? f.ht[j * W + i] : 0.0;
    const double D = ht + A(A_SN, q);  // ht + sshn at T(i,j)
    const double u_c = A(A_UN, q), u_w = A(A_UN, qw), u_s = A(A_UN, qs), u_wn = A(A_UN, qwn);
    const double v_c = A(A_VN, q), v_w = A(A_VN, qw), v_s = A(A_VN, qs), v_se = A(A_VN, qse);
    // continuity fluxes (sshn_u + hu) * un and (sshn_v + hv) * vn
    B(B_FLXU, t) = A(A_HUS, q) * u_c;
    B(B_FLXV, t) = A(A_HVS, q) * v_c;
    // dudx at T(i,j) (dudx_w of u face i, dudx_e of face i-1); dvdy likewise
    B(B_GX, t) = dvc(u_c - u_w, k.dx_t, k.r_dx_t, k.fast_div) * D;
    B(B_GY, t) = dvc(v_c - v_s, k.dy_t, k.r_dy_t, k.fast_div) * D;
    // x-advective flux of u through T(i,j): uu_w * u_w * depw of face i
    const double U = half(u_c + u_w) * k.dy_t;
    B(B_FXU, t) = (upwind(U, u_c, u_w) * U) * D;
    // y-advective flux of v through T(i,j): vv_s * v_s * deps of face j
    const double V = half(v_c + v_s) * k.dx_t;
    B(B_FYV, t) = (upwind(V, v_c, v_s) * V) * D;
    // south edge of u face (i,j): v_sc, v_s, deps, uu_s (unmasked form)
    const double vsc = half(v_s + v_se);
    B(B_VSC, t) = vsc;
    const double Vs = half(vsc) * k.dxv2;
    const double deps = half((A(A_HVS, qs) + A(A_HV, qse)) + A(A_SV, qse));
    B(B_FYU, t) = (upwind(Vs, u_c, u_s) * Vs) * deps;
    B(B_QY, t) = dvc(u_c - u_s, k.dyu2, k.r_dyu2, k.fast_div);
    // west edge of v face (i,j): u_wc, u_w, depw, vv_w (unmasked form)
    const double uwc = half(u_w + u_wn);
    B(B_UWC, t) = uwc;
    const double Uw = half(uwc) * k.dyu2;
    const double depw = half((A(A_HUS, qw) + A(A_HU, qwn)) + A(A_SU, qwn));
    B(B_FXV, t) = (upwind(Uw, v_c, v_w) * Uw) * depw;
    B(B_QX, t) = dvc(v_c - v_w, k.dxv2, k.r_dxv2, k.fast_div);
  }
  __syncthreads();

  // Each thread owns the cells (i, j0 + row) of its rows.  Regular cells
  // (wet 3x3 neighbourhood: continuity without bc_ssh, unmasked momentum, no
  // solid-wall or Flather change) are computed here; the others are queued
  // for the packed general pass below, so that a warp holding a few boundary
  // cells does not run both paths.  When both of a thread's cells are
  // regular they are computed in one straight-line block, so the compiler
  // can interleave two independent FP64 chains; the per-face global inputs
  // are loaded first and the results stored last, so no store can alias a
  // later load.
#pragma unroll
  for (int pb = 0; pb < T::RPT; pb += 2) {
    constexpr int NP = T::RPT >= 2 ? 2 : 1;  // rows taken together
    const int i = i0 + threadIdx.x;
    int c[NP], q[NP], r[NP];
    bool reg[NP];
#pragma unroll
    for (int e = 0; e < NP; e++) {
      const int row = threadIdx.y + (pb + e) * ROWS_PER_PASS, j = j0 + row;
      c[e] = j * W + i;
      q[e] = (row + HALO) * SX + (threadIdx.x + HALO);
      r[e] = (row + 1) * P1X + (threadIdx.x + 1);
      const bool live = i <= d.xe + 1 && j <= d.ye;
      bool regular = live && i >= d.xs && i <= d.xe - 1 && j >= d.ys && j <= d.ye - 1;
      if (regular) {
#pragma unroll
        for (int dj = -1; dj <= 1; dj++)
#pragma unroll
          for (int di = -1; di <= 1; di++) regular &= mk[q[e] + dj * SX + di] > 0;
      }
      reg[e] = regular;
      if (live && !regular) glist[atomicAdd(gcount, 1)] = row * TX + threadIdx.x;
    }
    double sau[NP], rhu[NP], sav[NP], rhv[NP];
#pragma unroll
    for (int e = 0; e < NP; e++)
      if (reg[e]) {
        sau[e] = f.ssha_u[c[e]];
        rhu[e] = f.r_hu[c[e]];
        sav[e] = f.ssha_v[c[e]];
        rhv[e] = f.r_hv[c[e]];
      }
    RegOut o[NP];
    if (NP == 2 && reg[0] && reg[NP - 1]) {
      o[0] = regular_cell<T>(a0, b1, q[0], r[0], sau[0], rhu[0], sav[0], rhv[0], k);
      o[NP - 1] = regular_cell<T>(a0, b1, q[NP - 1], r[NP - 1], sau[NP - 1], rhu[NP - 1],
                                  sav[NP - 1], rhv[NP - 1], k);
    } else {
#pragma unroll
      for (int e = 0; e < NP; e++)
        if (reg[e])
          o[e] = regular_cell<T>(a0, b1, q[e], r[e], sau[e], rhu[e], sav[e], rhv[e], k);
    }
#pragma unroll
    for (int e = 0; e < NP; e++)
      if (reg[e]) {
        fs.sshn_out[c[e]] = o[e].ssh;
        fs.un_out[c[e]] = o[e].u;
        fs.vn_out[c[e]] = o[e].v;
      }
  }
  __syncthreads();

  // ---- general cells: the reference's per-point code, in its order ----
  const int ngen = *gcount;
  for (int g = tid; g < ngen; g += NTHREADS) {
    const int row = glist[g] / TX, col = glist[g] - (glist[g] / TX) * TX;
    Ctx<SX> x;
    x.sn = sn;
    x.un = un;
    x.vn = vn;
    x.hu = f.hu;
    x.hv = f.hv;
    x.ht = f.ht;
    x.ssha_u = f.ssha_u;
    x.ssha_v = f.ssha_v;
    x.r_hu = f.r_hu;
    x.r_hv = f.r_hv;
    x.m = m;
    x.su_tile = &A(A_SU, 0);
    x.sv_tile = &A(A_SV, 0);
    x.W = W;
    x.i0 = i0;
    x.j0 = j0;
    x.d = d;
    x.k = k;
    general_cell(x, f, fs, p, tide, i0 + col, j0 + row);
  }  // general cells
#undef A
#undef B
}

bool in_fast_range(double d) {
  return d > 0.0 && d >= 0x1p-100 && d <= 0x1p100;
}

// The fast path's constants for one domain (host side).
inline FastConst make_fast_const(const Scalars& s, const UniformMetrics& um) {
  FastConst k;
  k.area_t = um.area_t, k.area_u = um.area_u, k.area_v = um.area_v;
  k.dx_u = um.dx_u, k.dx_v = um.dx_v, k.dx_t = um.dx_t;
  k.dy_u = um.dy_u, k.dy_v = um.dy_v, k.dy_t = um.dy_t;
  k.dxv2 = um.dx_v + um.dx_v;
  k.dyu2 = um.dy_u + um.dy_u;
  k.fric = 1.0 + s.cbfr * s.rdt;
  k.cor_u = 2. * s.omega * um.sin_u;
  k.cor_v = 2. * s.omega * um.sin_v;
  k.neg_g = -s.g;
  k.g = s.g;
  k.rdt = s.rdt;
  k.visc = s.visc;
  const double divisors[8] = {k.area_t, k.area_u, k.area_v, k.dx_t, k.dy_t,
                              k.dxv2,   k.dyu2,   k.fric};
  bool fast = true;
  for (double v : divisors) fast = fast && in_fast_range(v);
  k.fast_div = fast ? 1 : 0;
  k.r_area_t = 1.0 / k.area_t, k.r_area_u = 1.0 / k.area_u, k.r_area_v = 1.0 / k.area_v;
  k.r_dx_t = 1.0 / k.dx_t, k.r_dy_t = 1.0 / k.dy_t;
  k.r_dxv2 = 1.0 / k.dxv2, k.r_dyu2 = 1.0 / k.dyu2;
  k.r_fric = 1.0 / k.fric;
  return k;
}

}  // namespace
}  // namespace nl2d
