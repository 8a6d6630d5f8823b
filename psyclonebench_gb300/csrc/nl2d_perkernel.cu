// Reference-structured NEMOLite2D step on the GPU: one sm_103a kernel per
// loop nest of the manual C++ PSy layer
// (benchmarks/nemo/nemolite2d/manual_versions/psykal_cpp/time_step.cpp:53-136),
// launched in the same order over the same index ranges.
//
// This path is the exact drop-in for any input: it keeps all 13 fields as
// the reference does and touches them in the reference's order, so it is
// correct even for a state that the fused kernel cannot take (the first
// step after an upload, masks with chained Flather faces).  Built with
// -fmad=false: every FP64 operation is the IEEE operation the reference C
// source writes, so results are bit-identical to the reference's serial
// build compiled with -ffp-contract=off.
#include "nl2d_internal.h"

#include <cmath>

namespace nl2d {

namespace {

// 2-D launch over rows [y0,y1] and columns [x0,x1] (inclusive).
struct Range {
  int x0, x1, y0, y1;
};

constexpr int BX = 32, BY = 8;

inline dim3 grid_for(const Range& r) {
  int nx = r.x1 - r.x0 + 1, ny = r.y1 - r.y0 + 1;
  if (nx < 1) nx = 1;
  if (ny < 1) ny = 1;
  return dim3((nx + BX - 1) / BX, (ny + BY - 1) / BY);
}

__device__ __forceinline__ bool at(const Range& r, int& i, int& j) {
  i = r.x0 + blockIdx.x * BX + threadIdx.x;
  j = r.y0 + blockIdx.y * BY + threadIdx.y;
  return i <= r.x1 && j <= r.y1;
}

// Upwind weights 0.5 -/+ copysign(0.5, x) (momentum_{u,v}_kern.c).
__device__ __forceinline__ double wlo(double x) { return 0.5 - copysign(0.5, x); }
__device__ __forceinline__ double whi(double x) { return 0.5 + copysign(0.5, x); }

// K1: continuity_code, kernels/c_family/continuity_kern.c:90-117.
__global__ void __launch_bounds__(BX* BY)
    k_continuity(Fields f, int W, Range r, double rdt) {
  int i, j;
  if (!at(r, i, j)) return;
  const int c = j * W + i, w = c - 1, s = c - W;
  double r1 = (f.sshn_u[c] + f.hu[c]) * f.un[c];
  double r2 = (f.sshn_u[w] + f.hu[w]) * f.un[w];
  double r3 = (f.sshn_v[c] + f.hv[c]) * f.vn[c];
  double r4 = (f.sshn_v[s] + f.hv[s]) * f.vn[s];
  f.ssha_t[c] = f.sshn_t[c] + (r2 - r1 + r4 - r3) * rdt / f.area_t[c];
}

// K2: momentum_u_code, kernels/c_family/momentum_u_kern.c:150-262, with the
// metric binding of time_step.cpp:61-68 (e1u=dx_u, e1v=dx_v, e1t=dx_t,
// e2u=dy_u, e2t=dy_t, e12u=area_u).  sin(gphiu*d2r) comes precomputed.
__global__ void __launch_bounds__(BX* BY)
    k_momentum_u(Fields f, int W, Range r, Scalars p) {
  int i, j;
  if (!at(r, i, j)) return;
  const int c = j * W + i, e = c + 1, wst = c - 1, s = c - W, n = c + W,
            se = s + 1, ne = n + 1;
  const int* m = f.tmask;
  if (m[c] + m[e] <= 0) return;
  if (m[c] <= 0 || m[e] <= 0) return;
  const double *un = f.un, *vn = f.vn, *hu = f.hu, *hv = f.hv, *ht = f.ht,
               *sn = f.sshn_t, *su = f.sshn_u, *sv = f.sshn_v;

  double u_e = 0.5 * (un[c] + un[e]) * f.dy_t[e];
  double depe = ht[e] + sn[e];
  double u_w = 0.5 * (un[c] + un[wst]) * f.dy_t[c];
  double depw = ht[c] + sn[c];
  double v_sc = 0.5 * (vn[s] + vn[se]);
  double v_s = 0.5 * v_sc * (f.dx_v[s] + f.dx_v[se]);
  double deps = 0.5 * (hv[s] + sv[s] + hv[se] + sv[se]);
  double v_nc = 0.5 * (vn[c] + vn[e]);
  double v_n = 0.5 * v_nc * (f.dx_v[c] + f.dx_v[e]);
  double depn = 0.5 * (hv[c] + sv[c] + hv[e] + sv[e]);

  double uu_w = wlo(u_w) * un[c] + whi(u_w) * un[wst];
  double uu_e = whi(u_e) * un[c] + wlo(u_e) * un[e];
  const bool south_dry = m[s] <= 0 || m[se] <= 0;
  const bool north_dry = m[n] <= 0 || m[ne] <= 0;
  double uu_s = south_dry ? wlo(v_s) * un[c] : wlo(v_s) * un[c] + whi(v_s) * un[s];
  double uu_n = north_dry ? whi(v_n) * un[c] : whi(v_n) * un[c] + wlo(v_n) * un[n];
  double adv = uu_w * u_w * depw - uu_e * u_e * depe + uu_s * v_s * deps -
               uu_n * v_n * depn;

  double dudx_e = (un[e] - un[c]) / f.dx_t[e] * (ht[e] + sn[e]);
  double dudx_w = (un[c] - un[wst]) / f.dx_t[c] * (ht[c] + sn[c]);
  double dudy_s = south_dry ? 0.0
                            : (un[c] - un[s]) / (f.dy_u[c] + f.dy_u[s]) *
                                  (hu[c] + su[c] + hu[s] + su[s]);
  double dudy_n = north_dry ? 0.0
                            : (un[n] - un[c]) / (f.dy_u[c] + f.dy_u[n]) *
                                  (hu[c] + su[c] + hu[n] + su[n]);
  double vis = (dudx_e - dudx_w) * f.dy_u[c] + (dudy_n - dudy_s) * f.dx_u[c] * 0.5;
  vis = p.visc * vis;
  double cor = 0.5 * (2. * p.omega * f.sin_u[c] * (v_sc + v_nc)) * f.area_u[c] *
               (hu[c] + su[c]);
  double hpg = -p.g * (hu[c] + su[c]) * f.dy_u[c] * (sn[e] - sn[c]);
  f.ua[c] = (un[c] * (hu[c] + su[c]) + p.rdt * (adv + vis + cor + hpg) / f.area_u[c]) /
            (hu[c] + f.ssha_u[c]) / (1.0 + p.cbfr * p.rdt);
}

// K3: momentum_v_code, kernels/c_family/momentum_v_kern.c:125-241, metric
// binding of time_step.cpp:70-77 (e1v=dx_v, e1t=dx_t, e2u=dy_u, e2v=dy_v,
// e2t=dy_t, e12v=area_v).  Its first guard reads the east mask (:155).
__global__ void __launch_bounds__(BX* BY)
    k_momentum_v(Fields f, int W, Range r, Scalars p) {
  int i, j;
  if (!at(r, i, j)) return;
  const int c = j * W + i, e = c + 1, wst = c - 1, s = c - W, n = c + W,
            nw = n - 1, ne = n + 1;
  const int* m = f.tmask;
  if (m[c] + m[e] <= 0) return;
  if (m[c] <= 0 || m[n] <= 0) return;
  const double *un = f.un, *vn = f.vn, *hu = f.hu, *hv = f.hv, *ht = f.ht,
               *sn = f.sshn_t, *su = f.sshn_u, *sv = f.sshn_v;

  double v_n = 0.5 * (vn[c] + vn[n]) * f.dx_t[n];
  double depn = ht[n] + sn[n];
  double v_s = 0.5 * (vn[c] + vn[s]) * f.dx_t[c];
  double deps = ht[c] + sn[c];
  double u_wc = 0.5 * (un[wst] + un[nw]);
  double u_w = 0.5 * u_wc * (f.dy_u[wst] + f.dy_u[nw]);
  double depw = 0.50 * (hu[wst] + su[wst] + hu[nw] + su[nw]);
  double u_ec = 0.5 * (un[c] + un[n]);
  double u_e = 0.5 * u_ec * (f.dy_u[c] + f.dy_u[n]);
  double depe = 0.50 * (hu[c] + su[c] + hu[n] + su[n]);

  double vv_s = wlo(v_s) * vn[c] + whi(v_s) * vn[s];
  double vv_n = whi(v_n) * vn[c] + wlo(v_n) * vn[n];
  const bool west_dry = m[wst] <= 0 || m[nw] <= 0;
  const bool east_dry = m[e] <= 0 || m[ne] <= 0;
  double vv_w = west_dry ? wlo(u_w) * vn[c] : wlo(u_w) * vn[c] + whi(u_w) * vn[wst];
  double vv_e = east_dry ? whi(u_e) * vn[c] : whi(u_e) * vn[c] + wlo(u_e) * vn[e];
  double adv = vv_w * u_w * depw - vv_e * u_e * depe + vv_s * v_s * deps -
               vv_n * v_n * depn;

  double dvdy_n = (vn[n] - vn[c]) / f.dy_t[n] * (ht[n] + sn[n]);
  double dvdy_s = (vn[c] - vn[s]) / f.dy_t[c] * (ht[c] + sn[c]);
  double dvdx_w = west_dry ? 0.0
                           : (vn[c] - vn[wst]) / (f.dx_v[c] + f.dx_v[wst]) *
                                 (hv[c] + sv[c] + hv[wst] + sv[wst]);
  double dvdx_e = east_dry ? 0.0
                           : (vn[e] - vn[c]) / (f.dx_v[c] + f.dx_v[e]) *
                                 (hv[c] + sv[c] + hv[e] + sv[e]);
  double vis = (dvdy_n - dvdy_s) * f.dx_v[c] + (dvdx_e - dvdx_w) * f.dy_v[c] * 0.5;
  vis = p.visc * vis;
  double cor = -0.5 * (2. * p.omega * f.sin_v[c] * (u_ec + u_wc)) * f.area_v[c] *
               (hv[c] + sv[c]);
  double hpg = -p.g * (hv[c] + sv[c]) * f.dx_v[c] * (sn[n] - sn[c]);
  f.va[c] = (vn[c] * (hv[c] + sv[c]) + p.rdt * (adv + vis + cor + hpg) / f.area_v[c]) /
            ((hv[c] + f.ssha_v[c])) / (1.0 + p.cbfr * p.rdt);
}

// K4: bc_ssh_code, boundary_conditions_kern.c:178-203; `tide` is
// amp_tide * sin(omega_tide * istep * rdt) from the host.
__global__ void __launch_bounds__(BX* BY)
    k_bc_ssh(Fields f, int W, Range r, double tide) {
  int i, j;
  if (!at(r, i, j)) return;
  const int c = j * W + i;
  const int* m = f.tmask;
  if (m[c] <= 0) return;
  if (m[c - W] < 0 || m[c + W] < 0 || m[c + 1] < 0 || m[c - 1] < 0) f.ssha_t[c] = tide;
}

// K5, K6: bc_solid_u_code / bc_solid_v_code, boundary_conditions_kern.c:220-252.
__global__ void __launch_bounds__(BX* BY) k_bc_solid(double* vel, const int* m, int W,
                                                      Range r, int step) {
  int i, j;
  if (!at(r, i, j)) return;
  const int c = j * W + i;
  if (m[c] * m[c + step] == 0) vel[c] = 0.0;
}

// K7, K8: bc_flather_{u,v}_code, boundary_conditions_kern.c:271-333.  The
// parallel form is exact when no Flather face reads another Flather face
// (checked on the host from the mask); otherwise k_bc_flather_ordered walks
// each line in the reference loop order.
__device__ __forceinline__ void flather_at(double* vel, const double* h, const double* sf,
                                           const int* m, double g, int c, int step) {
  if (m[c] + m[c + step] <= -1) return;
  if (m[c] < 0)
    vel[c] = vel[c + step] + sqrt(g / h[c]) * (sf[c] - sf[c + step]);
  else if (m[c + step] < 0)
    vel[c] = vel[c - step] + sqrt(g / h[c]) * (sf[c] - sf[c - step]);
}

__global__ void __launch_bounds__(BX* BY)
    k_bc_flather(double* vel, const double* h, const double* sf, const int* m, double g,
                 int W, Range r, int step) {
  int i, j;
  if (!at(r, i, j)) return;
  flather_at(vel, h, sf, m, g, j * W + i, step);
}

// One thread per line: rows for u (the reference's inner loop runs along
// x), columns for v (its outer loop runs along y and carries the
// dependency, time_step_omp.cpp:116-119).
__global__ void k_bc_flather_ordered(double* vel, const double* h, const double* sf,
                                     const int* m, double g, int W, Range r, int step) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (step == 1) {
    const int j = r.y0 + t;
    if (j > r.y1) return;
    for (int i = r.x0; i <= r.x1; i++) flather_at(vel, h, sf, m, g, j * W + i, 1);
  } else {
    const int i = r.x0 + t;
    if (i > r.x1) return;
    for (int j = r.y0; j <= r.y1; j++) flather_at(vel, h, sf, m, g, j * W + i, step);
  }
}

// K9: the field copies of time_step.cpp:114-122 (rows ys-1 .. ye).
__global__ void __launch_bounds__(BX* BY) k_copy3(Fields f, int W, Range r) {
  int i, j;
  if (!at(r, i, j)) return;
  const int c = j * W + i;
  f.un[c] = f.ua[c];
  f.vn[c] = f.va[c];
  f.sshn_t[c] = f.ssha_t[c];
}

__global__ void __launch_bounds__(BX* BY)
    k_copy1(const double* __restrict__ src, double* __restrict__ dst, int W, Range r) {
  int i, j;
  if (!at(r, i, j)) return;
  dst[j * W + i] = src[j * W + i];
}

// K10, K11: next_sshu_code / next_sshv_code, time_update_kern.c:90-155.
__global__ void __launch_bounds__(BX* BY)
    k_next_ssh(double* sf, const double* sn, const int* m, const double* e12t,
               const double* e12f, int W, Range r, int step) {
  int i, j;
  if (!at(r, i, j)) return;
  const int c = j * W + i, n = c + step;
  if (m[c] + m[n] <= 0) return;
  if (m[c] * m[n] > 0) {
    double rtmp1 = e12t[c] * sn[c] + e12t[n] * sn[n];
    sf[c] = 0.5 * rtmp1 / e12f[c];
  } else if (m[c] <= 0) {
    sf[c] = sn[n];
  } else if (m[n] <= 0) {
    sf[c] = sn[c];
  }
}

}  // namespace

double tide_value(int istep, double rdt) {
  const double amp_tide = 0.2;
  const double omega_tide = 2.0 * 3.14159 / (12.42 * 3600.0);
  const double rtime = istep * rdt;
  return amp_tide * std::sin(omega_tide * rtime);
}

void launch_reference_step(const Fields& f, const Dims& d, const Scalars& s, int istep,
                           bool chain_u, bool chain_v, cudaStream_t st) {
  const int W = d.width, xs = d.xs, xe = d.xe, ys = d.ys, ye = d.ye;
  const dim3 blk(BX, BY);
  const Range interior{xs, xe, ys, ye};
  const Range u_int{xs, xe - 1, ys, ye};
  const Range v_int{xs, xe, ys, ye - 1};
  const Range u_whole{xs - 1, xe, ys - 1, ye + 1};
  const Range v_whole{xs - 1, xe + 1, ys - 1, ye};
  const Range copy{xs - 1, xe + 1, ys - 1, ye};

  k_continuity<<<grid_for(interior), blk, 0, st>>>(f, W, interior, s.rdt);
  k_momentum_u<<<grid_for(u_int), blk, 0, st>>>(f, W, u_int, s);
  k_momentum_v<<<grid_for(v_int), blk, 0, st>>>(f, W, v_int, s);
  k_bc_ssh<<<grid_for(interior), blk, 0, st>>>(f, W, interior, tide_value(istep, s.rdt));
  k_bc_solid<<<grid_for(u_whole), blk, 0, st>>>(f.ua, f.tmask, W, u_whole, 1);
  k_bc_solid<<<grid_for(v_whole), blk, 0, st>>>(f.va, f.tmask, W, v_whole, W);
  if (!chain_u) {
    k_bc_flather<<<grid_for(u_whole), blk, 0, st>>>(f.ua, f.hu, f.sshn_u, f.tmask, s.g, W,
                                                    u_whole, 1);
  } else {
    const int lines = u_whole.y1 - u_whole.y0 + 1;
    k_bc_flather_ordered<<<(lines + 127) / 128, 128, 0, st>>>(f.ua, f.hu, f.sshn_u, f.tmask,
                                                              s.g, W, u_whole, 1);
  }
  if (!chain_v) {
    k_bc_flather<<<grid_for(v_whole), blk, 0, st>>>(f.va, f.hv, f.sshn_v, f.tmask, s.g, W,
                                                    v_whole, W);
  } else {
    const int lines = v_whole.x1 - v_whole.x0 + 1;
    k_bc_flather_ordered<<<(lines + 127) / 128, 128, 0, st>>>(f.va, f.hv, f.sshn_v, f.tmask,
                                                              s.g, W, v_whole, W);
  }
  k_copy3<<<grid_for(copy), blk, 0, st>>>(f, W, copy);
  launch_next_ssh(f, d, st);
}

void launch_next_ssh(const Fields& f, const Dims& d, cudaStream_t st) {
  const int W = d.width;
  const dim3 blk(BX, BY);
  const Range u_int{d.xs, d.xe - 1, d.ys, d.ye};
  const Range v_int{d.xs, d.xe, d.ys, d.ye - 1};
  k_next_ssh<<<grid_for(u_int), blk, 0, st>>>(f.sshn_u, f.sshn_t, f.tmask, f.area_t,
                                              f.area_u, W, u_int, 1);
  k_next_ssh<<<grid_for(v_int), blk, 0, st>>>(f.sshn_v, f.sshn_t, f.tmask, f.area_t,
                                              f.area_v, W, v_int, W);
}

void launch_copy_region(const double* src, double* dst, const Dims& d, cudaStream_t st) {
  const Range copy{d.xs - 1, d.xe + 1, d.ys - 1, d.ye};
  k_copy1<<<grid_for(copy), dim3(BX, BY), 0, st>>>(src, dst, d.width, copy);
}

}  // namespace nl2d
