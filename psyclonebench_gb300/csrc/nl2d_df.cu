// The step's interior cells in double-float arithmetic (nl2d_df.cuh): the
// FP64-equivalent form.  Not bit-identical to the reference; held to the
// contract the reference's own comparisons use, relative L2 <= 1e-10 per
// field and checksums to 10 significant digits after 2000 steps.
//
// The state stays FP64 in HBM, in the fused path's ping-pong buffers.  One
// warp marches down a strip of rows over MW = 30 columns (one per lane,
// plus a halo lane on each side), exactly as the mixed-precision column
// march does (nl2d_mixed_march.cuh): rows j-1, j, j+1 of its column in
// registers, x neighbours by shuffles, every term two neighbouring updates
// share formed once; but every value is a double-float pair.  It writes the
// same cells the mixed march writes: interior cells whose 3x3 mask
// neighbourhood is wet and that lie one cell inside next_ssh's ranges, so
// every face they read takes next_ssh's two-sided formula and no momentum
// mask, bc_ssh, solid-wall or Flather rule applies.  Every other cell of the
// copy region is computed in exact FP64 by the fused tile kernel, launched
// on the tiles that hold such cells (nl2d_fused.cu).
//
// Loads split each FP64 state value into a pair from its bit pattern
// (split_bits; the depths and the reciprocal momentum denominators are split
// once at set-up); stores widen both halves from their bit patterns and add
// them in FP64 (join_bits): one FP64 instruction per stored value, none per
// loaded one.
#include "nl2d_df.cuh"
#include "nl2d_internal.h"

namespace nl2d {
using namespace dfk;
namespace {

constexpr int MW = kDfMarchCols;
constexpr int MR = 32;
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

__global__ void __launch_bounds__(32 * WARPS, 3)
    k_df_march(FusedState fs, DfFields ff, Dims d, DfConst k, int ncol, int nwarps, int mr) {
  const int warp = blockIdx.x * WARPS + (int)(threadIdx.x >> 5);
  if (warp >= nwarps) return;  // the whole warp leaves together
  const int gy = warp / ncol, gx = warp - gy * ncol;
  df_march(fs, ff, d, k, d.xs - 1 + gx * MW, d.ys - 1 + gy * mr, mr);
}

// The ensemble form: warp w takes units[w] = (domain, i0, j0) with the
// domain's buffers in doms[domain] (every domain shares the constants k).
__global__ void __launch_bounds__(32 * WARPS, 3)
    k_ensemble_df_march(const EnsDfDomain* __restrict__ doms, const int4* __restrict__ units,
                        int nunits, int parity, DfConst k, int mr) {
  const int w = blockIdx.x * WARPS + (int)(threadIdx.x >> 5);
  if (w >= nunits) return;  // the whole warp leaves together
  const int4 u = units[w];
  const EnsDfDomain& D = doms[u.x];
  df_march(D.fs[parity], D.ff, D.d, k, u.y, u.z, mr);
}

// FP64 arrays split into pairs once per set-up.
__global__ void k_split(const double* __restrict__ a, float2* __restrict__ out, long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const df p = from_double(a[t]);
    out[t] = make_float2(p.hi, p.lo);
  }
}

// Whether the march writes cell (i, j): the mixed march's rule.
__device__ __forceinline__ bool df_regular(const int* m, const Dims& d, int i, int j) {
  if (i < d.xs + 1 || i > d.xe - 1 || j < d.ys + 1 || j > d.ye - 1) return false;
  const int W = d.width;
#pragma unroll
  for (int dj = -1; dj <= 1; dj++)
#pragma unroll
    for (int di = -1; di <= 1; di++)
      if (m[(j + dj) * W + (i + di)] <= 0) return false;
  return true;
}

__global__ void k_df_flags(const int* __restrict__ m, Dims d, unsigned char* __restrict__ reg) {
  const long long n = (long long)d.width * d.height;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t / d.width), i = (int)(t - (long long)j * d.width);
    reg[t] = df_regular(m, d, i, j) ? 1 : 0;
  }
}

// Appends to `list` every tile of a tx x ty grid over the copy region
// (row-major, ntx tiles per row) that holds a cell of its kind the march
// does not write: side 1 the side strips (columns xs-1, xs, xe, xe+1 of
// rows ys+1 .. ye-1), side 0 every other such cell.  The two kinds cover
// every copy-region cell the march leaves; the order of the list does not
// matter (each tile writes its own cells).
__device__ __forceinline__ bool tile_has_work(const unsigned char* __restrict__ reg,
                                              const Dims& d, int tx, int ty, int i0, int j0,
                                              int side) {
  int any = 0;
  for (int t = threadIdx.x; t < tx * ty; t += blockDim.x) {
    const int i = i0 + t % tx, j = j0 + t / tx;
    if (i > d.xe + 1 || j > d.ye || reg[(size_t)j * d.width + i]) continue;
    const bool strip = (i <= d.xs || i >= d.xe) && j >= d.ys + 1 && j <= d.ye - 1;
    if (strip == (side == 1)) any = 1;
  }
  return __syncthreads_or(any) != 0;
}

__global__ void k_df_tiles(const unsigned char* __restrict__ reg, Dims d, int tx, int ty,
                           int ntx, int side, int* __restrict__ list, int* __restrict__ count) {
  const int b = blockIdx.x;
  const int i0 = d.xs - 1 + (b % ntx) * tx, j0 = d.ys - 1 + (b / ntx) * ty;
  if (tile_has_work(reg, d, tx, ty, i0, j0, side) && threadIdx.x == 0)
    list[atomicAdd(count + side, 1)] = b;
}

__global__ void k_selftest_df(const double* __restrict__ x, long long n, float* __restrict__ hi,
                              float* __restrict__ lo, double* __restrict__ joined,
                              double* __restrict__ widened) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const df p = split_bits(x[t]);
    hi[t] = p.hi;
    lo[t] = p.lo;
    joined[t] = join_bits(p);
    widened[t] = widen_bits(__double2float_rn(x[t]));
  }
}

}  // namespace

DfConst make_df_const(const Scalars& s, const UniformMetrics& um) {
  const double dxv2 = um.dx_v + um.dx_v, dyu2 = um.dy_u + um.dy_u;
  const double cor_u = 2. * s.omega * um.sin_u, cor_v = 2. * s.omega * um.sin_v;
  DfConst k;
  k.r_dx = from_double(1.0 / um.dx_t);
  k.r_dy = from_double(1.0 / um.dy_t);
  k.uu_x = from_double(0.5 * um.dy_t);
  k.uu_y = from_double(0.125 * dyu2);
  k.vv_x = from_double(0.125 * dxv2);
  k.vv_y = from_double(0.5 * um.dx_t);
  k.r_qu = from_double(1.0 / dyu2);
  k.r_qv = from_double(1.0 / dxv2);
  k.vis1_u = from_double(s.visc * um.dy_u);
  k.vis1_v = from_double(s.visc * um.dx_v);
  k.vis2_u = from_double(0.5 * s.visc * um.dx_u);
  k.vis2_v = from_double(0.5 * s.visc * um.dy_v);
  k.cor_u = from_double(0.25 * cor_u * um.area_u);
  k.cor_v = from_double(-0.25 * cor_v * um.area_v);
  k.hpg_u = from_double(-s.g * um.dy_u);
  k.hpg_v = from_double(-s.g * um.dx_v);
  k.rra_u = from_double(s.rdt / um.area_u);
  k.rra_v = from_double(s.rdt / um.area_v);
  k.face_u = from_double(0.5 * um.area_t / um.area_u);
  k.face_v = from_double(0.5 * um.area_t / um.area_v);
  k.rrat = from_double(s.rdt / um.area_t);
  k.r_fric = from_double(1.0 / (1.0 + s.cbfr * s.rdt));
  return k;
}

void launch_df_setup(const Fields& f, const Dims& d, const DfFields& ff, cudaStream_t st) {
  const long long n = (long long)d.width * d.height;
  k_split<<<152 * 8, 256, 0, st>>>(f.ht, ff.ht, n);
  k_split<<<152 * 8, 256, 0, st>>>(f.hu, ff.hu, n);
  k_split<<<152 * 8, 256, 0, st>>>(f.hv, ff.hv, n);
  k_split<<<152 * 8, 256, 0, st>>>(f.r_hu, ff.rhu, n);
  k_split<<<152 * 8, 256, 0, st>>>(f.r_hv, ff.rhv, n);
  k_df_flags<<<152 * 8, 256, 0, st>>>(f.tmask, d, ff.reg);
  cudaMemsetAsync(ff.count, 0, 2 * sizeof(int), st);
  const int nx = d.xe - d.xs + 3, ny = d.ye - d.ys + 2;
  const int rx = (nx + kDfRowsTX - 1) / kDfRowsTX, ry = (ny + kDfRowsTY - 1) / kDfRowsTY;
  const int cx = (nx + kDfColsTX - 1) / kDfColsTX, cy = (ny + kDfColsTY - 1) / kDfColsTY;
  k_df_tiles<<<rx * ry, 256, 0, st>>>(ff.reg, d, kDfRowsTX, kDfRowsTY, rx, 0, ff.tiles_rows,
                                      ff.count);
  k_df_tiles<<<cx * cy, 256, 0, st>>>(ff.reg, d, kDfColsTX, kDfColsTY, cx, 1, ff.tiles_cols,
                                      ff.count);
}

void launch_df_march(const FusedState& fs, const DfFields& ff, const Dims& d, const DfConst& k,
                     cudaStream_t st) {
  const int nx = d.xe - d.xs + 3, ny = d.ye - d.ys + 2;
  const int ncol = (nx + MW - 1) / MW;
  // strips of MR rows, halved (down to 8) until the grid holds about two
  // waves of warps
  int mr = MR;
  while (mr > 8 && (long long)ncol * ((ny + mr - 1) / mr) < 2 * 152 * 2 * WARPS) mr /= 2;
  const int nrow = (ny + mr - 1) / mr, nwarps = ncol * nrow;
  k_df_march<<<(nwarps + WARPS - 1) / WARPS, 32 * WARPS, 0, st>>>(fs, ff, d, k, ncol, nwarps,
                                                                  mr);
}

}  // namespace nl2d

extern "C" int nl2d_selftest_df(const double* x, long long n, float* hi, float* lo,
                                double* joined, double* widened) {
  if (!x || !hi || !lo || !joined || !widened || n <= 0 || n > (1LL << 26)) return 2;
  double *dx = nullptr, *dj = nullptr, *dw = nullptr;
  float *dh = nullptr, *dl = nullptr;
  const size_t b8 = (size_t)n * 8, b4 = (size_t)n * 4;
  bool ok = cudaMalloc(&dx, b8) == cudaSuccess && cudaMalloc(&dj, b8) == cudaSuccess &&
            cudaMalloc(&dw, b8) == cudaSuccess && cudaMalloc(&dh, b4) == cudaSuccess &&
            cudaMalloc(&dl, b4) == cudaSuccess;
  ok = ok && cudaMemcpy(dx, x, b8, cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    nl2d::k_selftest_df<<<152 * 4, 256>>>(dx, n, dh, dl, dj, dw);
    ok = cudaGetLastError() == cudaSuccess;
  }
  ok = ok && cudaMemcpy(hi, dh, b4, cudaMemcpyDeviceToHost) == cudaSuccess &&
       cudaMemcpy(lo, dl, b4, cudaMemcpyDeviceToHost) == cudaSuccess &&
       cudaMemcpy(joined, dj, b8, cudaMemcpyDeviceToHost) == cudaSuccess &&
       cudaMemcpy(widened, dw, b8, cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(dx);
  cudaFree(dj);
  cudaFree(dw);
  cudaFree(dh);
  cudaFree(dl);
  return ok ? 0 : 1;
}

namespace nl2d {

void launch_ens_df_march(const EnsDfDomain* doms, const int4* units, int nunits, int parity,
                         const DfConst& k, int march_rows, cudaStream_t st) {
  k_ensemble_df_march<<<(nunits + WARPS - 1) / WARPS, 32 * WARPS, 0, st>>>(doms, units, nunits,
                                                                           parity, k, march_rows);
}

void launch_df_split(const double* a, float2* out, long long n, cudaStream_t st) {
  k_split<<<152 * 8, 256, 0, st>>>(a, out, n);
}

void launch_df_flags(const int* tmask, const Dims& d, unsigned char* reg, cudaStream_t st) {
  k_df_flags<<<152 * 8, 256, 0, st>>>(tmask, d, reg);
}

}  // namespace nl2d
