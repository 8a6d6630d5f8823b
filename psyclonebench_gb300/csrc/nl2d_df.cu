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
#include "nl2d_df_march.cuh"

namespace nl2d {
using namespace dfk;
namespace {

using namespace dfm;
constexpr int MR = 32;

__global__ void __launch_bounds__(32 * WARPS, 3)
    k_df_march(FusedState fs, DfFields ff, Dims d, DfConst k, int ncol, int nwarps, int mr) {
  const int warp = blockIdx.x * WARPS + (int)(threadIdx.x >> 5);
  if (warp >= nwarps) return;  // the whole warp leaves together
  const int gy = warp / ncol, gx = warp - gy * ncol;
  df_march(fs, ff, d, k, d.xs - 1 + gx * MW, d.ys - 1 + gy * mr, mr);
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

void launch_df_split(const double* a, float2* out, long long n, cudaStream_t st) {
  k_split<<<152 * 8, 256, 0, st>>>(a, out, n);
}

void launch_df_flags(const int* tmask, const Dims& d, unsigned char* reg, cudaStream_t st) {
  k_df_flags<<<152 * 8, 256, 0, st>>>(tmask, d, reg);
}

}  // namespace nl2d
