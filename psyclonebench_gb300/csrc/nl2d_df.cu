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
// copy region (the exact cells) is computed in exact FP64 by the fused
// step's general per-cell code reading global memory (general_cell with a
// GlobalCtx, nl2d_fused_tile.cuh), one thread each, by blocks of the same
// launch spread evenly among the march's blocks.
//
// Loads split each FP64 state value into a pair from its bit pattern
// (split_bits; the depths and the reciprocal momentum denominators are split
// once at set-up); stores widen both halves from their bit patterns and add
// them in FP64 (join_bits): one FP64 instruction per stored value, none per
// loaded one.
#include "nl2d_df_march.cuh"
#include "nl2d_fused_tile.cuh"

namespace nl2d {
using namespace dfk;
namespace {

using namespace dfm;
constexpr int MR = 32;

// One step.  Of the grid's blocks, nring take the exact cells (128 each,
// one per thread; block b is one when floor((b+1) nring / grid) >
// floor(b nring / grid)), so that they spread evenly among the march's
// blocks and share the SMs with them: the march issues on the FP32 and
// integer pipes, the exact cells wait on the FP64 pipe.  The others march
// strips of mr rows over ncol column groups.  Both read the state buffers
// of fs and write disjoint cells.
__global__ void __launch_bounds__(32 * WARPS, 3)
    k_df_step(const __grid_constant__ FusedState fs, const __grid_constant__ DfFields ff,
              const __grid_constant__ Dims d, const __grid_constant__ DfConst k, int ncol,
              int nwarps, int mr, const __grid_constant__ Fields f,
              const __grid_constant__ Scalars p, const __grid_constant__ FastConst fk,
              const double* __restrict__ tide_table, int tide_index, double tide, int nring) {
  const long long grid = gridDim.x, b = blockIdx.x;
  const int q0 = (int)(b * nring / grid), q1 = (int)((b + 1) * nring / grid);
  if (q1 > q0) {  // exact-cell block q0
    const int g = q0 * (32 * WARPS) + (int)threadIdx.x;
    if (g < ff.n_ring) {
      const int c = ff.ring[g];
      const int j = c / d.width, i = c - j * d.width;
      const GlobalCtx x{fs.sshn_in, fs.un_in,    fs.vn_in, f.hu,      f.hv,
                        f.ht,       f.ssha_u,    f.ssha_v, f.r_hu,    f.r_hv,
                        f.tmask,    f.sshn_u,    f.sshn_v, d.width,   d,
                        fk};
      general_cell(x, f, fs, p, tide_table ? tide_table[tide_index] : tide, i, j);
    }
    return;
  }
  // march block b - q0: q0 exact-cell blocks precede it
  const int warp = (int)(b - q0) * WARPS + (int)(threadIdx.x >> 5);
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

// The exact cells: every copy-region cell the march does not write, listed
// in `ring` (cell indices, in no particular order) and counted in *count;
// ring == nullptr counts only.
__global__ void k_df_ring(const unsigned char* __restrict__ reg, Dims d, int* __restrict__ ring,
                          int* __restrict__ count) {
  const int nx = d.xe - d.xs + 3;
  const long long n = (long long)nx * (d.ye - d.ys + 2);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int j = d.ys - 1 + (int)(t / nx), i = d.xs - 1 + (int)(t % nx);
    const int c = j * d.width + i;
    if (!reg[c]) {
      const int k = atomicAdd(count, 1);
      if (ring) ring[k] = c;
    }
  }
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
}

void launch_df_ring(const Dims& d, const DfFields& ff, cudaStream_t st) {
  cudaMemsetAsync(ff.count, 0, sizeof(int), st);
  k_df_ring<<<152 * 8, 256, 0, st>>>(ff.reg, d, ff.ring, ff.count);
}

void launch_df_step(const Fields& f, const FusedState& fs, const Dims& d, const Scalars& s,
                    const UniformMetrics& um, const DfFields& ff, double tide,
                    const double* tide_table, int tide_index, cudaStream_t st) {
  const int nx = d.xe - d.xs + 3, ny = d.ye - d.ys + 2;
  const int ncol = (nx + MW - 1) / MW;
  // strips of MR rows, halved (down to 8) until the grid holds about two
  // waves of warps
  int mr = MR;
  while (mr > 8 && (long long)ncol * ((ny + mr - 1) / mr) < 2 * 152 * 2 * WARPS) mr /= 2;
  const int nrow = (ny + mr - 1) / mr, nwarps = ncol * nrow;
  const int nring = (ff.n_ring + 32 * WARPS - 1) / (32 * WARPS);
  k_df_step<<<(nwarps + WARPS - 1) / WARPS + nring, 32 * WARPS, 0, st>>>(
      fs, ff, d, make_df_const(s, um), ncol, nwarps, mr, f, s, make_fast_const(s, um),
      tide_table, tide_index, tide, nring);
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
