// Mixed-precision NEMOLite2D step: one sm_103a kernel per step.
//
// Velocities, fluxes and the momentum arithmetic are FP32; the sea-surface
// height — a small perturbation accumulated over thousands of steps on top
// of the depth — is carried as an unevaluated pair of floats (hi + lo,
// about 48 significant bits) and updated with an error-free two-sum
// (Knuth's TwoSum, then Dekker's Fast2Sum renormalisation), i.e.
// Kahan-compensated FP32.  No FP64 instruction runs per cell: on GB300 the
// FP64 pipe is ~70x slower than FP32, so this form is bound by HBM.
//
// State in HBM per cell: ssh (hi, lo) 8 B, un 4 B, vn 4 B (ping-pong), and
// the static ht, hu, hv (FP32) and tmask (int32).  Algorithmic traffic:
// read 8 + 4 + 4 + 3 x 4 + 4 = 32 B, write 16 B: 48 B per cell-step.  The
// momentum denominators 1 / (hu + ssha_u), 1 / (hv + ssha_v) are static
// FP32 arrays (8 B more per cell read).
//
// The operations follow the reference kernels (continuity_kern.c,
// momentum_{u,v}_kern.c, boundary_conditions_kern.c, time_update_kern.c)
// in the same order, in FP32, with divisions by step constants replaced by
// multiplications with their FP32 reciprocals; FMA contraction is allowed.
// The same preconditions as the FP64 fused step apply (uniform metrics, no
// chained Flather faces).
#include <cstring>

#include "nl2d_mixed_march.cuh"

namespace nl2d {
using namespace mixk;
namespace {

// The regular cells: one warp per MW columns x MR rows of the copy region.
// Both march kernels are held to 96 registers, 5 blocks of 4 warps per SM.
__global__ void __launch_bounds__(32 * MARCH_WARPS, 5)
    k_mixed_march(MixedFields mf, MixedState ms, Dims d, MarchConst k, int ncol, int nwarps,
                  int mr) {
  const int warp = blockIdx.x * MARCH_WARPS + (int)(threadIdx.x >> 5);
  if (warp >= nwarps) return;  // the whole warp leaves together
  const int gy = warp / ncol, gx = warp - gy * ncol;
  mixed_march(mf, ms, d, k, d.xs - 1 + gx * MW, d.ys - 1 + gy * mr, 0, mr);
}

// The copy region's other cells, one thread per listed cell.
__global__ void __launch_bounds__(128)
    k_mixed_general(MixedFields mf, MixedState ms, Fields f, Dims d, MixConst k,
                    const double* __restrict__ tide_table, int tide_index, double tide) {
  const double td = tide_table ? tide_table[tide_index] : tide;
  __shared__ EnsDom sd;  // the kernel's arguments as one descriptor in memory
  if (threadIdx.x == 0) {
    sd.mf = mf;
    sd.ms[0] = ms;
    sd.f = f;
    sd.d = d;
    sd.k = k;
    sd.off = 0;
  }
  __syncthreads();
  const GCtx x{sd.mf, sd.ms[0], sd.f, sd.d, sd.k};
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < mf.gcount;
       t += gridDim.x * blockDim.x) {
    const int c = mf.glist[t];
    const int j = c / d.width;
    general_cell(x, c - j * d.width, j, td);
  }
}

// ---- ensemble: the march over every domain; warp w takes units[w] =
// (domain, i0, j0) with the packed arrays' base pointers in mf / ms.  The
// step's constants are the kernel parameter k when every domain shares them;
// with EACH, each warp copies its domain's (mks[domain]) into its
// shared-memory slot first.
template <bool EACH>
__global__ void __launch_bounds__(32 * MARCH_WARPS, 5)
    k_ensemble_mixed_march(const EnsDom* __restrict__ doms, const int4* __restrict__ units,
                           int nunits, MixedFields mf, MixedState ms, MarchConst k,
                           const MarchConst* __restrict__ mks, int mr) {
  const int wib = (int)(threadIdx.x >> 5);
  const int w = blockIdx.x * MARCH_WARPS + wib;
  if (w >= nunits) return;  // the whole warp leaves together
  const int4 u = units[w];
  const Dims d = doms[u.x].d;
  if constexpr (EACH) {
    __shared__ MarchConst sk[MARCH_WARPS];
    constexpr int kWords = sizeof(MarchConst) / sizeof(float);
    const float* src = reinterpret_cast<const float*>(mks + u.x);
    float* dst = reinterpret_cast<float*>(sk + wib);
    for (int q = (int)(threadIdx.x & 31); q < kWords; q += 32) dst[q] = src[q];
    __syncwarp();
    mixed_march(mf, ms, d, sk[wib], u.y, u.z, doms[u.x].off, mr);
  } else {
    mixed_march(mf, ms, d, k, u.y, u.z, doms[u.x].off, mr);
  }
}

// The other cells of every domain's copy region: glist[t] = (domain, cell).
__global__ void __launch_bounds__(128)
    k_ensemble_mixed_general(const EnsDom* __restrict__ doms, const int2* __restrict__ glist,
                             int n, int parity, const double* __restrict__ tides) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int2 g = glist[t];
    const EnsDom& D = doms[g.x];
    const GCtx x{D.mf, D.ms[parity], D.f, D.d, D.k};
    const int j = g.y / D.d.width;
    general_cell(x, g.y - j * D.d.width, j, tides[g.x]);
  }
}

// March flags of domain `dom` and, when glist is not null, its general
// cells appended as (dom, cell); *count counts them either way.
__global__ void k_ensemble_mixed_flags(const EnsDom* __restrict__ doms, int dom,
                                       unsigned char* __restrict__ reg, int2* __restrict__ glist,
                                       int* __restrict__ count) {
  const EnsDom& D = doms[dom];
  const long long n = (long long)D.d.width * D.d.height;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t / D.d.width), i = (int)(t - (long long)j * D.d.width);
    const bool r = march_regular(D.f, D.d, i, j);
    reg[D.off + t] = r ? 1 : 0;
    if (!r && i >= D.d.xs - 1 && i <= D.d.xe + 1 && j >= D.d.ys - 1 && j <= D.d.ye) {
      const int slot = atomicAdd(count, 1);
      if (glist) glist[slot] = make_int2(dom, (int)t);
    }
  }
}

// march flags over the whole array; the copy region's other cells listed
__global__ void k_mixed_flags(Fields f, Dims d, unsigned char* __restrict__ reg,
                              int* __restrict__ glist, int* __restrict__ count) {
  const long long n = (long long)d.width * d.height;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t / d.width), i = (int)(t - (long long)j * d.width);
    const bool r = march_regular(f, d, i, j);
    reg[t] = r ? 1 : 0;
    if (!r && i >= d.xs - 1 && i <= d.xe + 1 && j >= d.ys - 1 && j <= d.ye)
      glist[atomicAdd(count, 1)] = (int)t;
  }
}

__global__ void k_to_mixed(const double* __restrict__ sn, const double* __restrict__ un,
                           const double* __restrict__ vn, const double* __restrict__ ht,
                           const double* __restrict__ hu, const double* __restrict__ hv,
                           const double* __restrict__ ssha_u,
                           const double* __restrict__ ssha_v, float2* __restrict__ sn2,
                           float* __restrict__ un_f, float* __restrict__ vn_f,
                           float* __restrict__ ht_f, float* __restrict__ hu_f,
                           float* __restrict__ hv_f, float* __restrict__ rhu,
                           float* __restrict__ rhv, long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const float hi = (float)sn[t];
    sn2[t] = make_float2(hi, (float)(sn[t] - (double)hi));
    un_f[t] = (float)un[t];
    vn_f[t] = (float)vn[t];
    if (ht_f) {
      ht_f[t] = (float)ht[t];
      hu_f[t] = (float)hu[t];
      hv_f[t] = (float)hv[t];
      rhu[t] = (float)(1.0 / (hu[t] + ssha_u[t]));
      rhv[t] = (float)(1.0 / (hv[t] + ssha_v[t]));
    }
  }
}

__global__ void k_from_mixed(const float2* __restrict__ sn2, const float* __restrict__ un_f,
                             const float* __restrict__ vn_f, double* __restrict__ sn,
                             double* __restrict__ un, double* __restrict__ vn, long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    sn[t] = (double)sn2[t].x + (double)sn2[t].y;
    un[t] = (double)un_f[t];
    vn[t] = (double)vn_f[t];
  }
}

}  // namespace

void launch_mixed_step(const MixedFields& mf, const MixedState& ms, const Fields& f,
                       const Dims& d, const Scalars& s, const UniformMetrics& um, double tide,
                       const double* tide_table, int tide_index, cudaStream_t st,
                       cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
  const MixConst k = make_mix_const(s, um);
  const int nx = d.xe - d.xs + 3, ny = d.ye - d.ys + 2;
  // Strips of MR rows, halved (down to 8) until the grid holds about two
  // waves of warps: a smaller domain trades halo rows for parallelism.
  const int ncol = (nx + MW - 1) / MW;
  int mr = MR;
  while (mr > 8 && (long long)ncol * ((ny + mr - 1) / mr) < 2 * 152 * 5 * MARCH_WARPS) mr /= 2;
  const int nrow = (ny + mr - 1) / mr, nwarps = ncol * nrow;
  // The general cells (a list of a few thousand, each a long chain of
  // global loads) and the march read the same buffers and write disjoint
  // cells: with a side stream the general pass starts first there and runs
  // beside the march's waves instead of after them.
  const bool beside = side && fork && join && mf.gcount > 0;
  if (beside) {
    cudaEventRecord(fork, st);
    cudaStreamWaitEvent(side, fork, 0);
    k_mixed_general<<<(mf.gcount + 127) / 128, 128, 0, side>>>(mf, ms, f, d, k, tide_table,
                                                               tide_index, tide);
  }
  k_mixed_march<<<(nwarps + MARCH_WARPS - 1) / MARCH_WARPS, 32 * MARCH_WARPS, 0, st>>>(
      mf, ms, d, make_march_const(k), ncol, nwarps, mr);
  if (beside) {
    cudaEventRecord(join, side);
    cudaStreamWaitEvent(st, join, 0);
  } else if (mf.gcount > 0) {
    k_mixed_general<<<(mf.gcount + 127) / 128, 128, 0, st>>>(mf, ms, f, d, k, tide_table,
                                                             tide_index, tide);
  }
}

void launch_ens_mixed_march(const void* doms, const int4* units, int nunits,
                            const MixedFields& mf, const MixedState& ms, const void* k,
                            const void* mks, int march_rows, cudaStream_t st) {
  const int grid = (nunits + MARCH_WARPS - 1) / MARCH_WARPS;
  if (mks) {
    k_ensemble_mixed_march<true><<<grid, 32 * MARCH_WARPS, 0, st>>>(
        (const EnsDom*)doms, units, nunits, mf, ms, MarchConst{}, (const MarchConst*)mks,
        march_rows);
    return;
  }
  MixConst kc;
  memcpy(&kc, k, sizeof kc);
  k_ensemble_mixed_march<false><<<grid, 32 * MARCH_WARPS, 0, st>>>(
      (const EnsDom*)doms, units, nunits, mf, ms, make_march_const(kc), nullptr, march_rows);
}


void launch_ens_mixed_general(const void* doms, const int2* glist, int n, int parity,
                              const double* tides, cudaStream_t st) {
  if (n > 0)
    k_ensemble_mixed_general<<<(n + 127) / 128, 128, 0, st>>>((const EnsDom*)doms, glist, n,
                                                               parity, tides);
}

void launch_ens_mixed_flags(const void* doms, int dom, unsigned char* reg, int2* glist,
                            int* count, cudaStream_t st) {
  k_ensemble_mixed_flags<<<64, 256, 0, st>>>((const EnsDom*)doms, dom, reg, glist, count);
}

int launch_mixed_flags(const Fields& f, const Dims& d, const MixedFields& mf, int* count,
                       cudaStream_t st) {
  if (cudaMemsetAsync(count, 0, sizeof(int), st) != cudaSuccess) return -1;
  k_mixed_flags<<<152 * 8, 256, 0, st>>>(f, d, mf.reg, mf.glist, count);
  int h = 0;
  if (cudaMemcpyAsync(&h, count, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return -1;
  return h;
}

void launch_to_mixed(const double* sn, const double* un, const double* vn, const Fields& f,
                     const MixedFields& mf, const MixedState& ms, const Dims& d, bool statics,
                     cudaStream_t st) {
  const long long n = (long long)d.width * d.height;
  k_to_mixed<<<152 * 8, 256, 0, st>>>(sn, un, vn, f.ht, f.hu, f.hv, f.ssha_u, f.ssha_v,
                                      ms.sn_out, ms.un_out, ms.vn_out,
                                      statics ? mf.ht : nullptr, mf.hu, mf.hv, mf.rhu, mf.rhv,
                                      n);
}

void launch_from_mixed(const float2* sn2, const float* un_f, const float* vn_f, double* sn,
                       double* un, double* vn, const Dims& d, cudaStream_t st) {
  const long long n = (long long)d.width * d.height;
  k_from_mixed<<<152 * 8, 256, 0, st>>>(sn2, un_f, vn_f, sn, un, vn, n);
}

}  // namespace nl2d
