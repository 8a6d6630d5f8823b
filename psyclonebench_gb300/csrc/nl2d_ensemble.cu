// Ensemble of independent NEMOLite2D domains (uneven sizes, bathymetries,
// tidal forcings and open sides) advanced by ONE persistent launch per step.
//
// Every domain keeps its own dl_esm_inf-style arrays, packed back to back
// in large device allocations.  The copy region of each domain is cut into
// TX x TY tiles; a persistent grid of (SM count x CTAs per SM) blocks walks
// a static tile schedule (contiguous cost-balanced chunks, or a
// longest-processing-time assignment) chosen by the autotuner.  Each tile
// is the fused step's tile function (nl2d_fused_tile.cuh), so a domain
// advanced here is bit-identical to the reference step with its tide
// parameters.  Steps are separate graph nodes: no grid-wide barrier inside
// a step, as tiles of a step are independent.
//
// Domains start from rest (ssh = u = v = 0), where the state is already
// step-consistent, so every step takes the fused path.
//
// Three forms share the domain layout: FP64 (the tiles above), mixed
// precision (its own FP32 / compensated state), and FP64-equivalent, which
// keeps the FP64 state and runs the double-float column march (nl2d_df.cu)
// over every domain's interior while, in the same launch, the fused step's
// general per-cell code takes every other cell in exact FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/nl2d_gpu.h"
#include "nl2d_df_march.cuh"
#include "nl2d_fused_tile.cuh"
#include "nl2d_mixed_march.cuh"

namespace nl2d {
namespace {

using EnsMixDomain = mixk::EnsDom;  // one domain of a mixed-precision ensemble

__global__ void __launch_bounds__(256)
    k_ensemble_mixed_checksums(const EnsMixDomain* __restrict__ doms, int parity,
                               double* __restrict__ out) {
  const int dom = blockIdx.x, fld = blockIdx.y;
  const EnsMixDomain& D = doms[dom];
  const MixedState& st = D.ms[parity];
  const int x0 = D.d.xs, y0 = D.d.ys;
  const int x1 = fld == 1 ? D.d.xe - 1 : D.d.xe, y1 = fld == 2 ? D.d.ye - 1 : D.d.ye;
  const int nx = x1 - x0 + 1, ny = y1 - y0 + 1;
  double acc = 0.0;
  for (int t = threadIdx.x; t < nx * ny; t += blockDim.x) {
    const int j = t / nx, i = t - j * nx;
    const size_t c = (size_t)(y0 + j) * D.d.width + (x0 + i);
    acc += fld == 0 ? fabs((double)st.sn_in[c].x + (double)st.sn_in[c].y)
                    : fabs((double)(fld == 1 ? st.un_in[c] : st.vn_in[c]));
  }
  __shared__ double wp[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) wp[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < 8 ? wp[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) out[(size_t)dom * 3 + fld] = acc;
  }
}

__global__ void k_mixed_statics(const double* __restrict__ ht, const double* __restrict__ hu,
                                const double* __restrict__ hv, float* __restrict__ fht,
                                float* __restrict__ fhu, float* __restrict__ fhv,
                                float* __restrict__ rhu, float* __restrict__ rhv, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
       t += (size_t)gridDim.x * blockDim.x) {
    fht[t] = (float)ht[t];
    fhu[t] = (float)hu[t];
    fhv[t] = (float)hv[t];
    rhu[t] = (float)(1.0 / hu[t]);  // ssha_u = ssha_v = 0 at rest
    rhv[t] = (float)(1.0 / hv[t]);
  }
}

// Ensemble: a persistent grid walks a tile list spanning many independent
// domains; CTA b takes tiles [first[b], first[b+1]).  `tides` holds this
// step's bc_ssh value per domain.
template <class T>
__global__ void __launch_bounds__(NTHREADS, T::kMinBlocks)
    k_ensemble_step(const EnsDomain* __restrict__ doms, const int4* __restrict__ tiles,
                    const int* __restrict__ first, int parity,
                    const double* __restrict__ tides) {
  extern __shared__ double smem[];
  const int t1 = first[blockIdx.x + 1];
  for (int t = first[blockIdx.x]; t < t1; t++) {
    const int4 tl = tiles[t];
    const EnsDomain& D = doms[tl.x];
    __syncthreads();  // the previous tile's last readers are done with smem
    fused_tile<T>(D.f, D.fs[parity], D.d, D.p, D.um, D.k, tides[tl.x], tl.y, tl.z, smem);
  }
}

// The FP64-equivalent form's exact part: a copy-region cell the
// double-float march does not write (the ring of boundary rows and columns,
// and cells beside land), given as (domain, cell index), by the fused step's
// general per-cell code reading the domain's arrays in global memory.  The
// result is the FP64 step's, bit for bit, with that domain's tide.
__device__ __forceinline__ void ring_cell(const EnsDomain* __restrict__ doms, int2 e, int parity,
                                          const double* __restrict__ tides) {
  const EnsDomain& D = doms[e.x];
  const FusedState& st = D.fs[parity];
  const GlobalCtx x{st.sshn_in, st.un_in,   st.vn_in, D.f.hu,    D.f.hv,    D.f.ht,
                    D.f.ssha_u, D.f.ssha_v, D.f.r_hu, D.f.r_hv,  D.f.tmask, D.f.sshn_u,
                    D.f.sshn_v, D.d.width,  D.d,      D.k};
  const int j = e.y / D.d.width, i = e.y - j * D.d.width;
  general_cell(x, D.f, st, D.p, tides[e.x], i, j);
}

// One launch per step of the FP64-equivalent form.  A block takes one of two
// roles: a march block runs four warps' (domain, i0, j0) units of the
// double-float column march (nl2d_df_march.cuh); a ring block runs 128 exact
// cells, one per thread.  The nring ring blocks are spread evenly through the
// grid (block b is one when floor((b+1) nring / grid) > floor(b nring /
// grid)), so both kinds share every SM: the march issues on the FP32 and
// integer pipes while the exact cells wait on the FP64 pipe.  Both read the
// state buffers of this parity and write disjoint cells.
//
// EACH: the domains' step constants differ; each march warp copies its
// domain's (dks[domain]) into its shared-memory slot and marches with those.
// Otherwise every domain takes the kernel parameter k.
template <bool EACH>
__global__ void __launch_bounds__(32 * dfm::WARPS, 3)
    k_ensemble_df_step(const EnsDfDomain* __restrict__ ddoms, const int4* __restrict__ units,
                       int nunits, const EnsDomain* __restrict__ doms,
                       const int2* __restrict__ cells, int ncells, int nring, int parity,
                       DfConst k, const DfConst* __restrict__ dks, int mr,
                       const double* __restrict__ tides) {
  const long long grid = gridDim.x, b = blockIdx.x;
  const int q0 = (int)(b * nring / grid), q1 = (int)((b + 1) * nring / grid);
  if (q1 > q0) {  // ring block q0
    const int g = q0 * (32 * dfm::WARPS) + (int)threadIdx.x;
    if (g < ncells) ring_cell(doms, cells[g], parity, tides);
    return;
  }
  // march block b - q0: q0 ring blocks precede it
  const int wib = (int)(threadIdx.x >> 5);
  const int w = (int)(b - q0) * dfm::WARPS + wib;
  if (w >= nunits) return;  // the whole warp leaves together
  const int4 u = units[w];
  const EnsDfDomain& D = ddoms[u.x];
  if constexpr (EACH) {
    __shared__ DfConst sk[dfm::WARPS];
    constexpr int kWords = sizeof(DfConst) / sizeof(float);
    const float* src = reinterpret_cast<const float*>(dks + u.x);
    float* dst = reinterpret_cast<float*>(sk + wib);
    for (int q = (int)(threadIdx.x & 31); q < kWords; q += 32) dst[q] = src[q];
    __syncwarp();
    dfm::df_march(D.fs[parity], D.ff, D.d, sk[wib], u.y, u.z, mr);
  } else {
    dfm::df_march(D.fs[parity], D.ff, D.d, k, u.y, u.z, mr);
  }
}

// The column marches' strip height until the autotuner chooses one (8, 16,
// 32 or 64 rows).
constexpr int kDefaultMarchRows = 32;

// The tile shapes the ensemble's FP64 kernel is built for (the autotuner's
// search space); shape 0 is the single-domain kernel's.
constexpr int kNumShapes = 5;
constexpr int kShapes[kNumShapes][2] = {{32, 16}, {32, 8}, {16, 16}, {64, 8}, {32, 32}};

template <class T>
bool set_ens_attr() {
  static bool attr = false;
  if (!attr)
    attr = cudaFuncSetAttribute(k_ensemble_step<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)T::kSmemBytes) == cudaSuccess;
  return attr;
}

// Opts the chosen shape's kernel into its dynamic shared memory (before any
// stream capture).
bool prepare_ens_step(int shape) {
  switch (shape) {
    case 1: return set_ens_attr<Tile<32, 8>>();
    case 2: return set_ens_attr<Tile<16, 16>>();
    case 3: return set_ens_attr<Tile<64, 8>>();
    case 4: return set_ens_attr<Tile<32, 32>>();
    default: return set_ens_attr<DefaultTile>();
  }
}

template <class T>
void launch_ens_step_shape(int nctas, const EnsDomain* doms, const int4* tiles, const int* first,
                           int parity, const double* tides, cudaStream_t st) {
  k_ensemble_step<T><<<nctas, dim3(T::TX, T::RPP), T::kSmemBytes, st>>>(doms, tiles, first,
                                                                         parity, tides);
}

void launch_ens_step(int shape, int nctas, const EnsDomain* doms, const int4* tiles,
                     const int* first, int parity, const double* tides, cudaStream_t st) {
  switch (shape) {
    case 1: launch_ens_step_shape<Tile<32, 8>>(nctas, doms, tiles, first, parity, tides, st); break;
    case 2: launch_ens_step_shape<Tile<16, 16>>(nctas, doms, tiles, first, parity, tides, st); break;
    case 3: launch_ens_step_shape<Tile<64, 8>>(nctas, doms, tiles, first, parity, tides, st); break;
    case 4: launch_ens_step_shape<Tile<32, 32>>(nctas, doms, tiles, first, parity, tides, st); break;
    default: launch_ens_step_shape<DefaultTile>(nctas, doms, tiles, first, parity, tides, st);
  }
}

// Per-domain checksums: block (dom, field) sums |f| over the domain's
// region for that field (T interior, u region, v region) in a fixed order.
__global__ void __launch_bounds__(256)
    k_ensemble_checksums(const EnsDomain* __restrict__ doms, int parity, int ndom,
                         double* __restrict__ out) {
  const int dom = blockIdx.x, fld = blockIdx.y;
  const EnsDomain& D = doms[dom];
  const FusedState& st = D.fs[parity];  // buffers read at this parity hold the state
  const double* f = fld == 0 ? st.sshn_in : (fld == 1 ? st.un_in : st.vn_in);
  const int x0 = D.d.xs, y0 = D.d.ys;
  const int x1 = fld == 1 ? D.d.xe - 1 : D.d.xe, y1 = fld == 2 ? D.d.ye - 1 : D.d.ye;
  const int nx = x1 - x0 + 1, ny = y1 - y0 + 1;
  double acc = 0.0;
  for (int t = threadIdx.x; t < nx * ny; t += blockDim.x) {
    const int j = t / nx, i = t - j * nx;
    acc += fabs(f[(size_t)(y0 + j) * D.d.width + (x0 + i)]);
  }
  __shared__ double wp[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) wp[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < 8 ? wp[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) out[(size_t)dom * 3 + fld] = acc;
  }
}

struct DomainHost {
  int W, H, xs, xe, ys, ye;
  double dx, dy, gphi, amp, period_h;
  size_t off;  // element offset of this domain in every packed array
  bool ready = false;
  // copy-region cells the FP64-equivalent form's march does not write
  // (row-major cell indices), from the mask
  std::vector<int> ring;
};

// The double-float march writes cell (i, j) when it lies one inside the
// interior's edge and its 3x3 mask neighbourhood is wet (df_regular in
// nl2d_df.cu); every other copy-region cell is listed here.
std::vector<int> ring_cells(const DomainHost& D, const int* m) {
  const int W = D.W;
  std::vector<int> out;
  // r[i] = wet(i-1) & wet(i) & wet(i+1) along row j
  auto row3 = [&](int j, std::vector<unsigned char>& r) {
    for (int i = 1; i < W - 1; i++)
      r[i] = m[j * W + i - 1] > 0 && m[j * W + i] > 0 && m[j * W + i + 1] > 0;
  };
  std::vector<unsigned char> a(W, 0), b(W, 0), c(W, 0);
  for (int j = D.ys - 1; j <= D.ye; j++) {
    const bool inner_row = j >= D.ys + 1 && j <= D.ye - 1;
    if (inner_row) {
      row3(j - 1, a);
      row3(j, b);
      row3(j + 1, c);
    }
    for (int i = D.xs - 1; i <= D.xe + 1; i++) {
      const bool march = inner_row && i >= D.xs + 1 && i <= D.xe - 1 && a[i] && b[i] && c[i];
      if (!march) out.push_back(j * W + i);
    }
  }
  return out;
}

struct Ens {
  int ndom = 0;
  Scalars sc{};
  std::vector<DomainHost> dom;
  size_t total = 0;  // packed elements
  double *sn[2] = {}, *un[2] = {}, *vn[2] = {};
  double *ht = nullptr, *hu = nullptr, *hv = nullptr, *zero = nullptr;
  double *r_hu = nullptr, *r_hv = nullptr;
  int* tmask = nullptr;
  EnsDomain* d_desc = nullptr;
  int4* d_tiles = nullptr;
  int* d_first = nullptr;
  int ntiles = 0, nctas = 0, ctas_per_sm = 2, policy = 0;
  double boundary_weight = 4.0;
  double* d_tides = nullptr;
  size_t tides_cap = 0;
  double* d_sums = nullptr;
  size_t sums_cap = 0;
  int parity = 0;
  cudaStream_t stream = nullptr;
  // the mixed form's general cells run on `side` (highest priority) beside
  // the march: fork / join by the two events
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_key[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  bool built = false;
  int shape = 0;        // index into kShapes: the FP64 kernel's tile
  int march_rows = kDefaultMarchRows;  // strip height of the column marches
  // mixed-precision form
  int precision = 0;
  float2* msn[2] = {};
  float *mun[2] = {}, *mvn[2] = {};
  float *mht = nullptr, *mhu = nullptr, *mhv = nullptr, *mrhu = nullptr, *mrhv = nullptr;
  EnsMixDomain* d_mdesc = nullptr;
  // the column march (built with the mixed form)
  bool march = false;
  mixk::MarchConst* d_mks = nullptr;  // per-domain march constants, or null when shared
  mixk::MixConst mk{};
  unsigned char* mreg = nullptr;
  int2* mglist = nullptr;
  int* mcount = nullptr;
  int mgn = 0;
  int4* d_units = nullptr;
  int nunits = 0;
  // FP64-equivalent form: (hi, lo) pairs of ht, hu, hv, r_hu, r_hv (one
  // allocation, `total` pairs each), the march flags, the domains'
  // descriptors and march units, and the list of exact cells
  float2* dfs = nullptr;
  unsigned char* dfreg = nullptr;
  EnsDfDomain* d_dfdesc = nullptr;
  DfConst dk{};
  int4* d_dfunits = nullptr;
  int ndfunits = 0;
  int2* dfring = nullptr;  // the exact cells, (domain, cell index)
  int ndfring = 0;
  DfConst* d_dks = nullptr;  // per-domain constants when they differ, else null
};

Ens g_ens;

bool ck(cudaError_t e) { return e == cudaSuccess; }

void ens_free() {
  Ens& e = g_ens;
  if (e.graph) cudaGraphExecDestroy(e.graph);
  e.graph = nullptr;
  for (int b = 0; b < 2; b++) {
    cudaFree(e.sn[b]);
    cudaFree(e.un[b]);
    cudaFree(e.vn[b]);
    e.sn[b] = e.un[b] = e.vn[b] = nullptr;
  }
  for (double** p : {&e.ht, &e.hu, &e.hv, &e.zero, &e.r_hu, &e.r_hv, &e.d_tides, &e.d_sums}) {
    cudaFree(*p);
    *p = nullptr;
  }
  for (int b = 0; b < 2; b++) {
    cudaFree(e.msn[b]);
    cudaFree(e.mun[b]);
    cudaFree(e.mvn[b]);
    e.msn[b] = nullptr;
    e.mun[b] = e.mvn[b] = nullptr;
  }
  for (float** p : {&e.mht, &e.mhu, &e.mhv, &e.mrhu, &e.mrhv}) {
    cudaFree(*p);
    *p = nullptr;
  }
  cudaFree(e.d_mdesc);
  e.d_mdesc = nullptr;
  cudaFree(e.mreg);
  cudaFree(e.mglist);
  cudaFree(e.mcount);
  cudaFree(e.d_units);
  cudaFree(e.d_mks);
  e.d_mks = nullptr;
  e.mreg = nullptr;
  e.mglist = nullptr;
  e.mcount = nullptr;
  e.d_units = nullptr;
  e.mgn = e.nunits = 0;
  e.march = false;
  cudaFree(e.dfs);
  cudaFree(e.dfreg);
  cudaFree(e.d_dfdesc);
  cudaFree(e.d_dfunits);
  cudaFree(e.dfring);
  cudaFree(e.d_dks);
  e.d_dks = nullptr;
  e.dfs = nullptr;
  e.dfreg = nullptr;
  e.d_dfdesc = nullptr;
  e.d_dfunits = nullptr;
  e.dfring = nullptr;
  e.ndfunits = e.ndfring = 0;
  e.precision = 0;
  cudaFree(e.tmask);
  cudaFree(e.d_desc);
  cudaFree(e.d_tiles);
  cudaFree(e.d_first);
  e.tmask = nullptr;
  e.d_desc = nullptr;
  e.d_tiles = nullptr;
  e.d_first = nullptr;
  if (e.stream) cudaStreamDestroy(e.stream);
  e.stream = nullptr;
  if (e.side) cudaStreamDestroy(e.side);
  if (e.fork) cudaEventDestroy(e.fork);
  if (e.join) cudaEventDestroy(e.join);
  e.side = nullptr;
  e.fork = e.join = nullptr;
  e.tides_cap = e.sums_cap = 0;
  e.built = false;
  e.ndom = 0;
  e.dom.clear();
  e.shape = 0;
  e.march_rows = kDefaultMarchRows;
}

// Flather chains or reads outside the array exclude a domain (the one-launch
// update equals the reference's serial Flather loops only without them).
bool mask_ok(const DomainHost& D, const int* m) {
  const int W = D.W;
  auto writes = [&](int c, int step) {
    return m[c] + m[c + step] > -1 && (m[c] < 0 || m[c + step] < 0);
  };
  for (int j = D.ys - 1; j <= D.ye + 1; j++)
    for (int i = D.xs - 1; i <= D.xe; i++) {
      const int c = j * W + i;
      if (!writes(c, 1)) continue;
      const int nb = m[c] < 0 ? i + 1 : i - 1;
      if (nb < 0) return false;
      if (nb >= D.xs - 1 && nb <= D.xe && writes(j * W + nb, 1)) return false;
    }
  for (int j = D.ys - 1; j <= D.ye; j++)
    for (int i = D.xs - 1; i <= D.xe + 1; i++) {
      const int c = j * W + i;
      if (!writes(c, W)) continue;
      const int nb = m[c] < 0 ? j + 1 : j - 1;
      if (nb < 0) return false;
      if (nb >= D.ys - 1 && nb <= D.ye && writes(nb * W + i, W)) return false;
    }
  return true;
}

double tide_at(const DomainHost& D, int istep, double rdt) {
  // bc_ssh_code (boundary_conditions_kern.c:183-192) with this domain's
  // amplitude and period; 0.2 m and 12.42 h give the reference's bits.
  const double omega_tide = 2.0 * 3.14159 / (D.period_h * 3600.0);
  const double rtime = istep * rdt;
  return D.amp * std::sin(omega_tide * rtime);
}

// Tile list and static schedule.
bool build_schedule(int TXv, int TYv) {
  Ens& e = g_ens;
  struct T {
    int dom, i0, j0;
    double cost;
  };
  std::vector<T> tiles;
  for (int k = 0; k < e.ndom; k++) {
    const DomainHost& D = e.dom[k];
    const int nx = D.xe - D.xs + 3, ny = D.ye - D.ys + 2;
    const int ntx = (nx + TXv - 1) / TXv, nty = (ny + TYv - 1) / TYv;
    for (int by = 0; by < nty; by++)
      for (int bx = 0; bx < ntx; bx++) {
        const int cx = std::min(TXv, nx - bx * TXv), cy = std::min(TYv, ny - by * TYv);
        // boundary tiles run the general per-cell path on their edge cells
        double edge = 0.0;
        if (bx == 0 || bx == ntx - 1) edge += cy;
        if (by == 0 || by == nty - 1) edge += cx;
        tiles.push_back({k, D.xs - 1 + bx * TXv, D.ys - 1 + by * TYv,
                         (double)(cx * cy) + e.boundary_weight * edge});
      }
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e.nctas = e.policy == 2 ? std::max<int>(1, (int)tiles.size()) : std::max(1, sms * e.ctas_per_sm);
  std::vector<int4> order;
  std::vector<int> first(e.nctas + 1, 0);
  if (e.policy == 2) {
    // one tile per CTA, in domain order: the hardware block scheduler
    // balances the load and keeps as many CTAs per SM as fit
    for (size_t t = 0; t < tiles.size(); t++) {
      order.push_back(make_int4(tiles[t].dom, tiles[t].i0, tiles[t].j0, 0));
      first[t + 1] = (int)t + 1;
    }
  } else if (e.policy == 1) {
    // longest processing time first: biggest tile to the least-loaded CTA
    std::vector<int> idx(tiles.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return tiles[a].cost > tiles[b].cost; });
    std::vector<double> load(e.nctas, 0.0);
    std::vector<std::vector<int>> bins(e.nctas);
    for (int t : idx) {
      const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      load[b] += tiles[t].cost;
      bins[b].push_back(t);
    }
    for (int b = 0; b < e.nctas; b++) {
      std::sort(bins[b].begin(), bins[b].end());  // keep each CTA's tiles in memory order
      first[b + 1] = first[b] + (int)bins[b].size();
      for (int t : bins[b]) order.push_back(make_int4(tiles[t].dom, tiles[t].i0, tiles[t].j0, 0));
    }
  } else {
    // contiguous chunks of (nearly) equal cost, in domain order
    double total = 0.0;
    for (const T& t : tiles) total += t.cost;
    double acc = 0.0;
    int b = 0;
    for (size_t t = 0; t < tiles.size(); t++) {
      while (b < e.nctas - 1 && acc >= total * (b + 1) / e.nctas) first[++b] = (int)t;
      acc += tiles[t].cost;
      order.push_back(make_int4(tiles[t].dom, tiles[t].i0, tiles[t].j0, 0));
    }
    while (b < e.nctas) first[++b] = (int)tiles.size();
  }
  e.ntiles = (int)order.size();
  cudaFree(e.d_tiles);
  cudaFree(e.d_first);
  e.d_tiles = nullptr;
  e.d_first = nullptr;
  if (!ck(cudaMalloc(&e.d_tiles, sizeof(int4) * std::max<size_t>(1, order.size()))) ||
      !ck(cudaMalloc(&e.d_first, sizeof(int) * first.size())))
    return false;
  if (!ck(cudaMemcpy(e.d_tiles, order.data(), sizeof(int4) * order.size(),
                     cudaMemcpyHostToDevice)) ||
      !ck(cudaMemcpy(e.d_first, first.data(), sizeof(int) * first.size(),
                     cudaMemcpyHostToDevice)))
    return false;
  if (e.graph) cudaGraphExecDestroy(e.graph);
  e.graph = nullptr;
  return true;
}

bool build_descriptors() {
  Ens& e = g_ens;
  std::vector<EnsDomain> desc(e.ndom);
  for (int k = 0; k < e.ndom; k++) {
    const DomainHost& D = e.dom[k];
    EnsDomain& x = desc[k];
    memset(&x, 0, sizeof x);
    const size_t o = D.off;
    x.f.ht = e.ht + o;
    x.f.hu = e.hu + o;
    x.f.hv = e.hv + o;
    x.f.tmask = e.tmask + o;
    // rest start: sshn_u / sshn_v, ua / va and ssha_u / ssha_v are zero where
    // no step writes them
    x.f.sshn_u = x.f.sshn_v = x.f.ua = x.f.va = x.f.ssha_u = x.f.ssha_v = e.zero + o;
    x.f.r_hu = e.r_hu + o;
    x.f.r_hv = e.r_hv + o;
    for (int p = 0; p < 2; p++) {
      x.fs[p].sshn_in = e.sn[p] + o;
      x.fs[p].un_in = e.un[p] + o;
      x.fs[p].vn_in = e.vn[p] + o;
      x.fs[p].sshn_out = e.sn[1 - p] + o;
      x.fs[p].un_out = e.un[1 - p] + o;
      x.fs[p].vn_out = e.vn[1 - p] + o;
    }
    x.d = Dims{D.xs, D.xe, D.ys, D.ye, D.W, D.H};
    x.p = e.sc;
    UniformMetrics um{};
    um.area_t = um.area_u = um.area_v = D.dx * D.dy;
    um.dx_u = um.dx_v = um.dx_t = D.dx;
    um.dy_u = um.dy_v = um.dy_t = D.dy;
    um.sin_u = um.sin_v = std::sin(D.gphi * e.sc.d2r);
    x.um = um;
    x.k = make_fast_const(e.sc, um);
  }
  cudaFree(e.d_desc);
  e.d_desc = nullptr;
  if (!ck(cudaMalloc(&e.d_desc, sizeof(EnsDomain) * e.ndom))) return false;
  return ck(cudaMemcpy(e.d_desc, desc.data(), sizeof(EnsDomain) * e.ndom,
                       cudaMemcpyHostToDevice));
}

// The column march's flags, general-cell list and units; its step constants
// are kernel parameters when every domain shares them, else one set per
// domain (e.d_mks).
bool build_march(const std::vector<EnsMixDomain>& desc) {
  Ens& e = g_ens;
  e.march = false;
  bool shared = true;
  for (const EnsMixDomain& x : desc) shared = shared && memcmp(&x.k, &desc[0].k, sizeof x.k) == 0;
  cudaFree(e.d_mks);
  e.d_mks = nullptr;
  if (!shared) {
    std::vector<mixk::MarchConst> mks(desc.size());
    for (size_t q = 0; q < desc.size(); q++) mks[q] = mixk::make_march_const(desc[q].k);
    if (!ck(cudaMalloc(&e.d_mks, sizeof(mixk::MarchConst) * mks.size())) ||
        !ck(cudaMemcpy(e.d_mks, mks.data(), sizeof(mixk::MarchConst) * mks.size(),
                       cudaMemcpyHostToDevice)))
      return false;
  }
  if (!e.mreg && (!ck(cudaMalloc(&e.mreg, e.total)) || !ck(cudaMalloc(&e.mcount, sizeof(int)))))
    return false;
  // two passes: count the general cells, then list them
  for (int pass = 0; pass < 2; pass++) {
    if (pass == 1) {
      cudaFree(e.mglist);
      e.mglist = nullptr;
      if (e.mgn > 0 && !ck(cudaMalloc(&e.mglist, sizeof(int2) * e.mgn))) return false;
    }
    if (!ck(cudaMemsetAsync(e.mcount, 0, sizeof(int), e.stream))) return false;
    for (int k = 0; k < e.ndom; k++)
      launch_ens_mixed_flags(e.d_mdesc, k, e.mreg, pass == 1 ? e.mglist : nullptr, e.mcount,
                             e.stream);
    int n = 0;
    if (!ck(cudaGetLastError()) ||
        !ck(cudaMemcpyAsync(&n, e.mcount, sizeof(int), cudaMemcpyDeviceToHost, e.stream)) ||
        !ck(cudaStreamSynchronize(e.stream)))
      return false;
    if (pass == 1 && n != e.mgn) return false;
    e.mgn = n;
  }
  std::vector<int4> units;
  for (const EnsMixDomain& x : desc) {
    const int nx = x.d.xe - x.d.xs + 3, ny = x.d.ye - x.d.ys + 2;
    const int dom = (int)(&x - desc.data());
    const int mr = e.march_rows;
    for (int gy = 0; gy < (ny + mr - 1) / mr; gy++)
      for (int gx = 0; gx < (nx + mixk::MW - 1) / mixk::MW; gx++)
        units.push_back(make_int4(dom, x.d.xs - 1 + gx * mixk::MW, x.d.ys - 1 + gy * mr, 0));
  }
  cudaFree(e.d_units);
  e.d_units = nullptr;
  if (!ck(cudaMalloc(&e.d_units, sizeof(int4) * units.size())) ||
      !ck(cudaMemcpy(e.d_units, units.data(), sizeof(int4) * units.size(),
                     cudaMemcpyHostToDevice)))
    return false;
  e.nunits = (int)units.size();
  e.mk = desc[0].k;
  e.march = true;
  return true;
}

bool build_mixed() {
  Ens& e = g_ens;
  const size_t n = e.total;
  if (!e.msn[0]) {
    for (int b = 0; b < 2; b++)
      if (!ck(cudaMalloc(&e.msn[b], n * sizeof(float2))) ||
          !ck(cudaMalloc(&e.mun[b], n * 4)) || !ck(cudaMalloc(&e.mvn[b], n * 4)))
        return false;
    for (float** p : {&e.mht, &e.mhu, &e.mhv, &e.mrhu, &e.mrhv})
      if (!ck(cudaMalloc(p, n * 4))) return false;
  }
  for (int b = 0; b < 2; b++)
    if (!ck(cudaMemset(e.msn[b], 0, n * sizeof(float2))) || !ck(cudaMemset(e.mun[b], 0, n * 4)) ||
        !ck(cudaMemset(e.mvn[b], 0, n * 4)))
      return false;
  k_mixed_statics<<<152 * 8, 256, 0, e.stream>>>(e.ht, e.hu, e.hv, e.mht, e.mhu, e.mhv, e.mrhu,
                                                 e.mrhv, n);
  if (!ck(cudaGetLastError())) return false;
  std::vector<EnsMixDomain> desc(e.ndom);
  for (int k = 0; k < e.ndom; k++) {
    const DomainHost& D = e.dom[k];
    EnsMixDomain& x = desc[k];
    memset(&x, 0, sizeof x);
    const size_t o = D.off;
    x.mf = MixedFields{e.mht + o, e.mhu + o, e.mhv + o, e.mrhu + o, e.mrhv + o};
    for (int p = 0; p < 2; p++) {
      x.ms[p].sn_in = e.msn[p] + o;
      x.ms[p].un_in = e.mun[p] + o;
      x.ms[p].vn_in = e.mvn[p] + o;
      x.ms[p].sn_out = e.msn[1 - p] + o;
      x.ms[p].un_out = e.mun[1 - p] + o;
      x.ms[p].vn_out = e.mvn[1 - p] + o;
    }
    x.f.tmask = e.tmask + o;
    x.f.sshn_u = x.f.sshn_v = x.f.ua = x.f.va = x.f.ssha_u = x.f.ssha_v = e.zero + o;
    x.d = Dims{D.xs, D.xe, D.ys, D.ye, D.W, D.H};
    UniformMetrics um{};
    um.area_t = um.area_u = um.area_v = D.dx * D.dy;
    um.dx_u = um.dx_v = um.dx_t = D.dx;
    um.dy_u = um.dy_v = um.dy_t = D.dy;
    um.sin_u = um.sin_v = std::sin(D.gphi * e.sc.d2r);
    x.k = mixk::make_mix_const(e.sc, um);
    x.off = o;
  }
  cudaFree(e.d_mdesc);
  e.d_mdesc = nullptr;
  if (!ck(cudaMalloc(&e.d_mdesc, sizeof(EnsMixDomain) * e.ndom)) ||
      !ck(cudaMemcpy(e.d_mdesc, desc.data(), sizeof(EnsMixDomain) * e.ndom,
                     cudaMemcpyHostToDevice)))
    return false;
  return build_march(desc);
}

UniformMetrics domain_metrics(const DomainHost& D, const Scalars& sc) {
  UniformMetrics um{};
  um.area_t = um.area_u = um.area_v = D.dx * D.dy;
  um.dx_u = um.dx_v = um.dx_t = D.dx;
  um.dy_u = um.dy_v = um.dy_t = D.dy;
  um.sin_u = um.sin_v = std::sin(D.gphi * sc.d2r);
  return um;
}

// Whether every domain has the same grid spacing and latitude, so that one
// set of step constants (kernel parameters) serves the whole march.
bool shared_constants() {
  const Ens& e = g_ens;
  for (const DomainHost& D : e.dom)
    if (D.dx != e.dom[0].dx || D.dy != e.dom[0].dy || D.gphi != e.dom[0].gphi) return false;
  return true;
}

// The FP64-equivalent form's set-up, after build_descriptors(): the
// double-float statics, the march flags, units and descriptors, and the
// list of exact cells (rebuilt whenever the ensemble is).
bool build_df() {
  Ens& e = g_ens;
  const size_t n = e.total;
  cudaStream_t st = e.stream;
  if (!e.dfs && (!ck(cudaMalloc(&e.dfs, 5 * n * sizeof(float2))) || !ck(cudaMalloc(&e.dfreg, n))))
    return false;
  float2* pr[5] = {e.dfs, e.dfs + n, e.dfs + 2 * n, e.dfs + 3 * n, e.dfs + 4 * n};
  const double* src[5] = {e.ht, e.hu, e.hv, e.r_hu, e.r_hv};
  for (int a = 0; a < 5; a++) launch_df_split(src[a], pr[a], (long long)n, st);
  if (!ck(cudaMemsetAsync(e.dfreg, 0, n, st))) return false;
  std::vector<EnsDfDomain> desc(e.ndom);
  std::vector<int4> units;
  std::vector<int2> ring;
  for (int k = 0; k < e.ndom; k++) {
    const DomainHost& D = e.dom[k];
    const size_t o = D.off;
    const Dims d{D.xs, D.xe, D.ys, D.ye, D.W, D.H};
    launch_df_flags(e.tmask + o, d, e.dfreg + o, st);
    for (int c : D.ring) ring.push_back(make_int2(k, c));
    EnsDfDomain& x = desc[k];
    memset(&x, 0, sizeof x);
    for (int p = 0; p < 2; p++)
      x.fs[p] = FusedState{e.sn[p] + o,     e.un[p] + o,     e.vn[p] + o,
                           e.sn[1 - p] + o, e.un[1 - p] + o, e.vn[1 - p] + o};
    x.ff.ht = pr[0] + o;
    x.ff.hu = pr[1] + o;
    x.ff.hv = pr[2] + o;
    x.ff.rhu = pr[3] + o;
    x.ff.rhv = pr[4] + o;
    x.ff.reg = e.dfreg + o;
    x.d = d;
    const int nx = D.xe - D.xs + 3, ny = D.ye - D.ys + 2, mr = e.march_rows;
    for (int gy = 0; gy < (ny + mr - 1) / mr; gy++)
      for (int gx = 0; gx < (nx + kDfMarchCols - 1) / kDfMarchCols; gx++)
        units.push_back(make_int4(k, D.xs - 1 + gx * kDfMarchCols, D.ys - 1 + gy * mr, 0));
  }
  if (!ck(cudaGetLastError()) || !ck(cudaStreamSynchronize(st))) return false;
  cudaFree(e.d_dfdesc);
  cudaFree(e.d_dfunits);
  cudaFree(e.dfring);
  e.d_dfdesc = nullptr;
  e.d_dfunits = nullptr;
  e.dfring = nullptr;
  if (!ck(cudaMalloc(&e.d_dfdesc, sizeof(EnsDfDomain) * e.ndom)) ||
      !ck(cudaMalloc(&e.d_dfunits, sizeof(int4) * units.size())) ||
      !ck(cudaMalloc(&e.dfring, sizeof(int2) * std::max<size_t>(1, ring.size()))) ||
      !ck(cudaMemcpy(e.d_dfdesc, desc.data(), sizeof(EnsDfDomain) * e.ndom,
                     cudaMemcpyHostToDevice)) ||
      !ck(cudaMemcpy(e.d_dfunits, units.data(), sizeof(int4) * units.size(),
                     cudaMemcpyHostToDevice)) ||
      !ck(cudaMemcpy(e.dfring, ring.data(), sizeof(int2) * ring.size(),
                     cudaMemcpyHostToDevice)))
    return false;
  e.ndfunits = (int)units.size();
  e.ndfring = (int)ring.size();
  e.dk = make_df_const(e.sc, domain_metrics(e.dom[0], e.sc));
  // the march's constants: kernel parameters when every domain shares them,
  // else one set per domain
  cudaFree(e.d_dks);
  e.d_dks = nullptr;
  if (!shared_constants()) {
    std::vector<DfConst> dks(e.ndom);
    for (int k = 0; k < e.ndom; k++) dks[k] = make_df_const(e.sc, domain_metrics(e.dom[k], e.sc));
    if (!ck(cudaMalloc(&e.d_dks, sizeof(DfConst) * e.ndom)) ||
        !ck(cudaMemcpy(e.d_dks, dks.data(), sizeof(DfConst) * e.ndom, cudaMemcpyHostToDevice)))
      return false;
  }
  return true;
}

// FP64 state of every domain back to rest.
bool zero_fp64_state() {
  Ens& e = g_ens;
  const size_t bytes = e.total * sizeof(double);
  cudaStreamSynchronize(e.stream);
  for (double* p : {e.sn[0], e.sn[1], e.un[0], e.un[1], e.vn[0], e.vn[1]})
    if (!ck(cudaMemset(p, 0, bytes))) return false;
  e.parity = 0;
  return true;
}

// Interior (ssh, u, v) of every domain, all of size nx x ny, as FP32
// [dom][ny][nx][3] (the emulator's snapshot layout).
__global__ void k_export_interior(const EnsDomain* __restrict__ doms, int parity, int ndom,
                                  int nx, int ny, float* __restrict__ out) {
  const long long n = (long long)ndom * nx * ny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int dom = (int)(t / ((long long)nx * ny));
    const int rem = (int)(t - (long long)dom * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    const EnsDomain& D = doms[dom];
    const size_t c = (size_t)(D.d.ys + j) * D.d.width + (D.d.xs + i);
    const FusedState& st = D.fs[parity];
    out[t * 3 + 0] = (float)st.sshn_in[c];
    out[t * 3 + 1] = (float)st.un_in[c];
    out[t * 3 + 2] = (float)st.vn_in[c];
  }
}

// The same from the mixed-precision state: ssh hi + lo, velocities as held.
__global__ void k_export_interior_mixed(const EnsMixDomain* __restrict__ doms, int parity,
                                        int ndom, int nx, int ny, float* __restrict__ out) {
  const long long n = (long long)ndom * nx * ny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int dom = (int)(t / ((long long)nx * ny));
    const int rem = (int)(t - (long long)dom * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    const EnsMixDomain& D = doms[dom];
    const size_t c = (size_t)(D.d.ys + j) * D.d.width + (D.d.xs + i);
    const MixedState& st = D.ms[parity];
    const float2 s2 = st.sn_in[c];
    out[t * 3 + 0] = s2.x + s2.y;
    out[t * 3 + 1] = st.un_in[c];
    out[t * 3 + 2] = st.vn_in[c];
  }
}

// The inverse: FP32 [dom][ny][nx][3] into the interior of the current FP64
// state (both ping-pong buffers, so cells no step writes stay consistent).
// The interior leaves out one piece of the solver's state: the velocity on
// an open boundary face west or south of the interior (the Flather face),
// which the next step's momentum reads.  It is set from the adjacent
// interior face (zero normal gradient), so the state after an import
// depends on the imported interior alone and not on what the solver held
// before; wall faces stay zero.
__global__ void k_import_interior(const EnsDomain* __restrict__ doms, int ndom, int nx, int ny,
                                  const float* __restrict__ in) {
  const long long n = (long long)ndom * nx * ny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int dom = (int)(t / ((long long)nx * ny));
    const int rem = (int)(t - (long long)dom * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    const EnsDomain& D = doms[dom];
    const int W = D.d.width;
    const size_t c = (size_t)(D.d.ys + j) * W + (D.d.xs + i);
    const double e = (double)in[t * 3 + 0], u = (double)in[t * 3 + 1],
                 v = (double)in[t * 3 + 2];
    const bool west_open = i == 0 && D.f.tmask[c - 1] < 0;
    const bool south_open = j == 0 && D.f.tmask[c - W] < 0;
    for (int p = 0; p < 2; p++) {
      const FusedState& st = D.fs[p];
      const_cast<double*>(st.sshn_in)[c] = e;
      const_cast<double*>(st.un_in)[c] = u;
      const_cast<double*>(st.vn_in)[c] = v;
      if (west_open) const_cast<double*>(st.un_in)[c - 1] = u;
      if (south_open) const_cast<double*>(st.vn_in)[c - W] = v;
    }
  }
}

__global__ void k_recip(const double* __restrict__ h, double* __restrict__ r, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
       t += (size_t)gridDim.x * blockDim.x) {
    const double dd = h[t] + 0.0;  // ssha_u / ssha_v are zero at rest
    r[t] = (dd >= 0x1p-100 && dd <= 0x1p100) ? 1.0 / dd : 0.0;
  }
}

}  // namespace
}  // namespace nl2d

using namespace nl2d;

extern "C" {

int nl2d_ens_create(int ndom, const int* dims6, const double* geo3, const double* tide2,
                    const double* phys6) {
  ens_free();
  Ens& e = g_ens;
  if (ndom < 1 || !dims6 || !geo3 || !tide2 || !phys6) return NL2D_ERR_ARGS;
  e.sc = Scalars{phys6[0], phys6[1], phys6[2], phys6[3], phys6[4], phys6[5]};
  e.dom.resize(ndom);
  size_t off = 0;
  for (int k = 0; k < ndom; k++) {
    DomainHost& D = e.dom[k];
    D.W = dims6[6 * k], D.H = dims6[6 * k + 1];
    D.xs = dims6[6 * k + 2], D.xe = dims6[6 * k + 3];
    D.ys = dims6[6 * k + 4], D.ye = dims6[6 * k + 5];
    if (D.xs < 1 || D.ys < 1 || D.xe < D.xs || D.ye < D.ys || D.xe > D.W - 2 ||
        D.ye > D.H - 2) {
      e.dom.clear();
      return NL2D_ERR_ARGS;
    }
    D.dx = geo3[3 * k], D.dy = geo3[3 * k + 1], D.gphi = geo3[3 * k + 2];
    D.amp = tide2[2 * k], D.period_h = tide2[2 * k + 1];
    D.off = off;
    off += ((size_t)D.W * D.H + 31) / 32 * 32;  // 256-byte aligned domain starts
  }
  e.ndom = ndom;
  e.total = off;
  const size_t bytes = off * sizeof(double);
  if (!ck(cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking))) return NL2D_ERR_CUDA;
  int least = 0, greatest = 0;
  if (!ck(cudaDeviceGetStreamPriorityRange(&least, &greatest)) ||
      !ck(cudaStreamCreateWithPriority(&e.side, cudaStreamNonBlocking, greatest)) ||
      !ck(cudaEventCreateWithFlags(&e.fork, cudaEventDisableTiming)) ||
      !ck(cudaEventCreateWithFlags(&e.join, cudaEventDisableTiming)))
    return NL2D_ERR_CUDA;
  for (int b = 0; b < 2; b++)
    if (!ck(cudaMalloc(&e.sn[b], bytes)) || !ck(cudaMalloc(&e.un[b], bytes)) ||
        !ck(cudaMalloc(&e.vn[b], bytes)))
      return NL2D_ERR_CUDA;
  for (double** p : {&e.ht, &e.hu, &e.hv, &e.zero, &e.r_hu, &e.r_hv})
    if (!ck(cudaMalloc(p, bytes))) return NL2D_ERR_CUDA;
  if (!ck(cudaMalloc(&e.tmask, off * sizeof(int)))) return NL2D_ERR_CUDA;
  for (double* p : {e.sn[0], e.sn[1], e.un[0], e.un[1], e.vn[0], e.vn[1], e.zero})
    if (!ck(cudaMemset(p, 0, bytes))) return NL2D_ERR_CUDA;
  if (!ck(cudaMemset(e.tmask, 0, off * sizeof(int)))) return NL2D_ERR_CUDA;
  e.parity = 0;
  return NL2D_OK;
}

int nl2d_ens_set_domain(int dom, const int* tmask, const double* ht, const double* hu,
                        const double* hv) {
  Ens& e = g_ens;
  if (dom < 0 || dom >= e.ndom || !tmask || !ht || !hu || !hv) return NL2D_ERR_ARGS;
  DomainHost& D = e.dom[dom];
  if (!mask_ok(D, tmask)) return NL2D_ERR_ARGS;
  D.ring = ring_cells(D, tmask);
  const size_t n = (size_t)D.W * D.H;
  for (size_t t = 0; t < n; t++)
    if (!(hu[t] > 0.0) || !(hv[t] > 0.0)) return NL2D_ERR_ARGS;
  if (!ck(cudaMemcpy(e.tmask + D.off, tmask, n * sizeof(int), cudaMemcpyHostToDevice)) ||
      !ck(cudaMemcpy(e.ht + D.off, ht, n * 8, cudaMemcpyHostToDevice)) ||
      !ck(cudaMemcpy(e.hu + D.off, hu, n * 8, cudaMemcpyHostToDevice)) ||
      !ck(cudaMemcpy(e.hv + D.off, hv, n * 8, cudaMemcpyHostToDevice)))
    return NL2D_ERR_CUDA;
  k_recip<<<64, 256, 0, e.stream>>>(e.hu + D.off, e.r_hu + D.off, n);
  k_recip<<<64, 256, 0, e.stream>>>(e.hv + D.off, e.r_hv + D.off, n);
  if (!ck(cudaGetLastError())) return NL2D_ERR_CUDA;
  D.ready = true;
  e.built = false;
  return NL2D_OK;
}

int nl2d_ens_schedule(int ctas_per_sm, int policy, double boundary_weight) {
  Ens& e = g_ens;
  if (ctas_per_sm < 1 || ctas_per_sm > 2 || policy < 0 || policy > 2 || boundary_weight < 0)
    return NL2D_ERR_ARGS;
  e.ctas_per_sm = ctas_per_sm;
  e.policy = policy;
  e.boundary_weight = boundary_weight;
  e.built = false;
  return NL2D_OK;
}

int nl2d_ens_tile(int tx, int ty, int march_rows) {
  Ens& e = g_ens;
  int shape = -1;
  for (int k = 0; k < kNumShapes; k++)
    if (kShapes[k][0] == tx && kShapes[k][1] == ty) shape = k;
  if (shape < 0 ||
      (march_rows != 8 && march_rows != 16 && march_rows != 32 && march_rows != 64))
    return NL2D_ERR_ARGS;
  e.shape = shape;
  e.march_rows = march_rows;
  e.built = false;
  return NL2D_OK;
}

int nl2d_ens_run(int istep0, int nsteps, int checksum_every, double* checksums_out,
                 double* ms_out) {
  nl2d::NvtxRange nvtx_range("nl2d_ens_run");
  Ens& e = g_ens;
  if (ms_out) *ms_out = 0.0;
  if (e.ndom < 1 || nsteps < 0 || checksum_every < 0) return NL2D_ERR_ARGS;
  for (const DomainHost& D : e.dom)
    if (!D.ready) return NL2D_ERR_STATE;
  if (!e.built) {
    // a rebuild may move every buffer a captured graph refers to
    if (e.graph) cudaGraphExecDestroy(e.graph);
    e.graph = nullptr;
    if (e.precision == 1) {
      if (!build_mixed()) return NL2D_ERR_CUDA;
      e.parity = 0;  // the mixed state was set to rest
    } else if (!build_descriptors() ||
               !build_schedule(kShapes[e.shape][0], kShapes[e.shape][1]) ||
               (e.precision == 2 && !build_df())) {
      return NL2D_ERR_CUDA;
    }
    e.built = true;
  }
  if (nsteps == 0) return NL2D_OK;
  const int nsums = checksum_every > 0 ? nsteps / checksum_every : 0;
  if (nsums > 0 && !checksums_out) return NL2D_ERR_ARGS;
  // per-step, per-domain tidal values (host libm)
  const size_t ntide = (size_t)nsteps * e.ndom;
  if (e.tides_cap < ntide) {
    cudaFree(e.d_tides);
    e.d_tides = nullptr;
    if (e.graph) cudaGraphExecDestroy(e.graph);
    e.graph = nullptr;
    if (!ck(cudaMalloc(&e.d_tides, ntide * 8))) return NL2D_ERR_CUDA;
    e.tides_cap = ntide;
  }
  std::vector<double> tides(ntide);
  for (int q = 0; q < nsteps; q++)
    for (int k = 0; k < e.ndom; k++)
      tides[(size_t)q * e.ndom + k] = tide_at(e.dom[k], istep0 + q, e.sc.rdt);
  if (!ck(cudaMemcpyAsync(e.d_tides, tides.data(), ntide * 8, cudaMemcpyHostToDevice,
                          e.stream)))
    return NL2D_ERR_CUDA;
  const size_t nsum_vals = (size_t)std::max(nsums, 1) * e.ndom * 3;
  if (e.sums_cap < nsum_vals) {
    cudaFree(e.d_sums);
    e.d_sums = nullptr;
    if (e.graph) cudaGraphExecDestroy(e.graph);
    e.graph = nullptr;
    if (!ck(cudaMalloc(&e.d_sums, nsum_vals * 8))) return NL2D_ERR_CUDA;
    e.sums_cap = nsum_vals;
  }
  const int key[8] = {nsteps,   checksum_every, e.parity, e.nctas,
                      e.policy, e.precision,    e.shape,  e.march_rows};
  if (!(e.graph && memcmp(key, e.graph_key, sizeof key) == 0)) {
    if (e.graph) cudaGraphExecDestroy(e.graph);
    e.graph = nullptr;
    cudaGraph_t g = nullptr;
    if (e.precision == 0 && !prepare_ens_step(e.shape)) return NL2D_ERR_CUDA;
    if (!ck(cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal)))
      return NL2D_ERR_CUDA;
    int par = e.parity;
    for (int q = 0; q < nsteps; q++) {
      double* sums = e.d_sums + (size_t)((q + 1) / std::max(checksum_every, 1) - 1) * e.ndom * 3;
      const bool want_sums = checksum_every > 0 && (q + 1) % checksum_every == 0;
      if (e.precision == 1) {
        const MixedFields mf{e.mht, e.mhu, e.mhv, e.mrhu, e.mrhv, e.mreg, nullptr, 0};
        const MixedState ms{e.msn[par], e.mun[par], e.mvn[par],
                            e.msn[1 - par], e.mun[1 - par], e.mvn[1 - par]};
        // the general cells (each a long chain of global loads) start first
        // on the side stream and run beside the march: both read the same
        // buffers and write disjoint cells
        cudaEventRecord(e.fork, e.stream);
        cudaStreamWaitEvent(e.side, e.fork, 0);
        launch_ens_mixed_general(e.d_mdesc, e.mglist, e.mgn, par,
                                 e.d_tides + (size_t)q * e.ndom, e.side);
        launch_ens_mixed_march(e.d_mdesc, e.d_units, e.nunits, mf, ms, &e.mk, e.d_mks,
                               e.march_rows, e.stream);
        cudaEventRecord(e.join, e.side);
        cudaStreamWaitEvent(e.stream, e.join, 0);
        par = 1 - par;
        if (want_sums)
          k_ensemble_mixed_checksums<<<dim3(e.ndom, 3), 256, 0, e.stream>>>(e.d_mdesc, par,
                                                                            sums);
      } else if (e.precision == 2) {
        constexpr int B = 32 * dfm::WARPS;
        const int nring = (e.ndfring + B - 1) / B;
        const int nmarch = (e.ndfunits + dfm::WARPS - 1) / dfm::WARPS;
        const double* tq = e.d_tides + (size_t)q * e.ndom;
        if (e.d_dks)
          k_ensemble_df_step<true><<<nring + nmarch, B, 0, e.stream>>>(
              e.d_dfdesc, e.d_dfunits, e.ndfunits, e.d_desc, e.dfring, e.ndfring, nring, par,
              e.dk, e.d_dks, e.march_rows, tq);
        else
          k_ensemble_df_step<false><<<nring + nmarch, B, 0, e.stream>>>(
              e.d_dfdesc, e.d_dfunits, e.ndfunits, e.d_desc, e.dfring, e.ndfring, nring, par,
              e.dk, nullptr, e.march_rows, tq);
        par = 1 - par;
        if (want_sums)
          k_ensemble_checksums<<<dim3(e.ndom, 3), 256, 0, e.stream>>>(e.d_desc, par, e.ndom,
                                                                      sums);
      } else {
        launch_ens_step(e.shape, e.nctas, e.d_desc, e.d_tiles, e.d_first, par,
                        e.d_tides + (size_t)q * e.ndom, e.stream);
        par = 1 - par;
        if (want_sums)
          k_ensemble_checksums<<<dim3(e.ndom, 3), 256, 0, e.stream>>>(e.d_desc, par, e.ndom,
                                                                      sums);
      }
    }
    if (!ck(cudaStreamEndCapture(e.stream, &g))) return NL2D_ERR_CUDA;
    const bool ok = ck(cudaGraphInstantiate(&e.graph, g, 0));
    cudaGraphDestroy(g);
    if (!ok) return NL2D_ERR_CUDA;
    memcpy(e.graph_key, key, sizeof key);
  }
  cudaEvent_t e0, e1;
  if (!ck(cudaEventCreate(&e0)) || !ck(cudaEventCreate(&e1))) return NL2D_ERR_CUDA;
  cudaStreamSynchronize(e.stream);
  cudaEventRecord(e0, e.stream);
  const bool launched = ck(cudaGraphLaunch(e.graph, e.stream));
  cudaEventRecord(e1, e.stream);
  const bool done = ck(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!launched || !done) return NL2D_ERR_CUDA;
  if (ms_out) *ms_out = ms;
  e.parity = (e.parity + nsteps) & 1;
  if (nsums > 0 && !ck(cudaMemcpy(checksums_out, e.d_sums, (size_t)nsums * e.ndom * 3 * 8,
                                  cudaMemcpyDeviceToHost)))
    return NL2D_ERR_CUDA;
  return NL2D_OK;
}

int nl2d_ens_read(int dom, double* sshn_t, double* un, double* vn) {
  Ens& e = g_ens;
  if (dom < 0 || dom >= e.ndom) return NL2D_ERR_ARGS;
  const DomainHost& D = e.dom[dom];
  const size_t n = (size_t)D.W * D.H;
  cudaStreamSynchronize(e.stream);
  if (e.precision == 1) {  // FP64 image of the mixed state
    std::vector<float2> s2(n);
    std::vector<float> f(n);
    if (sshn_t) {
      if (!ck(cudaMemcpy(s2.data(), e.msn[e.parity] + D.off, n * sizeof(float2),
                         cudaMemcpyDeviceToHost)))
        return NL2D_ERR_CUDA;
      for (size_t t = 0; t < n; t++) sshn_t[t] = (double)s2[t].x + (double)s2[t].y;
    }
    float* fsrc[2] = {e.mun[e.parity] + D.off, e.mvn[e.parity] + D.off};
    double* fdst[2] = {un, vn};
    for (int k = 0; k < 2; k++) {
      if (!fdst[k]) continue;
      if (!ck(cudaMemcpy(f.data(), fsrc[k], n * 4, cudaMemcpyDeviceToHost))) return NL2D_ERR_CUDA;
      for (size_t t = 0; t < n; t++) fdst[k][t] = (double)f[t];
    }
    return NL2D_OK;
  }
  double* src[3] = {e.sn[e.parity] + D.off, e.un[e.parity] + D.off, e.vn[e.parity] + D.off};
  double* dst[3] = {sshn_t, un, vn};
  for (int k = 0; k < 3; k++)
    if (dst[k] && !ck(cudaMemcpy(dst[k], src[k], n * 8, cudaMemcpyDeviceToHost)))
      return NL2D_ERR_CUDA;
  return NL2D_OK;
}

int nl2d_ens_info(long long* cells, int* ntiles, int* nctas) {
  const Ens& e = g_ens;
  long long c = 0;
  for (const DomainHost& D : e.dom) c += (long long)(D.xe - D.xs + 1) * (D.ye - D.ys + 1);
  if (cells) *cells = c;
  if (ntiles) *ntiles = e.ntiles;
  if (nctas) *nctas = e.nctas;
  return NL2D_OK;
}

int nl2d_ens_set_precision(int precision) {
  Ens& e = g_ens;
  if (precision < 0 || precision > 2) return NL2D_ERR_ARGS;
  if (e.ndom < 1) return NL2D_ERR_STATE;
  if (precision != e.precision) {
    e.precision = precision;
    e.built = false;  // the next run starts this form from rest
    if (e.graph) cudaGraphExecDestroy(e.graph);
    e.graph = nullptr;
    // the mixed form's rebuild sets its own state to rest
    if (precision != 1 && !zero_fp64_state()) return NL2D_ERR_CUDA;
  }
  return NL2D_OK;
}

int nl2d_ens_export_interior(float* d_out) {
  Ens& e = g_ens;
  if (e.ndom < 1 || !d_out || !e.built) return NL2D_ERR_STATE;
  const int nx = e.dom[0].xe - e.dom[0].xs + 1, ny = e.dom[0].ye - e.dom[0].ys + 1;
  for (const DomainHost& D : e.dom)
    if (D.xe - D.xs + 1 != nx || D.ye - D.ys + 1 != ny) return NL2D_ERR_ARGS;
  if (e.precision == 1)
    k_export_interior_mixed<<<152 * 8, 256, 0, e.stream>>>(e.d_mdesc, e.parity, e.ndom, nx, ny,
                                                           d_out);
  else
    k_export_interior<<<152 * 8, 256, 0, e.stream>>>(e.d_desc, e.parity, e.ndom, nx, ny, d_out);
  if (!ck(cudaGetLastError()) || !ck(cudaStreamSynchronize(e.stream))) return NL2D_ERR_CUDA;
  return NL2D_OK;
}

int nl2d_ens_import_interior(const float* d_in) {
  Ens& e = g_ens;
  if (e.ndom < 1 || !d_in || e.precision == 1 || !e.built) return NL2D_ERR_STATE;
  const int nx = e.dom[0].xe - e.dom[0].xs + 1, ny = e.dom[0].ye - e.dom[0].ys + 1;
  for (const DomainHost& D : e.dom)
    if (D.xe - D.xs + 1 != nx || D.ye - D.ys + 1 != ny) return NL2D_ERR_ARGS;
  k_import_interior<<<152 * 8, 256, 0, e.stream>>>(e.d_desc, e.ndom, nx, ny, d_in);
  if (!ck(cudaGetLastError()) || !ck(cudaStreamSynchronize(e.stream))) return NL2D_ERR_CUDA;
  return NL2D_OK;
}

int nl2d_ens_reset(void) {
  Ens& e = g_ens;
  if (e.ndom < 1) return NL2D_ERR_STATE;
  if (e.precision == 1) {
    e.built = false;  // mixed state is re-zeroed when rebuilt
    return NL2D_OK;
  }
  return zero_fp64_state() ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_ens_uses_march(void) { return g_ens.march ? 1 : 0; }

void nl2d_ens_destroy(void) { ens_free(); }

}  // extern "C"
