// Field checksum: sum of |f| over a rectangle of the field, the quantity
// dl_esm_inf's field_checksum prints (restated by regent/checksum.rg:12-31;
// used at psykal_cpp/nemolite2d.f90:118-121).
//
// Two deterministic passes: a fixed grid of blocks, each accumulating a
// grid-stride share of the rectangle in FP64 and reducing it with warp
// shuffles, writes one partial sum per block to a scratch array; one block
// then reduces the partials in a fixed order.  The association differs from
// the reference's serial sum, so results agree to rounding (about 1e-15
// relative), not bit for bit; repeated runs are bit-identical.
#include "nl2d_internal.h"

#include <atomic>

#include "../../include/nl2d_gpu.h"

namespace nl2d {
namespace {

constexpr int kBlocks = 152 * 4;  // a multiple of the SM count
constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum(double v, double* warp_partials) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_partials[wid] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? warp_partials[threadIdx.x] : 0.0;
  if (wid == 0) v = warp_sum(v);
  return v;
}

__device__ __forceinline__ double as_f64(double v) { return v; }
__device__ __forceinline__ double as_f64(float v) { return (double)v; }
__device__ __forceinline__ double as_f64(float2 v) { return (double)v.x + (double)v.y; }

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_abs_sum_partial(const T* __restrict__ f, int W, int x0, int nx, int y0, int ny,
                      double* __restrict__ partials) {
  __shared__ double wp[kThreads / 32];
  double acc = 0.0;
  const long long total = (long long)nx * ny;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t / nx), i = (int)(t - (long long)j * nx);
    acc += fabs(as_f64(f[(long long)(y0 + j) * W + (x0 + i)]));
  }
  acc = block_sum(acc, wp);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kThreads)
    k_abs_sum_final(const double* __restrict__ partials, int n, double* __restrict__ out) {
  __shared__ double wp[kThreads / 32];
  double acc = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) acc += partials[t];
  acc = block_sum(acc, wp);
  if (threadIdx.x == 0) *out = acc;
}

}  // namespace

int checksum_partials_needed() { return kBlocks; }

void launch_checksum(const double* f, int width, int x0, int x1, int y0, int y1,
                     double* partials, double* out, cudaStream_t st) {
  const int nx = x1 >= x0 ? x1 - x0 + 1 : 0, ny = y1 >= y0 ? y1 - y0 + 1 : 0;
  k_abs_sum_partial<<<kBlocks, kThreads, 0, st>>>(f, width, x0, nx, y0, ny, partials);
  k_abs_sum_final<<<1, kThreads, 0, st>>>(partials, kBlocks, out);
}

void launch_checksum_f32(const float* f, int width, int x0, int x1, int y0, int y1,
                         double* partials, double* out, cudaStream_t st) {
  const int nx = x1 >= x0 ? x1 - x0 + 1 : 0, ny = y1 >= y0 ? y1 - y0 + 1 : 0;
  k_abs_sum_partial<<<kBlocks, kThreads, 0, st>>>(f, width, x0, nx, y0, ny, partials);
  k_abs_sum_final<<<1, kThreads, 0, st>>>(partials, kBlocks, out);
}

void launch_checksum_f2(const float2* f, int width, int x0, int x1, int y0, int y1,
                        double* partials, double* out, cudaStream_t st) {
  const int nx = x1 >= x0 ? x1 - x0 + 1 : 0, ny = y1 >= y0 ? y1 - y0 + 1 : 0;
  k_abs_sum_partial<<<kBlocks, kThreads, 0, st>>>(f, width, x0, nx, y0, ny, partials);
  k_abs_sum_final<<<1, kThreads, 0, st>>>(partials, kBlocks, out);
}

}  // namespace nl2d

// ---- allocation-free variant ------------------------------------------
//
// Some callers cannot call cudaMalloc: a host model whose own memory
// manager owns every device buffer (an OpenACC / OpenMP-target Fortran
// driver that maps the fields itself), or a time loop that must not trigger
// the device-wide synchronisation an allocation can cause.  For them the
// partial sums live in this file-scope device array instead of a buffer the
// library allocates.  Every GPU that loads the library holds it until the
// process exits.
namespace {

constexpr int kNoAllocMaxPartials = 16384;  // 128 KiB per device
constexpr long long kNoAllocCellsPerPartial = 256LL * 16;  // one block, 16 cells a thread
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxPartials];

constexpr int kMaxDevices = 64;
// One cached address per device, filled on that device's first call.  Host
// threads may make their first calls at the same time; the entries are
// atomics, and every thread that looks an address up stores the same value.
std::atomic<double*> g_noalloc_addr[kMaxDevices];

// Device address of g_noalloc_partials on the current device.  In host
// code the array's name is only a host-side stand-in, so the address comes
// from cudaGetSymbolAddress, once per device, with that device current.
// The address stays valid as long as the device's context does: after a
// cudaDeviceReset, nl2d_noalloc_forget() (called by nl2d_finalize) drops it
// so that the next call looks it up again.
cudaError_t noalloc_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  double* p = g_noalloc_addr[dev].load(std::memory_order_relaxed);
  if (!p) {
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_partials);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev].store(p, std::memory_order_relaxed);
  }
  *out = p;
  return cudaSuccess;
}

}  // namespace

namespace nl2d {
void noalloc_forget() {
  for (auto& a : g_noalloc_addr) a.store(nullptr, std::memory_order_relaxed);
}
}  // namespace nl2d

// Sum of |d_field| over a rectangle without allocating: the library's two
// checksum kernels, with one partial sum per block of 4096 cells kept in
// g_noalloc_partials.  Rectangles of more than 16384 x 4096 = 67,108,864
// cells (8192 x 8192) are rejected.  The first call on a device looks up
// the array's device address; make that first call before any stream
// capture.  All calls share the array: two calls that overlap on the GPU
// (different streams, no ordering between them) race on it.
extern "C" int nl2d_field_checksum_noalloc(const double* d_field, int width, int x0, int x1,
                                           int y0, int y1, double* d_out, void* stream) {
  if (!d_field || !d_out || width < 1 || x0 < 0 || y0 < 0 || x1 >= width || x1 < x0 ||
      y1 < y0)
    return NL2D_ERR_ARGS;
  const long long cells = (long long)(x1 - x0 + 1) * (y1 - y0 + 1);
  const long long blocks = (cells + kNoAllocCellsPerPartial - 1) / kNoAllocCellsPerPartial;
  if (blocks > kNoAllocMaxPartials) return NL2D_ERR_TOO_LARGE;
  // A launch error that earlier work left pending in this thread belongs to
  // its caller: it is left in place (not cleared) and reported, and nothing
  // is launched, so the status below is this call's own.
  if (cudaPeekAtLastError() != cudaSuccess) return NL2D_ERR_CUDA;
  double* scratch = nullptr;
  if (noalloc_scratch(&scratch) != cudaSuccess) return NL2D_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  // Every partial the final pass reads is written by the first pass, so the
  // array needs no clearing between calls.
  nl2d::k_abs_sum_partial<<<(int)blocks, nl2d::kThreads, 0, st>>>(
      d_field, width, x0, x1 - x0 + 1, y0, y1 - y0 + 1, scratch);
  nl2d::k_abs_sum_final<<<1, nl2d::kThreads, 0, st>>>(scratch, (int)blocks, d_out);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}
