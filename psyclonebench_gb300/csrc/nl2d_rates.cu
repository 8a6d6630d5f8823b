// Issue rates of the arithmetic pipes the step forms are bound by (no
// counterpart in the reference): FP64 fused multiply-add, multiply and add,
// and FP32 fused multiply-add, each as eight independent dependency chains
// per thread over 8 CTAs of 256 threads per SM.  The benchmark divides the
// FP64 step's FP64-pipe instructions by the fastest FP64 rate measured here
// for the roofline of that form (it is bound by the FP64 pipe, not by HBM).
//
// Built with the library's -fmad=false: the FP64 chains use fma() explicitly
// and the plain add and multiply chains stay single operations.
#include "nl2d_internal.h"

#include "../../include/nl2d_gpu.h"

namespace nl2d {
namespace {

template <int OP>
__global__ void __launch_bounds__(256) k_rate_f64(double* out, double a, double b, int iters) {
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; q++) x[q] = 1.0 + 1e-3 * threadIdx.x + 0.1 * q;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      if (OP == 0) x[q] = fma(x[q], a, b);
      if (OP == 1) x[q] = x[q] * a;
      if (OP == 2) x[q] = x[q] + a;
    }
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 8; q++) s += x[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_rate_f32(float* out, float a, float b, int iters) {
  float x[8];
#pragma unroll
  for (int q = 0; q < 8; q++) x[q] = 1.0f + 1e-3f * threadIdx.x + 0.1f * q;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = fmaf(x[q], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < 8; q++) s += x[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace nl2d

using namespace nl2d;

extern "C" int nl2d_measure_pipe_rates(double out[4]) {
  if (!out) return NL2D_ERR_ARGS;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return NL2D_ERR_CUDA;
  const int nb = sms * 8, nt = 256, iters = 4096;
  double* od = nullptr;
  if (cudaMalloc(&od, (size_t)nb * nt * sizeof(double)) != cudaSuccess) return NL2D_ERR_CUDA;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool ok = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  for (int op = 0; op < 4 && ok; op++) {
    const int it = op == 3 ? iters * 8 : iters;
    auto launch = [&]() {
      if (op == 0) k_rate_f64<0><<<nb, nt>>>(od, 1.0000001, 1e-9, it);
      if (op == 1) k_rate_f64<1><<<nb, nt>>>(od, 1.0000001, 0.0, it);
      if (op == 2) k_rate_f64<2><<<nb, nt>>>(od, 1e-9, 0.0, it);
      if (op == 3) k_rate_f32<<<nb, nt>>>((float*)od, 1.0000001f, 1e-9f, it);
    };
    float best = 0.f;
    for (int rep = 0; rep < 3 && ok; rep++) {  // the first launch warms up
      launch();
      ok = cudaEventRecord(e0) == cudaSuccess;
      launch();
      ok = ok && cudaEventRecord(e1) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess;
      float ms = 0.f;
      ok = ok && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      if (ok && rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    const double ops = (double)nb * nt * it * 8;
    out[op] = ok && best > 0.f ? ops / (best * 1e-3) / 1e9 : 0.0;
  }
  ok = ok && cudaGetLastError() == cudaSuccess;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(od);
  return ok ? NL2D_OK : NL2D_ERR_CUDA;
}
