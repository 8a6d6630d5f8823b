// Learned emulator kernels: a 3x3 convolution as an implicit GEMM on the
// 5th-generation tensor cores (tcgen05, BF16 operands, FP32 accumulation in
// tensor memory), plus the small elementwise kernels training needs.
//
// Layouts.  Activations are NHWC BF16 with the channel count padded to a
// multiple of 16; weights are [tap][Cout][Cin] BF16 (tap = 3*dy + dx,
// dy, dx in 0..2 for offsets -1..1), Cin contiguous.  The GEMM of one CTA:
//   D[m][n] = sum over tap, k of A[m][(tap, k)] * B[n][(tap, k)]
// with m = 128 consecutive output pixels of one image row, n = output
// channel, k = input channel, A = the input shifted by the tap (zero
// outside the image).  D lives in tensor memory (128 lanes x Cout FP32
// columns); operands are staged in shared memory in the no-swizzle K-major
// core-matrix layout (8 rows x 16 bytes per core matrix, core matrices
// adjacent along K 128 bytes apart, along M/N 16*Cin bytes apart).
//
// The backward pass reuses the same kernel: the input gradient is the
// convolution of the output gradient with the tap-flipped, channel-
// transposed weights.  The weight gradient is a reduction over pixels done
// on the CUDA cores in FP32.
//
// Every wait on the MMA completion barrier is bounded; on timeout the
// kernel records an error flag, skips its epilogue, frees its tensor memory
// and returns.
#include <cuda_bf16.h>
#include <cstdint>

#include "../../include/nl2d_gpu.h"

namespace nl2d {
namespace emu {
namespace {

constexpr int kTileM = 128;       // pixels per CTA (one row segment)
constexpr int kThreads = 128;     // 4 warps: loaders, then the epilogue
constexpr int kTmemCols = 64;     // >= Cout (<= 64), a power of two >= 32
constexpr long long kMaxWaitCycles = 1LL << 31;  // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading (K)
// byte offset, stride (M/N) byte offset, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator, BF16
// A and B, both K-major, N = n, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(kTileM >> 4) << 24);
}

// Byte offset of element (row, k) of a K-major operand with `cin` columns.
__device__ __forceinline__ uint32_t core_off(int row, int k, int cin) {
  return (uint32_t)((row >> 3) * (cin * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__global__ void __launch_bounds__(kThreads)
    k_conv3x3_tc(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ w,
                 const float* __restrict__ bias, __nv_bfloat16* __restrict__ y,
                 float* __restrict__ y32, int H, int W, int cin, int cout, int relu,
                 int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t taddr_slot;

  const int segs = W / kTileM;
  const int seg = blockIdx.x % segs, row = blockIdx.x / segs, img = blockIdx.y;
  const int x0 = seg * kTileM;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t a_bytes = (uint32_t)kTileM * cin * 2;  // one tap's A tile
  const uint32_t b_bytes = (uint32_t)cout * cin * 2;    // one tap's weights
  unsigned char* a_s = smem;
  unsigned char* b_s = smem + 9 * a_bytes;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&taddr_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }

  // Stage the 9 shifted input tiles and the 9 weight taps (16-byte chunks).
  const int kc = cin >> 3;  // 16-byte chunks per pixel
  for (int t = tid; t < 9 * kTileM * kc; t += kThreads) {
    const int tap = t / (kTileM * kc), rem = t - tap * kTileM * kc;
    const int m = rem / kc, ch = rem - m * kc;
    const int yy = row + tap / 3 - 1, xx = x0 + m + tap % 3 - 1;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (yy >= 0 && yy < H && xx >= 0 && xx < W)
      v = *reinterpret_cast<const uint4*>(x + (((size_t)img * H + yy) * W + xx) * cin + ch * 8);
    *reinterpret_cast<uint4*>(a_s + tap * a_bytes + core_off(m, ch * 8, cin)) = v;
  }
  for (int t = tid; t < 9 * cout * kc; t += kThreads) {
    const int tap = t / (cout * kc), rem = t - tap * cout * kc;
    const int n = rem / kc, ch = rem - n * kc;
    const uint4 v =
        *reinterpret_cast<const uint4*>(w + ((size_t)tap * cout + n) * cin + ch * 8);
    *reinterpret_cast<uint4*>(b_s + tap * b_bytes + core_off(n, ch * 8, cin)) = v;
  }
  // make the generic-proxy stores visible to the tensor core (async proxy)
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = taddr_slot;

  if (tid == 0) {
    const uint32_t idesc = idesc_bf16(cout);
    const uint32_t lbo = 128, sbo = (uint32_t)cin * 16;
    int first = 1;
    for (int tap = 0; tap < 9; tap++)
      for (int q = 0; q < cin / 16; q++) {
        const uint64_t ad = smem_desc(smem_u32(a_s + tap * a_bytes) + q * 256, lbo, sbo);
        const uint64_t bd = smem_desc(smem_u32(b_s + tap * b_bytes) + q * 256, lbo, sbo);
        const uint32_t acc = first ? 0u : 1u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(taddr),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        first = 0;
      }
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(&mbar))
        : "memory");
  }

  // Thread 0 waits for the MMAs (phase 0 of the barrier), for at most ~1 s;
  // the outcome is shared so that every warp takes the same branch.
  __shared__ uint32_t s_done;
  if (tid == 0) {
    uint32_t ok = 0;
    const long long t0 = clock64();
    while (!ok) {
      asm volatile(
          "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
          "selp.u32 %0, 1, 0, p;\n}"
          : "=r"(ok)
          : "r"(smem_u32(&mbar)), "r"(0u)
          : "memory");
      if (!ok && clock64() - t0 > kMaxWaitCycles) break;
    }
    if (!ok) atomicExch(err, 1);
    s_done = ok;
  }
  __syncthreads();
  const uint32_t done = s_done;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (done) {
    // Epilogue: warp w reads accumulator rows (pixels) 32w .. 32w+31.
    const int m = warp * 32 + lane;
    const size_t pix = ((size_t)img * H + row) * W + x0 + m;
    for (int n0 = 0; n0 < cout; n0 += 16) {
      uint32_t r[16];
      const uint32_t ta = taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)n0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
          "%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
            "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
            "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      __align__(16) __nv_bfloat16 out[16];
#pragma unroll
      for (int q = 0; q < 16; q++) {
        float v = __uint_as_float(r[q]) + (bias ? bias[n0 + q] : 0.f);
        if (relu) v = fmaxf(v, 0.f);
        out[q] = __float2bfloat16(v);
        if (y32) y32[pix * cout + n0 + q] = v;
      }
      if (y) {
        uint4* dst = reinterpret_cast<uint4*>(y + pix * cout + n0);
        dst[0] = reinterpret_cast<const uint4*>(out)[0];
        dst[1] = reinterpret_cast<const uint4*>(out)[1];
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
                 "r"(kTmemCols));
}

}  // namespace
}  // namespace emu
}  // namespace nl2d

using namespace nl2d::emu;

extern "C" {

// 3x3 convolution (stride 1, zero padding 1) of a batch of NHWC BF16
// images on the tensor cores.  cin, cout: multiples of 16, cout <= 64;
// W a multiple of 128.  y (BF16) and/or y32 (FP32) receive bias + conv,
// ReLU'd if relu.  err: device int set to 1 if a wait timed out.
int nl2d_emu_conv3x3(const void* x, const void* w, const float* bias, void* y, float* y32,
                     int batch, int H, int W, int cin, int cout, int relu, int* err,
                     void* stream) {
  if (cin % 16 || cout % 16 || cout > 64 || cin < 16 || cin > 64 || W % kTileM || H < 1 ||
      batch < 1 || !x || !w || !err || (!y && !y32))
    return NL2D_ERR_ARGS;
  const size_t smem = 9 * ((size_t)kTileM * cin * 2 + (size_t)cout * cin * 2);
  static int attr_bytes = 0;
  if ((int)smem > attr_bytes) {
    if (cudaFuncSetAttribute(k_conv3x3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return NL2D_ERR_CUDA;
    attr_bytes = (int)smem;
  }
  const dim3 grid((unsigned)(H * (W / kTileM)), (unsigned)batch);
  k_conv3x3_tc<<<grid, kThreads, smem, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)x, (const __nv_bfloat16*)w, bias, (__nv_bfloat16*)y, y32, H, W, cin,
      cout, relu, err);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

}  // extern "C"
