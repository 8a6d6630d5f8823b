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

// Pixels staged per image row: the 128 of the tile plus one on each side,
// rounded up to a multiple of 8 (one core-matrix column of pixels).
constexpr int kRowPix = 136;

// Persistent 3x3 convolution.  Each CTA keeps the 9 weight taps in shared
// memory and walks tiles (image, row, 128-pixel segment) with a grid
// stride.  For a tile it stages the three input rows it needs once, in a
// layout where pixels of one 8-channel group are 16 bytes apart, so the
// tap (dy, dx) operand is the dy-th row block started dx pixels (16 * dx
// bytes) later: no per-tap copies.
__global__ void __launch_bounds__(kThreads)
    k_conv3x3_tc(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ w,
                 const float* __restrict__ bias, __nv_bfloat16* __restrict__ y,
                 float* __restrict__ y32, int batch, int H, int W, int cin, int cout, int relu,
                 int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t taddr_slot;
  __shared__ uint32_t s_done;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kc = cin >> 3;                                   // 8-channel groups
  const uint32_t lbo_a = kRowPix * 16;                       // next channel group
  const uint32_t row_bytes = (uint32_t)kc * lbo_a;           // one staged row
  const uint32_t b_bytes = (uint32_t)cout * cin * 2;         // one weight tap
  unsigned char* b_s = smem;
  unsigned char* a_s = smem + ((9 * b_bytes + 1023) & ~1023u);

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
  for (int t = tid; t < 9 * cout * kc; t += kThreads) {
    const int tap = t / (cout * kc), rem = t - tap * cout * kc;
    const int n = rem / kc, ch = rem - n * kc;
    const uint4 v =
        *reinterpret_cast<const uint4*>(w + ((size_t)tap * cout + n) * cin + ch * 8);
    *reinterpret_cast<uint4*>(b_s + tap * b_bytes + core_off(n, ch * 8, cin)) = v;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = taddr_slot;
  const uint32_t idesc = idesc_bf16(cout);

  const int segs = W / kTileM;
  const long long ntiles = (long long)batch * H * segs;
  uint32_t phase = 0;
  bool ok_all = true;
  for (long long tile = blockIdx.x; tile < ntiles && ok_all; tile += gridDim.x) {
    const int seg = (int)(tile % segs);
    const long long rr = tile / segs;
    const int row = (int)(rr % H), img = (int)(rr / H);
    const int x0 = seg * kTileM;
    // stage rows row-1 .. row+1, pixels x0-1 .. x0-1+kRowPix-1 (zero outside)
    for (int t = tid; t < 3 * kc * kRowPix; t += kThreads) {
      const int p = t % kRowPix, rem = t / kRowPix;
      const int ch = rem % kc, dy = rem / kc;
      const int yy = row + dy - 1, xx = x0 - 1 + p;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (yy >= 0 && yy < H && xx >= 0 && xx < W)
        v = *reinterpret_cast<const uint4*>(x + (((size_t)img * H + yy) * W + xx) * cin +
                                            ch * 8);
      *reinterpret_cast<uint4*>(a_s + dy * row_bytes + ch * lbo_a + p * 16) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
      int first = 1;
      for (int tap = 0; tap < 9; tap++) {
        const int dy = tap / 3, dx = tap % 3;
        for (int q = 0; q < cin / 16; q++) {
          const uint64_t ad =
              smem_desc(smem_u32(a_s + dy * row_bytes) + 2 * q * lbo_a + dx * 16, lbo_a, 128);
          const uint64_t bd =
              smem_desc(smem_u32(b_s + tap * b_bytes) + q * 256, 128, (uint32_t)cin * 16);
          const uint32_t acc = first ? 0u : 1u;
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(taddr),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
          first = 0;
        }
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar))
          : "memory");
      // bounded wait (~1 s) for this tile's MMAs
      uint32_t ok = 0;
      const long long t0 = clock64();
      while (!ok) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(smem_u32(&mbar)), "r"(phase)
            : "memory");
        if (!ok && clock64() - t0 > kMaxWaitCycles) break;
      }
      if (!ok) atomicExch(err, 1);
      s_done = ok;
    }
    __syncthreads();
    phase ^= 1u;
    ok_all = s_done != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok_all) {
      // epilogue: warp w owns accumulator rows (pixels) 32w .. 32w+31
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
        float v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) {
          v[q] = __uint_as_float(r[q]) + (bias ? bias[n0 + q] : 0.f);
          if (relu) v[q] = fmaxf(v[q], 0.f);
          out[q] = __float2bfloat16(v[q]);
        }
        if (y) {
          uint4* dst = reinterpret_cast<uint4*>(y + pix * cout + n0);
          dst[0] = reinterpret_cast<const uint4*>(out)[0];
          dst[1] = reinterpret_cast<const uint4*>(out)[1];
        }
        if (y32) {
          float4* dst = reinterpret_cast<float4*>(y32 + pix * cout + n0);
#pragma unroll
          for (int q = 0; q < 4; q++)
            dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
      }
    }
    // the next tile overwrites the staged rows and the accumulator
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
                 "r"(kTmemCols));
}

// Tap-flipped, channel-transposed weights for the input gradient:
// wt[8 - tap][ci][co] = w[tap][co][ci].
__global__ void k_flip_transpose(const __nv_bfloat16* __restrict__ w,
                                 __nv_bfloat16* __restrict__ wt, int cout, int cin) {
  const int n = 9 * cout * cin;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int tap = t / (cout * cin), rem = t - tap * cout * cin;
    const int co = rem / cin, ci = rem - co * cin;
    wt[((size_t)(8 - tap) * cin + ci) * cout + co] = w[t];
  }
}

// Weight and bias gradients of a 3x3 convolution, FP32 on the CUDA cores:
// dw[tap][co][ci] += sum_p dy[p][co] * x[p + off(tap)][ci],
// db[co] += sum_p dy[p][co].  Block (tap, chunk of rows); each thread owns
// a fixed set of (co, ci) pairs; a row segment of dy and of the shifted x
// is staged in shared memory; results are added atomically.
constexpr int kWgThreads = 256, kWgPix = 64;
__global__ void __launch_bounds__(kWgThreads)
    k_conv_wgrad(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ dy,
                 float* __restrict__ dw, float* __restrict__ db, int B, int H, int W, int cin,
                 int cout, int rows_per_block) {
  __shared__ float sx[kWgPix][64 + 1];
  __shared__ float sd[kWgPix][64 + 1];
  const int tap = blockIdx.x, dyo = tap / 3 - 1, dxo = tap % 3 - 1;
  const int npairs = cout * cin;
  float acc[12];
#pragma unroll
  for (int q = 0; q < 12; q++) acc[q] = 0.f;
  float bacc = 0.f;
  const long long rows_total = (long long)B * H;
  const long long r0 = (long long)blockIdx.y * rows_per_block;
  for (long long rr = r0; rr < r0 + rows_per_block && rr < rows_total; rr++) {
    const int img = (int)(rr / H), row = (int)(rr - (long long)img * H);
    for (int xb = 0; xb < W; xb += kWgPix) {
      __syncthreads();
      for (int t = threadIdx.x; t < kWgPix * 64; t += kWgThreads) {
        const int p = t >> 6, c = t & 63;
        const int xx = xb + p;
        float vd = 0.f, vx = 0.f;
        if (c < cout) vd = __bfloat162float(dy[(((size_t)img * H + row) * W + xx) * cout + c]);
        const int ys = row + dyo, xs2 = xx + dxo;
        if (c < cin && ys >= 0 && ys < H && xs2 >= 0 && xs2 < W)
          vx = __bfloat162float(x[(((size_t)img * H + ys) * W + xs2) * cin + c]);
        sd[p][c] = vd;
        sx[p][c] = vx;
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 12; q++) {
        const int pair = threadIdx.x + q * kWgThreads;
        if (pair < npairs) {
          const int co = pair / cin, ci = pair - co * cin;
          float a = acc[q];
          for (int p = 0; p < kWgPix; p++) a = fmaf(sd[p][co], sx[p][ci], a);
          acc[q] = a;
        }
      }
      if (tap == 4 && threadIdx.x < cout)
        for (int p = 0; p < kWgPix; p++) bacc += sd[p][threadIdx.x];
    }
  }
#pragma unroll
  for (int q = 0; q < 12; q++) {
    const int pair = threadIdx.x + q * kWgThreads;
    if (pair < npairs) atomicAdd(&dw[(size_t)tap * npairs + pair], acc[q]);
  }
  if (tap == 4 && threadIdx.x < cout) atomicAdd(&db[threadIdx.x], bacc);
}

// dx = (y > 0) ? g : 0 for a ReLU output y (BF16), g FP32 -> BF16.
__global__ void k_relu_bwd(const float* __restrict__ g, const __nv_bfloat16* __restrict__ y,
                           __nv_bfloat16* __restrict__ out, long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    out[t] = __float2bfloat16(__bfloat162float(y[t]) > 0.f ? g[t] : 0.f);
}

// Mean-squared error of the first `nc` of `cpad` predicted channels against
// an FP32 target [p][nc]; grad (BF16, [p][cpad], zero in padded channels)
// = 2 (pred - target) / (P * nc); loss accumulated into *loss.
__global__ void k_mse(const float* __restrict__ pred, const float* __restrict__ target,
                      __nv_bfloat16* __restrict__ grad, float* __restrict__ loss, long long P,
                      int nc, int cpad) {
  __shared__ float red[8];
  float acc = 0.f;
  const float scale = 2.f / (float)(P * nc);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < P * cpad;
       t += (long long)gridDim.x * blockDim.x) {
    const long long p = t / cpad;
    const int c = (int)(t - p * cpad);
    float gv = 0.f;
    if (c < nc) {
      const float d = pred[t] - target[p * nc + c];
      acc += d * d;
      gv = scale * d;
    }
    grad[t] = __float2bfloat16(gv);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += red[k];
    atomicAdd(loss, s / (float)(P * nc));
  }
}

// Adam on FP32 master weights; also writes the BF16 copy the convolution
// reads (bias: w16 == nullptr).
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, __nv_bfloat16* __restrict__ w16, int n,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.f - b1) * gt;
    const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    const float wt = w[t] - lr * (mt / c1) / (sqrtf(vt / c2) + eps);
    w[t] = wt;
    if (w16) w16[t] = __float2bfloat16(wt);
  }
}

// Network input and target for a batch of snapshot pairs.  snaps:
// [nsnap_total][H][W][3] FP32 states; statics: [ndom][H][W][2] (depth / 500,
// open-boundary indicator); forcing: [batch] tidal ssh at the target time.
// x (BF16 [b][H][W][cpad]): state / scale, depth, forcing * indicator, 0.
// target (FP32 [b][H][W][3], may be NULL): (next - state) / inc_scale.
__global__ void k_assemble(const float* __restrict__ snaps, const float* __restrict__ statics,
                           const int* __restrict__ src, const int* __restrict__ dom,
                           const float* __restrict__ forcing, float3 scale, float3 inc_scale,
                           __nv_bfloat16* __restrict__ x, float* __restrict__ target, int HW,
                           int cpad, int batch) {
  const long long n = (long long)batch * HW;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / HW), p = (int)(t - (long long)b * HW);
    const float* s0 = snaps + ((size_t)src[b] * HW + p) * 3;
    const float* st = statics + ((size_t)dom[b] * HW + p) * 2;
    __nv_bfloat16* xo = x + (size_t)t * cpad;
    xo[0] = __float2bfloat16(s0[0] / scale.x);
    xo[1] = __float2bfloat16(s0[1] / scale.y);
    xo[2] = __float2bfloat16(s0[2] / scale.z);
    xo[3] = __float2bfloat16(st[0]);
    xo[4] = __float2bfloat16(forcing[b] * st[1] / scale.x);
    for (int c = 5; c < cpad; c++) xo[c] = __float2bfloat16(0.f);
    if (target) {
      const float* s1 = s0 + (size_t)HW * 3;  // the next snapshot of the same domain
      float* to = target + (size_t)t * 3;
      to[0] = (s1[0] - s0[0]) / inc_scale.x;
      to[1] = (s1[1] - s0[1]) / inc_scale.y;
      to[2] = (s1[2] - s0[2]) / inc_scale.z;
    }
  }
}

// state += increment (first 3 of cpad FP32 output channels) * inc_scale.
__global__ void k_advance(float* __restrict__ state, const float* __restrict__ inc,
                          float3 inc_scale, long long P, int cpad) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < P;
       t += (long long)gridDim.x * blockDim.x) {
    state[t * 3 + 0] += inc[t * cpad + 0] * inc_scale.x;
    state[t * 3 + 1] += inc[t * cpad + 1] * inc_scale.y;
    state[t * 3 + 2] += inc[t * cpad + 2] * inc_scale.z;
  }
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
  const size_t wbytes = ((9 * (size_t)cout * cin * 2) + 1023) & ~(size_t)1023;
  const size_t smem = wbytes + 3 * (size_t)(cin / 8) * kRowPix * 16;
  static int attr_bytes = 0;
  if ((int)smem > attr_bytes) {
    if (cudaFuncSetAttribute(k_conv3x3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             96 * 1024) != cudaSuccess)
      return NL2D_ERR_CUDA;
    attr_bytes = 96 * 1024;
  }
  if (smem > 96 * 1024) return NL2D_ERR_ARGS;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long tiles = (long long)batch * H * (W / kTileM);
  const int grid = (int)(tiles < 2LL * sms ? tiles : 2LL * sms);  // two CTAs per SM
  k_conv3x3_tc<<<grid, kThreads, smem, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)x, (const __nv_bfloat16*)w, bias, (__nv_bfloat16*)y, y32, batch, H,
      W, cin, cout, relu, err);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_flip_transpose(const void* w, void* wt, int cout, int cin, void* stream) {
  if (!w || !wt || cout < 1 || cin < 1) return NL2D_ERR_ARGS;
  k_flip_transpose<<<64, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)w,
                                                          (__nv_bfloat16*)wt, cout, cin);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_conv_wgrad(const void* x, const void* dy, float* dw, float* db, int batch, int H,
                        int W, int cin, int cout, void* stream) {
  if (!x || !dy || !dw || !db || cin > 64 || cout > 64 || cin * cout > 12 * kWgThreads ||
      W % kWgPix)
    return NL2D_ERR_ARGS;
  const int rows = batch * H, rows_per_block = 8;
  const dim3 grid(9, (rows + rows_per_block - 1) / rows_per_block);
  k_conv_wgrad<<<grid, kWgThreads, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)x, (const __nv_bfloat16*)dy, dw, db, batch, H, W, cin, cout,
      rows_per_block);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_relu_bwd(const float* g, const void* y, void* out, long long n, void* stream) {
  k_relu_bwd<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(g, (const __nv_bfloat16*)y,
                                                         (__nv_bfloat16*)out, n);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_mse(const float* pred, const float* target, void* grad, float* loss, long long P,
                 int nc, int cpad, void* stream) {
  k_mse<<<152 * 4, 256, 0, (cudaStream_t)stream>>>(pred, target, (__nv_bfloat16*)grad, loss, P,
                                                    nc, cpad);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_adam(float* w, float* m, float* v, const float* g, void* w16, int n, float lr,
                  float b1, float b2, float eps, int step, void* stream) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<64, 256, 0, (cudaStream_t)stream>>>(w, m, v, g, (__nv_bfloat16*)w16, n, lr, b1, b2,
                                                eps, c1, c2);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_assemble(const float* snaps, const float* statics, const int* src,
                      const int* dom, const float* forcing, const float* scale6, void* x,
                      float* target, int HW, int cpad, int batch, void* stream) {
  if (!snaps || !statics || !src || !dom || !forcing || !scale6 || !x || cpad < 5)
    return NL2D_ERR_ARGS;
  k_assemble<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(
      snaps, statics, src, dom, forcing, make_float3(scale6[0], scale6[1], scale6[2]),
      make_float3(scale6[3], scale6[4], scale6[5]), (__nv_bfloat16*)x, target, HW, cpad, batch);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_advance(float* state, const float* inc, const float* inc_scale3, long long P,
                     int cpad, void* stream) {
  k_advance<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(
      state, inc, make_float3(inc_scale3[0], inc_scale3[1], inc_scale3[2]), P, cpad);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

}  // extern "C"
