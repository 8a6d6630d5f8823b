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
#include <algorithm>
#include <cstdint>

#include "../../include/nl2d_gpu.h"

namespace nl2d {
namespace emu {
namespace {

constexpr int kTileM = 128;       // pixels per CTA (one row segment)
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

// ---- 3x3 convolution ------------------------------------------------------
//
// Implicit GEMM on the tensor cores: M = 128 pixels of one image row,
// N = cout, K = 9 taps x cin.  The 9 weight taps stay in shared memory for
// the CTA's lifetime.  A staged input row keeps each 8-channel group of its
// pixels 16 bytes apart, so the operand of tap (dy, dx) is the dy-th row of
// the window started dx pixels (16 * dx bytes) later: a descriptor offset,
// no per-tap copies.  Warp-specialised and persistent: a CTA walks strips
// of kStripRows output rows of one 128-pixel column segment.  Input rows pass
// through a ring of kSlots shared-memory slots (each input row is staged
// once per strip instead of three times), the accumulator alternates
// between two TMEM buffers, and the three roles overlap:
//   warps 0-3  epilogue: TMEM -> bias, ReLU -> BF16 / FP32 stores
//   warp 4     one thread issues the MMAs of an output row once its three
//              input rows are staged and its TMEM buffer is free
//   warps 5-7  stage input rows into the ring
// Hand-offs are mbarriers: full[slot] (stagers -> MMA), empty[slot] (MMA
// completion -> stagers), done[buf] (MMA completion -> epilogue),
// drained[buf] (epilogue -> MMA).  Every wait is bounded (kMaxWaitCycles);
// one that runs out sets the error flag and a shared abort flag that ends
// every role's loop, and the MMA thread waits for its last commit before the
// tensor memory is freed.
constexpr int kStripRows = 8;
constexpr int kSlots = 4;      // the weight gradient's X ring
constexpr int kConvSlots = 5;  // the convolution's input ring: 3 rows read, 2 in flight
constexpr int kPipeThreads = 256;
constexpr int kEpiWarps = 4;
constexpr int kStageThreads = 96;  // warps 5-7
// 16-byte loads per staging thread per row: 8 channel groups x 136 pixels
// (cin = 64, the widest) fit in 96 x 12
constexpr int kStageBatch = 12;
static_assert(8 * kRowPix <= kStageThreads * kStageBatch, "a staged row must fit one batch");
constexpr int kPipeTmemCols = 128;  // two accumulators of up to 64 columns

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
// Waits for the phase with the given parity to complete; false if the wait
// ran out after max_cycles (flag and error set) or another role aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          volatile int* abort_flag, int* err,
                                          long long max_cycles = kMaxWaitCycles) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
    if (*abort_flag) return false;
    if (clock64() - t0 > max_cycles) {
      *abort_flag = 1;
      atomicExch(err, 1);
      return false;
    }
  }
}

// The failure path of the bounded waits, exercised on purpose: one thread
// waits on a barrier that nothing arrives on, gives up after max_cycles,
// sets the error flag and returns (err = 2 would mean the phase completed).
__global__ void k_selftest_wait(long long max_cycles, int* err) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  __syncthreads();
  if (threadIdx.x == 0 && mbar_wait(&bar, 0, &abort_flag, err, max_cycles)) atomicExch(err, 2);
}

struct StripWalk {  // work unit u -> (image, first row, rows, column segment)
  int img, y0, rows, x0;
  __device__ StripWalk(long long u, int H, int segs) {
    const int strips = (H + kStripRows - 1) / kStripRows;
    const int seg = (int)(u % segs);
    const long long r = u / segs;
    const int st = (int)(r % strips);
    img = (int)(r / strips);
    y0 = st * kStripRows;
    rows = min(kStripRows, H - y0);
    x0 = seg * kTileM;
  }
};

__global__ void __launch_bounds__(kPipeThreads)
    k_conv3x3_pipe(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ w,
                   const float* __restrict__ bias, __nv_bfloat16* __restrict__ y,
                   float* __restrict__ y32, int batch, int H, int W, int cin, int cout,
                   int relu, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full_bar[kConvSlots], empty_bar[kConvSlots];
  __shared__ __align__(8) uint64_t done_bar[2], drained_bar[2], last_bar;
  __shared__ uint32_t taddr_slot;
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kc = cin >> 3;
  const uint32_t lbo_a = kRowPix * 16;
  const uint32_t row_bytes = (uint32_t)kc * lbo_a;
  const uint32_t b_bytes = (uint32_t)cout * cin * 2;
  unsigned char* b_s = smem;
  unsigned char* ring = smem + ((9 * b_bytes + 1023) & ~1023u);
  volatile int* abort_v = &abort_flag;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&taddr_slot)),
                 "r"(kPipeTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int q = 0; q < kConvSlots; q++) {
      mbar_init(&full_bar[q], kStageThreads);
      mbar_init(&empty_bar[q], 1);
    }
    for (int q = 0; q < 2; q++) {
      mbar_init(&done_bar[q], 1);
      mbar_init(&drained_bar[q], kEpiWarps * 32);
    }
    mbar_init(&last_bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  for (int t = tid; t < 9 * cout * kc; t += kPipeThreads) {
    const int tap = t / (cout * kc), rem = t - tap * cout * kc;
    const int n = rem / kc, ch = rem - n * kc;
    const uint4 v =
        *reinterpret_cast<const uint4*>(w + ((size_t)tap * cout + n) * cin + ch * 8);
    *reinterpret_cast<uint4*>(b_s + tap * b_bytes + core_off(n, ch * 8, cin)) = v;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = taddr_slot;
  const int segs = W / kTileM;
  const long long units = (long long)batch * ((H + kStripRows - 1) / kStripRows) * segs;

  if (warp >= 5) {
    // ---- stagers: input rows y0-1 .. y0+rows of every strip, in order.
    // cp.async copies each 16-byte group of 8 channels straight into its
    // ring slot (zero-filled outside the image), so a stager does not hold
    // a row in registers: it starts row q, then waits for its own copies of
    // row q-1, makes them visible to the tensor core's (async) proxy and
    // marks that slot full.  Two rows are in flight per CTA (the ring's
    // other three slots hold the rows the MMAs read), where register
    // staging kept one.
    const int st = tid - 5 * 32;
    long long q = 0;      // input rows started so far (ring sequence)
    bool pending = false;  // row q-1 started, its slot not yet marked full
    for (long long u = blockIdx.x; u < units && !*abort_v; u += gridDim.x) {
      const StripWalk sw(u, H, segs);
      for (int a = 0; a < sw.rows + 2 && !*abort_v; a++, q++) {
        const int slot = (int)(q % kConvSlots);
        const int yy = sw.y0 - 1 + a;
        if (q >= kConvSlots &&
            !mbar_wait(&empty_bar[slot], (uint32_t)((q / kConvSlots - 1) & 1), abort_v, err))
          break;
        const uint32_t dst = smem_u32(ring + slot * row_bytes);
        for (int t = st; t < kc * kRowPix; t += kStageThreads) {
          const int p = t % kRowPix, ch = t / kRowPix;
          const int xx = sw.x0 - 1 + p;
          const bool in = yy >= 0 && yy < H && xx >= 0 && xx < W;
          const __nv_bfloat16* src =
              in ? x + (((size_t)sw.img * H + yy) * W + xx) * cin + ch * 8 : x;
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                           dst + (uint32_t)(ch * lbo_a + p * 16)),
                       "l"(src), "r"(in ? 16 : 0)
                       : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        if (pending) {  // row q-1 has landed once at most one group is open
          asm volatile("cp.async.wait_group 1;" ::: "memory");
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          mbar_arrive(&full_bar[(q - 1) % kConvSlots]);
        }
        pending = true;
      }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    if (pending && !*abort_v) {  // the last row started
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&full_bar[(q - 1) % kConvSlots]);
    }
  } else if (warp == 4) {
    // ---- MMA issuer ----
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16(cout);
      const uint64_t b_desc0 = smem_desc(smem_u32(b_s), 128, (uint32_t)cin * 16);
      const uint32_t a_kstep = (2 * lbo_a) >> 4;
      const int kcq = cin / 16;
      long long q = 0, p = 0;  // input rows consumed (sequence base), output rows issued
      bool issued = false;
      for (long long u = blockIdx.x; u < units && !*abort_v; u += gridDim.x) {
        const StripWalk sw(u, H, segs);
        const long long qb = q;  // sequence number of this strip's first input row
        // its first two input rows
        bool ok = mbar_wait(&full_bar[qb % kConvSlots], (uint32_t)((qb / kConvSlots) & 1),
                            abort_v, err) &&
                  mbar_wait(&full_bar[(qb + 1) % kConvSlots],
                            (uint32_t)(((qb + 1) / kConvSlots) & 1), abort_v, err);
        for (int o = 0; o < sw.rows && ok; o++, p++) {
          const long long qn = qb + o + 2;  // the new input row this output needs
          const int buf = (int)(p & 1);
          ok = mbar_wait(&full_bar[qn % kConvSlots], (uint32_t)((qn / kConvSlots) & 1), abort_v,
                         err);
          if (ok && p >= 2)
            ok = mbar_wait(&drained_bar[buf], (uint32_t)((p / 2 - 1) & 1), abort_v, err);
          if (!ok) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t dcol = taddr + (uint32_t)(buf * 64);
          // Operand descriptors: built once per input row and for tap 0, then
          // advanced by adding byte offsets / 16 to their address field
          // (shared addresses stay below 256 KB, so the field never carries
          // into the others): + dx for the tap's pixel shift, + 2 lbo / 16
          // per A K-step, + 256 / 16 per B K-step, + b_bytes / 16 per tap.
          uint64_t arow[3];
#pragma unroll
          for (int dy = 0; dy < 3; dy++)
            arow[dy] = smem_desc(smem_u32(ring + (int)((qb + o + dy) % kConvSlots) * row_bytes),
                                 lbo_a, 128);
          uint64_t btap = b_desc0;
          uint32_t acc = 0u;
#pragma unroll
          for (int tap = 0; tap < 9; tap++, btap += b_bytes >> 4) {
            uint64_t ad = arow[tap / 3] + (uint64_t)(tap % 3), bd = btap;
            for (int kq = 0; kq < kcq; kq++, ad += a_kstep, bd += 256 >> 4) {
              asm volatile(
                  "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dcol),
                  "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
              acc = 1u;
            }
          }
          issued = true;
          tc_commit(&done_bar[buf]);
          // input row o is not read by later outputs of this strip
          tc_commit(&empty_bar[(qb + o) % kConvSlots]);
        }
        q = qb + sw.rows + 2;
        if (ok) {  // the strip's last two input rows are free too
          tc_commit(&empty_bar[(q - 2) % kConvSlots]);
          tc_commit(&empty_bar[(q - 1) % kConvSlots]);
        } else {
          break;
        }
      }
      if (issued) {  // nothing may be in flight when the tensor memory is freed
        tc_commit(&last_bar);
        volatile int never = 0;
        if (!mbar_wait(&last_bar, 0, &never, err)) atomicExch(err, 1);
      }
    }
  } else {
    // ---- epilogue: warp w owns accumulator lanes (pixels) 32w .. 32w+31 ----
    long long p = 0;
    for (long long u = blockIdx.x; u < units && !*abort_v; u += gridDim.x) {
      const StripWalk sw(u, H, segs);
      for (int o = 0; o < sw.rows; o++, p++) {
        const int buf = (int)(p & 1);
        // warp-uniform outcome: tcgen05.ld below needs the whole warp
        const bool ok = mbar_wait(&done_bar[buf], (uint32_t)((p / 2) & 1), abort_v, err);
        if (!__all_sync(0xffffffffu, ok)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int m = warp * 32 + lane;
        const size_t pix = ((size_t)sw.img * H + sw.y0 + o) * W + sw.x0 + m;
        for (int n0 = 0; n0 < cout; n0 += 16) {
          uint32_t r[16];
          const uint32_t ta =
              taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(buf * 64 + n0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
              "%12,%13,%14,%15}, [%16];"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
              : "r"(ta));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          __align__(16) __nv_bfloat16 out[16];
          float v[16];
#pragma unroll
          for (int k = 0; k < 16; k++) {
            v[k] = __uint_as_float(r[k]) + (bias ? bias[n0 + k] : 0.f);
            if (relu) v[k] = fmaxf(v[k], 0.f);
            out[k] = __float2bfloat16(v[k]);
          }
          if (y) {
            uint4* dst = reinterpret_cast<uint4*>(y + pix * cout + n0);
            dst[0] = reinterpret_cast<const uint4*>(out)[0];
            dst[1] = reinterpret_cast<const uint4*>(out)[1];
          }
          if (y32) {
            float4* dst = reinterpret_cast<float4*>(y32 + pix * cout + n0);
#pragma unroll
            for (int k = 0; k < 4; k++)
              dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(&drained_bar[buf]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
                 "r"(kPipeTmemCols));
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

// Weight gradient on the tensor cores.  For each tap it is a GEMM over
// pixels, D[co][ci] = sum_p dY[p][co] X[p + off][ci], with both operands
// "MN-major" (channels contiguous per pixel, as the data already is):
// M = co (padded to 128 with zero rows), N = ci, K = pixels.  X is staged as
// in the convolution, so the tap (dy, dx) operand is again a row block
// started 16 * dx bytes later.  The nine accumulators (9 x ci FP32 columns)
// stay in tensor memory for the CTA's lifetime; at the end each CTA writes
// its partial sums to its own slot of `part`, and k_sum_parts adds the
// slots in CTA order, so that the gradient has the same bits on every run
// (atomic additions would sum in whatever order the CTAs finished).
constexpr int kWgTmemCols = 512;
constexpr int kWgGroups = 16;  // 128 M rows = 16 groups of 8 output channels
constexpr size_t kWgSmem = 120 * 1024;

__host__ __device__ constexpr uint32_t idesc_bf16_mn(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
         ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
}

// Laid out like the convolution: a CTA (alone on its SM: it holds all 512
// TMEM columns) walks strips of kStripRows rows of one 128-pixel segment:
//   warps 5-7  stage input rows (X) into a ring of kSlots slots
//   warps 0-3  stage gradient rows (dY) into a ring of 2 slots, then, at
//              the end, move the nine accumulators out of TMEM into dw
//   warp 4     one thread issues, per row, the 9 taps x 8 pixel chunks of
//              MMAs into the accumulators, which stay in TMEM throughout
// The bias gradient is a separate reduction (k_bias_grad).
constexpr int kWgYSlots = 2;
constexpr int kWgYThreads = 128;   // warps 0-3
constexpr int kWgYBatch = 16;      // 16-byte loads per thread per dY row (cout <= 128)

__global__ void __launch_bounds__(kPipeThreads)
    k_conv_wgrad_pipe(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ dy,
                      float* __restrict__ part, int batch, int H, int W, int cin, int cout,
                      int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t xfull[kSlots], xempty[kSlots];
  __shared__ __align__(8) uint64_t yfull[kWgYSlots], yempty[kWgYSlots], last_bar;
  __shared__ uint32_t taddr_slot;
  __shared__ int abort_flag, s_issued;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kc = cin >> 3, kco = cout >> 3;
  const uint32_t lbo_y = kTileM * 16;  // next group of 8 output channels (M)
  const uint32_t lbo_x = kRowPix * 16; // next group of 8 input channels (N)
  const uint32_t row_bytes = (uint32_t)kc * lbo_x;
  const uint32_t yslot_bytes = (uint32_t)kWgGroups * lbo_y;
  unsigned char* yring = smem;                               // kWgYSlots x 32 KB
  unsigned char* xring = smem + kWgYSlots * yslot_bytes;     // kSlots staged X rows
  volatile int* abort_v = &abort_flag;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&taddr_slot)),
                 "r"(kWgTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int q = 0; q < kSlots; q++) {
      mbar_init(&xfull[q], kStageThreads);
      mbar_init(&xempty[q], 1);
    }
    for (int q = 0; q < kWgYSlots; q++) {
      mbar_init(&yfull[q], kWgYThreads);
      mbar_init(&yempty[q], 1);
    }
    mbar_init(&last_bar, 1);
    abort_flag = 0;
    s_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  // rows co >= cout of the M = 128 operand stay zero in both dY slots
  for (int t = tid; t < kWgYSlots * kWgGroups * kTileM; t += kPipeThreads)
    *reinterpret_cast<uint4*>(yring + t * 16) = make_uint4(0, 0, 0, 0);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = taddr_slot;
  const int segs = W / kTileM;
  const long long units = (long long)batch * ((H + kStripRows - 1) / kStripRows) * segs;

  if (warp >= 5) {
    // ---- X stagers: input rows y0-1 .. y0+rows of every strip ----
    const int st = tid - 5 * 32;
    long long q = 0;
    for (long long u = blockIdx.x; u < units && !*abort_v; u += gridDim.x) {
      const StripWalk sw(u, H, segs);
      for (int a = 0; a < sw.rows + 2 && !*abort_v; a++, q++) {
        const int slot = (int)(q % kSlots);
        const int yy = sw.y0 - 1 + a;
        uint4 v[kStageBatch];
#pragma unroll
        for (int b = 0; b < kStageBatch; b++) {
          const int t = st + b * kStageThreads;
          v[b] = make_uint4(0, 0, 0, 0);
          if (t < kc * kRowPix) {
            const int p = t % kRowPix, ch = t / kRowPix;
            const int xx = sw.x0 - 1 + p;
            if (yy >= 0 && yy < H && xx >= 0 && xx < W)
              v[b] = *reinterpret_cast<const uint4*>(
                  x + (((size_t)sw.img * H + yy) * W + xx) * cin + ch * 8);
          }
        }
        if (q >= kSlots &&
            !mbar_wait(&xempty[slot], (uint32_t)((q / kSlots - 1) & 1), abort_v, err))
          break;
        unsigned char* dst = xring + slot * row_bytes;
#pragma unroll
        for (int b = 0; b < kStageBatch; b++) {
          const int t = st + b * kStageThreads;
          if (t < kc * kRowPix) {
            const int p = t % kRowPix, ch = t / kRowPix;
            *reinterpret_cast<uint4*>(dst + ch * lbo_x + p * 16) = v[b];
          }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&xfull[slot]);
      }
    }
  } else if (warp == 4) {
    // ---- MMA issuer ----
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_mn(cin);
      long long q = 0, p = 0;
      bool issued = false, ok = true;
      for (long long u = blockIdx.x; u < units && ok && !*abort_v; u += gridDim.x) {
        const StripWalk sw(u, H, segs);
        const long long qb = q;
        ok = mbar_wait(&xfull[qb % kSlots], (uint32_t)((qb / kSlots) & 1), abort_v, err) &&
             mbar_wait(&xfull[(qb + 1) % kSlots], (uint32_t)(((qb + 1) / kSlots) & 1),
                       abort_v, err);
        for (int o = 0; o < sw.rows && ok; o++, p++) {
          const long long qn = qb + o + 2;
          const int ys = (int)(p % kWgYSlots);
          ok = mbar_wait(&xfull[qn % kSlots], (uint32_t)((qn / kSlots) & 1), abort_v, err) &&
               mbar_wait(&yfull[ys], (uint32_t)((p / kWgYSlots) & 1), abort_v, err);
          if (!ok) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          // MN-major, no swizzle: LBO steps along K (8 pixels = 128 B), SBO
          // along M / N (the next 8 channels).  Descriptors built once per
          // row and advanced by adding byte offsets / 16 to their address
          // field (shared addresses stay below 256 KB): + 256 / 16 per
          // K-step, + dx for the tap's pixel shift.
          const uint64_t yrow = smem_desc(smem_u32(yring + ys * yslot_bytes), 128, lbo_y);
          uint64_t xrow[3];
#pragma unroll
          for (int dyr = 0; dyr < 3; dyr++)
            xrow[dyr] = smem_desc(smem_u32(xring + (int)((qb + o + dyr) % kSlots) * row_bytes),
                                  128, lbo_x);
#pragma unroll
          for (int tap = 0; tap < 9; tap++) {
            uint64_t ad = yrow, bd = xrow[tap / 3] + (uint64_t)(tap % 3);
#pragma unroll
            for (int kq = 0; kq < kTileM / 16; kq++, ad += 256 >> 4, bd += 256 >> 4) {
              const uint32_t acc = (issued || kq > 0) ? 1u : 0u;
              asm volatile(
                  "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                      taddr + (uint32_t)(tap * cin)),
                  "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
          }
          issued = true;
          tc_commit(&yempty[ys]);
          tc_commit(&xempty[(qb + o) % kSlots]);
        }
        q = qb + sw.rows + 2;
        if (ok) {
          tc_commit(&xempty[(q - 2) % kSlots]);
          tc_commit(&xempty[(q - 1) % kSlots]);
        }
      }
      s_issued = (issued && ok) ? 1 : 0;
      __threadfence_block();
      if (issued)
        tc_commit(&last_bar);  // arrives once every MMA above has completed
      else
        mbar_arrive(&last_bar);
    }
  } else {
    // ---- dY stagers, then the epilogue ----
    long long p = 0;
    for (long long u = blockIdx.x; u < units && !*abort_v; u += gridDim.x) {
      const StripWalk sw(u, H, segs);
      for (int o = 0; o < sw.rows && !*abort_v; o++, p++) {
        const int ys = (int)(p % kWgYSlots);
        const size_t pix0 = ((size_t)sw.img * H + sw.y0 + o) * W + sw.x0;
        uint4 v[kWgYBatch];
#pragma unroll
        for (int b = 0; b < kWgYBatch; b++) {
          const int t = tid + b * kWgYThreads;  // pixel t % 128, group t / 128
          if (t < kco * kTileM)
            v[b] = *reinterpret_cast<const uint4*>(dy + (pix0 + (t % kTileM)) * cout +
                                                   (t / kTileM) * 8);
        }
        if (p >= kWgYSlots &&
            !mbar_wait(&yempty[ys], (uint32_t)((p / kWgYSlots - 1) & 1), abort_v, err))
          break;
        unsigned char* dst = yring + ys * yslot_bytes;
#pragma unroll
        for (int b = 0; b < kWgYBatch; b++) {
          const int t = tid + b * kWgYThreads;
          if (t < kco * kTileM)
            *reinterpret_cast<uint4*>(dst + (t / kTileM) * lbo_y + (t % kTileM) * 16) = v[b];
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&yfull[ys]);
      }
    }
    // the accumulators: row co (lanes 32w .. 32w+31), 9 x cin columns
    volatile int never = 0;
    const bool done = mbar_wait(&last_bar, 0, &never, err);
    if (__all_sync(0xffffffffu, done) && s_issued && !*abort_v) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int co = warp * 32 + lane;
      for (int c0 = 0; c0 < 9 * cin; c0 += 16) {
        uint32_t r[16];
        const uint32_t ta = taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
            "%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
              "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
              "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(ta));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (co < cout) {
          const int tap = c0 / cin, ci0 = c0 - tap * cin;
          float* mine = part + (size_t)blockIdx.x * 9 * cout * cin;
#pragma unroll
          for (int k = 0; k < 16; k++)
            mine[((size_t)tap * cout + co) * cin + ci0 + k] = __uint_as_float(r[k]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
                 "r"(kWgTmemCols));
}

// Block b's partial bias gradient, part[b][co] = sum over its pixels of
// dy[p][co], in a fixed order (each thread a channel pair over a fixed set
// of rows, then the block's rows in order); k_sum_parts adds the blocks.
__global__ void __launch_bounds__(256)
    k_bias_grad(const __nv_bfloat16* __restrict__ dy, float* __restrict__ part, long long P,
                int cout) {
  __shared__ float sp[256 * 2];
  // thread -> one channel pair, rows strided over the grid
  const int pairs = cout >> 1;
  const int lanes_per_row = pairs;  // <= 64
  const int rows_per_block = blockDim.x / lanes_per_row;
  const int c2 = threadIdx.x % lanes_per_row, r0 = threadIdx.x / lanes_per_row;
  if (r0 < rows_per_block) {
    float s0 = 0.f, s1 = 0.f;
    for (long long pix = (long long)blockIdx.x * rows_per_block + r0; pix < P;
         pix += (long long)gridDim.x * rows_per_block) {
      const __nv_bfloat162 v = reinterpret_cast<const __nv_bfloat162*>(dy + pix * cout)[c2];
      s0 += __low2float(v);
      s1 += __high2float(v);
    }
    sp[r0 * cout + 2 * c2] = s0;
    sp[r0 * cout + 2 * c2 + 1] = s1;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < cout; c += blockDim.x) {
    float acc = 0.f;
    for (int r = 0; r < rows_per_block; r++) acc += sp[r * cout + c];
    part[(size_t)blockIdx.x * cout + c] = acc;
  }
}

// out[e] += part[0][e] + part[1][e] + ... in that order.
__global__ void k_sum_parts(const float* __restrict__ part, int nparts, long long nel,
                            float* __restrict__ out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel;
       e += (long long)gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int b = 0; b < nparts; b++) acc += part[(size_t)b * nel + e];
    out[e] += acc;
  }
}

// Scratch for the per-CTA partial gradients (grown on demand, kept).
float* g_parts = nullptr;
size_t g_parts_cap = 0;
bool ensure_parts(size_t n) {
  if (n <= g_parts_cap) return true;
  cudaFree(g_parts);
  g_parts = nullptr;
  g_parts_cap = 0;
  if (cudaMalloc(&g_parts, n * sizeof(float)) != cudaSuccess) return false;
  g_parts_cap = n;
  return true;
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
                      const float* __restrict__ weight, __nv_bfloat16* __restrict__ grad,
                      float* __restrict__ loss, long long P, int nc, int cpad) {
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
      const float w = weight ? weight[p] : 1.f;
      acc += w * d * d;
      gv = scale * w * d;
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

// Zero-mean, unit-variance noise that depends only on (seed, key): the sum
// of four uniforms from a 64-bit mix (splitmix64 finaliser), rescaled.
__device__ __forceinline__ float hash_noise(unsigned long long seed, unsigned long long key) {
  unsigned long long z = seed ^ (key * 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  float sum = 0.f;
#pragma unroll
  for (int q = 0; q < 4; q++) sum += (float)((z >> (16 * q)) & 0xFFFF) * (1.f / 65536.f);
  return (sum - 2.f) * 1.7320508f;  // variance of the sum is 4/12
}

// Per-pixel statics of a domain: depth (ht / 500 m), open-boundary
// indicator (1 on wet cells next to the open side), and 1 where the pixel's
// east (u) or north (v) face is a wall.
constexpr int kStatics = 4;

// Network inputs of `batch` domain states (each an H x W image of
// (ssh, u, v), u / v on the east / north face of the pixel's cell):
//   0-2  ssh - tidal ssh at the target time, u, v / state scales (ssh as a
//        departure from the tide keeps BF16's resolution where the level
//        follows the tide, next to the open side)
//   3    depth (ht / 500 m)
//   4    tidal ssh at the target time on cells next to the open side
//   5    ssh(i+1, j) - ssh(i, j)      (east-face pressure gradient)
//   6    ssh(i, j+1) - ssh(i, j)      (north-face pressure gradient)
//   7    sum of face depth x velocity out of the cell (flux divergence)
//   8    open-boundary indicator
//   9    ssh - tidal ssh on cells next to the open side (what the Flather
//        condition radiates out)
//   10, 11  east / north face is a wall
//   12-14   low BF16 parts of channels 0-2 (value - BF16(value)): next to
//        the open side the state is 20-50x its k-step change, so one BF16
//        (8-bit mantissa) would leave a few per cent of noise in what the
//        network predicts; high + low carry 16 bits
// Channels 5-7 and 9 are differences of nearly equal numbers, so they are
// formed in FP32 before the BF16 rounding; the scales of 5-7 come from the
// data.  A face outside the image (the closed or open boundary) contributes
// zero.
// With noise (training only) the input state is the snapshot plus white
// noise of the given standard deviations, the same value wherever a cell is
// read, and the target is the increment from that perturbed state.
struct Noisy {
  const float* img;
  float3 sd;
  unsigned long long seed, base;
  __device__ float get(int q, int ch) const {
    float v = img[(size_t)q * 3 + ch];
    const float s = ch == 0 ? sd.x : (ch == 1 ? sd.y : sd.z);
    if (s != 0.f) v += s * hash_noise(seed, (base + (unsigned long long)q) * 3ull + ch);
    return v;
  }
};

__global__ void k_assemble(const float* __restrict__ snaps, const float* __restrict__ statics,
                           const int* __restrict__ src, const int* __restrict__ dom,
                           const float* __restrict__ forcing, float3 scale, float3 inc_scale,
                           float3 dscale, float3 noise, unsigned long long seed,
                           __nv_bfloat16* __restrict__ x, float* __restrict__ target, int H,
                           int W, int cpad, int batch) {
  const long long HW = (long long)H * W;
  const long long n = (long long)batch * HW;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / HW), p = (int)(t - (long long)b * HW);
    const int r = p / W, c = p - r * W;
    const Noisy img{snaps + (size_t)src[b] * HW * 3, noise, seed,
                    (unsigned long long)b * (unsigned long long)HW};
    const float* sti = statics + (size_t)dom[b] * HW * kStatics;
    const float* st = sti + (size_t)p * kStatics;
    const int pe = c + 1 < W ? p + 1 : p, pw = c > 0 ? p - 1 : -1;
    const int pn = r + 1 < H ? p + W : p, ps = r > 0 ? p - W : -1;
    const float d = st[0];
    const float e0 = img.get(p, 0), u0 = img.get(p, 1), v0 = img.get(p, 2);
    const float gx = (pe != p ? img.get(pe, 0) : e0) - e0;
    const float gy = (pn != p ? img.get(pn, 0) : e0) - e0;
    float div = 0.5f * (d + sti[(size_t)pe * kStatics]) * u0 +
                0.5f * (d + sti[(size_t)pn * kStatics]) * v0;
    if (pw >= 0) div -= 0.5f * (d + sti[(size_t)pw * kStatics]) * img.get(pw, 1);
    if (ps >= 0) div -= 0.5f * (d + sti[(size_t)ps * kStatics]) * img.get(ps, 2);
    __nv_bfloat16* xo = x + (size_t)t * cpad;
    const float st0[3] = {(e0 - forcing[b]) / scale.x, u0 / scale.y, v0 / scale.z};
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {  // high and low BF16 parts
      const __nv_bfloat16 hi = __float2bfloat16(st0[ch]);
      xo[ch] = hi;
      xo[12 + ch] = __float2bfloat16(st0[ch] - __bfloat162float(hi));
    }
    xo[3] = __float2bfloat16(d);
    xo[4] = __float2bfloat16(forcing[b] * st[1] / scale.x);
    xo[5] = __float2bfloat16(gx / dscale.x);
    xo[6] = __float2bfloat16(gy / dscale.y);
    xo[7] = __float2bfloat16(div / dscale.z);
    xo[8] = __float2bfloat16(st[1]);
    xo[9] = __float2bfloat16((e0 - forcing[b]) * st[1] / scale.x);
    xo[10] = __float2bfloat16(st[2]);
    xo[11] = __float2bfloat16(st[3]);
    for (int ch = 15; ch < cpad; ch++) xo[ch] = __float2bfloat16(0.f);
    if (target) {
      // the next snapshot of the same domain
      const float* s1 = img.img + ((size_t)HW + p) * 3;
      float* to = target + (size_t)t * 3;
      to[0] = (s1[0] - e0) / inc_scale.x;
      to[1] = (s1[1] - u0) / inc_scale.y;
      to[2] = (s1[2] - v0) / inc_scale.z;
    }
  }
}

// state += increment (first 3 of cpad FP32 output channels) * inc_scale.
// With statics, the solver's boundary conditions are applied as the solver
// applies them: velocities on wall faces are held at zero, and the ssh of
// wet cells next to the open side is the tide at the target time.
__global__ void k_advance(float* __restrict__ state, const float* __restrict__ inc,
                          float3 inc_scale, const float* __restrict__ statics,
                          const int* __restrict__ dom, const float* __restrict__ forcing,
                          long long HW, long long P, int cpad) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < P;
       t += (long long)gridDim.x * blockDim.x) {
    float e = state[t * 3 + 0] + inc[t * cpad + 0] * inc_scale.x;
    float u = state[t * 3 + 1] + inc[t * cpad + 1] * inc_scale.y;
    float v = state[t * 3 + 2] + inc[t * cpad + 2] * inc_scale.z;
    if (statics) {
      const long long b = t / HW;
      const float* st = statics + ((size_t)dom[b] * HW + (t - b * HW)) * kStatics;
      if (st[1] > 0.f) e = forcing[b];
      if (st[2] > 0.f) u = 0.f;
      if (st[3] > 0.f) v = 0.f;
    }
    state[t * 3 + 0] = e;
    state[t * 3 + 1] = u;
    state[t * 3 + 2] = v;
  }
}

}  // namespace
}  // namespace emu
}  // namespace nl2d

using namespace nl2d::emu;

extern "C" {

// Test hook (no reference counterpart): runs k_selftest_wait and returns
// its status in *status: 1 when the wait ran out and reported it, as the
// convolution kernels' waits do.
int nl2d_selftest_wait(long long max_cycles, int* status) {
  if (!status || max_cycles < 1 || max_cycles > (1LL << 32)) return NL2D_ERR_ARGS;
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return NL2D_ERR_CUDA;
  cudaMemset(d, 0, sizeof(int));
  k_selftest_wait<<<1, 32>>>(max_cycles, d);
  const cudaError_t e = cudaMemcpy(status, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

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
  const size_t smem = wbytes + kConvSlots * (size_t)(cin / 8) * kRowPix * 16;
  constexpr int kMaxSmem = 200 * 1024;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_conv3x3_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kMaxSmem) != cudaSuccess)
      return NL2D_ERR_CUDA;
    attr = true;
  }
  if (smem > kMaxSmem) return NL2D_ERR_ARGS;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long units =
      (long long)batch * ((H + kStripRows - 1) / kStripRows) * (W / kTileM);
  // Persistent CTAs: as many as are resident at once.  Counted from the
  // kernel's registers (allocated per warp in units of 256) and shared
  // memory (dynamic + static + the driver's reserve per block), as the
  // hardware limits them; each CTA also holds kPipeTmemCols of the SM's 512
  // TMEM columns.  (cudaOccupancyMaxActiveBlocksPerMultiprocessor answered 1
  // here where 2 are resident, and the forward pass took 0.78 instead of
  // 0.51 ms.)
  static cudaFuncAttributes fa;
  static bool fa_ok = false;
  if (!fa_ok) {
    if (cudaFuncGetAttributes(&fa, k_conv3x3_pipe) != cudaSuccess) return NL2D_ERR_CUDA;
    fa_ok = true;
  }
  int regs_sm = 0, smem_sm = 0, smem_rsv = 0;
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  const int warp_regs = (fa.numRegs * 32 + 255) / 256 * 256;
  const int by_regs = regs_sm / (warp_regs * (kPipeThreads / 32));
  const int by_smem = smem_sm / (int)(smem + fa.sharedSizeBytes + smem_rsv);
  int per_sm = by_regs < by_smem ? by_regs : by_smem;
  per_sm = per_sm < 512 / kPipeTmemCols ? per_sm : 512 / kPipeTmemCols;
  per_sm = per_sm < 1 ? 1 : per_sm;
  const int grid = (int)(units < (long long)per_sm * sms ? units : (long long)per_sm * sms);
  k_conv3x3_pipe<<<grid, kPipeThreads, smem, (cudaStream_t)stream>>>(
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
                        int W, int cin, int cout, int* err, void* stream) {
  if (!x || !dy || !dw || !db || !err || cin % 16 || cin < 16 || 9 * cin > kWgTmemCols ||
      cout % 8 || cout < 8 || cout > 128 || W % kTileM || H < 1 || batch < 1)
    return NL2D_ERR_ARGS;
  // The kernel holds all 512 TMEM columns, so it must be alone on its SM:
  // asking for more than half an SM's shared memory guarantees that.
  const size_t need = (size_t)kWgYSlots * kWgGroups * kTileM * 16 +
                      (size_t)kSlots * (cin / 8) * kRowPix * 16;
  const size_t smem = need > kWgSmem ? need : kWgSmem;
  constexpr size_t kMaxSmem = 200 * 1024;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_conv_wgrad_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kMaxSmem) != cudaSuccess)
      return NL2D_ERR_CUDA;
    attr = true;
  }
  if (smem > kMaxSmem) return NL2D_ERR_ARGS;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long units =
      (long long)batch * ((H + kStripRows - 1) / kStripRows) * (W / kTileM);
  const int grid = (int)(units < sms ? units : sms);  // 512 TMEM columns: one CTA per SM
  constexpr int kBiasBlocks = 152 * 8;
  const long long nel = 9LL * cout * cin;
  if (!ensure_parts((size_t)std::max<long long>(grid * nel, (long long)kBiasBlocks * cout)))
    return NL2D_ERR_CUDA;
  const cudaStream_t st = (cudaStream_t)stream;
  k_conv_wgrad_pipe<<<grid, kPipeThreads, smem, st>>>(
      (const __nv_bfloat16*)x, (const __nv_bfloat16*)dy, g_parts, batch, H, W, cin, cout, err);
  k_sum_parts<<<(int)((nel + 255) / 256), 256, 0, st>>>(g_parts, grid, nel, dw);
  if (cudaGetLastError() != cudaSuccess) return NL2D_ERR_CUDA;
  k_bias_grad<<<kBiasBlocks, 256, 0, st>>>((const __nv_bfloat16*)dy, g_parts,
                                            (long long)batch * H * W, cout);
  k_sum_parts<<<1, 128, 0, st>>>(g_parts, kBiasBlocks, cout, db);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_relu_bwd(const float* g, const void* y, void* out, long long n, void* stream) {
  k_relu_bwd<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(g, (const __nv_bfloat16*)y,
                                                         (__nv_bfloat16*)out, n);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_mse(const float* pred, const float* target, const float* weight, void* grad,
                 float* loss, long long P, int nc, int cpad, void* stream) {
  if (!pred || !target || !grad || !loss || P < 1 || nc < 1 || cpad < nc) return NL2D_ERR_ARGS;
  k_mse<<<152 * 4, 256, 0, (cudaStream_t)stream>>>(pred, target, weight, (__nv_bfloat16*)grad,
                                                    loss, P, nc, cpad);
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
                      const int* dom, const float* forcing, const float* scale12,
                      unsigned long long seed, void* x, float* target, int H, int W, int cpad,
                      int batch, void* stream) {
  if (!snaps || !statics || !src || !dom || !forcing || !scale12 || !x || cpad < 15 || H < 1 ||
      W < 1 || batch < 1)
    return NL2D_ERR_ARGS;
  k_assemble<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(
      snaps, statics, src, dom, forcing, make_float3(scale12[0], scale12[1], scale12[2]),
      make_float3(scale12[3], scale12[4], scale12[5]),
      make_float3(scale12[6], scale12[7], scale12[8]),
      make_float3(scale12[9], scale12[10], scale12[11]), seed, (__nv_bfloat16*)x, target, H, W,
      cpad, batch);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

int nl2d_emu_advance(float* state, const float* inc, const float* inc_scale3,
                     const float* statics, const int* dom, const float* forcing, long long HW,
                     long long P, int cpad, void* stream) {
  if (!state || !inc || !inc_scale3 || (statics && (!dom || !forcing || HW < 1)) || P < 0 ||
      cpad < 3)
    return NL2D_ERR_ARGS;
  k_advance<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(
      state, inc, make_float3(inc_scale3[0], inc_scale3[1], inc_scale3[2]), statics, dom,
      forcing, HW, P, cpad);
  return cudaGetLastError() == cudaSuccess ? NL2D_OK : NL2D_ERR_CUDA;
}

}  // extern "C"
