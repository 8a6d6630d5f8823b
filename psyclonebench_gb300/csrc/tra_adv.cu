// Tracer advection (the NEMO tra_adv benchmark,
// benchmarks/nemo/tracer_advection/original/tra_adv.F90:107-257, in the
// per-iteration form of compute_in_subroutine/tra_adv_compute.F90:12-) on
// the GPU, bit-identical to the reference's operations (built with
// -fmad=false; SIGN is copysign, MAX / MIN pairwise left to right).
//
// Layout: Fortran a(ji, jj, jk) is a[(k * J + j) * I + i], 0-based.
//
// One iteration is two kernels:
//  * k_tra_horizontal_tiled: for every interior point (1 <= i <= I-2,
//    1 <= j <= J-2, k <= K-2) the x / y differences, MUSCL slopes with their
//    limiter, the upstream fluxes and the flux-divergence update, from the
//    previous iteration's field (ping-pong buffers: the update of one point
//    never sees another point's new value, as in the reference's separate
//    loops).
//  * k_tra_vertical: one thread per interior column marches up in k through
//    the vertical differences, slopes, fluxes and the final assignment.
// Work arrays are never stored: each value is recomputed where it is used.
// Two of the reference's work-array entries are read before the iteration
// writes them, so they come from earlier calls:
//  * zwx(jpi, :, :) (the x difference east of the last interior column)
//    holds the previous iteration's vertical differences of that column,
//    whose field never changes: tmask (m(k-1) - m(k)), pwn m at k = 1; on
//    the first iteration after registration it is zero (fresh pages).
//  * zwy(jpi, :, :) and zwy(:, jpj, :) are never written: zero.
// zind depends only on inputs, so it is computed once at registration.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/nl2d_gpu.h"
#include "nl2d_exact.cuh"  // bits, from_bits, half, pick
#include "nl2d_internal.h"  // NvtxRange

// On GB300 the FP64 pipe issues about 2 thread-operations per clock per SM,
// ~30x fewer than the integer pipe, and this iteration is FP64-bound.  The
// helpers below return the same bits as the IEEE expressions of the
// reference (named in each comment) for every input, with fewer FP64
// instructions.  Operands the integer forms do not cover (non-finite values,
// subnormal halves, overflowing doubles) take the IEEE expression itself in
// a separate, non-inlined function: as a real branch it costs nothing when
// not taken, whereas inlined, the compiler may predicate it and issue its
// FP64 instructions for every operand.
namespace {

using nl2d::bits;
using nl2d::from_bits;
using nl2d::half;  // 0.5 x, exact in integer arithmetic for normal x
using nl2d::pick;  // a + (+0) z: the operand, or a zero with the AND of both signs

constexpr long long kMag = 0x7fffffffffffffffLL;
constexpr long long kSign = (long long)0x8000000000000000ULL;
__device__ __forceinline__ bool finite(long long b) { return ((b >> 52) & 0x7ff) != 0x7ff; }

__device__ __forceinline__ double max2(double a, double b) { return a > b ? a : b; }

__device__ __noinline__ long long twice_abs_ieee(double x) { return bits(2.0 * fabs(x)); }
__device__ __noinline__ double slope_ieee(double a, double b) {
  return (a + b) * (0.25 + copysign(0.25, a * b));
}
__device__ __noinline__ double limit_ieee(double s, double p, double q) {
  const double a = fabs(s), b = 2.0 * fabs(p), c = 2.0 * fabs(q);
  const double m = a < b ? a : b;
  return copysign(1.0, s) * (m < c ? m : c);
}

// 2 |x| for finite x: one more in the exponent of a normal value, the
// magnitude shifted left for a subnormal one (the encoding is continuous
// across the boundary); the largest binade (2 |x| overflows) multiplies.
__device__ __forceinline__ long long twice_abs_bits(double x) {
  const long long m = bits(x) & kMag;
  const int ex = (int)(m >> 52);
  if (ex == 0) return m << 1;
  if (ex <= 2045) return m + (1LL << 52);
  return twice_abs_ieee(x);
}

// (a + b) (0.25 + SIGN(0.25, a b)) (tra_adv.F90:138-141, :210-211).  For
// finite a, b the product's sign is the XOR of theirs (also when it
// underflows or overflows), so the second factor is 0.5 or +0: the result
// is half(a + b), or a zero with the sign of a + b (if a + b is finite).
__device__ __forceinline__ double slope_raw(double a, double b) {
  const long long ab = bits(a), bb = bits(b);
  if (!finite(ab) || !finite(bb)) return slope_ieee(a, b);
  const double s = a + b;
  const long long sb = bits(s);
  if (!finite(sb)) return slope_ieee(a, b);
  if ((ab ^ bb) < 0) return from_bits(sb & kSign);  // factor 0.25 + (-0.25) = +0
  return half(s);
}

// SIGN(1, s) MIN(|s|, 2 |p|, 2 |q|) (tra_adv.F90:150-155, :214-216).  The
// three candidates are non-negative, so their order is the order of their
// bit patterns; multiplying the minimum by +-1 only sets its sign.
__device__ __forceinline__ double limit(double s, double p, double q) {
  const long long sb = bits(s), pb = bits(p), qb = bits(q);
  if (!finite(sb) || !finite(pb) || !finite(qb)) return limit_ieee(s, p, q);
  const long long a = sb & kMag, b = twice_abs_bits(p), c = twice_abs_bits(q);
  const long long m = a < b ? a : b;
  return from_bits((m < c ? m : c) | (sb & kSign));
}

// SIGN(0.5, v): 0.5 with v's sign bit (copysign), set in integer
// arithmetic.
__device__ __forceinline__ double half_sign(double v) {
  return from_bits(0x3FE0000000000000LL | (bits(v) & kSign));
}

// zu = SIGN(0.5, v) - 0.5 v 1 (tra_adv.F90:165, :173, :231).
__device__ __forceinline__ double courant(double z0, double v) { return z0 - half(v); }

// The upstream flux of tra_adv.F90:163-169 (x) / :171-177 (y): vel at the
// face, the field on the far (f1) and near (f0) side, their slopes.
// zalpha = 0.5 - SIGN(0.5, vel) is exactly 1 or +0, so
// zalpha zzwx + (1 - zalpha) zzwy is one operand plus a zero-weighted
// partner: pick().
__device__ __forceinline__ double upstream(double vel, double f1, double f0, double zind,
                                           double s1, double s0) {
  const double z0 = half_sign(vel);
  const double zu = courant(z0, vel);
  const double zzwx = f1 + zind * (zu * s1);
  const double zzwy = f0 + zind * (zu * s0);
  return vel * ((bits(vel) < 0) ? pick(zzwx, zzwy) : pick(zzwy, zzwx));
}

struct TraDev {
  const double *pun, *pvn, *pwn, *umask, *vmask, *tmask, *zind;
  int I, J, K;
};

__global__ void k_tra_zind(const double* __restrict__ tsn, const double* __restrict__ ztfreez,
                           const double* __restrict__ rnfmsk, const double* __restrict__ upsmsk,
                           const double* __restrict__ rnfmsk_z,
                           const double* __restrict__ tmask, double* __restrict__ zind, int I,
                           int J, int K) {
  const long long n = (long long)I * J * K;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t / ((long long)I * J));
    const long long p2 = t - (long long)k * I * J;
    const double zice = tsn[t] <= ztfreez[p2] + 0.1 ? 1.0 : 0.0;
    double z = max2(max2(rnfmsk[p2] * rnfmsk_z[k], upsmsk[p2]), zice) * tmask[t];
    zind[t] = 1 - z;
  }
}

// tra_adv.F90:122-194 for the interior points, from `mo` (the field before
// the iteration) into `mn` (whose other points already hold their
// unchanging values).  A CTA of kTx x kTy threads owns kTx x kTy interior
// points of one level and stages, in shared memory, the field with a
// 2-point halo, then the x / y differences, the limited slopes and the
// fluxes its points need, each once, shared by the neighbours.  The
// x difference east of the last interior column (i = I-1) is the entry the
// previous iteration's vertical part left in the reference's zwx (zero on
// the first iteration); y differences on the row j = J-1 are zero (never
// written there).
constexpr int kTx = 32, kTy = 16;

__global__ void __launch_bounds__(kTx * kTy)
    k_tra_horizontal_tiled(const double* __restrict__ mo, double* __restrict__ mn, TraDev d,
                           int first) {
  __shared__ double sm[kTy + 4][kTx + 4];   // m at (j0-2+r, i0-2+c)
  __shared__ double dx_[kTy][kTx + 3];      // x difference at i0-2+c
  __shared__ double dy_[kTy + 3][kTx];      // y difference at j0-2+r
  __shared__ double sx_[kTy][kTx + 2];      // x slope at i0-1+c
  __shared__ double sy_[kTy + 2][kTx];      // y slope at j0-1+r
  __shared__ double fx_[kTy][kTx + 1];      // x flux at i0-1+c
  __shared__ double fy_[kTy + 1][kTx];      // y flux at j0-1+r
  const int tid = threadIdx.y * kTx + threadIdx.x, nt = kTx * kTy;
  const int i0 = 1 + blockIdx.x * kTx, j0 = 1 + blockIdx.y * kTy, k = blockIdx.z;
  const int I = d.I, J = d.J;
  const size_t lev = (size_t)k * J * I;
  const bool f = first != 0;

  for (int t = tid; t < (kTy + 4) * (kTx + 4); t += nt) {
    const int r = t / (kTx + 4), c = t - r * (kTx + 4);
    const int i = i0 - 2 + c, j = j0 - 2 + r;
    sm[r][c] = (i >= 0 && i < I && j >= 0 && j < J) ? mo[lev + (size_t)j * I + i] : 0.0;
  }
  __syncthreads();
  for (int t = tid; t < kTy * (kTx + 3); t += nt) {  // x differences
    const int r = t / (kTx + 3), c = t - r * (kTx + 3);
    const int i = i0 - 2 + c, j = j0 + r;
    double v = 0.0;
    if (i >= 0 && j < J) {
      const size_t g = lev + (size_t)j * I + i;
      if (i <= I - 2) v = d.umask[g] * (sm[r + 2][c + 1] - sm[r + 2][c]);
      else if (i == I - 1 && !f)
        v = (k == 0) ? d.pwn[g] * sm[r + 2][c] : d.tmask[g] * (mo[g - (size_t)I * J] - sm[r + 2][c]);
    }
    dx_[r][c] = v;
  }
  for (int t = tid; t < (kTy + 3) * kTx; t += nt) {  // y differences
    const int r = t / kTx, c = t - r * kTx;
    const int i = i0 + c, j = j0 - 2 + r;
    double v = 0.0;
    if (j >= 0 && j <= J - 2 && i < I) {
      const size_t g = lev + (size_t)j * I + i;
      v = d.vmask[g] * (sm[r + 1][c + 2] - sm[r][c + 2]);
    }
    dy_[r][c] = v;
  }
  __syncthreads();
  for (int t = tid; t < kTy * (kTx + 2); t += nt) {  // x slopes at i0-1+c
    const int r = t / (kTx + 2), c = t - r * (kTx + 2);
    const double a = dx_[r][c + 1], b = dx_[r][c];
    sx_[r][c] = limit(slope_raw(a, b), b, a);
  }
  for (int t = tid; t < (kTy + 2) * kTx; t += nt) {  // y slopes at j0-1+r
    const int r = t / kTx, c = t - r * kTx;
    const double a = dy_[r + 1][c], b = dy_[r][c];
    sy_[r][c] = limit(slope_raw(a, b), b, a);
  }
  __syncthreads();
  for (int t = tid; t < kTy * (kTx + 1); t += nt) {  // x fluxes at i0-1+c
    const int r = t / (kTx + 1), c = t - r * (kTx + 1);
    const int i = i0 - 1 + c, j = j0 + r;
    double v = 0.0;
    if (i == 0) {
      v = dx_[r][c + 1];  // the flux loop starts at ji = 2: zwx(1) is still the difference
    } else if (i <= I - 2 && j < J) {
      const size_t g = lev + (size_t)j * I + i;
      v = upstream(d.pun[g], sm[r + 2][c + 2], sm[r + 2][c + 1], d.zind[g], sx_[r][c + 1],
                   sx_[r][c]);
    }
    fx_[r][c] = v;
  }
  for (int t = tid; t < (kTy + 1) * kTx; t += nt) {  // y fluxes at j0-1+r
    const int r = t / kTx, c = t - r * kTx;
    const int i = i0 + c, j = j0 - 1 + r;
    double v = 0.0;
    if (j == 0) {
      v = dy_[r + 1][c];
    } else if (j <= J - 2 && i < I) {
      const size_t g = lev + (size_t)j * I + i;
      v = upstream(d.pvn[g], sm[r + 2][c + 2], sm[r + 1][c + 2], d.zind[g], sy_[r + 1][c],
                   sy_[r][c]);
    }
    fy_[r][c] = v;
  }
  __syncthreads();
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  if (i <= I - 2 && j <= J - 2) {
    const int r = threadIdx.y, c = threadIdx.x;
    const double ztra = -(1.0 * (fx_[r][c + 1] - fx_[r][c] + fy_[r + 1][c] - fy_[r][c]));
    mn[lev + (size_t)j * I + i] = sm[r + 2][c + 2] + ztra;
  }
}

// tra_adv.F90:196-251 for one interior column, in place on m (the field
// after the horizontal update).
__global__ void __launch_bounds__(256) k_tra_vertical(double* __restrict__ m, TraDev d) {
  const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > d.I - 2 || j > d.J - 2) return;
  const size_t s = (size_t)d.I * d.J;
  const size_t c0 = (size_t)j * d.I + i;
  const int K = d.K;
  double mk = m[c0];
  double mk1 = m[c0 + s];  // K >= 2
  double zd1 = (1 <= K - 2) ? d.tmask[c0 + s] * (mk - mk1) : 0.0;
  double slk = 0.0;               // zslpx(:,:,1) = 0
  double fwk = d.pwn[c0] * mk;    // zwx(:,:,1) = pwn m
  for (int k = 0; k <= K - 2; k++) {
    const size_t c = c0 + (size_t)k * s;
    double mk2 = 0.0, zd2 = 0.0;
    if (k + 2 <= K - 1) mk2 = m[c + 2 * s];
    if (k + 2 <= K - 2) zd2 = d.tmask[c + 2 * s] * (mk1 - mk2);
    const double slk1 = (k + 1 <= K - 2) ? limit(slope_raw(zd1, zd2), zd2, zd1) : 0.0;
    const double p1 = d.pwn[c + s];
    const double z0w = half_sign(p1);
    const double zw = courant(z0w, p1);
    const double zind = d.zind[c];
    const double zzwx = mk1 + zind * (zw * slk1);
    const double zzwy = mk + zind * (zw * slk);
    // zalpha = 0.5 + SIGN(0.5, pwn): 1 for pwn >= +0, else +0
    const double fwk1 = p1 * ((bits(p1) < 0) ? pick(zzwy, zzwx) : pick(zzwx, zzwy));
    m[c] = -(1.0 * (fwk - fwk1));
    mk = mk1;
    mk1 = mk2;
    zd1 = zd2;
    slk = slk1;
    fwk = fwk1;
  }
}

}  // namespace

// ---- host side ---------------------------------------------------------------

namespace {

struct TraState {
  // registration key: the caller's arrays and extents
  const void* key[12] = {};
  int I = 0, J = 0, K = 0;
  bool registered = false;
  double* m[2] = {nullptr, nullptr};  // ping-pong copies of mydomain
  double *pun = nullptr, *pvn = nullptr, *pwn = nullptr, *umask = nullptr, *vmask = nullptr,
         *tmask = nullptr, *zind = nullptr;
  int cur = 0;                 // buffer holding the current field
  long long iters = 0;         // iterations since registration
  cudaStream_t stream = nullptr;
  int status = NL2D_OK;
  char msg[256] = "";
};
TraState g_tra;

void tra_fail(int code, const char* fmt, ...) {
  if (g_tra.status != NL2D_OK) return;  // keep the first error
  g_tra.status = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_tra.msg, sizeof g_tra.msg, fmt, ap);
  va_end(ap);
}

bool tra_ck(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  tra_fail(NL2D_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return false;
}

void tra_release() {
  TraState& s = g_tra;
  for (double** p : {&s.m[0], &s.m[1], &s.pun, &s.pvn, &s.pwn, &s.umask, &s.vmask, &s.tmask,
                     &s.zind}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  s.registered = false;
}

TraDev tra_dev() {
  const TraState& s = g_tra;
  return TraDev{s.pun, s.pvn, s.pwn, s.umask, s.vmask, s.tmask, s.zind, s.I, s.J, s.K};
}

// One iteration's two launches on the library's stream.
void tra_launch_iteration(int cur, bool first) {
  TraState& s = g_tra;
  const dim3 blk(kTx, kTy);
  const dim3 grd((s.I - 2 + kTx - 1) / kTx, (s.J - 2 + kTy - 1) / kTy, s.K - 1);
  k_tra_horizontal_tiled<<<grd, blk, 0, s.stream>>>(s.m[cur], s.m[cur ^ 1], tra_dev(),
                                                     first ? 1 : 0);
  const dim3 vblk(32, 8);
  const dim3 vgrd((s.I - 2 + 31) / 32, (s.J - 2 + 7) / 8, 1);
  k_tra_vertical<<<vgrd, vblk, 0, s.stream>>>(s.m[cur ^ 1], tra_dev());
}

bool tra_register(const double* ztfreez, const double* pun, const double* pvn, const double* pwn,
                  const double* umask, const double* vmask, const double* tmask,
                  const double* rnfmsk, const double* rnfmsk_z, const double* upsmsk,
                  const double* mydomain, const double* tsn, int I, int J, int K) {
  TraState& s = g_tra;
  const void* key[12] = {ztfreez, pun, pvn, pwn, umask, vmask, tmask, rnfmsk, rnfmsk_z,
                         upsmsk, mydomain, tsn};
  if (s.registered && s.I == I && s.J == J && s.K == K && !memcmp(key, s.key, sizeof key))
    return true;
  tra_release();
  if (!s.stream && !tra_ck(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking),
                           "cudaStreamCreateWithFlags"))
    return false;
  const size_t n3 = (size_t)I * J * K, b3 = n3 * sizeof(double);
  const size_t b2 = (size_t)I * J * sizeof(double);
  for (double** p : {&s.m[0], &s.m[1], &s.pun, &s.pvn, &s.pwn, &s.umask, &s.vmask, &s.tmask,
                     &s.zind})
    if (!tra_ck(cudaMalloc(p, b3), "cudaMalloc")) return false;
  double *d_tsn = nullptr, *d2[3] = {nullptr, nullptr, nullptr}, *d_rz = nullptr;
  bool ok = tra_ck(cudaMalloc(&d_tsn, b3), "cudaMalloc") &&
            tra_ck(cudaMalloc(&d_rz, K * sizeof(double)), "cudaMalloc");
  for (int q = 0; q < 3 && ok; q++) ok = tra_ck(cudaMalloc(&d2[q], b2), "cudaMalloc");
  const struct {
    double* dst;
    const double* src;
    size_t bytes;
  } up[] = {{s.m[0], mydomain, b3}, {s.pun, pun, b3},     {s.pvn, pvn, b3},
            {s.pwn, pwn, b3},       {s.umask, umask, b3}, {s.vmask, vmask, b3},
            {s.tmask, tmask, b3},   {d_tsn, tsn, b3},     {d2[0], ztfreez, b2},
            {d2[1], rnfmsk, b2},    {d2[2], upsmsk, b2},  {d_rz, rnfmsk_z, K * sizeof(double)}};
  for (const auto& u : up)
    if (ok) ok = tra_ck(cudaMemcpyAsync(u.dst, u.src, u.bytes, cudaMemcpyHostToDevice, s.stream),
                        "upload");
  if (ok) {
    ok = tra_ck(cudaMemcpyAsync(s.m[1], s.m[0], b3, cudaMemcpyDeviceToDevice, s.stream),
                "copy");
    k_tra_zind<<<152 * 8, 256, 0, s.stream>>>(d_tsn, d2[0], d2[1], d2[2], d_rz, s.tmask, s.zind,
                                              I, J, K);
    ok = ok && tra_ck(cudaGetLastError(), "k_tra_zind") &&
         tra_ck(cudaStreamSynchronize(s.stream), "registration");
  }
  cudaFree(d_tsn);
  cudaFree(d_rz);
  for (double* p : d2) cudaFree(p);
  if (!ok) {
    tra_release();
    return false;
  }
  memcpy(s.key, key, sizeof key);
  s.I = I;
  s.J = J;
  s.K = K;
  s.cur = 0;
  s.iters = 0;
  s.registered = true;
  return true;
}

}  // namespace

extern "C" {

void tra_adv_compute(const double* ztfreez, const double* pun, const double* pvn,
                     const double* pwn, const double* umask, const double* vmask,
                     const double* tmask, const double* rnfmsk, const double* rnfmsk_z,
                     const double* upsmsk, double* mydomain, const double* tsn, int jpi, int jpj,
                     int jpk) {
  nl2d::NvtxRange nvtx_range("tra_adv_compute");
  if (!ztfreez || !pun || !pvn || !pwn || !umask || !vmask || !tmask || !rnfmsk || !rnfmsk_z ||
      !upsmsk || !mydomain || !tsn || jpi < 3 || jpj < 3 || jpk < 2 ||
      (double)jpi * jpj * jpk > 4.0e9) {
    tra_fail(NL2D_ERR_ARGS, "tra_adv_compute: bad arrays or extents (%d x %d x %d)", jpi, jpj,
             jpk);
    return;
  }
  if (!tra_register(ztfreez, pun, pvn, pwn, umask, vmask, tmask, rnfmsk, rnfmsk_z, upsmsk,
                    mydomain, tsn, jpi, jpj, jpk))
    return;
  TraState& s = g_tra;
  tra_launch_iteration(s.cur, s.iters == 0);
  if (!tra_ck(cudaGetLastError(), "tra_adv iteration")) return;
  s.cur ^= 1;
  s.iters++;
}

int tra_adv_run(int niter, double* ms) {
  nl2d::NvtxRange nvtx_range("tra_adv_run");
  TraState& s = g_tra;
  if (!s.registered) return NL2D_ERR_STATE;
  if (niter < 0) return NL2D_ERR_ARGS;
  cudaEvent_t e0, e1;
  if (!tra_ck(cudaEventCreate(&e0), "cudaEventCreate") ||
      !tra_ck(cudaEventCreate(&e1), "cudaEventCreate"))
    return NL2D_ERR_CUDA;
  cudaEventRecord(e0, s.stream);
  for (int t = 0; t < niter; t++) {
    tra_launch_iteration(s.cur, s.iters == 0);
    s.cur ^= 1;
    s.iters++;
  }
  cudaEventRecord(e1, s.stream);
  bool ok = tra_ck(cudaGetLastError(), "tra_adv_run") &&
            tra_ck(cudaEventSynchronize(e1), "tra_adv_run");
  float t = 0.f;
  if (ok) cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ok ? NL2D_OK : NL2D_ERR_CUDA;
}

int tra_adv_read(double* mydomain) {
  TraState& s = g_tra;
  if (!s.registered) return NL2D_ERR_STATE;
  if (!mydomain) return NL2D_ERR_ARGS;
  const size_t b3 = (size_t)s.I * s.J * s.K * sizeof(double);
  if (!tra_ck(cudaMemcpyAsync(mydomain, s.m[s.cur], b3, cudaMemcpyDeviceToHost, s.stream),
              "tra_adv_read") ||
      !tra_ck(cudaStreamSynchronize(s.stream), "tra_adv_read"))
    return NL2D_ERR_CUDA;
  return NL2D_OK;
}

int tra_adv_checksum(double* out) {
  TraState& s = g_tra;
  if (!s.registered) return NL2D_ERR_STATE;
  if (!out) return NL2D_ERR_ARGS;
  std::vector<double> h((size_t)s.I * s.J * s.K);
  const int rc = tra_adv_read(h.data());
  if (rc != NL2D_OK) return rc;
  // tra_adv.F90:264-270, in the reference's loop order
  double sum = 0.0;
  for (int k = 0; k <= s.K - 2; k++)
    for (int j = 1; j <= s.J - 2; j++)
      for (int i = 1; i <= s.I - 2; i++) sum = sum + h[((size_t)k * s.J + j) * s.I + i];
  *out = sum;
  return NL2D_OK;
}

int tra_adv_last_error(char* buf, int len) {
  if (buf && len > 0) snprintf(buf, (size_t)len, "%s", g_tra.msg);
  const int st = g_tra.status;
  g_tra.status = NL2D_OK;
  g_tra.msg[0] = '\0';
  return st;
}

void tra_adv_finalize(void) {
  tra_release();
  if (g_tra.stream) cudaStreamDestroy(g_tra.stream);
  g_tra.stream = nullptr;
}

}  // extern "C"
