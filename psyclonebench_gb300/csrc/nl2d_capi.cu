// C-ABI of libnl2d_gpu (declared in include/nl2d_gpu.h): problem
// registration and residency, step-path selection, the reference-facing
// c_invoke_time_step / c_read_from_device / c_write_to_device, graph-captured
// multi-step runs and checksums.
#include "nl2d_internal.h"
#include "../../include/nl2d_gpu.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

namespace nl2d {
namespace {

constexpr int kNumFields = 13, kNumGrid = 12;

struct Registration {
  void* host[kNumFields + kNumGrid];  // caller's arrays, in ABI order
  int xs, xe, ys, ye, width, height;
};

struct State {
  bool registered = false;
  Registration reg{};
  Fields dev{};                // "primary" device arrays, one per reference array
  double* shadow[3] = {};      // ping-pong partners of sshn_t, un, vn
  int cur = 0;                 // 1: current sshn_t/un/vn live in the shadows
  bool consistent = false;     // a reference-structured step ran since the upload
  bool shadows_synced = false; // shadows equal primaries outside the copy region
  bool materialized = true;    // primaries hold the reference's arrays exactly
  bool fused_ok = false, chain_u = false, chain_v = false;
  UniformMetrics um{};
  Scalars sc{};
  double sin_d2r = NAN;
  int mode = NL2D_MODE_AUTO;
  int last_path = 0;
  cudaStream_t stream = nullptr;
  double* partials = nullptr;  // checksum scratch
  double* scan = nullptr;      // registration scan: flags word + reference values
  double* sums = nullptr;      // device checksum results
  int sums_cap = 0;
  double* tide_table = nullptr;
  int tide_cap = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_key[5] = {-1, -1, -1, -1, -1};
  // mixed-precision form
  int precision = 0;           // 0 FP64, 1 mixed, 2 FP64-equivalent (double-float)
  MixedFields mix{};
  int* mix_count = nullptr;    // device int for launch_mixed_flags
  float2* msn[2] = {};
  float* mun[2] = {};
  float* mvn[2] = {};
  int mcur = 0;
  bool mixed_valid = false;    // mixed buffers hold the current state
  bool mixed_ahead = false;    // ... and it is newer than the FP64 arrays
  int status = NL2D_OK;
  char msg[512] = {0};
  // FP64-equivalent form: split statics, march flags, the exact cells' list
  DfFields dfs{};
  bool df_valid = false;
  unsigned scan_flags = 0;     // last registration scan (kScan* bits)
  double grid_refs[11] = {};   // the metric arrays' and latitudes' reference values
  long long h2d_bytes = 0, d2h_bytes = 0;  // copied since registration
  void* slab = nullptr;        // the allocation the registration's arrays live in
  // Speculative registration (c_invoke_time_step over pinned arrays): the
  // arrays a fused step reads go first and steps start on `stream`; the
  // other arrays and the registration scan follow on `side`, and a later
  // call keeps the steps or takes them again by the scan's verdict.
  cudaStream_t side = nullptr;  // also the mixed form's general cells
  cudaEvent_t ess_done = nullptr, spec_ready = nullptr;
  cudaEvent_t side_fork = nullptr, side_join = nullptr;
  bool spec_pending = false;
  double* spec_backup[3] = {};  // sshn_t, un, vn as uploaded
  struct SpecOut {              // pinned host copy of the scan's results
    unsigned flags;
    double refs[11];
  }* spec_out = nullptr;
  std::vector<int> spec_steps;  // isteps taken before the verdict
  int spec_kept = 0, spec_redone = 0;  // verdicts since the library loaded
  // A speculative registration over pinned step arrays uploads them in
  // row bands on `side` (band b's copies complete band_up[b]) and its first
  // fused step runs band by band behind them, each band's tiles once their
  // rows and the next band's are on the device.  bands_pending: the bands'
  // depth reciprocals and shadow copies are still to be made (by the first
  // step, or by finish_bands for whatever comes first).
  static constexpr int kMaxBands = 8;
  cudaEvent_t band_up[kMaxBands] = {};
  cudaEvent_t backups_done = nullptr;  // spec_backup made (step 2 overwrites its source)
  int nbands = 0;
  int band_row[kMaxBands + 1] = {};   // array-row cuts
  int band_tile[kMaxBands + 1] = {};  // tile-row cuts of the fused step's grid
  bool bands_pending = false;
};

State g_state;

void set_error(int code, const char* fmt, ...) {
  if (g_state.status != NL2D_OK) return;  // keep the first error
  g_state.status = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_state.msg, sizeof g_state.msg, fmt, ap);
  va_end(ap);
}

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  set_error(NL2D_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return false;
}
#define CK(call) cuda_ok((call), #call)

double** field_slot(Fields& f, int k) {
  double** slots[kNumFields] = {&f.ssha_t, &f.sshn_t, &f.sshn_u, &f.sshn_v, &f.hu,
                                &f.hv,     &f.un,     &f.vn,     &f.ua,     &f.ht,
                                &f.ssha_u, &f.va,     &f.ssha_v};
  return slots[k];
}
double** grid_slot(Fields& f, int k) {  // k = 1..11 (0 is tmask)
  double** slots[kNumGrid] = {nullptr,  &f.area_t, &f.area_u, &f.area_v,
                              &f.dx_u,  &f.dx_v,   &f.dx_t,   &f.dy_u,
                              &f.dy_v,  &f.dy_t,   &f.gphiu,  &f.gphiv};
  return slots[k];
}

void invalidate_graph();

void drop_spec() {
  State& s = g_state;
  if (s.spec_pending && s.side) cudaStreamSynchronize(s.side);
  s.spec_pending = false;
  s.bands_pending = false;
  s.spec_steps.clear();
  for (double*& p : s.spec_backup) {
    cudaFree(p);
    p = nullptr;
  }
}

void free_device() {
  State& s = g_state;
  invalidate_graph();
  drop_spec();
  if (s.registered) {
    cudaFree(s.slab);  // every array of the registration
    s.slab = nullptr;
    for (int b = 0; b < 2; b++) {
      cudaFree(s.msn[b]);
      cudaFree(s.mun[b]);
      cudaFree(s.mvn[b]);
      s.msn[b] = nullptr;
      s.mun[b] = s.mvn[b] = nullptr;
    }
    cudaFree(s.mix.ht);
    cudaFree(s.mix.hu);
    cudaFree(s.mix.hv);
    cudaFree(s.mix.rhu);
    cudaFree(s.mix.rhv);
    cudaFree(s.mix.reg);
    cudaFree(s.mix.glist);
    cudaFree(s.mix_count);
    s.mix_count = nullptr;
    for (float2* a : {s.dfs.ht, s.dfs.hu, s.dfs.hv, s.dfs.rhu, s.dfs.rhv}) cudaFree(a);
    cudaFree(s.dfs.reg);
    cudaFree(s.dfs.ring);
    cudaFree(s.dfs.count);
    s.dfs = DfFields{};
    s.df_valid = false;
    s.mix = MixedFields{};
    s.mixed_valid = s.mixed_ahead = false;
  }
  s.dev = Fields{};
  for (double*& p : s.shadow) p = nullptr;
  s.registered = false;
}

Dims dims() {
  const Registration& r = g_state.reg;
  return Dims{r.xs, r.xe, r.ys, r.ye, r.width, r.height};
}

// Registration scans whole grids (16.8 M points at 4096^2) several times;
// split over the host's cores they take milliseconds instead of a third of
// a second.  f(lo, hi) runs on contiguous chunks of [begin, end).
template <class F>
void parallel_chunks(long long begin, long long end, F f) {
  const long long n = end - begin;
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (nt > 32) nt = 32;
  if (n < (1LL << 16) || nt == 1) {
    f(begin, end);
    return;
  }
  std::vector<std::thread> th;
  const long long chunk = (n + nt - 1) / nt;
  for (unsigned t = 0; t < nt; t++) {
    const long long lo = begin + (long long)t * chunk;
    const long long hi = std::min(end, lo + chunk);
    if (lo >= hi) break;
    th.emplace_back(f, lo, hi);
  }
  for (std::thread& x : th) x.join();
}

// sin(gphi * d2r) per point with the host libm, reusing the last value for
// runs of equal latitudes (a uniform grid costs one call per chunk).
void host_sines(const double* gphi, size_t n, double d2r, double* out) {
  parallel_chunks(0, (long long)n, [=](long long lo, long long hi) {
    double last_in = NAN, last_out = 0.0;
    for (long long k = lo; k < hi; k++) {
      if (!(gphi[k] == last_in) || std::signbit(gphi[k]) != std::signbit(last_in)) {
        last_in = gphi[k];
        last_out = std::sin(gphi[k] * d2r);
      }
      out[k] = last_out;
    }
  });
}

double* cur_sshn();
double* cur_un();
double* cur_vn();

// What registration needs to know about the problem it uploads, as bits:
// 0..8 metric array q (area_t, area_u, area_v, dx_u, dx_v, dx_t, dy_u, dy_v,
// dy_t) not bitwise uniform over [xs-1, xe+1] x [ys-1, ye+1] (every point a
// step reads it at); 9, 10 gphiu / gphiv not uniform over the whole array;
// 11 / 12 a Flather face in u / v reads another Flather face; 13 one would
// read outside the array (time_step.cpp's Flather loops are serial in those
// cases); 14 ssha_t differs from sshn_t on the copy region; 15 ua from un or
// va from vn there; 16 sshn_u or sshn_v is not what next_sshu / next_sshv
// make of sshn_t.  Bits 14-16 clear mean the state is what a step leaves
// (time_step.cpp:114-136 end every step with those copies and updates), so
// the first step may take the fused path.  Reference values are the
// region's first point of each metric array and gphi's first element,
// compared as bit patterns.
enum : unsigned {
  kScanMetrics = 0x1ffu,
  kScanGphiU = 1u << 9,
  kScanGphiV = 1u << 10,
  kScanChainU = 1u << 11,
  kScanChainV = 1u << 12,
  kScanOutside = 1u << 13,
  kScanSshaT = 1u << 14,
  kScanCopies = 1u << 15,
  kScanNextSsh = 1u << 16,
};

struct ScanIn {
  const double* metric[9];
  const double* gphi[2];
  const int* m;
  const double *sn, *un, *vn, *ua, *va, *sa, *snu, *snv;
  int xs, xe, ys, ye, W, H;
};

// next_sshu_code / next_sshv_code (time_update_kern.c:90-155) of one face
// with uniform areas: returns false where the kernel leaves the face alone.
// zero_pos: at and af are positive and finite, so two +0 heights give
// 0.5 * (at * +0 + at * +0) / af = +0 exactly, without the FP64 work (a
// state at rest is almost all +0).
__device__ __forceinline__ bool next_ssh_value(const int* m, const double* sn, int c, int step,
                                               double at, double af, bool zero_pos, double& v) {
  const int n = c + step;
  if (m[c] + m[n] <= 0) return false;
  if (m[c] * m[n] > 0) {
    if (zero_pos && (__double_as_longlong(sn[c]) | __double_as_longlong(sn[n])) == 0) {
      v = 0.0;
      return true;
    }
    const double rtmp1 = at * sn[c] + at * sn[n];
    v = 0.5 * rtmp1 / af;
  } else if (m[c] <= 0) {
    v = sn[n];
  } else {
    v = sn[c];
  }
  return true;
}

__global__ void k_register_scan(ScanIn in, unsigned* __restrict__ flags) {
  const int W = in.W;
  const int* m = in.m;
  auto writes = [m](int c, int step) {
    return m[c] + m[c + step] > -1 && (m[c] < 0 || m[c + step] < 0);
  };
  auto bits = [](double x) { return (unsigned long long)__double_as_longlong(x); };
  const size_t o = (size_t)(in.ys - 1) * W + (in.xs - 1);
  unsigned long long ref[9];
#pragma unroll
  for (int q = 0; q < 9; q++) ref[q] = bits(in.metric[q][o]);
  const unsigned long long g0 = bits(in.gphi[0][0]), g1 = bits(in.gphi[1][0]);
  // areas for the next_ssh check (meaningful only when uniform)
  const double at = in.metric[0][o], au = in.metric[1][o], av = in.metric[2][o];
  auto pos_finite = [](double x) { return x > 0.0 && x <= 1.7976931348623157e308; };
  const bool zu = pos_finite(at) && pos_finite(au), zv = pos_finite(at) && pos_finite(av);
  unsigned f = 0;
  // one row of the scanned region per block and pass: rows over blocks,
  // points of a row over threads (no index division)
  for (int j = in.ys - 1 + blockIdx.x; j <= in.ye + 1; j += gridDim.x)
  for (int i = in.xs - 1 + threadIdx.x; i <= in.xe + 1; i += blockDim.x) {
    const int c = j * W + i;
#pragma unroll
    for (int q = 0; q < 9; q++)
      if (bits(in.metric[q][c]) != ref[q]) f |= 1u << q;
    if (i <= in.xe && writes(c, 1)) {  // Flather u over [xs-1, xe] x [ys-1, ye+1]
      const int nb = m[c] < 0 ? i + 1 : i - 1;
      if (nb < 0)
        f |= kScanOutside;
      else if (nb >= in.xs - 1 && nb <= in.xe && writes(j * W + nb, 1))
        f |= kScanChainU;
    }
    if (j <= in.ye && writes(c, W)) {  // Flather v over [xs-1, xe+1] x [ys-1, ye]
      const int nb = m[c] < 0 ? j + 1 : j - 1;
      if (nb < 0)
        f |= kScanOutside;
      else if (nb >= in.ys - 1 && nb <= in.ye && writes(nb * W + i, W))
        f |= kScanChainV;
    }
    // the copy region [xs-1, xe+1] x [ys-1, ye]
    if (j <= in.ye) {
      if (bits(in.sa[c]) != bits(in.sn[c])) f |= kScanSshaT;
      if (bits(in.ua[c]) != bits(in.un[c]) || bits(in.va[c]) != bits(in.vn[c])) f |= kScanCopies;
    }
    if (j >= in.ys && j <= in.ye && i >= in.xs && i <= in.xe) {
      double v;
      if (i <= in.xe - 1 && next_ssh_value(m, in.sn, c, 1, at, au, zu, v) &&
          bits(v) != bits(in.snu[c]))
        f |= kScanNextSsh;
      if (j <= in.ye - 1 && next_ssh_value(m, in.sn, c, W, at, av, zv, v) &&
          bits(v) != bits(in.snv[c]))
        f |= kScanNextSsh;
    }
  }
  const long long n = (long long)W * in.H;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += stride) {
    if (bits(in.gphi[0][t]) != g0) f |= kScanGphiU;
    if (bits(in.gphi[1][t]) != g1) f |= kScanGphiV;
  }
  if (f) atomicOr(flags, f);
}

__global__ void k_fill(double* __restrict__ a, double v, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
       t += (size_t)gridDim.x * blockDim.x)
    a[t] = v;
}

// The Coriolis sines sin(gphi * d2r) on the device (the reference-
// structured path reads them per point) and their uniform values for the
// fused path.  A latitude uniform over the array takes one host sin per
// direction (the host libm, as the reference evaluates it); otherwise every
// point is evaluated on the host and the fused path applies only if the
// sines are uniform over the region the step reads.
bool update_sines(double d2r) {
  State& s = g_state;
  const Registration& r = s.reg;
  const size_t n = (size_t)r.width * r.height;
  bool uniform = true;
  if ((s.scan_flags & (kScanGphiU | kScanGphiV)) == 0) {
    s.um.sin_u = std::sin(s.grid_refs[9] * d2r);
    s.um.sin_v = std::sin(s.grid_refs[10] * d2r);
    k_fill<<<152 * 8, 256, 0, s.stream>>>(s.dev.sin_u, s.um.sin_u, n);
    k_fill<<<152 * 8, 256, 0, s.stream>>>(s.dev.sin_v, s.um.sin_v, n);
    if (!CK(cudaGetLastError())) return false;
  } else {
    std::unique_ptr<double[]> su(new double[n]), sv(new double[n]);
    host_sines((const double*)r.host[kNumFields + 10], n, d2r, su.get());
    host_sines((const double*)r.host[kNumFields + 11], n, d2r, sv.get());
    if (!CK(cudaMemcpy(s.dev.sin_u, su.get(), n * 8, cudaMemcpyHostToDevice)) ||
        !CK(cudaMemcpy(s.dev.sin_v, sv.get(), n * 8, cudaMemcpyHostToDevice)))
      return false;
    const int W = r.width;
    const size_t o = (size_t)(r.ys - 1) * W + (r.xs - 1);
    auto uniform_over = [&](const double* a, double& v) {
      v = a[o];
      uint64_t ref;
      memcpy(&ref, &v, 8);
      std::atomic<bool> ok{true};
      parallel_chunks(r.ys - 1, r.ye + 2, [&, ref](long long j0, long long j1) {
        for (long long j = j0; j < j1 && ok.load(std::memory_order_relaxed); j++) {
          const uint64_t* row = reinterpret_cast<const uint64_t*>(a + (size_t)j * W);
          uint64_t diff = 0;  // bitwise equality, branch-free along the row
          for (int i = r.xs - 1; i <= r.xe + 1; i++) diff |= row[i] ^ ref;
          if (diff) {
            ok.store(false, std::memory_order_relaxed);
            return;
          }
        }
      });
      return ok.load();
    };
    uniform &= uniform_over(su.get(), s.um.sin_u);
    uniform &= uniform_over(sv.get(), s.um.sin_v);
  }
  s.sin_d2r = d2r;
  const unsigned f = s.scan_flags;
  s.chain_u = (f & kScanChainU) != 0;
  s.chain_v = (f & kScanChainV) != 0;
  s.fused_ok = uniform && (f & (kScanMetrics | kScanOutside)) == 0 && !s.chain_u && !s.chain_v;
  return true;
}

// Launches the registration scan (k_register_scan) over the uploaded
// arrays on stream st; its flags word and the 11 reference values (the
// region's first point of each metric array, gphi's first elements) land
// in *flags_out / refs_out once st reaches them (host memory: pinned for a
// scan that the caller does not wait for).
// state: the sshn_t, un, vn to check (null: the current buffers).
bool launch_scan(cudaStream_t st, unsigned* flags_out, double* refs_out,
                 double* const* state = nullptr) {
  State& s = g_state;
  const Registration& r = s.reg;
  if (!s.scan && !CK(cudaMalloc(&s.scan, 4 * sizeof(double)))) return false;
  const double* g[11] = {s.dev.area_t, s.dev.area_u, s.dev.area_v, s.dev.dx_u,  s.dev.dx_v,
                         s.dev.dx_t,   s.dev.dy_u,   s.dev.dy_v,   s.dev.dy_t,  s.dev.gphiu,
                         s.dev.gphiv};
  ScanIn in{};
  for (int q = 0; q < 9; q++) in.metric[q] = g[q];
  in.gphi[0] = g[9];
  in.gphi[1] = g[10];
  in.m = s.dev.tmask;
  in.sn = state ? state[0] : cur_sshn();
  in.un = state ? state[1] : cur_un();
  in.vn = state ? state[2] : cur_vn();
  in.ua = s.dev.ua, in.va = s.dev.va, in.sa = s.dev.ssha_t;
  in.snu = s.dev.sshn_u, in.snv = s.dev.sshn_v;
  in.xs = r.xs, in.xe = r.xe, in.ys = r.ys, in.ye = r.ye, in.W = r.width, in.H = r.height;
  unsigned* d_flags = reinterpret_cast<unsigned*>(s.scan);
  if (!CK(cudaMemsetAsync(d_flags, 0, sizeof(unsigned), st))) return false;
  k_register_scan<<<152 * 8, 256, 0, st>>>(in, d_flags);
  if (!CK(cudaGetLastError())) return false;
  const size_t o = (size_t)(r.ys - 1) * r.width + (r.xs - 1);
  for (int q = 0; q < 11; q++)
    if (!CK(cudaMemcpyAsync(&refs_out[q], g[q] + (q < 9 ? o : 0), 8, cudaMemcpyDeviceToHost,
                            st)))
      return false;
  return CK(cudaMemcpyAsync(flags_out, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
}

// The scan's results into the state: the uniform metric values, the sines
// and the fused path's preconditions.
bool apply_scan(unsigned flags, const double* refs, double d2r) {
  State& s = g_state;
  s.scan_flags = flags;
  for (int q = 0; q < 11; q++) s.grid_refs[q] = refs[q];
  double* um[9] = {&s.um.area_t, &s.um.area_u, &s.um.area_v, &s.um.dx_u, &s.um.dx_v,
                   &s.um.dx_t,   &s.um.dy_u,   &s.um.dy_v,   &s.um.dy_t};
  for (int q = 0; q < 9; q++) *um[q] = s.grid_refs[q];
  return update_sines(d2r);
}

// The scan, waited for, then applied.  The state bits (14-16) matter only
// right after an upload.  Returns false on a CUDA error.
bool scan_grid(double d2r) {
  State& s = g_state;
  unsigned flags = 0;
  double refs[11];
  if (!launch_scan(s.stream, &flags, refs) || !CK(cudaStreamSynchronize(s.stream)))
    return false;
  return apply_scan(flags, refs, d2r);
}

bool same_registration(void* const* ptrs, int xs, int xe, int ys, int ye, int width,
                       int height) {
  const State& s = g_state;
  if (!s.registered) return false;
  const Registration& r = s.reg;
  if (r.xs != xs || r.xe != xe || r.ys != ys || r.ye != ye || r.width != width ||
      r.height != height)
    return false;
  for (int k = 0; k < kNumFields + kNumGrid; k++)
    if (r.host[k] != ptrs[k]) return false;
  return true;
}

// The second stream, at the device's highest priority: work queued there
// is scheduled ahead of the library stream's.
bool ensure_side() {
  State& s = g_state;
  if (s.side) return true;
  int least = 0, greatest = 0;
  if (!CK(cudaDeviceGetStreamPriorityRange(&least, &greatest))) return false;
  return CK(cudaStreamCreateWithPriority(&s.side, cudaStreamNonBlocking, greatest));
}

bool host_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // not a CUDA-known pointer: pageable
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Argument positions (c_invoke_time_step's order) of the arrays a fused
// step reads: every field but ssha_t, and the T mask.  The others (ssha_t,
// the metric and latitude arrays) only the registration scan and the
// reference-structured path read.
constexpr int kStepArrays[] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, kNumFields};
constexpr int kLateArrays[] = {0,  kNumFields + 1, kNumFields + 2, kNumFields + 3,
                               kNumFields + 4,  kNumFields + 5,  kNumFields + 6,
                               kNumFields + 7,  kNumFields + 8,  kNumFields + 9,
                               kNumFields + 10, kNumFields + 11};

bool upload(void* const* ptrs, int k, cudaStream_t st) {
  State& s = g_state;
  const size_t n = (size_t)s.reg.width * s.reg.height, esz = k == kNumFields ? 4 : 8;
  void* dst = k < kNumFields ? (void*)*field_slot(s.dev, k)
                             : (k == kNumFields ? (void*)s.dev.tmask
                                                : (void*)*grid_slot(s.dev, k - kNumFields));
  if (!CK(cudaMemcpyAsync(dst, ptrs[k], n * esz, cudaMemcpyHostToDevice, st))) return false;
  s.h2d_bytes += (long long)(n * esz);
  return true;
}

// Rows [r0, r1) of array k.
bool upload_rows(void* const* ptrs, int k, int r0, int r1, cudaStream_t st) {
  State& s = g_state;
  const size_t w = (size_t)s.reg.width, esz = k == kNumFields ? 4 : 8;
  char* dst = static_cast<char*>(
      k < kNumFields ? (void*)*field_slot(s.dev, k)
                     : (k == kNumFields ? (void*)s.dev.tmask
                                        : (void*)*grid_slot(s.dev, k - kNumFields)));
  const size_t off = (size_t)r0 * w * esz, bytes = (size_t)(r1 - r0) * w * esz;
  if (!CK(cudaMemcpyAsync(dst + off, static_cast<const char*>(ptrs[k]) + off, bytes,
                          cudaMemcpyHostToDevice, st)))
    return false;
  s.h2d_bytes += (long long)bytes;
  return true;
}

// speculate: the caller is c_invoke_time_step, which can take fused steps
// before the scan has answered (see State::spec_pending).
bool do_register(void* const* ptrs, int xs, int xe, int ys, int ye, int width, int height,
                 const Scalars& sc, bool speculate = false) {
  State& s = g_state;
  if (xs < 1 || ys < 1 || xe < xs || ye < ys || xe > width - 2 || ye > height - 2) {
    set_error(NL2D_ERR_ARGS,
              "internal region [%d,%d]x[%d,%d] does not fit a %dx%d array with a "
              "one-cell ring on each side",
              xs, xe, ys, ye, width, height);
    return false;
  }
  for (int k = 0; k < kNumFields + kNumGrid; k++)
    if (!ptrs[k]) {
      set_error(NL2D_ERR_ARGS, "array argument %d is NULL", k);
      return false;
    }
  free_device();
  if (!s.stream && !CK(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)))
    return false;
  Registration& r = s.reg;
  for (int k = 0; k < kNumFields + kNumGrid; k++) r.host[k] = ptrs[k];
  r.xs = xs, r.xe = xe, r.ys = ys, r.ye = ye, r.width = width, r.height = height;
  const size_t n = (size_t)width * height;
  s.registered = true;  // so free_device releases partial allocations
  s.h2d_bytes = s.d2h_bytes = 0;
  // One allocation carved into the registration's 32 arrays (256-byte
  // aligned): 34 separate cudaMalloc calls took 1.7-2.9 ms on the GB300
  // box, one of the same total 0.18 ms, and the first call waits for them
  // before its first copy.
  const size_t a8 = (n * 8 + 255) & ~(size_t)255, a4 = (n * 4 + 255) & ~(size_t)255;
  if (!CK(cudaMalloc(&s.slab, (size_t)(kNumFields + kNumGrid - 1 + 4 + 3) * a8 + a4)))
    return false;
  char* cut = static_cast<char*>(s.slab);
  auto take = [&cut](size_t bytes) {
    char* p = cut;
    cut += bytes;
    return p;
  };
  for (int k = 0; k < kNumFields; k++) *field_slot(s.dev, k) = (double*)take(a8);
  s.dev.tmask = (int*)take(a4);
  for (int k = 1; k < kNumGrid; k++) *grid_slot(s.dev, k) = (double*)take(a8);
  s.dev.sin_u = (double*)take(a8);
  s.dev.sin_v = (double*)take(a8);
  s.dev.r_hu = (double*)take(a8);
  s.dev.r_hv = (double*)take(a8);
  for (double*& p : s.shadow) p = (double*)take(a8);
  if (!s.partials &&
      !CK(cudaMalloc(&s.partials, sizeof(double) * checksum_partials_needed())))
    return false;
  s.sc = sc;
  s.cur = 0;
  s.shadows_synced = false;
  s.materialized = true;
  s.last_path = 0;
  // Speculation pays only when the other arrays' copies do not hold the
  // host: pinned sources, the FP64 fused path.  With the step arrays pinned
  // too, they go up in row bands that the first step follows.
  bool spec = speculate && s.precision == 0 && s.mode == NL2D_MODE_AUTO;
  for (int k : kLateArrays) spec = spec && host_pinned(ptrs[k]);
  bool banded = spec;
  for (int k : kStepArrays) banded = banded && host_pinned(ptrs[k]);
  if (banded) {
    if (!ensure_side()) return false;
    for (int b = 0; b < State::kMaxBands; b++)
      if (!s.band_up[b] && !CK(cudaEventCreateWithFlags(&s.band_up[b], cudaEventDisableTiming)))
        return false;
    if (!s.backups_done &&
        !CK(cudaEventCreateWithFlags(&s.backups_done, cudaEventDisableTiming)))
      return false;
    int th = 0;
    const int ntr = fused_step_tile_rows(dims(), &th);
    s.nbands = std::min(State::kMaxBands, ntr);
    for (int b = 0; b <= s.nbands; b++) {
      s.band_tile[b] = (int)((long long)ntr * b / s.nbands);
      s.band_row[b] = b == 0 ? 0 : (b == s.nbands ? height : ys - 1 + s.band_tile[b] * th);
    }
    for (int b = 0; b < s.nbands; b++) {
      for (int k : kStepArrays)
        if (!upload_rows(ptrs, k, s.band_row[b], s.band_row[b + 1], s.side)) return false;
      if (!CK(cudaEventRecord(s.band_up[b], s.side))) return false;
    }
  } else {
    // The arrays a fused step reads first (a pageable copy returns once its
    // source is staged, a pinned one at once).
    for (int k : kStepArrays)
      if (!upload(ptrs, k, s.stream)) return false;
    launch_depth_reciprocals(s.dev, dims(), s.stream);
    if (!CK(cudaGetLastError())) return false;
  }
  if (!spec) {
    for (int k : kLateArrays)
      if (!upload(ptrs, k, s.stream)) return false;
    if (!scan_grid(sc.d2r)) return false;
    // A state that is already what a step leaves needs no reference-
    // structured first step.
    s.consistent =
        s.fused_ok && (s.scan_flags & (kScanSshaT | kScanCopies | kScanNextSsh)) == 0;
    return true;
  }
  if (!ensure_side()) return false;
  if (!s.ess_done && (!CK(cudaEventCreateWithFlags(&s.ess_done, cudaEventDisableTiming)) ||
                      !CK(cudaEventCreateWithFlags(&s.spec_ready, cudaEventDisableTiming))))
    return false;
  if (!s.spec_out && !CK(cudaMallocHost(&s.spec_out, sizeof(State::SpecOut)))) return false;
  double* prim[3] = {s.dev.sshn_t, s.dev.un, s.dev.vn};
  // the backups of the uploaded state: on the side stream behind the bands
  // (the second step, which overwrites their source, waits for them), else
  // on the library's stream before the first step
  cudaStream_t bst = banded ? s.side : s.stream;
  for (int q = 0; q < 3; q++)
    if (!CK(cudaMalloc(&s.spec_backup[q], n * 8)) ||
        !CK(cudaMemcpyAsync(s.spec_backup[q], prim[q], n * 8, cudaMemcpyDeviceToDevice, bst)))
      return false;
  if (banded && !CK(cudaEventRecord(s.backups_done, s.side))) return false;
  // the other arrays and the scan behind the first steps, on the side
  // stream (nothing on the library's stream reads those arrays before the
  // verdict: resolve_spec makes it wait for them)
  if (!banded && (!CK(cudaEventRecord(s.ess_done, s.stream)) ||
                  !CK(cudaStreamWaitEvent(s.side, s.ess_done, 0))))
    return false;
  for (int k : kLateArrays)
    if (!upload(ptrs, k, s.side)) return false;
  // the scan checks the uploaded state in its backup: the steps taken
  // meanwhile overwrite the primary buffers
  if (!launch_scan(s.side, &s.spec_out->flags, s.spec_out->refs, s.spec_backup) ||
      !CK(cudaEventRecord(s.spec_ready, s.side)))
    return false;
  // Until then the fused path runs on the values the scan will compare
  // against: the region's first point of each metric array and the first
  // latitudes, read from the caller's arrays (the device copies are the same
  // bytes), and assumes the state is what a step leaves.
  const size_t o = (size_t)(ys - 1) * width + (xs - 1);
  double refs[11];
  for (int q = 0; q < 11; q++)
    refs[q] = static_cast<const double*>(ptrs[kNumFields + 1 + q])[q < 9 ? o : 0];
  for (int q = 0; q < 11; q++) s.grid_refs[q] = refs[q];
  double* um[9] = {&s.um.area_t, &s.um.area_u, &s.um.area_v, &s.um.dx_u, &s.um.dx_v,
                   &s.um.dx_t,   &s.um.dy_u,   &s.um.dy_v,   &s.um.dy_t};
  for (int q = 0; q < 9; q++) *um[q] = refs[q];
  s.um.sin_u = std::sin(refs[9] * sc.d2r);
  s.um.sin_v = std::sin(refs[10] * sc.d2r);
  s.sin_d2r = sc.d2r;
  s.scan_flags = 0;
  s.fused_ok = true;
  s.chain_u = s.chain_v = false;
  s.consistent = true;
  s.spec_pending = true;
  s.spec_steps.clear();
  s.bands_pending = banded;
  return true;
}

bool one_step(int istep);

// Makes what the banded first step would have made band by band (the depth
// reciprocals) when something else comes first, and orders the library's
// stream behind the bands and the backups.
bool finish_bands() {
  State& s = g_state;
  if (!s.bands_pending) return true;
  s.bands_pending = false;
  if (!CK(cudaStreamWaitEvent(s.stream, s.band_up[s.nbands - 1], 0)) ||
      !CK(cudaStreamWaitEvent(s.stream, s.backups_done, 0)))
    return false;
  launch_depth_reciprocals(s.dev, dims(), s.stream);
  return CK(cudaGetLastError());
}

// The first fused step of a banded registration: band b's tiles run once
// rows up to the end of band b + 1 are on the device (the tiles read two
// rows beyond their own, and a Flather face's momentum the reciprocal depth
// of the next row), after that band's depth reciprocals and shadow rows.
bool banded_first_step(const FusedState& fs, double tide) {
  State& s = g_state;
  s.bands_pending = false;
  const Dims d = dims();
  const size_t w = (size_t)s.reg.width;
  double* prim[3] = {s.dev.sshn_t, s.dev.un, s.dev.vn};
  for (int b = 0; b < s.nbands; b++) {
    const int nb = std::min(b + 1, s.nbands - 1);
    if (b == 0) {
      if (!CK(cudaStreamWaitEvent(s.stream, s.band_up[0], 0))) return false;
      launch_depth_reciprocals(s.dev, d, s.stream, s.band_row[0], s.band_row[1]);
    }
    if (nb > b) {
      if (!CK(cudaStreamWaitEvent(s.stream, s.band_up[nb], 0))) return false;
      launch_depth_reciprocals(s.dev, d, s.stream, s.band_row[nb], s.band_row[nb + 1]);
    }
    // the shadows (this step's output buffers) equal the uploaded state
    // outside the copy region
    const size_t off = s.band_row[b] * w, cnt = (s.band_row[b + 1] - s.band_row[b]) * w;
    for (int q = 0; q < 3; q++)
      if (!CK(cudaMemcpyAsync(s.shadow[q] + off, prim[q] + off, cnt * 8,
                              cudaMemcpyDeviceToDevice, s.stream)))
        return false;
    launch_fused_step_rows(s.dev, fs, d, s.sc, s.um, tide, s.band_tile[b], s.band_tile[b + 1],
                           s.stream);
  }
  s.shadows_synced = true;
  // the next step writes the primaries, which the backups copy
  return CK(cudaStreamWaitEvent(s.stream, s.backups_done, 0));
}

// Ends a speculative registration.  With wait false it returns at once
// unless the scan has answered.  The verdict either keeps the steps taken
// (the fused path's preconditions hold, the state was what a step leaves,
// the values assumed are the device's) or restores the uploaded sshn_t,
// un, vn and takes the same steps again by the path rules the scan decides,
// which gives the bits an unspeculative run gives.  Returns false on a CUDA
// error.
bool resolve_spec(bool wait) {
  State& s = g_state;
  if (!s.spec_pending) return true;
  if (!wait) {
    const cudaError_t q = cudaEventQuery(s.spec_ready);
    if (q == cudaErrorNotReady) return true;
    if (!CK(q)) return false;
  } else if (!CK(cudaEventSynchronize(s.spec_ready))) {
    return false;
  }
  if (!finish_bands()) return false;
  s.spec_pending = false;
  std::vector<int> steps;
  steps.swap(s.spec_steps);
  double assumed[11];
  for (int q = 0; q < 11; q++) assumed[q] = s.grid_refs[q];
  if (!CK(cudaStreamWaitEvent(s.stream, s.spec_ready, 0)) ||
      !apply_scan(s.spec_out->flags, s.spec_out->refs, s.sc.d2r))
    return false;
  const bool same = memcmp(assumed, s.grid_refs, sizeof assumed) == 0;
  const bool consistent =
      s.fused_ok && (s.scan_flags & (kScanSshaT | kScanCopies | kScanNextSsh)) == 0;
  bool ok = true;
  if (s.fused_ok && consistent && same) {
    s.spec_kept++;
  } else {
    s.spec_redone++;
    double* prim[3] = {s.dev.sshn_t, s.dev.un, s.dev.vn};
    const size_t n = (size_t)s.reg.width * s.reg.height;
    for (int q = 0; q < 3 && ok; q++)
      ok = CK(cudaMemcpyAsync(prim[q], s.spec_backup[q], n * 8, cudaMemcpyDeviceToDevice,
                              s.stream));
    s.cur = 0;
    s.shadows_synced = false;
    s.materialized = true;
    s.consistent = consistent;
    s.last_path = 0;
    invalidate_graph();
    for (size_t t = 0; t < steps.size() && ok; t++) ok = one_step(steps[t]);
    // the restoring copies read the backups: let them finish first
    ok = ok && CK(cudaStreamSynchronize(s.stream));
  }
  // (without a rollback nothing reads them: their copies finished before
  // the side stream started)
  for (double*& p : s.spec_backup) {
    cudaFree(p);
    p = nullptr;
  }
  return ok;
}


// Current device buffers of sshn_t / un / vn.
double* cur_sshn() { return g_state.cur ? g_state.shadow[0] : g_state.dev.sshn_t; }
double* cur_un() { return g_state.cur ? g_state.shadow[1] : g_state.dev.un; }
double* cur_vn() { return g_state.cur ? g_state.shadow[2] : g_state.dev.vn; }

bool sync_from_mixed();
bool ensure_df();

// Brings the primary device arrays to exactly what the reference would hold
// after the steps taken so far (for the mixed form: the FP64 image of its
// state).
bool materialize() {
  State& s = g_state;
  if (!sync_from_mixed()) return false;
  if (s.materialized) return true;
  if (s.cur) {  // the current state lives in the shadows: swap the roles
    std::swap(s.dev.sshn_t, s.shadow[0]);
    std::swap(s.dev.un, s.shadow[1]);
    std::swap(s.dev.vn, s.shadow[2]);
    s.cur = 0;
    invalidate_graph();  // it holds the old buffer roles
  }
  const Dims d = dims();
  // The copies of time_step.cpp:114-122 make un == ua, vn == va and
  // sshn_t == ssha_t on the copy region; outside it the fused step leaves
  // those arrays unchanged.  sshn_u / sshn_v are what next_sshu / next_sshv
  // make of the current sshn_t.
  launch_copy_region(s.dev.un, s.dev.ua, d, s.stream);
  launch_copy_region(s.dev.vn, s.dev.va, d, s.stream);
  launch_copy_region(s.dev.sshn_t, s.dev.ssha_t, d, s.stream);
  launch_next_ssh(s.dev, d, s.stream);
  if (!CK(cudaGetLastError())) return false;
  s.materialized = true;
  return true;
}

bool sync_shadows() {
  State& s = g_state;
  if (s.shadows_synced) return true;
  const size_t n = (size_t)s.reg.width * s.reg.height * 8;
  double* prim[3] = {s.dev.sshn_t, s.dev.un, s.dev.vn};
  for (int k = 0; k < 3; k++)
    if (!CK(cudaMemcpyAsync(s.shadow[k], prim[k], n, cudaMemcpyDeviceToDevice, s.stream)))
      return false;
  s.shadows_synced = true;
  return true;
}

bool can_fuse() {
  const State& s = g_state;
  if (s.precision == 1) return s.mode == NL2D_MODE_AUTO && s.fused_ok;
  return s.mode == NL2D_MODE_AUTO && s.fused_ok && s.consistent;
}

bool reference_step(int istep) {
  State& s = g_state;
  if (!finish_bands() || !materialize()) return false;
  launch_reference_step(s.dev, dims(), s.sc, istep, s.chain_u, s.chain_v, s.stream);
  if (!CK(cudaGetLastError())) return false;
  s.mixed_valid = false;
  s.consistent = true;
  s.shadows_synced = false;
  s.last_path = 1;
  return true;
}

void fused_launch(const double* tide_table, int tide_index, double tide) {
  State& s = g_state;
  if (s.precision == 1) {  // mixed form: ping-pong of the FP32 buffers
    MixedState ms;
    ms.sn_in = s.msn[s.mcur];
    ms.un_in = s.mun[s.mcur];
    ms.vn_in = s.mvn[s.mcur];
    ms.sn_out = s.msn[1 - s.mcur];
    ms.un_out = s.mun[1 - s.mcur];
    ms.vn_out = s.mvn[1 - s.mcur];
    launch_mixed_step(s.mix, ms, s.dev, dims(), s.sc, s.um, tide, tide_table, tide_index,
                      s.stream, s.side, s.side_fork, s.side_join);
    s.mcur = 1 - s.mcur;
    return;
  }
  s.mixed_valid = false;
  FusedState fs;
  fs.sshn_in = cur_sshn();
  fs.un_in = cur_un();
  fs.vn_in = cur_vn();
  const int nxt = 1 - s.cur;
  fs.sshn_out = nxt ? s.shadow[0] : s.dev.sshn_t;
  fs.un_out = nxt ? s.shadow[1] : s.dev.un;
  fs.vn_out = nxt ? s.shadow[2] : s.dev.vn;
  if (s.precision == 2) {
    // interior cells in double-float, the others in exact FP64, one launch
    launch_df_step(s.dev, fs, dims(), s.sc, s.um, s.dfs, tide, tide_table, tide_index, s.stream);
  } else if (s.bands_pending) {  // (never inside a graph: prepare_graph finishes them)
    banded_first_step(fs, tide);
  } else {
    launch_fused_step(s.dev, fs, dims(), s.sc, s.um, tide, tide_table, tide_index, s.stream);
  }
  s.cur = nxt;
}

// The FP64-equivalent form's static arrays (split depths and reciprocal
// denominators, march flags, the exact cells' list), made from the current
// FP64 arrays unless they already are.
bool ensure_df() {
  State& s = g_state;
  if (s.df_valid) return true;
  const Registration& r = s.reg;
  const size_t n = (size_t)r.width * r.height;
  if (!s.dfs.ht) {
    float2** arrs[5] = {&s.dfs.ht, &s.dfs.hu, &s.dfs.hv, &s.dfs.rhu, &s.dfs.rhv};
    for (float2** a : arrs)
      if (!CK(cudaMalloc(a, n * sizeof(float2)))) return false;
    if (!CK(cudaMalloc(&s.dfs.reg, n)) || !CK(cudaMalloc(&s.dfs.count, sizeof(int))))
      return false;
  }
  launch_df_setup(s.dev, dims(), s.dfs, s.stream);
  // two passes: count the exact cells, then list them
  cudaFree(s.dfs.ring);
  s.dfs.ring = nullptr;
  for (int pass = 0; pass < 2; pass++) {
    launch_df_ring(dims(), s.dfs, s.stream);
    int count = 0;
    if (!CK(cudaGetLastError()) ||
        !CK(cudaMemcpyAsync(&count, s.dfs.count, sizeof count, cudaMemcpyDeviceToHost,
                            s.stream)) ||
        !CK(cudaStreamSynchronize(s.stream)))
      return false;
    if (pass == 1 && count != s.dfs.n_ring) return false;
    s.dfs.n_ring = count;
    if (pass == 0 && !CK(cudaMalloc(&s.dfs.ring, sizeof(int) * std::max(1, count))))
      return false;
  }
  invalidate_graph();
  s.df_valid = true;
  return true;
}

// Converts the current FP64 state into the mixed buffers (both ping-pong
// partners, so cells no step writes agree) unless they already hold it.
bool ensure_mixed() {
  State& s = g_state;
  const size_t n = (size_t)s.reg.width * s.reg.height;
  if (!s.msn[0]) {
    for (int b = 0; b < 2; b++) {
      if (!CK(cudaMalloc(&s.msn[b], n * sizeof(float2))) ||
          !CK(cudaMalloc(&s.mun[b], n * sizeof(float))) ||
          !CK(cudaMalloc(&s.mvn[b], n * sizeof(float))))
        return false;
    }
    if (!CK(cudaMalloc(&s.mix.ht, n * 4)) || !CK(cudaMalloc(&s.mix.hu, n * 4)) ||
        !CK(cudaMalloc(&s.mix.hv, n * 4)) || !CK(cudaMalloc(&s.mix.rhu, n * 4)) ||
        !CK(cudaMalloc(&s.mix.rhv, n * 4)) || !CK(cudaMalloc(&s.mix.reg, n)) ||
        !CK(cudaMalloc(&s.mix.glist, n * sizeof(int))) ||
        !CK(cudaMalloc(&s.mix_count, sizeof(int))))
      return false;
    s.mixed_valid = false;
  }
  if (s.mixed_valid) return true;
  // the second stream and its events for the general cells' pass
  if (!ensure_side() ||
      (!s.side_fork && (!CK(cudaEventCreateWithFlags(&s.side_fork, cudaEventDisableTiming)) ||
                      !CK(cudaEventCreateWithFlags(&s.side_join, cudaEventDisableTiming)))))
    return false;
  if (!materialize()) return false;
  const Dims d = dims();
  for (int b = 0; b < 2; b++) {
    MixedState ms{};
    ms.sn_out = s.msn[b];
    ms.un_out = s.mun[b];
    ms.vn_out = s.mvn[b];
    launch_to_mixed(s.dev.sshn_t, s.dev.un, s.dev.vn, s.dev, s.mix, ms, d, b == 0, s.stream);
  }
  if (!CK(cudaGetLastError())) return false;
  // which cells the column march updates (the mask may have been rewritten)
  const int ng = launch_mixed_flags(s.dev, d, s.mix, s.mix_count, s.stream);
  if (ng < 0) {
    CK(cudaGetLastError());
    set_error(NL2D_ERR_CUDA, "mixed form: cell flags");
    return false;
  }
  s.mix.gcount = ng;
  s.mcur = 0;
  s.mixed_valid = true;
  s.mixed_ahead = false;
  invalidate_graph();
  return true;
}

// Writes the mixed state back into the FP64 arrays (sshn_t, un, vn; the
// derived arrays follow in materialize()).  The FP64 path then restarts
// with a reference-structured step.
bool sync_from_mixed() {
  State& s = g_state;
  if (!s.mixed_valid || !s.mixed_ahead) return true;
  if (s.cur) {
    std::swap(s.dev.sshn_t, s.shadow[0]);
    std::swap(s.dev.un, s.shadow[1]);
    std::swap(s.dev.vn, s.shadow[2]);
    s.cur = 0;
    invalidate_graph();
  }
  launch_from_mixed(s.msn[s.mcur], s.mun[s.mcur], s.mvn[s.mcur], s.dev.sshn_t, s.dev.un,
                    s.dev.vn, dims(), s.stream);
  if (!CK(cudaGetLastError())) return false;
  s.mixed_ahead = false;
  s.materialized = false;
  s.shadows_synced = false;
  s.consistent = false;
  return true;
}

bool fused_step(int istep) {
  State& s = g_state;
  if (s.precision != 0 && !finish_bands()) return false;
  if (s.precision == 1) {
    if (!ensure_mixed()) return false;
  } else if (!(s.bands_pending || sync_shadows()) || (s.precision == 2 && !ensure_df())) {
    return false;
  }
  fused_launch(nullptr, 0, tide_value(istep, s.sc.rdt));
  if (!CK(cudaGetLastError())) return false;
  if (s.precision == 1) {
    s.mixed_ahead = true;
    s.last_path = 3;
  } else {
    s.materialized = false;
    s.last_path = 2;
  }
  return true;
}

bool one_step(int istep) {
  const State& s = g_state;
  if (s.precision == 1) return s.fused_ok ? fused_step(istep) : reference_step(istep);
  return can_fuse() ? fused_step(istep) : reference_step(istep);
}

bool ensure_sums(int n) {
  State& s = g_state;
  if (s.sums_cap >= n) return true;
  invalidate_graph();  // a captured graph holds the old address
  if (s.sums) cudaFree(s.sums);
  s.sums = nullptr;
  s.sums_cap = 0;
  if (!CK(cudaMalloc(&s.sums, sizeof(double) * n))) return false;
  s.sums_cap = n;
  return true;
}

void enqueue_checksums(double* out3) {
  State& s = g_state;
  const Registration& r = s.reg;
  if (s.precision == 1 && s.mixed_valid) {
    launch_checksum_f2(s.msn[s.mcur], r.width, r.xs, r.xe, r.ys, r.ye, s.partials, out3,
                       s.stream);
    launch_checksum_f32(s.mun[s.mcur], r.width, r.xs, r.xe - 1, r.ys, r.ye, s.partials,
                        out3 + 1, s.stream);
    launch_checksum_f32(s.mvn[s.mcur], r.width, r.xs, r.xe, r.ys, r.ye - 1, s.partials,
                        out3 + 2, s.stream);
    return;
  }
  launch_checksum(cur_sshn(), r.width, r.xs, r.xe, r.ys, r.ye, s.partials, out3, s.stream);
  launch_checksum(cur_un(), r.width, r.xs, r.xe - 1, r.ys, r.ye, s.partials, out3 + 1,
                  s.stream);
  launch_checksum(cur_vn(), r.width, r.xs, r.xe, r.ys, r.ye - 1, s.partials, out3 + 2,
                  s.stream);
}

int find_field(const void* handle) {
  const State& s = g_state;
  if (!s.registered) return -1;
  for (int k = 0; k < kNumFields + kNumGrid; k++)
    if (s.reg.host[k] == handle) return k;
  return -1;
}

void* device_of(int k) {
  State& s = g_state;
  if (k < kNumFields) return *field_slot(s.dev, k);
  if (k == kNumFields) return s.dev.tmask;
  return *grid_slot(s.dev, k - kNumFields);
}

// Status handling for the int-returning entry points: each returns the
// error it raised itself; an older sticky error (from a void entry point)
// stays pending for nl2d_last_error().
struct CallScope {
  int saved;
  CallScope() : saved(g_state.status) { g_state.status = NL2D_OK; }
  int rc() const { return g_state.status; }
  ~CallScope() {
    if (g_state.status == NL2D_OK) g_state.status = saved;
  }
};

void invalidate_graph() {
  if (g_state.graph) cudaGraphExecDestroy(g_state.graph);
  g_state.graph = nullptr;
  for (int k = 0; k < 5; k++) g_state.graph_key[k] = -1;
}

// Uploads the tidal values of steps istep0 .. istep0+rest-1 and makes
// s.graph a graph of `rest` fused steps (with checksums after every
// checksum_every-th step counted from `done_before`), capturing it unless
// the cached one matches.  Nothing is launched; s.cur is left unchanged.
bool prepare_graph(int istep0, int rest, int checksum_every, int done_before) {
  State& s = g_state;
  if (!finish_bands()) return false;  // a graph's steps take the whole grid
  if (s.precision == 1 ? !ensure_mixed() : !sync_shadows()) return false;
  if (s.precision == 2 && !ensure_df()) return false;
  if (s.tide_cap < rest) {
    invalidate_graph();  // it holds the old table address
    if (s.tide_table) cudaFree(s.tide_table);
    s.tide_table = nullptr;
    s.tide_cap = 0;
    if (!CK(cudaMalloc(&s.tide_table, sizeof(double) * rest))) return false;
    s.tide_cap = rest;
  }
  std::vector<double> tides(rest);
  for (int q = 0; q < rest; q++) tides[q] = tide_value(istep0 + q, s.sc.rdt);
  if (!CK(cudaMemcpyAsync(s.tide_table, tides.data(), sizeof(double) * rest,
                          cudaMemcpyHostToDevice, s.stream)))
    return false;
  // pageable source: the copy is staged before the call returns
  const int phase = checksum_every > 0 ? done_before % checksum_every : 0;
  const int key[5] = {rest, checksum_every, phase, s.precision == 1 ? s.mcur : s.cur,
                      s.precision};
  if (s.graph && memcmp(key, s.graph_key, sizeof key) == 0) return true;
  invalidate_graph();
  const int cur0 = s.cur, mcur0 = s.mcur;
  cudaGraph_t graph;
  if (!CK(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal))) return false;
  for (int q = 0; q < rest; q++) {
    fused_launch(s.tide_table, q, 0.0);
    const int done = done_before + q + 1;
    if (checksum_every > 0 && done % checksum_every == 0)
      enqueue_checksums(s.sums + 3 * (done / checksum_every - 1));
  }
  s.cur = cur0;
  s.mcur = mcur0;
  if (!CK(cudaStreamEndCapture(s.stream, &graph))) return false;
  const bool ok = CK(cudaGraphInstantiate(&s.graph, graph, 0));
  cudaGraphDestroy(graph);
  if (!ok) return false;
  memcpy(s.graph_key, key, sizeof key);
  return true;
}

// Bookkeeping after a launched graph of n steps.
void advance_after_graph(int n) {
  State& s = g_state;
  if (s.precision == 1) {
    s.mcur = (s.mcur + n) & 1;
    s.mixed_ahead = true;
    s.last_path = 3;
  } else {
    s.cur = (s.cur + n) & 1;
    s.materialized = false;
    s.last_path = 2;
  }
}

}  // namespace
}  // namespace nl2d

using namespace nl2d;

#define NL2D_PTRS                                                                          \
  void* ptrs[kNumFields + kNumGrid] = {ssha_t, sshn_t, sshn_u, sshn_v, hu,   hv,    un,    \
                                       vn,     ua,     ht,     ssha_u, va,   ssha_v, tmask, \
                                       area_t, area_u, area_v, dx_u,   dx_v, dx_t,  dy_u,  \
                                       dy_v,   dy_t,   gphiu,  gphiv}

// ny rows of `width` bytes at the same pitch on both sides: one linear copy
// when the rows are whole (the usual read of a full field), else a 2-D one.
static bool copy_rows(char* dst, const char* src, size_t pitch, size_t width, int ny,
                      cudaMemcpyKind kind, cudaStream_t st) {
  if (width == pitch) return CK(cudaMemcpyAsync(dst, src, width * ny, kind, st));
  return CK(cudaMemcpy2DAsync(dst, pitch, src, pitch, width, ny, kind, st));
}

extern "C" {

void c_invoke_time_step(double* ssha_t, double* sshn_t, double* sshn_u, double* sshn_v,
                        double* hu, double* hv, double* un, double* vn, double* ua,
                        double* ht, double* ssha_u, double* va, double* ssha_v, int* tmask,
                        double* area_t, double* area_u, double* area_v, double* dx_u,
                        double* dx_v, double* dx_t, double* dy_u, double* dy_v, double* dy_t,
                        double* gphiu, double* gphiv, int istep, int internal_xstart,
                        int internal_xstop, int internal_ystart, int internal_ystop,
                        int width, int height, double rdt, double cbfr, double visc,
                        double omega, double d2r, double g) {
  nl2d::NvtxRange nvtx_range("c_invoke_time_step");
  NL2D_PTRS;
  State& s = g_state;
  const Scalars sc{rdt, cbfr, visc, omega, d2r, g};
  if (!same_registration(ptrs, internal_xstart, internal_xstop, internal_ystart,
                         internal_ystop, width, height)) {
    if (!do_register(ptrs, internal_xstart, internal_xstop, internal_ystart, internal_ystop,
                     width, height, sc, true))
      return;
  } else {
    // steps taken before the scan's verdict are replayed with the
    // registration's scalars: new ones wait for the verdict
    if (s.spec_pending && memcmp(&sc, &s.sc, sizeof sc) != 0 && !resolve_spec(true)) return;
    s.sc = sc;
    if (!(d2r == s.sin_d2r) && !update_sines(d2r)) return;
  }
  if (s.spec_pending && !resolve_spec(false)) return;
  if (!one_step(istep)) return;
  if (s.spec_pending) s.spec_steps.push_back(istep);
}

int nl2d_register(double* ssha_t, double* sshn_t, double* sshn_u, double* sshn_v, double* hu,
                  double* hv, double* un, double* vn, double* ua, double* ht, double* ssha_u,
                  double* va, double* ssha_v, int* tmask, double* area_t, double* area_u,
                  double* area_v, double* dx_u, double* dx_v, double* dx_t, double* dy_u,
                  double* dy_v, double* dy_t, double* gphiu, double* gphiv,
                  int internal_xstart, int internal_xstop, int internal_ystart,
                  int internal_ystop, int width, int height, double rdt, double cbfr,
                  double visc, double omega, double d2r, double g) {
  nl2d::NvtxRange nvtx_range("nl2d_register");
  NL2D_PTRS;
  CallScope scope;
  const Scalars sc{rdt, cbfr, visc, omega, d2r, g};
  do_register(ptrs, internal_xstart, internal_xstop, internal_ystart, internal_ystop, width,
              height, sc);
  return scope.rc();
}

void c_read_from_device(void* from, void* to, int startx, int starty, int nx, int ny,
                        bool blocking) {
  nl2d::NvtxRange nvtx_range("c_read_from_device");
  if (!resolve_spec(true)) return;
  State& s = g_state;
  const int k = find_field(from);
  if (k < 0) {
    set_error(NL2D_ERR_UNKNOWN_FIELD, "c_read_from_device: %p is not a registered field",
              from);
    return;
  }
  const Registration& r = s.reg;
  if (startx < 1 || starty < 1 || nx < 0 || ny < 0 || startx - 1 + nx > r.width ||
      starty - 1 + ny > r.height) {
    set_error(NL2D_ERR_ARGS, "c_read_from_device: region outside the %dx%d field", r.width,
              r.height);
    return;
  }
  // sshn_t, un and vn are read from the buffers that hold the current state
  // (the fused path's ping-pong partner agrees with the primary outside the
  // copy region); every other array is made what the reference holds first.
  const void* src = nullptr;
  if ((k == 1 || k == 6 || k == 7) && !(s.mixed_valid && s.mixed_ahead))
    src = k == 1 ? cur_sshn() : (k == 6 ? cur_un() : cur_vn());
  else if (!materialize())
    return;
  else
    src = device_of(k);
  const size_t esz = k == kNumFields ? 4 : 8, pitch = (size_t)r.width * esz;
  const size_t off = ((size_t)(starty - 1) * r.width + (startx - 1)) * esz;
  if (nx == 0 || ny == 0) return;
  if (!copy_rows((char*)to + off, (const char*)src + off, pitch, nx * esz, ny,
                 cudaMemcpyDeviceToHost, s.stream))
    return;
  s.d2h_bytes += (long long)nx * ny * (long long)esz;
  if (blocking) CK(cudaStreamSynchronize(s.stream));
}

void c_write_to_device(void* from, void* to, int startx, int starty, int nx, int ny,
                       bool blocking) {
  nl2d::NvtxRange nvtx_range("c_write_to_device");
  if (!resolve_spec(true)) return;
  State& s = g_state;
  const int k = find_field(to);
  if (k < 0) {
    set_error(NL2D_ERR_UNKNOWN_FIELD, "c_write_to_device: %p is not a registered field", to);
    return;
  }
  const Registration& r = s.reg;
  if (startx < 1 || starty < 1 || nx < 0 || ny < 0 || startx - 1 + nx > r.width ||
      starty - 1 + ny > r.height) {
    set_error(NL2D_ERR_ARGS, "c_write_to_device: region outside the %dx%d field", r.width,
              r.height);
    return;
  }
  if (k >= kNumFields && from != to) {
    set_error(NL2D_ERR_ARGS,
              "c_write_to_device: a grid array is written from its registered host array");
    return;
  }
  if (!materialize()) return;
  const size_t esz = k == kNumFields ? 4 : 8, pitch = (size_t)r.width * esz;
  const size_t off = ((size_t)(starty - 1) * r.width + (startx - 1)) * esz;
  if (nx > 0 && ny > 0 &&
      !copy_rows((char*)device_of(k) + off, (const char*)from + off, pitch, nx * esz, ny,
                 cudaMemcpyHostToDevice, s.stream))
    return;
  s.h2d_bytes += (long long)nx * ny * (long long)esz;
  // Any written array may break the fused path's preconditions: re-derive
  // them from the host copies where they can change, and take the next step
  // on the reference-structured path.
  s.consistent = false;
  s.shadows_synced = false;
  s.df_valid = false;  // its split statics and flags may be stale
  if (k == 4 || k == 5 || k == 10 || k == 12) {  // hu, hv, ssha_u, ssha_v
    launch_depth_reciprocals(s.dev, dims(), s.stream);
    if (!CK(cudaGetLastError())) return;
  }
  if (k >= kNumFields && !scan_grid(s.sc.d2r)) return;
  if (blocking) CK(cudaStreamSynchronize(s.stream));
}

// ---- checkpoint / resume (no reference counterpart) ----
// A checkpoint is the 13 fields exactly as c_read_from_device returns them
// (FP64, row-major [height][width], in c_invoke_time_step's order) after an
// 8-byte magic and eleven int32s: version, width, height, xs, xe, ys, ye,
// istep, field count, two reserved.  The grid (mask, metrics) is not in it:
// it comes from the namelist and set-up the caller repeats.
struct CheckpointHeader {
  char magic[8];
  int32_t version, width, height, xs, xe, ys, ye, istep, nfields, reserved[2];
};
constexpr char kCheckpointMagic[8] = {'N', 'L', '2', 'D', 'C', 'K', 'P', '1'};

int nl2d_checkpoint_write(const char* path, int istep) {
  nl2d::NvtxRange nvtx_range("nl2d_checkpoint_write");
  State& s = g_state;
  CallScope scope;
  if (!resolve_spec(true)) return scope.rc();
  if (!s.registered) {
    set_error(NL2D_ERR_STATE, "nl2d_checkpoint_write: no problem registered");
    return scope.rc();
  }
  if (!path) {
    set_error(NL2D_ERR_ARGS, "nl2d_checkpoint_write: path is NULL");
    return scope.rc();
  }
  if (!materialize()) return scope.rc();
  const Registration& r = s.reg;
  const size_t n = (size_t)r.width * r.height;
  std::vector<double> buf(n);
  FILE* f = fopen(path, "wb");
  if (!f) {
    set_error(NL2D_ERR_IO, "nl2d_checkpoint_write: cannot open %s", path);
    return scope.rc();
  }
  CheckpointHeader h{};
  memcpy(h.magic, kCheckpointMagic, 8);
  h.version = 1, h.width = r.width, h.height = r.height, h.xs = r.xs, h.xe = r.xe;
  h.ys = r.ys, h.ye = r.ye, h.istep = istep, h.nfields = kNumFields;
  bool ok = fwrite(&h, sizeof h, 1, f) == 1;
  for (int k = 0; k < kNumFields && ok; k++) {
    ok = CK(cudaMemcpyAsync(buf.data(), device_of(k), n * 8, cudaMemcpyDeviceToHost,
                            s.stream)) &&
         CK(cudaStreamSynchronize(s.stream));
    if (ok) ok = fwrite(buf.data(), 8, n, f) == n;
  }
  if (fclose(f) != 0) ok = false;
  if (!ok && s.status == NL2D_OK)
    set_error(NL2D_ERR_IO, "nl2d_checkpoint_write: writing %s", path);
  return scope.rc();
}

int nl2d_checkpoint_read(const char* path, int* istep) {
  nl2d::NvtxRange nvtx_range("nl2d_checkpoint_read");
  State& s = g_state;
  CallScope scope;
  if (!resolve_spec(true)) return scope.rc();
  if (!s.registered) {
    set_error(NL2D_ERR_STATE, "nl2d_checkpoint_read: no problem registered");
    return scope.rc();
  }
  if (!path || !istep) {
    set_error(NL2D_ERR_ARGS, "nl2d_checkpoint_read: NULL argument");
    return scope.rc();
  }
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_error(NL2D_ERR_IO, "nl2d_checkpoint_read: cannot open %s", path);
    return scope.rc();
  }
  const Registration& r = s.reg;
  CheckpointHeader h{};
  if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, kCheckpointMagic, 8) != 0 ||
      h.version != 1 || h.nfields != kNumFields) {
    fclose(f);
    set_error(NL2D_ERR_PARSE, "nl2d_checkpoint_read: %s is not a checkpoint", path);
    return scope.rc();
  }
  if (h.width != r.width || h.height != r.height || h.xs != r.xs || h.xe != r.xe ||
      h.ys != r.ys || h.ye != r.ye) {
    fclose(f);
    set_error(NL2D_ERR_ARGS, "nl2d_checkpoint_read: %s holds a %dx%d problem, not %dx%d", path,
              h.width, h.height, r.width, r.height);
    return scope.rc();
  }
  if (!materialize()) {
    fclose(f);
    return scope.rc();
  }
  const size_t n = (size_t)r.width * r.height;
  std::vector<double> buf(n);
  bool ok = true;
  for (int k = 0; k < kNumFields && ok; k++) {
    ok = fread(buf.data(), 8, n, f) == n;
    if (!ok) {
      set_error(NL2D_ERR_IO, "nl2d_checkpoint_read: %s is truncated", path);
      break;
    }
    ok = CK(cudaMemcpyAsync(device_of(k), buf.data(), n * 8, cudaMemcpyHostToDevice,
                            s.stream)) &&
         CK(cudaStreamSynchronize(s.stream));
  }
  fclose(f);
  if (!ok) return scope.rc();
  // as after c_write_to_device: the next step is reference-structured
  s.consistent = false;
  s.shadows_synced = false;
  s.df_valid = false;  // its split statics and flags may be stale
  s.mixed_valid = s.mixed_ahead = false;
  launch_depth_reciprocals(s.dev, dims(), s.stream);
  if (!CK(cudaGetLastError()) || !CK(cudaStreamSynchronize(s.stream))) return scope.rc();
  *istep = h.istep;
  return scope.rc();
}

int nl2d_last_error(char* msg, int msg_len) {
  State& s = g_state;
  const int st = s.status;
  if (msg && msg_len > 0) {
    strncpy(msg, s.msg, msg_len - 1);
    msg[msg_len - 1] = '\0';
  }
  s.status = NL2D_OK;
  s.msg[0] = '\0';
  return st;
}

void nl2d_finalize(void) {
  State& s = g_state;
  if (s.stream) cudaStreamSynchronize(s.stream);
  free_device();
  if (s.partials) cudaFree(s.partials);
  if (s.sums) cudaFree(s.sums);
  if (s.tide_table) cudaFree(s.tide_table);
  if (s.scan) cudaFree(s.scan);
  s.partials = s.sums = s.tide_table = s.scan = nullptr;
  s.sums_cap = s.tide_cap = 0;
  if (s.stream) cudaStreamDestroy(s.stream);
  s.stream = nullptr;
  if (s.side) cudaStreamDestroy(s.side);
  s.side = nullptr;
  if (s.ess_done) cudaEventDestroy(s.ess_done);
  if (s.spec_ready) cudaEventDestroy(s.spec_ready);
  s.ess_done = s.spec_ready = nullptr;
  if (s.side_fork) cudaEventDestroy(s.side_fork);
  if (s.side_join) cudaEventDestroy(s.side_join);
  s.side_fork = s.side_join = nullptr;
  if (s.spec_out) cudaFreeHost(s.spec_out);
  s.spec_out = nullptr;
  noalloc_forget();
}

int nl2d_set_mode(int mode) {
  resolve_spec(true);  // steps taken before the verdict keep their path rules
  State& s = g_state;
  const int old = s.mode;
  if (mode != NL2D_MODE_AUTO && mode != NL2D_MODE_REFERENCE) {
    set_error(NL2D_ERR_ARGS, "nl2d_set_mode: unknown mode %d", mode);
    return old;
  }
  s.mode = mode;
  return old;
}

int nl2d_last_path(void) { return g_state.last_path; }

int nl2d_set_precision(int precision) {
  resolve_spec(true);  // steps taken before the verdict keep their path rules
  State& s = g_state;
  const int old = s.precision;
  if (precision < 0 || precision > 2) {
    set_error(NL2D_ERR_ARGS, "nl2d_set_precision: unknown precision %d", precision);
    return old;
  }
  if (precision != old) {
    if (old == 1) sync_from_mixed();  // keep the mixed state, now in FP64
    s.precision = precision;
    invalidate_graph();
  }
  return old;
}

int nl2d_run_steps(int istep0, int nsteps, int checksum_every, double* checksums_out) {
  nl2d::NvtxRange nvtx_range("nl2d_run_steps");
  State& s = g_state;
  CallScope scope;
  if (!resolve_spec(true)) return scope.rc();
  if (!s.registered) {
    set_error(NL2D_ERR_STATE, "nl2d_run_steps: no problem registered");
    return scope.rc();
  }
  if (nsteps < 0 || checksum_every < 0) {
    set_error(NL2D_ERR_ARGS, "nl2d_run_steps: negative count");
    return scope.rc();
  }
  const int nsums = checksum_every > 0 ? nsteps / checksum_every : 0;
  if (nsums > 0 && !checksums_out) {
    set_error(NL2D_ERR_ARGS, "nl2d_run_steps: checksums_out is NULL");
    return scope.rc();
  }
  if (!ensure_sums(3 * (nsums > 0 ? nsums : 1))) return scope.rc();
  int k = 0;
  // The first step after an upload (or in reference mode, every step) runs
  // on the reference-structured path.
  while (k < nsteps && !can_fuse()) {
    if (!reference_step(istep0 + k)) return scope.rc();
    k++;
    if (checksum_every > 0 && k % checksum_every == 0)
      enqueue_checksums(s.sums + 3 * (k / checksum_every - 1));
  }
  const int rest = nsteps - k;
  if (rest > 0) {
    if (!prepare_graph(istep0 + k, rest, checksum_every, k)) return scope.rc();
    if (!CK(cudaGraphLaunch(s.graph, s.stream))) return scope.rc();
    advance_after_graph(rest);
  }
  if (nsums > 0) {
    if (!CK(cudaMemcpyAsync(checksums_out, s.sums, sizeof(double) * 3 * nsums,
                            cudaMemcpyDeviceToHost, s.stream)))
      return scope.rc();
    CK(cudaStreamSynchronize(s.stream));
  }
  return scope.rc();
}

int nl2d_timed_run(int istep0, int nsteps, double* ms_out) {
  nl2d::NvtxRange nvtx_range("nl2d_timed_run");
  State& s = g_state;
  CallScope scope;
  if (!resolve_spec(true)) return scope.rc();
  if (ms_out) *ms_out = 0.0;
  if (!s.registered) {
    set_error(NL2D_ERR_STATE, "nl2d_timed_run: no problem registered");
    return scope.rc();
  }
  if (nsteps < 1) return scope.rc();
  if (!can_fuse()) {
    if (s.mode != NL2D_MODE_AUTO || !s.fused_ok) {
      set_error(NL2D_ERR_STATE, "nl2d_timed_run: the fused path does not apply");
      return scope.rc();
    }
    // The untimed first step makes the state step-consistent.
    if (!reference_step(istep0)) return scope.rc();
    istep0++;
    if (--nsteps < 1) return scope.rc();
  }
  // Everything before the timed launch (shadow copies, tide upload, graph
  // capture) completes first, outside the timed region.
  if (!prepare_graph(istep0, nsteps, 0, 0) || !CK(cudaStreamSynchronize(s.stream)))
    return scope.rc();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (CK(cudaEventCreate(&e0)) && CK(cudaEventCreate(&e1)) &&
      CK(cudaEventRecord(e0, s.stream)) && CK(cudaGraphLaunch(s.graph, s.stream)) &&
      CK(cudaEventRecord(e1, s.stream)) && CK(cudaEventSynchronize(e1))) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms_out) *ms_out = ms;
    advance_after_graph(nsteps);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return scope.rc();
}

int nl2d_checksums(double out[3]) {
  nl2d::NvtxRange nvtx_range("nl2d_checksums");
  State& s = g_state;
  CallScope scope;
  if (!resolve_spec(true)) return scope.rc();
  auto take_status = [&]() { return scope.rc(); };
  if (!s.registered) {
    set_error(NL2D_ERR_STATE, "nl2d_checksums: no problem registered");
    return take_status();
  }
  if (!ensure_sums(3)) return take_status();
  enqueue_checksums(s.sums);
  if (!CK(cudaMemcpyAsync(out, s.sums, sizeof(double) * 3, cudaMemcpyDeviceToHost,
                          s.stream)))
    return take_status();
  if (!CK(cudaStreamSynchronize(s.stream))) return take_status();
  for (int k = 0; k < 3; k++)
    if (!std::isfinite(out[k])) {
      set_error(NL2D_ERR_NONFINITE, "checksum %d is not finite", k);
      break;
    }
  return take_status();
}

int nl2d_field_checksum(const void* field, int x0, int x1, int y0, int y1, double* out) {
  State& s = g_state;
  CallScope scope;
  if (!resolve_spec(true)) return scope.rc();
  auto take_status = [&]() { return scope.rc(); };
  const int k = find_field(field);
  if (k < 0 || k >= kNumFields) {
    set_error(NL2D_ERR_UNKNOWN_FIELD, "nl2d_field_checksum: %p is not a registered field",
              field);
    return take_status();
  }
  const Registration& r = s.reg;
  if (x0 < 0 || y0 < 0 || x1 >= r.width || y1 >= r.height) {
    set_error(NL2D_ERR_ARGS, "nl2d_field_checksum: region outside the field");
    return take_status();
  }
  if (!materialize() || !ensure_sums(3)) return take_status();
  launch_checksum((const double*)device_of(k), r.width, x0, x1, y0, y1, s.partials, s.sums,
                  s.stream);
  if (!CK(cudaMemcpyAsync(out, s.sums, sizeof(double), cudaMemcpyDeviceToHost, s.stream)))
    return take_status();
  CK(cudaStreamSynchronize(s.stream));
  return take_status();
}

int nl2d_sync(void) {
  State& s = g_state;
  CallScope scope;
  if (!resolve_spec(true)) return scope.rc();
  if (s.stream) CK(cudaStreamSynchronize(s.stream));
  return scope.rc();
}

int nl2d_transfer_bytes(long long out[2]) {
  const State& s = g_state;
  if (!out) return NL2D_ERR_ARGS;
  out[0] = s.h2d_bytes;
  out[1] = s.d2h_bytes;
  return NL2D_OK;
}

int nl2d_speculation_counts(int out[2]) {
  if (!out) return NL2D_ERR_ARGS;
  out[0] = g_state.spec_kept;
  out[1] = g_state.spec_redone;
  return NL2D_OK;
}

int nl2d_host_register(void* p, size_t bytes) {
  CallScope scope;
  if (!p || bytes == 0) {
    set_error(NL2D_ERR_ARGS, "nl2d_host_register: null pointer or zero size");
    return scope.rc();
  }
  CK(cudaHostRegister(p, bytes, cudaHostRegisterDefault));
  return scope.rc();
}

int nl2d_host_unregister(void* p) {
  CallScope scope;
  if (!p) {
    set_error(NL2D_ERR_ARGS, "nl2d_host_unregister: null pointer");
    return scope.rc();
  }
  CK(cudaHostUnregister(p));
  return scope.rc();
}

void* nl2d_device_ptr(const void* field) {
  if (!resolve_spec(true)) return nullptr;
  const int k = find_field(field);
  if (k < 0) return nullptr;
  if (!materialize()) return nullptr;
  return device_of(k);
}

}  // extern "C"
