// Internal types shared by the NEMOLite2D GPU translation units.
//
// Layout in HBM: every field is a row-major [height][width] FP64 array with
// element (ji, jj) at jj*width + ji (0-based), exactly the layout of a
// dl_esm_inf r2d_field's `data(width, height)` seen from C.  The T-mask is
// the same shape in int32.  The internal T region is [xs,xe] x [ys,ye].
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <cstdint>

#include "nl2d_df.cuh"

namespace nl2d {

// An NVTX range for the lifetime of the object: each public entry point
// names itself in a profiler's timeline (a no-op unless a tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Device copies of the 13 fields and 12 grid arrays that
// c_invoke_time_step receives (psykal_cpp/time_step.cpp:10-51), plus the
// Coriolis sines sin(gphi*d2r) evaluated once on the host with the host's
// libm (the reference evaluates them per point with the same libm).
struct Fields {
  double *ssha_t, *sshn_t, *sshn_u, *sshn_v, *hu, *hv, *un, *vn, *ua, *ht,
      *ssha_u, *va, *ssha_v;
  int* tmask;
  double *area_t, *area_u, *area_v, *dx_u, *dx_v, *dx_t, *dy_u, *dy_v, *dy_t,
      *gphiu, *gphiv;
  double *sin_u, *sin_v;
  // RN(1 / (hu + ssha_u)) and RN(1 / (hv + ssha_v)) (0 where out of the
  // range the exact reciprocal division needs), for the fused step.
  double *r_hu, *r_hv;
};

struct Dims {
  int xs, xe, ys, ye;  // internal T region, 0-based inclusive
  int width, height;
};

struct Scalars {
  double rdt, cbfr, visc, omega, d2r, g;
};

// Grid metrics when every metric array is uniform over the region the step
// reads (true for every dl_esm_inf grid built by grid_init with constant
// dx, dy and the f-plane latitude).  The fused kernel then takes them as
// scalars; each value is the array's value, so results do not change.
struct UniformMetrics {
  double area_t, area_u, area_v, dx_u, dx_v, dx_t, dy_u, dy_v, dy_t;
  double sin_u, sin_v;
};

// Tidal sea-surface height of bc_ssh_code
// (kernels/c_family/boundary_conditions_kern.c:183-192) at step `istep`,
// evaluated on the host with the host's libm.
double tide_value(int istep, double rdt);

// ---- launchers (nl2d_perkernel.cu) ----
// The reference-structured step: 11 launches in time_step.cpp's order.
// `chain_u` / `chain_v` select the ordered Flather kernels for masks in
// which one Flather face reads another Flather face.
void launch_reference_step(const Fields& f, const Dims& d, const Scalars& s,
                           int istep, bool chain_u, bool chain_v,
                           cudaStream_t st);
// next_sshu / next_sshv alone (time_update_kern.c:90-155).
void launch_next_ssh(const Fields& f, const Dims& d, cudaStream_t st);
// Copy of the copy region [xs-1, xe+1] x [ys-1, ye] from src to dst.
void launch_copy_region(const double* src, double* dst, const Dims& d,
                        cudaStream_t st);

// ---- fused FP64 step (nl2d_fused.cu) ----
struct FusedState {
  const double *sshn_in, *un_in, *vn_in;
  double *sshn_out, *un_out, *vn_out;
};
// `tide` is the bc_ssh value of this step, or, when `tide_table` is not
// null, tide_table[tide_index] (a device table; used by captured graphs).
void launch_fused_step(const Fields& f, const FusedState& fs, const Dims& d,
                       const Scalars& s, const UniformMetrics& um, double tide,
                       const double* tide_table, int tide_index,
                       cudaStream_t st);
// The rows of tiles the fused step's grid has for this domain, and the
// tile's height in cells (its tile rows start at row ys - 1).
int fused_step_tile_rows(const Dims& d, int* tile_height);
// The fused step on tile rows [row0, row1) of that grid only.
void launch_fused_step_rows(const Fields& f, const FusedState& fs, const Dims& d,
                            const Scalars& s, const UniformMetrics& um, double tide, int row0,
                            int row1, cudaStream_t st);

// ---- FP64-equivalent (double-float) form, nl2d_df.cu ----
// The fused path's FP64 state and buffers; the interior cells by a column
// march in double-float arithmetic, every other cell of the copy region (the
// exact cells: the boundary rows and columns and the cells beside land) in
// exact FP64 by the fused step's general per-cell code, in the same launch.
struct DfFields {
  float2 *ht, *hu, *hv, *rhu, *rhv;  // (hi, lo) splits of the FP64 arrays
  unsigned char* reg;                // 1 where the march writes the cell
  int* ring;                         // the exact cells (cell indices)
  int* count;                        // device: the exact-cell count
  int n_ring;                        // host copy of the count
};
// One domain of an FP64-equivalent ensemble (device descriptor): its state
// buffers per parity and its double-float statics, pointers into the
// ensemble's packed arrays.
struct EnsDfDomain {
  FusedState fs[2];
  DfFields ff;
  Dims d;
};
struct DfConst {
  dfk::df r_dx, r_dy, uu_x, uu_y, vv_x, vv_y, r_qu, r_qv, vis1_u, vis1_v, vis2_u, vis2_v;
  dfk::df cor_u, cor_v, hpg_u, hpg_v, rra_u, rra_v, face_u, face_v, rrat, r_fric;
};
DfConst make_df_const(const Scalars& s, const UniformMetrics& um);
constexpr int kDfMarchCols = 30;  // columns one warp of the march updates
// Splits the depths and reciprocal denominators and marks the march's cells.
void launch_df_setup(const Fields& f, const Dims& d, const DfFields& ff, cudaStream_t st);
// Counts the exact cells into ff.count and, with ff.ring set, lists them
// there (in no particular order: each is computed on its own).
void launch_df_ring(const Dims& d, const DfFields& ff, cudaStream_t st);
// One step of the form: one launch, the march's blocks and the exact cells'
// blocks interleaved.  `tide` as for the fused step.
void launch_df_step(const Fields& f, const FusedState& fs, const Dims& d, const Scalars& s,
                    const UniformMetrics& um, const DfFields& ff, double tide,
                    const double* tide_table, int tide_index, cudaStream_t st);
// Split of one packed FP64 array into (hi, lo) pairs; the march flags of one
// domain (tmask and reg point at the domain's first element).
void launch_df_split(const double* a, float2* out, long long n, cudaStream_t st);
void launch_df_flags(const int* tmask, const Dims& d, unsigned char* reg, cudaStream_t st);

// Recomputes Fields::r_hu / r_hv from hu, ssha_u, hv, ssha_v (array rows
// [row0, row1) only, when given).
void launch_depth_reciprocals(const Fields& f, const Dims& d, cudaStream_t st, int row0 = 0,
                              int row1 = -1);

// ---- mixed-precision step (nl2d_mixed.cu) ----
struct MixedFields {  // static FP32 copies of the depths and the
  float *ht, *hu, *hv;  // reciprocal momentum denominators
  float *rhu, *rhv;
  // Single domain only (the ensemble leaves them null): per-cell flags of
  // the cells the column march updates, and the list of the copy region's
  // other cells (glist[0 .. gcount)), from launch_mixed_flags.
  unsigned char* reg;
  int* glist;
  int gcount;
};
struct MixedState {  // ssh as (hi, lo) float pairs; velocities FP32
  const float2* sn_in;
  const float *un_in, *vn_in;
  float2* sn_out;
  float *un_out, *vn_out;
};
// side, fork, join (all or none): the general cells' pass starts first on
// stream `side` and runs beside the march (fork / join by the two events).
void launch_mixed_step(const MixedFields& mf, const MixedState& ms, const Fields& f,
                       const Dims& d, const Scalars& s, const UniformMetrics& um,
                       double tide, const double* tide_table, int tide_index,
                       cudaStream_t st, cudaStream_t side = nullptr,
                       cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);
// FP64 (sshn, un, vn) -> ms.{sn,un,vn}_out; with `statics`, also the FP32
// depths mf.{ht,hu,hv} from f.
void launch_to_mixed(const double* sn, const double* un, const double* vn,
                     const Fields& f, const MixedFields& mf, const MixedState& ms,
                     const Dims& d, bool statics, cudaStream_t st);
// The march flags and the general-cell list of mf (mf.reg and mf.glist
// allocated for width x height cells); `count` is one device int.  Returns
// the number of general cells (synchronises the stream), or -1 on a CUDA
// error.
int launch_mixed_flags(const Fields& f, const Dims& d, const MixedFields& mf, int* count,
                       cudaStream_t st);
// Ensemble form of the march (nl2d_mixed.cu, built with FMA contraction
// like the single-domain mixed step).  `doms` is a device array of the
// ensemble's mixed domain descriptors (mixk::EnsDom), `k` the host copy of
// the step constants when all domains share them (mixk::MixConst); else
// `mks` is a device array of each domain's march constants
// (mixk::MarchConst) and k is not read.
void launch_ens_mixed_march(const void* doms, const int4* units, int nunits,
                            const MixedFields& mf, const MixedState& ms, const void* k,
                            const void* mks, int march_rows, cudaStream_t st);
void launch_ens_mixed_general(const void* doms, const int2* glist, int n, int parity,
                              const double* tides, cudaStream_t st);
void launch_ens_mixed_flags(const void* doms, int dom, unsigned char* reg, int2* glist,
                            int* count, cudaStream_t st);
void launch_from_mixed(const float2* sn2, const float* un_f, const float* vn_f,
                       double* sn, double* un, double* vn, const Dims& d,
                       cudaStream_t st);

// ---- checksums (nl2d_checksum.cu) ----
// Sum of |f| over [x0,x1] x [y0,y1]; per-block partial sums go to
// `partials` (at least checksum_partials_needed() doubles) and the final
// FP64 value to *out, both on the device.
int checksum_partials_needed();
// Drops the cached device addresses of the allocation-free checksum's
// scratch array (nl2d_finalize calls it: after a device reset the next call
// looks the address up again).
void noalloc_forget();
void launch_checksum(const double* f, int width, int x0, int x1, int y0,
                     int y1, double* partials, double* out, cudaStream_t st);
// The same sums over FP32 fields and over (hi, lo) pairs (hi + lo in FP64).
void launch_checksum_f32(const float* f, int width, int x0, int x1, int y0,
                         int y1, double* partials, double* out, cudaStream_t st);
void launch_checksum_f2(const float2* f, int width, int x0, int x1, int y0,
                        int y1, double* partials, double* out, cudaStream_t st);

}  // namespace nl2d
