/*
 * libnl2d_gpu — GB300 (sm_103a) NEMOLite2D time step behind the PSyKAl C
 * boundary of the reference's manual C/C++ version.
 *
 * Reference paths are relative to benchmarks/nemo/nemolite2d/ of
 * stfc/PSycloneBench.
 *
 * Data residency follows the reference's GPU PSy layers
 * (manual_versions/psykal_cpp/time_step_omp_gpu.cpp:58,
 * manual_versions/psykal_c_opencl/time_step.c:179-640): the first
 * c_invoke_time_step for a set of arrays copies all 25 of them to the GPU
 * and every later call advances the device-resident copy.  The host arrays
 * are NOT updated by a step; the caller (dl_esm_inf's get_data(), through
 * the read_from_device hook installed in time_step_mod.f90:96-123) pulls a
 * field back with c_read_from_device.  A call with different array
 * addresses, extents or internal bounds registers a new problem (the old
 * device copy is dropped).
 *
 * Errors never abort the process and never trap the GPU: void entry points
 * record a sticky status that nl2d_last_error() returns.  Calls are not
 * re-entrant; one host thread drives the library, as in the reference.
 */
#ifndef NL2D_GPU_H
#define NL2D_GPU_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes of nl2d_last_error() and the int-returning entry points. */
#define NL2D_OK 0
#define NL2D_ERR_CUDA 1        /* a CUDA call failed (message has the text) */
#define NL2D_ERR_ARGS 2        /* inconsistent extents, bounds or pointers   */
#define NL2D_ERR_STATE 3       /* no problem registered yet                  */
#define NL2D_ERR_UNKNOWN_FIELD 4 /* pointer is not a registered field        */
#define NL2D_ERR_NONFINITE 5   /* a checksum found a NaN or an infinity      */
#define NL2D_ERR_TOO_LARGE 6   /* beyond a fixed capacity (no-alloc entry)   */
#define NL2D_ERR_IO 7          /* a file could not be opened or written      */
#define NL2D_ERR_PARSE 8       /* the namelist is not a valid &namctl group  */

/* Step paths (nl2d_set_mode). */
#define NL2D_MODE_AUTO 0       /* fused one-launch step whenever its preconditions hold */
#define NL2D_MODE_REFERENCE 1  /* always the 11-kernel reference-structured step        */

/*
 * One NEMOLite2D time step.  Replaces c_invoke_time_step of
 * manual_versions/psykal_cpp/time_step.cpp:10-51 (argument meaning and
 * order unchanged) in the 7-int form that the Fortran interface
 * manual_versions/psykal_cpp/time_step_mod.f90:8-31 declares and
 * time_step_omp_gpu.cpp:48 defines: `height` (size(data,2)) follows
 * `width`.  Internal bounds are 0-based (time_step_mod.f90:82-85).  As in
 * the reference, the caller may pass dx_v / dx_t in the dy_v / dy_t slots
 * (time_step_mod.f90:76-77); the arrays are used as given.
 *
 * Residency: the first call with a set of arrays uploads all 25 of them;
 * as with the reference's GPU layers (time_step_mod.f90:96-123) the device
 * copy is authoritative after that call, and host arrays change the device
 * state only through c_write_to_device.  When the uploaded state is what a
 * step leaves (ua == un, va == vn, ssha_t == sshn_t on the copy region,
 * sshn_u / sshn_v as next_sshu / next_sshv make them of sshn_t, as at the
 * reference's rest start), the first step already takes the fused path;
 * otherwise it is reference-structured.  With the arrays pinned
 * (nl2d_host_register) the first call uploads the arrays a fused step
 * reads in row bands and starts that step band by band behind them; the
 * other arrays (ssha_t, the metrics, the latitudes) and the registration
 * checks follow on a second stream.  If the checks refuse the fused path or
 * find a state that is not what a step leaves, the steps taken meanwhile
 * are undone and taken again by the reference's rules, so the results are
 * the same bits either way.  Every entry point but c_invoke_time_step waits
 * for the checks (and so for every copy) first.  As with any asynchronous
 * copy from pinned memory, the caller must not write the 25 arrays
 * directly until such a call (nl2d_sync, c_read_from_device, ...) has
 * returned; c_write_to_device, the way to change a registered array, waits
 * for them itself.
 */
void c_invoke_time_step(
    double *ssha_t, double *sshn_t, double *sshn_u, double *sshn_v,
    double *hu, double *hv, double *un, double *vn, double *ua, double *ht,
    double *ssha_u, double *va, double *ssha_v,
    int *tmask, double *area_t, double *area_u, double *area_v,
    double *dx_u, double *dx_v, double *dx_t, double *dy_u, double *dy_v,
    double *dy_t, double *gphiu, double *gphiv,
    int istep, int internal_xstart, int internal_xstop, int internal_ystart,
    int internal_ystop, int width, int height,
    double rdt, double cbfr, double visc, double omega, double d2r, double g);

/*
 * Device -> host copy of one field.  Replaces c_read_from_device of
 * manual_versions/psykal_c_opencl/time_step.c:788-798 (the read_from_device
 * hook of time_step_mod.f90:96-123).  `from` is the field's handle: the
 * host address that was passed for it to c_invoke_time_step (the psykal_cpp
 * contract has no separate device handle).  `to` is a host array with the
 * field's layout (row length = width); the region of columns
 * [startx, startx+nx) and rows [starty, starty+ny) (1-based, as dl_esm_inf
 * passes them) is copied into the same positions of `to`.  With blocking
 * false the copy is only ordered on the library's stream; nl2d_sync()
 * completes it.
 */
void c_read_from_device(void *from, void *to, int startx, int starty, int nx,
                        int ny, bool blocking);

/*
 * Host -> device copy of one field.  Replaces c_write_to_device of
 * manual_versions/psykal_c_opencl/time_step.c:802-810.  `from` is the host
 * source (field layout), `to` is the field's handle (its registered host
 * address).  The next step after a write runs the reference-structured path.
 */
void c_write_to_device(void *from, void *to, int startx, int starty, int nx,
                       int ny, bool blocking);

/* ---- additions (no counterpart in the reference; the reference path
 *      above does not depend on them) ---- */

/* Sticky status of the last failing call (NL2D_OK if none) and its text;
 * reading it clears it. */
int nl2d_last_error(char *msg, int msg_len);

/* Frees every device allocation (the reference keeps its device copies
 * until exit). */
void nl2d_finalize(void);

/* Selects the step path; returns the previous mode. */
int nl2d_set_mode(int mode);

/* Which path the last step took: 0 none, 1 reference-structured, 2 fused
 * FP64, 3 mixed precision. */
int nl2d_last_path(void);

/* Precision of later steps (the survey's nl2d_set_precision): 0 = FP64,
 * the reference's arithmetic (default); 1 = mixed: velocities, fluxes and
 * momentum in FP32 and the sea-surface height as a compensated FP32 pair.
 * The mixed form applies to problems the fused path accepts; it is not
 * bit-identical to the reference.  Reading a field (c_read_from_device)
 * returns the FP64 image of the mixed state; switching back to 0 continues
 * from that image.  2 = FP64-equivalent: the fused path with its interior
 * cells (3x3 wet, one cell inside next_ssh's ranges) computed in
 * double-float arithmetic (FP32 pairs, about 48 significant bits) and every
 * other cell in exact FP64, the state kept in FP64; not bit-identical, held
 * to relative L2 <= 1e-10 per field and checksums to 10 significant digits
 * after 2000 steps of the parity namelist.  Steps that cannot fuse take the
 * reference-structured path as for 0, and nl2d_last_path reports 2 for it.
 * Returns the previous precision. */
int nl2d_set_precision(int precision);

/* Registers and uploads a problem without stepping (same arguments as
 * c_invoke_time_step minus istep).  Returns a status code. */
int nl2d_register(
    double *ssha_t, double *sshn_t, double *sshn_u, double *sshn_v,
    double *hu, double *hv, double *un, double *vn, double *ua, double *ht,
    double *ssha_u, double *va, double *ssha_v,
    int *tmask, double *area_t, double *area_u, double *area_v,
    double *dx_u, double *dx_v, double *dx_t, double *dy_u, double *dy_v,
    double *dy_t, double *gphiu, double *gphiv,
    int internal_xstart, int internal_xstop, int internal_ystart,
    int internal_ystop, int width, int height,
    double rdt, double cbfr, double visc, double omega, double d2r, double g);

/* Advances the registered problem by nsteps steps, istep = istep0 ...
 * istep0+nsteps-1, as a captured CUDA graph on the fused path (or the
 * reference-structured launches where the fused path does not apply).  When
 * checksum_every > 0, the ssh / u / v checksums (nl2d_checksums) after every
 * checksum_every-th step are written to checksums_out[3*k .. 3*k+2], k = 0,
 * 1, ...; checksums_out must hold 3*(nsteps/checksum_every) doubles.
 * Returns a status code. */
int nl2d_run_steps(int istep0, int nsteps, int checksum_every,
                   double *checksums_out);

/* Advances the registered problem by nsteps fused steps from istep0 as one
 * graph launch timed with CUDA events on the library's stream; *ms_out gets
 * the device time of the launch.  Untimed set-up (a first
 * reference-structured step if the state needs one, graph capture) is done
 * before the timed region.  Returns NL2D_ERR_STATE if the fused path does
 * not apply to the problem. */
int nl2d_timed_run(int istep0, int nsteps, double *ms_out);

/* Checksums of the current state: sum |sshn_t| over the internal T region,
 * sum |un| over [xs, xe-1] x [ys, ye] and sum |vn| over [xs, xe] x
 * [ys, ye-1] — the regions the PSy layer updates (time_step.cpp:53-77).
 * Returns NL2D_ERR_NONFINITE if any sum is not finite. */
int nl2d_checksums(double out[3]);

/* Sum of |field| over columns [x0,x1], rows [y0,y1] (0-based, inclusive)
 * of a registered field (handle as for c_read_from_device). */
int nl2d_field_checksum(const void *field, int x0, int x1, int y0, int y1,
                        double *out);

/* Sum of |f| over columns [x0,x1], rows [y0,y1] (0-based, inclusive) of a
 * device-resident FP64 field `d_field` with row length `width`, written to
 * the device double `d_out`, queued on `stream` (a cudaStream_t; NULL for
 * the default stream).  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc (a host model whose own memory
 * manager owns all device buffers, or a loop that must not trigger the
 * synchronisation an allocation can cause) and allocates nothing.  Its
 * scratch is a fixed 128 KiB device array inside the library, held by every
 * GPU that loads it until exit; rectangles above 8192 x 8192 cells return
 * NL2D_ERR_TOO_LARGE.  The first call on a device looks up that array's
 * device address (make it before any stream capture) and keeps it until
 * nl2d_finalize; a caller that resets the device (cudaDeviceReset) calls
 * nl2d_finalize before the next call.  Calls that overlap on the GPU race
 * on the shared array.  A launch error that earlier work left pending in
 * the calling thread is reported as NL2D_ERR_CUDA and left in place, with
 * nothing launched.  Returns a status code; errors are not recorded for
 * nl2d_last_error(). */
int nl2d_field_checksum_noalloc(const double *d_field, int width, int x0,
                                int x1, int y0, int y1, double *d_out,
                                void *stream);

/* ---- ensemble of independent domains (no counterpart in the reference,
 *      which runs one domain per executable) ----
 * Domains start from rest; each has its own extents, T-mask, depths, grid
 * spacing, latitude and tide (bc_ssh of boundary_conditions_kern.c:178-203
 * with amplitude amp and period period_h; 0.2 m / 12.42 h is the
 * reference).  One persistent kernel launch advances every domain by one
 * step; a run of steps is one captured CUDA graph.  FP64 results are
 * bit-identical to the reference step of each domain. */

/* dims6[6k..6k+5] = width, height, xs, xe, ys, ye (0-based internal
 * region); geo3[3k..] = dx, dy, latitude (deg); tide2[2k..] = amp (m),
 * period (h); phys6 = rdt, cbfr, visc, omega, d2r, g. */
int nl2d_ens_create(int ndom, const int *dims6, const double *geo3,
                    const double *tide2, const double *phys6);
/* Static inputs of domain `dom` (width x height each).  Rejects masks with
 * chained Flather faces and non-positive depths. */
int nl2d_ens_set_domain(int dom, const int *tmask, const double *ht,
                        const double *hu, const double *hv);
/* Schedule knobs the autotuner searches: persistent CTAs per SM (1, 2),
 * tile assignment (0 contiguous cost-balanced chunks, 1 longest processing
 * time first, 2 one tile per CTA with as many CTAs as tiles, balanced by the
 * hardware block scheduler; the CTA count then does not apply) and the
 * cost weight of a boundary-tile edge cell. */
int nl2d_ens_schedule(int ctas_per_sm, int policy, double boundary_weight);
/* Tile knobs the autotuner searches (the reference's tiled OpenMP layer,
 * psykal_omp/time_step_mod.f90:587-1182, fixes its tile size per run): the
 * FP64 kernel's tile shape tx x ty, one of 32 x 16 (the default), 32 x 8,
 * 16 x 16, 64 x 8 and 32 x 32, and the column marches' strip height (the
 * mixed and FP64-equivalent forms), 8, 16, 32 (the default) or 64 rows.
 * Results do not depend on
 * either.  A new ensemble starts with the defaults.  Returns NL2D_ERR_ARGS
 * for other values. */
int nl2d_ens_tile(int tx, int ty, int march_rows);
/* Advances every domain nsteps steps (istep = istep0 ...); per-domain
 * ssh / u / v checksums after every checksum_every-th step go to
 * checksums_out[(s * ndom + dom) * 3 + f].  *ms_out: device time. */
int nl2d_ens_run(int istep0, int nsteps, int checksum_every,
                 double *checksums_out, double *ms_out);
/* Current sshn_t, un, vn of one domain (width x height host arrays; any may
 * be NULL). */
int nl2d_ens_read(int dom, double *sshn_t, double *un, double *vn);
/* Form of later runs: 0 FP64 (bit-identical to the reference), 1 mixed
 * precision (FP32 momentum, compensated-FP32 ssh), 2 FP64-equivalent (the
 * FP64 state; interior cells in double-float arithmetic, every other cell
 * exactly as form 0; held to relative L2 <= 1e-10 against form 0).  A
 * change of form restarts every domain from rest. */
int nl2d_ens_set_precision(int precision);
/* Puts every domain back at rest (step 0). */
int nl2d_ens_reset(void);
/* Interior cells over all domains, tiles, persistent CTAs. */
int nl2d_ens_info(long long *cells, int *ntiles, int *nctas);
void nl2d_ens_destroy(void);

/* ---- learned emulator (no counterpart in the reference) ---- */

/* 3x3 convolution (stride 1, zero padding 1) of `batch` NHWC BF16 images
 * (H x W, cin channels) with weights [9][cout][cin] BF16 (tap = 3*dy+dx) on
 * the tensor cores (tcgen05, FP32 accumulation); y (BF16) and/or y32
 * (FP32) receive conv + bias, ReLU'd if relu.  cin in {16,32,48,64}, cout a
 * multiple of 16 up to 64, W a multiple of 128.  All pointers are device
 * pointers; err (device int) is set to 1 if the kernel's bounded wait for
 * its MMAs ran out.  Queued on `stream`. */
int nl2d_emu_conv3x3(const void *x, const void *w, const float *bias, void *y,
                     float *y32, int batch, int H, int W, int cin, int cout,
                     int relu, int *err, void *stream);

/* wt[8 - tap][ci][cout] = w[tap][co][ci] (BF16): the weights of the
 * input-gradient convolution. */
int nl2d_emu_flip_transpose(const void *w, void *wt, int cout, int cin,
                            void *stream);
/* Adds the weight and bias gradients of a 3x3 convolution:
 * dw[tap][co][ci] += sum_p dy[p][co] x[p + off(tap)][ci], db[co] += sum_p
 * dy[p][co].  x [batch][H][W][cin], dy [batch][H][W][cout] BF16; dw, db
 * FP32.  Runs on the tensor cores (tcgen05, FP32 accumulation in tensor
 * memory, one persistent CTA per SM).  cin a multiple of 16 with 9*cin <=
 * 512, cout a multiple of 8 up to 128, W a multiple of 128; err (device
 * int) is set to 1 if a bounded MMA wait ran out. */
int nl2d_emu_conv_wgrad(const void *x, const void *dy, float *dw, float *db,
                        int batch, int H, int W, int cin, int cout, int *err,
                        void *stream);
/* out = (y > 0) ? g : 0 (y, out BF16; g FP32), n elements. */
int nl2d_emu_relu_bwd(const float *g, const void *y, void *out, long long n,
                      void *stream);
/* Mean-squared error of the first nc of cpad channels of pred [P][cpad]
 * against target [P][nc], each pixel weighted by weight[p] (FP32 [P], or
 * NULL for 1); grad (BF16, [P][cpad]) of the mean; loss += mean. */
int nl2d_emu_mse(const float *pred, const float *target, const float *weight,
                 void *grad, float *loss, long long P, int nc, int cpad,
                 void *stream);
/* One Adam step (bias-corrected, step >= 1) on FP32 weights; w16 (BF16
 * copy) may be NULL. */
int nl2d_emu_adam(float *w, float *m, float *v, const float *g, void *w16,
                  int n, float lr, float b1, float b2, float eps, int step,
                  void *stream);

/* Network inputs (BF16 [batch][H*W][cpad], cpad >= 15) and, if target !=
 * NULL, FP32 targets [batch][H*W][3] for snapshot pairs: sample b uses
 * snapshot src[b] of domain dom[b] (snapshot src[b] + 1 is its successor)
 * from snaps [n][H][W][3] and statics [ndom][H][W][4] (depth / 500,
 * open-boundary indicator, east face is a wall, north face is a wall);
 * forcing[b] is the tidal ssh at the target time.  Channels: ssh minus
 * that tide, u, v, depth, forcing, the east and north ssh differences and the depth-weighted
 * flux divergence (formed in FP32), the open-boundary indicator, ssh minus
 * the tide next to the open side, the two wall indicators, and the low
 * BF16 parts of the three state channels (value - BF16(value)).  scale12 (host
 * memory) = state scales (3), increment scales (3), scales of the three
 * difference channels (3), standard deviations (m, m/s, m/s) of white noise
 * added to the input state (3; zeros for none), drawn from `seed`; the
 * target is then the increment from the perturbed state.  Device pointers
 * otherwise. */
int nl2d_emu_assemble(const float *snaps, const float *statics, const int *src,
                      const int *dom, const float *forcing, const float *scale12,
                      unsigned long long seed, void *x, float *target, int H,
                      int W, int cpad, int batch, void *stream);
/* state[p][0..2] += inc[p][0..2] * inc_scale3[0..2] (inc is [P][cpad]).  If
 * statics is not NULL, sample p / HW belongs to domain dom[p / HW] and the
 * solver's boundary conditions are applied: velocities on wall faces
 * (statics channels 2, 3) are zero and the ssh of cells next to the open
 * side (channel 1) is forcing[p / HW], the tide at the target time. */
int nl2d_emu_advance(float *state, const float *inc, const float *inc_scale3,
                     const float *statics, const int *dom, const float *forcing,
                     long long HW, long long P, int cpad, void *stream);
/* 1 when the mixed-precision ensemble has been built (it runs the column
 * march: with the step's constants as kernel parameters when every domain
 * shares them, else each warp with its own domain's), 0 before. */
int nl2d_ens_uses_march(void);
/* Interior (ssh, u, v) of every ensemble domain (all the same size) into a
 * device FP32 array [dom][ny][nx][3], from the FP64 or the mixed-precision
 * state (ssh = hi + lo). */
int nl2d_ens_export_interior(float *d_out);

/* Sets the interior (ssh, u, v) of every ensemble domain from a device FP32
 * array [dom][ny][nx][3] (the emulator hands states back to the solver).
 * The velocity on an open boundary face west or south of the interior (the
 * Flather face, outside the array) is set from the adjacent interior face,
 * so the imported state does not depend on what the solver held before. */
int nl2d_ens_import_interior(const float *d_in);

/* Test hook: over n sampled doubles x (seeded), counts where the exact
 * FP64 helpers of the fused step differ from the IEEE expressions they
 * stand for — x / d (d in [2^-100, 2^100]), 0.5 * x, and the upwind pick
 * (0.5 - copysign(0.5, w)) * x + (0.5 + copysign(0.5, w)) * p.  out[3]
 * receives the three counts (NaN results compare equal).  Returns 0, 1 on
 * a CUDA error, 2 for d out of range. */
int nl2d_selftest_exact(long long n, unsigned long long seed, double d,
                        long long *out);

/* Test hook (no reference counterpart): counts, over n sampled operand
 * pairs, where the exact IEEE add and multiply done on the integer pipes
 * (nl2d_exact.cuh: dadd_i, dmul_i) differ from the FP64 instructions;
 * out[2] = the two counts.  Returns 0, or 1 on a CUDA error. */
int nl2d_selftest_intfp(long long n, unsigned long long seed, long long *out);

/* Test hook (no reference counterpart): the double-float march's
 * conversions (nl2d_df.cuh) on n host values x (1 .. 2^26): hi / lo =
 * split_bits(x), joined = join_bits of that pair, widened = widen_bits of x
 * rounded to FP32.  Returns 0, 1 on a CUDA error, 2 for bad arguments. */
int nl2d_selftest_df(const double *x, long long n, float *hi, float *lo,
                     double *joined, double *widened);

/* Test hook (no reference counterpart): one thread waits, through the
 * convolution kernels' bounded mbarrier wait, on a barrier that nothing
 * arrives on; after max_cycles (1 .. 2^32 clocks) the wait gives up and
 * sets the error flag.  *status = 1 then (2 would mean the phase completed,
 * 0 that the flag was not set).  The context stays usable. */
int nl2d_selftest_wait(long long max_cycles, int *status);

/* Checkpoint / resume (no reference counterpart; the reference keeps no
 * restart files).  nl2d_checkpoint_write stores the registered problem's 13
 * fields exactly as c_read_from_device returns them (FP64, row-major
 * [height][width], c_invoke_time_step's order), the extents and `istep`
 * (the caller's next step number) in `path`.  nl2d_checkpoint_read loads
 * such a file into the registered problem (same extents, else
 * NL2D_ERR_ARGS; not a checkpoint: NL2D_ERR_PARSE; I/O: NL2D_ERR_IO) and
 * returns the stored istep; the next step is then reference-structured, as
 * after c_write_to_device, so a resumed run equals the uninterrupted one
 * bit for bit.  The grid comes from the caller's own set-up. */
int nl2d_checkpoint_write(const char *path, int istep);
int nl2d_checkpoint_read(const char *path, int *istep);

/* Waits for all work queued by the library. */
int nl2d_sync(void);

/* Bytes copied host -> device (out[0]) and device -> host (out[1]) since the
 * current problem was registered. */
int nl2d_transfer_bytes(long long out[2]);

/* Page-locks (pins) a caller's host array of `bytes` bytes, or releases it
 * (no counterpart in the reference, whose OpenCL/OpenACC drivers copy from
 * pageable arrays).  A driver that registers its 25 arrays once, before its
 * first c_invoke_time_step, has the registration's upload and every
 * c_read_from_device / c_write_to_device copy run from pinned memory at the
 * host link's rate instead of through a staging buffer.  Pinning is slow
 * (the operating system locks every page), so it belongs to set-up.  Errors:
 * a null pointer or zero size: NL2D_ERR_ARGS; the CUDA call's failure
 * (e.g. the range is already pinned): NL2D_ERR_CUDA. */
int nl2d_host_register(void *p, size_t bytes);

/* Verdicts on speculative registrations since the library was loaded
 * (no counterpart in the reference): out[0] kept (the fused steps taken
 * before the checks answered stood), out[1] redone (they were undone and
 * taken again by the reference's rules). */
int nl2d_speculation_counts(int out[2]);
int nl2d_host_unregister(void *p);

/* Issue rates of this GPU's arithmetic pipes in Gop/s (no counterpart in
 * the reference): out = {FP64 FMA, FP64 multiply, FP64 add, FP32 FMA}, each
 * over eight independent chains per thread on every SM (best of two timed
 * launches).  The FP64 step is bound by the FP64 pipe; its roofline divides
 * by the fastest FP64 rate measured here.  Allocates a scratch buffer of
 * SMs x 8 x 256 doubles for the duration of the call. */
int nl2d_measure_pipe_rates(double out[4]);

/* ---- host side of the reference executable (no GPU needed) ---- */

/* Reads the &namctl group of a Fortran namelist file
 * (common/gocean2d_io_mod.f90:22-80 read_namelist): ints = jpiglo, jpjglo,
 * jphgr_msh, nit000, nitend, irecord; dbls = dx, dy, dep_const, rdt, cbfr,
 * visc.  Keys the file omits keep the reference's defaults.  NL2D_ERR_IO if
 * the file cannot be opened, NL2D_ERR_PARSE for a syntax error or a key
 * outside the group (the reference stops with "err found in reading
 * namelist file"). */
int nl2d_read_namelist(const char *path, int *ints, double *dbls);

/* The reference's single-rank start state into caller-owned row-major
 * [height][width] arrays (width >= jpiglo + 1, height >= jpjglo + 1,
 * internal T cells 1..jpiglo-2 x 1..jpjglo-2, 0-based): T mask
 * (common/model_mod.f90:94-249 setup_tpoints_mask, jphgr_msh 1-3), grid
 * metrics and T-point coordinates (original/nemolite2d.f90:218-290),
 * depths dep_const and a state at rest
 * (common/initialisation_mod.f90:7-63).  fields = the 13 field arrays in
 * c_invoke_time_step's order; metrics = area_t, area_u, area_v, dx_u, dx_v,
 * dx_t, dy_u, dy_v, dy_t, gphiu, gphiv; xt, yt may be NULL.  jphgr_msh = 0
 * (grid "read from file", a STOP in the reference) keeps the caller's tmask
 * as it is (see nl2d_read_grid_file) and sets up everything else. */
int nl2d_setup_model(int jphgr_msh, int jpiglo, int jpjglo, double dx,
                     double dy, double dep_const, int width, int height,
                     double *const *fields, int *tmask, double *const *metrics,
                     double *xt, double *yt);

/* Writes dir/go2d_<istp:5>_<rank:5>.dat exactly as model_write
 * (common/gocean2d_io_mod.f90:97-149) does: per internal T point x, y,
 * depth, ssh and the velocities averaged to the T point, `(6e16.7)`; an
 * empty record after each row.  Host arrays [][width]. */
int nl2d_model_write(const char *dir, int istp, int rank, int width, int xs,
                     int xe, int ys, int ye, const double *xt, const double *yt,
                     const double *ht, const double *sshn, const double *un,
                     const double *vn);

/* Writes dir/tmask_<rank:5>.dat as dump_tmask (common/model_mod.f90:251-291):
 * raw = every point of the nx x ny mask as `(3(I4,1x))`, else the internal T
 * points with coordinates as `(2e16.7,1x,I3)`. */
int nl2d_dump_tmask(const char *dir, int rank, int raw, int width, int nx,
                    int ny, const int *tmask, int xs, int xe, int ys, int ye,
                    const double *xt, const double *yt);

/* Reads a grid file of whitespace-separated "i j value" triples, one per
 * point of the nx x ny mask (1-based; any order; the raw layout of
 * dump_tmask, so a dumped mask reads back) into row-major [][width] `out`:
 * ints if is_int (a T mask), else doubles (T-point depths).
 * NL2D_ERR_PARSE unless every point appears exactly once. */
int nl2d_read_grid_file(const char *path, int nx, int ny, int width,
                        int is_int, void *out);

/* Face depths from T-point depths: hu = mean of the two T cells across the
 * east face, hv across the north face; the last column / row copies ht. */
int nl2d_face_depths(int width, int height, const double *ht, double *hu,
                     double *hv);

/* One value in the Fortran edit descriptor Ew.d (gfortran's layout) into
 * out (cap >= w + 1 bytes). */
int nl2d_format_e(double v, int w, int d, char *out, int cap);

/* ---- tracer advection (benchmarks/nemo/tracer_advection) ---- */

/* One iteration of the tracer-advection benchmark on the GPU, bit-identical
 * to the reference's operations.  Replaces tra_adv_compute
 * (compute_in_subroutine/tra_adv_compute.F90:12-14): same arrays in the
 * same order, Fortran layout a(ji, jj, jk) (ji fastest), extents by value.
 * The first call with a given set of arrays and extents uploads them and
 * starts a new run (the reference's work arrays start as fresh, zeroed
 * pages); later calls with the same arrays advance the device copy of
 * mydomain, which tra_adv_read copies back (the inputs are assumed
 * unchanged while registered).  jpi, jpj >= 3, jpk >= 2.  Errors are
 * recorded for tra_adv_last_error. */
void tra_adv_compute(const double *ztfreez, const double *pun,
                     const double *pvn, const double *pwn, const double *umask,
                     const double *vmask, const double *tmask,
                     const double *rnfmsk, const double *rnfmsk_z,
                     const double *upsmsk, double *mydomain, const double *tsn,
                     int jpi, int jpj, int jpk);
/* niter more iterations on the registered state; *ms = their device time
 * (CUDA events on the library's stream). */
int tra_adv_run(int niter, double *ms);
/* Copies the current mydomain (all jpi x jpj x jpk values) to the host. */
int tra_adv_read(double *mydomain);
/* The benchmark's checksum (tra_adv.F90:263-270): the sum of mydomain over
 * jk < jpk and the interior columns, in the reference's loop order. */
int tra_adv_checksum(double *out);
/* Sticky status of the tracer entry points (cleared by the call). */
int tra_adv_last_error(char *buf, int len);
/* Frees the device copies. */
void tra_adv_finalize(void);

/* Device address currently holding a registered field (for callers that
 * share device memory); NULL if unknown.  Valid until the next step. */
void *nl2d_device_ptr(const void *field);

#ifdef __cplusplus
}
#endif
#endif
