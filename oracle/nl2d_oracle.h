/*
 * CPU oracle for the NEMOLite2D time step — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as what the tests compare with (or, for the
 * baseline, as the timed CPU port).  The GPU product never links or calls it.
 *
 * It restates, in plain C, the reference's manual C++ PSy layer
 * (benchmarks/nemo/nemolite2d/manual_versions/psykal_cpp/time_step.cpp:10-137)
 * with the kernel bodies of benchmarks/nemo/nemolite2d/kernels/c_family/*.c,
 * plus the driver pieces that live in Fortran or in the absent dl_esm_inf
 * library (namelist reader, T-mask builder, grid metrics, initial state,
 * field checksum).  Built with -O2 -ffp-contract=off -fno-fast-math so that
 * every floating-point operation is the IEEE operation the C source names.
 */
#ifndef NL2D_ORACLE_H
#define NL2D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Same argument list as the reference's c_invoke_time_step
 * (psykal_cpp/time_step.cpp:10-51) plus the `height` the Fortran interface
 * passes after `width` (psykal_cpp/time_step_mod.f90:16,90). */
#define NL2D_ORACLE_STEP_ARGS                                                   \
    double *ssha_t, double *sshn_t, double *sshn_u, double *sshn_v,             \
    double *hu, double *hv, double *un, double *vn, double *ua, double *ht,     \
    double *ssha_u, double *va, double *ssha_v,                                 \
    int *tmask, double *area_t, double *area_u, double *area_v,                 \
    double *dx_u, double *dx_v, double *dx_t, double *dy_u, double *dy_v,       \
    double *dy_t, double *gphiu, double *gphiv,                                 \
    int istep, int internal_xstart, int internal_xstop, int internal_ystart,   \
    int internal_ystop, int width, int height,                                  \
    double rdt, double cbfr, double visc, double omega, double d2r, double g

/* One time step, serial loops in the reference order. */
void oracle_invoke_time_step(NL2D_ORACLE_STEP_ARGS);
/* One time step with the loop-level OpenMP worksharing of
 * psykal_cpp/time_step_omp.cpp:57-146 (bc_flather_v stays serial). */
void oracle_invoke_time_step_omp(NL2D_ORACLE_STEP_ARGS);
/* One time step with the partially fused loops of
 * psykal_cpp/time_step_ompopt.cpp:61-150 (continuity, bc_ssh and both
 * momentum kernels in one loop; next_sshu and next_sshv in one loop). */
void oracle_invoke_time_step_ompopt(NL2D_ORACLE_STEP_ARGS);

/* The serial step with the tidal amplitude (m) and period (h) of bc_ssh
 * as parameters (the reference hard-codes 0.2 m and 12.42 h,
 * boundary_conditions_kern.c:185-186); used for the ensemble's domains. */
void oracle_invoke_time_step_tide(NL2D_ORACLE_STEP_ARGS, double tide_amp,
                                  double tide_period_h);

/* &namctl reader (common/gocean2d_io_mod.f90:22-80).  ints = {jpiglo,
 * jpjglo, jphgr_msh, nit000, nitend, irecord}; dbls = {dx, dy, dep_const,
 * rdt, cbfr, visc}.  Returns 0, or -1 if the file cannot be read, or -2 on
 * an unknown key or malformed value. */
int oracle_read_namelist(const char *path, int ints[6], double dbls[6]);

/* T-mask of one rank that owns the whole domain
 * (common/model_mod.f90:94-249).  The mask array is width x height
 * (row-major, row = j); internal T cells are [xs,xe] x [ys,ye] (0-based).
 * Returns 0, or -1 for jphgr_msh outside 1..3. */
int oracle_setup_tmask(int jphgr_msh, int width, int height, int xs, int xe,
                       int ys, int ye, int *tmask);

/* Sum of |f| over rows [y0,y1] and columns [x0,x1] (inclusive, 0-based),
 * row by row, in one FP64 accumulator: the dl_esm_inf field_checksum as
 * restated by regent/checksum.rg:12-31. */
double oracle_field_checksum(const double *f, int width, int x0, int x1,
                             int y0, int y1);

#ifdef __cplusplus
}
#endif
#endif
