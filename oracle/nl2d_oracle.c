/*
 * CPU oracle for the NEMOLite2D time step — TEST INFRASTRUCTURE ONLY.
 * (See nl2d_oracle.h: only the tests, the smoke check and the benchmark's
 * CPU-baseline leg use this file; the GPU product never does.)
 *
 * A plain-C restatement of the reference PSy layer
 * benchmarks/nemo/nemolite2d/manual_versions/psykal_cpp/time_step.cpp:10-137
 * and of the kernels in benchmarks/nemo/nemolite2d/kernels/c_family/.
 * The floating-point expressions keep the reference's operand order, since
 * that order is what defines the bits of every result; everything else
 * (naming, argument passing, loop organisation) is this file's own.
 *
 * Paths below are relative to benchmarks/nemo/nemolite2d/ of the reference.
 */
#include "nl2d_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>

typedef struct {
    double *ssha_t, *sshn_t, *sshn_u, *sshn_v, *hu, *hv, *un, *vn, *ua, *ht;
    double *ssha_u, *va, *ssha_v;
    const int *tmask;
    const double *area_t, *area_u, *area_v, *dx_u, *dx_v, *dx_t, *dy_u,
        *dy_v, *dy_t, *gphiu, *gphiv;
    int istep, w;
    double rdt, cbfr, visc, omega, d2r, g;
    double tide_amp, tide_period_h;  /* 0.2 m and 12.42 h in the reference */
} step_t;

/* ---- kernels ----------------------------------------------------------- */

/* Continuity: kernels/c_family/continuity_kern.c:90-117. */
static void k_continuity(const step_t *s, int i, int j)
{
    const int c = j * s->w + i, w = c - 1, so = c - s->w;
    double fe = (s->sshn_u[c] + s->hu[c]) * s->un[c];
    double fw = (s->sshn_u[w] + s->hu[w]) * s->un[w];
    double fn = (s->sshn_v[c] + s->hv[c]) * s->vn[c];
    double fs = (s->sshn_v[so] + s->hv[so]) * s->vn[so];
    s->ssha_t[c] = s->sshn_t[c] + (fw - fe + fs - fn) * s->rdt / s->area_t[c];
}

/* Upwind weight pair (0.5 -/+ copysign(0.5, x)), as used throughout
 * momentum_{u,v}_kern.c. */
#define LO(x) (0.5 - copysign(0.5, (x)))
#define HI(x) (0.5 + copysign(0.5, (x)))

/* u-momentum: kernels/c_family/momentum_u_kern.c:150-262, with the metric
 * arguments bound as time_step.cpp:61-68 binds them
 * (e1u=dx_u, e1v=dx_v, e1t=dx_t, e2u=dy_u, e2t=dy_t, e12u=area_u). */
static void k_momentum_u(const step_t *s, int i, int j)
{
    const int W = s->w, c = j * W + i;
    const int e = c + 1, wst = c - 1, so = c - W, no = c + W, se = so + 1;
    const int *m = s->tmask;
    const double *un = s->un, *vn = s->vn, *hu = s->hu, *hv = s->hv;
    const double *ht = s->ht, *sn = s->sshn_t, *snu = s->sshn_u,
                 *snv = s->sshn_v;
    double u_e, u_w, v_n, v_s, v_nc, v_sc, depe, depw, deps, depn;
    double uu_e, uu_w, uu_n, uu_s, dudx_e, dudx_w, dudy_s, dudy_n;
    double adv, vis, cor, hpg;

    if (m[c] + m[e] <= 0) return;               /* :181 */
    if (m[c] <= 0 || m[e] <= 0) return;         /* :182 */

    u_e = 0.5 * (un[c] + un[e]) * s->dy_t[e];
    depe = ht[e] + sn[e];
    u_w = 0.5 * (un[c] + un[wst]) * s->dy_t[c];
    depw = ht[c] + sn[c];

    v_sc = 0.5 * (vn[so] + vn[se]);
    v_s = 0.5 * v_sc * (s->dx_v[so] + s->dx_v[se]);
    deps = 0.5 * (hv[so] + snv[so] + hv[se] + snv[se]);

    v_nc = 0.5 * (vn[c] + vn[e]);
    v_n = 0.5 * v_nc * (s->dx_v[c] + s->dx_v[e]);
    depn = 0.5 * (hv[c] + snv[c] + hv[e] + snv[e]);

    uu_w = LO(u_w) * un[c] + HI(u_w) * un[wst];
    uu_e = HI(u_e) * un[c] + LO(u_e) * un[e];
    if (m[so] <= 0 || m[se] <= 0)               /* :206 */
        uu_s = LO(v_s) * un[c];
    else
        uu_s = LO(v_s) * un[c] + HI(v_s) * un[so];
    if (m[no] <= 0 || m[no + 1] <= 0)           /* :214 */
        uu_n = HI(v_n) * un[c];
    else
        uu_n = HI(v_n) * un[c] + LO(v_n) * un[no];

    adv = uu_w * u_w * depw - uu_e * u_e * depe + uu_s * v_s * deps -
          uu_n * v_n * depn;

    dudx_e = (un[e] - un[c]) / s->dx_t[e] * (ht[e] + sn[e]);
    dudx_w = (un[c] - un[wst]) / s->dx_t[c] * (ht[c] + sn[c]);
    if (m[so] <= 0 || m[se] <= 0)               /* :229, slip wall */
        dudy_s = 0.0;
    else
        dudy_s = (un[c] - un[so]) / (s->dy_u[c] + s->dy_u[so]) *
                 (hu[c] + snu[c] + hu[so] + snu[so]);
    if (m[no] <= 0 || m[no + 1] <= 0)           /* :237 */
        dudy_n = 0.0;
    else
        dudy_n = (un[no] - un[c]) / (s->dy_u[c] + s->dy_u[no]) *
                 (hu[c] + snu[c] + hu[no] + snu[no]);

    vis = (dudx_e - dudx_w) * s->dy_u[c] + (dudy_n - dudy_s) * s->dx_u[c] * 0.5;
    vis = s->visc * vis;

    cor = 0.5 * (2. * s->omega * sin(s->gphiu[c] * s->d2r) * (v_sc + v_nc)) *
          s->area_u[c] * (hu[c] + snu[c]);

    hpg = -s->g * (hu[c] + snu[c]) * s->dy_u[c] * (sn[e] - sn[c]);

    s->ua[c] = (un[c] * (hu[c] + snu[c]) +
                s->rdt * (adv + vis + cor + hpg) / s->area_u[c]) /
               (hu[c] + s->ssha_u[c]) / (1.0 + s->cbfr * s->rdt);
}

/* v-momentum: kernels/c_family/momentum_v_kern.c:125-241, metric binding of
 * time_step.cpp:70-77 (e1v=dx_v, e1t=dx_t, e2u=dy_u, e2v=dy_v, e2t=dy_t,
 * e12v=area_v).  The first guard tests the EAST neighbour's mask (:155). */
static void k_momentum_v(const step_t *s, int i, int j)
{
    const int W = s->w, c = j * W + i;
    const int e = c + 1, wst = c - 1, so = c - W, no = c + W, nw = no - 1;
    const int *m = s->tmask;
    const double *un = s->un, *vn = s->vn, *hu = s->hu, *hv = s->hv;
    const double *ht = s->ht, *sn = s->sshn_t, *snu = s->sshn_u,
                 *snv = s->sshn_v;
    double u_e, u_w, v_n, v_s, u_ec, u_wc, depe, depw, deps, depn;
    double vv_e, vv_w, vv_n, vv_s, dvdx_e, dvdx_w, dvdy_n, dvdy_s;
    double adv, vis, cor, hpg;

    if (m[c] + m[e] <= 0) return;               /* :155 */
    if (m[c] <= 0 || m[no] <= 0) return;        /* :156 */

    v_n = 0.5 * (vn[c] + vn[no]) * s->dx_t[no];
    depn = ht[no] + sn[no];
    v_s = 0.5 * (vn[c] + vn[so]) * s->dx_t[c];
    deps = ht[c] + sn[c];

    u_wc = 0.5 * (un[wst] + un[nw]);
    u_w = 0.5 * u_wc * (s->dy_u[wst] + s->dy_u[nw]);
    depw = 0.50 * (hu[wst] + snu[wst] + hu[nw] + snu[nw]);

    u_ec = 0.5 * (un[c] + un[no]);
    u_e = 0.5 * u_ec * (s->dy_u[c] + s->dy_u[no]);
    depe = 0.50 * (hu[c] + snu[c] + hu[no] + snu[no]);

    vv_s = LO(v_s) * vn[c] + HI(v_s) * vn[so];
    vv_n = HI(v_n) * vn[c] + LO(v_n) * vn[no];
    if (m[wst] <= 0 || m[nw] <= 0)              /* :181 */
        vv_w = LO(u_w) * vn[c];
    else
        vv_w = LO(u_w) * vn[c] + HI(u_w) * vn[wst];
    if (m[e] <= 0 || m[no + 1] <= 0)            /* :189 */
        vv_e = HI(u_e) * vn[c];
    else
        vv_e = HI(u_e) * vn[c] + LO(u_e) * vn[e];

    adv = vv_w * u_w * depw - vv_e * u_e * depe + vv_s * v_s * deps -
          vv_n * v_n * depn;

    dvdy_n = (vn[no] - vn[c]) / s->dy_t[no] * (ht[no] + sn[no]);
    dvdy_s = (vn[c] - vn[so]) / s->dy_t[c] * (ht[c] + sn[c]);
    if (m[wst] <= 0 || m[nw] <= 0)              /* :207, slip wall */
        dvdx_w = 0.0;
    else
        dvdx_w = (vn[c] - vn[wst]) / (s->dx_v[c] + s->dx_v[wst]) *
                 (hv[c] + snv[c] + hv[wst] + snv[wst]);
    if (m[e] <= 0 || m[no + 1] <= 0)            /* :215 */
        dvdx_e = 0.0;
    else
        dvdx_e = (vn[e] - vn[c]) / (s->dx_v[c] + s->dx_v[e]) *
                 (hv[c] + snv[c] + hv[e] + snv[e]);

    vis = (dvdy_n - dvdy_s) * s->dx_v[c] + (dvdx_e - dvdx_w) * s->dy_v[c] * 0.5;
    vis = s->visc * vis;

    cor = -0.5 * (2. * s->omega * sin(s->gphiv[c] * s->d2r) * (u_ec + u_wc)) *
          s->area_v[c] * (hv[c] + snv[c]);

    hpg = -s->g * (hv[c] + snv[c]) * s->dx_v[c] * (sn[no] - sn[c]);

    s->va[c] = (vn[c] * (hv[c] + snv[c]) +
                s->rdt * (adv + vis + cor + hpg) / s->area_v[c]) /
               ((hv[c] + s->ssha_v[c])) / (1.0 + s->cbfr * s->rdt);
}

/* Tidal sea-surface height at wet cells next to an open (-1) cell:
 * kernels/c_family/boundary_conditions_kern.c:178-203 (amplitude 0.2 m,
 * period 12.42 h, the literal 3.14159; neighbour priority S, N, E, W). */
/* The ensemble form parametrises amplitude and period; with 0.2 m and
 * 12.42 h the operations, and so the bits, are the reference's. */
static void k_bc_ssh(const step_t *s, int i, int j)
{
    const int c = j * s->w + i;
    const int *m = s->tmask;
    double amp_tide = s->tide_amp;
    double omega_tide = 2.0 * 3.14159 / (s->tide_period_h * 3600.0);
    double rtime = s->istep * s->rdt;
    if (m[c] <= 0) return;
    if (m[c - s->w] < 0 || m[c + s->w] < 0 || m[c + 1] < 0 || m[c - 1] < 0)
        s->ssha_t[c] = amp_tide * sin(omega_tide * rtime);
}

/* Solid walls: boundary_conditions_kern.c:220-228 and :244-252. */
static void k_bc_solid_u(const step_t *s, int i, int j)
{
    const int c = j * s->w + i;
    if (s->tmask[c] * s->tmask[c + 1] == 0) s->ua[c] = 0.0;
}
static void k_bc_solid_v(const step_t *s, int i, int j)
{
    const int c = j * s->w + i;
    if (s->tmask[c] * s->tmask[c + s->w] == 0) s->va[c] = 0.0;
}

/* Flather radiation condition: boundary_conditions_kern.c:271-293 (u) and
 * :313-333 (v).  `step` is the neighbour offset (1 for u, width for v). */
static void k_bc_flather(double *vel, const double *h, const double *ssh_f,
                         const int *m, double g, int c, int step)
{
    if (m[c] + m[c + step] <= -1) return;
    if (m[c] < 0)
        vel[c] = vel[c + step] + sqrt(g / h[c]) * (ssh_f[c] - ssh_f[c + step]);
    else if (m[c + step] < 0)
        vel[c] = vel[c - step] + sqrt(g / h[c]) * (ssh_f[c] - ssh_f[c - step]);
}

/* Staggered ssh update: kernels/c_family/time_update_kern.c:90-112 (u,
 * step 1, area_u) and :132-155 (v, step width, area_v). */
static void k_next_ssh(double *ssh_f, const double *sn, const int *m,
                       const double *e12t, const double *e12f, int c, int step)
{
    const int n = c + step;
    double rtmp1;
    if (m[c] + m[n] <= 0) return;
    if (m[c] * m[n] > 0) {
        rtmp1 = e12t[c] * sn[c] + e12t[n] * sn[n];
        ssh_f[c] = 0.5 * rtmp1 / e12f[c];
    } else if (m[c] <= 0) {
        ssh_f[c] = sn[n];
    } else if (m[n] <= 0) {
        ssh_f[c] = sn[c];
    }
}

/* ---- PSy layer ----------------------------------------------------------- */

/* The loop nest of time_step.cpp:53-136.  `par` switches on the OpenMP
 * worksharing of time_step_omp.cpp:57-146 (never on bc_flather_v, whose
 * j loop carries a dependency, time_step_omp.cpp:116-119). */
static void psy_step(const step_t *s, int xs, int xe, int ys, int ye, int par)
{
    const int W = s->w;
    int i, j;
    (void)par;

#pragma omp parallel for private(i) if (par)
    for (j = ys; j <= ye; j++)
        for (i = xs; i <= xe; i++) k_continuity(s, i, j);

#pragma omp parallel for private(i) if (par)
    for (j = ys; j <= ye; j++)
        for (i = xs; i <= xe - 1; i++) k_momentum_u(s, i, j);

#pragma omp parallel for private(i) if (par)
    for (j = ys; j <= ye - 1; j++)
        for (i = xs; i <= xe; i++) k_momentum_v(s, i, j);

#pragma omp parallel for private(i) if (par)
    for (j = ys; j <= ye; j++)
        for (i = xs; i <= xe; i++) k_bc_ssh(s, i, j);

#pragma omp parallel for private(i) if (par)
    for (j = ys - 1; j <= ye + 1; j++)
        for (i = xs - 1; i <= xe; i++) k_bc_solid_u(s, i, j);

#pragma omp parallel for private(i) if (par)
    for (j = ys - 1; j <= ye; j++)
        for (i = xs - 1; i <= xe + 1; i++) k_bc_solid_v(s, i, j);

#pragma omp parallel for private(i) if (par)
    for (j = ys - 1; j <= ye + 1; j++)
        for (i = xs - 1; i <= xe; i++)
            k_bc_flather(s->ua, s->hu, s->sshn_u, s->tmask, s->g, j * W + i, 1);

    for (j = ys - 1; j <= ye; j++)
        for (i = xs - 1; i <= xe + 1; i++)
            k_bc_flather(s->va, s->hv, s->sshn_v, s->tmask, s->g, j * W + i, W);

    /* time_step.cpp:114-122: note the row bound j < ye + 1 */
#pragma omp parallel for private(i) if (par)
    for (j = ys - 1; j < ye + 1; j++)
        for (i = xs - 1; i <= xe + 1; i++) {
            const int c = j * W + i;
            s->un[c] = s->ua[c];
            s->vn[c] = s->va[c];
            s->sshn_t[c] = s->ssha_t[c];
        }

#pragma omp parallel for private(i) if (par)
    for (j = ys; j <= ye; j++)
        for (i = xs; i <= xe - 1; i++)
            k_next_ssh(s->sshn_u, s->sshn_t, s->tmask, s->area_t, s->area_u,
                       j * W + i, 1);

#pragma omp parallel for private(i) if (par)
    for (j = ys; j <= ye - 1; j++)
        for (i = xs; i <= xe; i++)
            k_next_ssh(s->sshn_v, s->sshn_t, s->tmask, s->area_t, s->area_v,
                       j * W + i, W);
}

/* The partially fused loop nest of psykal_cpp/time_step_ompopt.cpp:61-150,
 * the reference's faster OpenMP PSy layer: continuity, bc_ssh, momentum_u
 * and momentum_v in one loop over the whole internal region (so momentum_u
 * also runs at i = xe and momentum_v at j = ye, where the serial layer's
 * ranges stop one short), the boundary kernels and the copies as in the
 * worksharing layer, and next_sshu / next_sshv in one loop over
 * [xs, xe-1] x [ys, ye].  Its results need not equal the serial layer's bit
 * for bit at those edges; it is timed as a CPU baseline and checked against
 * the reference's own compiled ompopt layer. */
static void psy_step_ompopt(const step_t *s, int xs, int xe, int ys, int ye)
{
    const int W = s->w;
    int i, j;

#pragma omp parallel for private(i)
    for (j = ys; j <= ye; j++)
        for (i = xs; i <= xe; i++) {
            k_continuity(s, i, j);
            k_bc_ssh(s, i, j);
            k_momentum_u(s, i, j);
            k_momentum_v(s, i, j);
        }

#pragma omp parallel for private(i)
    for (j = ys - 1; j <= ye + 1; j++)
        for (i = xs - 1; i <= xe; i++) k_bc_solid_u(s, i, j);

#pragma omp parallel for private(i)
    for (j = ys - 1; j <= ye; j++)
        for (i = xs - 1; i <= xe + 1; i++) k_bc_solid_v(s, i, j);

#pragma omp parallel for private(i)
    for (j = ys - 1; j <= ye + 1; j++)
        for (i = xs - 1; i <= xe; i++)
            k_bc_flather(s->ua, s->hu, s->sshn_u, s->tmask, s->g, j * W + i, 1);

    for (j = ys - 1; j <= ye; j++)
        for (i = xs - 1; i <= xe + 1; i++)
            k_bc_flather(s->va, s->hv, s->sshn_v, s->tmask, s->g, j * W + i, W);

#pragma omp parallel for private(i)
    for (j = ys - 1; j < ye + 1; j++)
        for (i = xs - 1; i <= xe + 1; i++) {
            const int c = j * W + i;
            s->un[c] = s->ua[c];
            s->vn[c] = s->va[c];
            s->sshn_t[c] = s->ssha_t[c];
        }

#pragma omp parallel for private(i)
    for (j = ys; j <= ye; j++)
        for (i = xs; i <= xe - 1; i++) {
            k_next_ssh(s->sshn_u, s->sshn_t, s->tmask, s->area_t, s->area_u,
                       j * W + i, 1);
            k_next_ssh(s->sshn_v, s->sshn_t, s->tmask, s->area_t, s->area_v,
                       j * W + i, W);
        }
}

#define FILL_STEP(s)                                                          \
    step_t s = {ssha_t, sshn_t, sshn_u, sshn_v, hu, hv, un, vn, ua, ht,       \
                ssha_u, va, ssha_v, tmask, area_t, area_u, area_v, dx_u,      \
                dx_v, dx_t, dy_u, dy_v, dy_t, gphiu, gphiv, istep, width,    \
                rdt, cbfr, visc, omega, d2r, g, 0.2, 12.42};                  \
    (void)height

void oracle_invoke_time_step(NL2D_ORACLE_STEP_ARGS)
{
    FILL_STEP(s);
    psy_step(&s, internal_xstart, internal_xstop, internal_ystart,
             internal_ystop, 0);
}

void oracle_invoke_time_step_omp(NL2D_ORACLE_STEP_ARGS)
{
    FILL_STEP(s);
    psy_step(&s, internal_xstart, internal_xstop, internal_ystart,
             internal_ystop, 1);
}

void oracle_invoke_time_step_ompopt(NL2D_ORACLE_STEP_ARGS)
{
    FILL_STEP(s);
    psy_step_ompopt(&s, internal_xstart, internal_xstop, internal_ystart,
                    internal_ystop);
}

void oracle_invoke_time_step_tide(NL2D_ORACLE_STEP_ARGS, double tide_amp,
                                  double tide_period_h)
{
    FILL_STEP(s);
    s.tide_amp = tide_amp;
    s.tide_period_h = tide_period_h;
    psy_step(&s, internal_xstart, internal_xstop, internal_ystart,
             internal_ystop, 0);
}

/* ---- driver pieces ------------------------------------------------------ */

/* common/model_mod.f90:94-249 for a single rank that owns the whole global
 * domain (so every "global boundary" branch is taken).  The Fortran array
 * slices `tmask(xstop+1:, :)` run to the end of the array, so they cover
 * any padding columns/rows too; the assignments keep the Fortran order, so
 * the southern row (assigned last) wins at the corners. */
int oracle_setup_tmask(int jphgr_msh, int width, int height, int xs, int xe,
                       int ys, int ye, int *tmask)
{
    int i, j;
    if (jphgr_msh < 1 || jphgr_msh > 3) return -1;
    for (j = 0; j < height; j++)
        for (i = 0; i < width; i++)
            tmask[j * width + i] =
                (i >= xs && i <= xe && j >= ys && j <= ye) ? 1 : 0;
    for (j = 0; j < height; j++)           /* west: solid */
        for (i = 0; i < xs; i++) tmask[j * width + i] = 0;
    for (j = ye + 1; j < height; j++)      /* north: solid */
        for (i = 0; i < width; i++) tmask[j * width + i] = 0;
    for (j = 0; j < height; j++)           /* east: open for 2 and 3 */
        for (i = xe + 1; i < width; i++)
            tmask[j * width + i] = (jphgr_msh == 2 || jphgr_msh == 3) ? -1 : 0;
    for (j = 0; j < ys; j++)               /* south: open for 1 and 3 */
        for (i = 0; i < width; i++)
            tmask[j * width + i] = (jphgr_msh == 1 || jphgr_msh == 3) ? -1 : 0;
    return 0;
}

double oracle_field_checksum(const double *f, int width, int x0, int x1,
                             int y0, int y1)
{
    double sum = 0.0;
    int i, j;
    for (j = y0; j <= y1; j++)
        for (i = x0; i <= x1; i++) sum = sum + fabs(f[j * width + i]);
    return sum;
}

/* A Fortran namelist group `&namctl ... /` with `key = value` items,
 * `!` comments and case-insensitive keys (gocean2d_io_mod.f90:50-68 names
 * the keys and their defaults). */
int oracle_read_namelist(const char *path, int ints[6], double dbls[6])
{
    static const char *ikeys[6] = {"jpiglo", "jpjglo", "jphgr_msh",
                                   "nit000", "nitend", "irecord"};
    static const char *dkeys[6] = {"dx", "dy", "dep_const",
                                   "rdt", "cbfr", "visc"};
    const int idef[6] = {50, 100, 1, 1, 1000, 1};
    const double ddef[6] = {1000.0, 1000.0, 100.0, 10.0, 0.001, 100.0};
    char line[1024];
    int in_group = 0, done = 0, k;
    FILE *fp = fopen(path, "r");
    if (!fp) return -1;
    for (k = 0; k < 6; k++) { ints[k] = idef[k]; dbls[k] = ddef[k]; }
    while (!done && fgets(line, sizeof line, fp)) {
        char *p, *bang = strchr(line, '!');
        if (bang) *bang = '\0';
        for (p = line; *p; p++) *p = (char)tolower((unsigned char)*p);
        p = line;
        while (*p) {
            char key[64], *q;
            size_t n;
            while (*p && (isspace((unsigned char)*p) || *p == ',')) p++;
            if (!*p) break;
            if (!in_group) {
                if (strncmp(p, "&namctl", 7) == 0) { in_group = 1; p += 7; continue; }
                break;
            }
            if (*p == '/') { done = 1; break; }
            q = p;
            while (*q && (isalnum((unsigned char)*q) || *q == '_')) q++;
            n = (size_t)(q - p);
            if (n == 0 || n >= sizeof key) { fclose(fp); return -2; }
            memcpy(key, p, n);
            key[n] = '\0';
            p = q;
            while (*p && isspace((unsigned char)*p)) p++;
            if (*p != '=') { fclose(fp); return -2; }
            p++;
            {
                char *end;
                int found = 0;
                /* Fortran 'd' exponents become 'e' for strtod (within
                 * this value only: it ends at a blank, ',' or '/'). */
                while (*p && isspace((unsigned char)*p)) p++;
                for (q = p; *q && *q != ',' && *q != '/' && !isspace((unsigned char)*q); q++)
                    if (*q == 'd') *q = 'e';
                for (k = 0; k < 6 && !found; k++)
                    if (strcmp(key, ikeys[k]) == 0) {
                        long v = strtol(p, &end, 10);
                        if (end == p) { fclose(fp); return -2; }
                        ints[k] = (int)v;
                        p = end;
                        found = 1;
                    }
                for (k = 0; k < 6 && !found; k++)
                    if (strcmp(key, dkeys[k]) == 0) {
                        double v = strtod(p, &end);
                        if (end == p) { fclose(fp); return -2; }
                        dbls[k] = v;
                        p = end;
                        found = 1;
                    }
                if (!found) { fclose(fp); return -2; }
            }
        }
    }
    fclose(fp);
    return in_group ? 0 : -2;
}
