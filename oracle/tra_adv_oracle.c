/*
 * TEST INFRASTRUCTURE ONLY (what the tests compare with, never the product): a plain-C
 * restatement of the tracer-advection benchmark's iteration,
 * benchmarks/nemo/tracer_advection/original/tra_adv.F90:106-258, in the
 * form of the reference's per-iteration subroutine
 * (compute_in_subroutine/tra_adv_compute.F90:12-).  Every loop keeps the
 * reference's bounds and order and every expression its operation order
 * (Fortran evaluates a*b*c as (a*b)*c); built with -ffp-contract=off.
 *
 * Layout: Fortran array a(ji, jj, jk) (ji fastest) is a[((jk-1)*jpj +
 * (jj-1))*jpi + (ji-1)] here.  SIGN(a, b) is copysign(a, b) (gfortran keeps
 * the sign of a negative zero); MAX / MIN of three are evaluated pairwise
 * left to right.
 *
 * The work arrays zwx, zwy, zslpx, zslpy, zind belong to the caller and
 * persist across calls, as the reference's module-scope allocatables do.
 * The reference never initialises them; some entries are read before any
 * write (zwx(jpi,:,:) in the first iteration, zwy(jpi,:,:) and
 * zwy(:,jpj,:) always), so the caller passes them zeroed, the contents of
 * fresh pages.  The reference cannot be compiled here (Fortran, no
 * gfortran), so this restatement's parity is unpinned by the reference
 * itself.
 */
#include <math.h>
#include <stddef.h>

#include "tra_adv_oracle.h"

#define IX(i, j, k) ((((size_t)(k) - 1) * (size_t)jpj + ((size_t)(j) - 1)) * (size_t)jpi + \
                     ((size_t)(i) - 1))
#define IX2(i, j) (((size_t)(j) - 1) * (size_t)jpi + ((size_t)(i) - 1))

static double fmax3(double a, double b, double c)
{
    double m = a > b ? a : b; /* Fortran MAX: no NaNs arise here */
    return m > c ? m : c;
}

static double fmin3(double a, double b, double c)
{
    double m = a < b ? a : b;
    return m < c ? m : c;
}

/* tra_adv.F90:63-98: the benchmark's own initial values. */
void tra_oracle_init(int jpi, int jpj, int jpk, double *mydomain, double *tsn,
                     double *pun, double *pvn, double *pwn, double *umask,
                     double *vmask, double *tmask, double *ztfreez,
                     double *rnfmsk, double *upsmsk, double *rnfmsk_z)
{
    int ji, jj, jk;
    double r = (double)(jpi * jpj * jpk);
    for (jk = 1; jk <= jpk; jk++)
        for (jj = 1; jj <= jpj; jj++)
            for (ji = 1; ji <= jpi; ji++) {
                /* ji*jj*jk is a default (32-bit) integer product */
                double v = (double)(ji * jj * jk) / r;
                size_t c = IX(ji, jj, jk);
                umask[c] = v;
                mydomain[c] = v;
                pun[c] = v;
                pvn[c] = v;
                pwn[c] = v;
                vmask[c] = v;
                tsn[c] = v;
                tmask[c] = v;
            }
    r = (double)(jpi * jpj);
    for (jj = 1; jj <= jpj; jj++)
        for (ji = 1; ji <= jpi; ji++) {
            double v = (double)(ji * jj) / r;
            ztfreez[IX2(ji, jj)] = v;
            upsmsk[IX2(ji, jj)] = v;
            rnfmsk[IX2(ji, jj)] = v;
        }
    for (jk = 1; jk <= jpk; jk++)
        rnfmsk_z[jk - 1] = (double)(jk / jpk); /* integer division */
}

#define OMP_LOOP \
    _Pragma("omp parallel for private(ji, jj, zice, zu, z0u, zzwx, zv, z0v, zzwy, ztra, zalpha, zw, z0w) if (par)")

/* One iteration: tra_adv.F90:107-257 (the jt loop body).  With `par`,
 * each jk loop is an OpenMP worksharing loop (every loop writes only its
 * own jk level's elements, so the values do not change). */
static void step_impl(int jpi, int jpj, int jpk, double *mydomain,
                      const double *tsn, const double *pun, const double *pvn,
                      const double *pwn, const double *umask,
                      const double *vmask, const double *tmask,
                      const double *ztfreez, const double *rnfmsk,
                      const double *upsmsk, const double *rnfmsk_z, double *zwx,
                      double *zwy, double *zslpx, double *zslpy, double *zind,
                      int par)
{
    int ji, jj, jk;
    double zice, zu, z0u, zzwx, zv, z0v, zzwy, ztra, zbtr, zdt, zalpha, zw, z0w;
    (void)par;

    /* :107-120 */
    OMP_LOOP
    for (jk = 1; jk <= jpk; jk++)
        for (jj = 1; jj <= jpj; jj++)
            for (ji = 1; ji <= jpi; ji++) {
                size_t c = IX(ji, jj, jk);
                if (tsn[c] <= ztfreez[IX2(ji, jj)] + 0.1) zice = 1.0;
                else zice = 0.0;
                zind[c] = fmax3(rnfmsk[IX2(ji, jj)] * rnfmsk_z[jk - 1], upsmsk[IX2(ji, jj)],
                                zice) * tmask[c];
                zind[c] = 1 - zind[c];
            }

    /* :122-130 */
    for (jj = 1; jj <= jpj; jj++)
        for (ji = 1; ji <= jpi; ji++) {
            zwx[IX(ji, jj, jpk)] = 0.0;
            zwy[IX(ji, jj, jpk)] = 0.0;
        }
    OMP_LOOP
    for (jk = 1; jk <= jpk - 1; jk++)
        for (jj = 1; jj <= jpj - 1; jj++)
            for (ji = 1; ji <= jpi - 1; ji++) {
                size_t c = IX(ji, jj, jk);
                zwx[c] = umask[c] * (mydomain[IX(ji + 1, jj, jk)] - mydomain[c]);
                zwy[c] = vmask[c] * (mydomain[IX(ji, jj + 1, jk)] - mydomain[c]);
            }

    /* :132-143 */
    for (jj = 1; jj <= jpj; jj++)
        for (ji = 1; ji <= jpi; ji++) {
            zslpx[IX(ji, jj, jpk)] = 0.0;
            zslpy[IX(ji, jj, jpk)] = 0.0;
        }
    OMP_LOOP
    for (jk = 1; jk <= jpk - 1; jk++)
        for (jj = 2; jj <= jpj; jj++)
            for (ji = 2; ji <= jpi; ji++) {
                size_t c = IX(ji, jj, jk);
                double a = zwx[c], b = zwx[IX(ji - 1, jj, jk)];
                zslpx[c] = (a + b) * (0.25 + copysign(0.25, a * b));
                a = zwy[c];
                b = zwy[IX(ji, jj - 1, jk)];
                zslpy[c] = (a + b) * (0.25 + copysign(0.25, a * b));
            }

    /* :145-156 */
    OMP_LOOP
    for (jk = 1; jk <= jpk - 1; jk++)
        for (jj = 2; jj <= jpj; jj++)
            for (ji = 2; ji <= jpi; ji++) {
                size_t c = IX(ji, jj, jk);
                zslpx[c] = copysign(1.0, zslpx[c]) *
                           fmin3(fabs(zslpx[c]), 2.0 * fabs(zwx[IX(ji - 1, jj, jk)]),
                                 2.0 * fabs(zwx[c]));
                zslpy[c] = copysign(1.0, zslpy[c]) *
                           fmin3(fabs(zslpy[c]), 2.0 * fabs(zwy[IX(ji, jj - 1, jk)]),
                                 2.0 * fabs(zwy[c]));
            }

    /* :158-183 (the reference sets zdt = 1 at the top of each jk pass; it
     * is set once here, so no two OpenMP threads write it) */
    zdt = 1;
    OMP_LOOP
    for (jk = 1; jk <= jpk - 1; jk++)
        for (jj = 2; jj <= jpj - 1; jj++)
            for (ji = 2; ji <= jpi - 1; ji++) {
                size_t c = IX(ji, jj, jk);
                z0u = copysign(0.5, pun[c]);
                zalpha = 0.5 - z0u;
                zu = z0u - 0.5 * pun[c] * zdt;
                zzwx = mydomain[IX(ji + 1, jj, jk)] + zind[c] * (zu * zslpx[IX(ji + 1, jj, jk)]);
                zzwy = mydomain[c] + zind[c] * (zu * zslpx[c]);
                zwx[c] = pun[c] * (zalpha * zzwx + (1. - zalpha) * zzwy);

                z0v = copysign(0.5, pvn[c]);
                zalpha = 0.5 - z0v;
                zv = z0v - 0.5 * pvn[c] * zdt;
                zzwx = mydomain[IX(ji, jj + 1, jk)] + zind[c] * (zv * zslpy[IX(ji, jj + 1, jk)]);
                zzwy = mydomain[c] + zind[c] * (zv * zslpy[c]);
                zwy[c] = pvn[c] * (zalpha * zzwx + (1.0 - zalpha) * zzwy);
            }

    /* :185-194 (zbtr = 1. per point in the reference; set once here) */
    zbtr = 1.;
    OMP_LOOP
    for (jk = 1; jk <= jpk - 1; jk++)
        for (jj = 2; jj <= jpj - 1; jj++)
            for (ji = 2; ji <= jpi - 1; ji++) {
                size_t c = IX(ji, jj, jk);
                ztra = -(zbtr * (zwx[c] - zwx[IX(ji - 1, jj, jk)] + zwy[c] -
                                 zwy[IX(ji, jj - 1, jk)]));
                mydomain[c] = mydomain[c] + ztra;
            }

    /* :196-200 */
    for (jj = 1; jj <= jpj; jj++)
        for (ji = 1; ji <= jpi; ji++) {
            zwx[IX(ji, jj, 1)] = 0.0;
            zwx[IX(ji, jj, jpk)] = 0.0;
        }
    OMP_LOOP
    for (jk = 2; jk <= jpk - 1; jk++)
        for (jj = 1; jj <= jpj; jj++)
            for (ji = 1; ji <= jpi; ji++) {
                size_t c = IX(ji, jj, jk);
                zwx[c] = tmask[c] * (mydomain[IX(ji, jj, jk - 1)] - mydomain[c]);
            }

    /* :202-221 */
    for (jj = 1; jj <= jpj; jj++)
        for (ji = 1; ji <= jpi; ji++) zslpx[IX(ji, jj, 1)] = 0.0;
    OMP_LOOP
    for (jk = 2; jk <= jpk - 1; jk++)
        for (jj = 1; jj <= jpj; jj++)
            for (ji = 1; ji <= jpi; ji++) {
                size_t c = IX(ji, jj, jk);
                double a = zwx[c], b = zwx[IX(ji, jj, jk + 1)];
                zslpx[c] = (a + b) * (0.25 + copysign(0.25, a * b));
            }
    OMP_LOOP
    for (jk = 2; jk <= jpk - 1; jk++)
        for (jj = 1; jj <= jpj; jj++)
            for (ji = 1; ji <= jpi; ji++) {
                size_t c = IX(ji, jj, jk);
                zslpx[c] = copysign(1.0, zslpx[c]) *
                           fmin3(fabs(zslpx[c]), 2.0 * fabs(zwx[IX(ji, jj, jk + 1)]),
                                 2.0 * fabs(zwx[c]));
            }

    /* :223-241 */
    for (jj = 1; jj <= jpj; jj++)
        for (ji = 1; ji <= jpi; ji++)
            zwx[IX(ji, jj, 1)] = pwn[IX(ji, jj, 1)] * mydomain[IX(ji, jj, 1)];
    zdt = 1;
    zbtr = 1.;
    OMP_LOOP
    for (jk = 1; jk <= jpk - 1; jk++)
        for (jj = 2; jj <= jpj - 1; jj++)
            for (ji = 2; ji <= jpi - 1; ji++) {
                size_t c = IX(ji, jj, jk), c1 = IX(ji, jj, jk + 1);
                z0w = copysign(0.5, pwn[c1]);
                zalpha = 0.5 + z0w;
                zw = z0w - 0.5 * pwn[c1] * zdt * zbtr;
                zzwx = mydomain[c1] + zind[c] * (zw * zslpx[c1]);
                zzwy = mydomain[c] + zind[c] * (zw * zslpx[c]);
                zwx[c1] = pwn[c1] * (zalpha * zzwx + (1. - zalpha) * zzwy);
            }

    /* :243-251 */
    zbtr = 1.;
    OMP_LOOP
    for (jk = 1; jk <= jpk - 1; jk++)
        for (jj = 2; jj <= jpj - 1; jj++)
            for (ji = 2; ji <= jpi - 1; ji++) {
                size_t c = IX(ji, jj, jk);
                ztra = -(zbtr * (zwx[c] - zwx[IX(ji, jj, jk + 1)]));
                mydomain[c] = ztra;
            }
}

void tra_oracle_step(int jpi, int jpj, int jpk, double *mydomain,
                     const double *tsn, const double *pun, const double *pvn,
                     const double *pwn, const double *umask,
                     const double *vmask, const double *tmask,
                     const double *ztfreez, const double *rnfmsk,
                     const double *upsmsk, const double *rnfmsk_z, double *zwx,
                     double *zwy, double *zslpx, double *zslpy, double *zind)
{
    step_impl(jpi, jpj, jpk, mydomain, tsn, pun, pvn, pwn, umask, vmask, tmask, ztfreez,
              rnfmsk, upsmsk, rnfmsk_z, zwx, zwy, zslpx, zslpy, zind, 0);
}

void tra_oracle_step_omp(int jpi, int jpj, int jpk, double *mydomain,
                         const double *tsn, const double *pun, const double *pvn,
                         const double *pwn, const double *umask,
                         const double *vmask, const double *tmask,
                         const double *ztfreez, const double *rnfmsk,
                         const double *upsmsk, const double *rnfmsk_z, double *zwx,
                         double *zwy, double *zslpx, double *zslpy, double *zind)
{
    step_impl(jpi, jpj, jpk, mydomain, tsn, pun, pvn, pwn, umask, vmask, tmask, ztfreez,
              rnfmsk, upsmsk, rnfmsk_z, zwx, zwy, zslpx, zslpy, zind, 1);
}

/* tra_adv.F90:263-270: the sum of mydomain over jk < jpk and the interior
 * columns, in the reference's loop order. */
double tra_oracle_checksum(int jpi, int jpj, int jpk, const double *mydomain)
{
    double s = 0.0;
    int ji, jj, jk;
    for (jk = 1; jk <= jpk - 1; jk++)
        for (jj = 2; jj <= jpj - 1; jj++)
            for (ji = 2; ji <= jpi - 1; ji++) s = s + mydomain[IX(ji, jj, jk)];
    return s;
}
