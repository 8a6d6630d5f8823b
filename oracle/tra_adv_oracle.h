/* TEST INFRASTRUCTURE ONLY: the oracle of the tracer-advection benchmark
 * (see tra_adv_oracle.c). */
#ifndef TRA_ADV_ORACLE_H
#define TRA_ADV_ORACLE_H
void tra_oracle_init(int jpi, int jpj, int jpk, double *mydomain, double *tsn,
                     double *pun, double *pvn, double *pwn, double *umask,
                     double *vmask, double *tmask, double *ztfreez,
                     double *rnfmsk, double *upsmsk, double *rnfmsk_z);
void tra_oracle_step(int jpi, int jpj, int jpk, double *mydomain,
                     const double *tsn, const double *pun, const double *pvn,
                     const double *pwn, const double *umask,
                     const double *vmask, const double *tmask,
                     const double *ztfreez, const double *rnfmsk,
                     const double *upsmsk, const double *rnfmsk_z, double *zwx,
                     double *zwy, double *zslpx, double *zslpy, double *zind);
void tra_oracle_step_omp(int jpi, int jpj, int jpk, double *mydomain,
                         const double *tsn, const double *pun, const double *pvn,
                         const double *pwn, const double *umask,
                         const double *vmask, const double *tmask,
                         const double *ztfreez, const double *rnfmsk,
                         const double *upsmsk, const double *rnfmsk_z, double *zwx,
                         double *zwy, double *zslpx, double *zslpy, double *zind);
double tra_oracle_checksum(int jpi, int jpj, int jpk, const double *mydomain);
#endif
