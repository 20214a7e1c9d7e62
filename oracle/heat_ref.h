/* ORACLE -- TEST INFRASTRUCTURE ONLY.  CPU restatement of the reference's
 * heat-update loop; see heat_ref.c for what it follows and how it is pinned. */
#ifndef HEAT_REF_H
#define HEAT_REF_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
double heat_ref_factor(double h, double dt);
void heat_ref_update(double *u_new, const double *u_old, const double *rhs,
                     const double *kappa, int nz, int ny, int nx, double factor);
/* nsteps explicit steps; result left in u_old; returns steps taken. */
int heat_ref_steps(double *u_old, double *u_new, const double *rhs,
                   const double *kappa, int nz, int ny, int nx, double factor,
                   int nsteps, double *seconds);
/* while (t < T) { step; t += dt; }; result in u_old; returns steps taken. */
int heat_ref_run_T(double *u_old, double *u_new, const double *rhs,
                   const double *kappa, int nz, int ny, int nx, double factor,
                   double T, double dt, double *seconds);
int heat_ref_count_steps(double T, double dt);
void heat_ref_norm(const double *u, size_t n, double *l2, double *checksum);
int heat_ref_threads(void);
#ifdef __cplusplus
}
#endif
#endif
