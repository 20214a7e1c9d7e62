/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's heat-update time loop, used by the tests
 * as the checker and by bench.py as the timed CPU baseline.  The product
 * (libheat, heatdrv) never links, loads or calls this file.
 *
 * What it restates, in the reference's operation order:
 *   - the update expression  OpenMP_Single_Source/heat3D_variable_coeff.c:174-181
 *     (== 1-openmp.c:74-82 == 1-cuda.cu:103-111), evaluated left to right as
 *     ((u + rhs) + factor * S),  S = ((((A - B) + C) - D) + E) - F;
 *   - the OpenMP host parallelisation: one parallel region around the time
 *     loop, "omp for schedule(static)" over k, "omp single" pointer swap and
 *     t += dt (heat3D_variable_coeff.c:159-195);
 *   - the flat k-j-i layout with independent nx, ny, nz (1-openmp.c:28-29).
 * Built with -ffp-contract=off, as the reference serial is
 * (3D_Heat_Benchmark/NVIDIA-H100/Source-Results/OpenMP/Makefile:23), so no
 * multiply-add is fused and results are bit-identical to the reference.
 *
 * Parity is pinned: tests/test_oracle.py checks this file bit-for-bit against
 * the unmodified reference serial (built from its own sources by
 * oracle/build_ref.sh) and against the committed golden fixtures made from it.
 */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <omp.h>

#include "heat_ref.h"

#define IDX(k, j, i, ny, nx) ((size_t)(k) * (size_t)(ny) * (size_t)(nx) + (size_t)(j) * (size_t)(nx) + (size_t)(i))

/* One sweep of the update over the interior, inside an enclosing parallel
 * region (orphaned omp for).  rhs may be NULL, which means rhs == 0: u + 0.0
 * equals u for every u except -0.0, so results match a zero-filled rhs. */
static void sweep(double *restrict u_new, const double *restrict u_old,
                  const double *restrict rhs, const double *restrict kappa,
                  int nz, int ny, int nx, double factor) {
  int k;
#pragma omp for schedule(static)
  for (k = 1; k < nz - 1; k++)
    for (int j = 1; j < ny - 1; j++)
      for (int i = 1; i < nx - 1; i++) {
        size_t idx = IDX(k, j, i, ny, nx);
        size_t ip1 = idx + 1, im1 = idx - 1;
        size_t jp1 = idx + (size_t)nx, jm1 = idx - (size_t)nx;
        size_t kp1 = idx + (size_t)nx * ny, km1 = idx - (size_t)nx * ny;
        double base = rhs ? u_old[idx] + rhs[idx] : u_old[idx];
        u_new[idx] = base
          + factor * (
                (kappa[ip1] + kappa[idx]) * (u_old[ip1] - u_old[idx])
              - (kappa[idx] + kappa[im1]) * (u_old[idx] - u_old[im1])
              + (kappa[jp1] + kappa[idx]) * (u_old[jp1] - u_old[idx])
              - (kappa[idx] + kappa[jm1]) * (u_old[idx] - u_old[jm1])
              + (kappa[kp1] + kappa[idx]) * (u_old[kp1] - u_old[idx])
              - (kappa[idx] + kappa[km1]) * (u_old[idx] - u_old[km1]));
      }
}

double heat_ref_factor(double h, double dt) { return dt / h / h / 2.0; }

void heat_ref_update(double *u_new, const double *u_old, const double *rhs,
                     const double *kappa, int nz, int ny, int nx, double factor) {
#pragma omp parallel
  sweep(u_new, u_old, rhs, kappa, nz, ny, nx, factor);
}

/* Shared driver of both loop forms.  T < 0 selects the explicit count. */
static int run_loop(double *u_old, double *u_new, const double *rhs,
                    const double *kappa, int nz, int ny, int nx, double factor,
                    int nsteps, double T, double dt, double *seconds) {
  double *a = u_old, *b = u_new;
  int steps = 0;
  double t = 0.0;
  double t0 = omp_get_wtime();
#pragma omp parallel default(shared)
  {
    for (;;) {
      int go = (T < 0.0) ? (steps < nsteps) : (t < T);
      if (!go) break;
      sweep(b, a, rhs, kappa, nz, ny, nx, factor);
#pragma omp single
      {
        double *tmp = b; b = a; a = tmp;
        steps++;
        t += dt;
      }
    }
  }
  double t1 = omp_get_wtime();
  if (seconds) *seconds = t1 - t0;
  /* The result of the last step sits in a; hand it back in u_old. */
  if (a != u_old) {
    size_t n = (size_t)nz * ny * nx;
    for (size_t q = 0; q < n; ++q) u_old[q] = a[q];
  }
  return steps;
}

int heat_ref_steps(double *u_old, double *u_new, const double *rhs,
                   const double *kappa, int nz, int ny, int nx, double factor,
                   int nsteps, double *seconds) {
  if (nsteps < 0) return -1;
  return run_loop(u_old, u_new, rhs, kappa, nz, ny, nx, factor, nsteps, -1.0, 0.0, seconds);
}

int heat_ref_run_T(double *u_old, double *u_new, const double *rhs,
                   const double *kappa, int nz, int ny, int nx, double factor,
                   double T, double dt, double *seconds) {
  return run_loop(u_old, u_new, rhs, kappa, nz, ny, nx, factor, 0, T < 0.0 ? 0.0 : T, dt, seconds);
}

int heat_ref_count_steps(double T, double dt) {
  double t = 0.0;
  int steps = 0;
  while (t < T) { steps++; t += dt; }
  return steps;
}

/* Neumaier-compensated sums, sequential in index order: the accurate value
 * the device reductions are compared against. */
void heat_ref_norm(const double *u, size_t n, double *l2, double *checksum) {
  double s = 0.0, cs = 0.0, q = 0.0, cq = 0.0;
  for (size_t i = 0; i < n; ++i) {
    double x = u[i], x2 = u[i] * u[i];
    double t = s + x;
    cs += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
    s = t;
    double t2 = q + x2;
    cq += (fabs(q) >= fabs(x2)) ? (q - t2) + x2 : (x2 - t2) + q;
    q = t2;
  }
  if (checksum) *checksum = s + cs;
  if (l2) *l2 = sqrt(q + cq);
}

int heat_ref_threads(void) { return omp_get_max_threads(); }
