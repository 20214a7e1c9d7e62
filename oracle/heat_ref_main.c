/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.  Command-line front end of the CPU
 * restatement (heat_ref.c), used by the tests and by bench.py's CPU baseline.
 *
 *   heat_ref N [T]
 *       The reference serial's own problem and output, as
 *       OpenMP_Single_Source/heat3D_variable_coeff.c:61-210: prints
 *       "<s> timesteps complete", "Time = <sec> seconds",
 *       "h=..., dt=..., T=..., # time steps=<s>" and, unless WRITE_TXT is
 *       0/false/no, writes u_ref.txt (%.17g, k-j-i).
 *
 *   heat_ref --config C --nx X --ny Y --nz Z --steps S [--seed K] [--l2]
 *       Seeded synthetic inputs of benchmark configuration C (the same
 *       generator the library exports), S explicit steps; prints one JSON
 *       line with seconds, GLUP/s, threads and (with --l2) norm/checksum.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "heat_ref.h"
#include "heat.h"   /* heat_inputs_reference / heat_inputs_config (host-only) */

static int should_write_txt(void) {
  const char *e = getenv("WRITE_TXT");
  if (!e) return 1;
  if (!strcmp(e, "0") || !strcasecmp(e, "false") || !strcasecmp(e, "no")) return 0;
  return 1;
}

static int reference_mode(int n, double T) {
  size_t N = (size_t)n * n * n;
  double *kappa = malloc(N * sizeof(double)), *rhs = malloc(N * sizeof(double));
  double *u_old = malloc(N * sizeof(double)), *u_new = calloc(N, sizeof(double));
  if (!kappa || !rhs || !u_old || !u_new) { fprintf(stderr, "malloc failed\n"); return 1; }
  double h, dt;
  heat_inputs_reference(n, kappa, rhs, u_old, &h, &dt);
  double factor = heat_ref_factor(h, dt), sec = 0.0;
  int steps = heat_ref_run_T(u_old, u_new, rhs, kappa, n, n, n, factor, T, dt, &sec);
  printf("%d timesteps complete\n", steps);
  printf("Time = %.6f seconds\n", sec);
  printf("h=%g, dt=%g, T=%g, # time steps=%d\n", h, dt, T, steps);
  if (should_write_txt()) {
    FILE *f = fopen("u_ref.txt", "w");
    if (!f) { perror("fopen"); return 1; }
    for (size_t q = 0; q < N; ++q) fprintf(f, "%.17g\n", u_old[q]);
    fclose(f);
    printf("Solution written to %s\n", "u_ref.txt");
  }
  free(kappa); free(rhs); free(u_old); free(u_new);
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2 || argv[1][0] != '-') {
    int n = argc > 1 ? atoi(argv[1]) : 51;
    double T = argc > 2 ? atof(argv[2]) : 1.0;
    if (n < 3) { fprintf(stderr, "N must be >= 3\n"); return 2; }
    return reference_mode(n, T);
  }
  int cfg = 0, nx = 0, ny = 0, nz = 0, steps = 1, want_l2 = 0;
  unsigned long long seed = 0;
  for (int a = 1; a < argc; ++a) {
    const char *s = argv[a];
    const char *v = a + 1 < argc ? argv[a + 1] : NULL;
    if (!strcmp(s, "--config") && v) { cfg = atoi(v); ++a; }
    else if (!strcmp(s, "--n") && v) { nx = ny = nz = atoi(v); ++a; }
    else if (!strcmp(s, "--nx") && v) { nx = atoi(v); ++a; }
    else if (!strcmp(s, "--ny") && v) { ny = atoi(v); ++a; }
    else if (!strcmp(s, "--nz") && v) { nz = atoi(v); ++a; }
    else if (!strcmp(s, "--steps") && v) { steps = atoi(v); ++a; }
    else if (!strcmp(s, "--seed") && v) { seed = strtoull(v, NULL, 10); ++a; }
    else if (!strcmp(s, "--l2")) { want_l2 = 1; }
    else { fprintf(stderr, "unknown argument %s\n", s); return 2; }
  }
  if (nx < 3 || ny < 3 || nz < 3 || steps < 0) { fprintf(stderr, "bad sizes\n"); return 2; }
  size_t N = (size_t)nx * ny * nz;
  double *kappa = malloc(N * sizeof(double)), *u_old = malloc(N * sizeof(double));
  double *u_new = malloc(N * sizeof(double));
  if (!kappa || !u_old || !u_new) { fprintf(stderr, "malloc failed\n"); return 1; }
  double h, dt;
  if (heat_inputs_config(cfg, (uint64_t)seed, nx, ny, nz, kappa, u_old, &h, &dt) != 0) {
    fprintf(stderr, "input generation failed\n");
    return 1;
  }
  for (size_t q = 0; q < N; ++q) u_new[q] = u_old[q];
  double factor = heat_ref_factor(h, dt), sec = 0.0;
  int done = heat_ref_steps(u_old, u_new, NULL, kappa, nz, ny, nx, factor, steps, &sec);
  double upd = (double)(nx - 2) * (ny - 2) * (nz - 2) * done;
  printf("{\"config\": %d, \"nx\": %d, \"ny\": %d, \"nz\": %d, \"steps\": %d, "
         "\"seconds\": %.6f, \"glups\": %.6f, \"threads\": %d",
         cfg, nx, ny, nz, done, sec, sec > 0 ? upd / sec / 1e9 : 0.0, heat_ref_threads());
  if (want_l2) {
    double l2, cs;
    heat_ref_norm(u_old, N, &l2, &cs);
    printf(", \"l2\": %.17g, \"checksum\": %.17g", l2, cs);
  }
  printf("}\n");
  free(kappa); free(u_old); free(u_new);
  return 0;
}
