/*
 * heatdrv -- host driver of the GB300 heat solver with the reference's
 * command-line surface (OpenMP_Single_Source/1-openmp.c:87-241,
 * 3D_Heat_Benchmark/NVIDIA-H100/Source-Results/CUDA/1-cuda.cu:134-290).
 *
 *   heatdrv [N [T]]            reference problem: N^3 points (default 51),
 *                              final time T (default 1.0), reference init and
 *                              dt = h^2/(12*0.95); steps while (t < T).
 *   heatdrv --config C [--n N | --nx X --ny Y --nz Z] [--steps S] [--seed K]
 *           [--dt-policy ref|cfl0.9]
 *                              seeded synthetic inputs of configuration C.
 *   common: --bitexact  reference operation order, bit-identical results
 *           --naive     one thread per point (with --bitexact semantics)
 *           --hw-fp64   default form on the hardware FP64 pipe only
 *
 * Output keeps the reference's lines ("<s> timesteps complete",
 * "Time = <sec> seconds", "Solution written to <file>") so its run/aggregate
 * scripts parse it unchanged, and adds GLUP/s, L2 norm and checksum.  The
 * timer brackets the time loop and the final device synchronisation, as
 * 1-cuda.cu:231-257 does.  WRITE_TXT=0/false/no suppresses the %.17g k-j-i
 * dump, as the reference's should_write_txt().
 *
 * The dump is named after the binary the driver is invoked as, so a link
 * named like a reference binary takes its place in the reference's run and
 * verify scripts: 1-omp writes u_openmp_1gpu.txt (1-openmp.c:228), 1-cuda
 * writes u_cuda_1gpu.txt (1-cuda.cu:278), any other name u_gb300_1gpu.txt.
 * HEAT_DUMP=<file> overrides the name.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <time.h>

#include "heat.h"

static double wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int should_write_txt(void) {
  const char *e = getenv("WRITE_TXT");
  if (!e) return 1;
  if (!strcmp(e, "0") || !strcasecmp(e, "false") || !strcasecmp(e, "no")) return 0;
  return 1;
}

static const char *dump_name(const char *argv0) {
  const char *e = getenv("HEAT_DUMP");
  if (e && *e) return e;
  const char *base = strrchr(argv0, '/');
  base = base ? base + 1 : argv0;
  if (!strcmp(base, "1-omp")) return "u_openmp_1gpu.txt";
  if (!strcmp(base, "1-cuda")) return "u_cuda_1gpu.txt";
  return "u_gb300_1gpu.txt";
}

static void die(const char *what, int rc) {
  fprintf(stderr, "ERROR: %s: %s\n", what, heat_strerror(rc));
  exit(EXIT_FAILURE);
}

int main(int argc, char **argv) {
  int n = 51, nx = 0, ny = 0, nz = 0, cfg = -1, steps = -1;
  double T = 1.0;
  unsigned long long seed = 0;
  unsigned flags = 0;
  int dt_ref = 0, npos = 0;
  for (int a = 1; a < argc; ++a) {
    const char *s = argv[a];
    const char *v = a + 1 < argc ? argv[a + 1] : NULL;
    if (s[0] != '-' || (s[1] >= '0' && s[1] <= '9') || s[1] == '.') {
      if (npos == 0) n = atoi(s);
      else if (npos == 1) T = atof(s);
      ++npos;
    } else if (!strcmp(s, "--config") && v) { cfg = atoi(v[0] == 'c' ? v + 1 : v); ++a; }
    else if (!strcmp(s, "--n") && v) { nx = ny = nz = atoi(v); ++a; }
    else if (!strcmp(s, "--nx") && v) { nx = atoi(v); ++a; }
    else if (!strcmp(s, "--ny") && v) { ny = atoi(v); ++a; }
    else if (!strcmp(s, "--nz") && v) { nz = atoi(v); ++a; }
    else if (!strcmp(s, "--steps") && v) { steps = atoi(v); ++a; }
    else if (!strcmp(s, "--seed") && v) { seed = strtoull(v, NULL, 10); ++a; }
    else if (!strcmp(s, "--dt-policy") && v) { dt_ref = !strcmp(v, "ref"); ++a; }
    else if (!strcmp(s, "--bitexact")) flags |= HEAT_BITEXACT;
    else if (!strcmp(s, "--naive")) flags |= HEAT_NAIVE | HEAT_BITEXACT;
    else if (!strcmp(s, "--hw-fp64")) flags |= HEAT_HWFP64;
    else { fprintf(stderr, "unknown argument: %s\n", s); return 2; }
  }
  if (cfg < 0) nx = ny = nz = n;
  if (nx < 3 || ny < 3 || nz < 3) { fprintf(stderr, "grid must be at least 3 points per axis\n"); return 2; }

  printf("\n**** ONE GPU GB300 STARTS ****\n");
  size_t total = (size_t)nx * ny * nz;
  printf("\n=== MEMORY ESTIMATE (GLOBAL) ===\n");
  printf("Grid size: %d x %d x %d = %zu points\n", nx, ny, nz, total);
  printf("Memory per global array: %.3f GB\n", total * sizeof(double) / 1e9);
  printf("================================\n\n");

  double *kappa = malloc(total * sizeof(double)), *u0 = malloc(total * sizeof(double));
  double *rhs = NULL;
  if (!kappa || !u0) { fprintf(stderr, "ERROR: malloc failed (host arrays)\n"); return 1; }
  double h, dt;
  int rc;
  if (cfg < 0) {
    rhs = malloc(total * sizeof(double));
    if (!rhs) { fprintf(stderr, "ERROR: malloc failed (host arrays)\n"); return 1; }
    rc = heat_inputs_reference(n, kappa, rhs, u0, &h, &dt);
  } else {
    rc = heat_inputs_config(cfg, (uint64_t)seed, nx, ny, nz, kappa, u0, &h, &dt);
    if (dt_ref) dt = h * h / (12.0 * 0.95);
  }
  if (rc != HEAT_OK) die("input generation", rc);
  double factor = dt / h / h / 2.0;

  printf("=== SIMULATION PARAMETERS ===\n");
  printf("Grid size (n):           %d\n", nx);
  if (steps < 0) printf("Final time (T):          %.6f\n", T);
  else printf("Time steps:              %d\n", steps);
  printf("Grid spacing (h):        %.6e\n", h);
  printf("Time step (dt):          %.6e\n", dt);
  printf("Diffusion factor:        %.6e\n", factor);
  if (steps < 0) printf("Estimated timesteps:     ~%d\n", (int)(T / dt));
  printf("CFL condition (dt/h^2):  %.6f (should be < 0.5)\n", dt / (h * h));
  printf("Kernel form:             %s\n",
         (flags & HEAT_NAIVE) ? "naive bit-exact" : (flags & HEAT_BITEXACT) ? "bit-exact" : "default");
  printf("==============================\n\n");

  heat_desc d;
  memset(&d, 0, sizeof d);
  d.nx = nx; d.ny = ny; d.nz = nz; d.h = h; d.dt = dt;
  d.kappa = kappa; d.u0 = u0; d.rhs = rhs;
  d.precision = HEAT_FP64; d.flags = flags; d.stream = NULL;
  heat_ctx *ctx = NULL;
  rc = heat_init(&ctx, &d);
  if (rc != HEAT_OK) die("heat_init", rc);

  printf("\n=== SIMULATION STARTS ===\n");
  int done = 0;
  double t0 = wtime();
  if (steps < 0) rc = heat_run(ctx, T, &done);
  else { rc = heat_step(ctx, steps); done = steps; }
  if (rc == HEAT_OK) rc = heat_sync(ctx);
  double sec = wtime() - t0;
  if (rc != HEAT_OK) die("time loop", rc);
  printf("\n%d timesteps complete\n", done);
  printf("Time = %f seconds\n", sec);
  double upd = (double)(nx - 2) * (ny - 2) * (nz - 2) * done;
  printf("GLUP/s = %.3f\n", sec > 0 ? upd / sec / 1e9 : 0.0);
  double l2 = 0, cs = 0;
  rc = heat_norm(ctx, &l2, &cs);
  if (rc != HEAT_OK) die("heat_norm", rc);
  printf("L2 norm = %.17g\nchecksum = %.17g\n", l2, cs);
  printf("=== SIMULATION ENDS ===\n");

  if (should_write_txt()) {
    rc = heat_get_field(ctx, u0);
    if (rc != HEAT_OK) die("heat_get_field", rc);
    const char *dump = dump_name(argv[0]);
    FILE *f = fopen(dump, "w");
    if (!f) { perror("fopen"); return 1; }
    for (size_t q = 0; q < total; ++q) fprintf(f, "%.17g\n", u0[q]);
    if (fclose(f) != 0) { perror("fclose"); return 1; }
    printf("Solution written to %s\n", dump);
  }
  heat_destroy(ctx);
  free(kappa); free(u0); free(rhs);
  printf("\n**** ONE GPU GB300 FINISHED ****\n");
  return 0;
}
