/*
 * heat.h -- C ABI of the GB300 (sm_103a) 3D variable-coefficient heat solver.
 *
 * The solver advances   du/dt = div(kappa grad u) + f   on a uniform grid with
 * zero Dirichlet boundaries by explicit time steps.  Each step applies the
 * 7-point update of the reference serial solver
 *   OpenMP_Single_Source/heat3D_variable_coeff.c:174-181
 *   u_new = u_old + rhs + factor * ( (kE+kC)(uE-uC) - (kC+kW)(uC-uW)
 *                                  + (kN+kC)(uN-uC) - (kC+kS)(uC-uS)
 *                                  + (kU+kC)(uU-uC) - (kC+kD)(uC-uD) )
 * with factor = dt/h/h/2 (heat3D_variable_coeff.c:84) to every interior point.
 *
 * Layout everywhere in this header: k-j-i with i fastest, offset
 * k*ny*nx + j*nx + i, exactly the reference's IDX() (1-openmp.c:28-29).
 * x == i, y == j, z == k.  Boundary points (i,j,k at 0 or n-1) are never
 * written and keep the values they were given (zero in every reference run).
 *
 * Every function returns an int status: HEAT_OK (0) or a negative HEAT_E*
 * code; heat_strerror() turns it into text.  Nothing in the library calls
 * exit() or abort(); the reference exits from CUDA_CHECK
 * (3D_Heat_Benchmark/NVIDIA-H100/Source-Results/CUDA/1-cuda.cu:42-50), a
 * caller that wants that behaviour checks the status and exits itself.
 *
 * Threading: a heat_ctx is not thread-safe; distinct contexts may be driven
 * from distinct host threads.  All work of a context is ordered on one CUDA
 * stream (its own, or the one passed in heat_desc.stream).
 */
#ifndef HEAT_H
#define HEAT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define HEAT_OK        0
#define HEAT_EINVAL   (-1)   /* bad argument: sizes, NULL pointers, dt      */
#define HEAT_ENOMEM   (-2)   /* device or host allocation failed            */
#define HEAT_ECUDA    (-3)   /* a CUDA runtime call failed                  */
#define HEAT_ETIMEOUT (-4)   /* a bounded device-side wait ran out          */
#define HEAT_EBUDGET  (-5)   /* request exceeds the HBM budget (server)     */
#define HEAT_ENODEV   (-6)   /* no CUDA device, or not an sm_103 device     */
#define HEAT_ESTATE   (-7)   /* call not valid in the context's state       */

/* ---- precision forms ----------------------------------------------------- */
#define HEAT_FP64   0  /* FP64 fields; default kernel family (see flags)     */
#define HEAT_FP32C  1  /* FP32 u + BF16 Kahan carry, FP32 face coefficients  */

/* ---- flags (heat_desc.flags) ------------------------------------------- */
/* Reference operation order, no FMA contraction: results are bit-identical
 * to heat3D_variable_coeff.c built with -ffp-contract=off (the reference's
 * --fmad=false CUDA build, CUDA/Makefile:36-37).  Without this flag the
 * FP64 form uses precomputed face coefficients and is held to <=1e-12
 * relative error against the reference instead.                              */
#define HEAT_BITEXACT   0x1u
/* Force the one-thread-per-point kernel (debug / comparison only).           */
#define HEAT_NAIVE      0x2u
/* Use only the hardware FP64 pipe in the default FP64 form (no integer
 * accumulation); for comparison runs.                                         */
#define HEAT_HWFP64     0x4u
/* HEAT_FP32C: one time step per launch.  By default pairs of steps run in
 * one launch with TMA-staged plane tiles (bit-identical results).            */
#define HEAT_NO_TEMPORAL 0x8u

typedef struct heat_ctx heat_ctx;

/* Problem description.  The host arrays are read during heat_init only. */
typedef struct heat_desc {
  int nx, ny, nz;          /* points per axis, boundary included, each >= 3  */
  double h;                /* grid spacing                                   */
  double dt;               /* time step; factor = dt/h/h/2 inside            */
  const double *kappa;     /* host, nz*ny*nx, conductivity at points         */
  const double *u0;        /* host, nz*ny*nx, initial field (boundary kept)  */
  const double *rhs;       /* host, nz*ny*nx, per-step source; NULL = none   */
  int precision;           /* HEAT_FP64 | HEAT_FP32C                         */
  unsigned flags;          /* HEAT_BITEXACT | HEAT_NAIVE | HEAT_HWFP64 |
                              HEAT_NO_TEMPORAL                               */
  void *stream;            /* cudaStream_t to use, or NULL for an own stream */
} heat_desc;

/* ---- the solver ABI ------------------------------------------------------ */

/* Allocate device fields, copy kappa/u0/rhs in, precompute face coefficients.
 * Replaces the reference's host init + cudaMalloc/cudaMemcpy block
 * (1-cuda.cu:200-224, 1-openmp.c:153-179).                                   */
int heat_init(heat_ctx **out, const heat_desc *d);

/* Advance nsteps explicit steps (asynchronous on the context's stream).
 * Replaces the body of the reference's time loop, one heat_update() per step
 * plus the pointer swap (1-cuda.cu:238-250, 1-openmp.c:193-205).            */
int heat_step(heat_ctx *c, int nsteps);

/* Reference time-loop semantics: while (t < T) { step; t += dt; } with t an
 * FP64 host accumulator starting at 0 (heat3D_variable_coeff.c:155-193).
 * The step count is replicated on the host; *steps_out receives it.         */
int heat_run(heat_ctx *c, double T, int *steps_out);

/* L2 norm sqrt(sum u^2) and checksum sum u over all nz*ny*nx points of the
 * current field (FP64, deterministic two-pass warp-shuffle reduction).
 * No reference counterpart; rel-L2 follows compare.py:60 of the reference's
 * verify pipeline.  Synchronises the context's stream.                      */
int heat_norm(heat_ctx *c, double *l2, double *checksum);

/* L2 norm and checksum of a caller-owned FP64 device field u (dense k-j-i,
 * row length nx, nz*ny*nx doubles) that allocates nothing: no cudaMalloc,
 * no cudaFree, no host allocation.  No counterpart in the reference.
 * For callers that must not allocate while they run -- a serving loop whose
 * HBM is all committed to its admission budget or to another allocator, or a
 * monitoring hook between time steps that cannot take the device-wide stall
 * of cudaFree/cudaMalloc.  Its scratch is a static device array sized for
 * nz <= HEAT_NORM_NOALLOC_MAX_NZ planes (256 KiB, held by every GPU that loads
 * the library); larger nz returns HEAT_EINVAL.  The first call on a device
 * looks the array's address up.  All calls on a device share the array:
 * calls that overlap on the GPU race, so issue them from one stream.  Runs on
 * stream (cudaStream_t, NULL = legacy default) and synchronises it, so it
 * cannot be captured into a CUDA graph.  Summation order differs from heat_norm's, so results
 * agree with it to rounding (<= 1e-13 relative), not bit for bit.          */
#define HEAT_NORM_NOALLOC_MAX_NZ 16384
int heat_norm_noalloc(const double *u, int nz, int ny, int nx, double *l2,
                      double *checksum, void *stream);

/* Copy the current field (the reference's u_old after the swap,
 * 1-cuda.cu:264) to / from a host array of nz*ny*nx doubles, k-j-i.
 * For HEAT_FP32C the FP32 value plus its carry is widened to FP64.          */
int heat_get_field(heat_ctx *c, double *u_host);
int heat_set_field(heat_ctx *c, const double *u_host);

/* Wait for all work queued on the context's stream.                          */
int heat_sync(heat_ctx *c);

/* Steps taken so far and kernel launches issued so far by this context.     */
int heat_stats(heat_ctx *c, long long *steps_done, long long *kernel_launches);

/* Release device memory and the context's own stream.                        */
int heat_destroy(heat_ctx *c);

const char *heat_strerror(int status);

/* ---- batches: many grids advanced together over one tile table ---------- */

/* No counterpart in the reference (it runs one grid per process).  A batch
 * holds contexts of any size and form (HEAT_FP64 default or HEAT_BITEXACT,
 * HEAT_FP32C; not HEAT_NAIVE) on one device.  heat_batch_run advances every
 * context that still has scheduled steps by one step per launch of one kernel
 * per kind present (form x source term x the tuned blocks-per-SM variant),
 * each walking a tile table over all grids of its kind (FP32C grids whose
 * size class the tuner gave two steps per launch advance in pairs of steps);
 * grids of at least 2 M interior points step with their single-grid kernels
 * beside the table; runs of 16 steps are captured once as a CUDA graph and
 * replayed.  Per-context results are identical to heat_step on the context
 * alone.  While a context is in a batch, step it through the batch (stepping
 * it directly is detected and the batch rebuilds its table).                  */
typedef struct heat_batch heat_batch;
#define HEAT_BATCH_NO_GRAPHS     0x1u  /* plain launches only                  */
#define HEAT_BATCH_PERSISTENT    0x2u  /* resident blocks stride the tile table */
#define HEAT_BATCH_SERIAL_FORMS  0x4u  /* kinds one after another, one stream  */

int heat_batch_create(heat_batch **out, void *stream, unsigned flags);
/* Schedule `steps` more steps for c (adds c to the batch if new).            */
int heat_batch_add(heat_batch *b, heat_ctx *c, long long steps);
int heat_batch_remove(heat_batch *b, heat_ctx *c);
int heat_batch_pending(heat_batch *b, heat_ctx *c, long long *steps_left);
/* Run until every context's scheduled steps are done, or at most max_steps
 * batch steps if max_steps >= 0.  Synchronises the batch's stream.           */
int heat_batch_run(heat_batch *b, long long max_steps, long long *steps_taken);
int heat_batch_stats(heat_batch *b, long long *kernel_launches, long long *graph_launches,
                     long long *batch_steps);
int heat_batch_destroy(heat_batch *b);

/* Autotune the batch table kernels for one form (precision + HEAT_BITEXACT /
 * HEAT_HWFP64 flags) over the size classes (grid depth nz <= 64, 128, 256,
 * 384, 512, 1024, 2048, larger) up to max_nz (<= 0: all), and write the JSON
 * cache ($HEAT_TUNE_CACHE, else heat_tune.json beside the library; read again
 * when that path changes).  Per class it picks, by timing a GPU-filling batch
 * of that class, the z-chunk, the rows per thread, the blocks-per-SM variant
 * and, for HEAT_FP32C, the temporal depth (heat_tune_entry).  Classes already
 * cached are kept unless force != 0.  No counterpart in the reference, whose
 * launch shape is a fixed dim3 block(8,8,8) (1-cuda.cu:123-128).            */
int heat_tune_batch(int precision, unsigned flags, int max_nz, int force);
/* z-chunk the batch kernel will use for a grid of depth nz.                   */
int heat_tune_lookup(int precision, unsigned flags, int nz, int *kchunk);

/* Every choice the batch makes for a grid of depth nz of this form.         */
typedef struct heat_tune_entry {
  int kchunk;          /* planes per tile's z-walk                          */
  int rows;            /* rows per thread: tiles of 32 x (8 * rows) columns  */
  int blocks_per_sm;   /* table kernel variant: 2, 3 or 4 resident blocks    */
  int depth;           /* time steps per launch: 1, or 2 (HEAT_FP32C grids
                          without a source term, 32 x 16 TMA-staged tiles)   */
} heat_tune_entry;
int heat_tune_choice(int precision, unsigned flags, int nz, heat_tune_entry *out);

/* ---- continuous-batching solve server ------------------------------------ */

/* No counterpart in the reference.  A server owns one GPU worker thread, two
 * context-creation threads and `prep_threads` input-generation threads.
 * Submitted requests get seeded synthetic inputs (heat_inputs_config, into
 * pinned host buffers the server reuses; at most 16 GB ahead of admission),
 * are admitted in arrival order while their device bytes fit `budget_bytes`
 * (a request that does not fit waits; the next few behind it may go first),
 * stay device-resident until done, and advance together through a heat_batch
 * in ticks of `tick_steps` steps; new requests join at the next tick as memory
 * frees up.  A request larger than the whole budget completes with status
 * HEAT_EBUDGET.                                                              */
typedef struct heat_server heat_server;

typedef struct heat_request {
  int nx, ny, nz;          /* points per axis, each >= 3                      */
  long long steps;         /* explicit steps to take                          */
  int precision;           /* HEAT_FP64 (default form) | HEAT_FP32C           */
  int cfg;                 /* input distribution, as heat_inputs_config       */
  uint64_t seed;
  double *field_out;       /* optional host nz*ny*nx buffer for the final field,
                              valid until the request's result is polled      */
} heat_request;

typedef struct heat_result {
  uint64_t id;
  int status;              /* HEAT_OK, HEAT_EBUDGET, ...                      */
  double l2, checksum;     /* heat_norm of the final field                    */
  double submit_ms, admit_ms, done_ms;  /* since the server was created      */
  double updates;          /* interior points x steps                         */
} heat_result;

typedef struct heat_server_summary {
  long long submitted, admitted, completed, rejected, resident, queued;
  double p50_ms, p99_ms, mean_ms, max_ms;  /* submit-to-done latency         */
  double glups;            /* completed updates / (last done - first admit)   */
  double updates, busy_ms;
  size_t budget_bytes, bytes_in_use, peak_bytes;
  long long batch_steps, kernel_launches;
  double gpu_ms;           /* device time inside ticks (gaps: GPU waiting for the host) */
} heat_server_summary;

int heat_server_create(heat_server **out, size_t budget_bytes, int tick_steps, int prep_threads);
/* Thread-safe; returns at once with the request's id.                         */
int heat_server_submit(heat_server *s, const heat_request *r, uint64_t *id_out);
/* Move up to max finished results into out; *n_out = how many.               */
int heat_server_poll(heat_server *s, heat_result *out, int max, int *n_out);
/* Block until every submitted request has finished.                           */
int heat_server_wait_idle(heat_server *s);
int heat_server_stats(heat_server *s, heat_server_summary *st);
/* Stop: requests not yet admitted are dropped, resident ones finish.         */
int heat_server_destroy(heat_server *s);

/* ---- drop-in for the reference's per-step device call -------------------- */

/* Same signature and meaning as the reference's
 *   static void heat_update(double *u_new, const double *u_old,
 *                           const double *rhs, const double *kappa,
 *                           int nz, int ny, int nx, double factor,
 *                           int device_id)
 * (OpenMP_Single_Source/1-openmp.c:55-58; CUDA wrapper 1-cuda.cu:116-119):
 * device pointers, k-j-i layout with row length nx, updates every interior
 * point of u_new from u_old, never touches boundary points.  The result is
 * bit-identical to the reference's --fmad=false build.  rhs may be NULL.
 * Runs on the legacy default stream of device_id, as the reference's
 * <<<grid, block>>> launch does; returns a status instead of exiting.      */
int heat_update(double *u_new, const double *u_old, const double *rhs,
                const double *kappa, int nz, int ny, int nx, double factor,
                int device_id);

/* heat_update on an explicit stream (cudaStream_t passed as void*).          */
int heat_update_async(double *u_new, const double *u_old, const double *rhs,
                      const double *kappa, int nz, int ny, int nx,
                      double factor, void *stream);

/* ---- host-side input generators ------------------------------------------ */

/* The reference's own initial data (heat3D_variable_coeff.c:79-150,
 * 1-openmp.c:103-106,153-163) for an n^3 grid: h = 1/(n-1),
 * dt = h*h/(12*0.95), rhs = dt*(1+cos cos cos), kappa = 0.5+0.45 sin sin sin,
 * u0 = sin sin sin inside and exactly 0 on the boundary.  Arrays are n^3.   */
int heat_inputs_reference(int n, double *kappa, double *rhs, double *u0,
                          double *h_out, double *dt_out);

/* Synthetic inputs of the benchmark configurations (cfg 0..4, seeded):
 *   0: kappa = exp(0.5 g), g ~ N(0,1) i.i.d.; u0 ~ U[0,1) inside
 *   1: kappa = 1 + 0.9 sin(2 pi x) sin(4 pi y) cos(2 pi z);
 *      u0 = Gaussian bump, sigma 0.05, centre ~ U[0.3,0.7]^3
 *   2: kappa log-normal (sigma 1) smoothed by 3 passes of a 3^3 box filter;
 *      u0 ~ U[0,1) inside
 *   3, 4: as 0 (per-grid / per-request seeds)
 * h = 1/(max(nx,ny,nz)-1); dt = 0.9 h^2 / (6 kappa_max).  u0 is 0 on the
 * boundary.  Arrays are nz*ny*nx, k-j-i.                                     */
int heat_inputs_config(int cfg, uint64_t seed, int nx, int ny, int nz,
                       double *kappa, double *u0, double *h_out,
                       double *dt_out);

#ifdef __cplusplus
}
#endif

#endif /* HEAT_H */
