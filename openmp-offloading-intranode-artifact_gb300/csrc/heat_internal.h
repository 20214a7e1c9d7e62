// Internal declarations shared by the translation units of libheat.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "heat.h"

// Device layout of one field: nz planes of ny rows of `pitch` doubles
// (pitch >= nx, a multiple of 4 so every row starts on a 32-byte boundary).
// Padding columns hold zeros and are never read as data.
struct heat_geom {
  int nx, ny, nz;
  int pitch;          // elements per row on the device
  size_t plane;       // pitch * ny
  size_t elems;       // plane * nz
};

struct heat_ctx {
  heat_geom g;
  double h, dt, factor;
  int precision;
  unsigned flags;
  int device;
  cudaStream_t stream;
  bool own_stream;

  // FP64 state: ping-pong fields; cur indexes the current (u_old) one.
  double *u[2];
  int cur;
  double *rhs;              // NULL when the problem has no source term

  // Per-form coefficient planes (only the ones the chosen kernel uses).
  double *kappa;            // raw conductivity (naive kernel)
  double *ks[3];            // face kappa sums kx, ky, kz (bit-exact kernel)
  double *c0;               // centre weight 1 - sum of face weights (fast, FP64 pipe)
  double *cf[3];            // face weights factor*(kappa_a+kappa_b) (fast, FP64 pipe)
  unsigned long long *kq;   // round(factor*kappa*2^64) (fast, integer pipes)
  int hw_rows;              // warps per block on the FP64 pipe in the hybrid kernel

  // FP32C state.
  float *v[2];              // FP32 fields
  uint16_t *carry[2];       // BF16 Kahan carry planes
  float *fcf[3];            // FP32 face weights
  float *frhs;              // FP32 source (NULL when none)

  // Device flag a kernel sets when a bounded wait ran out (HEAT_ETIMEOUT).
  int *err;

  // Norm scratch: per-block partial sums, then the final pair.
  double *partials;
  int n_partials;

  long long steps_done;
  long long launches;
};

// ---- kernel launchers (each returns cudaError_t of the launch) ----------
namespace heat {

#ifdef __CUDACC__
// Face weight factor * (ka + kb) and centre weight
// 1 - (((((e + w) + n) + s) + u) + d) of the default FP64 form, every operation
// rounded on its own (no fused multiply-add), so every kernel that forms them
// gets the same bits.
__device__ __forceinline__ double fw(double factor, double ka, double kb) {
  return __dmul_rn(factor, __dadd_rn(ka, kb));
}
__device__ __forceinline__ double centre(double e, double w, double n, double s, double u,
                                         double d) {
  return __dsub_rn(1.0, __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(e, w), n), s), u), d));
}
#endif

constexpr int kNormBlocks = 152 * 4;   // partial-sum blocks of the norm pass

// Bound of every device-side mbarrier wait in the TMA kernels (try_wait
// attempts, each suspending up to ~2 us); a wait that runs out sets the
// context's error flag and the launch returns with its outputs unwritten.
constexpr unsigned kWaitLimit = 1u << 22;

// Planes per block for a launch of (tile_x x tile_y)-column tiles over the
// grid's interior: enough z-chunks that tiles x chunks reaches `want` blocks
// (16 per SM of GB300's 152 by default), at least 8 planes each.
inline int plane_chunk(const heat_geom &g, int tile_x, int tile_y, long want = 152L * 16) {
  const long tiles =
      (long)((g.nx - 2 + tile_x - 1) / tile_x) * ((g.ny - 2 + tile_y - 1) / tile_y);
  const long chunks = (want + tiles - 1) / tiles;
  const int interior = g.nz - 2;
  int kc = (int)((interior + chunks - 1) / chunks);
  if (kc < 8) kc = 8;
  if (kc > interior) kc = interior;
  return kc;
}

// Blocks of `kernel` resident on the current GPU at once: its occupancy per
// SM at `threads` threads and `smem` bytes of dynamic shared memory per block,
// times the SM count; 0 when the runtime cannot say (heat_abi.cpp).  The
// launchers look it up once per process (one GPU model per process).
long resident_blocks(const void *kernel, int threads, size_t smem);

// Planes per block for a launch of (tile_x x tile_y)-column tiles whose blocks
// run `resident` at a time: enough z-chunks that the launch spans about
// `waves` waves of resident blocks, so the last wave, which the GPU may run
// partly empty, is a small share of it; at least `min_planes` planes per chunk
// (each chunk re-reads its halo planes and refills its pipeline) unless that
// would leave fewer than two waves.  At 512^3 the default FP64 launch's 1,024
// tiles in 3 chunks made 5.05 waves of 608 blocks: 126.4 GLUP/s; 15 chunks
// (25 waves): 133.4.  Falls back to plane_chunk when `resident` is unknown.
inline int wave_chunk(const heat_geom &g, int tile_x, int tile_y, long resident,
                      long waves = 24, int min_planes = 16, int fill_planes = 8) {
  if (resident <= 0) return plane_chunk(g, tile_x, tile_y);
  const long tiles =
      (long)((g.nx - 2 + tile_x - 1) / tile_x) * ((g.ny - 2 + tile_y - 1) / tile_y);
  const int interior = g.nz - 2;
  long chunks = (resident * waves + tiles - 1) / tiles;
  const long max_chunks = interior / min_planes > 1 ? interior / min_planes : 1;
  if (chunks > max_chunks) chunks = max_chunks;
  // A grid too small for `waves` waves at that depth still gets two waves of
  // blocks where chunks of `fill_planes` planes allow it, so it does not leave
  // SMs idle.
  long fill = (2 * resident + tiles - 1) / tiles;
  if (fill > interior / fill_planes) fill = interior / fill_planes;
  if (chunks < fill) chunks = fill;
  if (chunks < 1) chunks = 1;
  return (int)((interior + chunks - 1) / chunks);
}

// heat_fp64_exact.cu (compiled with --fmad=false)
cudaError_t launch_exact_raw(double *u_new, const double *u_old, const double *rhs,
                             const double *kappa, const heat_geom &g, double factor,
                             cudaStream_t st);
cudaError_t launch_exact_faces(double *u_new, const double *u_old, const double *rhs,
                               double *const ks[3], const heat_geom &g, double factor,
                               cudaStream_t st);
cudaError_t launch_naive(double *u_new, const double *u_old, const double *rhs,
                         const double *kappa, const heat_geom &g, double factor,
                         cudaStream_t st);
cudaError_t launch_face_sums(double *const ks[3], const double *kappa, const heat_geom &g,
                             cudaStream_t st);

// heat_fp64_fast.cu
cudaError_t launch_fast_coeffs(double *c0, double *const cf[3], const double *kappa,
                               const heat_geom &g, double factor, cudaStream_t st);
cudaError_t launch_fast(double *u_new, const double *u_old, const double *rhs,
                        const double *c0, double *const cf[3], const heat_geom &g,
                        cudaStream_t st);

// heat_fp64_int.cu
// K and c0, cx, cy, cz in one pass (the two kernels below, fused; same values).
cudaError_t launch_weights_setup(unsigned long long *K, double *c0, double *const cf[3], int *bad,
                                 const double *kappa, const heat_geom &g, double factor,
                                 cudaStream_t st);
cudaError_t launch_kq_setup(unsigned long long *K, int *bad, const double *kappa,
                            const heat_geom &g, double factor, cudaStream_t st);
// hw_rows of the 8 warps in each block take the FP64 pipe, the rest the
// integer pipes; K may be NULL only when hw_rows == 8, c0/cf only when 0.
// err: the context's flag, set when a bounded wait of the TMA-staged kernel
// runs out (HEAT_ETIMEOUT).
cudaError_t launch_fast_mix(double *u_new, const double *u_old, const double *rhs,
                            const unsigned long long *K, const double *c0,
                            double *const cf[3], const heat_geom &g, int hw_rows,
                            int *err, cudaStream_t st);

// heat_fp64_tma.cu: the hw_rows = 4 split with every input staged by TMA
// (bit-identical to the k_fast_ws launch), with or without a source term.
bool fast_tma_usable(const heat_geom &g, bool rhs = false);
cudaError_t launch_fast_tma(double *u_new, const double *u_old, const unsigned long long *K,
                            const double *c0, double *const cf[3], const double *rhs,
                            const heat_geom &g, int *err, cudaStream_t st,
                            unsigned wait_limit = kWaitLimit);
// n steps of context c from buffer `cur` on stream st with its own
// single-grid kernels (two steps per launch where its form has them); the
// context's bookkeeping is untouched.  ctx_flips gives the parity of buffer
// swaps those n steps make (a two-step launch swaps once).
cudaError_t enqueue_ctx_steps(heat_ctx *c, int cur, long long n, cudaStream_t st,
                              long long *launches);
int ctx_flips(const heat_ctx *c, long long n);
// One step of context c from buffer `cur` with its single-grid one-step kernel.
cudaError_t enqueue_one_step(heat_ctx *c, int cur, cudaStream_t st, long long *launches);

// heat_fp32c.cu
cudaError_t launch_fp32c(float *v_new, uint16_t *c_new, const float *v, const uint16_t *cr,
                         float *const w[3], const float *rhs, const heat_geom &g,
                         cudaStream_t st);
cudaError_t launch_split(float *v, uint16_t *cr, const double *u, size_t total, cudaStream_t st);
cudaError_t launch_widen(double *u, const float *v, const uint16_t *cr, size_t total,
                         cudaStream_t st);
cudaError_t launch_f32_weights(float *const w[3], const double *kappa, const heat_geom &g,
                               double factor, cudaStream_t st);
cudaError_t launch_to_f32(float *o, const double *a, size_t total, cudaStream_t st);

// heat_fp32c_tma.cu: two steps per launch (temporal blocking, TMA staging).
// wait_limit bounds every mbarrier wait of the launch (kWaitLimit in product
// use; smaller only to exercise the failure path).
bool fp32c_tb2_ok(const heat_geom &g);
cudaError_t launch_fp32c_tb2(float *v_new, uint16_t *c_new, const float *v, const uint16_t *cr,
                             float *const w[3], const heat_geom &g, int *err, cudaStream_t st,
                             unsigned wait_limit = kWaitLimit);
// Whether a context steps with launch_fp32c_tb2.
bool two_step_form(const heat_ctx *c);
// HEAT_ETIMEOUT if a kernel of context c reported a bounded wait running out
// (the flag is cleared once reported), else HEAT_OK.  Synchronises c's stream.
int check_err(heat_ctx *c);
// Record a failed CUDA call for heat_strerror() and return HEAT_ECUDA.
int cuda_fail(cudaError_t e, const char *what);

// heat_reduce.cu
cudaError_t launch_norm_f64(const double *u, const heat_geom &g, double *partials,
                            int nblocks, cudaStream_t st);
// Norm of the FP32C state u = v - c (widened to FP64 per point).
cudaError_t launch_norm_f32c(const float *v, const uint16_t *cr, const heat_geom &g,
                             double *partials, int nblocks, cudaStream_t st);
// sum (a-b)^2, sum b^2 and max |a-b| of two FP64 fields of one geometry;
// partials needs 3*nblocks+3 doubles, results at partials[3*nblocks..].
cudaError_t launch_diff_f64(const double *a, const double *b, const heat_geom &g,
                            double *partials, int nblocks, cudaStream_t st);

}  // namespace heat
