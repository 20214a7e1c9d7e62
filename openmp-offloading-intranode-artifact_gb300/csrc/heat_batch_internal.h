// Device-side tables of the batched persistent kernel (heat_batch.cu) and the
// host helpers that build and tune them (heat_batch.cpp, heat_tune.cpp).
#pragma once

#include <cuda.h>

#include "heat_internal.h"

namespace heat {

enum BatchForm : int {
  kFormMix = 0,    // default FP64: hw_rows warps on the FP64 pipe, the rest integer
  kFormHw = 1,     // default FP64 on the FP64 pipe only
  kFormExact = 2,  // bit-exact FP64 (face kappa sums)
  kFormF32c = 3,   // FP32-compensated, one step per launch
  kFormMixWs = 4,  // default FP64, hw_rows = 4, no source term: warpgroup-split kernel
  kFormF32c2 = 5,  // FP32-compensated, two steps per launch (TMA-staged, 32 x 16 tiles)
};

// One grid of a batch as the kernel sees it.  f[b] / cr[b] are the two field
// (and carry) buffers; cur names the one that held the current field when the
// table was built, and each launch's `flip` says how many buffer swaps (mod 2)
// the grid has made since.
struct BatchGrid {
  int form;
  int nx, ny, nz, P;
  int hw_rows;
  int cur;
  int pad_;
  size_t S;
  double factor;
  void *f[2];
  uint16_t *cr[2];
  const void *rhs;
  const void *w[4];  // Mix/Hw: c0, cx, cy, cz   Exact: kx, ky, kz   F32c: wx, wy, wz
  const unsigned long long *kq;
  int *err;            // the context's error flag (bounded waits that ran out)
  const void *tmaps;   // F32c2: seven CUtensorMaps in device memory (v0 v1 c0 c1 wx wy wz)
};

// A tile of grid `grid` walking planes [k0, k1): 32 columns (tx) by 8 * rows
// rows (ty), each thread walking `rows` columns 8 rows apart; F32c2 tiles are
// 32 x 16 (two-step kernel's tile) and rows is 1.
struct BatchTile {
  int grid;
  int tx, ty;
  int k0, k1;
  int rows;
};

constexpr int kNumForms = 6;
// Blocks-per-SM variants of the table kernels (their register caps): 2, 3, 4.
constexpr int kNumMinb = 3;
constexpr int kMinbLo = 2;
// A kernel kind is (form, source term, blocks-per-SM variant):
// kind = (2 * form + (rhs != NULL)) * kNumMinb + (minb - kMinbLo).
constexpr int kNumKinds = 2 * kNumForms * kNumMinb;
inline int kind_of(int form, bool rhs, int minb) {
  return (2 * form + (rhs ? 1 : 0)) * kNumMinb + (minb - kMinbLo);
}
inline int form_of_kind(int kind) { return kind / (2 * kNumMinb); }
// Launch the batch kernel of one kind over `ntiles` tiles (all of that kind).
cudaError_t launch_batch(int kind, const BatchGrid *grids, const BatchTile *tiles, int ntiles,
                         int flip, int blocks, cudaStream_t st);
int batch_blocks_per_sm(int kind);
// Whether the warpgroup-split table kernel's variant for `minb` blocks per SM
// compiled to the register count its setmaxnreg bounds assume (else the
// general hybrid kernel runs those tiles).
bool batch_ws_usable(int minb = 4);
// heat_fp32c_tma.cu: the two-step FP32C table kernel and its per-grid maps.
cudaError_t launch_batch_fp32c_tb2(const BatchGrid *grids, const BatchTile *tiles, int ntiles,
                                   int flip, cudaStream_t st);
bool encode_fp32c_maps(CUtensorMap *m7, float *const v[2], uint16_t *const c[2],
                       float *const w[3], const heat_geom &g);

// Form of a context in the batch kernel, or -1 if the batch cannot run it.
int batch_form(const heat_ctx *c);

// The autotuner's choices for a size class (heat_tune.cpp): z-chunk, rows per
// thread, blocks-per-SM variant and temporal depth (FP32C: 2 = two steps per
// launch).  Classes not tuned yet get the defaults.
struct TuneChoice {
  int kchunk, rows, minb, depth;
};
TuneChoice tuned_choice(int form, int nz);
// Default blocks-per-SM variant of a form's table kernel.
inline int default_minb(int form) { return form == kFormMix ? 3 : 4; }

// heat_batch_run with the final stream synchronisation optional (sync=false:
// the launches are queued and the bookkeeping advanced on return).
int batch_run(heat_batch *b, long long max_steps, long long *steps_taken, bool sync);
cudaStream_t batch_stream(heat_batch *b);

}  // namespace heat
