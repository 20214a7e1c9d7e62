// Device-side tables of the batched persistent kernel (heat_batch.cu) and the
// host helpers that build and tune them (heat_batch.cpp, heat_tune.cpp).
#pragma once

#include "heat_internal.h"

namespace heat {

enum BatchForm : int {
  kFormMix = 0,    // default FP64: hw_rows warps on the FP64 pipe, the rest integer
  kFormHw = 1,     // default FP64 on the FP64 pipe only
  kFormExact = 2,  // bit-exact FP64 (face kappa sums)
  kFormF32c = 3,   // FP32-compensated
  kFormMixWs = 4,  // default FP64, hw_rows = 4, no source term: warpgroup-split kernel
};

// One grid of a batch as the kernel sees it.  f[b] / cr[b] are the two field
// (and carry) buffers; cur names the one that held the current field when the
// table was built, and each launch's `flip` says how many steps (mod 2) have
// been taken since.
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
};

// A (32 x 8)-column tile of grid `grid` walking planes [k0, k1).
struct BatchTile {
  int grid;
  int tx, ty;
  int k0, k1;
};

constexpr int kNumForms = 5;
// A kernel kind is (form, source term): kind = 2 * form + (rhs != NULL).
constexpr int kNumKinds = 2 * kNumForms;
// Launch the batch kernel of one kind over `ntiles` tiles (all of that kind).
cudaError_t launch_batch(int kind, const BatchGrid *grids, const BatchTile *tiles, int ntiles,
                         int flip, int blocks, cudaStream_t st);
int batch_blocks_per_sm(int kind);
// Whether the warpgroup-split table kernel compiled to the register count
// its setmaxnreg bounds assume (else kFormMix is used instead).
bool batch_ws_usable();

// Form of a context in the batch kernel, or -1 if the batch cannot run it.
int batch_form(const heat_ctx *c);
// z-chunk for a grid of this form and depth: the autotuner's cached choice for
// its size class, else a default.
int tuned_kchunk(int form, int nz);

// heat_batch_run with the final stream synchronisation optional (sync=false:
// the launches are queued and the bookkeeping advanced on return).
int batch_run(heat_batch *b, long long max_steps, long long *steps_taken, bool sync);
cudaStream_t batch_stream(heat_batch *b);

}  // namespace heat
