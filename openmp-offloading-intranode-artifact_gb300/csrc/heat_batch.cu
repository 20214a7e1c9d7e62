// Batched persistent kernel: one launch advances every grid of a batch by one
// time step.  The host builds a tile table -- (grid, tile x, tile y, z range)
// entries over all active grids -- and a fixed set of resident blocks strides
// through it (tile t goes to block t mod gridDim.x).  Each tile is a (32 x 8)
// set of (i, j) columns walking its z range with the same column walks the
// single-grid kernels use (heat_walk.cuh), so a grid's results are identical
// alone and in a batch.  Grids of different precision forms and sizes share a
// launch; no block ever waits on another, so the kernel needs no grid-wide
// synchronisation and cannot deadlock.

#include "heat_batch_internal.h"
#include "heat_walk.cuh"

namespace heat {
namespace {

constexpr int TX = 32, TY = 8;
typedef unsigned long long u64;

template <int FORM, bool RHS>
__device__ __forceinline__ void run_tile(const BatchGrid &g, size_t c, int kb, int ke,
                                         int src, int dst) {
  if (FORM == kFormMix) {
    if ((int)threadIdx.y < g.hw_rows)
      walk::walk_hw<RHS>((double *)g.f[dst], (const double *)g.f[src], (const double *)g.rhs,
                         (const double *)g.w[0], (const double *)g.w[1], (const double *)g.w[2],
                         (const double *)g.w[3], g.P, g.S, c, kb, ke);
    else
      walk::walk_int<RHS>((double *)g.f[dst], (const u64 *)g.f[src], (const double *)g.rhs, g.kq,
                          g.P, g.S, c, kb, ke);
  } else if (FORM == kFormHw) {
    walk::walk_hw<RHS>((double *)g.f[dst], (const double *)g.f[src], (const double *)g.rhs,
                       (const double *)g.w[0], (const double *)g.w[1], (const double *)g.w[2],
                       (const double *)g.w[3], g.P, g.S, c, kb, ke);
  } else if (FORM == kFormExact) {
    walk::walk_exact_faces<RHS>((double *)g.f[dst], (const double *)g.f[src],
                                (const double *)g.rhs, (const double *)g.w[0],
                                (const double *)g.w[1], (const double *)g.w[2], g.P, g.S, c, kb,
                                ke, g.factor);
  } else {
    walk::walk_fp32c<RHS>((float *)g.f[dst], g.cr[dst], (const float *)g.f[src], g.cr[src],
                          (const float *)g.w[0], (const float *)g.w[1], (const float *)g.w[2],
                          (const float *)g.rhs, g.P, g.S, c, kb, ke);
  }
}

// One kernel per (form, source term) kind, so each gets the register
// allocation (and occupancy) of its own column walk; the host launches one per
// kind present.
// Resident blocks per SM each kind is compiled for (caps its registers): the
// memory-bound forms want many warps in flight; the hybrid form takes 3 (80
// registers, a few spills), as its single-grid kernel does -- 123 GLUP/s on
// configuration 3's grids in the table alone, against 101 with 2.
template <int FORM>
struct MinBlocks {
  static constexpr int value = FORM == kFormMix ? 3 : 4;
};

template <int FORM, bool RHS>
__global__ void __launch_bounds__(TX *TY, MinBlocks<FORM>::value)
    k_batch(const BatchGrid *__restrict__ grids, const BatchTile *__restrict__ tiles, int ntiles,
            int flip) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    const BatchGrid &g = grids[tl.grid];
    const int i = 1 + tl.tx * TX + threadIdx.x;
    const int j = 1 + tl.ty * TY + threadIdx.y;
    if (i >= g.nx - 1 || j >= g.ny - 1) continue;
    const int src = g.cur ^ flip, dst = src ^ 1;
    const size_t c = (size_t)tl.k0 * g.S + (size_t)j * g.P + i;
    run_tile<FORM, RHS>(g, c, tl.k0, tl.k1, src, dst);
  }
}

// The default FP64 form's tiles (hw_rows = 4, no source term) as the
// single-grid k_fast_ws runs them: 4 blocks per SM, warps 0-3 walk the tile's
// FP64 rows and warps 4-7 its integer rows in separate code, each warpgroup
// starting with setmaxnreg at the launch count (64) so that ptxas allocates
// the two walks separately.
constexpr int kWsRegs = 64;

__global__ void __launch_bounds__(TX *TY, 4)
    k_batch_ws(const BatchGrid *__restrict__ grids, const BatchTile *__restrict__ tiles,
               int ntiles, int flip) {
  if (threadIdx.y < 4) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;\n" ::"n"(kWsRegs));
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const BatchTile tl = tiles[t];
      const BatchGrid &g = grids[tl.grid];
      const int i = 1 + tl.tx * TX + threadIdx.x;
      const int j = 1 + tl.ty * TY + threadIdx.y;
      if (i >= g.nx - 1 || j >= g.ny - 1) continue;
      const int src = g.cur ^ flip, dst = src ^ 1;
      const size_t c = (size_t)tl.k0 * g.S + (size_t)j * g.P + i;
      walk::walk_hw<false>((double *)g.f[dst], (const double *)g.f[src], nullptr,
                           (const double *)g.w[0], (const double *)g.w[1], (const double *)g.w[2],
                           (const double *)g.w[3], g.P, g.S, c, tl.k0, tl.k1);
    }
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;\n" ::"n"(kWsRegs));
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const BatchTile tl = tiles[t];
      const BatchGrid &g = grids[tl.grid];
      const int i = 1 + tl.tx * TX + threadIdx.x;
      const int j = 1 + tl.ty * TY + threadIdx.y;
      if (i >= g.nx - 1 || j >= g.ny - 1) continue;
      const int src = g.cur ^ flip, dst = src ^ 1;
      const size_t c = (size_t)tl.k0 * g.S + (size_t)j * g.P + i;
      walk::walk_int<false>((double *)g.f[dst], (const u64 *)g.f[src], nullptr, g.kq, g.P, g.S, c,
                            tl.k0, tl.k1);
    }
  }
}

template <int FORM, bool RHS>
int occupancy() {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<FORM, RHS>, TX * TY, 0) !=
      cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return nb > 0 ? nb : 1;
}

}  // namespace

cudaError_t launch_batch(int kind, const BatchGrid *grids, const BatchTile *tiles, int ntiles,
                         int flip, int blocks, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  const dim3 b(TX, TY);
#define HEAT_BATCH_CASE(F, R)                                                   \
  case 2 * (F) + (R):                                                           \
    k_batch<(F), (R)><<<blocks, b, 0, st>>>(grids, tiles, ntiles, flip);        \
    break;
  if (kind == 2 * kFormMixWs) {
    k_batch_ws<<<blocks, b, 0, st>>>(grids, tiles, ntiles, flip);
    return cudaGetLastError();
  }
  switch (kind) {
    HEAT_BATCH_CASE(kFormMix, 0)
    HEAT_BATCH_CASE(kFormMix, 1)
    HEAT_BATCH_CASE(kFormHw, 0)
    HEAT_BATCH_CASE(kFormHw, 1)
    HEAT_BATCH_CASE(kFormExact, 0)
    HEAT_BATCH_CASE(kFormExact, 1)
    HEAT_BATCH_CASE(kFormF32c, 0)
    HEAT_BATCH_CASE(kFormF32c, 1)
    default: return cudaErrorInvalidValue;
  }
#undef HEAT_BATCH_CASE
  return cudaGetLastError();
}

bool batch_ws_usable() {
  static const bool ok = [] {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, k_batch_ws) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return a.numRegs == kWsRegs;
  }();
  return ok;
}

int batch_blocks_per_sm(int kind) {
  if (kind == 2 * kFormMixWs) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_ws, TX * TY, 0) != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
    return nb > 0 ? nb : 1;
  }
  if (kind == 2 * kFormMixWs + 1) return 1;  // not produced (source-term grids use kFormMix)
  switch (kind) {
    case 2 * kFormMix: return occupancy<kFormMix, false>();
    case 2 * kFormMix + 1: return occupancy<kFormMix, true>();
    case 2 * kFormHw: return occupancy<kFormHw, false>();
    case 2 * kFormHw + 1: return occupancy<kFormHw, true>();
    case 2 * kFormExact: return occupancy<kFormExact, false>();
    case 2 * kFormExact + 1: return occupancy<kFormExact, true>();
    case 2 * kFormF32c: return occupancy<kFormF32c, false>();
    default: return occupancy<kFormF32c, true>();
  }
}

}  // namespace heat
