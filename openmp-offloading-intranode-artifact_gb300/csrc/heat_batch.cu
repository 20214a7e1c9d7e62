// Batched table kernels: one launch per kind advances every grid of that kind
// in a batch by one time step.  The host builds a tile table -- (grid, tile x,
// tile y, z range, rows per thread) entries over all active grids -- and the
// blocks stride through it (tile t goes to block t mod gridDim.x; by default
// one block per tile).  Each tile is a 32 x (8 * rows) set of (i, j) columns
// walking its z range with the same column walks the single-grid kernels use
// (heat_walk.cuh), so a grid's results are identical alone and in a batch,
// whatever the tile shape and blocks-per-SM variant the autotuner picked.
// Grids of different sizes share a launch; no block ever waits on another, so
// the kernels need no grid-wide synchronisation and cannot deadlock.  (FP32C
// grids the tuner gave two steps per launch run k_batch_fp32c_tb2 in
// heat_fp32c_tma.cu instead.)

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

// One kernel per kind -- (form, source term, blocks per SM) -- so each gets the
// register allocation (and occupancy) of its own column walk and of the
// variant the autotuner picked for the grids' size class; the host launches
// one per kind present.  A tile is 32 columns by 8 * rows rows: each thread
// walks its column in rows j, j + 8, ... one after another (the row's position
// mod 8 is the thread's y, so the FP64 / integer row split is the same for
// every rows value and the results are identical to the single-grid kernels').
template <int FORM, bool RHS, int MINB>
__global__ void __launch_bounds__(TX *TY, MINB)
    k_batch(const BatchGrid *__restrict__ grids, const BatchTile *__restrict__ tiles, int ntiles,
            int flip) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    const BatchGrid &g = grids[tl.grid];
    const int i = 1 + tl.tx * TX + threadIdx.x;
    if (i >= g.nx - 1) continue;
    const int src = g.cur ^ flip, dst = src ^ 1;
    for (int r = 0; r < tl.rows; ++r) {
      const int j = 1 + (tl.ty * tl.rows + r) * TY + threadIdx.y;
      if (j >= g.ny - 1) break;
      const size_t c = (size_t)tl.k0 * g.S + (size_t)j * g.P + i;
      run_tile<FORM, RHS>(g, c, tl.k0, tl.k1, src, dst);
    }
  }
}

// The default FP64 form's tiles (hw_rows = 4, no source term) as the
// single-grid k_fast_ws runs them: warps 0-3 walk the tile's FP64 rows and
// warps 4-7 its integer rows in separate code, each warpgroup starting with
// setmaxnreg at the launch count (65536 / (256 MINB), rounded down to 8) so
// that ptxas allocates the two walks separately.
template <int MINB>
struct WsRegs {
  static constexpr int value = (65536 / (TX * TY * MINB)) / 8 * 8;
};

template <int MINB>
__global__ void __launch_bounds__(TX *TY, MINB)
    k_batch_ws(const BatchGrid *__restrict__ grids, const BatchTile *__restrict__ tiles,
               int ntiles, int flip) {
  constexpr int REGS = WsRegs<MINB>::value;
  if (threadIdx.y < 4) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;\n" ::"n"(REGS));
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const BatchTile tl = tiles[t];
      const BatchGrid &g = grids[tl.grid];
      const int i = 1 + tl.tx * TX + threadIdx.x;
      if (i >= g.nx - 1) continue;
      const int src = g.cur ^ flip, dst = src ^ 1;
      for (int r = 0; r < tl.rows; ++r) {
        const int j = 1 + (tl.ty * tl.rows + r) * TY + threadIdx.y;
        if (j >= g.ny - 1) break;
        const size_t c = (size_t)tl.k0 * g.S + (size_t)j * g.P + i;
        walk::walk_hw<false>((double *)g.f[dst], (const double *)g.f[src], nullptr,
                             (const double *)g.w[0], (const double *)g.w[1],
                             (const double *)g.w[2], (const double *)g.w[3], g.P, g.S, c, tl.k0,
                             tl.k1);
      }
    }
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;\n" ::"n"(REGS));
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const BatchTile tl = tiles[t];
      const BatchGrid &g = grids[tl.grid];
      const int i = 1 + tl.tx * TX + threadIdx.x;
      if (i >= g.nx - 1) continue;
      const int src = g.cur ^ flip, dst = src ^ 1;
      for (int r = 0; r < tl.rows; ++r) {
        const int j = 1 + (tl.ty * tl.rows + r) * TY + threadIdx.y;
        if (j >= g.ny - 1) break;
        const size_t c = (size_t)tl.k0 * g.S + (size_t)j * g.P + i;
        walk::walk_int<false>((double *)g.f[dst], (const u64 *)g.f[src], nullptr, g.kq, g.P, g.S,
                              c, tl.k0, tl.k1);
      }
    }
  }
}

template <class K>
int occupancy_of(K kernel) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, TX * TY, 0) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return nb > 0 ? nb : 1;
}

template <int MINB>
bool ws_variant_usable() {
  static const bool ok = [] {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, k_batch_ws<MINB>) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return a.numRegs == WsRegs<MINB>::value;
  }();
  return ok;
}

// Every table kernel of one form and source term, indexed by variant.
template <int FORM, bool RHS>
cudaError_t launch_form(int v, const BatchGrid *grids, const BatchTile *tiles, int ntiles,
                        int flip, int blocks, cudaStream_t st) {
  const dim3 b(TX, TY);
  switch (v) {
    case 0: k_batch<FORM, RHS, 2><<<blocks, b, 0, st>>>(grids, tiles, ntiles, flip); break;
    case 1: k_batch<FORM, RHS, 3><<<blocks, b, 0, st>>>(grids, tiles, ntiles, flip); break;
    default: k_batch<FORM, RHS, 4><<<blocks, b, 0, st>>>(grids, tiles, ntiles, flip); break;
  }
  return cudaGetLastError();
}

template <int FORM, bool RHS>
int occupancy_form(int v) {
  switch (v) {
    case 0: return occupancy_of(k_batch<FORM, RHS, 2>);
    case 1: return occupancy_of(k_batch<FORM, RHS, 3>);
    default: return occupancy_of(k_batch<FORM, RHS, 4>);
  }
}

}  // namespace

cudaError_t launch_batch(int kind, const BatchGrid *grids, const BatchTile *tiles, int ntiles,
                         int flip, int blocks, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  const int form = form_of_kind(kind);
  const bool rhs = (kind / kNumMinb) & 1;
  const int v = kind % kNumMinb;
  if (form == kFormF32c2) return rhs ? cudaErrorInvalidValue
                                     : launch_batch_fp32c_tb2(grids, tiles, ntiles, flip, st);
  if (form == kFormMixWs) {
    if (rhs) return cudaErrorInvalidValue;
    const dim3 b(TX, TY);
    switch (v) {
      case 0: k_batch_ws<2><<<blocks, b, 0, st>>>(grids, tiles, ntiles, flip); break;
      case 1: k_batch_ws<3><<<blocks, b, 0, st>>>(grids, tiles, ntiles, flip); break;
      default: k_batch_ws<4><<<blocks, b, 0, st>>>(grids, tiles, ntiles, flip); break;
    }
    return cudaGetLastError();
  }
#define HEAT_BATCH_CASE(F)                                                            \
  case F:                                                                             \
    return rhs ? launch_form<F, true>(v, grids, tiles, ntiles, flip, blocks, st)      \
               : launch_form<F, false>(v, grids, tiles, ntiles, flip, blocks, st);
  switch (form) {
    HEAT_BATCH_CASE(kFormMix)
    HEAT_BATCH_CASE(kFormHw)
    HEAT_BATCH_CASE(kFormExact)
    HEAT_BATCH_CASE(kFormF32c)
    default: return cudaErrorInvalidValue;
  }
#undef HEAT_BATCH_CASE
}

bool batch_ws_usable(int minb) {
  switch (minb) {
    case 2: return ws_variant_usable<2>();
    case 3: return ws_variant_usable<3>();
    default: return ws_variant_usable<4>();
  }
}

int batch_blocks_per_sm(int kind) {
  const int form = form_of_kind(kind);
  const bool rhs = (kind / kNumMinb) & 1;
  const int v = kind % kNumMinb;
  if (form == kFormF32c2) return 2;  // the two-step kernel: 640 threads, 2 blocks per SM
  if (form == kFormMixWs) {
    if (rhs) return 1;  // not produced (source-term grids use kFormMix)
    switch (v) {
      case 0: return occupancy_of(k_batch_ws<2>);
      case 1: return occupancy_of(k_batch_ws<3>);
      default: return occupancy_of(k_batch_ws<4>);
    }
  }
  switch (form) {
    case kFormMix: return rhs ? occupancy_form<kFormMix, true>(v) : occupancy_form<kFormMix, false>(v);
    case kFormHw: return rhs ? occupancy_form<kFormHw, true>(v) : occupancy_form<kFormHw, false>(v);
    case kFormExact:
      return rhs ? occupancy_form<kFormExact, true>(v) : occupancy_form<kFormExact, false>(v);
    default: return rhs ? occupancy_form<kFormF32c, true>(v) : occupancy_form<kFormF32c, false>(v);
  }
}

}  // namespace heat
