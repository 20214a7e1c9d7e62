// Default FP64 form: the hybrid launch (FP64-pipe and integer-pipe warps in
// one kernel) and the per-point fixed-point weights it needs.  The two
// column walks and the integer evaluation are in heat_walk.cuh.

#include <algorithm>
#include <cstdlib>

#include "heat_internal.h"
#include "heat_walk.cuh"

namespace heat {
namespace {

constexpr int TX = 32, TY = 8;
typedef unsigned long long u64;
typedef long long i64;

// Hybrid launch: grid rows j with (j - 1) mod 8 < hw_rows walk their columns
// on the FP64 pipe and the others on the integer pipes, so both kinds of
// execution unit on each SM work at once.  The split is by global row, so any
// block height (TYB rows) gives the same assignment -- and the batch kernel's
// 8-row tiles the same too.  hw_rows = 0 is integer only.
template <bool RHS, int TYB, int MINB>
__global__ void __launch_bounds__(TX *TYB, MINB)
    k_fast_mix(double *__restrict__ un, const double *__restrict__ u,
               const double *__restrict__ rhs, const u64 *__restrict__ K,
               const double *__restrict__ c0, const double *__restrict__ cx,
               const double *__restrict__ cy, const double *__restrict__ cz, int nx, int ny,
               int nz, int P, size_t S, int kchunk, int hw_rows) {
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TYB + threadIdx.y;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (i >= nx - 1 || j >= ny - 1 || kb >= ke) return;
  const size_t c = (size_t)kb * S + (size_t)j * P + i;
  if (((j - 1) & 7) < hw_rows)
    walk::walk_hw<RHS>(un, u, rhs, c0, cx, cy, cz, P, S, c, kb, ke);
  else
    walk::walk_int<RHS>(un, reinterpret_cast<const u64 *>(u), rhs, K, P, S, c, kb, ke);
}

// The hw_rows = 4 split as one launch of 4 blocks per SM (64 registers per
// thread) whose two warpgroups run separate code: warps 0-3 the FP64 rows,
// warps 4-7 the integer rows.  Each warpgroup starts with setmaxnreg at the
// launch count (64): no registers move between them, but the instruction
// bounds each region for ptxas's allocator, which then spills half as much
// (76 B against 152 B without it).  Measured at 512^3: 111 GLUP/s (114 since
// the FP64 walk's loop is unrolled by 2) against 99 for the same kernel
// without setmaxnreg and 102-105 for k_fast_mix at 3
// blocks per SM; moving registers from the FP64 to the integer warpgroup
// (56/72, 48/80) or 3 blocks per SM with any split measured 83-105.  The host
// launches it only when the compiled register count is kWsRegs, since a
// setmaxnreg.inc above the launch count would wait for registers forever.
constexpr int kWsRegs = 64;

template <bool RHS, int MINB = 4, int REGS = kWsRegs>
__global__ void __launch_bounds__(256, MINB)
    k_fast_ws(double *__restrict__ un, const double *__restrict__ u,
              const double *__restrict__ rhs, const u64 *__restrict__ K,
              const double *__restrict__ c0, const double *__restrict__ cx,
              const double *__restrict__ cy, const double *__restrict__ cz, int nx, int ny,
              int nz, int P, size_t S, int kchunk) {
  if (threadIdx.y < 4) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;\n" ::"n"(REGS));
    const int i = 1 + blockIdx.x * TX + threadIdx.x;
    const int j = 1 + blockIdx.y * TY + threadIdx.y;
    const int kb = 1 + blockIdx.z * kchunk;
    const int ke = min(kb + kchunk, nz - 1);
    if (i >= nx - 1 || j >= ny - 1 || kb >= ke) return;
    const size_t c = (size_t)kb * S + (size_t)j * P + i;
    walk::walk_hw<RHS, RHS ? 1 : 2>(un, u, rhs, c0, cx, cy, cz, P, S, c, kb, ke);
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;\n" ::"n"(REGS));
    const int i = 1 + blockIdx.x * TX + threadIdx.x;
    const int j = 1 + blockIdx.y * TY + threadIdx.y;
    const int kb = 1 + blockIdx.z * kchunk;
    const int ke = min(kb + kchunk, nz - 1);
    if (i >= nx - 1 || j >= ny - 1 || kb >= ke) return;
    const size_t c = (size_t)kb * S + (size_t)j * P + i;
    walk::walk_int<RHS>(un, reinterpret_cast<const u64 *>(u), rhs, K, P, S, c, kb, ke);
  }
}

// K[c] = round(factor * kappa[c] * 2^64) from the error-free product
// p + q = factor * kappa (q = fma(factor, kappa, -p)); padding columns get 0.
// bad[0] is set when the fixed-point form cannot represent the problem:
// negative or non-finite kappa, factor*kappa >= 1/4, or a centre weight
// 1 - sum_f factor (kappa_a + kappa_b) below 2^-40.
__global__ void k_kq_setup(u64 *__restrict__ K, int *__restrict__ bad,
                           const double *__restrict__ kap, int nx, int ny, int nz, int P,
                           size_t S, double factor) {
  // One row (j, k) per block iteration, its points across the threads: no
  // per-point index division.
  const long rows = (long)ny * nz;
  for (long r = blockIdx.x; r < rows; r += gridDim.x)
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    const int j = (int)(r % ny), k = (int)(r / ny);
    const size_t c = (size_t)k * S + (size_t)j * P + i;
    if (i >= nx) {
      K[c] = 0;
      continue;
    }
    double kc = kap[c];
    double p = factor * kc;
    double q = fma(factor, kc, -p);
    bool ok = isfinite(kc) && kc >= 0.0 && isfinite(p) && p < 0.25;
    u64 v = 0;
    if (ok) {
      double hp = ldexp(p, 64), hq = ldexp(q, 64);
      v = __double2ull_rn(hp);
      v = (u64)((i64)v + __double2ll_rn(hq));
    }
    K[c] = v;
    if (ok && i > 0 && j > 0 && k > 0 && i < nx - 1 && j < ny - 1 && k < nz - 1) {
      double s = factor * ((kc + kap[c + 1]) + (kc + kap[c - 1]) + (kc + kap[c + P]) +
                           (kc + kap[c - P]) + (kc + kap[c + S]) + (kc + kap[c - S]));
      if (!(s <= 1.0 - 0x1p-40)) ok = false;
    }
    if (!ok) atomicOr(bad, 1);
  }
}


// k_kq_setup and k_fast_coeffs (heat_fp64_fast.cu) in one pass, the same
// values bit for bit (both form the weights with fw / centre, every operation
// rounded on its own, so no contraction choice of the compiler can differ): each
// thread walks one (i, j) column over a chunk of planes, keeping kappa and the
// z-face weight of the plane below in registers, so a point forms its three
// stored face weights cx, cy, cz, re-forms only the two lower in-plane ones
// (cx[c-1], cy[c-P]; same operands, same rounding) for its centre weight
//   c0 = 1 - (((((cx[c] + cx[c-1]) + cy[c]) + cy[c-P]) + cz[c]) + cz[c-S]),
// and takes the fixed-point check from the same sum: a centre weight below
// 2^-40 (k_kq_setup's bound on factor * sum of the six kappa sums; the two sums
// differ by a few ulps) marks the problem as outside the fixed-point range.
// About 22 FP64 operations per point against 42 for the two kernels.
__global__ void __launch_bounds__(256)
    k_weights_setup(u64 *__restrict__ K, double *__restrict__ c0, double *__restrict__ cx,
                    double *__restrict__ cy, double *__restrict__ cz, int *__restrict__ bad,
                    const double *__restrict__ kap, int nx, int ny, int nz, int P, size_t S,
                    double factor, int kchunk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  const int k0 = blockIdx.z * kchunk;
  const int k1 = min(k0 + kchunk, nz);
  if (i >= P || k0 >= k1) return;
  size_t c = (size_t)k0 * S + (size_t)j * P + i;
  if (i >= nx) {  // padding column
    for (int k = k0; k < k1; ++k, c += S) {
      K[c] = 0;
      c0[c] = cx[c] = cy[c] = cz[c] = 0.0;
    }
    return;
  }
  bool ok_all = true;
  double kc = kap[c];
  double zd = (k0 > 0) ? fw(factor, kap[c - S], kc) : 0.0;  // cz of the plane below
  for (int k = k0; k < k1; ++k, c += S) {
    const double ku = (k + 1 < nz) ? kap[c + S] : 0.0;
    // fixed-point weight, as k_kq_setup
    const double p = factor * kc;
    const double q = fma(factor, kc, -p);
    bool ok = isfinite(kc) && kc >= 0.0 && isfinite(p) && p < 0.25;
    u64 v = 0;
    if (ok) {
      v = __double2ull_rn(p * 0x1p64);
      v = (u64)((i64)v + __double2ll_rn(q * 0x1p64));
    }
    K[c] = v;
    // face weights, as k_fast_coeffs
    const double wx = (i + 1 < nx) ? fw(factor, kc, kap[c + 1]) : 0.0;
    const double wy = (j + 1 < ny) ? fw(factor, kc, kap[c + P]) : 0.0;
    const double wz = (k + 1 < nz) ? fw(factor, kc, ku) : 0.0;
    cx[c] = wx;
    cy[c] = wy;
    cz[c] = wz;
    double w = 0.0;
    if (i > 0 && j > 0 && k > 0 && i < nx - 1 && j < ny - 1 && k < nz - 1) {
      w = centre(wx, fw(factor, kap[c - 1], kc), wy, fw(factor, kap[c - P], kc), wz, zd);
      if (ok && !(w >= 0x1p-40)) ok = false;
    }
    c0[c] = w;
    ok_all &= ok;
    zd = wz;
    kc = ku;
  }
  if (!ok_all) atomicOr(bad, 1);
}

}  // namespace

cudaError_t launch_weights_setup(unsigned long long *K, double *c0, double *const cf[3], int *bad,
                                 const double *kappa, const heat_geom &g, double factor,
                                 cudaStream_t st) {
  // z-chunks so that the columns times chunks reach ~2048 threads per SM
  const long cols = (long)g.pitch * g.ny;
  const long want = 152L * 2048;
  const int chunks = (int)std::max(1L, std::min<long>(g.nz, (want + cols - 1) / cols));
  const int kc = (g.nz + chunks - 1) / chunks;
  dim3 gr((g.pitch + 255) / 256, g.ny, (g.nz + kc - 1) / kc);
  k_weights_setup<<<gr, 256, 0, st>>>(K, c0, cf[0], cf[1], cf[2], bad, kappa, g.nx, g.ny, g.nz,
                                      g.pitch, g.plane, factor, kc);
  return cudaGetLastError();
}

cudaError_t launch_kq_setup(unsigned long long *K, int *bad, const double *kappa,
                            const heat_geom &g, double factor, cudaStream_t st) {
  k_kq_setup<<<152 * 8, 256, 0, st>>>(K, bad, kappa, g.nx, g.ny, g.nz, g.pitch, g.plane, factor);
  return cudaGetLastError();
}

namespace {

template <bool RHS, int TYB, int MINB>
void launch_mix_shape(double *u_new, const double *u_old, const double *rhs,
                      const unsigned long long *K, const double *c0, double *const cf[3],
                      const heat_geom &g, int hw_rows, cudaStream_t st) {
  static const long resident =
      resident_blocks((const void *)k_fast_mix<RHS, TYB, MINB>, TX * TYB, 0);
  const int kc = wave_chunk(g, TX, TYB, resident);
  dim3 gr((g.nx - 2 + TX - 1) / TX, (g.ny - 2 + TYB - 1) / TYB, (g.nz - 2 + kc - 1) / kc);
  k_fast_mix<RHS, TYB, MINB><<<gr, dim3(TX, TYB), 0, st>>>(
      u_new, u_old, rhs, K, c0, cf[0], cf[1], cf[2], g.nx, g.ny, g.nz, g.pitch, g.plane, kc,
      hw_rows);
}

// True when k_fast_ws<RHS> compiled to exactly kWsRegs registers per thread
// (checked once per process).
template <bool RHS, int MINB = 4, int REGS = kWsRegs>
bool ws_usable() {
  static const bool ok = [] {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, k_fast_ws<RHS, MINB, REGS>) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return a.numRegs == REGS;
  }();
  return ok;
}

template <bool RHS, int MINB = 4, int REGS = kWsRegs>
void launch_ws(double *u_new, const double *u_old, const double *rhs,
               const unsigned long long *K, const double *c0, double *const cf[3],
               const heat_geom &g, cudaStream_t st) {
  static const long resident =
      resident_blocks((const void *)k_fast_ws<RHS, MINB, REGS>, TX * TY, 0);
  const int kc = wave_chunk(g, TX, TY, resident);
  dim3 gr((g.nx - 2 + TX - 1) / TX, (g.ny - 2 + TY - 1) / TY, (g.nz - 2 + kc - 1) / kc);
  k_fast_ws<RHS, MINB, REGS><<<gr, dim3(TX, TY), 0, st>>>(u_new, u_old, rhs, K, c0, cf[0], cf[1],
                                                          cf[2], g.nx, g.ny, g.nz, g.pitch,
                                                          g.plane, kc);
}

}  // namespace

cudaError_t launch_fast_mix(double *u_new, const double *u_old, const double *rhs,
                            const unsigned long long *K, const double *c0,
                            double *const cf[3], const heat_geom &g, int hw_rows,
                            int *err, cudaStream_t st) {
  if (hw_rows < 0) hw_rows = 0;
  if (hw_rows > 8) hw_rows = 8;
  // Default split: the TMA-staged launch (heat_fp64_tma.cu), same bits as
  // k_fast_ws, with or without a source term; HEAT_FP64_NO_TMA=1 selects
  // k_fast_ws for comparison runs.
  static const bool no_tma = [] {
    const char *e = std::getenv("HEAT_FP64_NO_TMA");
    return e && e[0] == '1';
  }();
  if (hw_rows == 4 && err && !no_tma && fast_tma_usable(g, rhs != nullptr))
    return launch_fast_tma(u_new, u_old, K, c0, cf, rhs, g, err, st);
  // Default split (hw_rows = 4): k_fast_ws.  Other splits: 8-row blocks with
  // registers capped for 3 resident blocks per SM (a few spills, more warps
  // to hide the integer walk's load latency): 101 GLUP/s at 512^3 against 94
  // for 2 blocks per SM.
  // With a source term the walks need more registers: the same split at 3
  // blocks per SM (80 registers, no spills) runs the reference problem at 97
  // GLUP/s (512^3) against 74 for k_fast_mix and 78 at 4 blocks per SM.
  if (!rhs && hw_rows == 4 && ws_usable<false>())
    launch_ws<false>(u_new, u_old, rhs, K, c0, cf, g, st);
  else if (rhs && hw_rows == 4 && ws_usable<true, 3, 80>())
    launch_ws<true, 3, 80>(u_new, u_old, rhs, K, c0, cf, g, st);
  else if (rhs)
    launch_mix_shape<true, 8, 2>(u_new, u_old, rhs, K, c0, cf, g, hw_rows, st);
  else
    launch_mix_shape<false, 8, 3>(u_new, u_old, rhs, K, c0, cf, g, hw_rows, st);
  return cudaGetLastError();
}

}  // namespace heat
