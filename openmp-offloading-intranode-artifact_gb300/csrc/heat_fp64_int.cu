// Default FP64 form: the hybrid launch (FP64-pipe and integer-pipe warps in
// one kernel) and the per-point fixed-point weights it needs.  The two
// column walks and the integer evaluation are in heat_walk.cuh.

#include "heat_internal.h"
#include "heat_walk.cuh"

namespace heat {
namespace {

constexpr int TX = 32, TY = 8;
typedef unsigned long long u64;
typedef long long i64;

// Hybrid launch: in every (32 x 8) block the first hw_rows warps walk their
// columns on the FP64 pipe and the others on the integer pipes, so both
// kinds of execution unit on each SM work at once.  Both paths compute the
// same update (to within their roundings); hw_rows = 0 is integer only.
template <bool RHS>
__global__ void __launch_bounds__(TX *TY)
    k_fast_mix(double *__restrict__ un, const double *__restrict__ u,
               const double *__restrict__ rhs, const u64 *__restrict__ K,
               const double *__restrict__ c0, const double *__restrict__ cx,
               const double *__restrict__ cy, const double *__restrict__ cz, int nx, int ny,
               int nz, int P, size_t S, int kchunk, int hw_rows) {
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (i >= nx - 1 || j >= ny - 1 || kb >= ke) return;
  const size_t c = (size_t)kb * S + (size_t)j * P + i;
  if ((int)threadIdx.y < hw_rows)
    walk::walk_hw<RHS>(un, u, rhs, c0, cx, cy, cz, P, S, c, kb, ke);
  else
    walk::walk_int<RHS>(un, reinterpret_cast<const u64 *>(u), rhs, K, P, S, c, kb, ke);
}

// K[c] = round(factor * kappa[c] * 2^64) from the error-free product
// p + q = factor * kappa (q = fma(factor, kappa, -p)); padding columns get 0.
// bad[0] is set when the fixed-point form cannot represent the problem:
// negative or non-finite kappa, factor*kappa >= 1/4, or a centre weight
// 1 - sum_f factor (kappa_a + kappa_b) below 2^-40.
__global__ void k_kq_setup(u64 *__restrict__ K, int *__restrict__ bad,
                           const double *__restrict__ kap, int nx, int ny, int nz, int P,
                           size_t S, double factor) {
  size_t total = S * nz;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < total;
       c += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(c % P);
    int j = (int)((c / P) % ny);
    int k = (int)(c / S);
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

int choose_kchunk(const heat_geom &g) {
  long tiles = (long)((g.nx - 2 + TX - 1) / TX) * ((g.ny - 2 + TY - 1) / TY);
  long want = 152L * 16;
  long chunks = (want + tiles - 1) / tiles;
  int interior = g.nz - 2;
  int kchunk = (int)((interior + chunks - 1) / chunks);
  if (kchunk < 8) kchunk = 8;
  if (kchunk > interior) kchunk = interior;
  return kchunk;
}

}  // namespace

cudaError_t launch_kq_setup(unsigned long long *K, int *bad, const double *kappa,
                            const heat_geom &g, double factor, cudaStream_t st) {
  k_kq_setup<<<152 * 8, 256, 0, st>>>(K, bad, kappa, g.nx, g.ny, g.nz, g.pitch, g.plane, factor);
  return cudaGetLastError();
}

cudaError_t launch_fast_mix(double *u_new, const double *u_old, const double *rhs,
                            const unsigned long long *K, const double *c0,
                            double *const cf[3], const heat_geom &g, int hw_rows,
                            cudaStream_t st) {
  int kc = choose_kchunk(g);
  dim3 gr((g.nx - 2 + TX - 1) / TX, (g.ny - 2 + TY - 1) / TY, (g.nz - 2 + kc - 1) / kc);
  dim3 b(TX, TY);
  if (hw_rows < 0) hw_rows = 0;
  if (hw_rows > TY) hw_rows = TY;
  if (rhs)
    k_fast_mix<true><<<gr, b, 0, st>>>(u_new, u_old, rhs, K, c0, cf[0], cf[1], cf[2], g.nx, g.ny,
                                       g.nz, g.pitch, g.plane, kc, hw_rows);
  else
    k_fast_mix<false><<<gr, b, 0, st>>>(u_new, u_old, rhs, K, c0, cf[0], cf[1], cf[2], g.nx,
                                        g.ny, g.nz, g.pitch, g.plane, kc, hw_rows);
  return cudaGetLastError();
}

}  // namespace heat
