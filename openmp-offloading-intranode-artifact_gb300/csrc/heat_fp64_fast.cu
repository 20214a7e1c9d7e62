// Default FP64 form: the same update rewritten as a weighted sum of the seven
// stencil values,
//   u_new = rhs + c0*uC + cE*uE + cW*uW + cN*uN + cS*uS + cU*uU + cD*uD,
// with the face weights c_f = factor*(kappa_a + kappa_b) and the centre
// weight c0 = 1 - sum_f c_f precomputed once per context in FP64.  Algebraically
// identical to the reference's
//   u + rhs + factor * sum_f +-(kappa_a+kappa_b)(u_b - u_a)
// (OpenMP_Single_Source/heat3D_variable_coeff.c:174-181); the rounding
// differs, and the result is held to <= 1e-12 relative error against the
// reference instead of bit identity.  7 FP64 operations per point instead of
// 26 as written (17 with shared face fluxes).

#include "heat_internal.h"
#include "heat_walk.cuh"

namespace heat {
namespace {

constexpr int TX = 32, TY = 8;

__global__ void k_fast_coeffs(double *__restrict__ c0, double *__restrict__ cx,
                              double *__restrict__ cy, double *__restrict__ cz,
                              const double *__restrict__ kap, int nx, int ny, int nz, int P,
                              size_t S, double factor) {
  // One row (j, k) per block iteration, its points across the threads: no
  // per-point index division.
  const long rows = (long)ny * nz;
  for (long r = blockIdx.x; r < rows; r += gridDim.x)
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    const int j = (int)(r % ny), k = (int)(r / ny);
    const size_t c = (size_t)k * S + (size_t)j * P + i;
    bool in = i < nx;
    double kc = in ? kap[c] : 0.0;
    cx[c] = (i + 1 < nx) ? fw(factor, kc, kap[c + 1]) : 0.0;
    cy[c] = (in && j + 1 < ny) ? fw(factor, kc, kap[c + P]) : 0.0;
    cz[c] = (in && k + 1 < nz) ? fw(factor, kc, kap[c + S]) : 0.0;
    double w = 0.0;
    if (in && i > 0 && j > 0 && k > 0 && i < nx - 1 && j < ny - 1 && k < nz - 1)
      w = centre(fw(factor, kc, kap[c + 1]), fw(factor, kap[c - 1], kc), fw(factor, kc, kap[c + P]),
                 fw(factor, kap[c - P], kc), fw(factor, kc, kap[c + S]), fw(factor, kap[c - S], kc));
    c0[c] = w;
  }
}

template <bool RHS>
__global__ void __launch_bounds__(TX *TY)
    k_fast_hw(double *__restrict__ un, const double *__restrict__ u,
              const double *__restrict__ rhs, const double *__restrict__ c0,
              const double *__restrict__ cx, const double *__restrict__ cy,
              const double *__restrict__ cz, int nx, int ny, int nz, int P, size_t S,
              int kchunk) {
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (i >= nx - 1 || j >= ny - 1 || kb >= ke) return;
  const size_t c = (size_t)kb * S + (size_t)j * P + i;
  walk::walk_hw<RHS>(un, u, rhs, c0, cx, cy, cz, P, S, c, kb, ke);
}


}  // namespace

cudaError_t launch_fast_coeffs(double *c0, double *const cf[3], const double *kappa,
                               const heat_geom &g, double factor, cudaStream_t st) {
  k_fast_coeffs<<<152 * 8, 256, 0, st>>>(c0, cf[0], cf[1], cf[2], kappa, g.nx, g.ny, g.nz,
                                         g.pitch, g.plane, factor);
  return cudaGetLastError();
}

cudaError_t launch_fast(double *u_new, const double *u_old, const double *rhs,
                        const double *c0, double *const cf[3], const heat_geom &g,
                        cudaStream_t st) {
  static const long res_rhs = resident_blocks((const void *)k_fast_hw<true>, TX * TY, 0);
  static const long res_plain = resident_blocks((const void *)k_fast_hw<false>, TX * TY, 0);
  const int kc = wave_chunk(g, TX, TY, rhs ? res_rhs : res_plain);
  dim3 gr((g.nx - 2 + TX - 1) / TX, (g.ny - 2 + TY - 1) / TY, (g.nz - 2 + kc - 1) / kc);
  dim3 b(TX, TY);
  if (rhs)
    k_fast_hw<true><<<gr, b, 0, st>>>(u_new, u_old, rhs, c0, cf[0], cf[1], cf[2], g.nx, g.ny,
                                      g.nz, g.pitch, g.plane, kc);
  else
    k_fast_hw<false><<<gr, b, 0, st>>>(u_new, u_old, rhs, c0, cf[0], cf[1], cf[2], g.nx,
                                       g.ny, g.nz, g.pitch, g.plane, kc);
  return cudaGetLastError();
}

}  // namespace heat
