// Bit-exact FP64 kernels: the reference's operation order with every
// operation rounded separately (no fused multiply-add).  This translation unit
// is compiled with --fmad=false, and the arithmetic is written with the
// explicit round-to-nearest intrinsics (__dadd_rn, __dsub_rn, __dmul_rn),
// which the compiler never contracts, so the result does not depend on the
// contraction flag either way.
//
// Reference expression (OpenMP_Single_Source/heat3D_variable_coeff.c:174-181,
// 1-cuda.cu:103-111):
//   u_new = (u + rhs) + factor * S,
//   S = ((((A - B) + C) - D) + E) - F,
//   A = (kE+kC)(uE-uC)  B = (kC+kW)(uC-uW)  C = (kN+kC)(uN-uC)
//   D = (kC+kS)(uC-uS)  E = (kU+kC)(uU-uC)  F = (kC+kD)(uC-uD)
// A face flux is the same rounded value seen from both cells that share the
// face (IEEE addition is commutative), so the z-march below carries E of
// plane k as F of plane k+1 and stays bit-identical.

#include <cstdlib>

#include "heat_internal.h"
#include "heat_walk.cuh"

namespace heat {
namespace {

using walk::combine;
using walk::flux;

// One thread per point, the reference CUDA kernel's shape (block 8x8x8,
// 1-cuda.cu:85-131), arbitrary row pitch.
template <bool RHS>
__global__ void k_naive(double *__restrict__ un, const double *__restrict__ u,
                        const double *__restrict__ rhs, const double *__restrict__ kap,
                        int nx, int ny, int nz, int P, size_t S, double factor) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  int k = blockIdx.z * blockDim.z + threadIdx.z;
  if (k < 1 || k >= nz - 1 || j < 1 || j >= ny - 1 || i < 1 || i >= nx - 1) return;
  size_t c = (size_t)k * S + (size_t)j * P + i;
  double uc = u[c], kc = kap[c];
  double A = flux(__dadd_rn(kap[c + 1], kc), u[c + 1], uc);
  double B = flux(__dadd_rn(kc, kap[c - 1]), uc, u[c - 1]);
  double C = flux(__dadd_rn(kap[c + P], kc), u[c + P], uc);
  double D = flux(__dadd_rn(kc, kap[c - P]), uc, u[c - P]);
  double E = flux(__dadd_rn(kap[c + S], kc), u[c + S], uc);
  double F = flux(__dadd_rn(kc, kap[c - S]), uc, u[c - S]);
  un[c] = combine(RHS ? __dadd_rn(uc, rhs[c]) : uc, factor, A, B, C, D, E, F);
}

// z-marching kernels: a (32 x 8) thread tile of (i, j) columns walks a chunk
// of planes; the lower flux and the two z-neighbours stay in registers.
constexpr int TX = 32, TY = 8;

// z-marching kernel: a (32 x 8) thread tile of columns walks a chunk of
// planes; the lower flux and the z-neighbours stay in registers.  The west
// face flux comes from the neighbouring lane: B at column i is the value A of
// column i-1 (same operands, same order), so each point computes one x-flux
// instead of two.  A warp covers 31 output columns; its lane 0 walks the
// column west of them only to hand over its A.  Lanes past the grid's
// interior walk the last interior column (in-bounds loads) and store nothing.
// RAW forms the face kappa sums from kappa as the reference does each step
// (the drop-in heat_update); otherwise they are read precomputed, once per
// context: kx[c] = kappa[c] + kappa[c+1], ky[c] = kappa[c] + kappa[c+P],
// kz[c] = kappa[c] + kappa[c+S] -- the same values, 3 additions per point fewer.
constexpr int SX = 31;

template <bool RHS, bool RAW>
__global__ void __launch_bounds__(TX *TY)
    k_exact_shfl(double *__restrict__ un, const double *__restrict__ u,
                 const double *__restrict__ rhs, const double *__restrict__ kap,
                 const double *__restrict__ kx, const double *__restrict__ ky,
                 const double *__restrict__ kz, int nx, int ny, int nz, int P, size_t S,
                 double factor, int kchunk) {
  const int lane = threadIdx.x;
  const int i = blockIdx.x * SX + lane;  // lane 0: the column west of the outputs
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (j >= ny - 1 || kb >= ke) return;  // uniform across the warp
  const bool store = lane >= 1 && i <= nx - 2;
  const int ic = min(i, nx - 2);
  size_t c = (size_t)kb * S + (size_t)j * P + ic;
  double uc = u[c];
  double kc = RAW ? kap[c] : 0.0;
  double F = RAW ? flux(__dadd_rn(kc, kap[c - S]), uc, u[c - S]) : flux(kz[c - S], uc, u[c - S]);
  for (int k = kb; k < ke; ++k, c += S) {
    const double uu = u[c + S];
    const double ku = RAW ? kap[c + S] : 0.0;
    const double A = RAW ? flux(__dadd_rn(kap[c + 1], kc), u[c + 1], uc)
                         : flux(kx[c], u[c + 1], uc);
    const double B = __shfl_up_sync(0xffffffffu, A, 1);
    const double C = RAW ? flux(__dadd_rn(kap[c + P], kc), u[c + P], uc)
                         : flux(ky[c], u[c + P], uc);
    const double D = RAW ? flux(__dadd_rn(kc, kap[c - P]), uc, u[c - P])
                         : flux(ky[c - P], uc, u[c - P]);
    const double E = RAW ? flux(__dadd_rn(ku, kc), uu, uc) : flux(kz[c], uu, uc);
    if (store) un[c] = combine(RHS ? __dadd_rn(uc, rhs[c]) : uc, factor, A, B, C, D, E, F);
    F = E;
    uc = uu;
    kc = ku;
  }
}

template <bool RHS, bool RAW>
void launch_shfl(double *u_new, const double *u_old, const double *rhs, const double *kappa,
                 double *const ks[3], const heat_geom &g, double factor, cudaStream_t st) {
  const int kc = plane_chunk(g, SX, TY);
  dim3 gr((g.nx - 2 + SX - 1) / SX, (g.ny - 2 + TY - 1) / TY, (g.nz - 2 + kc - 1) / kc);
  k_exact_shfl<RHS, RAW><<<gr, dim3(TX, TY), 0, st>>>(
      u_new, u_old, rhs, kappa, ks ? ks[0] : nullptr, ks ? ks[1] : nullptr,
      ks ? ks[2] : nullptr, g.nx, g.ny, g.nz, g.pitch, g.plane, factor, kc);
}

__global__ void k_face_sums(double *__restrict__ kx, double *__restrict__ ky,
                            double *__restrict__ kz, const double *__restrict__ kap,
                            int nx, int ny, int nz, int P, size_t S) {
  // One row (j, k) per block iteration, its points across the threads: no
  // per-point index division.
  const long rows = (long)ny * nz;
  for (long r = blockIdx.x; r < rows; r += gridDim.x)
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    const int j = (int)(r % ny), k = (int)(r / ny);
    const size_t c = (size_t)k * S + (size_t)j * P + i;
    kx[c] = (i + 1 < nx) ? __dadd_rn(kap[c], kap[c + 1]) : 0.0;
    ky[c] = (j + 1 < ny && i < nx) ? __dadd_rn(kap[c], kap[c + P]) : 0.0;
    kz[c] = (k + 1 < nz && i < nx) ? __dadd_rn(kap[c], kap[c + S]) : 0.0;
  }
}


}  // namespace

cudaError_t launch_naive(double *u_new, const double *u_old, const double *rhs,
                         const double *kappa, const heat_geom &g, double factor,
                         cudaStream_t st) {
  dim3 b(8, 8, 8), gr((g.nx + 7) / 8, (g.ny + 7) / 8, (g.nz + 7) / 8);
  if (rhs)
    k_naive<true><<<gr, b, 0, st>>>(u_new, u_old, rhs, kappa, g.nx, g.ny, g.nz, g.pitch,
                                    g.plane, factor);
  else
    k_naive<false><<<gr, b, 0, st>>>(u_new, u_old, rhs, kappa, g.nx, g.ny, g.nz, g.pitch,
                                     g.plane, factor);
  return cudaGetLastError();
}

cudaError_t launch_exact_raw(double *u_new, const double *u_old, const double *rhs,
                             const double *kappa, const heat_geom &g, double factor,
                             cudaStream_t st) {
  // the lane-shuffled walk: 23.9 GLUP/s at 512^3 against 21.9 for k_exact_raw
  if (rhs)
    launch_shfl<true, true>(u_new, u_old, rhs, kappa, nullptr, g, factor, st);
  else
    launch_shfl<false, true>(u_new, u_old, rhs, kappa, nullptr, g, factor, st);
  return cudaGetLastError();
}

cudaError_t launch_exact_faces(double *u_new, const double *u_old, const double *rhs,
                               double *const ks[3], const heat_geom &g, double factor,
                               cudaStream_t st) {
  // the lane-shuffled walk: 31.9 GLUP/s at 512^3 against 29.7 for k_exact_faces
  if (rhs)
    launch_shfl<true, false>(u_new, u_old, rhs, nullptr, ks, g, factor, st);
  else
    launch_shfl<false, false>(u_new, u_old, rhs, nullptr, ks, g, factor, st);
  return cudaGetLastError();
}

cudaError_t launch_face_sums(double *const ks[3], const double *kappa, const heat_geom &g,
                             cudaStream_t st) {
  k_face_sums<<<152 * 8, 256, 0, st>>>(ks[0], ks[1], ks[2], kappa, g.nx, g.ny, g.nz,
                                       g.pitch, g.plane);
  return cudaGetLastError();
}

}  // namespace heat
