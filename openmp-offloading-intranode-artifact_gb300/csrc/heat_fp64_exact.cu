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

// z-marching kernel.  A (32 x 8) thread tile walks a chunk of planes; each
// thread owns one column i of RY adjacent rows, and the lower flux and the
// z-neighbours of each row stay in registers.  Two face fluxes are shared
// instead of recomputed (a face flux is the same rounded value seen from both
// cells that share the face):
//   - x: B at column i is A of column i-1 (same operands, same order), taken
//     from the neighbouring lane.  A warp covers 31 output columns; its lane 0
//     walks the column west of them only to hand over its A.  Lanes past the
//     grid's interior walk the last interior column (in-bounds loads) and
//     store nothing.
//   - y: C of row j is D of row j+1, so a thread computes RY+1 y-fluxes for
//     its RY outputs instead of 2 RY.  Row t of a thread (t = 0 .. RY+1) is
//     grid row j0-1+t; rows past the grid are clamped to the last row so every
//     load stays in bounds, and only interior rows store (an interior row reads
//     rows j-1, j, j+1 only, none of them clamped).
// RAW forms the face kappa sums from kappa as the reference does each step
// (the drop-in heat_update); otherwise they are read precomputed, once per
// context: kx[c] = kappa[c] + kappa[c+1], ky[c] = kappa[c] + kappa[c+P],
// kz[c] = kappa[c] + kappa[c+S] -- the same values, fewer additions per point.
// Three rows per thread measured best at 512^3 (GLUP/s, drop-in / context
// form): one row 24.0 / 31.9, two 26.4 / 34.6, three 26.7 / 35.1, four
// 26.3 / 34.5 (123 registers).
constexpr int TX = 32, TY = 8;
constexpr int SX = 31;
constexpr int RY = 3;

template <bool RHS, bool RAW>
__global__ void __launch_bounds__(TX *TY)
    k_exact_rows(double *__restrict__ un, const double *__restrict__ u,
                 const double *__restrict__ rhs, const double *__restrict__ kap,
                 const double *__restrict__ kx, const double *__restrict__ ky,
                 const double *__restrict__ kz, int nx, int ny, int nz, int P, size_t S,
                 double factor, int kchunk) {
  const int lane = threadIdx.x;
  const int i = blockIdx.x * SX + lane;  // lane 0: the column west of the outputs
  const int j0 = 1 + (blockIdx.y * TY + threadIdx.y) * RY;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (j0 >= ny - 1 || kb >= ke) return;  // uniform across the warp
  const bool xs = lane >= 1 && i <= nx - 2;
  const int ic = min(i, nx - 2);
  size_t ro[RY + 2];
#pragma unroll
  for (int t = 0; t < RY + 2; ++t) ro[t] = (size_t)min(j0 - 1 + t, ny - 1) * P + ic;
  size_t pl = (size_t)kb * S;
  double uc[RY + 2], kc[RY + 2], F[RY];
#pragma unroll
  for (int t = 0; t < RY + 2; ++t) {
    uc[t] = u[pl + ro[t]];
    kc[t] = RAW ? kap[pl + ro[t]] : 0.0;
  }
#pragma unroll
  for (int r = 0; r < RY; ++r) {
    const size_t q = pl - S + ro[r + 1];
    F[r] = RAW ? flux(__dadd_rn(kc[r + 1], kap[q]), uc[r + 1], u[q])
               : flux(kz[q], uc[r + 1], u[q]);
  }
  for (int k = kb; k < ke; ++k, pl += S) {
    double uu[RY + 2], ku[RY + 2], G[RY + 1];
#pragma unroll
    for (int t = 0; t < RY + 2; ++t) {
      uu[t] = u[pl + S + ro[t]];
      ku[t] = RAW ? kap[pl + S + ro[t]] : 0.0;
    }
    // G[t]: the flux through the face between rows t and t+1
#pragma unroll
    for (int t = 0; t <= RY; ++t)
      G[t] = RAW ? flux(__dadd_rn(kc[t + 1], kc[t]), uc[t + 1], uc[t])
                 : flux(ky[pl + ro[t]], uc[t + 1], uc[t]);
#pragma unroll
    for (int r = 0; r < RY; ++r) {
      const int t = r + 1;
      const size_t q = pl + ro[t];
      const double A = RAW ? flux(__dadd_rn(kap[q + 1], kc[t]), u[q + 1], uc[t])
                           : flux(kx[q], u[q + 1], uc[t]);
      const double B = __shfl_up_sync(0xffffffffu, A, 1);
      const double E = RAW ? flux(__dadd_rn(ku[t], kc[t]), uu[t], uc[t]) : flux(kz[q], uu[t], uc[t]);
      if (xs && j0 + r <= ny - 2)
        un[q] = combine(RHS ? __dadd_rn(uc[t], rhs[q]) : uc[t], factor, A, B, G[t], G[t - 1], E,
                        F[r]);
      F[r] = E;
    }
#pragma unroll
    for (int t = 0; t < RY + 2; ++t) {
      uc[t] = uu[t];
      kc[t] = ku[t];
    }
  }
}

template <bool RHS, bool RAW>
void launch_rows(double *u_new, const double *u_old, const double *rhs, const double *kappa,
                 double *const ks[3], const heat_geom &g, double factor, cudaStream_t st) {
  static const long resident = resident_blocks((const void *)k_exact_rows<RHS, RAW>, TX * TY, 0);
  const int kc = wave_chunk(g, SX, TY * RY, resident);
  dim3 gr((g.nx - 2 + SX - 1) / SX, (g.ny - 2 + TY * RY - 1) / (TY * RY),
          (g.nz - 2 + kc - 1) / kc);
  k_exact_rows<RHS, RAW><<<gr, dim3(TX, TY), 0, st>>>(
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
  if (rhs)
    launch_rows<true, true>(u_new, u_old, rhs, kappa, nullptr, g, factor, st);
  else
    launch_rows<false, true>(u_new, u_old, rhs, kappa, nullptr, g, factor, st);
  return cudaGetLastError();
}

cudaError_t launch_exact_faces(double *u_new, const double *u_old, const double *rhs,
                               double *const ks[3], const heat_geom &g, double factor,
                               cudaStream_t st) {
  if (rhs)
    launch_rows<true, false>(u_new, u_old, rhs, nullptr, ks, g, factor, st);
  else
    launch_rows<false, false>(u_new, u_old, rhs, nullptr, ks, g, factor, st);
  return cudaGetLastError();
}

cudaError_t launch_face_sums(double *const ks[3], const double *kappa, const heat_geom &g,
                             cudaStream_t st) {
  k_face_sums<<<152 * 8, 256, 0, st>>>(ks[0], ks[1], ks[2], kappa, g.nx, g.ny, g.nz,
                                       g.pitch, g.plane);
  return cudaGetLastError();
}

}  // namespace heat
