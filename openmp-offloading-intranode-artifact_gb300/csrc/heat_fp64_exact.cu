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

// z-marching kernels: a (32 x 8) thread tile of (i, j) columns walks a chunk
// of planes; the lower flux and the two z-neighbours stay in registers.
constexpr int TX = 32, TY = 8;

template <bool RHS>
__global__ void __launch_bounds__(TX *TY)
    k_exact_raw(double *__restrict__ un, const double *__restrict__ u,
                const double *__restrict__ rhs, const double *__restrict__ kap, int nx,
                int ny, int nz, int P, size_t S, double factor, int kchunk) {
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (i >= nx - 1 || j >= ny - 1 || kb >= ke) return;
  size_t c = (size_t)kb * S + (size_t)j * P + i;
  double ud = u[c - S], uc = u[c];
  double kd = kap[c - S], kc = kap[c];
  double F = flux(__dadd_rn(kc, kd), uc, ud);
  for (int k = kb; k < ke; ++k, c += S) {
    double uu = u[c + S], ku = kap[c + S];
    double A = flux(__dadd_rn(kap[c + 1], kc), u[c + 1], uc);
    double B = flux(__dadd_rn(kc, kap[c - 1]), uc, u[c - 1]);
    double C = flux(__dadd_rn(kap[c + P], kc), u[c + P], uc);
    double D = flux(__dadd_rn(kc, kap[c - P]), uc, u[c - P]);
    double E = flux(__dadd_rn(ku, kc), uu, uc);
    un[c] = combine(RHS ? __dadd_rn(uc, rhs[c]) : uc, factor, A, B, C, D, E, F);
    F = E;
    uc = uu;
    kc = ku;
  }
}

// Same walk with the face kappa sums precomputed once per context:
// kx[c] = kappa[c] + kappa[c+1], ky[c] = kappa[c] + kappa[c+P],
// kz[c] = kappa[c] + kappa[c+S].  Each is the value the reference forms
// anew every step, so the result is unchanged and 3 additions per point go.
template <bool RHS>
__global__ void __launch_bounds__(TX *TY)
    k_exact_faces(double *__restrict__ un, const double *__restrict__ u,
                  const double *__restrict__ rhs, const double *__restrict__ kx,
                  const double *__restrict__ ky, const double *__restrict__ kz, int nx,
                  int ny, int nz, int P, size_t S, double factor, int kchunk) {
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (i >= nx - 1 || j >= ny - 1 || kb >= ke) return;
  const size_t c = (size_t)kb * S + (size_t)j * P + i;
  walk::walk_exact_faces<RHS>(un, u, rhs, kx, ky, kz, P, S, c, kb, ke, factor);
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


dim3 zgrid(const heat_geom &g, int kchunk) {
  return dim3((g.nx - 2 + TX - 1) / TX, (g.ny - 2 + TY - 1) / TY,
              (g.nz - 2 + kchunk - 1) / kchunk);
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
  int kc = plane_chunk(g, TX, TY);
  dim3 gr = zgrid(g, kc), b(TX, TY);
  if (rhs)
    k_exact_raw<true><<<gr, b, 0, st>>>(u_new, u_old, rhs, kappa, g.nx, g.ny, g.nz, g.pitch,
                                        g.plane, factor, kc);
  else
    k_exact_raw<false><<<gr, b, 0, st>>>(u_new, u_old, rhs, kappa, g.nx, g.ny, g.nz,
                                         g.pitch, g.plane, factor, kc);
  return cudaGetLastError();
}

cudaError_t launch_exact_faces(double *u_new, const double *u_old, const double *rhs,
                               double *const ks[3], const heat_geom &g, double factor,
                               cudaStream_t st) {
  int kc = plane_chunk(g, TX, TY);
  dim3 gr = zgrid(g, kc), b(TX, TY);
  if (rhs)
    k_exact_faces<true><<<gr, b, 0, st>>>(u_new, u_old, rhs, ks[0], ks[1], ks[2], g.nx, g.ny,
                                          g.nz, g.pitch, g.plane, factor, kc);
  else
    k_exact_faces<false><<<gr, b, 0, st>>>(u_new, u_old, rhs, ks[0], ks[1], ks[2], g.nx,
                                           g.ny, g.nz, g.pitch, g.plane, factor, kc);
  return cudaGetLastError();
}

cudaError_t launch_face_sums(double *const ks[3], const double *kappa, const heat_geom &g,
                             cudaStream_t st) {
  k_face_sums<<<152 * 8, 256, 0, st>>>(ks[0], ks[1], ks[2], kappa, g.nx, g.ny, g.nz,
                                       g.pitch, g.plane);
  return cudaGetLastError();
}

}  // namespace heat
