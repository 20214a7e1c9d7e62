// FP32-compensated precision form (HEAT_FP32C).
//
// State per point: v (FP32) and a Kahan carry c (BF16); the represented value
// is u = v - c.  Face weights are averaged once in FP64 and rounded to FP32:
//   wx[p] = (float)(factor * (kappa[p] + kappa[p+1]))   (likewise wy, wz),
// which is the reference's factor*(kappa_a + kappa_b)
// (OpenMP_Single_Source/heat3D_variable_coeff.c:174-181) evaluated once.
// Each step forms the increment in FP32,
//   d = rhs + sum_f w_f (v_f - v_C),
// and adds it by compensated (Kahan) summation:
//   y = d - c;  t = v + y;  c' = (t - v) - y;  v' = t.
// The carry keeps the part of each addition that FP32 rounds away, to BF16's
// 8 significant bits, so the running sum keeps about 32 bits where plain
// FP32 accumulation would keep 24.  The Kahan operations use the explicit
// round-to-nearest intrinsics so no contraction or reassociation can remove
// them.  Bytes per update: v 4+4, carry 2+2, face weights 3x4.

#include "heat_internal.h"
#include "heat_walk.cuh"

namespace heat {
namespace {

constexpr int TX = 32, TY = 8;

using walk::bf2f;
using walk::f2bf;

template <bool RHS>
__global__ void __launch_bounds__(TX *TY)
    k_fp32c(float *__restrict__ vn, uint16_t *__restrict__ cn, const float *__restrict__ v,
            const uint16_t *__restrict__ cr, const float *__restrict__ wx,
            const float *__restrict__ wy, const float *__restrict__ wz,
            const float *__restrict__ rhs, int nx, int ny, int nz, int P, size_t S,
            int kchunk) {
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (i >= nx - 1 || j >= ny - 1 || kb >= ke) return;
  const size_t c = (size_t)kb * S + (size_t)j * P + i;
  walk::walk_fp32c<RHS>(vn, cn, v, cr, wx, wy, wz, rhs, P, S, c, kb, ke);
}

// Split an FP64 field into (v, c) with v = fl32(u), c = bf16(v - u); padding 0.
__global__ void k_split(float *__restrict__ v, uint16_t *__restrict__ cr,
                        const double *__restrict__ u, size_t total) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const double x = u[p];
    const float f = (float)x;
    v[p] = f;
    cr[p] = f2bf((float)((double)f - x));
  }
}

// u = v - c in FP64.
__global__ void k_widen(double *__restrict__ u, const float *__restrict__ v,
                        const uint16_t *__restrict__ cr, size_t total) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x)
    u[p] = (double)v[p] - (double)bf2f(cr[p]);
}

__global__ void k_f32_weights(float *__restrict__ wx, float *__restrict__ wy,
                              float *__restrict__ wz, const double *__restrict__ kap, int nx,
                              int ny, int nz, int P, size_t S, double factor) {
  // One row (j, k) per block iteration, its points across the threads: no
  // per-point index division.
  const long rows = (long)ny * nz;
  for (long r = blockIdx.x; r < rows; r += gridDim.x)
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    const int j = (int)(r % ny), k = (int)(r / ny);
    const size_t c = (size_t)k * S + (size_t)j * P + i;
    bool in = i < nx;
    double kc = in ? kap[c] : 0.0;
    wx[c] = (i + 1 < nx) ? (float)(factor * (kc + kap[c + 1])) : 0.0f;
    wy[c] = (in && j + 1 < ny) ? (float)(factor * (kc + kap[c + P])) : 0.0f;
    wz[c] = (in && k + 1 < nz) ? (float)(factor * (kc + kap[c + S])) : 0.0f;
  }
}

__global__ void k_to_f32(float *__restrict__ o, const double *__restrict__ a, size_t total) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x)
    o[p] = (float)a[p];
}


}  // namespace

cudaError_t launch_fp32c(float *v_new, uint16_t *c_new, const float *v, const uint16_t *cr,
                         float *const w[3], const float *rhs, const heat_geom &g,
                         cudaStream_t st) {
  static const long res_rhs = resident_blocks((const void *)k_fp32c<true>, TX * TY, 0);
  static const long res_plain = resident_blocks((const void *)k_fp32c<false>, TX * TY, 0);
  const int kc = wave_chunk(g, TX, TY, rhs ? res_rhs : res_plain);
  dim3 gr((g.nx - 2 + TX - 1) / TX, (g.ny - 2 + TY - 1) / TY, (g.nz - 2 + kc - 1) / kc);
  dim3 b(TX, TY);
  if (rhs)
    k_fp32c<true><<<gr, b, 0, st>>>(v_new, c_new, v, cr, w[0], w[1], w[2], rhs, g.nx, g.ny,
                                    g.nz, g.pitch, g.plane, kc);
  else
    k_fp32c<false><<<gr, b, 0, st>>>(v_new, c_new, v, cr, w[0], w[1], w[2], rhs, g.nx, g.ny,
                                     g.nz, g.pitch, g.plane, kc);
  return cudaGetLastError();
}

cudaError_t launch_split(float *v, uint16_t *cr, const double *u, size_t total, cudaStream_t st) {
  k_split<<<152 * 8, 256, 0, st>>>(v, cr, u, total);
  return cudaGetLastError();
}

cudaError_t launch_widen(double *u, const float *v, const uint16_t *cr, size_t total,
                         cudaStream_t st) {
  k_widen<<<152 * 8, 256, 0, st>>>(u, v, cr, total);
  return cudaGetLastError();
}

cudaError_t launch_f32_weights(float *const w[3], const double *kappa, const heat_geom &g,
                               double factor, cudaStream_t st) {
  k_f32_weights<<<152 * 8, 256, 0, st>>>(w[0], w[1], w[2], kappa, g.nx, g.ny, g.nz, g.pitch,
                                         g.plane, factor);
  return cudaGetLastError();
}

cudaError_t launch_to_f32(float *o, const double *a, size_t total, cudaStream_t st) {
  k_to_f32<<<152 * 8, 256, 0, st>>>(o, a, total);
  return cudaGetLastError();
}

}  // namespace heat
