// FP64 L2 norm and checksum of a field: sum u^2 and sum u over all nz*ny*nx
// points (padding columns excluded).  Two passes with a fixed assignment of
// rows to blocks and fixed shuffle trees, so the result is deterministic run
// to run:
//   pass 1: block b sums rows b, b+G, b+2G, ... (threads stride the row),
//           warp-shuffle then shared-memory tree -> partials[2b], [2b+1];
//   pass 2: one block folds the G partial pairs in index order -> partials[2G],
//           partials[2G+1].

#include "heat_internal.h"

namespace heat {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums of (a, b) over the block; valid in thread 0.
__device__ __forceinline__ void block_sum2(double &a, double &b) {
  __shared__ double sa[kThreads / 32], sb[kThreads / 32];
  a = warp_sum(a);
  b = warp_sum(b);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sa[w] = a; sb[w] = b; }
  __syncthreads();
  if (w == 0) {
    a = l < kThreads / 32 ? sa[l] : 0.0;
    b = l < kThreads / 32 ? sb[l] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
  }
}

__global__ void __launch_bounds__(kThreads)
    k_norm_pass1(const double *__restrict__ u, int nx, int rows, int P,
                 double *__restrict__ partials) {
  double s = 0.0, q = 0.0;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const double *row = u + (size_t)r * P;
    for (int i = threadIdx.x; i < nx; i += kThreads) {
      double x = row[i];
      s += x;
      q = fma(x, x, q);
    }
  }
  block_sum2(s, q);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = s;
    partials[2 * blockIdx.x + 1] = q;
  }
}

__global__ void __launch_bounds__(kThreads)
    k_norm_pass2(double *__restrict__ partials, int nblocks) {
  double s = 0.0, q = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += kThreads) {
    s += partials[2 * b];
    q += partials[2 * b + 1];
  }
  block_sum2(s, q);
  if (threadIdx.x == 0) {
    partials[2 * nblocks] = s;
    partials[2 * nblocks + 1] = q;
  }
}

__global__ void __launch_bounds__(kThreads)
    k_norm_pass1_f32c(const float *__restrict__ v, const uint16_t *__restrict__ cr, int nx,
                      int rows, int P, double *__restrict__ partials) {
  double s = 0.0, q = 0.0;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const size_t o = (size_t)r * P;
    for (int i = threadIdx.x; i < nx; i += kThreads) {
      double x = (double)v[o + i] - (double)__uint_as_float(((unsigned)cr[o + i]) << 16);
      s += x;
      q = fma(x, x, q);
    }
  }
  block_sum2(s, q);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = s;
    partials[2 * blockIdx.x + 1] = q;
  }
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void __launch_bounds__(kThreads)
    k_diff_pass1(const double *__restrict__ a, const double *__restrict__ b, int nx, int rows,
                 int P, double *__restrict__ partials) {
  double d2 = 0.0, b2 = 0.0, mx = 0.0;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const size_t o = (size_t)r * P;
    for (int i = threadIdx.x; i < nx; i += kThreads) {
      const double x = a[o + i], y = b[o + i], d = x - y;
      d2 = fma(d, d, d2);
      b2 = fma(y, y, b2);
      mx = fmax(mx, fabs(d));
    }
  }
  __shared__ double sm[kThreads / 32];
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) mx = warp_max(threadIdx.x < kThreads / 32 ? sm[threadIdx.x] : 0.0);
  __syncthreads();
  block_sum2(d2, b2);
  if (threadIdx.x == 0) {
    partials[3 * blockIdx.x] = d2;
    partials[3 * blockIdx.x + 1] = b2;
    partials[3 * blockIdx.x + 2] = mx;
  }
}

__global__ void __launch_bounds__(kThreads)
    k_diff_pass2(double *__restrict__ partials, int nblocks) {
  double d2 = 0.0, b2 = 0.0, mx = 0.0;
  for (int k = threadIdx.x; k < nblocks; k += kThreads) {
    d2 += partials[3 * k];
    b2 += partials[3 * k + 1];
    mx = fmax(mx, partials[3 * k + 2]);
  }
  __shared__ double sm[kThreads / 32];
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) mx = warp_max(threadIdx.x < kThreads / 32 ? sm[threadIdx.x] : 0.0);
  __syncthreads();
  block_sum2(d2, b2);
  if (threadIdx.x == 0) {
    partials[3 * nblocks] = d2;
    partials[3 * nblocks + 1] = b2;
    partials[3 * nblocks + 2] = mx;
  }
}

}  // namespace

cudaError_t launch_norm_f32c(const float *v, const uint16_t *cr, const heat_geom &g,
                             double *partials, int nblocks, cudaStream_t st) {
  k_norm_pass1_f32c<<<nblocks, kThreads, 0, st>>>(v, cr, g.nx, g.ny * g.nz, g.pitch, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_norm_pass2<<<1, kThreads, 0, st>>>(partials, nblocks);
  return cudaGetLastError();
}

cudaError_t launch_diff_f64(const double *a, const double *b, const heat_geom &g,
                            double *partials, int nblocks, cudaStream_t st) {
  k_diff_pass1<<<nblocks, kThreads, 0, st>>>(a, b, g.nx, g.ny * g.nz, g.pitch, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_diff_pass2<<<1, kThreads, 0, st>>>(partials, nblocks);
  return cudaGetLastError();
}

cudaError_t launch_norm_f64(const double *u, const heat_geom &g, double *partials,
                            int nblocks, cudaStream_t st) {
  k_norm_pass1<<<nblocks, kThreads, 0, st>>>(u, g.nx, g.ny * g.nz, g.pitch, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_norm_pass2<<<1, kThreads, 0, st>>>(partials, nblocks);
  return cudaGetLastError();
}

}  // namespace heat
