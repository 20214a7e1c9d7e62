// heat_norm_noalloc(): L2 norm and checksum of a caller-owned FP64 field that
// allocates nothing on the device or the host.
//
// Who needs it: callers that must not call cudaMalloc/cudaFree while they run.
// A serving loop that has handed all of its HBM to an admission budget (or a
// framework whose caching allocator owns the device memory) has nothing left
// for a stray allocation, and a monitoring hook that checks a field between
// time steps cannot afford the device-wide synchronisation that cudaFree (and
// often cudaMalloc) imposes on every other stream.  heat_norm() needs a context,
// which owns a scratch buffer allocated at heat_init(); this variant keeps its
// scratch in a fixed static device array instead.
//
// Scratch: g_norm_scratch holds one (sum, sum of squares) pair per plane plus
// the final pair -- 2 * HEAT_NORM_NOALLOC_MAX_NZ + 2 doubles (256 KiB), held by
// every GPU that loads the library until the process exits.  Fields with more
// than HEAT_NORM_NOALLOC_MAX_NZ planes are rejected with HEAT_EINVAL.
//
// Host code cannot use g_norm_scratch's name as a device address (on the host
// it names a shadow variable).  The first call on each device, with that
// device current, looks the address up with cudaGetSymbolAddress and caches it
// per device; make that first call on a device before any stream capture.
// Every call on a device shares the array and it keeps the last call's
// contents; each pass writes every slot it later reads, so nothing has to be
// cleared.  Calls that overlap on the same GPU race on the array: issue them
// from one stream, or order them on the host.

#include <cmath>
#include <mutex>

#include "heat_internal.h"

namespace {

constexpr int kMaxNz = HEAT_NORM_NOALLOC_MAX_NZ;
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_norm_scratch[2 * kMaxNz + 2];

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sums of (a, b), valid in thread 0.
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

// One block per plane: scratch[2k], scratch[2k+1] = sum u, sum u^2 of plane k.
__global__ void __launch_bounds__(kThreads)
    k_plane_sums(const double *__restrict__ u, int ny, int nx, double *__restrict__ scratch) {
  const size_t plane = (size_t)ny * nx;
  const double *p = u + (size_t)blockIdx.x * plane;
  double s = 0.0, q = 0.0;
  for (size_t t = threadIdx.x; t < plane; t += kThreads) {
    const double x = p[t];
    s += x;
    q = fma(x, x, q);
  }
  block_sum2(s, q);
  if (threadIdx.x == 0) {
    scratch[2 * blockIdx.x] = s;
    scratch[2 * blockIdx.x + 1] = q;
  }
}

// Fold the nz plane pairs in index order into scratch[2*kMaxNz], [2*kMaxNz+1].
__global__ void __launch_bounds__(kThreads) k_fold(double *__restrict__ scratch, int nz) {
  double s = 0.0, q = 0.0;
  for (int k = threadIdx.x; k < nz; k += kThreads) {
    s += scratch[2 * k];
    q += scratch[2 * k + 1];
  }
  block_sum2(s, q);
  if (threadIdx.x == 0) {
    scratch[2 * kMaxNz] = s;
    scratch[2 * kMaxNz + 1] = q;
  }
}

struct DeviceScratch {
  std::once_flag once;
  double *ptr = nullptr;
  cudaError_t err = cudaSuccess;
};
DeviceScratch g_scratch[kMaxDevices];

}  // namespace

extern "C" int heat_norm_noalloc(const double *u, int nz, int ny, int nx, double *l2,
                                 double *checksum, void *stream) {
  if (!u || nz < 1 || ny < 1 || nx < 1) return HEAT_EINVAL;
  if (nz > kMaxNz) return HEAT_EINVAL;  // beyond the static scratch
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return HEAT_ENODEV;
  }
  DeviceScratch &ds = g_scratch[dev];
  std::call_once(ds.once, [&ds] {
    ds.err = cudaGetSymbolAddress(reinterpret_cast<void **>(&ds.ptr), g_norm_scratch);
  });
  if (ds.err != cudaSuccess || !ds.ptr) return HEAT_ECUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_plane_sums<<<nz, kThreads, 0, st>>>(u, ny, nx, ds.ptr);
  k_fold<<<1, kThreads, 0, st>>>(ds.ptr, nz);
  if (cudaGetLastError() != cudaSuccess) return HEAT_ECUDA;
  double r[2];
  if (cudaMemcpyAsync(r, ds.ptr + 2 * kMaxNz, sizeof r, cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  if (checksum) *checksum = r[0];
  if (l2) *l2 = std::sqrt(r[1]);
  return HEAT_OK;
}
