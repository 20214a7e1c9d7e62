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
// Scratch: g_norm_scratch holds one (sum, sum of squares) pair per partial
// sum plus the final pair -- 2 * kSlots + 2 doubles (256 KiB), held by every
// GPU that loads the library until the process exits.  Each plane is cut into
// C chunks (as many as keep about 8 blocks per SM busy, within kSlots / nz),
// one block per (chunk, plane), so a shallow, wide field uses the whole GPU.
// Fields with more than HEAT_NORM_NOALLOC_MAX_NZ (= kSlots) planes are
// rejected with HEAT_EINVAL.
//
// Host code cannot use g_norm_scratch's name as a device address (on the host
// it names a shadow variable).  The first call on each device, with that
// device current, looks the address up with cudaGetSymbolAddress and keeps it
// for that device once the lookup succeeded (a failed lookup is reported and
// tried again on the next call); make that first call on a device before any
// stream capture.  A cudaDeviceReset() of the device releases the array and
// the kept address with it: do not call this entry point on a device after
// resetting it in the same process.  Every call on a device shares the array
// and it keeps the last call's contents; each pass writes every slot it later
// reads, so nothing has to be cleared.  Calls that overlap on the same GPU
// race on the array: issue them from one stream, or order them on the host.

#include <algorithm>
#include <cmath>
#include <mutex>

#include "heat_internal.h"

namespace {

constexpr int kSlots = HEAT_NORM_NOALLOC_MAX_NZ;  // partial-sum pairs
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;
constexpr int kWantBlocks = 152 * 8;  // about 8 blocks per SM of GB300

static __device__ __align__(256) double g_norm_scratch[2 * kSlots + 2];

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

// Block (x, k) sums points [x * chunk, min((x + 1) * chunk, plane)) of plane k
// into slot k * gridDim.x + x: scratch[2 slot] = sum u, [2 slot + 1] = sum u^2.
__global__ void __launch_bounds__(kThreads)
    k_chunk_sums(const double *__restrict__ u, size_t plane, size_t chunk,
                 double *__restrict__ scratch) {
  const double *p = u + (size_t)blockIdx.y * plane;
  const size_t b = (size_t)blockIdx.x * chunk;
  const size_t e = b + chunk < plane ? b + chunk : plane;
  double s = 0.0, q = 0.0;
  for (size_t t = b + threadIdx.x; t < e; t += kThreads) {
    const double x = p[t];
    s += x;
    q = fma(x, x, q);
  }
  block_sum2(s, q);
  if (threadIdx.x == 0) {
    const size_t slot = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
    scratch[2 * slot] = s;
    scratch[2 * slot + 1] = q;
  }
}

// Fold the first nslots pairs (each thread its strided share in index order,
// then a fixed tree) into scratch[2 * kSlots], [2 * kSlots + 1].
__global__ void __launch_bounds__(kThreads) k_fold(double *__restrict__ scratch, int nslots) {
  double s = 0.0, q = 0.0;
  for (int k = threadIdx.x; k < nslots; k += kThreads) {
    s += scratch[2 * k];
    q += scratch[2 * k + 1];
  }
  block_sum2(s, q);
  if (threadIdx.x == 0) {
    scratch[2 * kSlots] = s;
    scratch[2 * kSlots + 1] = q;
  }
}

// The scratch array's device address on each device, kept once looked up.
struct DeviceScratch {
  std::mutex mu;
  double *ptr = nullptr;
};
DeviceScratch g_scratch[kMaxDevices];

int scratch_address(int dev, double **out) {
  DeviceScratch &ds = g_scratch[dev];
  std::lock_guard<std::mutex> lk(ds.mu);
  if (!ds.ptr) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_norm_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return heat::cuda_fail(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                             "heat_norm_noalloc: cudaGetSymbolAddress of its scratch");
    }
    ds.ptr = static_cast<double *>(p);
  }
  *out = ds.ptr;
  return HEAT_OK;
}

}  // namespace

extern "C" int heat_norm_noalloc(const double *u, int nz, int ny, int nx, double *l2,
                                 double *checksum, void *stream) {
  if (!u || nz < 1 || ny < 1 || nx < 1) return HEAT_EINVAL;
  if (nz > kSlots) return HEAT_EINVAL;  // beyond the static scratch
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return HEAT_ENODEV;
  }
  double *scratch = nullptr;
  if (int rc = scratch_address(dev, &scratch)) return rc;
  const size_t plane = (size_t)ny * nx;
  // Chunks per plane: enough blocks to fill the GPU, within the slots, and no
  // more chunks than a plane has block-sized pieces.
  long chunks = (kWantBlocks + nz - 1) / nz;
  chunks = std::min<long>(chunks, kSlots / nz);
  chunks = std::min<long>(chunks, (long)((plane + kThreads - 1) / kThreads));
  chunks = std::max<long>(chunks, 1);
  const size_t chunk = (plane + chunks - 1) / chunks;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_chunk_sums<<<dim3((unsigned)chunks, (unsigned)nz), kThreads, 0, st>>>(u, plane, chunk, scratch);
  k_fold<<<1, kThreads, 0, st>>>(scratch, (int)(chunks * nz));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return heat::cuda_fail(e, "heat_norm_noalloc launch");
  double r[2];
  e = cudaMemcpyAsync(r, scratch + 2 * kSlots, sizeof r, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return heat::cuda_fail(e, "heat_norm_noalloc");
  }
  if (checksum) *checksum = r[0];
  if (l2) *l2 = std::sqrt(r[1]);
  return HEAT_OK;
}
