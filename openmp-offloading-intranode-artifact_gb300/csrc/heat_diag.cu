// FP64 pipe-rate probe and the bounded-wait check (include/heat_diag.h).

#include "heat_diag.h"
#include "heat_internal.h"
#include "heat_tma.cuh"

namespace {

__global__ void k_fp64_chains(double *out, double a, double b, int iters) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int it = 0; it < iters; ++it) {
    x0 = fma(x0, b, a); x1 = fma(x1, b, a); x2 = fma(x2, b, a); x3 = fma(x3, b, a);
    x4 = fma(x4, b, a); x5 = fma(x5, b, a); x6 = fma(x6, b, a); x7 = fma(x7, b, a);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// Thread 0 initialises an mbarrier that nothing ever arrives at and waits
// for its first phase with the bounded wait the TMA kernels use, capped at
// `attempts` tries; timed_out[0] = 1 when the wait gave up.  No copy is in
// flight, so giving up leaves nothing behind.
__global__ void k_wait_unsignalled(unsigned attempts, int *timed_out) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    heat::tma::mbar_init(&bar);
    heat::tma::mbar_init_fence();
    timed_out[0] = heat::tma::mbar_wait(&bar, 0u, attempts) ? 0 : 1;
  }
}

}  // namespace

extern "C" int heat_diag_fp64_rate(double *gops_out) {
  if (!gops_out) return HEAT_EINVAL;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ENODEV;
  }
  const int blocks = sms * 8, threads = 256, iters = 1024;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = HEAT_OK;
  float ms = 0.f;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ENOMEM;
  }
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = HEAT_ECUDA;
    goto done;
  }
  k_fp64_chains<<<blocks, threads>>>(out, 1e-9, 1.0000001, iters);  // warm-up
  cudaEventRecord(e0);
  k_fp64_chains<<<blocks, threads>>>(out, 1e-9, 1.0000001, iters);
  cudaEventRecord(e1);
  if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess ||
      ms <= 0.f) {
    rc = HEAT_ECUDA;
    goto done;
  }
  *gops_out = (double)blocks * threads * iters * 8 / (ms * 1e-3) / 1e9;
done:
  cudaGetLastError();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return rc;
}

extern "C" int heat_diag_wait_timeout(unsigned attempts, int *timed_out) {
  // at most the TMA kernels' own limit, so the check cannot hold the GPU longer
  if (!timed_out || attempts == 0 || attempts > heat::tma::kWaitLimit) return HEAT_EINVAL;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ENODEV;
  }
  int *d = nullptr, h = -1;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ENOMEM;
  }
  int rc = HEAT_ECUDA;
  if (cudaMemcpy(d, &h, sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess) {
    k_wait_unsignalled<<<1, 32>>>(attempts, d);
    if (cudaGetLastError() == cudaSuccess &&
        cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess)
      rc = h == 1 ? HEAT_ETIMEOUT : h == 0 ? HEAT_OK : HEAT_ECUDA;
  }
  cudaGetLastError();
  cudaFree(d);
  *timed_out = h;
  return rc;
}
