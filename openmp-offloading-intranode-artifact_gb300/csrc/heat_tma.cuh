// TMA plane-tile loads and mbarrier waits for kernels that stage plane tiles
// in shared memory (heat_fp32c_tma.cu; the bounded wait is also checked by
// heat_diag_wait_timeout in heat_diag.cu).
//
// A block's thread 0 issues cp.async.bulk.tensor 3-D box loads of plane tiles
// into a shared-memory ring; each ring slot completes on its own mbarrier
// (transaction-count based).  Waits are bounded: mbar_wait gives up after a
// fixed number of try_wait attempts and the caller turns that into an error
// status instead of hanging.

#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>

#include "heat_internal.h"

namespace heat {
namespace tma {
namespace {

constexpr unsigned kSuspendNs = 2000;      // try_wait suspend-time hint
using heat::kWaitLimit;  // bounded wait: attempts before giving up (heat_internal.h)

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(b)) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect(unsigned long long *b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}

// try_wait with a suspend-time hint: the waiting thread sleeps in the
// instruction (up to ~the hint) instead of spinning and taking issue slots
// from the warps that compute.
__device__ __forceinline__ bool mbar_try(unsigned long long *b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity: false when `limit`
// attempts passed without it completing.
__device__ __forceinline__ bool mbar_wait(unsigned long long *b, unsigned parity,
                                         unsigned limit = kWaitLimit) {
  for (unsigned it = 0; it < limit; ++it)
    if (mbar_try(b, parity)) return true;
  return false;
}

// Orders this thread's earlier generic-proxy accesses of shared memory before
// the async-proxy (TMA) writes that follow.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 3-D box load of `map` at element coordinates (x, y, z) into dst; the box's
// x origin times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void load3(void *dst, const CUtensorMap *map, int x, int y, int z,
                                      unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
inline EncodeTiledFn encoder() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    // the entry point as the CUDA 12.0 driver API defines it
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (EncodeTiledFn) nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// Tensor map of a field laid out as geometry g (nx x ny x nz points, rows of
// g.pitch elements, planes of g.plane elements) with a (box_x x box_y x 1)
// box; out-of-range elements of a box read as zero.
inline bool encode_field(CUtensorMap *m, const void *base, CUtensorMapDataType type, size_t es,
                         const heat_geom &g, unsigned box_x, unsigned box_y) {
  EncodeTiledFn fn = encoder();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
  cuuint64_t strides[2] = {(cuuint64_t)g.pitch * es, (cuuint64_t)g.plane * es};
  cuuint32_t box[3] = {box_x, box_y, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return fn(m, type, 3, const_cast<void *>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace
}  // namespace tma
}  // namespace heat
