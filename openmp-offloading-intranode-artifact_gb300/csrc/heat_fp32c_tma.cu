// FP32-compensated form, two time steps per launch (temporal blocking), with
// plane tiles staged into shared memory by TMA.
//
// A block owns a (32 x 16) tile of output columns and walks a chunk of planes;
// it has one thread per point of the tile plus a 1-point halo (34 x 18).
// For every plane p the block's thread 0 issues TMA 3-D box loads
// (cp.async.bulk.tensor) of the five input arrays -- v, carry, wx, wy, wz --
// covering the tile plus a 2-point halo into one slot of a 4-deep shared
// memory ring, completing on that slot's mbarrier; loads run two planes ahead
// of use.  Each iteration k then
//   1. computes step t+1 on plane k+1 over the tile plus a 1-point halo
//      (34 x 18 points) from ring planes k, k+1, k+2 into a 3-plane ring of
//      intermediate values, and
//   2. computes step t+2 on plane k-1 over the tile from intermediate planes
//      k-2, k-1, k and writes it to global memory.
// Running step t+2 one plane behind step t+1 leaves one block barrier per
// plane (it publishes the landed input plane and the previous iteration's
// intermediate plane together); at 48 registers two blocks fit on an SM.
// Global traffic per two updates: the five input arrays read once (plus the
// halo, mostly served by L2) and v, carry written once -- about half of two
// single steps.  The per-point arithmetic is exactly the single-step column
// walk's (walk_fp32c: same operations, same order, the intermediate carry
// rounded to BF16 as the single step stores it), so two steps here are
// bit-identical to two single steps.  Points on the grid boundary keep their
// values at both levels.
//
// Every mbarrier wait is bounded: if a load does not complete within the
// limit the block records the failure in *err, waits (bounded) for its other
// loads in flight, and returns; the host reports HEAT_ETIMEOUT.

#include <cuda.h>

#include "heat_batch_internal.h"
#include "heat_internal.h"
#include "heat_tma.cuh"
#include "heat_walk.cuh"

namespace heat {
namespace {

constexpr int OX = 32, OY = 16;          // output tile
constexpr int BXF = 40, BXC = 48, BY = OY + 4;  // TMA boxes (float arrays, BF16 carry)
constexpr int L1X = OX + 2, L1Y = OY + 2;   // step-(t+1) region
constexpr int NT = ((L1X * L1Y + 31) / 32) * 32;  // one thread per step-(t+1) point
constexpr int R = 4;                     // ring depth (planes)
static_assert((R & (R - 1)) == 0, "slot index p & (R - 1) needs R a power of two");

constexpr int kPlaneF = BXF * BY;        // floats per float-array plane tile
constexpr int kPlaneC = BXC * BY;        // BF16 per carry plane tile
constexpr unsigned kSlotBytes = 4u * kPlaneF * 4u + 2u * kPlaneC;  // v, wx, wy, wz + carry
// A TMA tile copy writes shared memory from a 128-byte aligned address, so
// each array of a slot starts on a 128-byte boundary: arrays are strided by
// their box size rounded up to 128 bytes (the copies still move box bytes).
constexpr int kStrideF = (kPlaneF * 4 + 127) / 128 * 128 / 4;
constexpr int kStrideC = (kPlaneC * 2 + 127) / 128 * 128 / 2;
static_assert((kStrideF * 4) % 128 == 0 && (kStrideC * 2) % 128 == 0,
              "slot arrays must start on 128-byte boundaries");

struct __align__(128) Slot {
  float v[kStrideF];
  float wx[kStrideF];
  float wy[kStrideF];
  float wz[kStrideF];
  uint16_t c[kStrideC];
};
static_assert(sizeof(Slot) % 128 == 0, "ring slots must start on 128-byte boundaries");

struct Smem {
  Slot ring[R];
  float v1[3][NT];
  unsigned long long bar[R];
};

using tma::mbar_expect;
using tma::mbar_init;
using tma::mbar_wait;
using tma::smem_u32;

__device__ __forceinline__ void tma_load3(void *dst, const CUtensorMap *map, int x, int y, int z,
                                          unsigned long long *bar) {
  tma::load3(dst, map, x, y, z, bar);
}

struct Maps {
  CUtensorMap v, c, wx, wy, wz;
};

// Where a tile finds its five tensor maps: the single-grid kernel's
// __grid_constant__ parameters, or seven maps per grid in device memory for
// the batch table (buffer `src` of v and carry, then wx, wy, wz).
struct ParamMaps {
  const Maps &in;
  __device__ __forceinline__ const CUtensorMap *v() const { return &in.v; }
  __device__ __forceinline__ const CUtensorMap *c() const { return &in.c; }
  __device__ __forceinline__ const CUtensorMap *wx() const { return &in.wx; }
  __device__ __forceinline__ const CUtensorMap *wy() const { return &in.wy; }
  __device__ __forceinline__ const CUtensorMap *wz() const { return &in.wz; }
};
struct TableMaps {
  const CUtensorMap *tm;
  int src;
  __device__ __forceinline__ const CUtensorMap *v() const { return &tm[src]; }
  __device__ __forceinline__ const CUtensorMap *c() const { return &tm[2 + src]; }
  __device__ __forceinline__ const CUtensorMap *wx() const { return &tm[4]; }
  __device__ __forceinline__ const CUtensorMap *wy() const { return &tm[5]; }
  __device__ __forceinline__ const CUtensorMap *wz() const { return &tm[6]; }
};

// Two steps over one (32 x 16)-column tile with origin (x0, y0), planes
// [kb, ke), of a field whose five input arrays the maps describe.  Writes vn
// / cn.  When a bounded wait runs out it sets *err and returns once its own
// loads in flight have landed.
template <class M>
__device__ __forceinline__ void tb2_tile(const M &maps, float *__restrict__ vn,
                                         uint16_t *__restrict__ cn, int x0, int y0, int nx,
                                         int ny, int nz, int P, size_t S, int kb, int ke,
                                         int *__restrict__ err, unsigned wait_limit) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
  const int tid = threadIdx.x;
  const int X0 = x0 - 5, X0c = x0 - 9, Y0 = y0 - 2;  // box origins (X0 % 4 == 0, X0c % 8 == 0)
  const int pmin = max(kb - 2, 0), pmax = min(ke + 1, nz - 1);

  if (tid == 0) {
    for (int s = 0; s < R; ++s) mbar_init(&sm.bar[s]);
    tma::mbar_init_fence();
  }
  __syncthreads();

  // Warp 0 keeps the bookkeeping (which slots have a load in flight, and each
  // slot's next completion parity) and alone spins on the mbarrier; thread 0
  // issues the TMA.  The block barrier after the wait hands the landed tile to
  // the other warps, which skip all of it (a warp-uniform branch).
  unsigned pending = 0, phase = 0;
  bool failed = false;
  const bool waiter = tid < 32;
  auto issue = [&](int p) {
    if (!waiter || p < pmin || p > pmax) return;
    const int s = p & (R - 1);
    pending |= 1u << s;
    if (tid != 0) return;
    Slot &sl = sm.ring[s];
    unsigned long long *b = &sm.bar[s];
    tma::fence_proxy_async();
    mbar_expect(b, kSlotBytes);
    tma_load3(sl.v, maps.v(), X0, Y0, p, b);
    tma_load3(sl.wx, maps.wx(), X0, Y0, p, b);
    tma_load3(sl.wy, maps.wy(), X0, Y0, p, b);
    tma_load3(sl.wz, maps.wz(), X0, Y0, p, b);
    tma_load3(sl.c, maps.c(), X0c, Y0, p, b);
  };
  auto wait_plane = [&](int p) {
    if (!waiter || p < pmin || p > pmax || failed) return;
    const int s = p & (R - 1);
    if (!mbar_wait(&sm.bar[s], (phase >> s) & 1u, wait_limit)) {
      failed = true;
      return;
    }
    phase ^= 1u << s;
    pending &= ~(1u << s);
  };

  for (int p = kb - 2; p <= kb + 1; ++p) issue(p);

  // This thread's step-(t+1) point (lx, ly) in the (34 x 18) region and its
  // smem offsets; threads with 1 <= lx <= 32, 1 <= ly <= 16 also own an
  // output point.  Like the single-step walk, each thread carries its own
  // column along z in registers: the centre values of the input planes, the
  // step-(t+1) values it computed, and the face weights it already loaded;
  // only neighbours come from shared memory.
  const bool l1_ok = tid < L1X * L1Y;
  const int lx = tid % L1X, ly = tid / L1X;
  const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
  const int o = (ly + 1) * BXF + (lx + 4);     // float box offset
  const int oc = (ly + 1) * BXC + (lx + 8);    // carry box offset
  const bool edge = gx <= 0 || gy <= 0 || gx >= nx - 1 || gy >= ny - 1;
  const bool out_ok = l1_ok && lx >= 1 && lx <= OX && ly >= 1 && ly <= OY && gx < nx - 1 &&
                      gy < ny - 1;

  struct W {
    float x, xm, y, ym, z;  // wx[c], wx[c-1], wy[c], wy[c-P], wz[c] at one plane
  };
  // Step t+1 on plane p at this thread's point from centre values vm, v0, vp
  // (planes p-1, p, p+1) and wz at plane p-1; returns the new value and carry
  // and the plane's weights.
  auto level1 = [&](int p, float vm, float v0, float vp, float wzm, W &wp, float &t1,
                    float &c1) {
    const Slot &cur = sm.ring[p & (R - 1)];
    wp.x = cur.wx[o];
    wp.xm = cur.wx[o - 1];
    wp.y = cur.wy[o];
    wp.ym = cur.wy[o - BXF];
    wp.z = cur.wz[o];
    const float cc0 = walk::bf2f(cur.c[oc]);
    if (edge || p == 0 || p == nz - 1) {
      t1 = v0;
      c1 = cc0;
      return;
    }
    float d = 0.0f;
    d = fmaf(wp.x, cur.v[o + 1] - v0, d);
    d = fmaf(wp.xm, cur.v[o - 1] - v0, d);
    d = fmaf(wp.y, cur.v[o + BXF] - v0, d);
    d = fmaf(wp.ym, cur.v[o - BXF] - v0, d);
    d = fmaf(wp.z, vp - v0, d);
    d = fmaf(wzm, vm - v0, d);
    const float yk = __fsub_rn(d, cc0);
    t1 = __fadd_rn(v0, yk);
    c1 = walk::bf2f(walk::f2bf(__fsub_rn(__fsub_rn(t1, v0), yk)));
  };

  // Prologue: intermediate planes kb-1 and kb.  A failed wait stops the whole
  // block (the decision is made block-wide).
  wait_plane(kb - 2);
  wait_plane(kb - 1);
  wait_plane(kb);
  wait_plane(kb + 1);
  failed = __syncthreads_or(failed);
  // Level-1 window: v(p-1), v(p), wz(p-1) for the next plane p to compute.
  float vm = 0.f, v0 = 0.f, wzm = 0.f;
  // Level-2 window at the top of iteration k: own step-(t+1) values at planes
  // k-2, k-1, k, the carries at k-1, k, the weights at k-1, k and wz at k-2.
  float l1a = 0.f, l1b = 0.f, l1cc = 0.f;
  float c1b = 0.f, c1cc = 0.f;
  W wb{}, wcc{};
  float wza = 0.f;
  if (!failed && l1_ok) {
    if (kb - 2 >= 0) {
      vm = sm.ring[(kb - 2) & (R - 1)].v[o];
      wzm = sm.ring[(kb - 2) & (R - 1)].wz[o];
    }
    v0 = sm.ring[(kb - 1) & (R - 1)].v[o];
    float vp = sm.ring[kb & (R - 1)].v[o];
    level1(kb - 1, vm, v0, vp, wzm, wb, l1b, c1b);
    sm.v1[(kb - 1) % 3][tid] = l1b;
    vm = v0;
    v0 = vp;
    wzm = wb.z;
    vp = sm.ring[(kb + 1) & (R - 1)].v[o];
    level1(kb, vm, v0, vp, wzm, wcc, l1cc, c1cc);
    sm.v1[kb % 3][tid] = l1cc;
    vm = v0;
    v0 = vp;
    wzm = wcc.z;
  }
  // The prologue's reads of planes kb-2 and kb-1 are done: their slots take
  // planes kb+2 and kb+3.
  __syncthreads();
  if (!failed) {
    issue(kb + 2);
    issue(kb + 3);
  }

  // Step t+2 runs one plane behind step t+1: iteration k computes step t+1 on
  // plane k+1 and step t+2 on plane k-1, so the one barrier at the top of an
  // iteration publishes both the landed plane k+2 and the previous
  // iteration's step-(t+1) plane k, and retires ring slot k mod R and
  // intermediate slot (k+1) mod 3 for reuse.  Iteration kb writes no output
  // (plane kb-1 is outside the chunk); iteration ke computes no step t+1.
  // Intermediate slots of planes k-1, k, k+1 and the output offset of plane
  // k-1, advanced with k.
  int ia = (kb + 2) % 3, ib = kb % 3, ic = (kb + 1) % 3;
  size_t g = (size_t)(kb - 1) * S + (size_t)gy * P + gx;
  // Unrolled by the intermediate ring's period (3): the slot indices and the
  // shift of the carried values resolve to fixed registers in each copy
  // (512^3: 325 GLUP/s unrolled by 3, 308 not unrolled, 286 by 2, 321 by 6,
  // 284 by 12, which spills).
#pragma unroll 3
  for (int k = kb; k <= ke && !failed; ++k, g += S) {
    wait_plane(k + 2);
    failed = __syncthreads_or(failed);
    if (failed) break;
    issue(k + 4);
    W wn{};
    float l1p = 0.f, c1p = 0.f;
    if (k + 1 <= ke && l1_ok) {
      const float vp = sm.ring[(k + 2) & (R - 1)].v[o];
      level1(k + 1, vm, v0, vp, wzm, wn, l1p, c1p);
      sm.v1[ic][tid] = l1p;
      vm = v0;
      v0 = vp;
      wzm = wn.z;
    }
    if (k - 1 >= kb && out_ok) {
      const float *vk = sm.v1[ia];
      float d = 0.0f;
      d = fmaf(wb.x, vk[tid + 1] - l1b, d);
      d = fmaf(wb.xm, vk[tid - 1] - l1b, d);
      d = fmaf(wb.y, vk[tid + L1X] - l1b, d);
      d = fmaf(wb.ym, vk[tid - L1X] - l1b, d);
      d = fmaf(wb.z, l1cc - l1b, d);
      d = fmaf(wza, l1a - l1b, d);
      const float yk = __fsub_rn(d, c1b);
      const float t = __fadd_rn(l1b, yk);
      const float cc = __fsub_rn(__fsub_rn(t, l1b), yk);
      vn[g] = t;
      cn[g] = walk::f2bf(cc);
    }
    l1a = l1b;
    l1b = l1cc;
    l1cc = l1p;
    c1b = c1cc;
    c1cc = c1p;
    wza = wb.z;
    wb = wcc;
    wcc = wn;
    const int t3 = ia;
    ia = ib;
    ib = ic;
    ic = t3;
  }
  if (failed) {
    if (tid == 0) atomicExch(err, 1);
    // Let the block's own loads in flight land before its shared memory goes
    // (each wait bounded).
    if (waiter)
      for (int s = 0; s < R; ++s)
        if (pending & (1u << s)) mbar_wait(&sm.bar[s], (phase >> s) & 1u);
  }
}

__global__ void __launch_bounds__(NT, 2)
    k_fp32c_tb2(const __grid_constant__ Maps in, float *__restrict__ vn,
                uint16_t *__restrict__ cn, int nx, int ny, int nz, int P, size_t S, int kchunk,
                int *__restrict__ err, unsigned wait_limit) {
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (kb >= ke) return;
  tb2_tile(ParamMaps{in}, vn, cn, 1 + OX * blockIdx.x, 1 + OY * blockIdx.y, nx, ny, nz, P, S, kb,
           ke, err, wait_limit);
}

// The batch table's two-step FP32C tiles: one block per tile, hardware
// scheduled.  Grid g's maps are in device memory, seven per grid: v and carry
// of buffers 0 and 1, then wx, wy, wz; each launch reads buffer cur ^ flip.
__global__ void __launch_bounds__(NT, 2)
    k_batch_fp32c_tb2(const BatchGrid *__restrict__ grids, const BatchTile *__restrict__ tiles,
                      int flip) {
  const BatchTile tl = tiles[blockIdx.x];
  const BatchGrid &g = grids[tl.grid];
  const int src = g.cur ^ flip, dst = src ^ 1;
  const CUtensorMap *tm = static_cast<const CUtensorMap *>(g.tmaps);
  // The maps were written by a host copy before the launch; order the tensor
  // proxy's reads of them after it.
  if (threadIdx.x < 7)
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tm + threadIdx.x)
                 : "memory");
  __syncthreads();
  tb2_tile(TableMaps{tm, src}, (float *)g.f[dst], g.cr[dst], 1 + OX * tl.tx, 1 + OY * tl.ty, g.nx,
           g.ny, g.nz, g.P, g.S, tl.k0, tl.k1, g.err, kWaitLimit);
}

bool encode(CUtensorMap *m, const void *base, bool bf16, const heat_geom &g) {
  return tma::encode_field(m, base,
                           bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                           bf16 ? 2 : 4, g, bf16 ? BXC : BXF, BY);
}

}  // namespace

size_t fp32c_tb2_smem() { return sizeof(Smem) + 128; }

cudaError_t launch_batch_fp32c_tb2(const BatchGrid *grids, const BatchTile *tiles, int ntiles,
                                   int flip, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  static bool attr =
      cudaFuncSetAttribute(k_batch_fp32c_tb2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)fp32c_tb2_smem()) == cudaSuccess;
  if (!attr) return cudaErrorInvalidConfiguration;
  k_batch_fp32c_tb2<<<ntiles, NT, fp32c_tb2_smem(), st>>>(grids, tiles, flip);
  return cudaGetLastError();
}

bool encode_fp32c_maps(CUtensorMap *m7, float *const v[2], uint16_t *const c[2],
                       float *const w[3], const heat_geom &g) {
  return encode(&m7[0], v[0], false, g) && encode(&m7[1], v[1], false, g) &&
         encode(&m7[2], c[0], true, g) && encode(&m7[3], c[1], true, g) &&
         encode(&m7[4], w[0], false, g) && encode(&m7[5], w[1], false, g) &&
         encode(&m7[6], w[2], false, g);
}

// Whether the two-step kernel can run this geometry: row and plane strides in
// bytes must be multiples of 16 for TMA (pitch a multiple of 8 points).
bool fp32c_tb2_ok(const heat_geom &g) {
  return (g.pitch % 8) == 0 && g.nx >= 3 && tma::encoder() != nullptr;
}

cudaError_t launch_fp32c_tb2(float *v_new, uint16_t *c_new, const float *v, const uint16_t *cr,
                             float *const w[3], const heat_geom &g, int *err, cudaStream_t st,
                             unsigned wait_limit) {
  if (wait_limit > tma::kWaitLimit) wait_limit = tma::kWaitLimit;
  Maps m;
  if (!encode(&m.v, v, false, g) || !encode(&m.c, cr, true, g) || !encode(&m.wx, w[0], false, g) ||
      !encode(&m.wy, w[1], false, g) || !encode(&m.wz, w[2], false, g))
    return cudaErrorInvalidValue;
  static bool attr = cudaFuncSetAttribute(k_fp32c_tb2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)fp32c_tb2_smem()) == cudaSuccess;
  if (!attr) return cudaErrorInvalidConfiguration;
  const int bx = (g.nx - 2 + OX - 1) / OX, by = (g.ny - 2 + OY - 1) / OY;
  const int interior = g.nz - 2;
  // Each chunk recomputes step t+1 on its halo planes, so chunks are deeper
  // than the single-step launches': 96 planes at least (512^3: 330 GLUP/s,
  // against 324 / 320 / 309 for 64 / 48 / 32 and 311 for 128, where 3 chunks
  // leave 5.05 waves), 16 where a small grid needs more chunks to fill the GPU.
  static const long resident = resident_blocks((const void *)k_fp32c_tb2, NT, fp32c_tb2_smem());
  const int kchunk = wave_chunk(g, OX, OY, resident, 24, 96, 16);
  dim3 grid(bx, by, (interior + kchunk - 1) / kchunk);
  k_fp32c_tb2<<<grid, NT, fp32c_tb2_smem(), st>>>(m, v_new, c_new, g.nx, g.ny, g.nz, g.pitch,
                                                  g.plane, kchunk, err, wait_limit);
  return cudaGetLastError();
}

}  // namespace heat
