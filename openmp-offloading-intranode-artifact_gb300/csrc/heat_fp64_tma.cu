// Default FP64 form, no source term: the warpgroup-split launch with the
// integer rows' plane tiles staged by TMA and every value decoded once.
//
// Same split and the same arithmetic as k_fast_ws (heat_fp64_int.cu): blocks of
// 32 x 8 columns walk a z-chunk; warps 0-3 walk the FP64-pipe rows
// ((j - 1) mod 8 < 4) exactly as there, warps 4-7 evaluate the integer rows
// with walk::int_point, so the results are bit-identical to k_fast_ws and to
// the batch table kernels.  What changes is how the integer rows get their
// inputs.  In k_fast_ws every integer thread loads its five neighbours' u and
// K from global memory and decodes the four in-plane ones itself: each value is
// decoded five times, and the loads, their 64-bit addresses and the prefetch
// registers (spilled) cost about 420 warp instructions per point.  Here:
//
//   * per plane, one thread issues TMA 3-D box loads (cp.async.bulk.tensor) of
//     u and K over the integer rows plus a one-point halo (34 x 6 points; rows
//     j0+3 .. j0+8 of the block's rows j0 .. j0+7) into a 4-deep shared-memory
//     ring, each slot completing on its own mbarrier;
//   * a decode pass turns plane k+1 of the ring into (exponent, aligned
//     significand) pairs in a 3-deep decoded ring -- each thread decodes its own
//     column and 76 threads the halo, 1.6 decodes per point instead of 5;
//   * one named barrier per plane (the integer warpgroup's alone, reducing a
//     failure flag) publishes the decoded plane, and the evaluation of plane k
//     reads its in-plane neighbours and K from shared memory; z-neighbours stay
//     in registers.
//
// Three decoded slots make one barrier per plane enough: plane k+1 is written
// while a slower thread may still read plane k-1's slot, and plane k's slot was
// published by the previous barrier.  A raw slot is refilled three planes ahead,
// once the barrier shows every thread is done with the plane it held (its K and,
// for non-finite stencils, its raw bits are read during that plane's evaluation).
//
// Every mbarrier wait is bounded: a wait that runs out makes the warpgroup stop
// at the next barrier (the flag is OR-reduced), the issuing thread waits
// (bounded) for its loads in flight, *err is set and the host reports
// HEAT_ETIMEOUT.  The FP64 warps have no waits and finish their rows.

#include <cuda.h>

#include "heat_internal.h"
#include "heat_tma.cuh"
#include "heat_walk.cuh"

namespace heat {
namespace {

typedef unsigned long long u64;
typedef long long i64;

constexpr int TX = 32, TY = 8;
constexpr int RW = TX + 2;   // region columns: i0 - 1 .. i0 + 32
constexpr int RH = 6;        // region rows: the 4 integer rows and one on each side
constexpr int RP = RW * RH;  // 204 points
constexpr int RPAD = 208;    // per-array stride: 1664 bytes, a multiple of 128
constexpr int NR = 4;        // TMA ring depth (planes)
constexpr int ND = 3;        // decoded ring depth (planes)
constexpr int kIntThreads = 128;
constexpr int kBarInt = 1;   // named barrier id of the integer warpgroup
constexpr unsigned kSlotBytes = 2u * RP * 8u;  // u box + K box (OOB-filled boxes count in full)
static_assert((NR & (NR - 1)) == 0, "slot index p & (NR - 1) needs NR a power of two");
static_assert((RPAD * 8) % 128 == 0 && RPAD >= RP, "TMA destinations start on 128-byte boundaries");

struct __align__(128) RawSlot {
  u64 u[RPAD];
  u64 k[RPAD];
};
static_assert(sizeof(RawSlot) % 128 == 0, "ring slots start on 128-byte boundaries");

struct SmemT {
  RawSlot raw[NR];
  i64 m[ND][RPAD];  // decoded significands << 9, signed
  int e[ND][RPAD];  // decoded biased exponents (subnormals and zero: 1)
  u64 bar[NR];
};

struct IntMaps {
  CUtensorMap u, k;
};

// Named barrier over the integer warpgroup that also ORs a flag across it.
__device__ __forceinline__ bool bar_or(bool flag) {
  unsigned r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "barrier.cta.red.or.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((unsigned)flag), "n"(kBarInt), "n"(kIntThreads)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void bar_int() {
  asm volatile("barrier.cta.sync %0, %1;" ::"n"(kBarInt), "n"(kIntThreads) : "memory");
}

constexpr int kTmaRegs = 64;

template <int REGS = kTmaRegs>
__global__ void __launch_bounds__(TX *TY, 4)
    k_fast_tma(const __grid_constant__ IntMaps maps, double *__restrict__ un,
               const double *__restrict__ u, const double *__restrict__ c0,
               const double *__restrict__ cx, const double *__restrict__ cy,
               const double *__restrict__ cz, int nx, int ny, int nz, int P, size_t S,
               int kchunk, int *__restrict__ err, unsigned wait_limit) {
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (kb >= ke) return;  // whole block
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  if (threadIdx.y < 4) {
    // FP64-pipe rows: the column walk of k_fast_ws, global loads, no barriers.
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;\n" ::"n"(REGS));
    if (i >= nx - 1 || j >= ny - 1) return;
    const size_t c = (size_t)kb * S + (size_t)j * P + i;
    walk::walk_hw<false, 2>(un, u, nullptr, c0, cx, cy, cz, P, S, c, kb, ke);
    return;
  }
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;\n" ::"n"(REGS));
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemT &sm = *reinterpret_cast<SmemT *>(smem_raw);

  const int t = threadIdx.x + 32 * (threadIdx.y - 4);  // 0 .. 127
  const int own = (threadIdx.y - 3) * RW + threadIdx.x + 1;  // region rows 1..4, columns 1..32
  const bool active = i < nx - 1 && j < ny - 1;
  const int X0 = blockIdx.x * TX;      // region column 0 = grid column i0 - 1 (x * 8 B % 16 == 0)
  const int Y0 = blockIdx.y * TY + 4;  // region row 0 = grid row j0 + 3
  // The halo point this thread decodes besides its own: rows 0 and 5, then
  // columns 0 and 33 of rows 1..4 (76 points), or none.
  int p2 = -1;
  if (t < RW) p2 = t;
  else if (t < 2 * RW) p2 = (RH - 1) * RW + (t - RW);
  else if (t < 2 * RW + 4) p2 = (1 + t - 2 * RW) * RW;
  else if (t < 2 * RW + 8) p2 = (1 + t - 2 * RW - 4) * RW + RW - 1;

  if (t == 0) {
    for (int s = 0; s < NR; ++s) tma::mbar_init(&sm.bar[s]);
    tma::mbar_init_fence();
  }
  bar_int();

  // Every thread tracks the ring's completion parities and waits itself (with
  // a suspend hint); thread 0 also issues the loads and tracks what is in
  // flight for the drain after a failure.
  unsigned phase = 0, pending = 0;
  auto issue = [&](int p) {
    if (p > ke) return;
    const int s = p & (NR - 1);
    pending |= 1u << s;
    if (t != 0) return;
    RawSlot &sl = sm.raw[s];
    tma::fence_proxy_async();
    tma::mbar_expect(&sm.bar[s], kSlotBytes);
    tma::load3(sl.u, &maps.u, X0, Y0, p, &sm.bar[s]);
    tma::load3(sl.k, &maps.k, X0, Y0, p, &sm.bar[s]);
  };
  auto wait = [&](int p) -> bool {
    const int s = p & (NR - 1);
    if (!tma::mbar_wait(&sm.bar[s], (phase >> s) & 1u, wait_limit)) return false;
    phase ^= 1u << s;
    pending &= ~(1u << s);
    return true;
  };
  // Decode plane p of the ring into decoded slot d; returns this thread's own
  // column value (raw bits and decoded).
  auto decode_pass = [&](int p, int d, u64 &braw, walk::Dec &dec) {
    const RawSlot &sl = sm.raw[p & (NR - 1)];
    braw = sl.u[own];
    dec = walk::decode(braw);
    sm.e[d][own] = dec.e;
    sm.m[d][own] = dec.m9;
    if (p2 >= 0) {
      const walk::Dec h = walk::decode(sl.u[p2]);
      sm.e[d][p2] = h.e;
      sm.m[d][p2] = h.m9;
    }
  };

  for (int p = kb - 1; p <= kb + 2; ++p) issue(p);

  bool failed = false;
  // Own column below the chunk (plane kb - 1) and the decoded plane kb.
  u64 bd = 0, bc = 0, Kd = 0;
  walk::Dec dd{1, 0}, dc{1, 0};
  int dcur = kb % ND;  // decoded slot of plane k
  if (wait(kb - 1)) {
    const RawSlot &sl = sm.raw[(kb - 1) & (NR - 1)];
    bd = sl.u[own];
    Kd = sl.k[own];
    dd = walk::decode(bd);
  } else {
    failed = true;
  }
  if (!failed && wait(kb))
    decode_pass(kb, dcur, bc, dc);
  else
    failed = true;

  size_t c = (size_t)kb * S + (size_t)j * P + i;
  for (int k = kb; k < ke; ++k, c += S) {
    const int dnext = dcur == ND - 1 ? 0 : dcur + 1;
    u64 bu = 0;
    walk::Dec du{1, 0};
    if (!failed) {
      if (wait(k + 1))
        decode_pass(k + 1, dnext, bu, du);
      else
        failed = true;
    }
    // Publishes decoded plane k+1 (read next iteration) and retires the raw
    // slot of plane k - 1, which takes plane k + 3.
    if (bar_or(failed)) {
      failed = true;
      break;
    }
    issue(k + 3);
    const RawSlot &rk = sm.raw[k & (NR - 1)];
    const u64 Kc = rk.k[own];
    if (active) {
      const int *ek = sm.e[dcur];
      const i64 *mk = sm.m[dcur];
      const walk::Dec de{ek[own + 1], mk[own + 1]}, dw{ek[own - 1], mk[own - 1]};
      const walk::Dec dn{ek[own + RW], mk[own + RW]}, ds{ek[own - RW], mk[own - RW]};
      const u64 Ku = sm.raw[(k + 1) & (NR - 1)].k[own];
      const u64 bcc = bc, bdd = bd, buu = bu;
      un[c] = walk::int_point<false>(
          dc, du, dd, de, dw, dn, ds, Kc, Ku, Kd, rk.k[own + 1], rk.k[own - 1], rk.k[own + RW],
          rk.k[own - RW], 0ull, [&] {
            return walk::Raw7{bcc, rk.u[own + 1], rk.u[own - 1], rk.u[own + RW], rk.u[own - RW],
                              buu, bdd};
          });
    }
    bd = bc;
    bc = bu;
    dd = dc;
    dc = du;
    Kd = Kc;
    dcur = dnext;
  }
  if (failed && t == 0) {
    atomicExch(err, 1);
    // The block's shared memory must outlive its loads in flight (each wait
    // bounded by the product limit).
    for (int s = 0; s < NR; ++s)
      if (pending & (1u << s)) tma::mbar_wait(&sm.bar[s], (phase >> s) & 1u);
  }
}

size_t tma_smem() { return sizeof(SmemT) + 128; }

bool encode_u64(CUtensorMap *m, const void *base, const heat_geom &g) {
  return tma::encode_field(m, base, CU_TENSOR_MAP_DATA_TYPE_UINT64, 8, g, RW, RH);
}

}  // namespace

// Usable when the tensor-map encoder is available, the field rows are
// multiples of 16 bytes (pitch a multiple of 2 points: always, it is a
// multiple of 4) and the kernel compiled to the register count its setmaxnreg
// bounds assume.
bool fast_tma_usable(const heat_geom &g) {
  static const bool ok = [] {
    if (!tma::encoder()) return false;
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, k_fast_tma<>) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (a.numRegs != kTmaRegs) return false;
    return cudaFuncSetAttribute(k_fast_tma<>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tma_smem()) == cudaSuccess;
  }();
  return ok && (g.pitch % 2) == 0;
}

cudaError_t launch_fast_tma(double *u_new, const double *u_old, const unsigned long long *K,
                            const double *c0, double *const cf[3], const heat_geom &g, int *err,
                            cudaStream_t st, unsigned wait_limit) {
  IntMaps m;
  if (!encode_u64(&m.u, u_old, g) || !encode_u64(&m.k, K, g)) return cudaErrorInvalidValue;
  if (wait_limit > tma::kWaitLimit) wait_limit = tma::kWaitLimit;
  const int kc = plane_chunk(g, TX, TY);
  dim3 gr((g.nx - 2 + TX - 1) / TX, (g.ny - 2 + TY - 1) / TY, (g.nz - 2 + kc - 1) / kc);
  k_fast_tma<><<<gr, dim3(TX, TY), tma_smem(), st>>>(m, u_new, u_old, c0, cf[0], cf[1], cf[2],
                                                     g.nx, g.ny, g.nz, g.pitch, g.plane, kc, err,
                                                     wait_limit);
  return cudaGetLastError();
}

}  // namespace heat
