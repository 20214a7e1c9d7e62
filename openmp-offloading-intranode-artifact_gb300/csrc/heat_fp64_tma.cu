// Default FP64 form: the warpgroup-split launch with every input staged in
// shared memory by TMA and every integer-row value decoded once, with or
// without a source term (then a 34 x 4 box of it per slot at each
// warpgroup's own rows, 3 blocks per SM at 80 registers instead of 4 at 64).
//
// Same split and the same arithmetic as k_fast_ws (heat_fp64_int.cu): blocks of
// 32 x 8 columns walk a z-chunk; warps 0-3 evaluate the FP64-pipe rows
// ((j - 1) mod 8 < 4) with the 7-FMA weighted sum in HwCol's order, warps 4-7
// the integer rows with walk::int_point, so the results are bit-identical to
// k_fast_ws and to the batch table kernels.  What changes is how the rows get
// their inputs.  In k_fast_ws every thread loads its stencil (and, on the
// integer rows, decodes its four in-plane neighbours) from global memory: each
// integer-row value is decoded five times, and the loads, their 64-bit
// addresses and the prefetch registers cost about 420 warp instructions per
// integer point and 107 per FP64 point.  Here each warpgroup has its own
// 4-deep shared-memory ring of plane tiles, filled by TMA 3-D box loads
// (cp.async.bulk.tensor) that one thread issues three planes ahead, each slot
// completing on its own mbarrier:
//
//   * FP64 rows j0 .. j0+3: u over rows j0-1 .. j0+4 and the weights c0, cx, cz
//     (rows j0 .. j0+3) and cy (rows j0-1 .. j0+3), 34 columns (i0-1 .. i0+32);
//   * integer rows j0+4 .. j0+7: u and the fixed-point K over rows j0+3 ..
//     j0+8, 34 columns; a decode pass turns plane k+1 into (exponent, aligned
//     significand) pairs in a 3-deep decoded ring -- each thread decodes its
//     own column and 76 threads the halo, 1.6 decodes per point instead of 5.
//
// One named barrier per plane and warpgroup (reducing a failure flag)
// publishes the landed (and decoded) plane and retires the slot of plane k-1,
// which then takes plane k+3.  Three decoded slots make that one barrier
// enough: plane k+1 is written while a slower thread may still read plane
// k-1's slot, and plane k's slot was published by the previous barrier.  The
// two warpgroups never wait on each other.
//
// Every mbarrier wait is bounded: a wait that runs out makes its warpgroup stop
// at the next barrier (the flag is OR-reduced), the issuing thread waits
// (bounded) for its loads in flight, *err is set and the host reports
// HEAT_ETIMEOUT.

#include <cuda.h>

#include <cstring>

#include "heat_internal.h"
#include "heat_tma.cuh"
#include "heat_walk.cuh"

namespace heat {
namespace {

typedef unsigned long long u64;
typedef long long i64;

constexpr int TX = 32, TY = 8;
constexpr int RW = TX + 2;   // box columns: i0 - 1 .. i0 + 32 (origin x * 8 B is 16-byte aligned)
constexpr int NR = 4;        // TMA ring depth (planes), each warpgroup
constexpr int ND = 3;        // decoded ring depth (planes)
constexpr int kWgThreads = 128;
constexpr int kBarHw = 1, kBarInt = 2;  // named barrier ids of the two warpgroups
static_assert((NR & (NR - 1)) == 0, "slot index p & (NR - 1) needs NR a power of two");

// Padded element count of an array of `rows` box rows: each array of a slot
// starts on a 128-byte boundary, as TMA shared-memory destinations must.
constexpr int pad128(int rows) { return (rows * RW * 8 + 127) / 128 * 128 / 8; }

// Integer rows' slot: u and K over rows j0+3 .. j0+8.
constexpr int kIntRows = 6;
constexpr int kIntPts = kIntRows * RW;  // 204
constexpr int kIntPad = pad128(kIntRows);
// With a source term each slot also holds its rows' source values (a 34 x 4
// box at the warpgroup's own rows).
constexpr int kRPad = pad128(4);
template <bool RHS>
struct __align__(128) IntSlotT {
  u64 u[kIntPad];
  u64 k[kIntPad];
};
template <>
struct __align__(128) IntSlotT<true> {
  u64 u[kIntPad];
  u64 k[kIntPad];
  u64 r[kRPad];
};
template <bool RHS>  // OOB-filled boxes count in full
constexpr unsigned kIntSlotBytes = 2u * kIntPts * 8u + (RHS ? 4u * RW * 8u : 0u);

// FP64 rows' slot: u over rows j0-1 .. j0+4, c0 / cx / cz over rows j0 .. j0+3,
// cy over rows j0-1 .. j0+3.
constexpr int kHwPad6 = pad128(6), kHwPad4 = pad128(4), kHwPad5 = pad128(5);
template <bool RHS>
struct __align__(128) HwSlotT {
  double u[kHwPad6];
  double c0[kHwPad4];
  double cx[kHwPad4];
  double cz[kHwPad4];
  double cy[kHwPad5];
};
template <>
struct __align__(128) HwSlotT<true> {
  double u[kHwPad6];
  double c0[kHwPad4];
  double cx[kHwPad4];
  double cz[kHwPad4];
  double cy[kHwPad5];
  double r[kRPad];
};
template <bool RHS>
constexpr unsigned kHwSlotBytes = (6u + 3u * 4u + 5u + (RHS ? 4u : 0u)) * RW * 8u;
static_assert(sizeof(IntSlotT<false>) % 128 == 0 && sizeof(HwSlotT<false>) % 128 == 0 &&
                  sizeof(IntSlotT<true>) % 128 == 0 && sizeof(HwSlotT<true>) % 128 == 0,
              "ring slots start on 128-byte boundaries");
static_assert((kIntPad * 8) % 128 == 0 && (kHwPad4 * 8) % 128 == 0 && (kHwPad5 * 8) % 128 == 0 &&
                  (kHwPad6 * 8) % 128 == 0,
              "every array of a slot starts on a 128-byte boundary");

template <bool RHS>
struct SmemT {
  HwSlotT<RHS> hw[NR];
  IntSlotT<RHS> in[NR];
  i64 m[ND][kIntPad];  // decoded significands << 9, signed
  int e[ND][kIntPad];  // decoded biased exponents (subnormals and zero: 1)
  u64 hbar[NR];
  u64 ibar[NR];
};

struct Maps {
  CUtensorMap u;            // box 34 x 6 (both warpgroups, different origins)
  CUtensorMap k;            // box 34 x 6
  CUtensorMap c0, cx, cz;   // box 34 x 4
  CUtensorMap cy;           // box 34 x 5
  CUtensorMap r;            // box 34 x 4 (source term; set only with one)
};

// Named barrier over one warpgroup that also ORs a flag across it.
template <int ID>
__device__ __forceinline__ bool bar_or(bool flag) {
  unsigned r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "barrier.cta.red.or.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((unsigned)flag), "n"(ID), "n"(kWgThreads)
      : "memory");
  return r != 0;
}

template <int ID>
__device__ __forceinline__ void bar_wg() {
  asm volatile("barrier.cta.sync %0, %1;" ::"n"(ID), "n"(kWgThreads) : "memory");
}

// One warpgroup's ring bookkeeping: every thread tracks the completion
// parities and waits itself (with a suspend hint); thread 0 of the warpgroup
// issues the loads and, after a failure, waits for the ones in flight.
struct Ring {
  unsigned phase = 0, pending = 0;

  __device__ __forceinline__ bool wait(u64 *bars, int p, unsigned limit) {
    const int s = p & (NR - 1);
    if (!tma::mbar_wait(&bars[s], (phase >> s) & 1u, limit)) return false;
    phase ^= 1u << s;
    pending &= ~(1u << s);
    return true;
  }
  __device__ __forceinline__ void drain(u64 *bars) {
    for (int s = 0; s < NR; ++s)
      if (pending & (1u << s)) tma::mbar_wait(&bars[s], (phase >> s) & 1u);
  }
};


// FP64-pipe rows j0 .. j0+3 (warps 0-3): HwCol's weighted sum from staged
// tiles.  Returns true if a wait ran out.
template <bool RHS>
__device__ __forceinline__ bool hw_rows(const Maps &maps, SmemT<RHS> &sm,
                                        double *__restrict__ un, int i, int j, int nx, int ny,
                                        int P, size_t S, int kb, int ke, unsigned wait_limit) {
  typedef HwSlotT<RHS> HwSlot;
  const int t = threadIdx.x + 32 * threadIdx.y;                  // 0 .. 127
  const int ou = (threadIdx.y + 1) * RW + threadIdx.x + 1;       // u, cy: box rows from j0 - 1
  const int ow = threadIdx.y * RW + threadIdx.x + 1;             // c0, cx, cz: box rows from j0
  const bool active = i < nx - 1 && j < ny - 1;
  const int X0 = blockIdx.x * TX, YU = blockIdx.y * TY, YW = YU + 1;
  if (t == 0) {
    for (int s = 0; s < NR; ++s) tma::mbar_init(&sm.hbar[s]);
    tma::mbar_init_fence();
  }
  bar_wg<kBarHw>();
  Ring r;
  auto issue = [&](int p) {
    if (p > ke) return;
    const int s = p & (NR - 1);
    r.pending |= 1u << s;
    if (t != 0) return;
    HwSlot &sl = sm.hw[s];
    u64 *b = &sm.hbar[s];
    tma::fence_proxy_async();
    tma::mbar_expect(b, kHwSlotBytes<RHS>);
    tma::load3(sl.u, &maps.u, X0, YU, p, b);
    tma::load3(sl.c0, &maps.c0, X0, YW, p, b);
    tma::load3(sl.cx, &maps.cx, X0, YW, p, b);
    tma::load3(sl.cz, &maps.cz, X0, YW, p, b);
    tma::load3(sl.cy, &maps.cy, X0, YU, p, b);
    if constexpr (RHS) tma::load3(sl.r, &maps.r, X0, YW, p, b);
  };
  for (int p = kb - 1; p <= kb + 2; ++p) issue(p);
  bool failed = false;
  double ud = 0.0, uc = 0.0, wd = 0.0;
  if (r.wait(sm.hbar, kb - 1, wait_limit)) {
    const HwSlot &sl = sm.hw[(kb - 1) & (NR - 1)];
    ud = sl.u[ou];
    wd = sl.cz[ow];
  } else {
    failed = true;
  }
  if (!failed && r.wait(sm.hbar, kb, wait_limit))
    uc = sm.hw[kb & (NR - 1)].u[ou];
  else
    failed = true;
  size_t c = (size_t)kb * S + (size_t)j * P + i;
  for (int k = kb; k < ke; ++k, c += S) {
    if (!failed && !r.wait(sm.hbar, k + 1, wait_limit)) failed = true;
    if (bar_or<kBarHw>(failed)) {
      failed = true;
      break;
    }
    issue(k + 3);  // into the slot of plane k - 1, which every thread is done with
    const HwSlot &sk = sm.hw[k & (NR - 1)];
    const double uu = sm.hw[(k + 1) & (NR - 1)].u[ou];
    const double wu = sk.cz[ow];
    if (active) {
      // HwCol::step's operation order (bit-identical results)
      double acc;
      if constexpr (RHS)
        acc = fma(sk.c0[ow], uc, sk.r[ow]);
      else
        acc = sk.c0[ow] * uc;
      acc = fma(sk.cx[ow], sk.u[ou + 1], acc);
      acc = fma(sk.cx[ow - 1], sk.u[ou - 1], acc);
      acc = fma(sk.cy[ou], sk.u[ou + RW], acc);
      acc = fma(sk.cy[ou - RW], sk.u[ou - RW], acc);
      acc = fma(wu, uu, acc);
      acc = fma(wd, ud, acc);
      un[c] = acc;
    }
    ud = uc;
    uc = uu;
    wd = wu;
  }
  if (failed && t == 0) r.drain(sm.hbar);
  return failed;
}

// Integer rows j0+4 .. j0+7 (warps 4-7): walk::int_point from decoded tiles.
// Returns true if a wait ran out.
template <bool RHS>
__device__ __forceinline__ bool int_rows(const Maps &maps, SmemT<RHS> &sm,
                                         double *__restrict__ un, int i, int j, int nx, int ny,
                                         int P, size_t S, int kb, int ke, unsigned wait_limit) {
  typedef IntSlotT<RHS> IntSlot;
  const int t = threadIdx.x + 32 * (threadIdx.y - 4);        // 0 .. 127
  const int own = (threadIdx.y - 3) * RW + threadIdx.x + 1;  // box rows 1..4, columns 1..32
  const bool active = i < nx - 1 && j < ny - 1;
  const int X0 = blockIdx.x * TX, Y0 = blockIdx.y * TY + 4;  // box row 0 = grid row j0 + 3
  // The halo point this thread decodes besides its own: rows 0 and 5, then
  // columns 0 and 33 of rows 1..4 (76 points), or none.
  int p2 = -1;
  if (t < RW) p2 = t;
  else if (t < 2 * RW) p2 = (kIntRows - 1) * RW + (t - RW);
  else if (t < 2 * RW + 4) p2 = (1 + t - 2 * RW) * RW;
  else if (t < 2 * RW + 8) p2 = (1 + t - 2 * RW - 4) * RW + RW - 1;

  if (t == 0) {
    for (int s = 0; s < NR; ++s) tma::mbar_init(&sm.ibar[s]);
    tma::mbar_init_fence();
  }
  bar_wg<kBarInt>();
  Ring r;
  auto issue = [&](int p) {
    if (p > ke) return;
    const int s = p & (NR - 1);
    r.pending |= 1u << s;
    if (t != 0) return;
    IntSlot &sl = sm.in[s];
    u64 *b = &sm.ibar[s];
    tma::fence_proxy_async();
    tma::mbar_expect(b, kIntSlotBytes<RHS>);
    tma::load3(sl.u, &maps.u, X0, Y0, p, b);
    tma::load3(sl.k, &maps.k, X0, Y0, p, b);
    if constexpr (RHS) tma::load3(sl.r, &maps.r, X0, Y0 + 1, p, b);  // own rows only
  };
  // Decode plane p of the ring into decoded slot d; returns this thread's own
  // column value (raw bits and decoded).
  auto decode_pass = [&](int p, int d, u64 &braw, walk::Dec &dec) {
    const IntSlot &sl = sm.in[p & (NR - 1)];
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
  if (r.wait(sm.ibar, kb - 1, wait_limit)) {
    const IntSlot &sl = sm.in[(kb - 1) & (NR - 1)];
    bd = sl.u[own];
    Kd = sl.k[own];
    dd = walk::decode(bd);
  } else {
    failed = true;
  }
  if (!failed && r.wait(sm.ibar, kb, wait_limit))
    decode_pass(kb, dcur, bc, dc);
  else
    failed = true;

  size_t c = (size_t)kb * S + (size_t)j * P + i;
  for (int k = kb; k < ke; ++k, c += S) {
    const int dnext = dcur == ND - 1 ? 0 : dcur + 1;
    u64 bu = 0;
    walk::Dec du{1, 0};
    if (!failed) {
      if (r.wait(sm.ibar, k + 1, wait_limit))
        decode_pass(k + 1, dnext, bu, du);
      else
        failed = true;
    }
    // Publishes decoded plane k+1 (read next iteration) and retires the raw
    // slot of plane k - 1, which takes plane k + 3.
    if (bar_or<kBarInt>(failed)) {
      failed = true;
      break;
    }
    issue(k + 3);
    const IntSlot &rk = sm.in[k & (NR - 1)];
    const u64 Kc = rk.k[own];
    if (active) {
      const int *ek = sm.e[dcur];
      const i64 *mk = sm.m[dcur];
      const walk::Dec de{ek[own + 1], mk[own + 1]}, dw{ek[own - 1], mk[own - 1]};
      const walk::Dec dn{ek[own + RW], mk[own + RW]}, ds{ek[own - RW], mk[own - RW]};
      const u64 Ku = sm.in[(k + 1) & (NR - 1)].k[own];
      const u64 bcc = bc, bdd = bd, buu = bu;
      u64 br = 0ull;
      if constexpr (RHS) br = rk.r[own - RW];  // the source box starts at box row 1
      un[c] = walk::int_point<RHS>(
          dc, du, dd, de, dw, dn, ds, Kc, Ku, Kd, rk.k[own + 1], rk.k[own - 1], rk.k[own + RW],
          rk.k[own - RW], br, [&] {
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
  if (failed && t == 0) r.drain(sm.ibar);
  return failed;
}

template <bool RHS, int MINB, int REGS>
__global__ void __launch_bounds__(TX *TY, MINB)
    k_fast_tma(const __grid_constant__ Maps maps, double *__restrict__ un, int nx, int ny,
               int nz, int P, size_t S, int kchunk, int *__restrict__ err, unsigned wait_limit) {
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kb + kchunk, nz - 1);
  if (kb >= ke) return;  // whole block
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemT<RHS> &sm = *reinterpret_cast<SmemT<RHS> *>(smem_raw);
  const int i = 1 + blockIdx.x * TX + threadIdx.x;
  const int j = 1 + blockIdx.y * TY + threadIdx.y;
  bool failed;
  // Each warpgroup's code starts with setmaxnreg at the launch count: no
  // registers move, but each region is bounded for the register allocator.
  if (threadIdx.y < 4) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;\n" ::"n"(REGS));
    failed = hw_rows(maps, sm, un, i, j, nx, ny, P, S, kb, ke, wait_limit);
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;\n" ::"n"(REGS));
    failed = int_rows(maps, sm, un, i, j, nx, ny, P, S, kb, ke, wait_limit);
  }
  if (failed && (threadIdx.x | (threadIdx.y & 3)) == 0) atomicExch(err, 1);
}

// Launch shape per variant: without a source term 4 blocks per SM at 64
// registers (47 KB of shared memory each); with one 3 blocks per SM at 80
// registers (56 KB: the source boxes would not fit four).
template <bool RHS>
struct Variant {
  static constexpr int kMinb = RHS ? 3 : 4;
  static constexpr int kRegs = RHS ? 80 : 64;
  static size_t smem() { return sizeof(SmemT<RHS>) + 128; }
  static auto kernel() { return k_fast_tma<RHS, kMinb, kRegs>; }
  // The kernel compiled to the register count its setmaxnreg counts assume.
  static bool usable() {
    static const bool ok = [] {
      if (!tma::encoder()) return false;
      cudaFuncAttributes a;
      if (cudaFuncGetAttributes(&a, kernel()) != cudaSuccess) {
        cudaGetLastError();
        return false;
      }
      if (a.numRegs != kRegs) return false;
      return cudaFuncSetAttribute(kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem()) == cudaSuccess;
    }();
    return ok;
  }
};

bool encode_f64(CUtensorMap *m, const void *base, const heat_geom &g, unsigned rows) {
  return tma::encode_field(m, base, CU_TENSOR_MAP_DATA_TYPE_UINT64, 8, g, RW, rows);
}

template <bool RHS>
cudaError_t launch_variant(const Maps &m, double *u_new, const heat_geom &g, int *err,
                           cudaStream_t st, unsigned wait_limit) {
  typedef Variant<RHS> V;
  static const long resident = resident_blocks((const void *)V::kernel(), TX * TY, V::smem());
  const int kc = wave_chunk(g, TX, TY, resident);
  dim3 gr((g.nx - 2 + TX - 1) / TX, (g.ny - 2 + TY - 1) / TY, (g.nz - 2 + kc - 1) / kc);
  V::kernel()<<<gr, dim3(TX, TY), V::smem(), st>>>(m, u_new, g.nx, g.ny, g.nz, g.pitch, g.plane,
                                                   kc, err, wait_limit);
  return cudaGetLastError();
}

}  // namespace

// Usable when the tensor-map encoder is available, the field rows are
// multiples of 16 bytes (pitch a multiple of 2 points: always, it is a
// multiple of 4) and the variant compiled to the register count its setmaxnreg
// counts assume.
bool fast_tma_usable(const heat_geom &g, bool rhs) {
  const bool ok = rhs ? Variant<true>::usable() : Variant<false>::usable();
  return ok && (g.pitch % 2) == 0;
}

cudaError_t launch_fast_tma(double *u_new, const double *u_old, const unsigned long long *K,
                            const double *c0, double *const cf[3], const double *rhs,
                            const heat_geom &g, int *err, cudaStream_t st, unsigned wait_limit) {
  Maps m;
  if (!encode_f64(&m.u, u_old, g, 6) || !encode_f64(&m.k, K, g, 6) ||
      !encode_f64(&m.c0, c0, g, 4) || !encode_f64(&m.cx, cf[0], g, 4) ||
      !encode_f64(&m.cz, cf[2], g, 4) || !encode_f64(&m.cy, cf[1], g, 5) ||
      (rhs && !encode_f64(&m.r, rhs, g, 4)))
    return cudaErrorInvalidValue;
  if (!rhs) std::memset(&m.r, 0, sizeof m.r);
  if (wait_limit > tma::kWaitLimit) wait_limit = tma::kWaitLimit;
  return rhs ? launch_variant<true>(m, u_new, g, err, st, wait_limit)
             : launch_variant<false>(m, u_new, g, err, st, wait_limit);
}

}  // namespace heat
