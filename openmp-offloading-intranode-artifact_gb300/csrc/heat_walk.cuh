// Per-column "walks" shared by the single-grid kernels and the batched
// persistent kernel: each walks one (i, j) column of a grid over planes
// [kb, ke), z-neighbours held in registers, and writes the new values.  The
// same code runs alone and in a batch, so a grid's results do not depend on
// how it was launched.
//
// Integer-pipe evaluation of the default FP64 form (walk_int):
// GB300's FP64 pipe retires about 2 lane-operations per clock per SM, while
// its integer pipes retire 64 (logic, shifts, IMAD) to 128 (IADD) lane-ops
// per clock and run concurrently with it.  walk_int evaluates the update
//
//   u_new = uC + rhs + sum_f w_f (u_f - uC),   w_f = factor (kappa_a + kappa_b)
//
// (the reference's expression, OpenMP_Single_Source/heat3D_variable_coeff.c:
// 174-181, regrouped) in 64-bit fixed point and rounds once to FP64:
//
//   1. each FP64 value x = m 2^(e-1075) (m signed, |m| < 2^53; subnormals
//      decoded exactly) is aligned to the largest exponent E of the cell's
//      stencil:  A = (m << 9) >> (E - e),  so |A| < 2^62 and the unit of A is
//      2^(E-1084);
//   2. differences D_f = A_f - A_C are exact;
//   3. face weights are exact integer sums W_f = K_a + K_b of the per-point
//      K = round(factor kappa 2^64), computed once per context from an
//      error-free product, so sum_f w_f and the centre weight 1 - sum_f w_f
//      are represented exactly;
//   4. acc = A_C + A_rhs + sum_f D_f W_f / 2^64, each product's high word
//      formed from the three 32x32 partial products that reach it;
//   5. acc is rounded to nearest-even FP64.
// The truncations in steps 1 and 4 are below 2^-57 of the largest term, so
// the result is within 0.5 ulp (+ ~2^-56 relative) of the exact value of the
// update with these weights: as accurate as the reference's own FP64
// evaluation, and held to <= 1e-12 relative error against it.
//
// The representation needs |acc| < 2^63, which holds when every centre weight
// 1 - sum_f w_f is >= 0 (the explicit scheme's stability condition) and each
// factor*kappa < 1/4.  k_kq_setup checks both; contexts that fail it use the
// FP64-pipe kernel alone.  Infinite or NaN inputs in a stencil take a
// per-point FP64 path.

#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace heat {
namespace walk {
namespace {

typedef unsigned long long u64;
typedef long long i64;

// ---- bit-exact FP64 (reference operation order, every operation rounded) ----
__device__ __forceinline__ double flux(double ksum, double ub, double ua) {
  return __dmul_rn(ksum, __dsub_rn(ub, ua));
}

// base is u + rhs (or u alone when the problem has no source term: u + 0.0
// equals u for every value but -0.0, which these fields never hold).
__device__ __forceinline__ double combine(double base, double factor, double A, double B,
                                          double C, double D, double E, double F) {
  double s = __dsub_rn(__dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(A, B), C), D), E), F);
  return __dadd_rn(base, __dmul_rn(factor, s));
}

template <bool RHS>
__device__ __forceinline__ void walk_exact_faces(double *__restrict__ un,
                                                 const double *__restrict__ u,
                                                 const double *__restrict__ rhs,
                                                 const double *__restrict__ kx,
                                                 const double *__restrict__ ky,
                                                 const double *__restrict__ kz, int P,
                                                 size_t S, size_t c, int kb, int ke,
                                                 double factor) {
  double uc = u[c];
  double F = flux(kz[c - S], uc, u[c - S]);
  for (int k = kb; k < ke; ++k, c += S) {
    double uu = u[c + S];
    double A = flux(kx[c], u[c + 1], uc);
    double B = flux(kx[c - 1], uc, u[c - 1]);
    double C = flux(ky[c], u[c + P], uc);
    double D = flux(ky[c - P], uc, u[c - P]);
    double E = flux(kz[c], uu, uc);
    un[c] = combine(RHS ? __dadd_rn(uc, rhs[c]) : uc, factor, A, B, C, D, E, F);
    F = E;
    uc = uu;
  }
}

// ---- default FP64 form: integer pipes and FP64 pipe ----
struct Dec {
  int e;    // biased exponent, subnormals and zero mapped to 1
  i64 m9;   // signed significand << 9  (|m9| < 2^62)
};

__device__ __forceinline__ Dec decode(u64 b) {
  Dec d;
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  int ex = (int)((hi >> 20) & 0x7ffu);
  const unsigned mh = (hi & 0xfffffu) | (ex ? 0x100000u : 0u);
  d.e = max(ex, 1);
  const u64 mag9 = ((((u64)mh) << 32) | lo) << 9;
  d.m9 = ((int)hi < 0) ? -(i64)mag9 : (i64)mag9;
  return d;
}

__device__ __forceinline__ i64 align(const Dec &d, int E) {
  return d.m9 >> min(E - d.e, 63);
}

// acc += floor-ish(Dp * W / 2^64) for unsigned Dp, W < 2^63: the three
// partial products that reach the high word (d1 w1, hi(d1 w0), hi(d0 w1));
// the dropped terms are below 3 units of acc.
__device__ __forceinline__ void mac_hi(u64 &acc, u64 Dp, u64 W) {
  unsigned alo = (unsigned)acc, ahi = (unsigned)(acc >> 32);
  const unsigned d0 = (unsigned)Dp, d1 = (unsigned)(Dp >> 32);
  const unsigned w0 = (unsigned)W, w1 = (unsigned)(W >> 32);
  asm("mad.lo.cc.u32 %0, %2, %4, %0;\n\t"
      "madc.hi.u32   %1, %2, %4, %1;\n\t"
      "mad.hi.cc.u32 %0, %2, %5, %0;\n\t"
      "addc.u32      %1, %1, 0;\n\t"
      "mad.hi.cc.u32 %0, %3, %4, %0;\n\t"
      "addc.u32      %1, %1, 0;"
      : "+r"(alo), "+r"(ahi)
      : "r"(d1), "r"(d0), "r"(w1), "r"(w0));
  acc = ((u64)ahi << 32) | alo;
}

// Round acc * 2^(E-1084) to the nearest FP64 value (ties to even).
__device__ __forceinline__ double encode(i64 acc, int E) {
  if (acc == 0) return 0.0;
  const u64 s = acc < 0 ? 0x8000000000000000ull : 0ull;
  const u64 mag = acc < 0 ? (u64)(-acc) : (u64)acc;
  const int lz = __clzll((i64)mag);
  const u64 norm = mag << lz;
  const int be = E + 2 - lz;
  if (be >= 1 && be < 2047) {
    const u64 mant = norm >> 11, rem = norm & 0x7ffull;
    const u64 up = (rem > 0x400ull) | ((rem == 0x400ull) & (mant & 1ull));
    return __longlong_as_double((i64)(s | ((((u64)(be - 1)) << 52) + mant + up)));
  }
  return ldexp((double)acc, E - 1084);  // subnormal or overflowing result
}

__device__ __noinline__ double slow_point(double uc, double ue, double uw, double un, double us,
                                          double uu, double ud, double r, u64 Kc, u64 Ke,
                                          u64 Kw, u64 Kn, u64 Ks, u64 Ku, u64 Kd) {
  const double s = 0x1p-64;
  double acc = uc + r;
  acc += (double)(Kc + Ke) * s * (ue - uc);
  acc += (double)(Kc + Kw) * s * (uw - uc);
  acc += (double)(Kc + Kn) * s * (un - uc);
  acc += (double)(Kc + Ks) * s * (us - uc);
  acc += (double)(Kc + Ku) * s * (uu - uc);
  acc += (double)(Kc + Kd) * s * (ud - uc);
  return acc;
}

constexpr u64 kSign = 0x8000000000000000ull;

// Raw bits of a point's stencil, for the per-point FP64 path that inputs
// with infinities or NaNs take.
struct Raw7 {
  u64 c, e, w, n, s, u, d;
};

// One point of the integer-pipe evaluation from its decoded stencil and the
// fixed-point weights K of the point and its six neighbours; br is the bits
// of the source term (RHS only).  raw() yields the stencil's raw bits, read
// only on the per-point FP64 path.
template <bool RHS, class RawFn>
__device__ __forceinline__ double int_point(const Dec &dc, const Dec &du, const Dec &dd,
                                            const Dec &de, const Dec &dw, const Dec &dn,
                                            const Dec &ds, u64 Kc, u64 Ku, u64 Kd, u64 Ke,
                                            u64 Kw, u64 Kn, u64 Ks, u64 br, RawFn raw) {
  int E = max(max(max(dc.e, du.e), max(dd.e, de.e)), max(max(dw.e, dn.e), ds.e));
  Dec dr;
  if (RHS) {
    dr = decode(br);
    E = max(E, dr.e);
  }
  if (E < 2047) {
    const i64 Ac = align(dc, E);
    const u64 We = Kc + Ke, Ww = Kc + Kw, Wn = Kc + Kn, Ws = Kc + Ks, Wu = Kc + Ku, Wd = Kc + Kd;
    // Each product is taken of D + 2^63 (D = A_f - A_C, |D| < 2^63) so it is
    // unsigned; the offsets sum to (sum_f W_f) / 2, removed up front.  (+ 2^63
    // is the same as ^ 2^63 modulo 2^64, and folds into the subtraction.)
    u64 acc = (u64)Ac - ((We + Ww + Wn + Ws + Wu + Wd) >> 1);
    mac_hi(acc, (u64)(align(de, E) - Ac) + kSign, We);
    mac_hi(acc, (u64)(align(dw, E) - Ac) + kSign, Ww);
    mac_hi(acc, (u64)(align(dn, E) - Ac) + kSign, Wn);
    mac_hi(acc, (u64)(align(ds, E) - Ac) + kSign, Ws);
    mac_hi(acc, (u64)(align(du, E) - Ac) + kSign, Wu);
    mac_hi(acc, (u64)(align(dd, E) - Ac) + kSign, Wd);
    if (RHS) acc += (u64)align(dr, E);
    return encode((i64)acc, E);
  }
  const Raw7 r = raw();
  return slow_point(__longlong_as_double(r.c), __longlong_as_double(r.e),
                    __longlong_as_double(r.w), __longlong_as_double(r.n),
                    __longlong_as_double(r.s), __longlong_as_double(r.u),
                    __longlong_as_double(r.d), RHS ? __longlong_as_double(br) : 0.0, Kc, Ke, Kw,
                    Kn, Ks, Ku, Kd);
}

// Column state of the integer-pipe walk: one (i, j) column, advanced one
// plane per step(); the next plane's loads are issued one step ahead.
template <bool RHS>
struct IntCol {
  size_t c;
  u64 bd, bc, Kd, Kc;
  Dec dd, dc;
  u64 nu, ne, nw, nn, ns, mu, me, mw, mn, ms;

  __device__ __forceinline__ void fetch(const u64 *__restrict__ ub, const u64 *__restrict__ K,
                                        int P, size_t S, size_t q) {
    nu = ub[q + S]; ne = ub[q + 1]; nw = ub[q - 1]; nn = ub[q + P]; ns = ub[q - P];
    mu = K[q + S]; me = K[q + 1]; mw = K[q - 1]; mn = K[q + P]; ms = K[q - P];
  }

  __device__ __forceinline__ void start(const u64 *__restrict__ ub, const u64 *__restrict__ K,
                                        int P, size_t S, size_t c_) {
    c = c_;
    bd = ub[c - S];
    bc = ub[c];
    dd = decode(bd);
    dc = decode(bc);
    Kd = K[c - S];
    Kc = K[c];
    fetch(ub, K, P, S, c);
  }

  // Writes the new value of plane c and moves to the next plane; `more`
  // says whether a next plane follows (its loads are issued now).
  __device__ __forceinline__ void step(double *__restrict__ un, const u64 *__restrict__ ub,
                                       const double *__restrict__ rhs,
                                       const u64 *__restrict__ K, int P, size_t S, bool more) {
    const u64 bu = nu, be = ne, bw = nw, bn = nn, bs = ns;
    const u64 Ku = mu, Ke = me, Kw = mw, Kn = mn, Ks = ms;
    if (more) fetch(ub, K, P, S, c + S);
    const Dec du = decode(bu), de = decode(be), dw = decode(bw), dn = decode(bn), ds = decode(bs);
    const u64 br = RHS ? (u64)__double_as_longlong(rhs[c]) : 0ull;
    const u64 bcc = bc, bdd = bd;
    un[c] = int_point<RHS>(dc, du, dd, de, dw, dn, ds, Kc, Ku, Kd, Ke, Kw, Kn, Ks, br,
                                [=] { return Raw7{bcc, be, bw, bn, bs, bu, bdd}; });
    bd = bc;
    bc = bu;
    dd = dc;
    dc = du;
    Kd = Kc;
    Kc = Ku;
    c += S;
  }
};

// The integer-pipe walk over one (i, j) column, planes [kb, ke).
template <bool RHS>
__device__ __forceinline__ void walk_int(double *__restrict__ un, const u64 *__restrict__ ub,
                                         const double *__restrict__ rhs,
                                         const u64 *__restrict__ K, int P, size_t S,
                                         size_t c, int kb, int ke) {
  IntCol<RHS> col;
  col.start(ub, K, P, S, c);
  for (int k = kb; k < ke; ++k) col.step(un, ub, rhs, K, P, S, k + 1 < ke);
}

// Column state of the FP64-pipe walk (precomputed double weights, 7 FMA per
// point).  The plane's loads are issued one step ahead: next to the integer
// warps of the hybrid launch these warps are few, and would otherwise wait
// on memory instead of keeping the FP64 pipe busy.
template <bool RHS>
struct HwCol {
  size_t c;
  double ud, uc, wd;
  double nu, nwu, nc0, nr, nxe, nxw, nyn, nys, ne, nw, nn, ns;

  __device__ __forceinline__ void fetch(const double *__restrict__ u,
                                        const double *__restrict__ rhs,
                                        const double *__restrict__ c0,
                                        const double *__restrict__ cx,
                                        const double *__restrict__ cy,
                                        const double *__restrict__ cz, int P, size_t S,
                                        size_t q) {
    nu = u[q + S];
    nwu = cz[q];
    nc0 = c0[q];
    nr = RHS ? rhs[q] : 0.0;
    nxe = cx[q];
    nxw = cx[q - 1];
    nyn = cy[q];
    nys = cy[q - P];
    ne = u[q + 1];
    nw = u[q - 1];
    nn = u[q + P];
    ns = u[q - P];
  }

  __device__ __forceinline__ void start(const double *__restrict__ u,
                                        const double *__restrict__ rhs,
                                        const double *__restrict__ c0,
                                        const double *__restrict__ cx,
                                        const double *__restrict__ cy,
                                        const double *__restrict__ cz, int P, size_t S,
                                        size_t c_) {
    c = c_;
    ud = u[c - S];
    uc = u[c];
    wd = cz[c - S];
    fetch(u, rhs, c0, cx, cy, cz, P, S, c);
  }

  __device__ __forceinline__ void step(double *__restrict__ un, const double *__restrict__ u,
                                       const double *__restrict__ rhs,
                                       const double *__restrict__ c0,
                                       const double *__restrict__ cx,
                                       const double *__restrict__ cy,
                                       const double *__restrict__ cz, int P, size_t S,
                                       bool more) {
    const double uu = nu, wu = nwu, w0 = nc0, r = nr, xe = nxe, xw = nxw, yn = nyn, ys = nys;
    const double ue = ne, uw = nw, un_ = nn, us = ns;
    if (more) fetch(u, rhs, c0, cx, cy, cz, P, S, c + S);
    double acc = RHS ? fma(w0, uc, r) : w0 * uc;
    acc = fma(xe, ue, acc);
    acc = fma(xw, uw, acc);
    acc = fma(yn, un_, acc);
    acc = fma(ys, us, acc);
    acc = fma(wu, uu, acc);
    acc = fma(wd, ud, acc);
    un[c] = acc;
    ud = uc;
    uc = uu;
    wd = wu;
    c += S;
  }
};

// The FP64-pipe walk over one (i, j) column, planes [kb, ke); the plane loop
// unrolled UNROLL times.
template <bool RHS, int UNROLL = 1>
__device__ __forceinline__ void walk_hw(double *__restrict__ un, const double *__restrict__ u,
                                        const double *__restrict__ rhs,
                                        const double *__restrict__ c0,
                                        const double *__restrict__ cx,
                                        const double *__restrict__ cy,
                                        const double *__restrict__ cz, int P, size_t S,
                                        size_t c, int kb, int ke) {
  HwCol<RHS> col;
  col.start(u, rhs, c0, cx, cy, cz, P, S, c);
  // Unrolled by 2, the prefetch registers alternate instead of being copied
  // into the working ones each plane: k_fast_ws without a source term asks
  // for it (512^3: 114 GLUP/s against 111.5; by 3 or 4 no gain).  The batch
  // kernels do not: there it adds spills (k_batch_ws 288 B against 184).
#pragma unroll (UNROLL)
  for (int k = kb; k < ke; ++k) col.step(un, u, rhs, c0, cx, cy, cz, P, S, k + 1 < ke);
}

// ---- FP32-compensated form ----
__device__ __forceinline__ float bf2f(uint16_t b) {
  return __uint_as_float(((unsigned)b) << 16);
}
__device__ __forceinline__ uint16_t f2bf(float x) {
  __nv_bfloat16 h = __float2bfloat16_rn(x);
  return *reinterpret_cast<uint16_t *>(&h);
}

template <bool RHS>
__device__ __forceinline__ void walk_fp32c(float *__restrict__ vn, uint16_t *__restrict__ cn,
                                           const float *__restrict__ v,
                                           const uint16_t *__restrict__ cr,
                                           const float *__restrict__ wx,
                                           const float *__restrict__ wy,
                                           const float *__restrict__ wz,
                                           const float *__restrict__ rhs, int P, size_t S,
                                           size_t c, int kb, int ke) {
  float vd = v[c - S], vc = v[c];
  float wd = wz[c - S];
  // The plane's loads are issued one iteration ahead (the walk is bound by
  // memory latency, not arithmetic).
  float nu = v[c + S], nwz = wz[c], ne = v[c + 1], nw = v[c - 1], nn = v[c + P], ns = v[c - P];
  float nwx = wx[c], nwxm = wx[c - 1], nwy = wy[c], nwym = wy[c - P];
  uint16_t ncr = cr[c];
  float nr = RHS ? rhs[c] : 0.0f;
  for (int k = kb; k < ke; ++k, c += S) {
    const float vu = nu, wu = nwz, ve = ne, vw = nw, vn_ = nn, vs = ns;
    const float w_e = nwx, w_w = nwxm, w_n = nwy, w_s = nwym, r = nr;
    const uint16_t cc0 = ncr;
    if (k + 1 < ke) {
      const size_t q = c + S;
      nu = v[q + S];
      nwz = wz[q];
      ne = v[q + 1];
      nw = v[q - 1];
      nn = v[q + P];
      ns = v[q - P];
      nwx = wx[q];
      nwxm = wx[q - 1];
      nwy = wy[q];
      nwym = wy[q - P];
      ncr = cr[q];
      if (RHS) nr = rhs[q];
    }
    float d = r;
    d = fmaf(w_e, ve - vc, d);
    d = fmaf(w_w, vw - vc, d);
    d = fmaf(w_n, vn_ - vc, d);
    d = fmaf(w_s, vs - vc, d);
    d = fmaf(wu, vu - vc, d);
    d = fmaf(wd, vd - vc, d);
    const float y = __fsub_rn(d, bf2f(cc0));
    const float t = __fadd_rn(vc, y);
    const float cc = __fsub_rn(__fsub_rn(t, vc), y);
    vn[c] = t;
    cn[c] = f2bf(cc);
    vd = vc;
    vc = vu;
    wd = wu;
  }
}

}  // namespace
}  // namespace walk
}  // namespace heat
