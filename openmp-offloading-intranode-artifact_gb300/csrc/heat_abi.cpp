// extern "C" solver ABI (include/heat.h): context lifetime, field transfer,
// the time loop and the drop-in heat_update().  Host code only; the kernels
// live in the heat_*.cu translation units.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>

#include "heat_diag.h"
#include "heat_internal.h"

namespace {

thread_local char g_last_error[256] = "";

// Warps (of 8 per block) of the hybrid FP64 kernel that run on the FP64 pipe;
// the others run the integer-pipe evaluation.
constexpr int kDefaultHwRows = 4;

using heat::check_err;
using heat::cuda_fail;
using heat::two_step_form;

#define CK(call)                                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

bool geom_ok(int nx, int ny, int nz) {
  if (nx < 3 || ny < 3 || nz < 3) return false;
  // Rows, planes and fields must be indexable with the kernels' int / size_t
  // arithmetic: keep each axis and the row count within int range.
  if ((long long)ny * nz > 0x7fffffffLL) return false;
  if (nx > (1 << 28)) return false;
  return true;
}

// Row pitch: a multiple of 4 points (32-byte FP64 rows); FP32C fields use a
// multiple of 8 so BF16 carry rows are multiples of 16 bytes for TMA.
heat_geom make_geom(int nx, int ny, int nz, int align = 4) {
  heat_geom g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.pitch = (nx + align - 1) / align * align;
  g.plane = (size_t)g.pitch * ny;
  g.elems = g.plane * nz;
  return g;
}

// Device memory of contexts comes from one stream-ordered pool per device, so
// creating and destroying contexts (the server does so continuously) never
// calls cudaMalloc/cudaFree, whose device-wide synchronisation would stall
// every other stream.  Freed blocks stay cached up to a quarter of the device
// memory for reuse.
cudaMemPool_t device_pool(int dev) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    uint64_t keep = total_b / 4;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    cudaGetLastError();
    pools[dev] = pool;
  }
  return pools[dev];
}

template <class T>
int dalloc(T **p, size_t count, cudaStream_t st) {
  *p = nullptr;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaMemPool_t pool = device_pool(dev);
  cudaError_t e = pool ? cudaMallocFromPoolAsync((void **)p, count * sizeof(T), pool, st)
                       : cudaMalloc((void **)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    std::snprintf(g_last_error, sizeof g_last_error, "cudaMalloc of %zu bytes: %s",
                  count * sizeof(T), cudaGetErrorString(e));
    return HEAT_ENOMEM;
  }
  return HEAT_OK;
}

// Copy a dense host k-j-i array into the pitched device layout (one
// contiguous copy when the rows carry no padding).
int upload(double *dst, const double *src, const heat_geom &g, cudaStream_t st) {
  if (g.pitch == g.nx) {
    CK(cudaMemcpyAsync(dst, src, g.elems * sizeof(double), cudaMemcpyHostToDevice, st));
    return HEAT_OK;
  }
  CK(cudaMemcpy2DAsync(dst, (size_t)g.pitch * sizeof(double), src, (size_t)g.nx * sizeof(double),
                       (size_t)g.nx * sizeof(double), (size_t)g.ny * g.nz,
                       cudaMemcpyHostToDevice, st));
  return HEAT_OK;
}

int download(double *dst, const double *src, const heat_geom &g, cudaStream_t st) {
  if (g.pitch == g.nx) {
    CK(cudaMemcpyAsync(dst, src, g.elems * sizeof(double), cudaMemcpyDeviceToHost, st));
    return HEAT_OK;
  }
  CK(cudaMemcpy2DAsync(dst, (size_t)g.nx * sizeof(double), src, (size_t)g.pitch * sizeof(double),
                       (size_t)g.nx * sizeof(double), (size_t)g.ny * g.nz,
                       cudaMemcpyDeviceToHost, st));
  return HEAT_OK;
}

void free_ctx(heat_ctx *c) {
  if (!c) return;
  void *ptrs[] = {c->u[0],   c->u[1],     c->rhs,      c->kappa,    c->ks[0],   c->ks[1],
                  c->ks[2],  c->c0,       c->cf[0],    c->cf[1],    c->cf[2],   c->kq,
                  c->v[0],   c->v[1],     c->carry[0], c->carry[1], c->fcf[0],  c->fcf[1],
                  c->fcf[2], c->frhs,     c->partials, c->err};
  for (void *p : ptrs)
    if (p) cudaFreeAsync(p, c->stream);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

// One step of context c from buffer `cur` into buffer cur ^ 1 on stream st,
// with the kernel its form selects; the context's bookkeeping is untouched.
cudaError_t enqueue_one(heat_ctx *c, int cur, cudaStream_t st) {
  const heat_geom &g = c->g;
  double *uo = c->u[cur], *un = c->u[cur ^ 1];
  if (c->precision == HEAT_FP32C)
    return heat::launch_fp32c(c->v[cur ^ 1], c->carry[cur ^ 1], c->v[cur], c->carry[cur], c->fcf,
                              c->frhs, g, st);
  if (c->flags & HEAT_NAIVE) return heat::launch_naive(un, uo, c->rhs, c->kappa, g, c->factor, st);
  if (c->flags & HEAT_BITEXACT)
    return heat::launch_exact_faces(un, uo, c->rhs, c->ks, g, c->factor, st);
  if (c->kq)
    return heat::launch_fast_mix(un, uo, c->rhs, c->kq, c->c0, c->cf, g, c->hw_rows, c->err, st);
  return heat::launch_fast(un, uo, c->rhs, c->c0, c->cf, g, st);
}

int launch_step(heat_ctx *c) {
  cudaError_t e = enqueue_one(c, c->cur, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
  c->launches += 1;
  c->cur ^= 1;
  c->steps_done += 1;
  return HEAT_OK;
}

int widen_current(heat_ctx *c, double **out) {
  int rc = dalloc(out, c->g.elems, c->stream);
  if (rc != HEAT_OK) return rc;
  cudaError_t e = heat::launch_widen(*out, c->v[c->cur], c->carry[c->cur], c->g.elems, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "widen");
  c->launches += 1;
  return HEAT_OK;
}

// Upload a host FP64 field through tmp (device, g.elems doubles) into both
// FP32C state buffers.
int load_split(heat_ctx *c, double *tmp, const double *u_host) {
  const heat_geom &g = c->g;
  CK(cudaMemsetAsync(tmp, 0, g.elems * sizeof(double), c->stream));
  int rc = upload(tmp, u_host, g, c->stream);
  if (rc != HEAT_OK) return rc;
  cudaError_t e = heat::launch_split(c->v[0], c->carry[0], tmp, g.elems, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "split");
  c->launches += 1;
  CK(cudaMemcpyAsync(c->v[1], c->v[0], g.elems * sizeof(float), cudaMemcpyDeviceToDevice,
                     c->stream));
  CK(cudaMemcpyAsync(c->carry[1], c->carry[0], g.elems * sizeof(uint16_t),
                     cudaMemcpyDeviceToDevice, c->stream));
  return HEAT_OK;
}

// A second stream for a context's set-up: work enqueued on it starts after
// everything already on the context's stream, and join() makes the context's
// stream wait for it.  Released (after its work completes) on every return.
struct SideStream {
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;

  bool begin(cudaStream_t main) {
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(ev, main) != cudaSuccess || cudaStreamWaitEvent(s, ev, 0) != cudaSuccess) {
      cudaGetLastError();
      release();
      return false;
    }
    return true;
  }
  cudaError_t join(cudaStream_t main) {
    cudaError_t e = cudaEventRecord(ev, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(main, ev, 0);
    return e;
  }
  void release() {
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
      s = nullptr;
    }
    if (ev) {
      cudaEventDestroy(ev);
      ev = nullptr;
    }
  }
  ~SideStream() { release(); }
};

// Fields of at least this many bytes upload u0 on a side stream, overlapping
// the kappa upload and the weight set-up kernels.
constexpr size_t kSideUploadBytes = 64u << 20;

int init_fp64(heat_ctx *c, const heat_desc *d) {
  const heat_geom &g = c->g;
  const size_t bytes = g.elems * sizeof(double);
  int rc = HEAT_OK;
  double *kap = nullptr;  // raw kappa on the device (kept only for the naive kernel)
  SideStream side;
  bool split = false;
  cudaStream_t ust = c->stream;  // stream of the u0 upload
#define TRY(x)                    \
  do {                            \
    rc = (x);                     \
    if (rc != HEAT_OK) goto done; \
  } while (0)
  TRY(dalloc(&c->u[0], g.elems, c->stream));
  TRY(dalloc(&c->u[1], g.elems, c->stream));
  TRY(dalloc(&kap, g.elems, c->stream));
  TRY(dalloc(&c->partials, 2 * heat::kNormBlocks + 2, c->stream));
  c->n_partials = heat::kNormBlocks;
  TRY(dalloc(&c->err, 1, c->stream));
  // Padding columns are zeroed; without padding the uploads cover everything.
  if (cudaMemsetAsync(c->err, 0, sizeof(int), c->stream) != cudaSuccess ||
      (g.pitch != g.nx && (cudaMemsetAsync(c->u[0], 0, bytes, c->stream) != cudaSuccess ||
                           cudaMemsetAsync(kap, 0, bytes, c->stream) != cudaSuccess))) {
    rc = cuda_fail(cudaGetLastError(), "cudaMemset");
    goto done;
  }
  // kappa first: the weight set-up kernels need it, and u0 (and the source
  // term) then upload on the side stream while they run.
  if (d->rhs) TRY(dalloc(&c->rhs, g.elems, c->stream));
  if (d->rhs && g.pitch != g.nx && cudaMemsetAsync(c->rhs, 0, bytes, c->stream) != cudaSuccess) {
    rc = cuda_fail(cudaGetLastError(), "cudaMemset");
    goto done;
  }
  TRY(upload(kap, d->kappa, g, c->stream));
  split = bytes >= kSideUploadBytes && side.begin(c->stream);
  if (split) ust = side.s;
  TRY(upload(c->u[0], d->u0, g, ust));
  // u_new starts as a copy of u0, so its boundary holds the same values
  // (the reference seeds both buffers from u0, 1-cuda.cu:219-222).
  if (cudaMemcpyAsync(c->u[1], c->u[0], bytes, cudaMemcpyDeviceToDevice, ust) != cudaSuccess) {
    rc = cuda_fail(cudaGetLastError(), "cudaMemcpy u0");
    goto done;
  }
  if (d->rhs) TRY(upload(c->rhs, d->rhs, g, ust));
  if (c->flags & HEAT_NAIVE) {
    c->kappa = kap;
    kap = nullptr;
  } else if (c->flags & HEAT_BITEXACT) {
    for (int a = 0; a < 3; ++a) TRY(dalloc(&c->ks[a], g.elems, c->stream));
    {
      cudaError_t e = heat::launch_face_sums(c->ks, kap, g, c->stream);
      if (e != cudaSuccess) { rc = cuda_fail(e, "face sums"); goto done; }
      c->launches += 1;
    }
  } else {
    bool use_int = !(c->flags & HEAT_HWFP64);
    c->hw_rows = kDefaultHwRows;
    if (const char *ev = std::getenv("HEAT_HW_ROWS")) {  // tuning knob, 0..8
      int v = std::atoi(ev);
      if (v >= 0 && v <= 8) c->hw_rows = v;
    }
    if (c->hw_rows == 8) use_int = false;
    // Both weight sets (the hybrid's two kinds of rows) come from one fused
    // pass; HEAT_SETUP_SPLIT=1 runs the two separate kernels instead (same
    // values; for comparison).
    const char *sp = std::getenv("HEAT_SETUP_SPLIT");
    const bool fused = use_int && c->hw_rows > 0 && !(sp && sp[0] == '1') &&
                       g.ny <= 65535;  // one grid row of blocks per grid row j
    if (fused) {
      TRY(dalloc(&c->c0, g.elems, c->stream));
      for (int a = 0; a < 3; ++a) TRY(dalloc(&c->cf[a], g.elems, c->stream));
    }
    if (use_int) {
      // Integer-pipe form: per-point fixed-point factor*kappa.  Falls back to
      // the FP64-pipe kernel when the fixed-point range check fails.
      TRY(dalloc(&c->kq, g.elems, c->stream));
      int bad = 0;
      int *d_bad = reinterpret_cast<int *>(c->partials);
      cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(int), c->stream);
      if (e == cudaSuccess)
        e = fused ? heat::launch_weights_setup(c->kq, c->c0, c->cf, d_bad, kap, g, c->factor,
                                               c->stream)
                  : heat::launch_kq_setup(c->kq, d_bad, kap, g, c->factor, c->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) { rc = cuda_fail(e, "fixed-point setup"); goto done; }
      c->launches += 1;
      if (bad) {
        cudaFreeAsync(c->kq, c->stream);
        c->kq = nullptr;
        use_int = false;
      }
    }
    if (!fused && (!use_int || c->hw_rows > 0)) {
      TRY(dalloc(&c->c0, g.elems, c->stream));
      for (int a = 0; a < 3; ++a) TRY(dalloc(&c->cf[a], g.elems, c->stream));
      cudaError_t e = heat::launch_fast_coeffs(c->c0, c->cf, kap, g, c->factor, c->stream);
      if (e != cudaSuccess) { rc = cuda_fail(e, "coefficients"); goto done; }
      c->launches += 1;
    }
  }
  if (split && side.join(c->stream) != cudaSuccess) {
    rc = cuda_fail(cudaGetLastError(), "u0 upload join");
    goto done;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess)
    rc = cuda_fail(cudaGetLastError(), "heat_init sync");
done:
  side.release();
  if (kap) cudaFreeAsync(kap, c->stream);
  return rc;
#undef TRY
}

int init_fp32c(heat_ctx *c, const heat_desc *d) {
  const heat_geom &g = c->g;
  int rc = HEAT_OK;
  double *tmp = nullptr;  // FP64 staging buffer for u0, kappa and rhs
  cudaError_t e = cudaSuccess;
#define TRY(x)                    \
  do {                            \
    rc = (x);                     \
    if (rc != HEAT_OK) goto done; \
  } while (0)
  for (int b = 0; b < 2; ++b) {
    TRY(dalloc(&c->v[b], g.elems, c->stream));
    TRY(dalloc(&c->carry[b], g.elems, c->stream));
  }
  for (int a = 0; a < 3; ++a) TRY(dalloc(&c->fcf[a], g.elems, c->stream));
  TRY(dalloc(&c->partials, 2 * heat::kNormBlocks + 2, c->stream));
  c->n_partials = heat::kNormBlocks;
  TRY(dalloc(&c->err, 1, c->stream));
  if (cudaMemsetAsync(c->err, 0, sizeof(int), c->stream) != cudaSuccess) {
    rc = cuda_fail(cudaGetLastError(), "cudaMemset");
    goto done;
  }
  TRY(dalloc(&tmp, g.elems, c->stream));
  TRY(load_split(c, tmp, d->u0));
  if (cudaMemsetAsync(tmp, 0, g.elems * sizeof(double), c->stream) != cudaSuccess) {
    rc = cuda_fail(cudaGetLastError(), "cudaMemset");
    goto done;
  }
  TRY(upload(tmp, d->kappa, g, c->stream));
  e = heat::launch_f32_weights(c->fcf, tmp, g, c->factor, c->stream);
  if (e != cudaSuccess) { rc = cuda_fail(e, "FP32 weights"); goto done; }
  c->launches += 1;
  if (d->rhs) {
    TRY(dalloc(&c->frhs, g.elems, c->stream));
    if (cudaMemsetAsync(tmp, 0, g.elems * sizeof(double), c->stream) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "cudaMemset");
      goto done;
    }
    TRY(upload(tmp, d->rhs, g, c->stream));
    e = heat::launch_to_f32(c->frhs, tmp, g.elems, c->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "FP32 rhs"); goto done; }
    c->launches += 1;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess)
    rc = cuda_fail(cudaGetLastError(), "heat_init sync");
done:
  if (tmp) cudaFreeAsync(tmp, c->stream);
  return rc;
#undef TRY
}

}  // namespace

namespace heat {

long resident_blocks(const void *kernel, int threads, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) !=
          cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (long)per_sm * sms;
}

int cuda_fail(cudaError_t e, const char *what) {
  std::snprintf(g_last_error, sizeof g_last_error, "%s: %s", what, cudaGetErrorString(e));
  return HEAT_ECUDA;
}

bool two_step_form(const heat_ctx *c) {
  return c->precision == HEAT_FP32C && !c->frhs && !(c->flags & HEAT_NO_TEMPORAL) &&
         fp32c_tb2_ok(c->g);
}

int check_err(heat_ctx *c) {
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, c->err, sizeof flag, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (flag) {
    CK(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return HEAT_ETIMEOUT;
  }
  return HEAT_OK;
}

cudaError_t enqueue_ctx_steps(heat_ctx *c, int cur, long long n, cudaStream_t st,
                              long long *launches) {
  long long s = 0;
  cudaError_t e = cudaSuccess;
  if (two_step_form(c))
    for (; s + 2 <= n && e == cudaSuccess; s += 2) {
      // two steps per launch: the result lands in the other buffer
      e = launch_fp32c_tb2(c->v[cur ^ 1], c->carry[cur ^ 1], c->v[cur], c->carry[cur], c->fcf, c->g,
                           c->err, st);
      cur ^= 1;
      if (launches) ++*launches;
    }
  for (; s < n && e == cudaSuccess; ++s) {
    e = enqueue_one(c, cur, st);
    cur ^= 1;
    if (launches) ++*launches;
  }
  return e;
}

cudaError_t enqueue_one_step(heat_ctx *c, int cur, cudaStream_t st, long long *launches) {
  if (launches) ++*launches;
  return enqueue_one(c, cur, st);
}

int ctx_flips(const heat_ctx *c, long long n) {
  return (int)((two_step_form(c) ? n / 2 + n % 2 : n) & 1);
}

}  // namespace heat

extern "C" {

const char *heat_strerror(int status) {
  switch (status) {
    case HEAT_OK: return "ok";
    case HEAT_EINVAL: return "invalid argument";
    case HEAT_ENOMEM: return g_last_error[0] ? g_last_error : "out of memory";
    case HEAT_ECUDA: return g_last_error[0] ? g_last_error : "CUDA error";
    case HEAT_ETIMEOUT: return "device-side wait timed out";
    case HEAT_EBUDGET: return "request exceeds the HBM budget";
    case HEAT_ENODEV: return "no usable CUDA device";
    case HEAT_ESTATE: return "call not valid in this state";
    default: return "unknown status";
  }
}

int heat_init(heat_ctx **out, const heat_desc *d) {
  if (!out) return HEAT_EINVAL;
  *out = nullptr;
  if (!d || !d->kappa || !d->u0) return HEAT_EINVAL;
  if (!geom_ok(d->nx, d->ny, d->nz)) return HEAT_EINVAL;
  if (!(d->h > 0.0) || !(d->dt > 0.0) || !std::isfinite(d->h) || !std::isfinite(d->dt))
    return HEAT_EINVAL;
  if (d->precision != HEAT_FP64 && d->precision != HEAT_FP32C) return HEAT_EINVAL;
  if (d->precision == HEAT_FP32C && (d->flags & (HEAT_BITEXACT | HEAT_NAIVE)))
    return HEAT_EINVAL;

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return HEAT_ENODEV;
  }

  heat_ctx *c = new (std::nothrow) heat_ctx();
  if (!c) return HEAT_ENOMEM;
  c->g = make_geom(d->nx, d->ny, d->nz, d->precision == HEAT_FP32C ? 8 : 4);
  c->h = d->h;
  c->dt = d->dt;
  c->factor = d->dt / d->h / d->h / 2.0;  // as heat3D_variable_coeff.c:84
  c->precision = d->precision;
  c->flags = d->flags;
  cudaGetDevice(&c->device);
  if (d->stream) {
    c->stream = (cudaStream_t)d->stream;
    c->own_stream = false;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete c;
      return cuda_fail(e, "cudaStreamCreate");
    }
    c->own_stream = true;
  }
  int rc = (c->precision == HEAT_FP64) ? init_fp64(c, d) : init_fp32c(c, d);
  if (rc != HEAT_OK) {
    free_ctx(c);
    return rc;
  }
  *out = c;
  return HEAT_OK;
}

int heat_step(heat_ctx *c, int nsteps) {
  if (!c || nsteps < 0) return HEAT_EINVAL;
  int s = 0;
  if (two_step_form(c)) {
    // Two steps per launch; the result lands in the other buffer.
    for (; s + 2 <= nsteps; s += 2) {
      cudaError_t e = heat::launch_fp32c_tb2(c->v[c->cur ^ 1], c->carry[c->cur ^ 1], c->v[c->cur],
                                             c->carry[c->cur], c->fcf, c->g, c->err, c->stream);
      if (e != cudaSuccess) return cuda_fail(e, "two-step kernel launch");
      c->launches += 1;
      c->cur ^= 1;
      c->steps_done += 2;
    }
  }
  for (; s < nsteps; ++s) {
    int rc = launch_step(c);
    if (rc != HEAT_OK) return rc;
  }
  return HEAT_OK;
}

int heat_run(heat_ctx *c, double T, int *steps_out) {
  if (!c) return HEAT_EINVAL;
  // Replicate the reference's host accumulation exactly
  // (heat3D_variable_coeff.c:155-192): the count depends on the rounding of
  // the running sum, not on T/dt.
  double t = 0.0;
  long long steps = 0;
  while (t < T) {
    ++steps;
    t += c->dt;
    if (steps > 0x7fffffffLL) return HEAT_EINVAL;
  }
  int rc = heat_step(c, (int)steps);
  if (steps_out) *steps_out = (int)steps;
  return rc;
}

int heat_norm(heat_ctx *c, double *l2, double *checksum) {
  if (!c) return HEAT_EINVAL;
  cudaError_t e =
      (c->precision == HEAT_FP64)
          ? heat::launch_norm_f64(c->u[c->cur], c->g, c->partials, c->n_partials, c->stream)
          : heat::launch_norm_f32c(c->v[c->cur], c->carry[c->cur], c->g, c->partials,
                                   c->n_partials, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "norm launch");
  c->launches += 2;
  double r[2];
  CK(cudaMemcpyAsync(r, c->partials + 2 * c->n_partials, sizeof r, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (int rc = check_err(c)) return rc;
  if (checksum) *checksum = r[0];
  if (l2) *l2 = std::sqrt(r[1]);
  return HEAT_OK;
}

// The field is copied out even when a kernel's bounded wait ran out, but the
// call then returns HEAT_ETIMEOUT: the copy holds whatever that launch left.
int heat_get_field(heat_ctx *c, double *u_host) {
  if (!c || !u_host) return HEAT_EINVAL;
  if (c->precision == HEAT_FP64) {
    int rc = download(u_host, c->u[c->cur], c->g, c->stream);
    if (rc != HEAT_OK) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return check_err(c);
  }
  double *tmp = nullptr;
  int rc = widen_current(c, &tmp);
  if (rc == HEAT_OK) rc = download(u_host, tmp, c->g, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (tmp) cudaFreeAsync(tmp, c->stream);
  if (rc != HEAT_OK) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "heat_get_field");
  return check_err(c);
}

int heat_set_field(heat_ctx *c, const double *u_host) {
  if (!c || !u_host) return HEAT_EINVAL;
  // Both buffers take the new field so the boundary stays consistent in
  // whichever one the next step writes.
  if (c->precision == HEAT_FP64) {
    int rc = upload(c->u[c->cur], u_host, c->g, c->stream);
    if (rc != HEAT_OK) return rc;
    CK(cudaMemcpyAsync(c->u[c->cur ^ 1], c->u[c->cur], c->g.elems * sizeof(double),
                       cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return HEAT_OK;
  }
  double *tmp = nullptr;
  int rc = dalloc(&tmp, c->g.elems, c->stream);
  if (rc != HEAT_OK) return rc;
  rc = load_split(c, tmp, u_host);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  cudaFreeAsync(tmp, c->stream);
  if (rc != HEAT_OK) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "heat_set_field");
  return HEAT_OK;
}

int heat_sync(heat_ctx *c) {
  if (!c) return HEAT_EINVAL;
  CK(cudaStreamSynchronize(c->stream));
  return check_err(c);
}

int heat_stats(heat_ctx *c, long long *steps_done, long long *kernel_launches) {
  if (!c) return HEAT_EINVAL;
  if (steps_done) *steps_done = c->steps_done;
  if (kernel_launches) *kernel_launches = c->launches;
  return HEAT_OK;
}

int heat_destroy(heat_ctx *c) {
  if (!c) return HEAT_EINVAL;
  cudaStreamSynchronize(c->stream);
  free_ctx(c);
  return HEAT_OK;
}

int heat_update_async(double *u_new, const double *u_old, const double *rhs,
                      const double *kappa, int nz, int ny, int nx, double factor,
                      void *stream) {
  if (!u_new || !u_old || !kappa || u_new == u_old) return HEAT_EINVAL;
  if (!geom_ok(nx, ny, nz)) return HEAT_EINVAL;
  heat_geom g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.pitch = nx;  // the reference's dense layout, IDX() of 1-openmp.c:28-29
  g.plane = (size_t)nx * ny;
  g.elems = g.plane * nz;
  cudaError_t e = heat::launch_exact_raw(u_new, u_old, rhs, kappa, g, factor,
                                         (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "heat_update launch");
  return HEAT_OK;
}

int heat_update(double *u_new, const double *u_old, const double *rhs, const double *kappa,
                int nz, int ny, int nx, double factor, int device_id) {
  if (device_id >= 0) {
    int cur = -1;
    CK(cudaGetDevice(&cur));
    if (cur != device_id) CK(cudaSetDevice(device_id));
  }
  return heat_update_async(u_new, u_old, rhs, kappa, nz, ny, nx, factor, (void *)cudaStreamLegacy);
}

int heat_diag_fp32c_timeout(heat_ctx *c) {
  if (!c) return HEAT_EINVAL;
  if (!two_step_form(c)) return HEAT_ESTATE;
  // The product two-step kernel with a wait limit of 0 attempts: its first
  // wait gives up, it sets the context's error flag, drains its own loads in
  // flight (with the full bounded wait) and returns without writing a point.
  // The context's buffers and step count are left as they were.
  cudaError_t e = heat::launch_fp32c_tb2(c->v[c->cur ^ 1], c->carry[c->cur ^ 1], c->v[c->cur],
                                         c->carry[c->cur], c->fcf, c->g, c->err, c->stream, 0u);
  if (e != cudaSuccess) return cuda_fail(e, "two-step kernel launch");
  c->launches += 1;
  return HEAT_OK;
}

int heat_diag_fp64_timeout(heat_ctx *c) {
  if (!c) return HEAT_EINVAL;
  // Only contexts that step with the TMA-staged default FP64 launch.
  if (c->precision != HEAT_FP64 || !c->kq || c->hw_rows != 4 ||
      !heat::fast_tma_usable(c->g, c->rhs != nullptr))
    return HEAT_ESTATE;
  cudaError_t e = heat::launch_fast_tma(c->u[c->cur ^ 1], c->u[c->cur], c->kq, c->c0, c->cf,
                                        c->rhs, c->g, c->err, c->stream, 0u);
  if (e != cudaSuccess) return cuda_fail(e, "default FP64 kernel launch");
  c->launches += 1;
  return HEAT_OK;
}

int heat_diag_field_diff(heat_ctx *a, heat_ctx *b, double *max_abs, double *rel_l2) {
  if (!a || !b) return HEAT_EINVAL;
  if (a->g.nx != b->g.nx || a->g.ny != b->g.ny || a->g.nz != b->g.nz) return HEAT_EINVAL;
  CK(cudaStreamSynchronize(a->stream));
  CK(cudaStreamSynchronize(b->stream));
  double *fa = nullptr, *fb = nullptr, *part = nullptr, *ta = nullptr, *tb = nullptr;
  int rc = HEAT_OK;
  const int nb = heat::kNormBlocks;
  double r[3] = {0, 0, 0};
  cudaError_t e = cudaSuccess;
  if (a->precision == HEAT_FP64) fa = a->u[a->cur];
  else if ((rc = widen_current(a, &ta)) == HEAT_OK) fa = ta;
  if (rc == HEAT_OK) {
    if (b->precision == HEAT_FP64) fb = b->u[b->cur];
    else if ((rc = widen_current(b, &tb)) == HEAT_OK) fb = tb;
  }
  if (rc == HEAT_OK) rc = dalloc(&part, 3 * (size_t)nb + 3, (cudaStream_t)0);
  if (rc == HEAT_OK) {
    e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = heat::launch_diff_f64(fa, fb, a->g, part, nb, (cudaStream_t)0);
    if (e == cudaSuccess)
      e = cudaMemcpy(r, part + 3 * nb, sizeof r, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(e, "field diff");
  }
  if (ta) cudaFreeAsync(ta, a->stream);
  if (tb) cudaFreeAsync(tb, b->stream);
  if (part) cudaFreeAsync(part, (cudaStream_t)0);
  if (rc != HEAT_OK) return rc;
  if (max_abs) *max_abs = r[2];
  if (rel_l2) *rel_l2 = r[1] > 0 ? std::sqrt(r[0] / r[1]) : std::sqrt(r[0]);
  return HEAT_OK;
}

}  // extern "C"
