// Autotuner of the batched table kernels, per precision form and size class,
// cached to a JSON file.
//
// Size classes are by grid depth nz (the z extent each tile column walks):
// nz <= 64, 128, 256, 384, 512, 1024, 2048 and larger.  Per class the tuner
// chooses
//   kchunk : planes per tile's z-walk (8 ... 512, or the whole depth),
//   rows   : rows each thread walks, 8 apart (tile height 8 x rows: 8 or 16),
//   minb   : the table kernel compiled for 2, 3 or 4 resident blocks per SM
//            (its register cap per thread: 128, 80 or 64),
//   depth  : time steps per launch, 1, or 2 for FP32C grids (the two-step TMA
//            kernel on 32 x 16 tiles),
// one after another (coordinate descent from the defaults 32 / 1 / the form's
// default / 1).  For a class it builds a batch that fills the GPU the way a
// real batch does: copies of one synthetic grid of that depth
// (configuration-0 fields; x and y extents min(nz, 384); enough copies for
// ~48M points, at most 64), times each candidate for 2 warm-up + 6 timed steps
// (CUDA events, graphs off), and keeps the fastest.  Batches look their grids'
// classes up in the cache; classes not tuned yet use the defaults.
//
// Cache file: $HEAT_TUNE_CACHE, else heat_tune.json next to libheat.so (read
// again whenever that path changes).  One entry per line:
//   {"form": F, "nz_max": N, "kchunk": K, "rows": R, "minb": M, "depth": D, "glups": G},
// (entries written before rows / minb / depth existed read with the defaults).

#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "heat_batch_internal.h"

namespace heat {
void batch_set_override(heat_batch *b, const TuneChoice &ch);
}

namespace {

struct TuneEntry {
  int form, nz_max;
  heat::TuneChoice ch;
  double glups;
};

const int kClasses[] = {64, 128, 256, 384, 512, 1024, 2048, 1 << 30};
constexpr int kDefaultKchunk = 32;

std::mutex g_mu;
std::vector<TuneEntry> g_table;
bool g_loaded = false;
std::string g_loaded_path;
char g_device[256] = "";

std::string cache_path() {
  if (const char *e = std::getenv("HEAT_TUNE_CACHE")) return e;
  Dl_info info;
  if (dladdr(reinterpret_cast<void *>(&cache_path), &info) && info.dli_fname) {
    std::string p = info.dli_fname;
    size_t s = p.rfind('/');
    return (s == std::string::npos ? std::string(".") : p.substr(0, s)) + "/heat_tune.json";
  }
  return "heat_tune.json";
}

heat::TuneChoice default_choice(int form) {
  return {kDefaultKchunk, 1, heat::default_minb(form), 1};
}

void load_locked() {
  const std::string path = cache_path();
  if (g_loaded && path == g_loaded_path) return;
  g_loaded = true;
  g_loaded_path = path;
  g_table.clear();
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) return;
  char line[512];
  while (std::fgets(line, sizeof line, f)) {
    const char *p = std::strstr(line, "{\"form\":");
    if (!p) continue;
    TuneEntry t{};
    int kc = 0;
    if (std::sscanf(p, "{\"form\": %d, \"nz_max\": %d, \"kchunk\": %d", &t.form, &t.nz_max,
                    &kc) != 3 ||
        kc <= 0 || t.form < 0 || t.form >= heat::kNumForms)
      continue;
    t.ch = default_choice(t.form);
    t.ch.kchunk = kc;
    int v = 0;
    if (const char *q = std::strstr(p, "\"rows\":"); q && std::sscanf(q, "\"rows\": %d", &v) == 1 &&
        v >= 1 && v <= 2)
      t.ch.rows = v;
    if (const char *q = std::strstr(p, "\"minb\":"); q && std::sscanf(q, "\"minb\": %d", &v) == 1 &&
        v >= heat::kMinbLo && v < heat::kMinbLo + heat::kNumMinb)
      t.ch.minb = v;
    if (const char *q = std::strstr(p, "\"depth\":");
        q && std::sscanf(q, "\"depth\": %d", &v) == 1 && v >= 1 && v <= 2)
      t.ch.depth = v;
    if (const char *q = std::strstr(p, "\"glups\":")) std::sscanf(q, "\"glups\": %lf", &t.glups);
    g_table.push_back(t);
  }
  std::fclose(f);
}

int save_locked() {
  FILE *f = std::fopen(cache_path().c_str(), "w");
  if (!f) return HEAT_EINVAL;
  std::fprintf(f, "{\"device\": \"%s\", \"entries\": [\n", g_device);
  for (size_t i = 0; i < g_table.size(); ++i) {
    const TuneEntry &t = g_table[i];
    std::fprintf(f,
                 " {\"form\": %d, \"nz_max\": %d, \"kchunk\": %d, \"rows\": %d, \"minb\": %d, "
                 "\"depth\": %d, \"glups\": %.3f}%s\n",
                 t.form, t.nz_max, t.ch.kchunk, t.ch.rows, t.ch.minb, t.ch.depth, t.glups,
                 i + 1 < g_table.size() ? "," : "");
  }
  std::fprintf(f, "]}\n");
  std::fclose(f);
  g_loaded_path = cache_path();
  return HEAT_OK;
}

int class_of(int nz) {
  for (int c : kClasses)
    if (nz <= c) return c;
  return kClasses[sizeof kClasses / sizeof kClasses[0] - 1];
}

int form_of(int precision, unsigned flags) {
  if (precision == HEAT_FP32C) return heat::kFormF32c;
  if (flags & HEAT_BITEXACT) return heat::kFormExact;
  if (flags & HEAT_HWFP64) return heat::kFormHw;
  return heat::kFormMix;
}

// GLUP/s of a batch of identical grids with the choices ch.
double time_candidate(std::vector<heat_ctx *> &cs, heat_batch *b, const heat::TuneChoice &ch,
                      cudaStream_t st) {
  heat::batch_set_override(b, ch);
  long long taken = 0;
  for (heat_ctx *c : cs)
    if (heat_batch_add(b, c, 2) != HEAT_OK) return -1;
  if (heat_batch_run(b, -1, &taken) != HEAT_OK) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int steps = 6;
  for (heat_ctx *c : cs) heat_batch_add(b, c, steps);
  cudaEventRecord(e0, st);
  int rc = heat_batch_run(b, -1, &taken);
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != HEAT_OK || ms <= 0.f) return -1;
  const heat_ctx *c = cs[0];
  const double upd =
      (double)(c->g.nx - 2) * (c->g.ny - 2) * (c->g.nz - 2) * steps * (double)cs.size();
  return upd / (ms * 1e-3) / 1e9;
}

}  // namespace

namespace heat {

TuneChoice tuned_choice(int form, int nz) {
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  const int cls = class_of(nz);
  for (const TuneEntry &t : g_table)
    if (t.form == form && t.nz_max == cls) return t.ch;
  return default_choice(form);
}

}  // namespace heat

extern "C" int heat_tune_batch(int precision, unsigned flags, int max_nz, int force) {
  if (precision != HEAT_FP64 && precision != HEAT_FP32C) return HEAT_EINVAL;
  const int form = form_of(precision, flags);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess)
      std::snprintf(g_device, sizeof g_device, "%s", prop.name);
    else
      cudaGetLastError();
  }
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  int rc = HEAT_OK;
  for (int cls : kClasses) {
    if (max_nz > 0 && cls > class_of(max_nz)) break;
    {
      std::lock_guard<std::mutex> lk(g_mu);
      bool have = false;
      for (const TuneEntry &t : g_table) have |= (t.form == form && t.nz_max == cls);
      if (have && !force) continue;
    }
    const int nz = std::min(cls, 1024);
    const int nxy = std::min(nz, 384);
    const double pts = (double)nxy * nxy * nz;
    const int copies = (int)std::max(1.0, std::min(64.0, std::ceil(48e6 / pts)));
    std::vector<double> kappa((size_t)nxy * nxy * nz), u0(kappa.size());
    double h = 0, dt = 0;
    rc = heat_inputs_config(0, 7, nxy, nxy, nz, kappa.data(), u0.data(), &h, &dt);
    if (rc != HEAT_OK) break;
    heat_desc d{};
    d.nx = nxy;
    d.ny = nxy;
    d.nz = nz;
    d.h = h;
    d.dt = dt;
    d.kappa = kappa.data();
    d.u0 = u0.data();
    d.precision = precision;
    d.flags = flags & (HEAT_BITEXACT | HEAT_HWFP64);
    d.stream = st;
    std::vector<heat_ctx *> cs;
    for (int q = 0; q < copies && rc == HEAT_OK; ++q) {
      heat_ctx *c = nullptr;
      rc = heat_init(&c, &d);
      if (rc == HEAT_OK) cs.push_back(c);
    }
    heat_batch *b = nullptr;
    if (rc == HEAT_OK) rc = heat_batch_create(&b, st, HEAT_BATCH_NO_GRAPHS);
    heat::TuneChoice best_ch = default_choice(form);
    double best = -1;
    if (rc == HEAT_OK) {
      // one parameter at a time, each from the best choice so far
      auto consider = [&](heat::TuneChoice ch) {
        const double g = time_candidate(cs, b, ch, st);
        if (g > best) {
          best = g;
          best_ch = ch;
        }
      };
      for (int kc : {8, 16, 32, 64, 128, 256, 512, nz - 2}) {
        if (kc > nz - 2) continue;
        heat::TuneChoice ch = best_ch;
        ch.kchunk = kc;
        consider(ch);
      }
      for (int rows : {1, 2}) {
        heat::TuneChoice ch = best_ch;
        ch.rows = rows;
        if (rows != best_ch.rows) consider(ch);
      }
      for (int m = heat::kMinbLo; m < heat::kMinbLo + heat::kNumMinb; ++m) {
        heat::TuneChoice ch = best_ch;
        ch.minb = m;
        if (m != best_ch.minb) consider(ch);
      }
      if (form == heat::kFormF32c) {
        heat::TuneChoice ch = best_ch;
        ch.depth = 2;
        consider(ch);
      }
    }
    if (b) heat_batch_destroy(b);
    for (heat_ctx *c : cs) heat_destroy(c);
    if (rc != HEAT_OK) break;
    if (best <= 0) {
      rc = HEAT_ECUDA;
      break;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    g_table.erase(std::remove_if(g_table.begin(), g_table.end(),
                                 [&](const TuneEntry &t) { return t.form == form && t.nz_max == cls; }),
                  g_table.end());
    g_table.push_back({form, cls, best_ch, best});
  }
  cudaStreamDestroy(st);
  std::lock_guard<std::mutex> lk(g_mu);
  int src = save_locked();
  return rc != HEAT_OK ? rc : src;
}

extern "C" int heat_tune_lookup(int precision, unsigned flags, int nz, int *kchunk) {
  if (!kchunk || nz < 3) return HEAT_EINVAL;
  *kchunk = heat::tuned_choice(form_of(precision, flags), nz).kchunk;
  return HEAT_OK;
}

extern "C" int heat_tune_choice(int precision, unsigned flags, int nz, heat_tune_entry *out) {
  if (!out || nz < 3) return HEAT_EINVAL;
  if (precision != HEAT_FP64 && precision != HEAT_FP32C) return HEAT_EINVAL;
  const heat::TuneChoice ch = heat::tuned_choice(form_of(precision, flags), nz);
  out->kchunk = ch.kchunk;
  out->rows = ch.rows;
  out->blocks_per_sm = ch.minb;
  out->depth = ch.depth;
  return HEAT_OK;
}
