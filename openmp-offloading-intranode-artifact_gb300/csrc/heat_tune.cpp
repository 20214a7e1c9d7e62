// Autotuner of the batched kernel's z-chunk, per precision form and size class,
// cached to a JSON file.
//
// Size classes are by grid depth nz (the z extent each tile column walks):
// nz <= 64, 128, 256, 384, 512, 1024, 2048 and larger.  For a class the tuner
// builds a batch that fills the GPU the way a real batch does: copies of one
// synthetic grid of that depth (configuration-0 fields; x and y extents
// min(nz, 384); enough copies for ~48M points, at most 64), runs it with each
// candidate z-chunk (8 ... 512, and the whole depth) for 2 warm-up + 6 timed
// steps (CUDA events, graphs off), and keeps the fastest.  Batches look their
// grids' classes up in the cache; classes not tuned yet use 32 planes.
//
// Cache file: $HEAT_TUNE_CACHE, else heat_tune.json next to libheat.so.  One
// entry per line:  {"form": F, "nz_max": N, "kchunk": K, "glups": G},

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
void batch_set_kchunk_override(heat_batch *b, int kchunk);
}

namespace {

struct TuneEntry {
  int form, nz_max, kchunk;
  double glups;
};

const int kClasses[] = {64, 128, 256, 384, 512, 1024, 2048, 1 << 30};
constexpr int kDefaultKchunk = 32;

std::mutex g_mu;
std::vector<TuneEntry> g_table;
bool g_loaded = false;
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

void load_locked() {
  if (g_loaded) return;
  g_loaded = true;
  FILE *f = std::fopen(cache_path().c_str(), "r");
  if (!f) return;
  char line[512];
  while (std::fgets(line, sizeof line, f)) {
    const char *p = std::strstr(line, "{\"form\":");
    if (!p) continue;
    TuneEntry t{};
    if (std::sscanf(p, "{\"form\": %d, \"nz_max\": %d, \"kchunk\": %d, \"glups\": %lf", &t.form,
                    &t.nz_max, &t.kchunk, &t.glups) == 4 &&
        t.kchunk > 0)
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
    std::fprintf(f, " {\"form\": %d, \"nz_max\": %d, \"kchunk\": %d, \"glups\": %.3f}%s\n", t.form,
                 t.nz_max, t.kchunk, t.glups, i + 1 < g_table.size() ? "," : "");
  }
  std::fprintf(f, "]}\n");
  std::fclose(f);
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

// GLUP/s of a batch of identical grids at z-chunk kc.
double time_candidate(std::vector<heat_ctx *> &cs, heat_batch *b, int kc, cudaStream_t st) {
  heat::batch_set_kchunk_override(b, kc);
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

int tuned_kchunk(int form, int nz) {
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  const int cls = class_of(nz);
  for (const TuneEntry &t : g_table)
    if (t.form == form && t.nz_max == cls) return t.kchunk;
  return kDefaultKchunk;
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
    int best_k = kDefaultKchunk;
    double best = -1;
    if (rc == HEAT_OK) {
      std::vector<int> cands = {8, 16, 32, 64, 128, 256, 512, nz - 2};
      for (int kc : cands) {
        if (kc > nz - 2) continue;
        double g = time_candidate(cs, b, kc, st);
        if (g > best) {
          best = g;
          best_k = kc;
        }
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
    g_table.push_back({form, cls, best_k, best});
  }
  cudaStreamDestroy(st);
  std::lock_guard<std::mutex> lk(g_mu);
  int src = save_locked();
  return rc != HEAT_OK ? rc : src;
}

extern "C" int heat_tune_lookup(int precision, unsigned flags, int nz, int *kchunk) {
  if (!kchunk || nz < 3) return HEAT_EINVAL;
  *kchunk = heat::tuned_kchunk(form_of(precision, flags), nz);
  return HEAT_OK;
}
