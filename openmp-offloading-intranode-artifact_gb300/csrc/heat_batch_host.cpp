// heat_batch_*: many contexts advanced together by one launch per kernel kind
// per time step over a shared tile table (heat_batch.cu), with runs of steps
// captured once as a CUDA graph and replayed.  Host code only.
//
// Launch shape: by default one block per tile, scheduled by the hardware; with
// HEAT_BATCH_PERSISTENT a fixed set of resident blocks strides the table
// instead.  On configuration 3 (64 uneven grids, half FP64, half FP32C) the
// hardware-scheduled shape measured 92 GLUP/s against 86 for the persistent
// one, whose blocks serialise each tile's start-up loads.  Kinds (form x
// source term x blocks-per-SM variant) present together run on their own
// streams (created on first use), forked from and joined to the batch stream,
// unless HEAT_BATCH_SERIAL_FORMS.  Each grid's z-chunk, rows per thread,
// variant and (FP32C) temporal depth come from the autotuner's cache for its
// depth class (heat_tune.cpp).
//
// Grids large enough to fill the GPU alone (HEAT_BATCH_SOLO_POINTS interior
// points, default 2,000,000) are stepped with their single-grid kernels
// instead -- the FP64 hybrid launch, and two FP32C steps per launch -- on a
// stream of their own beside the table kernels; the tile table carries the
// small grids, which one launch per grid would leave the GPU mostly idle for.
// On configuration 3 (64 grids of 48..384 points per axis) the table alone
// measured 129 GLUP/s, with solo grids 137.
//
// Bookkeeping: every active context advances one step per batch step; the
// device table records each grid's current buffer at build time and each
// launch gets the parity of the steps taken since.  A captured graph records
// every grid's current buffer, and is replayed only while they match (a run
// of an even number of steps returns table grids to the same buffers, and
// two-step launches swap once per two steps).  Table grids with two steps per
// launch ("pairs") swap like solo grids: n steps are n / 2 two-step table
// launches (flips counted from pair_flips) and, for an odd n, one single step
// with the grid's own kernel.  The table is rebuilt (and the graph
// re-captured) when the set of active contexts changes.

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <new>
#include <vector>

#include "heat_batch_internal.h"

struct heat_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  unsigned flags = 0;
  heat::TuneChoice override_ = {0, 0, 0, 0};  // fields > 0 replace the tuned choices

  struct Entry {
    heat_ctx *ctx;
    long long remaining;
    long long base_steps;  // ctx->steps_done when the table was built
    bool solo;             // stepped with its single-grid kernels
    bool pairs;            // in the table with two steps per launch (FP32C, depth 2)
  };
  std::vector<Entry> entries;
  std::vector<int> active;  // entry indices in table order, then solo entries
  std::vector<int> solo;    // the active entries stepped alone
  long long solo_points = 2000000;
  cudaStream_t solo_stream = nullptr;
  cudaEvent_t solo_join = nullptr;

  // Two device copies of the tables: a rebuild fills the one not used by the
  // launches still in flight (each copy's event marks its last use).
  heat::BatchGrid *g_buf[2] = {nullptr, nullptr};
  size_t g_cap[2] = {0, 0};
  heat::BatchTile *t_buf[2] = {nullptr, nullptr};
  size_t t_cap[2] = {0, 0};
  CUtensorMap *m_buf[2] = {nullptr, nullptr};  // two-step tiles' tensor maps, 7 per grid
  size_t m_cap[2] = {0, 0};
  std::vector<int> pairs;       // active entries in the table with two steps per launch
  long long pair_flips = 0;     // buffer swaps of those grids since the table was built
  cudaEvent_t table_ev[2] = {nullptr, nullptr};
  bool table_used[2] = {false, false};
  // Table uploads run on their own stream (a pageable upload first waits for
  // everything queued on its stream; this one has nothing queued), and the
  // batch stream waits on copy_ev before the next launch.
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev = nullptr;
  int tb = 0;                          // table copy in use
  heat::BatchGrid *d_grids = nullptr;  // == g_buf[tb]
  heat::BatchTile *d_tiles = nullptr;  // == t_buf[tb]
  int ntiles = 0;
  // Tiles are grouped by form: form f owns [tile_begin[f], tile_begin[f] + tile_count[f]).
  int tile_begin[heat::kNumKinds] = {};
  int tile_count[heat::kNumKinds] = {};
  int form_blocks[heat::kNumKinds] = {};
  int nforms = 0;
  // Side streams and events for running the forms' kernels side by side.
  cudaStream_t side[heat::kNumKinds] = {};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[heat::kNumKinds] = {};
  bool dirty = true;
  long long since_build = 0;

  cudaGraphExec_t gexec = nullptr;
  std::vector<int> graph_curs;  // each active context's current buffer at capture
  long long graph_launches_per = 0;
  int graph_steps = 16;  // even

  int blocks_per_sm[heat::kNumKinds] = {};
  int sms = 0;
  bool persistent = false;  // resident blocks stride the tile table (HEAT_BATCH_PERSISTENT)
  bool concurrent = true;   // forms run side by side on their own streams
  long long launches = 0, graph_launches = 0, batch_steps = 0;
};

namespace heat {

int batch_form(const heat_ctx *c) {
  if (c->precision == HEAT_FP32C) return kFormF32c;
  if (c->flags & HEAT_NAIVE) return -1;
  if (c->flags & HEAT_BITEXACT) return kFormExact;
  if (!c->kq) return kFormHw;
  return (c->hw_rows == 4 && !c->rhs && batch_ws_usable(4)) ? kFormMixWs : kFormMix;
}

void batch_set_override(heat_batch *b, const TuneChoice &ch) {
  b->override_ = ch;
  b->dirty = true;
}

}  // namespace heat

namespace {

void drop_graph(heat_batch *b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->graph_curs.clear();
}

// Whether the captured graph's launches read the buffers every active
// context currently holds.
bool graph_matches(const heat_batch *b) {
  if (!b->gexec || b->graph_curs.size() != b->active.size()) return false;
  for (size_t a = 0; a < b->active.size(); ++a)
    if (b->entries[b->active[a]].ctx->cur != b->graph_curs[a]) return false;
  return true;
}

void release(heat_batch *b) {
  drop_graph(b);
  for (int f = 0; f < heat::kNumKinds; ++f) {
    if (b->side[f]) {
      cudaStreamSynchronize(b->side[f]);
      cudaStreamDestroy(b->side[f]);
    }
    if (b->join_ev[f]) cudaEventDestroy(b->join_ev[f]);
  }
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  if (b->solo_stream) {
    cudaStreamSynchronize(b->solo_stream);
    cudaStreamDestroy(b->solo_stream);
  }
  if (b->solo_join) cudaEventDestroy(b->solo_join);
  if (b->copy_stream) {
    cudaStreamSynchronize(b->copy_stream);
    cudaStreamDestroy(b->copy_stream);
  }
  if (b->copy_ev) cudaEventDestroy(b->copy_ev);
  for (int i = 0; i < 2; ++i) {
    if (b->g_buf[i]) cudaFree(b->g_buf[i]);
    if (b->t_buf[i]) cudaFree(b->t_buf[i]);
    if (b->m_buf[i]) cudaFree(b->m_buf[i]);
    if (b->table_ev[i]) cudaEventDestroy(b->table_ev[i]);
  }
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

template <class T>
int grow(T **p, size_t *cap, size_t need) {
  if (need <= *cap) return HEAT_OK;
  size_t n = std::max(need, *cap * 2);
  T *q = nullptr;
  if (cudaMalloc((void **)&q, n * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ENOMEM;
  }
  if (*p) cudaFree(*p);
  *p = q;
  *cap = n;
  return HEAT_OK;
}

bool grid_has_rhs(const heat_ctx *c) {
  return c->precision == HEAT_FP32C ? c->frhs != nullptr : c->rhs != nullptr;
}

heat::BatchGrid describe(const heat_ctx *c, int form) {
  heat::BatchGrid g{};
  g.form = form;
  g.nx = c->g.nx;
  g.ny = c->g.ny;
  g.nz = c->g.nz;
  g.P = c->g.pitch;
  g.S = c->g.plane;
  g.factor = c->factor;
  g.cur = c->cur;
  g.hw_rows = c->hw_rows;
  g.err = c->err;
  if (form == heat::kFormF32c || form == heat::kFormF32c2) {
    g.f[0] = c->v[0];
    g.f[1] = c->v[1];
    g.cr[0] = c->carry[0];
    g.cr[1] = c->carry[1];
    g.rhs = c->frhs;
    for (int a = 0; a < 3; ++a) g.w[a] = c->fcf[a];
  } else {
    g.f[0] = c->u[0];
    g.f[1] = c->u[1];
    g.rhs = c->rhs;
    if (form == heat::kFormExact) {
      for (int a = 0; a < 3; ++a) g.w[a] = c->ks[a];
    } else {
      g.w[0] = c->c0;
      for (int a = 0; a < 3; ++a) g.w[a + 1] = c->cf[a];
      g.kq = c->kq;
      if (form == heat::kFormHw) g.hw_rows = 8;
    }
  }
  return g;
}

// Throughput guesses (GLUP/s on GB300) used only to split the SMs between
// forms that run side by side.
const double kFormRate[heat::kNumForms] = {100.0, 80.0, 29.0, 200.0, 110.0, 300.0};

// A side stream (and its join event) for kind f, created on first use.
bool ensure_side(heat_batch *b, int f) {
  if (b->side[f]) return true;
  if (cudaStreamCreateWithFlags(&b->side[f], cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join_ev[f], cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

int rebuild(heat_batch *b) {
  drop_graph(b);
  b->active.clear();
  b->solo.clear();
  b->pairs.clear();
  b->pair_flips = 0;
  std::vector<heat::BatchGrid> grids;
  std::vector<heat::BatchTile> per_form[heat::kNumKinds];
  std::vector<CUtensorMap> maps;      // the two-step grids' maps, 7 each
  std::vector<std::pair<int, int>> map_at;  // (grid index, first map)
  double work[heat::kNumKinds] = {};
  for (size_t e = 0; e < b->entries.size(); ++e) {
    heat_batch::Entry &en = b->entries[e];
    if (en.remaining <= 0) continue;
    heat_ctx *c = en.ctx;
    en.base_steps = c->steps_done;
    en.pairs = false;
    const long long pts = (long long)(c->g.nx - 2) * (c->g.ny - 2) * (c->g.nz - 2);
    en.solo = b->solo_points > 0 && pts >= b->solo_points;
    if (en.solo) {
      b->solo.push_back((int)e);
      continue;
    }
    int form = heat::batch_form(c);
    // The autotuner's choices for the grid's form and depth class (the
    // warpgroup-split form shares the hybrid form's entries).
    const int tform = form == heat::kFormMixWs ? heat::kFormMix : form;
    heat::TuneChoice ch = heat::tuned_choice(tform, c->g.nz);
    if (b->override_.kchunk > 0) ch.kchunk = b->override_.kchunk;
    if (b->override_.rows > 0) ch.rows = b->override_.rows;
    if (b->override_.minb > 0) ch.minb = b->override_.minb;
    if (b->override_.depth > 0) ch.depth = b->override_.depth;
    const int minb = std::max(heat::kMinbLo, std::min(ch.minb, heat::kMinbLo + heat::kNumMinb - 1));
    if (form == heat::kFormF32c && ch.depth == 2 && heat::two_step_form(c)) form = heat::kFormF32c2;
    if (form == heat::kFormMixWs && !heat::batch_ws_usable(minb)) form = heat::kFormMix;
    const int kind = heat::kind_of(form, grid_has_rhs(c), form == heat::kFormF32c2 ? heat::kMinbLo : minb);
    const int gi = (int)grids.size();
    grids.push_back(describe(c, form));
    b->active.push_back((int)e);
    const int interior = c->g.nz - 2;
    int kc = std::max(1, std::min(ch.kchunk, interior));
    int rows = std::max(1, std::min(ch.rows, 2)), tile_h = 8 * rows;
    if (form == heat::kFormF32c2) {
      en.pairs = true;
      b->pairs.push_back((int)e);
      map_at.push_back({gi, (int)maps.size()});
      maps.resize(maps.size() + 7);
      if (!heat::encode_fp32c_maps(&maps[maps.size() - 7], c->v, c->carry, c->fcf, c->g))
        return HEAT_ECUDA;
      // two steps per 32 x 16 tile; the temporal blocking wants long z-walks
      kc = std::max(kc, std::min(16, interior));
      rows = 1;
      tile_h = 16;
    }
    const int ntx = (c->g.nx - 2 + 31) / 32, nty = (c->g.ny - 2 + tile_h - 1) / tile_h;
    for (int k0 = 1; k0 < c->g.nz - 1; k0 += kc) {
      const int k1 = std::min(k0 + kc, c->g.nz - 1);
      for (int ty = 0; ty < nty; ++ty)
        for (int tx = 0; tx < ntx; ++tx) per_form[kind].push_back({gi, tx, ty, k0, k1, rows});
    }
    work[kind] += (double)(c->g.nx - 2) * (c->g.ny - 2) * interior / kFormRate[form];
  }
  b->active.insert(b->active.end(), b->solo.begin(), b->solo.end());
  std::vector<heat::BatchTile> tiles;
  double total = 0;
  b->nforms = 0;
  for (int f = 0; f < heat::kNumKinds; ++f) {
    b->tile_begin[f] = (int)tiles.size();
    b->tile_count[f] = (int)per_form[f].size();
    tiles.insert(tiles.end(), per_form[f].begin(), per_form[f].end());
    total += work[f];
    if (b->tile_count[f] > 0) ++b->nforms;
  }
  // Resident blocks per form: the whole GPU for a lone form; with several
  // forms, each gets SMs in proportion to its estimated time so they finish
  // together while sharing every SM.
  for (int f = 0; f < heat::kNumKinds; ++f) {
    if (b->tile_count[f] == 0) {
      b->form_blocks[f] = 0;
      continue;
    }
    if (!b->persistent) {
      b->form_blocks[f] = b->tile_count[f];  // one tile per block, hardware-scheduled
      continue;
    }
    const double share = (b->nforms == 1 || total <= 0 || !b->concurrent) ? 1.0 : work[f] / total;
    long long full = (long long)b->blocks_per_sm[f] * b->sms;
    long long nb = std::max(1LL, (long long)(share * full + 0.5));
    b->form_blocks[f] = (int)std::min<long long>(nb, b->tile_count[f]);
  }
  // Fill the table copy the in-flight launches are not using (waiting, if
  // need be, for the launches that used it last).
  const int nb = b->tb ^ 1;
  if (b->table_used[nb] && cudaEventSynchronize(b->table_ev[nb]) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  int rc = grow(&b->g_buf[nb], &b->g_cap[nb], std::max<size_t>(1, grids.size()));
  if (rc == HEAT_OK) rc = grow(&b->t_buf[nb], &b->t_cap[nb], std::max<size_t>(1, tiles.size()));
  if (rc == HEAT_OK && !maps.empty()) rc = grow(&b->m_buf[nb], &b->m_cap[nb], maps.size());
  if (rc != HEAT_OK) return rc;
  for (const auto &gm : map_at) grids[gm.first].tmaps = b->m_buf[nb] + gm.second;
  for (int f = 0; f < heat::kNumKinds; ++f)
    if (b->tile_count[f] && !ensure_side(b, f)) return HEAT_ECUDA;
  if (!maps.empty() && cudaMemcpyAsync(b->m_buf[nb], maps.data(), maps.size() * sizeof(CUtensorMap),
                                       cudaMemcpyHostToDevice, b->copy_stream) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  // Pageable sources: the copies are staged before the calls return.
  if (!grids.empty() &&
      (cudaMemcpyAsync(b->g_buf[nb], grids.data(), grids.size() * sizeof(heat::BatchGrid),
                       cudaMemcpyHostToDevice, b->copy_stream) != cudaSuccess ||
       cudaMemcpyAsync(b->t_buf[nb], tiles.data(), tiles.size() * sizeof(heat::BatchTile),
                       cudaMemcpyHostToDevice, b->copy_stream) != cudaSuccess ||
       cudaEventRecord(b->copy_ev, b->copy_stream) != cudaSuccess ||
       cudaStreamWaitEvent(b->stream, b->copy_ev, 0) != cudaSuccess)) {
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  b->tb = nb;
  b->d_grids = b->g_buf[nb];
  b->d_tiles = b->t_buf[nb];
  b->ntiles = (int)tiles.size();
  b->since_build = 0;
  b->dirty = false;
  return HEAT_OK;
}

// Account n steps for every active context.
void advance(heat_batch *b, long long n) {
  for (int e : b->active) {
    heat_batch::Entry &en = b->entries[e];
    en.ctx->steps_done += n;
    if ((en.solo || en.pairs) ? heat::ctx_flips(en.ctx, n) : (n & 1)) en.ctx->cur ^= 1;
    en.remaining -= n;
  }
  b->pair_flips += n / 2 + n % 2;
  b->since_build += n;
  b->batch_steps += n;
}

// The solo grids' n steps, one grid after another, on stream st.
cudaError_t enqueue_solo(heat_batch *b, int n, cudaStream_t st, long long *launches) {
  cudaError_t err = cudaSuccess;
  for (size_t a = 0; a < b->solo.size() && err == cudaSuccess; ++a) {
    heat_ctx *c = b->entries[b->solo[a]].ctx;
    err = heat::enqueue_ctx_steps(c, c->cur, n, st, launches);
  }
  return err;
}

// n steps of one kind's tiles on stream st: one launch per step with the step
// parity (p + s) for single-step kinds; for the two-step FP32C kind, n / 2
// two-step launches (each swapping the grids' buffers once, counted from
// pair_flips) and, for an odd n, one single step of each such grid with its
// single-grid kernel.
cudaError_t enqueue_kind(heat_batch *b, int f, int p, int n, cudaStream_t st,
                         long long *launches) {
  cudaError_t err = cudaSuccess;
  if (heat::form_of_kind(f) != heat::kFormF32c2) {
    for (int s = 0; s < n && err == cudaSuccess; ++s)
      err = heat::launch_batch(f, b->d_grids, b->d_tiles + b->tile_begin[f], b->tile_count[f],
                               (p + s) & 1, b->form_blocks[f], st);
    *launches += n;
    return err;
  }
  for (int s = 0; s < n / 2 && err == cudaSuccess; ++s) {
    err = heat::launch_batch(f, b->d_grids, b->d_tiles + b->tile_begin[f], b->tile_count[f],
                             (int)((b->pair_flips + s) & 1), b->form_blocks[f], st);
    *launches += 1;
  }
  if (n & 1)
    for (size_t a = 0; a < b->pairs.size() && err == cudaSuccess; ++a) {
      heat_ctx *c = b->entries[b->pairs[a]].ctx;
      err = heat::enqueue_one_step(c, c->cur ^ ((n / 2) & 1), st, launches);
    }
  return err;
}

// Enqueue `n` steps starting at parity p: each kind's kernel on its own side
// stream (forked from and joined to the batch stream) when several are
// present, so a memory-bound and a compute-bound form share the SMs; the solo
// grids on a further side stream.  *launches counts the kernels.
cudaError_t enqueue_steps(heat_batch *b, int p, int n, long long *launches) {
  cudaError_t err = cudaSuccess;
  const int parts = b->nforms + (b->solo.empty() ? 0 : 1);
  if (parts <= 1 || !b->concurrent) {
    for (int f = 0; f < heat::kNumKinds && err == cudaSuccess; ++f)
      if (b->tile_count[f]) err = enqueue_kind(b, f, p, n, b->stream, launches);
    if (err == cudaSuccess) err = enqueue_solo(b, n, b->stream, launches);
    return err;
  }
  err = cudaEventRecord(b->fork_ev, b->stream);
  if (err == cudaSuccess && !b->solo.empty()) {
    err = cudaStreamWaitEvent(b->solo_stream, b->fork_ev, 0);
    if (err == cudaSuccess) err = enqueue_solo(b, n, b->solo_stream, launches);
    if (err == cudaSuccess) err = cudaEventRecord(b->solo_join, b->solo_stream);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(b->stream, b->solo_join, 0);
  }
  for (int f = 0; f < heat::kNumKinds && err == cudaSuccess; ++f) {
    if (!b->tile_count[f]) continue;
    err = cudaStreamWaitEvent(b->side[f], b->fork_ev, 0);
    if (err == cudaSuccess) err = enqueue_kind(b, f, p, n, b->side[f], launches);
    if (err == cudaSuccess) err = cudaEventRecord(b->join_ev[f], b->side[f]);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(b->stream, b->join_ev[f], 0);
  }
  return err;
}

void mark_table_use(heat_batch *b) {
  cudaEventRecord(b->table_ev[b->tb], b->stream);
  b->table_used[b->tb] = true;
}

int launch_plain(heat_batch *b, int n) {
  long long nl = 0;
  if (enqueue_steps(b, (int)(b->since_build & 1), n, &nl) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  mark_table_use(b);
  b->launches += nl;
  advance(b, n);
  return HEAT_OK;
}

int capture_graph(heat_batch *b) {
  drop_graph(b);
  cudaGraph_t graph = nullptr;
  if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  const int p = (int)(b->since_build & 1);
  long long nl = 0;
  cudaError_t err = enqueue_steps(b, p, b->graph_steps, &nl);
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
  if (err != cudaSuccess || e2 != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  cudaError_t e3 = cudaGraphInstantiate(&b->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e3 != cudaSuccess) {
    b->gexec = nullptr;
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  b->graph_curs.clear();
  for (int e : b->active) b->graph_curs.push_back(b->entries[e].ctx->cur);
  b->graph_launches_per = nl;
  return HEAT_OK;
}

}  // namespace

extern "C" {

int heat_batch_create(heat_batch **out, void *stream, unsigned flags) {
  if (!out) return HEAT_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return HEAT_ENODEV;
  }
  heat_batch *b = new (std::nothrow) heat_batch();
  if (!b) return HEAT_ENOMEM;
  b->flags = flags;
  cudaGetDevice(&b->device);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  for (int f = 0; f < heat::kNumKinds; ++f) b->blocks_per_sm[f] = heat::batch_blocks_per_sm(f);
  b->persistent = (flags & HEAT_BATCH_PERSISTENT) != 0;
  b->concurrent = (flags & HEAT_BATCH_SERIAL_FORMS) == 0;
  bool ok = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->table_ev[0], cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->table_ev[1], cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->copy_ev, cudaEventDisableTiming) == cudaSuccess &&
            cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaStreamCreateWithFlags(&b->solo_stream, cudaStreamNonBlocking) == cudaSuccess &&
       cudaEventCreateWithFlags(&b->solo_join, cudaEventDisableTiming) == cudaSuccess;
  if (const char *ev = std::getenv("HEAT_BATCH_SOLO_POINTS")) b->solo_points = std::atoll(ev);
  if (!ok) {
    cudaGetLastError();
    release(b);
    return HEAT_ECUDA;
  }
  if (stream) {
    b->stream = (cudaStream_t)stream;
  } else {
    // Graph capture needs a stream other than the legacy default one.
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      delete b;
      return HEAT_ECUDA;
    }
    b->own_stream = true;
  }
  *out = b;
  return HEAT_OK;
}

int heat_batch_add(heat_batch *b, heat_ctx *c, long long steps) {
  if (!b || !c || steps < 0) return HEAT_EINVAL;
  if (c->device != b->device || heat::batch_form(c) < 0) return HEAT_EINVAL;
  for (auto &en : b->entries)
    if (en.ctx == c) {
      if (en.remaining <= 0 && steps > 0) b->dirty = true;
      en.remaining += steps;
      return HEAT_OK;
    }
  // Work already queued on the context's own stream finishes first.
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    cudaGetLastError();
    return HEAT_ECUDA;
  }
  b->entries.push_back({c, steps, c->steps_done});
  if (steps > 0) b->dirty = true;
  return HEAT_OK;
}

int heat_batch_remove(heat_batch *b, heat_ctx *c) {
  if (!b || !c) return HEAT_EINVAL;
  for (size_t e = 0; e < b->entries.size(); ++e)
    if (b->entries[e].ctx == c) {
      // A context with steps left may be in launches still running.
      if (b->entries[e].remaining > 0 && cudaStreamSynchronize(b->stream) != cudaSuccess) {
        cudaGetLastError();
        return HEAT_ECUDA;
      }
      b->entries.erase(b->entries.begin() + (long)e);
      b->dirty = true;
      return HEAT_OK;
    }
  return HEAT_EINVAL;
}

int heat_batch_pending(heat_batch *b, heat_ctx *c, long long *steps_left) {
  if (!b || !c) return HEAT_EINVAL;
  for (auto &en : b->entries)
    if (en.ctx == c) {
      if (steps_left) *steps_left = en.remaining > 0 ? en.remaining : 0;
      return HEAT_OK;
    }
  return HEAT_EINVAL;
}

}  // extern "C"

namespace heat {

// heat_batch_run without the final synchronisation: launches are queued on
// the batch stream and the host bookkeeping (steps, current buffers) is
// already advanced when it returns.
int batch_run(heat_batch *b, long long max_steps, long long *steps_taken, bool sync) {
  if (!b) return HEAT_EINVAL;
  long long done = 0;
  int rc = HEAT_OK;
  // Work queued on the member contexts' own streams (e.g. steps taken outside
  // the batch) finishes first; a context stepped outside the batch since the
  // table was built has moved its current buffer, so the table is rebuilt.
  for (auto &en : b->entries)
    if (cudaStreamSynchronize(en.ctx->stream) != cudaSuccess) {
      cudaGetLastError();
      return HEAT_ECUDA;
    }
  for (int e : b->active)
    if (b->entries[e].ctx->steps_done != b->entries[e].base_steps + b->since_build) b->dirty = true;
  for (;;) {
    if (b->dirty) {
      rc = rebuild(b);
      if (rc != HEAT_OK) break;
    }
    if (b->active.empty()) break;
    long long m = -1;
    for (int e : b->active) {
      long long r = b->entries[e].remaining;
      if (m < 0 || r < m) m = r;
    }
    if (max_steps >= 0) m = std::min(m, max_steps - done);
    if (m <= 0) break;
    const bool graphs = !(b->flags & HEAT_BATCH_NO_GRAPHS);
    if (graphs && m >= b->graph_steps) {
      if (b->gexec && !graph_matches(b)) {
        // the graph was captured with other current buffers: one plain step
        // (table grids swap with step parity), else capture anew
        rc = launch_plain(b, 1);
        if (rc != HEAT_OK) break;
        ++done;
        --m;
        if (!graph_matches(b)) drop_graph(b);
      }
      if (m >= b->graph_steps) {
        if (!b->gexec) {
          rc = capture_graph(b);
          if (rc != HEAT_OK) break;
        }
        const long long reps = m / b->graph_steps;
        for (long long r = 0; r < reps; ++r) {
          if (cudaGraphLaunch(b->gexec, b->stream) != cudaSuccess) {
            cudaGetLastError();
            rc = HEAT_ECUDA;
            break;
          }
          b->graph_launches += 1;
          b->launches += b->graph_launches_per;
          mark_table_use(b);
          advance(b, b->graph_steps);
          done += b->graph_steps;
        }
        if (rc != HEAT_OK) break;
        m -= reps * b->graph_steps;
      }
    }
    if (m > 0) {
      rc = launch_plain(b, (int)m);
      if (rc != HEAT_OK) break;
      done += m;
    }
    for (int e : b->active)
      if (b->entries[e].remaining <= 0) b->dirty = true;
    if (max_steps >= 0 && done >= max_steps) break;
  }
  if (sync && cudaStreamSynchronize(b->stream) != cudaSuccess) {
    cudaGetLastError();
    if (rc == HEAT_OK) rc = HEAT_ECUDA;
  }
  // A member whose TMA-staged launches (the kernels with device-side waits:
  // FP32C two-step, default FP64) reported a wait running out makes the run
  // return HEAT_ETIMEOUT; every member's flag is read (and cleared) so none is
  // reported twice.
  if (sync)
    for (auto &en : b->entries) {
      const int e = check_err(en.ctx);
      if (rc == HEAT_OK && e != HEAT_OK) rc = e;
    }
  if (steps_taken) *steps_taken = done;
  return rc;
}

cudaStream_t batch_stream(heat_batch *b) { return b->stream; }

}  // namespace heat

extern "C" {

int heat_batch_run(heat_batch *b, long long max_steps, long long *steps_taken) {
  return heat::batch_run(b, max_steps, steps_taken, true);
}

int heat_batch_stats(heat_batch *b, long long *kernel_launches, long long *graph_launches,
                     long long *batch_steps) {
  if (!b) return HEAT_EINVAL;
  if (kernel_launches) *kernel_launches = b->launches;
  if (graph_launches) *graph_launches = b->graph_launches;
  if (batch_steps) *batch_steps = b->batch_steps;
  return HEAT_OK;
}

int heat_batch_destroy(heat_batch *b) {
  if (!b) return HEAT_EINVAL;
  if (b->stream) cudaStreamSynchronize(b->stream);
  release(b);
  return HEAT_OK;
}

}  // extern "C"
