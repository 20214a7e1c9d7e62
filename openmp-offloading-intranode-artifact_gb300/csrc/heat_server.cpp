// heat_server_*: a continuous-batching solve server on one GPU.
//
// Requests (grid size, step count, precision, seeded inputs) are submitted from
// any thread.  Prep threads generate each request's host inputs off the GPU
// path.  One GPU worker thread runs the loop
//
//   admit:   take prepared requests in arrival order while their device bytes
//            fit the HBM budget (a request that does not fit waits; the next
//            few behind it may be admitted first if they fit) and hand them
//            to the init threads, which create their contexts (uploads and
//            set-up kernels; fields stay device-resident until they finish);
//   attach:  add contexts that are ready to the batch with their step counts;
//   advance: queue at most `tick_steps` batch steps -- every resident solve
//            advances together, whatever its size and form -- and record a
//            tick event; the worker does not wait for the tick;
//   retire:  solves whose last step ran in a tick that has completed report
//            their norm (and field, if asked), release their memory and
//            budget, and become results.
//
// Admission and retirement of one tick overlap with the GPU running the
// previous ones (at most three ticks are queued), so requests arriving while
// others are on the GPU join at the next tick as memory frees up, and their
// work overlaps on the device.  Each request's context has its own stream;
// contexts allocate from the library's stream-ordered pool, so neither
// admission nor retirement synchronises the device.  Latency of a request =
// completion time - submission time.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <utility>
#include <vector>

#include "heat_batch_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  uint64_t id = 0;
  heat_request req{};
  double submit_ms = 0, admit_ms = 0;
  size_t bytes = 0;
  double *kappa = nullptr, *u0 = nullptr;  // pinned host inputs (server pool)
  size_t kappa_cap = 0, u0_cap = 0;
  double h = 0, dt = 0;
  int status = HEAT_OK;
  int init_rc = HEAT_OK;
  heat_ctx *ctx = nullptr;
  bool finished = false;          // all steps queued
  cudaEvent_t finish_ev = nullptr;  // tick event after its last step (null: none ran)
};

// Device bytes a request holds while resident (fields, coefficient planes,
// and the FP64 staging buffer heat_init uses), pitch padding included.
size_t request_bytes(const heat_request &r) {
  const size_t pitch = ((size_t)r.nx + 3) & ~(size_t)3;
  const size_t pts = pitch * (size_t)r.ny * (size_t)r.nz;
  return pts * (r.precision == HEAT_FP32C ? 32 : 64) + (1u << 20);
}

}  // namespace

// Pinned host buffers for request inputs, reused across requests: inputs are
// generated straight into page-locked memory (no page faults on fresh
// allocations once warm) and uploaded asynchronously at full link speed.
// Buffers come in power-of-two size classes from 1 MiB; unused buffers are
// kept up to `keep` bytes.
class PinnedPool {
 public:
  explicit PinnedPool(size_t keep) : keep_(keep) {}
  ~PinnedPool() {
    for (auto &c : free_)
      for (void *p : c.second) cudaFreeHost(p);
  }
  // A buffer of at least `bytes` (its capacity in *cap), or nullptr.
  void *get(size_t bytes, size_t *cap) {
    size_t c = size_t(1) << 20;
    while (c < bytes) c <<= 1;
    {
      std::lock_guard<std::mutex> lk(mu_);
      auto &v = free_[c];
      if (!v.empty()) {
        void *p = v.back();
        v.pop_back();
        kept_ -= c;
        *cap = c;
        return p;
      }
    }
    void *p = nullptr;
    if (cudaHostAlloc(&p, c, cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    *cap = c;
    return p;
  }
  void put(void *p, size_t cap) {
    if (!p) return;
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (kept_ + cap <= keep_) {
        free_[cap].push_back(p);
        kept_ += cap;
        return;
      }
    }
    cudaFreeHost(p);
  }

 private:
  std::mutex mu_;
  std::map<size_t, std::vector<void *>> free_;
  size_t kept_ = 0, keep_;
};

struct heat_server {
  size_t budget = 0;
  size_t prep_cap = 0;  // host bytes of prepared inputs held ahead of admission
  int tick_steps = 64;
  int queue_ticks = 3;  // ticks queued on the GPU ahead of the host (HEAT_SERVER_QUEUE_TICKS)
  Clock::time_point t0;

  std::mutex mu;
  std::condition_variable cv_prep, cv_work, cv_idle, cv_init;
  std::deque<Job *> submitted;   // waiting for input generation
  std::deque<Job *> ready;       // inputs generated, waiting for admission
  std::deque<Job *> to_init;     // admitted (budget reserved), context not yet created
  std::deque<Job *> inited;      // context created (or failed), not yet in the batch
  int initing = 0;
  bool stop_init = false;
  std::vector<Job *> resident;   // on the GPU
  std::vector<heat_result> done; // not yet polled
  std::vector<double> latencies;
  uint64_t next_id = 1;
  bool stop = false;
  int preparing = 0;

  size_t in_use = 0, peak = 0, ready_bytes = 0;
  long long n_submitted = 0, n_admitted = 0, n_completed = 0, n_rejected = 0;
  double updates_done = 0;
  double busy_ms = 0;            // wall time the worker spent advancing solves
  double first_admit_ms = -1, last_done_ms = 0;

  heat_batch *batch = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;
  std::vector<cudaEvent_t> ev_free;   // recycled tick events
  std::deque<cudaEvent_t> ev_live;    // tick events of queued ticks, oldest first
  // Timing events bracketing each tick on the server stream: their summed
  // spans are the time the GPU spent in ticks (gaps are the GPU waiting for
  // the host).
  std::deque<std::pair<cudaEvent_t, cudaEvent_t>> spans;
  std::vector<cudaEvent_t> span_free;
  double gpu_ms = 0;
  PinnedPool *pinned = nullptr;
  std::vector<std::thread> preps;
  std::vector<std::thread> inits;
  std::thread worker;
  int worker_status = HEAT_OK;
};

namespace {

double now_ms(const heat_server *s) {
  return std::chrono::duration<double, std::milli>(Clock::now() - s->t0).count();
}

// Return a job's input buffers to the pool (after their upload completed).
void release_inputs(heat_server *s, Job *j) {
  s->pinned->put(j->kappa, j->kappa_cap);
  s->pinned->put(j->u0, j->u0_cap);
  j->kappa = j->u0 = nullptr;
  j->kappa_cap = j->u0_cap = 0;
}

void finish(heat_server *s, Job *j, int status, double l2, double cs) {
  heat_result r{};
  r.id = j->id;
  r.status = status;
  r.l2 = l2;
  r.checksum = cs;
  r.submit_ms = j->submit_ms;
  r.admit_ms = j->admit_ms;
  r.done_ms = now_ms(s);
  r.updates = status == HEAT_OK ? (double)(j->req.nx - 2) * (j->req.ny - 2) * (j->req.nz - 2) *
                                      (double)j->req.steps
                                : 0.0;
  std::lock_guard<std::mutex> lk(s->mu);
  s->done.push_back(r);
  if (status == HEAT_OK) {
    s->n_completed += 1;
    s->latencies.push_back(r.done_ms - r.submit_ms);
    s->updates_done += r.updates;
    s->last_done_ms = r.done_ms;
  } else {
    s->n_rejected += 1;
  }
  s->cv_idle.notify_all();
}

void prep_loop(heat_server *s) {
  cudaSetDevice(s->device);  // pinned allocations belong to the server's device context
  for (;;) {
    Job *j = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // Bound host memory held by prepared inputs (look-ahead of the queue).
      s->cv_prep.wait(lk, [&] {
        return s->stop || (!s->submitted.empty() && s->ready_bytes < s->prep_cap);
      });
      if (s->stop) return;
      j = s->submitted.front();
      s->submitted.pop_front();
      s->preparing += 1;
    }
    const heat_request &r = j->req;
    const size_t n = (size_t)r.nx * r.ny * r.nz;
    int rc = HEAT_OK;
    j->kappa = (double *)s->pinned->get(n * sizeof(double), &j->kappa_cap);
    j->u0 = (double *)s->pinned->get(n * sizeof(double), &j->u0_cap);
    if (!j->kappa || !j->u0) rc = HEAT_ENOMEM;
    if (rc == HEAT_OK)
      rc = heat_inputs_config(r.cfg, r.seed, r.nx, r.ny, r.nz, j->kappa, j->u0, &j->h, &j->dt);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->preparing -= 1;
      if (rc == HEAT_OK) {
        s->ready.push_back(j);
        s->ready_bytes += n * 16;
        s->cv_work.notify_one();
      }
    }
    if (rc != HEAT_OK) {
      release_inputs(s, j);
      finish(s, j, rc, 0, 0);
      delete j;
    }
  }
}

// Admit prepared jobs that fit (reserving their device bytes) and hand them
// to the init threads; returns the number admitted.
int admit(heat_server *s) {
  std::lock_guard<std::mutex> lk(s->mu);
  const int window = 8;  // how far past a blocked head the scan looks
  int looked = 0, n = 0;
  for (auto it = s->ready.begin(); it != s->ready.end() && looked < window; ++looked) {
    Job *j = *it;
    if (s->in_use + j->bytes <= s->budget) {
      s->in_use += j->bytes;
      s->peak = std::max(s->peak, s->in_use);
      s->ready_bytes -= (size_t)j->req.nx * j->req.ny * j->req.nz * 16;
      s->to_init.push_back(j);
      it = s->ready.erase(it);
      ++n;
    } else {
      ++it;
    }
  }
  if (n) {
    s->cv_prep.notify_all();
    s->cv_init.notify_all();
  }
  return n;
}

// Init thread: creates the contexts of admitted jobs (uploads, set-up kernels,
// waiting for them), off the worker thread that keeps the GPU fed with ticks.
void init_loop(heat_server *s) {
  cudaSetDevice(s->device);
  for (;;) {
    Job *j = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_init.wait(lk, [&] { return s->stop_init || !s->to_init.empty(); });
      if (s->to_init.empty()) return;
      j = s->to_init.front();
      s->to_init.pop_front();
      s->initing += 1;
    }
    heat_desc d{};
    d.nx = j->req.nx;
    d.ny = j->req.ny;
    d.nz = j->req.nz;
    d.h = j->h;
    d.dt = j->dt;
    d.kappa = j->kappa;
    d.u0 = j->u0;
    d.precision = j->req.precision;
    d.stream = nullptr;  // own stream: the context's work never waits on the batch
    int rc = heat_init(&j->ctx, &d);
    if (rc == HEAT_OK) rc = heat_sync(j->ctx);
    release_inputs(s, j);
    j->init_rc = rc;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->initing -= 1;
      s->inited.push_back(j);
    }
    s->cv_work.notify_one();
  }
}

// Add contexts that are ready to the batch; returns the number added.
int attach(heat_server *s) {
  std::deque<Job *> got;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    got.swap(s->inited);
  }
  int n = 0;
  for (Job *j : got) {
    int rc = j->init_rc;
    if (rc == HEAT_OK) rc = heat_batch_add(s->batch, j->ctx, j->req.steps);
    j->admit_ms = now_ms(s);
    if (rc != HEAT_OK) {
      if (j->ctx) heat_destroy(j->ctx);
      j->ctx = nullptr;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->in_use -= j->bytes;
      }
      finish(s, j, rc, 0, 0);
      delete j;
      continue;
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->n_admitted += 1;
      if (s->first_admit_ms < 0) s->first_admit_ms = j->admit_ms;
      s->resident.push_back(j);
    }
    ++n;
  }
  return n;
}

// Retire finished solves whose last tick has completed (all of them if
// `block`, waiting as needed).
void retire(heat_server *s, bool block) {
  std::vector<Job *> res;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    res = s->resident;
  }
  for (Job *j : res) {
    if (!j->finished) continue;
    if (j->finish_ev) {
      if (!block && cudaEventQuery(j->finish_ev) == cudaErrorNotReady) continue;
      cudaGetLastError();
      // The norm (on the context's stream) follows the tick's kernels.
      cudaStreamWaitEvent(j->ctx->stream, j->finish_ev, 0);
    }
    double l2 = 0, cs = 0;
    int rc = heat_norm(j->ctx, &l2, &cs);
    if (rc == HEAT_OK && j->req.field_out) rc = heat_get_field(j->ctx, j->req.field_out);
    heat_batch_remove(s->batch, j->ctx);
    heat_destroy(j->ctx);
    j->ctx = nullptr;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->in_use -= j->bytes;
      s->resident.erase(std::find(s->resident.begin(), s->resident.end(), j));
    }
    finish(s, j, rc, l2, cs);
    delete j;
  }
}

cudaEvent_t take_span_event(heat_server *s) {
  cudaEvent_t e = nullptr;
  if (!s->span_free.empty()) {
    e = s->span_free.back();
    s->span_free.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    e = nullptr;
  }
  return e;
}

// Add the spans of completed ticks to gpu_ms (all of them if `block`).
void collect_spans(heat_server *s, bool block) {
  while (!s->spans.empty()) {
    auto sp = s->spans.front();
    if (block) cudaEventSynchronize(sp.second);
    if (cudaEventQuery(sp.second) != cudaSuccess) {
      cudaGetLastError();
      break;
    }
    float ms = 0;
    if (cudaEventElapsedTime(&ms, sp.first, sp.second) == cudaSuccess) {
      std::lock_guard<std::mutex> lk(s->mu);
      s->gpu_ms += ms;
    }
    cudaGetLastError();
    s->spans.pop_front();
    s->span_free.push_back(sp.first);
    s->span_free.push_back(sp.second);
  }
}

cudaEvent_t take_event(heat_server *s) {
  cudaEvent_t e = nullptr;
  if (!s->ev_free.empty()) {
    e = s->ev_free.back();
    s->ev_free.pop_back();
  } else if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    e = nullptr;
  }
  return e;
}

// Return tick events no job refers to any more and whose ticks completed.
void recycle_events(heat_server *s) {
  while (s->ev_live.size() > 1) {
    cudaEvent_t e = s->ev_live.front();
    bool used = false;
    for (Job *j : s->resident) used |= (j->finish_ev == e);
    if (used || cudaEventQuery(e) == cudaErrorNotReady) break;
    cudaGetLastError();
    s->ev_live.pop_front();
    s->ev_free.push_back(e);
  }
}

void worker_loop(heat_server *s) {
  cudaSetDevice(s->device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // With contexts being created and nothing resident, wait for them
      // rather than rescanning a queue whose head cannot be admitted yet.
      const auto in_init = [&] { return !s->to_init.empty() || s->initing > 0; };
      s->cv_work.wait(lk, [&] {
        return s->stop || !s->resident.empty() || !s->inited.empty() ||
               (!s->ready.empty() && !in_init());
      });
      if (s->stop && s->resident.empty() && s->inited.empty() && !in_init()) break;
    }
    admit(s);
    attach(s);
    retire(s, false);
    std::vector<Job *> res;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      res = s->resident;
    }
    bool active = false;
    for (Job *j : res) {
      long long left = 0;
      heat_batch_pending(s->batch, j->ctx, &left);
      if (left > 0) active = true;
      else if (!j->finished) j->finished = true;  // nothing to run (0 steps)
    }
    if (active) {
      const double t = now_ms(s);
      long long taken = 0;
      cudaEvent_t span0 = take_span_event(s);
      if (span0) cudaEventRecord(span0, s->stream);
      int rc = heat::batch_run(s->batch, s->tick_steps, &taken, false);
      cudaEvent_t span1 = span0 ? take_span_event(s) : nullptr;
      if (span1) {
        cudaEventRecord(span1, s->stream);
        s->spans.emplace_back(span0, span1);
      } else if (span0) {
        s->span_free.push_back(span0);
      }
      cudaEvent_t ev = take_event(s);
      if (ev) {
        cudaEventRecord(ev, s->stream);
        s->ev_live.push_back(ev);
      }
      for (Job *j : res) {
        if (j->finished) continue;
        long long left = 0;
        heat_batch_pending(s->batch, j->ctx, &left);
        if (left == 0) {
          j->finished = true;
          j->finish_ev = ev;
        }
      }
      // At most queue_ticks ticks queued: wait for the oldest beyond that.
      if ((int)s->ev_live.size() >= s->queue_ticks)
        cudaEventSynchronize(s->ev_live[s->ev_live.size() - s->queue_ticks]);
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->busy_ms += now_ms(s) - t;
        if (rc != HEAT_OK) s->worker_status = rc;
      }
      recycle_events(s);
      collect_spans(s, false);
    } else {
      // Nothing left to run: retire what finished (waiting for its tick), and
      // reject requests that can never fit the budget.
      retire(s, true);
      recycle_events(s);
      std::vector<Job *> reject;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->resident.empty())
          for (auto it = s->ready.begin(); it != s->ready.end();) {
            if ((*it)->bytes > s->budget) {
              s->ready_bytes -= (size_t)(*it)->req.nx * (*it)->req.ny * (*it)->req.nz * 16;
              reject.push_back(*it);
              it = s->ready.erase(it);
            } else {
              ++it;
            }
          }
      }
      for (Job *j : reject) {
        release_inputs(s, j);
        finish(s, j, HEAT_EBUDGET, 0, 0);
        delete j;
      }
    }
  }
  cudaStreamSynchronize(s->stream);
  collect_spans(s, true);
  for (cudaEvent_t e : s->span_free) cudaEventDestroy(e);
  s->span_free.clear();
  for (cudaEvent_t e : s->ev_live) cudaEventDestroy(e);
  for (cudaEvent_t e : s->ev_free) cudaEventDestroy(e);
  s->ev_live.clear();
  s->ev_free.clear();
}

}  // namespace

extern "C" {

int heat_server_create(heat_server **out, size_t budget_bytes, int tick_steps, int prep_threads) {
  if (!out || budget_bytes == 0 || tick_steps < 1 || prep_threads < 1) return HEAT_EINVAL;
  *out = nullptr;
  heat_server *s = new (std::nothrow) heat_server();
  if (!s) return HEAT_ENOMEM;
  s->budget = budget_bytes;
  s->prep_cap = std::min<size_t>(budget_bytes, (size_t)16 << 30);
  s->tick_steps = tick_steps;
  s->t0 = Clock::now();
  cudaGetDevice(&s->device);
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete s;
    return HEAT_ECUDA;
  }
  // HEAT_SERVER_BATCH_FLAGS: heat_batch_create flags of the server's batch
  // (e.g. 1 = no graphs); a tuning knob.
  unsigned bflags = 0;
  if (const char *ev = std::getenv("HEAT_SERVER_BATCH_FLAGS")) bflags = (unsigned)std::atoi(ev);
  if (const char *ev = std::getenv("HEAT_SERVER_QUEUE_TICKS"))
    s->queue_ticks = std::max(1, std::min(8, std::atoi(ev)));
  int rc = heat_batch_create(&s->batch, s->stream, bflags);
  if (rc != HEAT_OK) {
    cudaStreamDestroy(s->stream);
    delete s;
    return rc;
  }
  s->pinned = new (std::nothrow) PinnedPool(s->prep_cap);
  if (!s->pinned) {
    heat_batch_destroy(s->batch);
    cudaStreamDestroy(s->stream);
    delete s;
    return HEAT_ENOMEM;
  }
  for (int t = 0; t < prep_threads; ++t) s->preps.emplace_back(prep_loop, s);
  for (int t = 0; t < 2; ++t) s->inits.emplace_back(init_loop, s);
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return HEAT_OK;
}

int heat_server_submit(heat_server *s, const heat_request *r, uint64_t *id_out) {
  if (!s || !r) return HEAT_EINVAL;
  if (r->nx < 3 || r->ny < 3 || r->nz < 3 || r->steps < 0 || r->cfg < 0 || r->cfg > 4 ||
      (r->precision != HEAT_FP64 && r->precision != HEAT_FP32C))
    return HEAT_EINVAL;
  Job *j = new (std::nothrow) Job();
  if (!j) return HEAT_ENOMEM;
  j->req = *r;
  j->bytes = request_bytes(*r);
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) {
    delete j;
    return HEAT_ESTATE;
  }
  j->id = s->next_id++;
  j->submit_ms = now_ms(s);
  s->n_submitted += 1;
  s->submitted.push_back(j);
  s->cv_prep.notify_one();
  if (id_out) *id_out = j->id;
  return HEAT_OK;
}

int heat_server_poll(heat_server *s, heat_result *out, int max, int *n_out) {
  if (!s || (!out && max > 0) || max < 0) return HEAT_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  int n = std::min<int>(max, (int)s->done.size());
  for (int i = 0; i < n; ++i) out[i] = s->done[i];
  s->done.erase(s->done.begin(), s->done.begin() + n);
  if (n_out) *n_out = n;
  return s->worker_status;
}

int heat_server_wait_idle(heat_server *s) {
  if (!s) return HEAT_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_idle.wait(lk, [&] {
    return (s->n_completed + s->n_rejected == s->n_submitted) || s->worker_status != HEAT_OK;
  });
  return s->worker_status;
}

int heat_server_stats(heat_server *s, heat_server_summary *st) {
  if (!s || !st) return HEAT_EINVAL;
  std::memset(st, 0, sizeof *st);
  std::vector<double> lat;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    st->submitted = s->n_submitted;
    st->admitted = s->n_admitted;
    st->completed = s->n_completed;
    st->rejected = s->n_rejected;
    st->resident = (long long)s->resident.size();
    st->queued = (long long)(s->submitted.size() + s->ready.size()) + s->preparing;
    st->budget_bytes = s->budget;
    st->bytes_in_use = s->in_use;
    st->peak_bytes = s->peak;
    st->busy_ms = s->busy_ms;
    st->gpu_ms = s->gpu_ms;
    st->updates = s->updates_done;
    const double span = s->last_done_ms - std::max(0.0, s->first_admit_ms);
    st->glups = span > 0 ? s->updates_done / (span * 1e-3) / 1e9 : 0.0;
    lat = s->latencies;
  }
  if (!lat.empty()) {
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) {
      size_t k = (size_t)std::min<double>((double)lat.size() - 1, p * (double)(lat.size() - 1) + 0.5);
      return lat[k];
    };
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    st->max_ms = lat.back();
    double sum = 0;
    for (double x : lat) sum += x;
    st->mean_ms = sum / (double)lat.size();
  }
  long long kl = 0, gl = 0, bs = 0;
  heat_batch_stats(s->batch, &kl, &gl, &bs);
  st->kernel_launches = kl;
  st->batch_steps = bs;
  return HEAT_OK;
}

int heat_server_destroy(heat_server *s) {
  if (!s) return HEAT_EINVAL;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_prep.notify_all();
  s->cv_work.notify_all();
  for (auto &t : s->preps) t.join();
  {
    // Requests not yet admitted are dropped (the prep threads have stopped);
    // admitted ones finish.
    std::lock_guard<std::mutex> lk(s->mu);
    for (Job *j : s->submitted) delete j;
    for (Job *j : s->ready) {
      release_inputs(s, j);
      delete j;
    }
    s->submitted.clear();
    s->ready.clear();
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop_init = true;
  }
  s->cv_init.notify_all();
  for (auto &t : s->inits) t.join();
  heat_batch_destroy(s->batch);
  cudaStreamDestroy(s->stream);
  delete s->pinned;
  delete s;
  return HEAT_OK;
}

}  // extern "C"
