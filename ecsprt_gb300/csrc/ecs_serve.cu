// Request loop of libecsgpu (ecs_serve.h): worker threads, first-come
// first-served admission against an HBM budget, resident slots, solve
// requests as one CUDA-graph launch each, simulation instances stepped in
// turn with the other work.
//
// The reference has no counterpart: its solver (src/solver.c:107-203) and
// simulation (src/pic.c) each run one instance per process.  What a slot
// computes is exactly what ecs_solve_density / ecs_step compute on their own.

#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "ecs_internal.cuh"
#include "ecs_serve.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Parameters equal field by field (the int block and the double block; the
// bytes between them are padding).
bool same_params(const EcsParams &a, const EcsParams &b) {
  constexpr size_t ints = offsetof(EcsParams, rhs_type) + sizeof(int32_t);
  constexpr size_t dbl = offsetof(EcsParams, dx);
  static_assert(sizeof(EcsParams) > dbl, "EcsParams layout");
  return memcmp(&a, &b, ints) == 0 && memcmp((const char *)&a + dbl, (const char *)&b + dbl, sizeof(EcsParams) - dbl) == 0;
}

struct Slot {
  EcsCtx *ctx = nullptr;
  cudaStream_t stream = nullptr;  // the slot's own stream, prioritised by grid size
  EcsParams p;
  int kind = ECS_SERVE_SOLVE;
  int64_t bytes = 0;
  bool busy = false;
  bool broken = false;  // a request timed out on it: its stream may still run
  uint64_t last_used = 0;
  int64_t launches_seen = 0;
};

struct Job {
  int64_t id = 0;
  int kind = ECS_SERVE_SOLVE;
  EcsParams p;
  EcsSolveRequest solve;
  EcsSimRequest sim;
  int64_t bytes = 0;
  double t_submit = 0.0, t_admit = 0.0;
  Slot *slot = nullptr;
  bool fresh = false;   // the slot is new: create its context first
  bool reused = false;
  int steps_done = 0;
  double device_seconds = 0.0;
  EcsSolveStats last;
  int status = ECS_OK;
  char message[160] = {0};
};

}  // namespace

struct EcsServer {
  EcsServeConfig cfg;
  int device = 0;
  int prio_least = 0, prio_greatest = 0;  // the device's stream priority range
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job *> pending;  // submitted, not admitted (served in order)
  std::deque<Job *> ready;    // admitted simulations waiting for their next step
  std::deque<EcsServeResult> done;
  std::vector<Slot *> slots;
  std::vector<std::thread> workers;
  bool quit = false;
  int64_t next_id = 1;
  int64_t used = 0, peak_used = 0;
  int running = 0, peak_running = 0;
  int64_t submitted = 0, completed = 0, failed = 0, polled = 0;
  int64_t created = 0, hits = 0, evictions = 0, launches = 0;
  uint64_t tick = 0;
  double busy_since = 0.0, busy_total = 0.0;
  std::vector<double> solve_lat, step_lat;
};

namespace {

// Admission of the oldest pending request (lock held).  Takes an idle slot
// with the same parameters, or charges a new slot to the budget, evicting
// idle solve slots (least recently used first) when that makes it fit.
bool admit(EcsServer *s, Job *j, std::vector<Slot *> &evict) {
  if (j->kind == ECS_SERVE_SOLVE) {
    for (Slot *sl : s->slots) {
      if (!sl->busy && !sl->broken && sl->kind == ECS_SERVE_SOLVE && same_params(sl->p, j->p)) {
        sl->busy = true;
        j->slot = sl;
        j->reused = true;
        s->hits++;
        return true;
      }
    }
  }
  const int64_t budget = s->cfg.hbm_budget_bytes;
  if (s->used + j->bytes > budget) {
    std::vector<Slot *> idle;
    int64_t freeable = 0;
    for (Slot *sl : s->slots)
      if (!sl->busy && !sl->broken) {
        idle.push_back(sl);
        freeable += sl->bytes;
      }
    if (s->used - freeable + j->bytes > budget) return false;
    std::sort(idle.begin(), idle.end(), [](const Slot *a, const Slot *b) { return a->last_used < b->last_used; });
    for (Slot *sl : idle) {
      if (s->used + j->bytes <= budget) break;
      s->slots.erase(std::find(s->slots.begin(), s->slots.end(), sl));
      s->used -= sl->bytes;
      s->evictions++;
      evict.push_back(sl);
    }
  }
  Slot *sl = new Slot();
  sl->p = j->p;
  sl->kind = j->kind;
  sl->bytes = j->bytes;
  sl->busy = true;
  s->slots.push_back(sl);
  s->used += j->bytes;
  s->peak_used = std::max(s->peak_used, s->used);
  s->created++;
  j->slot = sl;
  j->fresh = true;
  return true;
}

// Next unit of work (lock held): the oldest pending request if it can be
// admitted (nothing overtakes it), else the next step of a simulation.
Job *take_work(EcsServer *s, std::vector<Slot *> &evict) {
  if (!s->pending.empty()) {
    Job *j = s->pending.front();
    if (admit(s, j, evict)) {
      s->pending.pop_front();
      j->t_admit = now_s();
      return j;
    }
  }
  if (!s->ready.empty()) {
    Job *j = s->ready.front();
    s->ready.pop_front();
    return j;
  }
  return nullptr;
}

// A slot's context on a stream of its own whose priority grows with the
// grid (8 cells a step of the range from 2^15 cells on): a large solve is not
// starved by the small ones around it, which keeps the latency tail short.
int create_slot_ctx(EcsServer *s, Slot *sl, const EcsParams &p, int64_t np) {
  const int64_t n = (int64_t)p.Nx * p.Ny * p.Nz;
  int level = 0;
  for (int64_t c = (int64_t)1 << 15; c < n && level < 8; c <<= 3) level++;
  int prio = s->prio_least - level;  // numerically smaller is higher priority
  if (prio < s->prio_greatest) prio = s->prio_greatest;
  if (cudaStreamCreateWithPriority(&sl->stream, cudaStreamNonBlocking, prio) != cudaSuccess) {
    cudaGetLastError();
    sl->stream = nullptr;
  }
  const int rc = ecs_ctx_create(&p, s->cfg.precision, np, sl->stream, &sl->ctx);
  if (rc && sl->stream) {
    cudaStreamDestroy(sl->stream);
    sl->stream = nullptr;
  }
  return rc;
}
void destroy_slot_ctx(Slot *sl) {
  if (sl->ctx) ecs_ctx_destroy(sl->ctx);
  if (sl->stream) cudaStreamDestroy(sl->stream);
  sl->ctx = nullptr;
  sl->stream = nullptr;
}

void fail(Job *j, int rc, const char *msg) {
  j->status = rc;
  snprintf(j->message, sizeof j->message, "%s", msg ? msg : ecs_status_string(rc));
}

// Wait for an event with a deadline (the context's own work only).
int wait_event(EcsCtx *ctx, cudaEvent_t ev, double timeout) {
  const double t_end = now_s() + timeout;
  for (;;) {
    cudaError_t e = cudaEventQuery(ev);
    if (e == cudaSuccess) return ECS_OK;
    if (e != cudaErrorNotReady) return ecs_cuda_check(ctx, e, "request wait");
    if (now_s() > t_end) return ecs_fail(ctx, ECS_ERR_TIMEOUT, "request still running after %.1f s", timeout);
    std::this_thread::yield();
  }
}

void run_solve(EcsServer *s, Job *j) {
  Slot *sl = j->slot;
  int rc;
  if (j->fresh) {
    if ((rc = create_slot_ctx(s, sl, j->p, 0))) {
      fail(j, rc, ecs_last_error(nullptr));
      return;
    }
    j->fresh = false;
  }
  EcsCtx *ctx = sl->ctx;
  const EcsSolveRequest &r = j->solve;
  rc = ecs_request_launch(ctx, r.density, r.phi_out, r.flux_scale, r.rtol, r.max_it);
  if (!rc) {
    const double timeout = s->cfg.timeout_seconds > 0 ? s->cfg.timeout_seconds : 60.0;
    rc = wait_event(ctx, ctx->ev_solve[1], timeout);
    if (rc == ECS_ERR_TIMEOUT) sl->broken = true;
  }
  if (!rc) rc = ecs_request_finish(ctx, &j->last);
  j->device_seconds = j->last.seconds;
  if (rc) fail(j, rc, ecs_last_error(ctx));
}

// One step of a simulation (its slot is created and loaded on the first).
void run_sim_step(EcsServer *s, Job *j) {
  Slot *sl = j->slot;
  const EcsSimRequest &r = j->sim;
  int rc;
  if (j->fresh) {
    if ((rc = create_slot_ctx(s, sl, j->p, r.np))) {
      fail(j, rc, ecs_last_error(nullptr));
      return;
    }
    j->fresh = false;
    ecs_set_seed(sl->ctx, r.seed);
    if (r.sort_every > 0) ecs_set_sort_every(sl->ctx, r.sort_every);
    if ((rc = ecs_particles_upload(sl->ctx, r.pos, r.vel, r.np))) {
      fail(j, rc, ecs_last_error(sl->ctx));
      return;
    }
  }
  EcsCtx *ctx = sl->ctx;
  EcsStepStats st;
  memset(&st, 0, sizeof st);
  const double t0 = now_s();
  rc = ecs_step(ctx, r.dt, r.rtol, r.max_it, &st);
  const double t1 = now_s();
  if (r.step_seconds) r.step_seconds[j->steps_done] = t1 - t0;
  j->steps_done++;
  j->device_seconds += st.solve.seconds;
  j->last = st.solve;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->step_lat.push_back(t1 - t0);
  }
  if (rc) {
    fail(j, rc, ecs_last_error(ctx));
    return;
  }
  if (j->steps_done == r.nsteps) {
    if (r.phi_out && (rc = ecs_phi_download(ctx, r.phi_out))) fail(j, rc, ecs_last_error(ctx));
    else if (r.pos_out && r.vel_out && (rc = ecs_particles_download(ctx, r.pos_out, r.vel_out)))
      fail(j, rc, ecs_last_error(ctx));
  }
}

EcsServeResult result_of(const Job *j, double t_end) {
  EcsServeResult res;
  memset(&res, 0, sizeof res);
  res.id = j->id;
  res.kind = j->kind;
  res.status = j->status;
  res.latency = t_end - j->t_submit;
  res.queued = j->t_admit > 0 ? j->t_admit - j->t_submit : res.latency;
  res.device_seconds = j->device_seconds;
  res.solve = j->last;
  res.steps = j->steps_done;
  res.slot_reused = j->reused ? 1 : 0;
  memcpy(res.message, j->message, sizeof res.message);
  return res;
}

void worker_main(EcsServer *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    Job *j = nullptr;
    std::vector<Slot *> evict;
    while (!s->quit && !(j = take_work(s, evict))) s->cv_work.wait(lk);
    if (!j) return;
    if (s->running++ == 0) s->busy_since = now_s();
    s->peak_running = std::max(s->peak_running, s->running);
    lk.unlock();
    for (Slot *e : evict) {
      destroy_slot_ctx(e);
      delete e;
    }
    if (j->kind == ECS_SERVE_SOLVE) run_solve(s, j);
    else run_sim_step(s, j);
    Slot *sl = j->slot;
    const int64_t nl = sl->ctx ? ecs_launch_count(sl->ctx) : 0;
    const bool finished = j->kind == ECS_SERVE_SOLVE || j->status != ECS_OK || j->steps_done >= j->sim.nsteps;
    // a simulation's slot, or a slot whose context never came up, goes away
    const bool drop = finished && (j->kind == ECS_SERVE_SIM || !sl->ctx);
    if (drop) destroy_slot_ctx(sl);
    const double t_end = now_s();
    lk.lock();
    s->launches += nl - sl->launches_seen;
    sl->launches_seen = nl;
    if (--s->running == 0) s->busy_total += t_end - s->busy_since;
    if (!finished) {
      s->ready.push_back(j);
    } else {
      if (drop) {
        s->slots.erase(std::find(s->slots.begin(), s->slots.end(), sl));
        s->used -= sl->bytes;
        delete sl;
      } else if (!sl->broken) {
        sl->busy = false;
        sl->last_used = ++s->tick;
      }
      EcsServeResult res = result_of(j, t_end);
      if (j->status == ECS_OK) s->completed++;
      else s->failed++;
      if (j->kind == ECS_SERVE_SOLVE && j->status == ECS_OK) s->solve_lat.push_back(res.latency);
      s->done.push_back(res);
      delete j;
      s->cv_done.notify_all();
    }
    s->cv_work.notify_all();
  }
}

int submit(EcsServer *s, Job *j, int64_t *id) {
  if (j->bytes > s->cfg.hbm_budget_bytes) {
    delete j;
    return ECS_ERR_NOMEM;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->quit) {
    delete j;
    return ECS_ERR_STATE;
  }
  j->id = s->next_id++;
  j->t_submit = now_s();
  s->pending.push_back(j);
  s->submitted++;
  if (id) *id = j->id;
  s->cv_work.notify_one();
  return ECS_OK;
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  size_t r = (size_t)std::ceil(q * (double)v.size());  // nearest rank
  if (r < 1) r = 1;
  return v[std::min(r, v.size()) - 1];
}

bool grid_ok(const EcsParams *p) {
  return p && p->ndim == 3 && p->Nx > 0 && p->Ny > 0 && p->Nz > 0;
}

}  // namespace

extern "C" {

int64_t ecs_serve_request_bytes(const EcsParams *p, int precision, int kind, int64_t np) {
  if (!p) return -1;
  return ecs_ctx_device_bytes(p, precision, kind == ECS_SERVE_SIM ? np : 0);
}

int ecs_serve_create(const EcsServeConfig *cfg, EcsServer **out) {
  if (!cfg || !out || cfg->max_inflight < 1 || cfg->max_inflight > 256 || cfg->hbm_budget_bytes <= 0 ||
      (cfg->precision != ECS_PREC_FP64 && cfg->precision != ECS_PREC_MIXED))
    return ECS_ERR_INVALID;
  *out = nullptr;
  EcsServer *s = new (std::nothrow) EcsServer();
  if (!s) return ECS_ERR_NOMEM;
  s->cfg = *cfg;
  cudaGetDevice(&s->device);
  if (cudaDeviceGetStreamPriorityRange(&s->prio_least, &s->prio_greatest) != cudaSuccess) {
    cudaGetLastError();
    s->prio_least = s->prio_greatest = 0;
  }
  for (int w = 0; w < cfg->max_inflight; w++) s->workers.emplace_back(worker_main, s);
  *out = s;
  return ECS_OK;
}

int ecs_serve_destroy(EcsServer *s) {
  if (!s) return ECS_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->quit = true;
    s->cv_work.notify_all();
  }
  for (auto &t : s->workers) t.join();
  for (Job *j : s->pending) delete j;
  for (Job *j : s->ready) delete j;
  for (Slot *sl : s->slots) {
    destroy_slot_ctx(sl);
    delete sl;
  }
  delete s;
  return ECS_OK;
}

int ecs_serve_submit_solve(EcsServer *s, const EcsParams *p, const EcsSolveRequest *r, int64_t *id) {
  if (!s || !grid_ok(p) || !r || !r->density || !r->phi_out || !(r->rtol > 0) || r->max_it < 1) return ECS_ERR_INVALID;
  Job *j = new (std::nothrow) Job();
  if (!j) return ECS_ERR_NOMEM;
  j->kind = ECS_SERVE_SOLVE;
  j->p = *p;
  j->solve = *r;
  memset(&j->last, 0, sizeof j->last);
  j->bytes = ecs_serve_request_bytes(p, s->cfg.precision, ECS_SERVE_SOLVE, 0);
  return submit(s, j, id);
}

int ecs_serve_submit_sim(EcsServer *s, const EcsParams *p, const EcsSimRequest *r, int64_t *id) {
  if (!s || !grid_ok(p) || !r || r->np < 0 || (r->np > 0 && (!r->pos || !r->vel)) || r->nsteps < 1 ||
      !(r->rtol > 0) || r->max_it < 1 || !(r->dt > 0))
    return ECS_ERR_INVALID;
  Job *j = new (std::nothrow) Job();
  if (!j) return ECS_ERR_NOMEM;
  j->kind = ECS_SERVE_SIM;
  j->p = *p;
  j->sim = *r;
  memset(&j->last, 0, sizeof j->last);
  j->bytes = ecs_serve_request_bytes(p, s->cfg.precision, ECS_SERVE_SIM, r->np);
  return submit(s, j, id);
}

int ecs_serve_poll(EcsServer *s, EcsServeResult *out, int max, int timeout_ms) {
  if (!s || !out || max < 1) return ECS_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && timeout_ms > 0)
    s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [s] { return !s->done.empty(); });
  int n = 0;
  while (n < max && !s->done.empty()) {
    out[n++] = s->done.front();
    s->done.pop_front();
  }
  s->polled += n;
  return n;
}

int64_t ecs_serve_pending(EcsServer *s) {
  if (!s) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  return s->submitted - s->polled;
}

int ecs_serve_stats(EcsServer *s, EcsServeStats *st) {
  if (!s || !st) return ECS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  memset(st, 0, sizeof *st);
  st->submitted = s->submitted;
  st->completed = s->completed;
  st->failed = s->failed;
  st->solves = (int64_t)s->solve_lat.size();
  st->solve_p50 = percentile(s->solve_lat, 0.50);
  st->solve_p99 = percentile(s->solve_lat, 0.99);
  double sum = 0.0, mx = 0.0;
  for (double v : s->solve_lat) {
    sum += v;
    mx = std::max(mx, v);
  }
  st->solve_mean = s->solve_lat.empty() ? 0.0 : sum / (double)s->solve_lat.size();
  st->solve_max = mx;
  st->steps = (int64_t)s->step_lat.size();
  st->step_p50 = percentile(s->step_lat, 0.50);
  st->step_p99 = percentile(s->step_lat, 0.99);
  st->device_bytes = s->used;
  st->peak_device_bytes = s->peak_used;
  st->peak_inflight = s->peak_running;
  st->slots = (int32_t)s->slots.size();
  st->slots_created = s->created;
  st->slot_hits = s->hits;
  st->evictions = s->evictions;
  st->gpu_launches = s->launches;
  st->busy_seconds = s->busy_total + (s->running > 0 ? now_s() - s->busy_since : 0.0);
  return ECS_OK;
}

int ecs_serve_reset_stats(EcsServer *s) {
  if (!s) return ECS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->solve_lat.clear();
  s->step_lat.clear();
  s->submitted -= s->polled;
  s->polled = 0;
  s->completed = s->failed = 0;
  s->created = s->hits = s->evictions = s->launches = 0;
  s->peak_used = s->used;
  s->peak_running = s->running;
  s->busy_total = 0.0;
  if (s->running > 0) s->busy_since = now_s();
  return ECS_OK;
}

int ecs_solve_density(EcsCtx *ctx, const double *density, const double flux_scale[3], double rtol, int max_it,
                      double *phi_out, EcsSolveStats *stats) {
  if (!ctx || !density || !flux_scale || !phi_out || !(rtol > 0) || max_it < 1) return ECS_ERR_INVALID;
  int rc = ecs_request_launch(ctx, density, phi_out, flux_scale, rtol, max_it);
  if (rc) return rc;
  ECS_CUDA(ctx, cudaEventSynchronize(ctx->ev_solve[1]));
  EcsSolveStats st;
  memset(&st, 0, sizeof st);
  rc = ecs_request_finish(ctx, &st);
  if (stats) *stats = st;
  return rc;
}

void *ecs_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void ecs_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

}  // extern "C"
