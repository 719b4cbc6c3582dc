// Event server: continuous batching of independent hydro events on one GPU
// (the ccake_server_* entry points of include/ccake_gpu.h).
//
// One scheduler thread owns the GPU work. Each pass it
//   1. admits queued events (FIFO) while the resident device bytes stay within
//      the budget: context, upload, initialisation (e -> s inversion, first
//      smoothing) on the event's own stream;
//   2. for every running event whose last quantum has completed (a CUDA event
//      query, no blocking), reads the stop-rule probe the quantum left in
//      pinned memory (frozen-particle count, largest T, tau, error counters)
//      and either retires the event (every particle frozen out with
//      particlization, or tau at tau_max) or enqueues the next quantum:
//      steps_per_launch RK2 steps (CUDA-graph launches) and the probe;
//   3. sleeps briefly when nothing changed.
// Events therefore share the GPU through concurrent streams, and an event
// submitted while others run starts as soon as memory allows.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ccake_gpu.h"
#include "internal.hpp"

namespace {

using Clock = std::chrono::steady_clock;

struct Event {
  int64_t ticket = 0;
  ccake_config cfg{};
  double tau_max = 0.0;
  int64_t n = 0;
  std::vector<double> cols[10];   // x y eta e_or_s rhoB rhoS rhoQ ux uy ueta
  bool has[10] = {};
  ccake_ctx* ctx = nullptr;
  int32_t state = 0;              // 0 queued, 1 running, 2 done, 3 failed
  int32_t status = 0;
  int32_t steps = 0, frozen = 0;
  double tau = 0.0;
  Clock::time_point t_submit, t_admit, t_done;
  int64_t bytes = 0;
  bool counted = false;           // bytes included in the server's bytes_in_use
  bool inflight = false;
  int quantum = 0;
  cudaEvent_t mark = nullptr;
  ccake::Probe* dev = nullptr;
  ccake::Probe* host = nullptr;   // pinned
};

}  // namespace

struct ccake_server {
  ccake_server_config cfg{};
  int device = 0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv_idle;
  std::deque<Event*> queue;
  std::vector<Event*> running;
  std::map<int64_t, Event*> events;
  int64_t next_ticket = 1;
  int64_t bytes_in_use = 0;
  bool stop = false;
};

namespace {

void free_event_gpu(Event* e) {
  if (e->ctx) ccake_ctx_destroy(e->ctx);
  if (e->mark) cudaEventDestroy(e->mark);
  if (e->dev) cudaFree(e->dev);
  if (e->host) cudaFreeHost(e->host);
  e->ctx = nullptr;
  e->mark = nullptr;
  e->dev = nullptr;
  e->host = nullptr;
}

// Context, upload and initialisation of a queued event (scheduler thread).
ccake_status_t admit(Event* e) {
  ccake_status_t s = ccake_ctx_create(&e->cfg, &e->ctx);
  if (s) return s;
  ccake_particles_soa soa{};
  soa.n = e->n;
  const double* c[10];
  for (int k = 0; k < 10; k++) c[k] = e->has[k] ? e->cols[k].data() : nullptr;
  soa.x = c[0]; soa.y = c[1]; soa.eta = c[2]; soa.e_or_s = c[3]; soa.rhoB = c[4]; soa.rhoS = c[5];
  soa.rhoQ = c[6]; soa.ux = c[7]; soa.uy = c[8]; soa.ueta = c[9];
  if ((s = ccake_load_particles(e->ctx, &soa))) return s;
  if ((s = ccake_initialize(e->ctx))) return s;
  int64_t b = 0;
  ccake_device_bytes(e->ctx, &b);
  e->bytes = b;
  if (cudaEventCreateWithFlags(&e->mark, cudaEventDisableTiming) != cudaSuccess ||
      cudaMalloc(&e->dev, sizeof(ccake::Probe)) != cudaSuccess ||
      cudaMallocHost(&e->host, sizeof(ccake::Probe)) != cudaSuccess)
    return CCAKE_ERR_NOMEM;
  for (int k = 0; k < 10; k++) std::vector<double>().swap(e->cols[k]);   // host copy no longer needed
  e->tau = e->cfg.t0;
  return CCAKE_OK;
}

void scheduler(ccake_server* srv) {
  cudaSetDevice(srv->device);
  while (true) {
    bool progressed = false;
    // 1. admissions
    while (true) {
      Event* e = nullptr;
      {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return;
        if (srv->queue.empty() || (int)srv->running.size() >= srv->cfg.max_active) break;
        Event* head = srv->queue.front();
        const int64_t need = ccake_internal::estimate_bytes(head->cfg, head->n);
        if (!srv->running.empty() && srv->bytes_in_use + need > srv->cfg.hbm_budget_bytes) break;
        srv->queue.pop_front();
        srv->bytes_in_use += need;
        e = head;
        e->bytes = need;
      }
      const int64_t est = e->bytes;
      const ccake_status_t s = admit(e);
      std::lock_guard<std::mutex> lk(srv->mu);
      e->t_admit = Clock::now();
      srv->bytes_in_use += (s ? 0 : e->bytes) - est;
      if (s) {
        e->state = 3;
        e->status = s;
        e->t_done = Clock::now();
        free_event_gpu(e);
      } else {
        e->state = 1;
        e->counted = true;
        srv->running.push_back(e);
      }
      progressed = true;
    }
    // 2. running events
    std::vector<Event*> run;
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      run = srv->running;
    }
    for (Event* e : run) {
      if (e->inflight) {
        const cudaError_t q = cudaEventQuery(e->mark);
        if (q == cudaErrorNotReady) continue;
        e->inflight = false;
        progressed = true;
        bool failed = q != cudaSuccess;
        int32_t st = failed ? CCAKE_ERR_CUDA : 0;
        {
          std::lock_guard<std::mutex> lk(srv->mu);
          e->steps += e->quantum;
          if (!failed) e->tau = e->host->tau;
        }
        if (!failed) {
          const ccake::Probe& pr = *e->host;
          ccake_internal::ctx_set_time(e->ctx, pr.tau);
          // the failure raised first decides the event's status
          const ccake_status_t kind[4] = {CCAKE_ERR_EOS, CCAKE_ERR_NEG_ENTROPY, CCAKE_ERR_NONFINITE,
                                          CCAKE_ERR_CAPACITY};
          const int first = pr.err[ccake::E_FIRST] - 1;
          if (first >= 0 && first < 4) st = kind[first];
          else if (pr.err[ccake::E_EOS]) st = CCAKE_ERR_EOS;
          else if (pr.err[ccake::E_NEGS]) st = CCAKE_ERR_NEG_ENTROPY;
          else if (pr.err[ccake::E_NONFINITE]) st = CCAKE_ERR_NONFINITE;
          else if (pr.err[ccake::E_NBR_OVERFLOW]) st = CCAKE_ERR_CAPACITY;
          failed = st != 0;
          if (!failed) {
            // the reference's stop rule: every particle frozen out (with
            // particlization) or tau at tau_max
            const bool cold = e->cfg.particlization && pr.frozen >= e->n;
            if (cold || e->tau >= e->tau_max - 0.5 * e->cfg.dt) {
              std::lock_guard<std::mutex> lk(srv->mu);
              e->frozen = cold ? 1 : 0;
              e->state = 2;
              e->t_done = Clock::now();
              srv->running.erase(std::find(srv->running.begin(), srv->running.end(), e));
              continue;
            }
          }
        }
        if (failed) {
          cudaGetLastError();
          std::lock_guard<std::mutex> lk(srv->mu);
          e->state = 3;
          e->status = st;
          e->t_done = Clock::now();
          srv->running.erase(std::find(srv->running.begin(), srv->running.end(), e));
          continue;
        }
      }
      // next quantum
      const int left = (int)std::ceil((e->tau_max - e->tau) / e->cfg.dt - 0.5);
      const int k = std::max(1, std::min(srv->cfg.steps_per_launch, left));
      ccake_status_t s = ccake_internal::step_enqueue(e->ctx, k);
      if (!s) s = ccake_internal::probe_enqueue(e->ctx, e->dev, e->host);
      if (!s && cudaEventRecord(e->mark, ccake_internal::ctx_stream(e->ctx)) != cudaSuccess) s = CCAKE_ERR_CUDA;
      if (s) {
        std::lock_guard<std::mutex> lk(srv->mu);
        e->state = 3;
        e->status = s;
        e->t_done = Clock::now();
        srv->running.erase(std::find(srv->running.begin(), srv->running.end(), e));
        continue;
      }
      e->quantum = k;
      e->inflight = true;
      progressed = true;
    }
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      if (srv->queue.empty() && srv->running.empty()) srv->cv_idle.notify_all();
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

}  // namespace

extern "C" {

ccake_status_t ccake_server_create(const ccake_server_config* cfg, ccake_server** out) {
  if (!out) return CCAKE_ERR_INVALID;
  *out = nullptr;
  ccake_server* srv = new ccake_server;
  if (cfg) srv->cfg = *cfg;
  if (srv->cfg.max_active <= 0) srv->cfg.max_active = 32;
  if (srv->cfg.steps_per_launch <= 0) srv->cfg.steps_per_launch = 20;
  cudaGetDevice(&srv->device);
  if (srv->cfg.hbm_budget_bytes <= 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      delete srv;
      return CCAKE_ERR_CUDA;
    }
    srv->cfg.hbm_budget_bytes = (int64_t)(0.8 * (double)fr);
  }
  srv->th = std::thread(scheduler, srv);
  *out = srv;
  return CCAKE_OK;
}

ccake_status_t ccake_server_destroy(ccake_server* srv) {
  if (!srv) return CCAKE_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->th.join();
  for (auto& kv : srv->events) {
    Event* e = kv.second;
    if (e->ctx) cudaStreamSynchronize(ccake_internal::ctx_stream(e->ctx));
    free_event_gpu(e);
    delete e;
  }
  delete srv;
  return CCAKE_OK;
}

ccake_status_t ccake_server_submit(ccake_server* srv, const ccake_config* cfg, const ccake_particles_soa* p,
                                   double tau_max, int64_t* ticket) {
  if (!srv || !cfg || !p || !ticket || p->n <= 0 || !p->x || !p->y || !p->e_or_s || !p->ux || !p->uy)
    return CCAKE_ERR_INVALID;
  if (!(tau_max > cfg->t0) || !(cfg->dt > 0)) return CCAKE_ERR_INVALID;
  // an event that could never fit the budget is refused at once (it would
  // otherwise wait at the head of the queue for memory that never frees)
  if (ccake_internal::estimate_bytes(*cfg, p->n) > srv->cfg.hbm_budget_bytes) {
    *ticket = 0;
    return CCAKE_ERR_CAPACITY;
  }
  Event* e = new Event;
  e->cfg = *cfg;
  e->tau_max = tau_max;
  e->n = p->n;
  const double* c[10] = {p->x, p->y, p->eta, p->e_or_s, p->rhoB, p->rhoS, p->rhoQ, p->ux, p->uy, p->ueta};
  for (int k = 0; k < 10; k++)
    if (c[k]) {
      e->cols[k].assign(c[k], c[k] + p->n);
      e->has[k] = true;
    }
  e->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(srv->mu);
  e->ticket = srv->next_ticket++;
  srv->events[e->ticket] = e;
  srv->queue.push_back(e);
  *ticket = e->ticket;
  return CCAKE_OK;
}

ccake_status_t ccake_estimate_device_bytes(const ccake_config* cfg, int64_t n, int64_t* bytes) {
  if (!cfg || n <= 0 || !bytes) return CCAKE_ERR_INVALID;
  *bytes = ccake_internal::estimate_bytes(*cfg, n);
  return CCAKE_OK;
}

ccake_status_t ccake_server_poll(ccake_server* srv, int64_t ticket, ccake_event_result* out) {
  if (!srv || !out) return CCAKE_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->events.find(ticket);
  if (it == srv->events.end()) return CCAKE_ERR_INVALID;
  const Event* e = it->second;
  std::memset(out, 0, sizeof(*out));
  out->ticket = e->ticket;
  out->particles = e->n;
  out->state = e->state;
  out->status = e->status;
  out->steps = e->steps;
  out->frozen = e->frozen;
  out->tau = e->tau;
  out->device_bytes = e->bytes;
  if (e->state >= 1) out->queue_s = std::chrono::duration<double>(e->t_admit - e->t_submit).count();
  if (e->state >= 2) out->latency_s = std::chrono::duration<double>(e->t_done - e->t_submit).count();
  return CCAKE_OK;
}

ccake_status_t ccake_server_wait_all(ccake_server* srv) {
  if (!srv) return CCAKE_ERR_INVALID;
  std::unique_lock<std::mutex> lk(srv->mu);
  srv->cv_idle.wait(lk, [&] { return srv->stop || (srv->queue.empty() && srv->running.empty()); });
  return CCAKE_OK;
}

ccake_status_t ccake_server_copy_out(ccake_server* srv, int64_t ticket, const char* field, double* host_out) {
  if (!srv || !field || !host_out) return CCAKE_ERR_INVALID;
  Event* e = nullptr;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->events.find(ticket);
    if (it == srv->events.end()) return CCAKE_ERR_INVALID;
    e = it->second;
    if (e->state != 2) return CCAKE_ERR_STATE;
  }
  return ccake_copy_out(e->ctx, field, host_out);
}

ccake_status_t ccake_server_release(ccake_server* srv, int64_t ticket) {
  if (!srv) return CCAKE_ERR_INVALID;
  Event* e = nullptr;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->events.find(ticket);
    if (it == srv->events.end()) return CCAKE_ERR_INVALID;
    e = it->second;
    if (e->state < 2) return CCAKE_ERR_STATE;
    srv->events.erase(it);
    if (e->counted) srv->bytes_in_use -= e->bytes;
  }
  free_event_gpu(e);
  delete e;
  return CCAKE_OK;
}

}  // extern "C"
