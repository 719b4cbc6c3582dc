// Event server: continuous batching of independent hydro events on one GPU
// (the ccake_server_* entry points of include/ccake_gpu.h).
//
// One scheduler thread owns the GPU work. Each pass it
//   1. admits queued events (FIFO) while the resident device bytes stay within
//      the budget: context, upload, initialisation (e -> s inversion, first
//      smoothing);
//   2. advances the resident events.
//      Mixed-form events (precision 1, no hypersurface output) of the same
//      dimension form a group: their particles are advanced together by
//      grouped launches, one launch of each step kernel for every
//      kGroupMax events of the group (GroupArgs: the events' descriptors in
//      the launch's parameters, their stop-rule state in device memory).
//      One CUDA graph holds a candidate-list period of RK2 steps for the
//      whole group: before every step the device applies each event's stop
//      rule (every particle frozen out with particlization, tau_max, or a
//      failure flagged by the kernels) and retires the event, whose blocks
//      then return at once. Between periods the host rebuilds each event's
//      candidate list (growing its capacity if needed), retires the events
//      the device stopped, lets admitted events join, and re-captures the
//      graph when the group changed. A group event's particles see exactly
//      the kernels they see when the event runs alone (ccake_step with
//      precision 1 is a group of one), so its results are the same bits.
//      Other events advance each on its own stream in quanta of
//      steps_per_launch RK2 steps (graph launches) followed by a one-block
//      probe (frozen count, largest T, tau, error counters) copied to pinned
//      memory; their stop rule is applied after each quantum;
//   3. sleeps briefly when nothing changed. Completion is seen by
//      cudaEventQuery; the thread blocks on the GPU only for the list builds
//      between a group's periods.
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
  bool grouped = false;           // advanced by its dimension's group
  bool inflight = false;
  int quantum = 0;
  cudaEvent_t mark = nullptr;
  ccake::Probe* dev = nullptr;
  ccake::Probe* host = nullptr;   // pinned
};

// Resident mixed-form events of one dimension, advanced together.
struct Group {
  int dim = 2;
  int period = 0;                  // RK2 steps a graph launch advances (a list period)
  std::vector<Event*> members;     // order of the state table
  std::vector<Event*> joining;     // admitted, join at the next period
  ccake::EventState* d_state = nullptr;
  ccake::EventState* h_state = nullptr;   // pinned: the states after a period
  int state_cap = 0;
  std::vector<ccake::GroupArgs> chunks;   // launch arguments, kGroupMax events each
  int32_t* h_cand = nullptr;       // pinned: largest candidate count of each event's build
  int cand_cap = 0;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t mark = nullptr;
  bool dirty = true, inflight = false;
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
  Group groups[2];                 // dimension 2 and 3
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

void free_group(Group& g) {
  if (g.stream) cudaStreamSynchronize(g.stream);
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  if (g.d_state) cudaFree(g.d_state);
  if (g.h_state) cudaFreeHost(g.h_state);
  if (g.h_cand) cudaFreeHost(g.h_cand);
  if (g.mark) cudaEventDestroy(g.mark);
  if (g.stream) cudaStreamDestroy(g.stream);
  g = Group{};
}

bool alloc_probe(Event* e) {
  return cudaEventCreateWithFlags(&e->mark, cudaEventDisableTiming) == cudaSuccess &&
         cudaMalloc(&e->dev, sizeof(ccake::Probe)) == cudaSuccess &&
         cudaMallocHost(&e->host, sizeof(ccake::Probe)) == cudaSuccess;
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
  if (!e->grouped && !alloc_probe(e)) return CCAKE_ERR_NOMEM;
  if (e->grouped && (s = ccake_internal::group_join(e->ctx))) return s;
  for (int k = 0; k < 10; k++) std::vector<double>().swap(e->cols[k]);   // host copy no longer needed
  e->tau = e->cfg.t0;
  return CCAKE_OK;
}

bool groupable(const ccake_config& c) {
  return c.precision == 1 && !(c.particlization && c.surface) && !c.using_diffusion;
}

void finish(ccake_server* srv, Event* e, int32_t state, int32_t status) {
  std::lock_guard<std::mutex> lk(srv->mu);
  e->state = state;
  e->status = status;
  e->t_done = Clock::now();
  auto it = std::find(srv->running.begin(), srv->running.end(), e);
  if (it != srv->running.end()) srv->running.erase(it);
}

// Capacity for `need` entries, at least doubling (cap is updated only on success).
int grown(int cap, int need) { return std::max(need, 2 * cap + 8); }

template <class T>
bool ensure_device(T*& p, int& cap, int need) {
  if (need <= cap) return true;
  const int c = grown(cap, need);
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  if (cudaMalloc(&p, (size_t)c * sizeof(T)) != cudaSuccess) return false;
  cap = c;
  return true;
}

template <class T>
bool ensure_pinned(T*& p, int& cap, int need) {
  if (need <= cap) return true;
  const int c = grown(cap, need);
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  if (cudaMallocHost(&p, (size_t)c * sizeof(T)) != cudaSuccess) return false;
  cap = c;
  return true;
}

// State table, launch arguments and period graph of the group's members.
ccake_status_t rebuild_group(Group& g) {
  const int nev = (int)g.members.size();
  int pinned_cap = g.state_cap;   // the pinned copy grows with the device table
  if (!ensure_pinned(g.h_state, pinned_cap, nev)) return CCAKE_ERR_NOMEM;
  if (!ensure_device(g.d_state, g.state_cap, nev)) return CCAKE_ERR_NOMEM;
  std::vector<ccake::EventState> st((size_t)nev);
  g.chunks.clear();
  bool freeze = false;
  for (int k = 0; k < nev; k++) {
    Event* e = g.members[(size_t)k];
    ccake::EventState& x = st[(size_t)k];
    std::memset(&x, 0, sizeof(x));
    x.tau_max = e->tau_max;
    x.tau = e->tau;
    x.steps = e->steps;
    x.active = 1;
    freeze = freeze || e->cfg.particlization;
    if (k % ccake::kGroupMax == 0) {
      g.chunks.emplace_back();
      ccake::GroupArgs& a = g.chunks.back();
      std::memset(&a, 0, sizeof(a));
      a.state = g.d_state + k;
    }
    ccake::GroupArgs& a = g.chunks.back();
    ccake_internal::group_desc(e->ctx, &a.ev[a.nev]);
    const int nb = (int)((e->n + ccake::kBlock - 1) / ccake::kBlock);
    a.first_block[a.nev + 1] = a.first_block[a.nev] + nb;
    a.nev++;
  }
  if (cudaMemcpyAsync(g.d_state, st.data(), (size_t)nev * sizeof(ccake::EventState), cudaMemcpyHostToDevice,
                      g.stream) != cudaSuccess ||
      cudaStreamSynchronize(g.stream) != cudaSuccess)
    return CCAKE_ERR_CUDA;
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  g.exec = nullptr;
  g.graph = nullptr;
  if (cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return CCAKE_ERR_CUDA;
  for (int k = 0; k < g.period; k++) {
    for (const ccake::GroupArgs& a : g.chunks) ccake::launch_stop_group(a, g.stream);
    for (int sub = 1; sub <= 2; sub++) {
      for (const ccake::GroupArgs& a : g.chunks) ccake::launch_passA_mixed(a, g.dim, g.stream);
      for (const ccake::GroupArgs& a : g.chunks)
        ccake::launch_passB_mixed(a, g.dim, ccake::B_EOM | ccake::B_UPDATE | (sub == 2 ? ccake::B_WRITE_Y0 : 0),
                                  sub, g.stream);
      for (const ccake::GroupArgs& a : g.chunks) ccake::launch_clock_group(a, sub, g.stream);
    }
    if (freeze)
      for (const ccake::GroupArgs& a : g.chunks) ccake::launch_freeze_group(a, g.stream);
  }
  for (const ccake::GroupArgs& a : g.chunks) ccake::launch_stop_group(a, g.stream);
  cudaMemcpyAsync(g.h_state, g.d_state, (size_t)nev * sizeof(ccake::EventState), cudaMemcpyDeviceToHost, g.stream);
  if (cudaStreamEndCapture(g.stream, &g.graph) != cudaSuccess ||
      cudaGraphInstantiate(&g.exec, g.graph, 0) != cudaSuccess)
    return CCAKE_ERR_CUDA;
  g.dirty = false;
  return CCAKE_OK;
}

// The group after a completed period: retire the events the device stopped.
void collect_group(ccake_server* srv, Group& g) {
  std::vector<Event*> keep;
  for (size_t k = 0; k < g.members.size(); k++) {
    Event* e = g.members[k];
    const ccake::EventState& h = g.h_state[k];
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      e->steps = h.steps;
      e->tau = h.tau;
    }
    if (h.active) {
      keep.push_back(e);
      continue;
    }
    ccake_internal::group_leave(e->ctx, h.tau);
    e->frozen = h.frozen_stop;
    finish(srv, e, h.status ? 3 : 2, h.status);
    g.dirty = true;
  }
  g.members.swap(keep);
}

// A period of the group: list builds (capacities grown where needed), the
// graph re-captured if the group changed, then launched.
void launch_group(ccake_server* srv, Group& g) {
  if (!g.joining.empty()) {
    g.members.insert(g.members.end(), g.joining.begin(), g.joining.end());
    g.joining.clear();
    g.dirty = true;
  }
  if (g.members.empty()) return;
  const int nev = (int)g.members.size();
  ccake_status_t s = CCAKE_OK;
  if (!ensure_pinned(g.h_cand, g.cand_cap, nev)) s = CCAKE_ERR_NOMEM;
  if (!s) {
    for (int k = 0; k < nev; k++) ccake_internal::group_build(g.members[(size_t)k]->ctx, g.stream, &g.h_cand[k]);
    if (cudaStreamSynchronize(g.stream) != cudaSuccess) s = CCAKE_ERR_CUDA;
  }
  std::vector<Event*> keep;
  for (int k = 0; k < nev && !s; k++) {
    Event* e = g.members[(size_t)k];
    bool changed = false;
    const ccake_status_t es = ccake_internal::group_grow(e->ctx, g.h_cand[k], &changed);
    if (es) {
      finish(srv, e, 3, es);
      g.dirty = true;
      continue;
    }
    g.dirty = g.dirty || changed;
    keep.push_back(e);
  }
  if (!s) g.members.swap(keep);
  if (!s && g.members.empty()) return;
  if (!s && g.dirty) s = rebuild_group(g);
  if (!s && (cudaGraphLaunch(g.exec, g.stream) != cudaSuccess || cudaEventRecord(g.mark, g.stream) != cudaSuccess))
    s = CCAKE_ERR_CUDA;
  if (s) {
    // the group cannot run: its events fail
    cudaGetLastError();
    for (Event* e : g.members) finish(srv, e, 3, s);
    g.members.clear();
    g.dirty = true;
    return;
  }
  g.inflight = true;
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
      e->grouped = groupable(e->cfg);
      ccake_status_t s = admit(e);
      if (!s && e->grouped) {
        // the group's period is the event's candidate-list period; an event
        // whose period differs advances alone
        Group& g = srv->groups[e->cfg.dim == 3 ? 1 : 0];
        const int period = ccake_internal::list_period(e->ctx);
        if (g.members.empty() && g.joining.empty() && !g.inflight) g.period = period;
        if (period != g.period) {
          e->grouped = false;
          if (!alloc_probe(e)) s = CCAKE_ERR_NOMEM;
        } else {
          g.joining.push_back(e);
        }
      }
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
    // 2a. groups
    for (int gi = 0; gi < 2; gi++) {
      Group& g = srv->groups[gi];
      if (g.inflight) {
        const cudaError_t q = cudaEventQuery(g.mark);
        if (q == cudaErrorNotReady) continue;
        g.inflight = false;
        progressed = true;
        if (q != cudaSuccess) {
          cudaGetLastError();
          for (Event* e : g.members) finish(srv, e, 3, CCAKE_ERR_CUDA);
          g.members.clear();
          g.dirty = true;
        } else {
          collect_group(srv, g);
        }
      }
      if (!g.inflight && (!g.members.empty() || !g.joining.empty())) {
        if (!g.stream) {
          g.dim = gi == 1 ? 3 : 2;
          if (cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking) != cudaSuccess ||
              cudaEventCreateWithFlags(&g.mark, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            for (Event* e : g.joining) finish(srv, e, 3, CCAKE_ERR_CUDA);
            g.joining.clear();
            continue;
          }
        }
        launch_group(srv, g);
        progressed = true;
      }
    }
    // 2b. events advanced alone
    std::vector<Event*> run;
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      for (Event* e : srv->running)
        if (!e->grouped) run.push_back(e);
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
            // the reference's stop rule after the quantum: every particle
            // frozen out (with particlization) or tau at tau_max
            const bool cold = e->cfg.particlization && pr.frozen >= e->n;
            if (cold || e->tau >= e->tau_max - 0.5 * e->cfg.dt) {
              e->frozen = cold ? 1 : 0;
              finish(srv, e, 2, 0);
              continue;
            }
          }
        }
        if (failed) {
          cudaGetLastError();
          finish(srv, e, 3, st);
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
        finish(srv, e, 3, s);
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
  for (Group& g : srv->groups) free_group(g);
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
  out->grouped = e->grouped ? 1 : 0;
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
