// Host side of libccake_gpu.so: the C ABI declared in include/ccake_gpu.h.
// Owns device memory, orders particles by neighbour cell, sequences the
// kernels of a derivative evaluation and captures one RK2 step in a CUDA
// graph that ccake_step replays.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "ccake_gpu.h"
#include "internal.hpp"
#include "kernels.cuh"
#include "mlp.cuh"

using namespace ccake;

struct ccake_ctx {
  ccake_config cfg{};
  RunConst rc{};
  EosDev eos{};
  Ptrs p{};
  int64_t n = 0;
  std::vector<int32_t> perm;   // storage slot -> caller's index
  cudaStream_t stream = nullptr;
  bool loaded = false, initialized = false;
  double t = 0.0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  std::string err;
  double* dbuf = nullptr;
  int32_t* ibuf = nullptr;
  double* d_table = nullptr;
  float* d_table_f = nullptr;   // FP32 densities of the nodes (mixed-form Newton Jacobians)
  // pre-inverted tables: values, description (host and device copies)
  double* pre_v = nullptr;
  int64_t pre_count = 0;
  PreinvView pre_host{};
  PreinvView* pre_dev = nullptr;
  int records_form = 0;   // which smoothing record matches the state: 0 FP64, 1 mixed
  bool evaluated = false; // derivatives were evaluated since the initialisation
  // candidate list: skin (fm), validity and rebuild schedule
  double skin = 0.0;
  bool lists_valid = false;
  int steps_since_build = 0;
  cudaGraph_t build_graph = nullptr;
  cudaGraphExec_t build_exec = nullptr;
  // kernels launched through the step and list-build graphs (kernel nodes of
  // a graph times its launches), for ccake_kernel_launches
  int64_t step_kernels = 0, build_kernels = 0, launches = 0;
  // learned Newton seed: parameters, gradients, Adam moments (4 x mlp::kParams FP32)
  float* mlp_buf = nullptr;
  double* mlp_sse = nullptr;
  int32_t* mlp_err = nullptr;
  MlpNorm mlp_norm{};
  bool mlp_ready = false;
  int32_t* d_count = nullptr;   // one int32 (frozen-particle count)
  // scratch of the two-pass batch inversion (capacity + 1 int32)
  int32_t* eos_scratch = nullptr;
  int64_t eos_scratch_cap = 0;
  // initial viscous input (ccake_set_initial_viscous): trace, pi^{xx xy xeta yy yeta}
  double* init_visc = nullptr;
  int init_bulk = 0, init_shear = 0;
  // initial diffusion currents (ccake_set_initial_diffusion): q^i of charge c at row 3c + i
  double* init_q = nullptr;
  // the mixed form's step kernels are grouped launches (GroupArgs); alone,
  // the event is a group of one: its arguments and its device-side state
  GroupArgs grp{};
  EventState* d_state = nullptr;
  int nblk = 0;
};

namespace {

ccake_status_t fail(ccake_ctx* c, ccake_status_t s, const std::string& msg) {
  if (c) c->err = msg;
  return s;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(ctx, CCAKE_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// Kernel nodes of a captured graph.
int64_t kernel_nodes(cudaGraph_t g) {
  size_t m = 0;
  if (cudaGraphGetNodes(g, nullptr, &m) != cudaSuccess || m == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(m);
  if (cudaGraphGetNodes(g, nodes.data(), &m) != cudaSuccess) return 0;
  int64_t k = 0;
  for (size_t i = 0; i < m; i++) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
  }
  return k;
}

void drop_graph(ccake_ctx* ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  if (ctx->build_exec) cudaGraphExecDestroy(ctx->build_exec);
  if (ctx->build_graph) cudaGraphDestroy(ctx->build_graph);
  ctx->graph_exec = nullptr;
  ctx->graph = nullptr;
  ctx->build_exec = nullptr;
  ctx->build_graph = nullptr;
}

void free_lists(ccake_ctx* ctx) {
  if (ctx->p.nbr_idx) cudaFree(ctx->p.nbr_idx);
  if (ctx->p.nbr_f) cudaFree(ctx->p.nbr_f);
  if (ctx->p.nbr_fe) cudaFree(ctx->p.nbr_fe);
  ctx->p.nbr_idx = nullptr;
  ctx->p.nbr_f = nullptr;
  ctx->p.nbr_fe = nullptr;
  ctx->p.K = 0;
}

// The neighbour list of capacity K (with the factorised kernel's second
// gradient factor when it is on).
static bool alloc_lists(ccake_ctx* ctx, int K) {
  const size_t m = (size_t)K * ctx->n;
  if (cudaMalloc(&ctx->p.nbr_idx, m * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&ctx->p.nbr_f, m * sizeof(double)) != cudaSuccess)
    return false;
  if (ctx->rc.cfg.dim == 3 && ctx->rc.cfg.factorized_kernel &&
      cudaMalloc(&ctx->p.nbr_fe, m * sizeof(double)) != cudaSuccess)
    return false;
  return true;
}

void free_candidates(ccake_ctx* ctx) {
  if (ctx->p.cand_idx) cudaFree(ctx->p.cand_idx);
  ctx->p.cand_idx = nullptr;
  ctx->p.Kc = 0;
  ctx->lists_valid = false;
}

void free_buffers(ccake_ctx* ctx) {
  drop_graph(ctx);
  free_lists(ctx);
  free_candidates(ctx);
  if (ctx->dbuf) cudaFree(ctx->dbuf);
  if (ctx->ibuf) cudaFree(ctx->ibuf);
  if (ctx->p.fz) cudaFree(ctx->p.fz);
  if (ctx->p.fo_rows) cudaFree(ctx->p.fo_rows);
  if (ctx->p.fo_count) cudaFree(ctx->p.fo_count);
  if (ctx->p.dif) cudaFree(ctx->p.dif);
  if (ctx->p.recQ) cudaFree(ctx->p.recQ);
  ctx->p.dif = ctx->p.recQ = nullptr;
  if (ctx->init_visc) cudaFree(ctx->init_visc);
  if (ctx->init_q) cudaFree(ctx->init_q);
  ctx->init_visc = ctx->init_q = nullptr;
  if (ctx->d_state) cudaFree(ctx->d_state);
  ctx->d_state = nullptr;
  ctx->nblk = 0;
  ctx->init_bulk = ctx->init_shear = 0;
  ctx->dbuf = nullptr;
  ctx->ibuf = nullptr;
  ctx->p.fz = ctx->p.fo_rows = nullptr;
  ctx->p.fo_count = nullptr;
}

// Neighbour-cell grid: the reference's box (twice the IC lower corner,
// mirrored; src/system_state.cpp:656-692), widened to hold every particle,
// cell edge >= 2h + skin (the candidate-list radius).
Grid make_grid(const ccake_config& cfg, const ccake_particles_soa* h, double skin) {
  Grid g{};
  const double cut = 2.0 * cfg.hT + skin;
  const double corner[3] = {cfg.xmin, cfg.ymin, cfg.etamin};
  const double* xs[3] = {h->x, h->y, h->eta};
  for (int k = 0; k < 3; k++) {
    if (k >= cfg.dim) { g.lo[k] = -cfg.hT; g.nc[k] = 1; g.inv_cs[k] = 1.0 / (2.0 * cfg.hT); continue; }
    double lo = 2.0 * corner[k], hi = -2.0 * corner[k];
    double mn = 1e300, mx = -1e300;
    for (int64_t i = 0; i < h->n; i++) { mn = std::min(mn, xs[k][i]); mx = std::max(mx, xs[k][i]); }
    lo = std::min(lo, mn - cut);
    hi = std::max(hi, mx + cut);
    int nc = (int)std::floor((hi - lo) / cut);
    nc = std::max(1, std::min(nc, 1 << 14));
    g.lo[k] = lo;
    g.nc[k] = nc;
    g.inv_cs[k] = nc / (hi - lo);
  }
  g.ncell = g.nc[0] * g.nc[1] * g.nc[2];
  return g;
}

int host_cell(const Grid& g, int k, double x) {
  int c = (int)std::floor((x - g.lo[k]) * g.inv_cs[k]);
  return c < 0 ? 0 : (c >= g.nc[k] ? g.nc[k] - 1 : c);
}

ccake_status_t check_errors(ccake_ctx* ctx) {
  int32_t e[NERR];
  CK(cudaMemcpyAsync(e, ctx->p.err, sizeof(e), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  // the failure raised first decides the status; the message counts them all
  const ccake_status_t kind[4] = {CCAKE_ERR_EOS, CCAKE_ERR_NEG_ENTROPY, CCAKE_ERR_NONFINITE, CCAKE_ERR_CAPACITY};
  const std::string what[4] = {" particles without an EoS solution", " particles with negative entropy",
                               " non-finite particles",
                               " particles exceed the neighbour-list capacity " + std::to_string(ctx->p.K)};
  int first = e[E_FIRST] - 1;
  if (first < 0 || first > 3)
    for (int k = 3; k >= 0; k--) if (e[k]) first = k;
  if (first < 0) return CCAKE_OK;
  std::string msg = std::to_string(e[first]) + what[first];
  for (int k = 0; k < 4; k++)
    if (k != first && e[k]) msg += "; then " + std::to_string(e[k]) + what[k];
  return fail(ctx, kind[first], msg);
}

ccake_status_t reset_errors(ccake_ctx* ctx) {
  CK(cudaMemsetAsync(ctx->p.err, 0, sizeof(int32_t) * NERR, ctx->stream));
  return CCAKE_OK;
}

// doubles per particle in the double slab (state, fields, records)
constexpr int64_t kDoublesPerParticle =
    RA + RB + 2 + RAF / 2 + RBF / 2 + 2 * NY + 1 + NTH + 1 + 3 + 1 + 1 + 1 + NPI + NGRAD + NDER + 1 + 1 + 3 + 1;

// The smoothing record of each precision form is written by that form's
// pass B; before a pass A of the other form runs, it is packed from the state.
void ensure_records(ccake_ctx* ctx, int form) {
  if (ctx->records_form == form) return;
  if (form == 1) launch_pack_mixed(ctx->rc, ctx->p, ctx->stream);
  else launch_pack_fp64(ctx->rc, ctx->p, ctx->stream);
  ctx->records_form = form;
}

// The event's descriptor: constants, EoS with FP32 table Newton Jacobians
// (the residual stays FP64), arrays.
void fill_desc(const ccake_ctx* ctx, EventDesc* d) {
  d->rc = ctx->rc;
  d->eos = ctx->eos;
  d->eos.jac32 = 1;
  d->p = ctx->p;
}

// The event's arguments of the grouped mixed kernels (a group of one),
// refreshed from the context before those kernels are launched or captured.
ccake_status_t sync_slot(ccake_ctx* ctx) {
  if (!ctx->d_state) return fail(ctx, CCAKE_ERR_STATE, "load particles first");
  ctx->grp.nev = 1;
  ctx->grp.first_block[0] = 0;
  ctx->grp.first_block[1] = ctx->nblk;
  ctx->grp.state = ctx->d_state;
  fill_desc(ctx, &ctx->grp.ev[0]);
  return CCAKE_OK;
}

void enqueue_passA(ccake_ctx* ctx) {
  if (ctx->cfg.precision == 1) launch_passA_mixed(ctx->grp, ctx->cfg.dim, ctx->stream);
  else launch_passA(ctx->rc, ctx->eos, ctx->p, A_WITH_THERMO, ctx->stream);
}

void enqueue_passB(ccake_ctx* ctx, int mode, int sub) {
  if (ctx->cfg.precision == 1)
    launch_passB_mixed(ctx->grp, ctx->cfg.dim, mode, sub, ctx->stream);
  else launch_passB(ctx->rc, ctx->p, mode, sub == 1 ? 0.5 * ctx->cfg.dt : ctx->cfg.dt, ctx->stream);
}

void enqueue_clock(ccake_ctx* ctx, int sub) {
  if (ctx->cfg.precision == 1) launch_clock_group(ctx->grp, sub, ctx->stream);
  else launch_clock(ctx->p, sub, ctx->cfg.dt, ctx->stream);
}

// Cell list and candidate list at the current positions.
void enqueue_build(ccake_ctx* ctx) {
  launch_build_cells(ctx->rc, ctx->p, ctx->stream);
  cudaMemsetAsync(ctx->p.cand_max, 0, sizeof(int32_t), ctx->stream);
  launch_candidates(ctx->rc, ctx->p, ctx->stream);
}

// List capacity for a count: 1.25x plus 16, in multiples of 16.
int capacity_for(int count) { return ((count * 5 / 4 + 16) + 15) / 16 * 16; }

// After a candidate build: when the largest candidate count exceeds the
// capacity of the candidate list (entries past it were dropped) or of the
// neighbour list (the neighbours of a particle are among its candidates), the
// lists are reallocated larger and built again. Particles that crowd together
// (compressing flows) thus never overflow the lists; the reference's Verlet
// list has no fixed capacity either. The graphs that hold the old pointers
// are dropped and captured again at their next use.
ccake_status_t grow_lists(ccake_ctx* ctx) {
  for (int attempt = 0; attempt < 4; attempt++) {
    int32_t mx = 0;
    CK(cudaMemcpyAsync(&mx, ctx->p.cand_max, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (mx <= ctx->p.Kc && mx <= ctx->p.K) return CCAKE_OK;
    drop_graph(ctx);
    if (mx > ctx->p.Kc) {
      const int Kc = capacity_for(mx);
      free_candidates(ctx);
      if (cudaMalloc(&ctx->p.cand_idx, (size_t)Kc * ctx->n * sizeof(int32_t)) != cudaSuccess)
        return fail(ctx, CCAKE_ERR_NOMEM, "candidate list allocation");
      ctx->p.Kc = Kc;
    }
    if (mx > ctx->p.K) {
      const int K = capacity_for(mx);
      free_lists(ctx);
      if (!alloc_lists(ctx, K)) return fail(ctx, CCAKE_ERR_NOMEM, "neighbour list allocation");
      ctx->p.K = K;
    }
    enqueue_build(ctx);
  }
  return fail(ctx, CCAKE_ERR_CAPACITY, "candidate list did not settle");
}

// Steps a candidate list stays valid from time tau: a particle moves at most
// dt * vmax per RK2 step in (x, y, eta_s) coordinates (|v| < 1 by
// construction, v^eta < 1/tau), so no pair can close from beyond 2h + skin to
// within 2h while R dt vmax <= skin / 2.
int build_every(const ccake_ctx* ctx, double tau) {
  const double vmax = (ctx->cfg.dim == 3 && ctx->cfg.coord == 0) ? std::max(1.0, 1.0 / tau) : 1.0;
  return std::max(1, (int)std::floor(ctx->skin / (2.0 * ctx->cfg.dt * vmax)));
}

// Rebuilds the lists when the schedule asks for it (before a step).
ccake_status_t maybe_rebuild(ccake_ctx* ctx, bool graph) {
  if (ctx->lists_valid && ctx->steps_since_build < build_every(ctx, ctx->t)) return CCAKE_OK;
  if (graph) {
    if (!ctx->build_exec) {
      CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      enqueue_build(ctx);
      CK(cudaStreamEndCapture(ctx->stream, &ctx->build_graph));
      CK(cudaGraphInstantiate(&ctx->build_exec, ctx->build_graph, 0));
      ctx->build_kernels = kernel_nodes(ctx->build_graph);
    }
    CK(cudaGraphLaunch(ctx->build_exec, ctx->stream));
    ctx->launches += ctx->build_kernels;
  } else {
    enqueue_build(ctx);
  }
  ccake_status_t s = grow_lists(ctx);
  if (s) return s;
  ctx->lists_valid = true;
  ctx->steps_since_build = 0;
  return CCAKE_OK;
}

// The freeze-out stage after a step (SPHWorkstation::freeze_out_particles).
void enqueue_freeze(ccake_ctx* ctx) {
  if (ctx->cfg.surface && ctx->p.fz) {
    // gradients, theta and shv_nabla_u of the evaluation just done, then the
    // status machine with snapshots and hypersurface rows
    const int mixed = ctx->cfg.precision == 1 ? 1 : 0;
    if (mixed) launch_gradients_mixed(ctx->grp, ctx->cfg.dim, ctx->stream);
    else launch_passB(ctx->rc, ctx->p, B_GRADS, 0.0, ctx->stream);
    launch_diagnostics(ctx->rc, ctx->p, mixed, ctx->stream);
    launch_freeze_surface(ctx->rc, ctx->p, mixed, ctx->cfg.dt, ctx->stream);
  } else if (ctx->cfg.precision == 1) {
    launch_freeze_group(ctx->grp, ctx->stream);
  } else {
    launch_freeze(ctx->rc, ctx->p, ctx->stream);
  }
}

void enqueue_substep(ccake_ctx* ctx, int sub) {
  enqueue_passA(ctx);
  enqueue_passB(ctx, B_EOM | B_UPDATE | (sub == 2 ? B_WRITE_Y0 : 0), sub);
  enqueue_clock(ctx, sub);
  if (sub == 2 && ctx->cfg.particlization) enqueue_freeze(ctx);
}

// Captures the RK2 step graph (two substeps) if it is not held; the mixed
// form's slot is made current first (its kernels read it when they run).
ccake_status_t ensure_step_graph(ccake_ctx* ctx) {
  if (ctx->graph_exec) return CCAKE_OK;
  ccake_status_t s;
  if (ctx->cfg.precision == 1 && (s = sync_slot(ctx))) return s;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_substep(ctx, 1);
  enqueue_substep(ctx, 2);
  CK(cudaStreamEndCapture(ctx->stream, &ctx->graph));
  CK(cudaGraphInstantiate(&ctx->graph_exec, ctx->graph, 0));
  ctx->step_kernels = kernel_nodes(ctx->graph);
  return CCAKE_OK;
}

struct FieldRef {
  const double* base;
  bool ok;
};

FieldRef field_ref(ccake_ctx* ctx, const std::string& k) {
  const Ptrs& p = ctx->p;
  const int64_t n = ctx->n;
  auto Y = [&](int s) { return FieldRef{p.y + s * n, true}; };
  static const char* thn[NTH] = {"T", "muB", "muS", "muQ", "p", "s", "rhoB", "rhoS", "rhoQ", "e", "w", "cs2",
                                 "dwds", "dwdB", "dwdS", "dwdQ"};
  for (int q = 0; q < NTH; q++) if (k == thn[q]) return FieldRef{p.th + q * n, true};
  if (k == "x") return Y(Y_X0);
  if (k == "y") return Y(Y_X1);
  if (k == "eta") return Y(Y_X2);
  if (k == "ext_s") return Y(Y_ES);
  if (k == "ext_B") return Y(Y_EB);
  if (k == "ext_S") return Y(Y_ESS);
  if (k == "ext_Q") return Y(Y_EQ);
  if (k == "ext_bulk") return Y(Y_EBULK);
  if (k == "Ez") return Y(Y_EZ);
  for (int q = 0; q < 3; q++) {
    const std::string d = std::to_string(q);
    if (k == "u" + d) return Y(Y_U0 + q);
    if (k == "v" + d) return FieldRef{p.v + q * n, true};
    if (k == "gradP" + d) return FieldRef{p.grads + (G_P + q) * n, true};
    if (k == "gradE" + d) return FieldRef{p.grads + (G_E + q) * n, true};
    if (k == "gradBulk" + d) return FieldRef{p.grads + (G_B + q) * n, true};
    if (k == "gradshear" + d) return FieldRef{p.grads + (G_SH + q) * n, true};
    if (k == "divshear" + d) return FieldRef{p.grads + (G_DS + q) * n, true};
    if (k == "du_dt" + d) return FieldRef{p.derivs + (D_DU0 + q) * n, true};
  }
  for (int q = 0; q < 5; q++) {
    if (k == "ext_shv" + std::to_string(q)) return Y(Y_SHV0 + q);
    if (k == "d_ext_shv" + std::to_string(q)) return FieldRef{p.derivs + (D_DSHV0 + q) * n, true};
  }
  for (int q = 0; q < 9; q++) if (k == "gradV" + std::to_string(q)) return FieldRef{p.grads + (G_V + q) * n, true};
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++)
      if (k == "shv" + std::to_string(a) + std::to_string(b)) return FieldRef{p.pi + pi_slot(a, b) * n, true};
  if (k == "gamma") return FieldRef{p.gam, true};
  if (k == "sigma_lab") return FieldRef{p.slab, true};
  if (k == "sigma") return FieldRef{p.sig, true};
  if (k == "bulk") return FieldRef{p.bulk, true};
  if (k == "d_ext_s") return FieldRef{p.derivs + D_DS * n, true};
  if (k == "d_ext_bulk") return FieldRef{p.derivs + D_DBULK * n, true};
  if (k == "dEz") return FieldRef{p.derivs + D_DEZ * n, true};
  if (k == "eta_pi") return FieldRef{p.derivs + D_ETA * n, true};
  if (k == "tau_pi") return FieldRef{p.derivs + D_TAUPI * n, true};
  if (k == "zeta_Pi") return FieldRef{p.derivs + D_ZETA * n, true};
  if (k == "tau_Pi") return FieldRef{p.derivs + D_TAUBULK * n, true};
  if (k == "in_s") return FieldRef{p.in_s, true};
  if (k == "theta") return FieldRef{p.derivs + D_THETA * n, true};
  for (int q = 0; q < 5; q++)
    if (k == "sigma_tensor" + std::to_string(q)) return FieldRef{p.derivs + (D_SIG0 + q) * n, true};
  if (k == "shear_knudsen") return FieldRef{p.derivs + D_KNS * n, true};
  if (k == "bulk_knudsen") return FieldRef{p.derivs + D_KNB * n, true};
  if (k == "inverse_reynolds_shear") return FieldRef{p.derivs + D_IRS * n, true};
  if (k == "inverse_reynolds_bulk") return FieldRef{p.derivs + D_IRB * n, true};
  if (p.dif) {
    // diffusion sector, charge letters B, S, Q
    auto F = [&](int slot) { return FieldRef{p.dif + (size_t)slot * n, true}; };
    const char ch[3] = {'B', 'S', 'Q'};
    for (int c = 0; c < 3; c++) {
      const std::string C(1, ch[c]);
      if (k == "d_ext_" + C) return F(F_DN + c);
      for (int m = 0; m < 4; m++)
        if (k == "q" + C + std::to_string(m)) return F(F_Q + 4 * c + m);
      for (int i = 0; i < 3; i++) {
        if (k == "ext_q" + C + std::to_string(i)) return F(F_YQ + 3 * c + i);
        if (k == "d_ext_q" + C + std::to_string(i)) return F(F_DYQ + 3 * c + i);
        if (k == "grad_alpha" + std::to_string(i) + C) return F(F_GA + 3 * i + c);
      }
      if (k == "div_qa" + C) return F(F_DQ + c);
      if (k == "grad_qa" + C) return F(F_GQ + c);
      if (k == "kn_diff" + C) return F(F_KN + c);
      if (k == "ire_diff" + C) return F(F_IR + c);
    }
    for (int j = 0; j < 12; j++)
      if (k == "dalpha" + std::to_string(j)) return F(F_DA + j);
  }
  return FieldRef{nullptr, false};
}

}  // namespace

// learned Newton seed: helpers
namespace {

ccake_status_t ensure_mlp(ccake_ctx* ctx) {
  if (ctx->mlp_buf) return CCAKE_OK;
  if (cudaMalloc(&ctx->mlp_buf, 4 * mlp::kParams * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&ctx->mlp_sse, sizeof(double)) != cudaSuccess || cudaMalloc(&ctx->mlp_err, sizeof(int32_t)) != cudaSuccess)
    return fail(ctx, CCAKE_ERR_NOMEM, "network allocation");
  CK(cudaMemsetAsync(ctx->mlp_buf, 0, 4 * mlp::kParams * sizeof(float), ctx->stream));
  CK(cudaMemsetAsync(ctx->mlp_err, 0, sizeof(int32_t), ctx->stream));
  return CCAKE_OK;
}

ccake_status_t mlp_check(ccake_ctx* ctx) {
  int32_t e = 0;
  CK(cudaMemcpyAsync(&e, ctx->mlp_err, sizeof(e), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  if (e) {
    cudaMemsetAsync(ctx->mlp_err, 0, sizeof(int32_t), ctx->stream);
    return fail(ctx, CCAKE_ERR_CUDA, "tensor-core wait expired in the seed network");
  }
  return CCAKE_OK;
}

// Device scratch freed on scope exit.
struct Scratch {
  std::vector<void*> p;
  template <class T>
  T* get(size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, count * sizeof(T)) != cudaSuccess) return nullptr;
    p.push_back(q);
    return static_cast<T*>(q);
  }
  ~Scratch() {
    for (void* q : p) cudaFree(q);
  }
};

}  // namespace


// Scratch of the two-pass batch inversion, grown on demand (NULL when the
// allocation fails: the single-pass kernel is used).
static int32_t* eos_scratch(ccake_ctx* ctx, int64_t n) {
  if (n > ctx->eos_scratch_cap) {
    if (ctx->eos_scratch) cudaFree(ctx->eos_scratch);
    ctx->eos_scratch = nullptr;
    ctx->eos_scratch_cap = 0;
    if (cudaMalloc(&ctx->eos_scratch, (size_t)(n + 1) * sizeof(int32_t)) != cudaSuccess) {
      cudaGetLastError();
      ctx->eos_scratch = nullptr;
      return nullptr;
    }
    ctx->eos_scratch_cap = n;
  }
  return ctx->eos_scratch;
}

// ---------------------------------------------------------------------------
// hooks for the event server
// ---------------------------------------------------------------------------
namespace ccake_internal {

ccake_status_t step_enqueue(ccake_ctx* ctx, int n) {
  if (!ctx || !ctx->initialized || n < 0) return CCAKE_ERR_STATE;
  ccake_status_t st;
  if (ctx->cfg.precision == 1 && (st = sync_slot(ctx))) return st;
  ensure_records(ctx, ctx->cfg.precision);
  ccake_status_t s;
  for (int k = 0; k < n; k++) {
    if ((s = maybe_rebuild(ctx, true)) || (s = ensure_step_graph(ctx))) return s;
    CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->launches += ctx->step_kernels;
    ctx->steps_since_build++;
  }
  return CCAKE_OK;
}

ccake_status_t probe_enqueue(ccake_ctx* ctx, Probe* dev, Probe* host) {
  launch_probe(ctx->p, dev, ctx->stream);
  CK(cudaMemcpyAsync(host, dev, sizeof(Probe), cudaMemcpyDeviceToHost, ctx->stream));
  return CCAKE_OK;
}

ccake_status_t clear_errors(ccake_ctx* ctx) { return reset_errors(ctx); }

cudaStream_t ctx_stream(ccake_ctx* ctx) { return ctx->stream; }
void ctx_set_time(ccake_ctx* ctx, double t) { ctx->t = t; }

void group_desc(ccake_ctx* ctx, EventDesc* out) { fill_desc(ctx, out); }

int list_period(ccake_ctx* ctx) { return build_every(ctx, ctx->t); }

ccake_status_t group_join(ccake_ctx* ctx) {
  ccake_status_t s = reset_errors(ctx);
  if (s) return s;
  ensure_records(ctx, 1);
  CK(cudaStreamSynchronize(ctx->stream));
  return CCAKE_OK;
}

void group_build(ccake_ctx* ctx, cudaStream_t s, int32_t* host_cand_max) {
  launch_build_cells(ctx->rc, ctx->p, s);
  cudaMemsetAsync(ctx->p.cand_max, 0, sizeof(int32_t), s);
  launch_candidates(ctx->rc, ctx->p, s);
  cudaMemcpyAsync(host_cand_max, ctx->p.cand_max, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
}

ccake_status_t group_grow(ccake_ctx* ctx, int32_t cand_max, bool* changed) {
  *changed = false;
  if (cand_max <= ctx->p.Kc && cand_max <= ctx->p.K) return CCAKE_OK;
  *changed = true;
  // the build just done left cand_max on the device: grow_lists reads it,
  // reallocates and builds again on the context's stream
  return grow_lists(ctx);
}

void group_leave(ccake_ctx* ctx, double tau) {
  ctx->t = tau;
  ctx->records_form = 1;
  ctx->lists_valid = false;   // stepped alone later, it builds its lists first
  ctx->evaluated = true;
}

int64_t estimate_bytes(const ccake_config& cfg, int64_t n) {
  // state and records, plus neighbour and candidate lists at the lattice
  // densities of the bundled workloads (48 / 447 neighbours in 2-D / 3-D)
  const int64_t K = cfg.dim == 3 ? 688 : 96, Kc = cfg.dim == 3 ? 912 : 112;
  const int64_t dif = cfg.using_diffusion ? (int64_t)(NDIF + RQ) * 8 : 0;   // diffusion slabs and record
  return n * (kDoublesPerParticle * 8 + 8 * 4 + K * 12 + Kc * 4 + dif) + (int64_t)(1 << 20);
}

}  // namespace ccake_internal

extern "C" {

const char* ccake_status_string(ccake_status_t s) {
  switch (s) {
    case CCAKE_OK: return "ok";
    case CCAKE_ERR_INVALID: return "invalid argument";
    case CCAKE_ERR_CUDA: return "CUDA error";
    case CCAKE_ERR_EOS: return "EoS inversion failed";
    case CCAKE_ERR_NEG_ENTROPY: return "negative entropy";
    case CCAKE_ERR_CAPACITY: return "buffer too small";
    case CCAKE_ERR_STATE: return "call out of order";
    case CCAKE_ERR_NOMEM: return "out of device memory";
    case CCAKE_ERR_NONFINITE: return "non-finite state";
  }
  return "unknown";
}

const char* ccake_last_error(const ccake_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

ccake_status_t ccake_ctx_create(const ccake_config* cfg, ccake_ctx** out) {
  if (!cfg || !out) return CCAKE_ERR_INVALID;
  *out = nullptr;
  if (cfg->dim != 2 && cfg->dim != 3) return CCAKE_ERR_INVALID;
  if (cfg->coord != 0 && cfg->coord != 1) return CCAKE_ERR_INVALID;
  if (cfg->eos_kind < 0 || cfg->eos_kind > 2) return CCAKE_ERR_INVALID;
  if (cfg->precision != 0 && cfg->precision != 1) return CCAKE_ERR_INVALID;
  if (!(cfg->skin_frac >= 0.0)) return CCAKE_ERR_INVALID;
  if (!(cfg->hT > 0) || !(cfg->t0 > 0) || !(cfg->dt > 0)) return CCAKE_ERR_INVALID;
  // the factorised 3-D kernel runs in the FP64 form
  if (cfg->dim == 3 && cfg->factorized_kernel && (cfg->precision != 0 || !(cfg->hEta > 0.0)))
    return CCAKE_ERR_INVALID;
  // initial inversion seed: the reference's, or the learned one (table EoS)
  if (cfg->seed_mode != CCAKE_SEED_REFERENCE &&
      !(cfg->seed_mode == CCAKE_SEED_LEARNED && cfg->eos_kind == 2 && !cfg->input_as_entropy))
    return CCAKE_ERR_INVALID;
  // second-order coefficient modes: DEFAULT or DISABLED, and IS for the two deltas
  for (int32_t m : {cfg->tau_pipi_mode, cfg->lambda_piPi_mode, cfg->phi6_mode, cfg->phi7_mode, cfg->lambda_Pipi_mode,
                    cfg->phi1_mode, cfg->phi3_mode})
    if (m != CCAKE_COEF_DEFAULT && m != CCAKE_COEF_DISABLED) return CCAKE_ERR_INVALID;
  for (int32_t m : {cfg->delta_pipi_mode, cfg->delta_PiPi_mode})
    if (m < CCAKE_COEF_DEFAULT || m > CCAKE_COEF_DISABLED) return CCAKE_ERR_INVALID;
  // the diffusion sector (both forms) with the constant_over_T2 or
  // kappaB_coth coefficients
  if (cfg->using_diffusion && cfg->diffusion_mode != 0 && cfg->diffusion_mode != 2)
    return CCAKE_ERR_INVALID;
  ccake_ctx* ctx = new ccake_ctx;
  ctx->cfg = *cfg;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return CCAKE_ERR_CUDA;
  }
  RunConst& rc = ctx->rc;
  rc.cfg = *cfg;
  const int D = cfg->dim;
  const double h = cfg->hT;
  set_kernel_constants(rc, D, h);
  if (D == 3 && cfg->factorized_kernel) {
    // W_2D(r_perp, hT) W_1D(|d eta|, hEta); the list keeps the reference's
    // 2 hT sphere (src/system_state.cpp:650-719)
    rc.kperp = kernel_const(2, h);
    rc.keta = kernel_const(1, cfg->hEta);
    rc.k0 = rc.kperp.wn * rc.keta.wn;
  }
  // skin: at least one RK2 step of travel at the largest coordinate speed
  // (tau only grows from t0), so that a list lasts a step or more
  const double vmax0 = (D == 3 && cfg->coord == 0) ? std::max(1.0, 1.0 / cfg->t0) : 1.0;
  ctx->skin = std::max((cfg->skin_frac > 0.0 ? cfg->skin_frac : 0.1) * 2.0 * h, 2.0 * cfg->dt * vmax0 * (1.0 + 1e-6));
  rc.cutc2 = (2.0 * h + ctx->skin) * (2.0 * h + ctx->skin);
  rc.fcutc2 = (float)rc.cutc2;
  EosDev& e = ctx->eos;
  e.kind = cfg->eos_kind;
  e.thermo_mode = cfg->thermo_mode;
  e.restrict_mu_T = cfg->restrict_mu_T_ratios ? 1 : 0;
  e.own = make_scales(cfg->eos_c, cfg->eos_T0, cfg->eos_muB0, cfg->eos_muQ0, cfg->eos_muS0);
  e.conf = e.cdiag = e.own;
  if (e.kind != 2) {   // a table kind sets it with the table
    double x4[4] = {cfg->freeze_out_T, 0, 0, 0}, o[17];
    model_thermo(e, chain_model(e.kind, 0), x4, o);
    rc.efreeze = o[5];
  }
  *out = ctx;
  return CCAKE_OK;
}

ccake_status_t ccake_ctx_destroy(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  free_buffers(ctx);
  if (ctx->mlp_buf) cudaFree(ctx->mlp_buf);
  if (ctx->mlp_sse) cudaFree(ctx->mlp_sse);
  if (ctx->mlp_err) cudaFree(ctx->mlp_err);
  if (ctx->eos_scratch) cudaFree(ctx->eos_scratch);
  if (ctx->d_count) cudaFree(ctx->d_count);
  if (ctx->d_table) cudaFree(ctx->d_table);
  if (ctx->d_table_f) cudaFree(ctx->d_table_f);
  if (ctx->pre_v) cudaFree(ctx->pre_v);
  if (ctx->pre_dev) cudaFree(ctx->pre_dev);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return CCAKE_OK;
}

ccake_status_t ccake_load_particles(ccake_ctx* ctx, const ccake_particles_soa* h) {
  if (!ctx || !h || h->n <= 0 || !h->x || !h->y || !h->e_or_s || !h->ux || !h->uy) return CCAKE_ERR_INVALID;
  if (ctx->cfg.dim == 3 && (!h->eta || !h->ueta)) return fail(ctx, CCAKE_ERR_INVALID, "dim 3 needs eta and ueta");
  if (h->n > (int64_t)0x3fffffff) return fail(ctx, CCAKE_ERR_INVALID, "too many particles");
  // positions and velocities place the particles in cells: non-finite ones
  // are rejected here (a non-finite density is the EoS's to report)
  {
    const double* cols[6] = {h->x, h->y, ctx->cfg.dim == 3 ? h->eta : nullptr, h->ux, h->uy,
                             ctx->cfg.dim == 3 ? h->ueta : nullptr};
    for (int c = 0; c < 6; c++)
      if (cols[c])
        for (int64_t i = 0; i < h->n; i++)
          if (!std::isfinite(cols[c][i]))
            return fail(ctx, CCAKE_ERR_INVALID, "non-finite position or velocity at particle " + std::to_string(i));
  }
  free_buffers(ctx);
  const int64_t n = h->n;
  ctx->n = n;
  ctx->rc.grid = make_grid(ctx->cfg, h, ctx->skin);
  const Grid& g = ctx->rc.grid;
  // storage order: by neighbour cell, then by input index
  std::vector<int64_t> key(n);
  for (int64_t i = 0; i < n; i++) {
    int64_t c = host_cell(g, 0, h->x[i]) + (int64_t)g.nc[0] * host_cell(g, 1, h->y[i]);
    if (ctx->cfg.dim == 3) c += (int64_t)g.nc[0] * g.nc[1] * host_cell(g, 2, h->eta[i]);
    key[i] = c;
  }
  ctx->perm.resize(n);
  std::iota(ctx->perm.begin(), ctx->perm.end(), 0);
  std::stable_sort(ctx->perm.begin(), ctx->perm.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
  // device memory: one double slab, one int slab
  const size_t nd = (size_t)n * kDoublesPerParticle + (size_t)kTotBlocks * 6 + 8;
  const size_t ni = (size_t)n * 8 + (size_t)g.ncell * 2 + 1 + NERR + 1 + 2 * (size_t)scan_tiles(g.ncell) + 1 + 8;
  if (cudaMalloc(&ctx->dbuf, nd * sizeof(double)) != cudaSuccess) return fail(ctx, CCAKE_ERR_NOMEM, "device allocation");
  if (cudaMalloc(&ctx->ibuf, ni * sizeof(int32_t)) != cudaSuccess) return fail(ctx, CCAKE_ERR_NOMEM, "device allocation");
  CK(cudaMemsetAsync(ctx->dbuf, 0, nd * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->ibuf, 0, ni * sizeof(int32_t), ctx->stream));
  Ptrs& p = ctx->p;
  p.n = (int)n;
  double* d = ctx->dbuf;
  auto take = [&](size_t k) { double* r = d; d += k * n; return r; };
  // the records come first: their slabs are multiples of 32 bytes a
  // particle, so the 16- and 32-byte vector loads stay aligned for any n
  static_assert(RA % 4 == 0 && RB % 4 == 0 && RAF % 8 == 0 && RBF % 8 == 0, "record alignment");
  p.recA = take(RA); p.recB = take(RB);
  p.recAf = reinterpret_cast<float*>(take(RAF / 2));
  p.recBf = reinterpret_cast<float*>(take(RBF / 2));
  p.posf = reinterpret_cast<float4*>(take(2));
  p.y = take(NY); p.y0 = take(NY); p.m = take(1); p.th = take(NTH); p.gam = take(1); p.v = take(3);
  p.slab = take(1); p.sig = take(1); p.bulk = take(1); p.pi = take(NPI);
  p.grads = take(NGRAD); p.derivs = take(NDER); p.in_e = take(1); p.in_s = take(1); p.in_rho = take(3);
  p.frz1_e = take(1);
  p.partials = d;
  d += (size_t)kTotBlocks * 6;
  p.clock = reinterpret_cast<Clock*>(d);
  int32_t* ip = ctx->ibuf;
  auto itake = [&](size_t k) { int32_t* r = ip; ip += k; return r; };
  p.eos_id = itake(n); p.eos_iters = itake(n); p.btrack = itake(n); p.freeze = itake(n);
  p.cell_of = itake(n); p.cell_rank = itake(n); p.cell_idx = itake(n); p.cand_cnt = itake(n);
  p.cell_count = itake(g.ncell); p.cell_start = itake(g.ncell + 1); p.err = itake(NERR); p.cand_max = itake(1);
  p.scan_aux = itake(2 * (size_t)scan_tiles(g.ncell) + 1);
  // upload permuted inputs
  std::vector<double> tmp((size_t)n);
  auto up = [&](const double* src, double* dst) -> ccake_status_t {
    for (int64_t k = 0; k < n; k++) tmp[k] = src ? src[ctx->perm[k]] : 0.0;
    CK(cudaMemcpyAsync(dst, tmp.data(), n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return CCAKE_OK;
  };
  if (ctx->cfg.using_diffusion) {
    // diffusion slabs (zero: no initial current unless one is set)
    if (cudaMalloc(&p.dif, (size_t)NDIF * n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&p.recQ, (size_t)RQ * n * sizeof(double)) != cudaSuccess)
      return fail(ctx, CCAKE_ERR_NOMEM, "diffusion allocation");
    CK(cudaMemsetAsync(p.dif, 0, (size_t)NDIF * n * sizeof(double), ctx->stream));
    CK(cudaMemsetAsync(p.recQ, 0, (size_t)RQ * n * sizeof(double), ctx->stream));
  }
  ccake_status_t s;
  if ((s = up(h->x, p.y + Y_X0 * n)) || (s = up(h->y, p.y + Y_X1 * n)) ||
      (s = up(ctx->cfg.dim == 3 ? h->eta : nullptr, p.y + Y_X2 * n)) || (s = up(h->ux, p.y + Y_U0 * n)) ||
      (s = up(h->uy, p.y + Y_U1 * n)) || (s = up(ctx->cfg.dim == 3 ? h->ueta : nullptr, p.y + Y_U2 * n)) ||
      (s = up(h->e_or_s, p.in_e)) || (s = up(h->rhoB, p.in_rho)) || (s = up(h->rhoS, p.in_rho + n)) ||
      (s = up(h->rhoQ, p.in_rho + 2 * n)))
    return s;
  // the event's device-side state for the grouped mixed kernels: active,
  // no tau limit (the host decides how many steps it takes alone)
  ctx->nblk = (int)((n + kBlock - 1) / kBlock);
  if (cudaMalloc(&ctx->d_state, sizeof(EventState)) != cudaSuccess)
    return fail(ctx, CCAKE_ERR_NOMEM, "device allocation");
  {
    EventState st{};
    st.tau_max = 1e300;
    st.active = 1;
    CK(cudaMemcpyAsync(ctx->d_state, &st, sizeof(st), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  ctx->loaded = true;
  ctx->initialized = false;
  return CCAKE_OK;
}

ccake_status_t ccake_set_initial_viscous(ccake_ctx* ctx, const double* trace, const double* pi) {
  if (!ctx || (!trace && !pi)) return CCAKE_ERR_INVALID;
  if (!ctx->loaded) return fail(ctx, CCAKE_ERR_STATE, "load particles first");
  if (ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "set the initial viscous state before initialize");
  const int64_t n = ctx->n;
  if (!ctx->init_visc && cudaMalloc(&ctx->init_visc, 6 * (size_t)n * sizeof(double)) != cudaSuccess)
    return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
  std::vector<double> tmp((size_t)n);
  auto up = [&](const double* src, int row) -> ccake_status_t {
    for (int64_t k = 0; k < n; k++) tmp[k] = src[ctx->perm[k]];
    CK(cudaMemcpyAsync(ctx->init_visc + (size_t)row * n, tmp.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return CCAKE_OK;
  };
  ccake_status_t s;
  if (trace) {
    if ((s = up(trace, 0))) return s;
    ctx->init_bulk = 1;
  }
  if (pi) {
    for (int k = 0; k < 5; k++)
      if ((s = up(pi + (size_t)k * n, 1 + k))) return s;
    ctx->init_shear = 1;
  }
  return CCAKE_OK;
}

ccake_status_t ccake_set_initial_diffusion(ccake_ctx* ctx, const double* q) {
  if (!ctx || !q) return CCAKE_ERR_INVALID;
  if (!ctx->loaded) return fail(ctx, CCAKE_ERR_STATE, "load particles first");
  if (!ctx->p.dif) return fail(ctx, CCAKE_ERR_STATE, "the diffusion sector is off");
  if (ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "set the initial current before initialize");
  const int64_t n = ctx->n;
  if (!ctx->init_q && cudaMalloc(&ctx->init_q, 9 * (size_t)n * sizeof(double)) != cudaSuccess)
    return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
  std::vector<double> tmp((size_t)n);
  for (int c = 0; c < 3; c++)
    for (int i = 0; i < 3; i++) {
      const double* src = q + (size_t)(4 * c + i + 1) * n;
      for (int64_t k = 0; k < n; k++) tmp[k] = src[ctx->perm[k]];
      CK(cudaMemcpyAsync(ctx->init_q + (size_t)(3 * c + i) * n, tmp.data(), n * sizeof(double),
                         cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
  return CCAKE_OK;
}

ccake_status_t ccake_initialize(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (!ctx->loaded) return fail(ctx, CCAKE_ERR_STATE, "load particles first");
  if (ctx->eos.kind == 2 && !ctx->d_table) return fail(ctx, CCAKE_ERR_STATE, "set the EoS table first");
  const double t0 = ctx->cfg.t0;
  Clock c{t0, t0, t0, 0, 0, 0.0, 0.0, 1.0 / t0, 1.0 / (t0 * t0)};
  CK(cudaMemcpyAsync(ctx->p.clock, &c, sizeof(Clock), cudaMemcpyHostToDevice, ctx->stream));
  ccake_status_t s = reset_errors(ctx);
  if (s) return s;
  if (ctx->cfg.particlization && ctx->cfg.surface) {
    // freeze-out snapshots (zero, as the reference's freeze_array) and the
    // hypersurface rows, one a particle at most
    const size_t n = (size_t)ctx->n;
    if (!ctx->p.fz && (cudaMalloc(&ctx->p.fz, 6 * NSF * n * sizeof(double)) != cudaSuccess ||
                       cudaMalloc(&ctx->p.fo_rows, n * kFoRow * sizeof(double)) != cudaSuccess ||
                       cudaMalloc(&ctx->p.fo_count, sizeof(int32_t)) != cudaSuccess))
      return fail(ctx, CCAKE_ERR_NOMEM, "freeze-out snapshot allocation");
    CK(cudaMemsetAsync(ctx->p.fz, 0, 6 * NSF * n * sizeof(double), ctx->stream));
    CK(cudaMemsetAsync(ctx->p.fo_count, 0, sizeof(int32_t), ctx->stream));
    drop_graph(ctx);
  }
  // neighbour-list capacity: 1.5x the largest initial neighbour count + 16
  // (pass A flags an overflow, reported as CCAKE_ERR_CAPACITY)
  {
    launch_build_cells(ctx->rc, ctx->p, ctx->stream);
    launch_neighbour_counts(ctx->rc, ctx->p, ctx->p.btrack, ctx->stream);
    std::vector<int32_t> cnt((size_t)ctx->n);
    CK(cudaMemcpyAsync(cnt.data(), ctx->p.btrack, ctx->n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const int mx = *std::max_element(cnt.begin(), cnt.end());
    const int K = ((mx * 3 / 2 + 16) + 15) / 16 * 16;
    if (K != ctx->p.K) {
      drop_graph(ctx);
      free_lists(ctx);
      if (!alloc_lists(ctx, K)) return fail(ctx, CCAKE_ERR_NOMEM, "neighbour list allocation");
      ctx->p.K = K;
    }
  }
  launch_init_state(ctx->rc, ctx->p, ctx->stream);
  if (ctx->cfg.seed_mode == CCAKE_SEED_LEARNED) {
    // the seed network maps every particle's (e, rho) to a (T, mu) seed
    if (!ctx->mlp_ready) return fail(ctx, CCAKE_ERR_STATE, "seed_mode learned: train the seed network first");
    double *in4 = nullptr, *tbqs = nullptr;
    if (cudaMalloc(&in4, (size_t)4 * ctx->n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&tbqs, (size_t)4 * ctx->n * sizeof(double)) != cudaSuccess) {
      if (in4) cudaFree(in4);
      return fail(ctx, CCAKE_ERR_NOMEM, "seed allocation");
    }
    launch_pack_inputs(ctx->p, in4, ctx->stream);
    launch_mlp_seed(MlpDev{ctx->mlp_buf, ctx->mlp_norm}, ctx->n, in4, tbqs, ctx->mlp_err, ctx->stream);
    launch_init_invert(ctx->rc, ctx->eos, ctx->p, tbqs, ctx->stream);
    const cudaError_t e1 = cudaStreamSynchronize(ctx->stream);
    cudaFree(in4);
    cudaFree(tbqs);
    if (e1 != cudaSuccess) return fail(ctx, CCAKE_ERR_CUDA, cudaGetErrorString(e1));
    if ((s = mlp_check(ctx))) return s;
  } else {
    launch_init_invert(ctx->rc, ctx->eos, ctx->p, nullptr, ctx->stream);
  }
  // a particle without a solution even at zero charge ends the
  // initialisation here, as the reference throws (src/sph_workstation.cpp:
  // 1840-1846); its eos_id (-1) stays for the caller to read
  if ((s = check_errors(ctx))) return s;
  // candidate-list capacity: 1.5x the largest count + 16 (a build flags an
  // overflow, reported as CCAKE_ERR_CAPACITY)
  {
    launch_build_cells(ctx->rc, ctx->p, ctx->stream);
    const int keep = ctx->p.Kc;
    ctx->p.Kc = 0;   // count only
    launch_candidates(ctx->rc, ctx->p, ctx->stream);
    ctx->p.Kc = keep;
    std::vector<int32_t> cnt((size_t)ctx->n);
    CK(cudaMemcpyAsync(cnt.data(), ctx->p.cand_cnt, ctx->n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const int mx = *std::max_element(cnt.begin(), cnt.end());
    const int Kc = ((mx * 3 / 2 + 16) + 15) / 16 * 16;
    if (Kc > ctx->p.Kc) {
      drop_graph(ctx);
      free_candidates(ctx);
      if (cudaMalloc(&ctx->p.cand_idx, (size_t)Kc * ctx->n * sizeof(int32_t)) != cudaSuccess)
        return fail(ctx, CCAKE_ERR_NOMEM, "candidate list allocation");
      ctx->p.Kc = Kc;
    }
  }
  ctx->lists_valid = false;
  s = maybe_rebuild(ctx, false);
  if (s) return s;
  launch_passA(ctx->rc, ctx->eos, ctx->p, A_SMOOTH_ONLY, ctx->stream);   // initial sigma
  launch_init_ext(ctx->rc, ctx->p, ctx->stream);
  const int64_t n = ctx->n;
  if (ctx->p.dif || ctx->init_bulk || ctx->init_shear) {
    // initial smoothing, then calculate_extensive_shv, set_bulk_Pi and
    // set_diffusion against its sigma (src/sph_workstation.cpp:394-457,
    // :1350-1458), then the thermodynamics, pi, Pi and q^mu
    launch_passA(ctx->rc, ctx->eos, ctx->p, A_SMOOTH_ONLY, ctx->stream);
    launch_init_viscous(ctx->p, ctx->init_visc, ctx->init_bulk, ctx->init_shear, ctx->stream);
    launch_init_diffusion(ctx->p, ctx->init_q, ctx->stream);
    launch_thermo(ctx->rc, ctx->eos, ctx->p, ctx->stream);
    if (ctx->p.dif)
      CK(cudaMemcpyAsync(ctx->p.dif + (size_t)F_YQ0 * n, ctx->p.dif + (size_t)F_YQ * n, 9 * n * sizeof(double),
                         cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    launch_passA(ctx->rc, ctx->eos, ctx->p, A_WITH_THERMO, ctx->stream);   // initial smoothing
  }
  CK(cudaMemcpyAsync(ctx->p.y0, ctx->p.y, NY * n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  s = check_errors(ctx);
  if (s) return s;
  ctx->records_form = 0;
  ctx->t = ctx->cfg.t0;
  ctx->initialized = true;
  return CCAKE_OK;
}

ccake_status_t ccake_step(ccake_ctx* ctx, int32_t n_steps) {
  if (!ctx || n_steps < 0) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  ccake_status_t s = reset_errors(ctx);
  if (s) return s;
  if (ctx->cfg.precision == 1 && (s = sync_slot(ctx))) return s;
  ensure_records(ctx, ctx->cfg.precision);
  if ((s = ensure_step_graph(ctx))) return s;
  for (int k = 0; k < n_steps; k++) {
    if ((s = maybe_rebuild(ctx, true)) || (s = ensure_step_graph(ctx))) return s;
    CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->launches += ctx->step_kernels;
    ctx->steps_since_build++;
    ctx->evaluated = true;
  }
  s = check_errors(ctx);
  Clock c;
  CK(cudaMemcpy(&c, ctx->p.clock, sizeof(Clock), cudaMemcpyDeviceToHost));
  ctx->t = c.t;
  return s;
}

ccake_status_t ccake_step_timed(ccake_ctx* ctx, int32_t n_steps, float* device_ms) {
  if (!ctx || n_steps < 0 || !device_ms) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  ccake_status_t s = ccake_step(ctx, 0);   // builds the graph, clears errors
  if (s) return s;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, ctx->stream));
  for (int k = 0; k < n_steps; k++) {
    if ((s = maybe_rebuild(ctx, true)) || (s = ensure_step_graph(ctx))) return s;
    CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->launches += ctx->step_kernels;
    ctx->steps_since_build++;
    ctx->evaluated = true;
  }
  CK(cudaEventRecord(e1, ctx->stream));
  CK(cudaEventSynchronize(e1));
  CK(cudaEventElapsedTime(device_ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s = check_errors(ctx);
  Clock c;
  CK(cudaMemcpy(&c, ctx->p.clock, sizeof(Clock), cudaMemcpyDeviceToHost));
  ctx->t = c.t;
  return s;
}

ccake_status_t ccake_kernel_launches(const ccake_ctx* ctx, int64_t* launches) {
  if (!ctx || !launches) return CCAKE_ERR_INVALID;
  *launches = ctx->launches;
  return CCAKE_OK;
}

ccake_status_t ccake_profile_phases(ccake_ctx* ctx, int32_t n_steps, double* ms3) {
  if (!ctx || n_steps <= 0 || !ms3) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  ccake_status_t s = reset_errors(ctx);
  if (s) return s;
  ensure_records(ctx, ctx->cfg.precision);
  cudaEvent_t ev[4];
  for (int q = 0; q < 4; q++) CK(cudaEventCreate(&ev[q]));
  double acc[3] = {0, 0, 0};
  for (int k = 0; k < n_steps; k++) {
    for (int sub = 1; sub <= 2; sub++) {
      CK(cudaEventRecord(ev[0], ctx->stream));
      if (sub == 1 && (s = maybe_rebuild(ctx, false))) return s;
      if (ctx->cfg.precision == 1 && (s = sync_slot(ctx))) return s;   // the lists may have grown
      CK(cudaEventRecord(ev[1], ctx->stream));
      enqueue_passA(ctx);
      CK(cudaEventRecord(ev[2], ctx->stream));
      enqueue_passB(ctx, B_EOM | B_UPDATE | (sub == 2 ? B_WRITE_Y0 : 0), sub);
      CK(cudaEventRecord(ev[3], ctx->stream));
      enqueue_clock(ctx, sub);
      if (sub == 2 && ctx->cfg.particlization) enqueue_freeze(ctx);
      if (sub == 2) ctx->steps_since_build++;
      CK(cudaEventSynchronize(ev[3]));
      float m;
      for (int q = 0; q < 3; q++) {
        CK(cudaEventElapsedTime(&m, ev[q], ev[q + 1]));
        acc[q] += m;
      }
    }
  }
  for (int q = 0; q < 4; q++) cudaEventDestroy(ev[q]);
  for (int q = 0; q < 3; q++) ms3[q] = acc[q] / (2.0 * n_steps);
  s = check_errors(ctx);
  Clock c;
  CK(cudaMemcpy(&c, ctx->p.clock, sizeof(Clock), cudaMemcpyDeviceToHost));
  ctx->t = c.t;
  return s;
}

ccake_status_t ccake_device_bytes(const ccake_ctx* ctx, int64_t* bytes) {
  if (!ctx || !bytes) return CCAKE_ERR_INVALID;
  const int64_t n = ctx->n;
  const int64_t nd = n * kDoublesPerParticle;
  const int64_t ni = n * 8 + (int64_t)ctx->rc.grid.ncell * 2 + 2 * (int64_t)scan_tiles(ctx->rc.grid.ncell);
  *bytes = nd * 8 + ni * 4 + (int64_t)ctx->p.K * n * 12 + (int64_t)ctx->p.Kc * n * 4;
  if (ctx->p.dif) *bytes += (int64_t)(NDIF + RQ) * n * 8;
  if (ctx->init_q) *bytes += 9 * n * 8;
  if (ctx->init_visc) *bytes += 6 * n * 8;
  return CCAKE_OK;
}

ccake_status_t ccake_continue_evolution(ccake_ctx* ctx, double max_tau, int32_t* keep_going) {
  if (!ctx || !keep_going) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  bool keep = true;
  if (ctx->cfg.particlization) {
    if (!ctx->d_count && cudaMalloc(&ctx->d_count, sizeof(int32_t)) != cudaSuccess)
      return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
    launch_count_frozen(ctx->p, ctx->d_count, ctx->stream);
    int32_t frozen = 0;
    CK(cudaMemcpyAsync(&frozen, ctx->d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    keep = frozen < ctx->n;
  }
  *keep_going = (keep && ctx->t <= max_tau) ? 1 : 0;
  return CCAKE_OK;
}

ccake_status_t ccake_build_neighbours(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (!ctx->loaded) return fail(ctx, CCAKE_ERR_STATE, "load particles first");
  launch_build_cells(ctx->rc, ctx->p, ctx->stream);
  if (ctx->p.cand_idx) {
    launch_candidates(ctx->rc, ctx->p, ctx->stream);
    ctx->lists_valid = true;
    ctx->steps_since_build = 0;
  }
  return check_errors(ctx);
}

ccake_status_t ccake_smooth_fields(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  ensure_records(ctx, 0);   // the phase entry points run the FP64 form
  ccake_status_t s = maybe_rebuild(ctx, false);   // lists valid by the schedule are kept
  if (s) return s;
  launch_passA(ctx->rc, ctx->eos, ctx->p, A_SMOOTH_ONLY, ctx->stream);
  return check_errors(ctx);
}

ccake_status_t ccake_update_thermo(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  ccake_status_t s = reset_errors(ctx);
  if (s) return s;
  launch_thermo(ctx->rc, ctx->eos, ctx->p, ctx->stream);
  return check_errors(ctx);
}

ccake_status_t ccake_update_viscosities(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  launch_visc(ctx->rc, ctx->p, ctx->stream);
  return check_errors(ctx);
}

ccake_status_t ccake_smooth_gradients(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  launch_passB(ctx->rc, ctx->p, B_GRADS, 0.0, ctx->stream);
  return check_errors(ctx);
}

ccake_status_t ccake_time_derivatives(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  launch_passB(ctx->rc, ctx->p, B_GRADS | B_EOM | B_DERIVS, 0.0, ctx->stream);
  return check_errors(ctx);
}

ccake_status_t ccake_get_time(const ccake_ctx* ctx, double* t) {
  if (!ctx || !t) return CCAKE_ERR_INVALID;
  *t = ctx->t;
  return CCAKE_OK;
}

ccake_status_t ccake_get_count(const ccake_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return CCAKE_ERR_INVALID;
  *n = ctx->n;
  return CCAKE_OK;
}

ccake_status_t ccake_conservation(ccake_ctx* ctx, ccake_totals* out) {
  if (!ctx || !out) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  launch_totals(ctx->rc, ctx->p, kTotBlocks, ctx->stream);
  std::vector<double> part((size_t)kTotBlocks * 6);
  CK(cudaMemcpyAsync(part.data(), ctx->p.partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < kTotBlocks; b++)
    for (int q = 0; q < 6; q++) acc[q] += part[b * 6 + q];
  *out = ccake_totals{acc[0], acc[1], acc[2], acc[3], acc[4], acc[5]};
  return CCAKE_OK;
}

ccake_status_t ccake_copy_out(ccake_ctx* ctx, const char* field, double* host_out) {
  if (!ctx || !field || !host_out) return CCAKE_ERR_INVALID;
  if (!ctx->loaded) return fail(ctx, CCAKE_ERR_STATE, "load particles first");
  FieldRef f = field_ref(ctx, field);
  if (!f.ok) return fail(ctx, CCAKE_ERR_INVALID, std::string("unknown field ") + field);
  std::vector<double> tmp((size_t)ctx->n);
  CK(cudaMemcpyAsync(tmp.data(), f.base, ctx->n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int64_t k = 0; k < ctx->n; k++) host_out[ctx->perm[k]] = tmp[k];
  return CCAKE_OK;
}

ccake_status_t ccake_copy_out_int(ccake_ctx* ctx, const char* field, int32_t* host_out) {
  if (!ctx || !field || !host_out) return CCAKE_ERR_INVALID;
  if (!ctx->loaded) return fail(ctx, CCAKE_ERR_STATE, "load particles first");
  const std::string k(field);
  const int32_t* base = k == "btrack" ? ctx->p.btrack : k == "eos_id" ? ctx->p.eos_id
                      : k == "eos_iters" ? ctx->p.eos_iters : k == "freeze" ? ctx->p.freeze : nullptr;
  if (!base) return fail(ctx, CCAKE_ERR_INVALID, "unknown field " + k);
  std::vector<int32_t> tmp((size_t)ctx->n);
  CK(cudaMemcpyAsync(tmp.data(), base, ctx->n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int64_t q = 0; q < ctx->n; q++) host_out[ctx->perm[q]] = tmp[q];
  return CCAKE_OK;
}

ccake_status_t ccake_get_neighbours(ccake_ctx* ctx, int32_t* offsets, int32_t* idx, int64_t idx_cap, int64_t* count) {
  if (!ctx || !offsets || !count) return CCAKE_ERR_INVALID;
  if (!ctx->loaded) return fail(ctx, CCAKE_ERR_STATE, "load particles first");
  const int64_t n = ctx->n;
  int32_t* d_cnt = nullptr;
  CK(cudaMalloc(&d_cnt, (n + 1) * sizeof(int32_t)));
  launch_build_cells(ctx->rc, ctx->p, ctx->stream);
  launch_neighbour_counts(ctx->rc, ctx->p, d_cnt, ctx->stream);
  std::vector<int32_t> cnt(n), off(n + 1, 0);
  cudaError_t e = cudaMemcpyAsync(cnt.data(), d_cnt, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) { cudaFree(d_cnt); return fail(ctx, CCAKE_ERR_CUDA, cudaGetErrorString(e)); }
  for (int64_t k = 0; k < n; k++) off[k + 1] = off[k] + cnt[k];
  const int64_t m = off[n];
  *count = m;
  // offsets in the caller's order
  std::vector<int32_t> inv(n);
  for (int64_t k = 0; k < n; k++) inv[ctx->perm[k]] = (int32_t)k;
  offsets[0] = 0;
  for (int64_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + cnt[inv[i]];
  if (!idx || idx_cap < m) { cudaFree(d_cnt); return fail(ctx, CCAKE_ERR_CAPACITY, "idx_cap too small"); }
  int32_t *d_off = nullptr, *d_idx = nullptr;
  CK(cudaMalloc(&d_off, (n + 1) * sizeof(int32_t)));
  CK(cudaMalloc(&d_idx, std::max<int64_t>(m, 1) * sizeof(int32_t)));
  CK(cudaMemcpyAsync(d_off, off.data(), (n + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
  launch_neighbour_fill(ctx->rc, ctx->p, d_off, d_idx, ctx->stream);
  std::vector<int32_t> all(m);
  CK(cudaMemcpyAsync(all.data(), d_idx, m * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(d_cnt);
  cudaFree(d_off);
  cudaFree(d_idx);
  for (int64_t i = 0; i < n; i++) {
    const int32_t k = inv[i];
    int32_t* row = idx + offsets[i];
    for (int32_t j = 0; j < cnt[k]; j++) row[j] = ctx->perm[all[off[k] + j]];
    std::sort(row, row + cnt[k]);
  }
  return check_errors(ctx);
}

ccake_status_t ccake_eos_table_fallback_scales(const int32_t* n, const double* lo, const double* d,
                                              const double* fields, double freeze_out_T, double* conf5,
                                              double* cdiag5) {
  if (!n || !lo || !d || !fields || !conf5 || !cdiag5 || !(freeze_out_T > 0)) return CCAKE_ERR_INVALID;
  EosDev host{};
  host.kind = 2;
  double mx[4];
  for (int k = 0; k < 4; k++) {
    if (n[k] < 1 || !(d[k] >= 0.0) || !std::isfinite(lo[k])) return CCAKE_ERR_INVALID;
    host.tab.n[k] = n[k];
    host.tab.lo[k] = lo[k];
    host.tab.d[k] = d[k];
    mx[k] = lo[k] + d[k] * (n[k] - 1);   // grid maxima (get_tbqs_maxima_no_ext)
  }
  host.tab.f = fields;
  // the reference's matching (src/eos_initialization.cpp:276-341 for the
  // tanh-conformal and conformal fallbacks, :343-403 and :404-464 for the
  // conformal-diagonal one): p/T^4 at Tmax = 1.1 T_FO fixes c (T0 = 1), and
  // p at (Tmax, mu_max) on each axis fixes that axis' scale
  const double Tmax = 1.1 * freeze_out_T;
  auto p_at = [&](double T, double mB, double mQ, double mS) {
    double x4[4] = {T, mB, mQ, mS}, o[17];
    table_thermo(host.tab, x4, o);
    return o[0];
  };
  const double pT = p_at(Tmax, 0.0, 0.0, 0.0);
  const double c = pT / (Tmax * Tmax * Tmax * Tmax);
  conf5[0] = cdiag5[0] = c;
  conf5[1] = cdiag5[1] = 1.0;
  for (int a = 1; a < 4; a++) {   // muB, muQ, muS: the scales' order
    if (std::fabs(mx[a]) < 1e-30) { conf5[1 + a] = cdiag5[1 + a] = 1.0; continue; }
    double x[4] = {Tmax, 0.0, 0.0, 0.0};
    x[a] = mx[a];
    const double pv = p_at(x[0], x[1], x[2], x[3]);
    conf5[1 + a] = std::pow(c, 0.25) * mx[a] / std::sqrt(std::sqrt(pv) - std::sqrt(pT));
    cdiag5[1 + a] = std::pow(c / (pv - pT), 0.25) * mx[a];
  }
  for (int q = 0; q < 5; q++)
    if (!(conf5[q] > 0.0) || !(cdiag5[q] > 0.0) || !std::isfinite(conf5[q]) || !std::isfinite(cdiag5[q]))
      return CCAKE_ERR_INVALID;
  return CCAKE_OK;
}

ccake_status_t ccake_set_eos_table(ccake_ctx* ctx, const int32_t* n, const double* lo, const double* d,
                                   const double* fields, const double* conf5_in, const double* cdiag5_in) {
  if (!ctx || !n || !lo || !d || !fields) return CCAKE_ERR_INVALID;
  if (ctx->eos.kind != 2) return fail(ctx, CCAKE_ERR_INVALID, "eos_kind is not 2 (table)");
  size_t nodes = 1;
  for (int k = 0; k < 4; k++) {
    if (n[k] < 1 || !(d[k] >= 0.0) || !std::isfinite(lo[k])) return fail(ctx, CCAKE_ERR_INVALID, "bad table axis");
    nodes *= (size_t)n[k];
  }
  if (nodes > ((size_t)1 << 31)) return fail(ctx, CCAKE_ERR_INVALID, "table too large");
  // fallback scales: given, or matched to the table as the reference does
  double ref_conf[5], ref_cdiag[5];
  const double* conf5 = conf5_in;
  const double* cdiag5 = cdiag5_in;
  if (!conf5 || !cdiag5) {
    if (ccake_eos_table_fallback_scales(n, lo, d, fields, ctx->cfg.freeze_out_T, ref_conf, ref_cdiag))
      return fail(ctx, CCAKE_ERR_INVALID, "the table gives no fallback scales at 1.1 T_FO");
    if (!conf5) conf5 = ref_conf;
    if (!cdiag5) cdiag5 = ref_cdiag;
  }
  for (int q = 0; q < 5; q++)
    if (!(conf5[q] > 0.0) || !(cdiag5[q] > 0.0)) return fail(ctx, CCAKE_ERR_INVALID, "bad fallback scales");
  drop_graph(ctx);
  if (ctx->d_table) cudaFree(ctx->d_table);
  if (ctx->d_table_f) cudaFree(ctx->d_table_f);
  ctx->d_table = nullptr;
  ctx->d_table_f = nullptr;
  if (cudaMalloc(&ctx->d_table, nodes * 17 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&ctx->d_table_f, nodes * 8 * sizeof(float)) != cudaSuccess)
    return fail(ctx, CCAKE_ERR_NOMEM, "table allocation");
  CK(cudaMemcpyAsync(ctx->d_table, fields, nodes * 17 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  launch_table_f32(ctx->d_table, ctx->d_table_f, (int64_t)nodes, ctx->stream);
  CK(cudaStreamSynchronize(ctx->stream));
  EosDev& e = ctx->eos;
  for (int k = 0; k < 4; k++) {
    e.tab.n[k] = n[k];
    e.tab.lo[k] = lo[k];
    e.tab.d[k] = d[k];
    e.tab.id[k] = d[k] > 0.0 ? 1.0 / d[k] : 0.0;
  }
  e.conf = make_scales(conf5[0], conf5[1], conf5[2], conf5[3], conf5[4]);
  e.cdiag = make_scales(cdiag5[0], cdiag5[1], cdiag5[2], cdiag5[3], cdiag5[4]);
  // e(T_FO, 0, 0, 0) from the table, evaluated on the host copy
  EosDev host = e;
  host.tab.f = fields;
  host.tab.fd = nullptr;
  host.pre = nullptr;
  double x4[4] = {ctx->cfg.freeze_out_T, 0, 0, 0}, o[17];
  model_thermo(host, M_TABLE, x4, o);
  ctx->rc.efreeze = o[5];
  e.tab.f = ctx->d_table;
  e.tab.fd = ctx->d_table_f;
  return CCAKE_OK;
}

ccake_status_t ccake_set_eos_table_file(ccake_ctx* ctx, const char* eos_path, int32_t normalize_by_T,
                                        const double* conf5, const double* cdiag5) {
  if (!ctx || !eos_path) return CCAKE_ERR_INVALID;
  std::string path(eos_path);
  struct stat st{};
  if (stat(path.c_str(), &st) == 0 && S_ISDIR(st.st_mode)) path += "/thermo.dat";
  FILE* fh = std::fopen(path.c_str(), "rb");
  if (!fh) return fail(ctx, CCAKE_ERR_INVALID, "cannot open " + path);
  std::string text;
  {
    char buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof(buf), fh)) > 0) text.append(buf, k);
    std::fclose(fh);
  }
  const char* c = text.c_str();
  const char* end = c + text.size();
  // header: the grid sizes
  int32_t n[4];
  {
    const char* eol = static_cast<const char*>(std::memchr(c, '\n', end - c));
    if (!eol) return fail(ctx, CCAKE_ERR_INVALID, "no header line");
    std::string head(c, eol);
    int k = std::sscanf(head.c_str(), "%d %d %d %d", &n[0], &n[1], &n[2], &n[3]);
    if (k != 4) return fail(ctx, CCAKE_ERR_INVALID, "the header must hold 4 grid sizes");
    c = eol + 1;
  }
  size_t nodes = 1;
  for (int k = 0; k < 4; k++) {
    if (n[k] < 1) return fail(ctx, CCAKE_ERR_INVALID, "bad grid size");
    nodes *= (size_t)n[k];
    // a row is 21 numbers of at least two characters: grid sizes the file
    // cannot hold are rejected before anything is allocated
    if (nodes > (text.size() / 42) + 1) return fail(ctx, CCAKE_ERR_INVALID, "the table has fewer rows than its grid sizes give");
  }
  std::vector<double> grid(nodes * 4), fields(nodes * 17);
  size_t row = 0;
  while (c < end && row < nodes) {
    while (c < end && (*c == ' ' || *c == '\t' || *c == '\r' || *c == '\n')) c++;
    if (c >= end) break;
    for (int q = 0; q < 21; q++) {
      char* stop = nullptr;
      const double v = std::strtod(c, &stop);
      if (stop == c) return fail(ctx, CCAKE_ERR_INVALID, "row " + std::to_string(row) + ": expected 21 numbers");
      c = stop;
      if (q < 4) grid[row * 4 + q] = v;
      else fields[row * 17 + (q - 4)] = v;
    }
    row++;
  }
  if (row != nodes) return fail(ctx, CCAKE_ERR_INVALID, "the table has fewer rows than its grid sizes give");
  // axes to fm^-1, grids rebuilt from the extremes; field units
  const double hc1 = 1.0 / 197.3269804;
  static const int pw[17] = {4, 3, 3, 3, 3, 4, 0, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2};
  double lo[4], hi[4], d[4];
  for (int k = 0; k < 4; k++) { lo[k] = 1e300; hi[k] = -1e300; }
  for (size_t r = 0; r < nodes; r++)
    for (int k = 0; k < 4; k++) {
      const double v = grid[r * 4 + k] * hc1;
      grid[r * 4 + k] = v;
      lo[k] = std::min(lo[k], v);
      hi[k] = std::max(hi[k], v);
    }
  for (int k = 0; k < 4; k++) {
    d[k] = n[k] <= 1 ? 0.0 : (hi[k] - lo[k]) / (n[k] - 1.0);
    if (!std::isfinite(lo[k]) || !std::isfinite(hi[k]) || (n[k] > 1 && !(d[k] > 0.0)))
      return fail(ctx, CCAKE_ERR_INVALID, "grid axis " + std::to_string(k) + " is not an increasing finite range");
  }
  for (double v : fields)
    if (!std::isfinite(v)) return fail(ctx, CCAKE_ERR_INVALID, "non-finite table value");
  for (size_t r = 0; r < nodes; r++) {
    const double T = grid[r * 4];
    for (int q = 0; q < 17; q++) {
      if (pw[q] == 0) continue;
      fields[r * 17 + q] *= normalize_by_T ? std::pow(T, pw[q]) : std::pow(hc1, pw[q]);
    }
  }
  return ccake_set_eos_table(ctx, n, lo, d, fields.data(), conf5, cdiag5);
}

ccake_status_t ccake_sph_kernel(int32_t dim, double h, int64_t n, const double* r2, double* w, double* fg) {
  if ((dim != 2 && dim != 3) || !(h > 0.0) || !std::isfinite(h) || n < 0) return CCAKE_ERR_INVALID;
  if (n == 0) return CCAKE_OK;
  if (!r2 || !w || !fg) return CCAKE_ERR_INVALID;
  for (int64_t i = 0; i < n; i++)
    if (!(r2[i] >= 0.0) || !std::isfinite(r2[i])) return CCAKE_ERR_INVALID;
  RunConst rc{};
  set_kernel_constants(rc, dim, h);
  double* d = nullptr;
  if (cudaMalloc(&d, n * 3 * sizeof(double)) != cudaSuccess) return CCAKE_ERR_NOMEM;
  cudaError_t err = cudaMemcpy(d, r2, n * sizeof(double), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    launch_sph_kernel(rc, n, d, d + n, d + 2 * n, 0);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpy(w, d + n, n * sizeof(double), cudaMemcpyDeviceToHost);
  if (err == cudaSuccess) err = cudaMemcpy(fg, d + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return err == cudaSuccess ? CCAKE_OK : CCAKE_ERR_CUDA;
}

ccake_status_t ccake_eos_thermo_batch(ccake_ctx* ctx, int32_t chain_index, int64_t n, const double* tbqs,
                                      double* out17) {
  if (!ctx || n < 0 || !tbqs || !out17) return CCAKE_ERR_INVALID;
  if (chain_index < 0 || chain_index >= chain_len(ctx->eos.kind)) return CCAKE_ERR_INVALID;
  if (ctx->eos.kind == 2 && !ctx->d_table) return fail(ctx, CCAKE_ERR_STATE, "set the EoS table first");
  if (n == 0) return CCAKE_OK;
  double *d_x = nullptr, *d_o = nullptr;
  if (cudaMalloc(&d_x, n * 4 * sizeof(double)) != cudaSuccess) return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
  if (cudaMalloc(&d_o, n * 17 * sizeof(double)) != cudaSuccess) {
    cudaFree(d_x);
    return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
  }
  cudaMemcpyAsync(d_x, tbqs, n * 4 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  launch_eos_thermo(ctx->eos, chain_index, n, d_x, d_o, ctx->stream);
  cudaMemcpyAsync(out17, d_o, n * 17 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  const cudaError_t err = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_x);
  cudaFree(d_o);
  if (err != cudaSuccess) return fail(ctx, CCAKE_ERR_CUDA, cudaGetErrorString(err));
  CK(cudaGetLastError());
  return CCAKE_OK;
}

ccake_status_t ccake_eos_invert_device(ccake_ctx* ctx, int32_t entropy_mode, int32_t seed_mode, int64_t n,
                                       const double* d_in4, double* d_tbqs, double* d_th16, int32_t* d_status,
                                       int32_t* d_iters, void* stream) {
  if (!ctx || n < 0 || (n > 0 && (!d_in4 || !d_tbqs || !d_status))) return CCAKE_ERR_INVALID;
  if (seed_mode < CCAKE_SEED_REFERENCE || seed_mode > CCAKE_SEED_LEARNED) return CCAKE_ERR_INVALID;
  if (ctx->eos.kind == 2 && !ctx->d_table) return fail(ctx, CCAKE_ERR_STATE, "set the EoS table first");
  if (seed_mode == CCAKE_SEED_LEARNED && !ctx->mlp_ready) return fail(ctx, CCAKE_ERR_STATE, "train the seed network first");
  if (n == 0) return CCAKE_OK;
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  if (seed_mode == CCAKE_SEED_LEARNED)
    launch_mlp_seed(MlpDev{ctx->mlp_buf, ctx->mlp_norm}, n, d_in4, d_tbqs, ctx->mlp_err, cs);
  launch_eos_batch(ctx->eos, entropy_mode, seed_mode, n, d_in4, d_tbqs, d_th16, d_status, d_iters,
                   eos_scratch(ctx, n), cs);
  CK(cudaGetLastError());
  return CCAKE_OK;
}

// ---------------------------------------------------------------------------
// learned Newton seed
// ---------------------------------------------------------------------------
ccake_status_t ccake_mlp_train(ccake_ctx* ctx, int64_t n_samples, int32_t epochs, int32_t batch, double lr,
                               uint64_t seed, double* final_mse) {
  if (!ctx || n_samples < 128 || epochs < 1 || batch < 128 || batch > n_samples || !(lr > 0.0))
    return CCAKE_ERR_INVALID;
  if (ctx->eos.kind != 2 || !ctx->d_table) return fail(ctx, CCAKE_ERR_STATE, "the seed network needs the EoS table");
  ccake_status_t st = ensure_mlp(ctx);
  if (st) return st;
  Scratch sc;
  float* feat = sc.get<float>(4 * (size_t)n_samples);
  float* tgt = sc.get<float>(4 * (size_t)n_samples);
  int32_t* okf = sc.get<int32_t>((size_t)n_samples);
  if (!feat || !tgt || !okf) return fail(ctx, CCAKE_ERR_NOMEM, "training-set allocation");
  launch_mlp_samples(ctx->eos, n_samples, seed, feat, tgt, okf, ctx->stream);
  // standardisation from the first rows (up to 262,144)
  const int64_t m = std::min<int64_t>(n_samples, 262144);
  std::vector<float> hf(4 * m), ht(4 * m);
  std::vector<int32_t> hok(m);
  CK(cudaMemcpyAsync(hf.data(), feat, 4 * m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ht.data(), tgt, 4 * m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(hok.data(), okf, m * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  MlpNorm nm{};
  {
    double s1[8] = {0}, s2[8] = {0};
    int64_t c = 0;
    for (int64_t i = 0; i < m; i++) {
      if (!hok[i]) continue;
      c++;
      for (int k = 0; k < 4; k++) {
        s1[k] += hf[4 * i + k]; s2[k] += (double)hf[4 * i + k] * hf[4 * i + k];
        s1[4 + k] += ht[4 * i + k]; s2[4 + k] += (double)ht[4 * i + k] * ht[4 * i + k];
      }
    }
    if (c < 16) return fail(ctx, CCAKE_ERR_EOS, "too few valid training states in the table");
    for (int k = 0; k < 8; k++) {
      const double mu = s1[k] / c, sd = std::sqrt(std::max(s2[k] / c - mu * mu, 1e-12));
      if (k < 4) { nm.in_mean[k] = (float)mu; nm.in_std[k] = (float)sd; }
      else { nm.out_mean[k - 4] = (float)mu; nm.out_std[k - 4] = (float)sd; }
    }
  }
  launch_mlp_standardise(nm, n_samples, feat, tgt, ctx->stream);
  // Glorot-uniform weights, zero biases (64-bit LCG of the seed)
  std::vector<float> prm(mlp::kParams, 0.0f);
  {
    uint64_t r = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto uni = [&]() {
      r = r * 6364136223846793005ull + 1442695040888963407ull;
      return (double)(r >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int nout, int nin) {
      const double a = std::sqrt(6.0 / (nin + nout));
      for (int i = 0; i < nout * nin; i++) prm[off + i] = (float)((2.0 * uni() - 1.0) * a);
    };
    fill(mlp::kW1, 64, 4);
    fill(mlp::kW2, 64, 64);
    fill(mlp::kW3, 64, 64);
    fill(mlp::kW4, 4, 64);
  }
  float* P = ctx->mlp_buf;
  float* G = P + mlp::kParams;
  float* M1 = G + mlp::kParams;
  float* V = M1 + mlp::kParams;
  CK(cudaMemcpyAsync(P, prm.data(), mlp::kParams * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(M1, 0, 2 * mlp::kParams * sizeof(float), ctx->stream));
  ctx->mlp_ready = false;
  const int64_t steps = n_samples / batch;
  const int64_t total = (int64_t)epochs * steps;
  int64_t t = 0;
  double sse = 0.0;
  for (int ep = 0; ep < epochs; ep++) {
    CK(cudaMemsetAsync(ctx->mlp_sse, 0, sizeof(double), ctx->stream));
    for (int64_t s = 0; s < steps; s++) {
      CK(cudaMemsetAsync(G, 0, mlp::kParams * sizeof(float), ctx->stream));
      launch_mlp_grad(P, batch, feat + 4 * s * (int64_t)batch, tgt + 4 * s * (int64_t)batch, G, ctx->mlp_sse,
                      ctx->mlp_err, ctx->stream);
      t++;
      const double c = 0.5 * (1.0 + std::cos(M_PI * (double)t / (double)total));
      launch_mlp_adam(P, G, M1, V, (float)(lr * (0.05 + 0.95 * c)), (int)t, ctx->stream);
    }
    if (ep == epochs - 1 || ep % 8 == 0) {
      if ((st = mlp_check(ctx))) return st;
    }
  }
  CK(cudaMemcpyAsync(&sse, ctx->mlp_sse, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if ((st = mlp_check(ctx))) return st;
  if (final_mse) *final_mse = sse / (4.0 * (double)batch * (double)steps);
  ctx->mlp_norm = nm;
  ctx->mlp_ready = true;
  return CCAKE_OK;
}

ccake_status_t ccake_mlp_get_params(ccake_ctx* ctx, float* params, float* norm16) {
  if (!ctx || !params || !norm16) return CCAKE_ERR_INVALID;
  if (!ctx->mlp_ready) return fail(ctx, CCAKE_ERR_STATE, "no seed network");
  CK(cudaMemcpyAsync(params, ctx->mlp_buf, mlp::kParams * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::memcpy(norm16, &ctx->mlp_norm, sizeof(MlpNorm));
  return CCAKE_OK;
}

ccake_status_t ccake_mlp_set_params(ccake_ctx* ctx, const float* params, const float* norm16) {
  if (!ctx || !params || !norm16) return CCAKE_ERR_INVALID;
  for (int k = 4; k < 8; k++)
    if (!(norm16[k] > 0.0f) || !(norm16[8 + k] > 0.0f)) return fail(ctx, CCAKE_ERR_INVALID, "non-positive std");
  ccake_status_t st = ensure_mlp(ctx);
  if (st) return st;
  CK(cudaMemcpyAsync(ctx->mlp_buf, params, mlp::kParams * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::memcpy(&ctx->mlp_norm, norm16, sizeof(MlpNorm));
  ctx->mlp_ready = true;
  return CCAKE_OK;
}

ccake_status_t ccake_mlp_forward(ccake_ctx* ctx, int64_t n, const float* feat, float* out) {
  if (!ctx || n < 0 || (n > 0 && (!feat || !out))) return CCAKE_ERR_INVALID;
  if (!ctx->mlp_ready) return fail(ctx, CCAKE_ERR_STATE, "no seed network");
  if (n == 0) return CCAKE_OK;
  Scratch sc;
  float* df = sc.get<float>(4 * (size_t)n);
  float* dout = sc.get<float>(4 * (size_t)n);
  if (!df || !dout) return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
  CK(cudaMemcpyAsync(df, feat, 4 * n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  launch_mlp_forward(ctx->mlp_buf, n, df, dout, ctx->mlp_err, ctx->stream);
  CK(cudaMemcpyAsync(out, dout, 4 * n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  return mlp_check(ctx);
}

ccake_status_t ccake_mlp_gradient(ccake_ctx* ctx, int64_t n, const float* feat, const float* tgt, float* grad,
                                  double* sse) {
  if (!ctx || n <= 0 || !feat || !tgt || !grad) return CCAKE_ERR_INVALID;
  if (!ctx->mlp_ready) return fail(ctx, CCAKE_ERR_STATE, "no seed network");
  Scratch sc;
  float* df = sc.get<float>(4 * (size_t)n);
  float* dt = sc.get<float>(4 * (size_t)n);
  if (!df || !dt) return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
  float* G = ctx->mlp_buf + mlp::kParams;
  CK(cudaMemcpyAsync(df, feat, 4 * n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dt, tgt, 4 * n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(G, 0, mlp::kParams * sizeof(float), ctx->stream));
  CK(cudaMemsetAsync(ctx->mlp_sse, 0, sizeof(double), ctx->stream));
  launch_mlp_grad(ctx->mlp_buf, n, df, dt, G, ctx->mlp_sse, ctx->mlp_err, ctx->stream);
  CK(cudaMemcpyAsync(grad, G, mlp::kParams * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  double s = 0.0;
  CK(cudaMemcpyAsync(&s, ctx->mlp_sse, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  ccake_status_t st = mlp_check(ctx);
  if (sse) *sse = s;
  return st;
}

ccake_status_t ccake_eos_invert_batch(ccake_ctx* ctx, int32_t entropy_mode, int64_t n, const double* in4,
                                      double* tbqs, double* th16, int32_t* status, int32_t* iters) {
  return ccake_eos_invert_batch_ex(ctx, entropy_mode, CCAKE_SEED_REFERENCE, n, in4, tbqs, th16, status, iters);
}

ccake_status_t ccake_eos_invert_batch_ex(ccake_ctx* ctx, int32_t entropy_mode, int32_t seed_mode, int64_t n,
                                         const double* in4, double* tbqs, double* th16, int32_t* status,
                                         int32_t* iters) {
  if (!ctx || n < 0 || !in4 || !tbqs || !status) return CCAKE_ERR_INVALID;
  if (seed_mode < CCAKE_SEED_REFERENCE || seed_mode > CCAKE_SEED_LEARNED) return CCAKE_ERR_INVALID;
  if (ctx->eos.kind == 2 && !ctx->d_table) return fail(ctx, CCAKE_ERR_STATE, "set the EoS table first");
  if (seed_mode == CCAKE_SEED_LEARNED && !ctx->mlp_ready) return fail(ctx, CCAKE_ERR_STATE, "train the seed network first");
  if (n == 0) return CCAKE_OK;
  double *d_in = nullptr, *d_x = nullptr, *d_th = nullptr;
  int32_t *d_st = nullptr, *d_it = nullptr;
  CK(cudaMalloc(&d_in, n * 4 * sizeof(double)));
  CK(cudaMalloc(&d_x, n * 4 * sizeof(double)));
  if (th16) CK(cudaMalloc(&d_th, n * 16 * sizeof(double)));
  CK(cudaMalloc(&d_st, n * sizeof(int32_t)));
  if (iters) CK(cudaMalloc(&d_it, n * sizeof(int32_t)));
  CK(cudaMemcpyAsync(d_in, in4, n * 4 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(d_x, tbqs, n * 4 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  if (seed_mode == CCAKE_SEED_LEARNED)
    launch_mlp_seed(MlpDev{ctx->mlp_buf, ctx->mlp_norm}, n, d_in, d_x, ctx->mlp_err, ctx->stream);
  launch_eos_batch(ctx->eos, entropy_mode, seed_mode, n, d_in, d_x, d_th, d_st, d_it, eos_scratch(ctx, n),
                   ctx->stream);
  CK(cudaMemcpyAsync(tbqs, d_x, n * 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (th16) CK(cudaMemcpyAsync(th16, d_th, n * 16 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(status, d_st, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  if (iters) CK(cudaMemcpyAsync(iters, d_it, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(d_in);
  cudaFree(d_x);
  if (d_th) cudaFree(d_th);
  cudaFree(d_st);
  if (d_it) cudaFree(d_it);
  CK(cudaGetLastError());
  return CCAKE_OK;
}

ccake_status_t ccake_hydro_numbers(ccake_ctx* ctx) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (!ctx->initialized) return fail(ctx, CCAKE_ERR_STATE, "initialize first");
  const int64_t n = ctx->n;
  if (!ctx->evaluated) {
    // before the first step no derivative evaluation happened: the
    // reference's stored numbers are still zero
    CK(cudaMemsetAsync(ctx->p.derivs + (size_t)D_THETA * n, 0, (size_t)(NDER - D_THETA) * n * sizeof(double),
                       ctx->stream));
    if (ctx->p.dif)
      CK(cudaMemsetAsync(ctx->p.dif + (size_t)F_KN * n, 0, 6 * (size_t)n * sizeof(double), ctx->stream));
    return check_errors(ctx);
  }
  // the step keeps its gradients in registers: the gradient sums of the last
  // evaluation run again from its records and neighbour list (unchanged since),
  // then the equations of motion from the stored inputs
  const int mixed = ctx->records_form == 1 ? 1 : 0;
  ccake_status_t st;
  if (mixed && (st = sync_slot(ctx))) return st;
  if (mixed) launch_gradients_mixed(ctx->grp, ctx->cfg.dim, ctx->stream);
  else launch_passB(ctx->rc, ctx->p, B_GRADS, 0.0, ctx->stream);
  launch_diagnostics(ctx->rc, ctx->p, mixed, ctx->stream);
  return check_errors(ctx);
}

ccake_status_t ccake_write_system_state(ccake_ctx* ctx, const char* path) {
  if (!ctx || !path) return CCAKE_ERR_INVALID;
  ccake_status_t st = ccake_hydro_numbers(ctx);
  if (st) return st;
  const int64_t n = ctx->n;
  const int D = ctx->cfg.dim;
  static const char* names[] = {"x", "y", "eta", "p", "T", "muB", "muS", "muQ", "e", "rhoB", "rhoS", "rhoQ", "s",
                                "eta_pi", "zeta_Pi", "tau_Pi", "tau_pi", "theta", "inverse_reynolds_shear",
                                "inverse_reynolds_bulk", "shear_knudsen", "bulk_knudsen", "shv00", "shv11", "shv22",
                                "shv01", "shv02", "shv12", "shv13", "shv23", "shv33", "u0", "u1", "u2", "gamma"};
  constexpr int NF = sizeof(names) / sizeof(names[0]);
  std::vector<std::vector<double>> f(NF, std::vector<double>((size_t)n));
  for (int q = 0; q < NF; q++)
    if ((st = ccake_copy_out(ctx, names[q], f[q].data()))) return st;
  std::vector<int32_t> frz((size_t)n), eid((size_t)n);
  if ((st = ccake_copy_out_int(ctx, "freeze", frz.data()))) return st;
  if ((st = ccake_copy_out_int(ctx, "eos_id", eid.data()))) return st;
  // diffusion Knudsen and inverse Reynolds numbers (B, S, Q), zero without
  // the sector
  static const char* dnames[6] = {"kn_diffB", "kn_diffS", "kn_diffQ", "ire_diffB", "ire_diffS", "ire_diffQ"};
  std::vector<std::vector<double>> dn(6, std::vector<double>((size_t)n, 0.0));
  if (ctx->p.dif)
    for (int q = 0; q < 6; q++)
      if ((st = ccake_copy_out(ctx, dnames[q], dn[q].data()))) return st;
  std::ofstream out(path);
  if (!out.is_open()) return fail(ctx, CCAKE_ERR_INVALID, std::string("cannot write ") + path);
  // src/output.cpp:102-181 (print_system_state_to_txt), the same stream
  // manipulators in the same places: the header time and the first row's
  // time come out in the default format, every later number in scientific
  // notation with 6 digits; positions and velocities padded to 3 components;
  // energies and chemical potentials in GeV; the six diffusion numbers
  // (zero without the sector) and no causality check (0).
  const double t = ctx->t;
  const double hc = kHbarcGeVfm;
  out << t << "\n";
  for (int64_t i = 0; i < n; i++) {
    auto F = [&](int q) { return f[q][(size_t)i]; };
    out << i << " " << t << " " << std::setprecision(6) << std::scientific;
    for (int k = 0; k < 3; k++) out << (k < D ? F(k) : 0.0) << " ";
    out << F(3) * hc << " " << F(4) * hc << " " << F(5) * hc << " " << F(6) * hc << " " << F(7) * hc << " "
        << F(8) * hc << " ";
    for (int q = 9; q <= 30; q++) out << F(q) << " ";
    for (int k = 0; k < 3; k++) out << (k < D ? F(31 + k) : 0.0) << " ";
    const int model = chain_model(ctx->eos.kind, eid[(size_t)i]);
    const char* eos_name = model == M_TABLE  ? "table"
                           : model == M_TANH  ? "tanh_conformal"
                           : model == M_CDIAG ? "conformal_diagonal"
                                              : "conformal";
    out << F(34) << " " << frz[(size_t)i] << " " << eos_name << " " << 0 << " ";
    for (int k = 0; k < 6; k++) out << dn[k][(size_t)i] << " ";
    out << "\n";
  }
  out << std::flush;
  if (!out.good()) return fail(ctx, CCAKE_ERR_INVALID, std::string("write failed: ") + path);
  return CCAKE_OK;
}

ccake_status_t ccake_preinverted_build(ccake_ctx* ctx, const ccake_preinv_config* cfg) {
  if (!ctx || !cfg) return CCAKE_ERR_INVALID;
  if (ctx->eos.kind == 2 && !ctx->d_table) return fail(ctx, CCAKE_ERR_STATE, "set the EoS table first");
  PreinvView P{};
  int64_t tiles = 1;
  for (int k = 0; k < 4; k++) {
    P.nt[k] = cfg->exp_hi[k] - cfg->exp_lo[k] + 1;
    if (P.nt[k] < 1 || P.nt[k] > kPreMaxTiles) return fail(ctx, CCAKE_ERR_INVALID, "1 to 8 decades an axis");
    P.e_lo[k] = cfg->exp_lo[k];
    tiles *= P.nt[k];
  }
  if (cfg->nodes < 2 || cfg->nodes > 64) return fail(ctx, CCAKE_ERR_INVALID, "2 to 64 nodes a tile axis");
  P.N = cfg->nodes;
  for (int k = 0; k < 4; k++)
    for (int j = 0; j < P.nt[k]; j++) {
      const int e = cfg->exp_lo[k] + j;
      P.mn[k][j] = std::pow(10., (double)e);
      P.st[k][j] = std::pow(10., (double)(e + 1)) / P.N;
    }
  const int64_t tn = (int64_t)P.N * P.N * P.N * P.N, total = tiles * tn;
  if (ctx->pre_v) cudaFree(ctx->pre_v);
  ctx->pre_v = nullptr;
  ctx->pre_count = 0;
  if (ctx->eos.pre) {
    ctx->eos.pre = nullptr;
    drop_graph(ctx);
  }
  if (cudaMalloc(&ctx->pre_v, (size_t)total * kPreVars * sizeof(double)) != cudaSuccess)
    return fail(ctx, CCAKE_ERR_NOMEM, "pre-inverted table allocation");
  P.v = ctx->pre_v;
  // chunks of whole tiles, about 4M nodes at a time
  const int64_t per = std::max<int64_t>(1, ((int64_t)1 << 22) / tn), chunk = per * tn;
  double *in4 = nullptr, *tbqs = nullptr, *th16 = nullptr;
  int32_t* st = nullptr;
  if (cudaMalloc(&in4, chunk * 4 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&tbqs, chunk * 4 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&th16, chunk * 16 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&st, chunk * sizeof(int32_t)) != cudaSuccess) {
    cudaFree(in4); cudaFree(tbqs); cudaFree(th16); cudaFree(st);
    return fail(ctx, CCAKE_ERR_NOMEM, "pre-inverted table scratch");
  }
  if (!ctx->d_count && cudaMalloc(&ctx->d_count, sizeof(int32_t)) != cudaSuccess) return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
  CK(cudaMemsetAsync(ctx->d_count, 0, sizeof(int32_t), ctx->stream));
  int32_t* scratch = eos_scratch(ctx, chunk);
  for (int64_t t0 = 0; t0 < tiles; t0 += per) {
    const int64_t cnt = std::min(per, tiles - t0) * tn;
    launch_preinv_grid(P, t0, cnt, in4, tbqs, ctx->stream);
    launch_eos_batch(ctx->eos, 1, 0, cnt, in4, tbqs, th16, st, nullptr, scratch, ctx->stream);
    launch_preinv_pack(cnt, th16, st, ctx->pre_v + (size_t)t0 * tn * kPreVars, ctx->d_count, ctx->stream);
  }
  int32_t nfail = 0;
  CK(cudaMemcpyAsync(&nfail, ctx->d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(in4); cudaFree(tbqs); cudaFree(th16); cudaFree(st);
  if (!ctx->pre_dev && cudaMalloc(&ctx->pre_dev, sizeof(PreinvView)) != cudaSuccess)
    return fail(ctx, CCAKE_ERR_NOMEM, "allocation");
  CK(cudaMemcpy(ctx->pre_dev, &P, sizeof(PreinvView), cudaMemcpyHostToDevice));
  ctx->pre_host = P;
  ctx->pre_count = total;
  // the reference's generator aborts at a node without a solution
  if (nfail > 0) return fail(ctx, CCAKE_ERR_EOS, std::to_string(nfail) + " table nodes without an EoS solution");
  CK(cudaGetLastError());
  return CCAKE_OK;
}

ccake_status_t ccake_preinverted_use(ccake_ctx* ctx, int32_t on) {
  if (!ctx) return CCAKE_ERR_INVALID;
  if (on && !ctx->pre_count) return fail(ctx, CCAKE_ERR_STATE, "build the pre-inverted tables first");
  if (on && ctx->cfg.using_diffusion)
    return fail(ctx, CCAKE_ERR_INVALID, "the diffusion sector needs the Newton EoS (alpha derivatives)");
  const PreinvView* want = on ? ctx->pre_dev : nullptr;
  if (ctx->eos.pre != want) {
    ctx->eos.pre = want;
    drop_graph(ctx);   // the step graph holds the EoS description by value
  }
  return CCAKE_OK;
}

ccake_status_t ccake_preinverted_lookup(ccake_ctx* ctx, int64_t n, const double* sBSQ, double* out11) {
  if (!ctx || n < 0 || (n > 0 && (!sBSQ || !out11))) return CCAKE_ERR_INVALID;
  if (!ctx->pre_count) return fail(ctx, CCAKE_ERR_STATE, "build the pre-inverted tables first");
  if (n == 0) return CCAKE_OK;
  double *d_in = nullptr, *d_out = nullptr;
  CK(cudaMalloc(&d_in, n * 4 * sizeof(double)));
  CK(cudaMalloc(&d_out, n * kPreVars * sizeof(double)));
  CK(cudaMemcpyAsync(d_in, sBSQ, n * 4 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  launch_preinv_lookup(ctx->pre_dev, n, d_in, d_out, ctx->stream);
  CK(cudaMemcpyAsync(out11, d_out, n * kPreVars * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(d_in);
  cudaFree(d_out);
  CK(cudaGetLastError());
  return CCAKE_OK;
}

ccake_status_t ccake_preinverted_lookup_device(ccake_ctx* ctx, int64_t n, const double* d_sBSQ, double* d_out11,
                                               void* stream) {
  if (!ctx || n < 0) return CCAKE_ERR_INVALID;
  if (!ctx->pre_count) return fail(ctx, CCAKE_ERR_STATE, "build the pre-inverted tables first");
  launch_preinv_lookup(ctx->pre_dev, n, d_sBSQ, d_out11, static_cast<cudaStream_t>(stream));
  CK(cudaGetLastError());
  return CCAKE_OK;
}

ccake_status_t ccake_preinverted_copy(ccake_ctx* ctx, int64_t* count, double* host) {
  if (!ctx || !count) return CCAKE_ERR_INVALID;
  *count = ctx->pre_count;
  if (host && ctx->pre_count) {
    CK(cudaMemcpy(host, ctx->pre_v, (size_t)ctx->pre_count * kPreVars * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return CCAKE_OK;
}

ccake_status_t ccake_freeze_out_rows(ccake_ctx* ctx, int64_t* count, int32_t* width, double* rows) {
  if (!ctx || !count || !width) return CCAKE_ERR_INVALID;
  const int D = ctx->cfg.dim;
  const int W = D == 2 ? 40 : 45;
  *width = W + 2;
  *count = 0;
  if (!ctx->p.fo_count) return CCAKE_OK;
  int32_t k = 0;
  CK(cudaMemcpyAsync(&k, ctx->p.fo_count, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  k = std::min<int32_t>(k, (int32_t)ctx->n);
  *count = k;
  if (!rows || k == 0) return CCAKE_OK;
  std::vector<double> raw((size_t)k * kFoRow);
  CK(cudaMemcpy(raw.data(), ctx->p.fo_rows, raw.size() * sizeof(double), cudaMemcpyDeviceToHost));
  // the reference writes a step's rows in particle order (input order here)
  std::vector<int> ord((size_t)k);
  std::iota(ord.begin(), ord.end(), 0);
  auto key = [&](int r) {
    const double* q = raw.data() + (size_t)r * kFoRow;
    return std::make_pair((int64_t)q[0], (int64_t)ctx->perm[(size_t)q[1]]);
  };
  std::sort(ord.begin(), ord.end(), [&](int a, int b) { return key(a) < key(b); });
  for (int r = 0; r < k; r++) {
    const double* q = raw.data() + (size_t)ord[(size_t)r] * kFoRow;
    double* o = rows + (size_t)r * (W + 2);
    o[0] = q[0];
    o[1] = (double)ctx->perm[(size_t)q[1]];
    for (int c = 0; c < W; c++) o[2 + c] = q[2 + c];
  }
  return CCAKE_OK;
}

ccake_status_t ccake_write_freeze_out(ccake_ctx* ctx, const char* path, double B, double S, double Q) {
  if (!ctx || !path) return CCAKE_ERR_INVALID;
  int64_t k = 0;
  int32_t w = 0;
  ccake_status_t st = ccake_freeze_out_rows(ctx, &k, &w, nullptr);
  if (st) return st;
  std::vector<double> rows((size_t)k * w);
  if (k && (st = ccake_freeze_out_rows(ctx, &k, &w, rows.data()))) return st;
  std::ofstream out(path);
  if (!out.is_open()) return fail(ctx, CCAKE_ERR_INVALID, std::string("cannot write ") + path);
  // Output::print_freeze_out / flush_freeze_out (src/output.cpp:417-497):
  // the header "# B S Q", then the rows in the stream's default format
  out << "# " << B << " " << S << " " << Q << "\n";
  for (int64_t r = 0; r < k; r++) {
    const double* q = rows.data() + (size_t)r * w;
    for (int c = 2; c < w - 1; c++) out << q[c] << " ";
    out << q[w - 1] << "\n";
  }
  out << std::flush;
  if (!out.good()) return fail(ctx, CCAKE_ERR_INVALID, std::string("write failed: ") + path);
  return CCAKE_OK;
}

}  // extern "C"
