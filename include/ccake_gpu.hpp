// ccake_gpu.hpp -- header-only C++ shim over the C ABI (ccake_gpu.h) that keeps
// the reference's call surface, so call sites written against CCAKE's
// BSQHydro / SPHWorkstation / Evolver / EquationOfState drop in:
//
//   reference                                           this shim
//   BSQHydro<D,TEOM>::read_in_initial_conditions()      BSQHydro::read_in_initial_conditions(soa)
//   BSQHydro<D,TEOM>::initialize_hydrodynamics()        BSQHydro::initialize_hydrodynamics()
//   BSQHydro<D,TEOM>::run()                             BSQHydro::run()
//   SPHWorkstation::smooth_all_particle_fields(t2)      SPHWorkstation::smooth_all_particle_fields()
//   SPHWorkstation::update_all_particle_thermodynamics  SPHWorkstation::update_all_particle_thermodynamics()
//   SPHWorkstation::update_all_particle_viscosities     SPHWorkstation::update_all_particle_viscosities()
//   SPHWorkstation::smooth_all_particle_gradients(t2)   SPHWorkstation::smooth_all_particle_gradients()
//   SPHWorkstation::get_time_derivatives(dt)            SPHWorkstation::get_time_derivatives()
//   SPHWorkstation::advance_timestep(dt, rk_order)      SPHWorkstation::advance_timestep(dt, rk_order)
//   SPHWorkstation::continue_evolution()                SPHWorkstation::continue_evolution()
//   Evolver<D>::execute_timestep(dt, rk_order, f)       Evolver::execute_timestep(dt, rk_order)
//   EquationOfState::update_s / s_out                   EquationOfState::update_s / s_out
//   SystemState::conservation_energy/entropy/BSQ        SystemState::conservation()
//
// (reference: include/BSQHydro.h:43-68, include/sph_workstation.h:102-156,
//  include/evolver.h:107-108, include/eos.h:196-208, include/system_state.h:34-201)
// Errors become exceptions on this side only; the C boundary stays plain C.
#ifndef CCAKE_GPU_HPP
#define CCAKE_GPU_HPP

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ccake_gpu.h"

namespace ccake {
namespace gpu {

class Error : public std::runtime_error {
 public:
  Error(ccake_status_t s, const std::string& what) : std::runtime_error(what), status(s) {}
  ccake_status_t status;
};

inline void check(ccake_status_t s, const ccake_ctx* ctx, const char* what) {
  if (s != CCAKE_OK)
    throw Error(s, std::string(what) + ": " + ccake_status_string(s) + " (" + ccake_last_error(ctx) + ")");
}

// Device-resident particle system of one event.
class SystemState {
 public:
  explicit SystemState(const ccake_config& cfg) {
    check(ccake_ctx_create(&cfg, &ctx_), nullptr, "ccake_ctx_create");
  }
  ~SystemState() { if (ctx_) ccake_ctx_destroy(ctx_); }
  SystemState(const SystemState&) = delete;
  SystemState& operator=(const SystemState&) = delete;

  ccake_ctx* ctx() const { return ctx_; }
  double t() const { double v = 0; check(ccake_get_time(ctx_, &v), ctx_, "ccake_get_time"); return v; }
  int64_t n_particles() const { int64_t v = 0; check(ccake_get_count(ctx_, &v), ctx_, "ccake_get_count"); return v; }
  ccake_totals conservation() {
    ccake_totals t{};
    check(ccake_conservation(ctx_, &t), ctx_, "ccake_conservation");
    return t;
  }
  std::vector<double> field(const char* name) {
    std::vector<double> out((size_t)n_particles());
    check(ccake_copy_out(ctx_, name, out.data()), ctx_, "ccake_copy_out");
    return out;
  }
  void reset_neighbour_list() { check(ccake_build_neighbours(ctx_), ctx_, "ccake_build_neighbours"); }

 private:
  ccake_ctx* ctx_ = nullptr;
};

// Time integrator: explicit midpoint RK2 (the only order the configurations use).
class Evolver {
 public:
  explicit Evolver(SystemState& s) : s_(s) {}
  void execute_timestep(double /*dt: fixed in ccake_config*/, int rk_order) {
    if (rk_order != 2) throw Error(CCAKE_ERR_INVALID, "only rk_order 2 is implemented");
    check(ccake_step(s_.ctx(), 1), s_.ctx(), "ccake_step");
  }

 private:
  SystemState& s_;
};

class SPHWorkstation {
 public:
  SPHWorkstation(SystemState& s, double max_tau) : s_(s), evolver_(s), max_tau_(max_tau) {}
  void initialize() { check(ccake_initialize(s_.ctx()), s_.ctx(), "ccake_initialize"); }
  void smooth_all_particle_fields() { check(ccake_smooth_fields(s_.ctx()), s_.ctx(), "ccake_smooth_fields"); }
  void update_all_particle_thermodynamics() { check(ccake_update_thermo(s_.ctx()), s_.ctx(), "ccake_update_thermo"); }
  void update_all_particle_viscosities() {
    check(ccake_update_viscosities(s_.ctx()), s_.ctx(), "ccake_update_viscosities");
  }
  void smooth_all_particle_gradients() { check(ccake_smooth_gradients(s_.ctx()), s_.ctx(), "ccake_smooth_gradients"); }
  // all ten phases of one derivative evaluation at the current state
  void get_time_derivatives() {
    smooth_all_particle_fields();
    update_all_particle_thermodynamics();
    update_all_particle_viscosities();
    check(ccake_time_derivatives(s_.ctx()), s_.ctx(), "ccake_time_derivatives");
  }
  void advance_timestep(double dt, int rk_order) { evolver_.execute_timestep(dt, rk_order); }
  // the IC's initial currents (set_diffusion, src/sph_workstation.cpp:
  // 1441-1458): q holds 12 rows of n, q^mu of charge c at row 4c + mu
  void set_diffusion(const double* q) {
    check(ccake_set_initial_diffusion(s_.ctx(), q), s_.ctx(), "ccake_set_initial_diffusion");
  }
  // the IC's initial shear and bulk (calculate_extensive_shv, set_bulk_Pi,
  // src/sph_workstation.cpp:1350-1430); either may be null
  void set_initial_viscous(const double* trace, const double* pi) {
    check(ccake_set_initial_viscous(s_.ctx(), trace, pi), s_.ctx(), "ccake_set_initial_viscous");
  }
  // stop rule: every particle frozen out (with particlization) or t > max_tau
  // (src/sph_workstation.cpp:1992-2024)
  bool continue_evolution() const {
    int32_t keep = 0;
    check(ccake_continue_evolution(s_.ctx(), max_tau_, &keep), s_.ctx(), "ccake_continue_evolution");
    return keep != 0;
  }

 private:
  SystemState& s_;
  Evolver evolver_;
  double max_tau_;
};

// Batch form of the EoS inversion; the single-point calls of the reference
// map onto batches of one.
class EquationOfState {
 public:
  explicit EquationOfState(SystemState& s) : s_(s) {}
  // (s, B, S, Q) -> thermo; seed tbqs = (T, muB, muQ, muS) in/out
  bool update_s(double sin, double Bin, double Sin, double Qin, double tbqs[4], double th16[16]) {
    const double in[4] = {sin, Bin, Sin, Qin};
    int32_t st = -1;
    check(ccake_eos_invert_batch(s_.ctx(), 1, 1, in, tbqs, th16, &st, nullptr), s_.ctx(), "update_s");
    return st >= 0;
  }
  // (e, B, S, Q) -> s; solution_found as in the reference
  double s_out(double ein, double Bin, double Sin, double Qin, bool& solution_found) {
    const double in[4] = {ein, Bin, Sin, Qin};
    double tbqs[4] = {580.0 / 197.3269804, 0, 0, 0}, th[16];
    int32_t st = -1;
    check(ccake_eos_invert_batch(s_.ctx(), 0, 1, in, tbqs, th, &st, nullptr), s_.ctx(), "s_out");
    solution_found = st >= 0;
    return th[5];
  }

 private:
  SystemState& s_;
};

class BSQHydro {
 public:
  BSQHydro(const ccake_config& cfg, double max_tau)
      : sys_(cfg), ws_(sys_, max_tau), dt_(cfg.dt), diffusion_(cfg.using_diffusion != 0) {}
  void read_in_initial_conditions(const ccake_particles_soa& soa) {
    check(ccake_load_particles(sys_.ctx(), &soa), sys_.ctx(), "ccake_load_particles");
  }
  // BSQHydro::read_ccake (src/BSQHydro.cpp:206-425) with the settings it
  // consults, then the IC's initial currents (input_initial_diffusion) and,
  // when asked, its initial shear (input_initial_shear) and bulk
  // (bulk_from_trace)
  void read_ccake(const char* path, const ccake_ic_options& opt, bool initial_shear = false,
                  bool bulk_from_trace = false) {
    ccake_ic* ic = nullptr;
    check(ccake_ic_read_ccake(path, &opt, &ic), sys_.ctx(), "ccake_ic_read_ccake");
    std::unique_ptr<ccake_ic, void (*)(ccake_ic*)> keep(ic, ccake_ic_free);
    ccake_particles_soa soa{};
    check(ccake_ic_particles(ic, &soa), sys_.ctx(), "ccake_ic_particles");
    read_in_initial_conditions(soa);
    const int64_t n = soa.n;
    auto column = [&](const char* name, double* dst) {
      check(ccake_ic_column(ic, name, dst), sys_.ctx(), "ccake_ic_column");
    };
    // (without the sector the reference keeps the currents but never evolves them)
    if (opt.input_initial_diffusion && diffusion_) {
      static const char* qn[12] = {"qB0", "qB1", "qB2", "qB3", "qS0", "qS1", "qS2", "qS3", "qQ0", "qQ1", "qQ2", "qQ3"};
      std::vector<double> q((size_t)(12 * n));
      for (int r = 0; r < 12; r++) column(qn[r], q.data() + (size_t)r * n);
      ws_.set_diffusion(q.data());
    }
    if (initial_shear || bulk_from_trace) {
      static const char* pn[6] = {"pixx", "pixy", "pixeta", "piyy", "piyeta", "pietaeta"};
      std::vector<double> trace((size_t)n), pi((size_t)(6 * n));
      column("bulk", trace.data());
      for (int r = 0; r < 6; r++) column(pn[r], pi.data() + (size_t)r * n);
      ws_.set_initial_viscous(bulk_from_trace ? trace.data() : nullptr, initial_shear ? pi.data() : nullptr);
    }
  }
  void initialize_hydrodynamics() { ws_.initialize(); }
  // time loop of src/BSQHydro.cpp:745-814 (no output writers)
  void run(int max_steps = -1) {
    int k = 0;
    while (ws_.continue_evolution() && (max_steps < 0 || k < max_steps)) {
      ws_.advance_timestep(dt_, 2);
      k++;
    }
  }
  SystemState& system() { return sys_; }
  SPHWorkstation& workstation() { return ws_; }

 private:
  SystemState sys_;
  SPHWorkstation ws_;
  double dt_;
  bool diffusion_;
};

}  // namespace gpu
}  // namespace ccake

#endif  // CCAKE_GPU_HPP
