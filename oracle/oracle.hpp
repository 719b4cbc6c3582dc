// CPU FP64 oracle for the CCAKE per-timestep SPH hot path.
//
// TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path is
// compared against; it is never linked into, loaded by, or called from the
// product library. Only the tests, the smoke check and the CPU-baseline leg of
// the benchmark load it.
//
// It restates, in plain C++17 (+OpenMP over particles), the algorithms of the
// reference (the-nuclear-confectionery/CCAKE). Each routine cites the reference
// file:line it follows. The reference itself cannot be built here (Kokkos,
// Cabana, GSL, HDF5 and yaml-cpp are absent), so parity is pinned against the
// reference's own unit-test golden values (kernel, smoothing, gradient, RK2,
// multilinear interpolation) and against the analytic ideal Gubser flow.
//
// Units follow the reference: T, mu in fm^-1; e, p in fm^-4; s, rho in fm^-3.
#pragma once
#include <cstdint>
#include <vector>
#include <string>

namespace orc {

constexpr double kHbarcGeVfm = 0.1973269804;   // include/constants.h:16
constexpr double kHbarcMeVfm = 197.3269804;    // include/constants.h:17
constexpr double kTiny = 1e-25;                // include/eos_header.h:16
constexpr double kTbqsInf = 1e10;              // include/eos_header.h:17

enum EosKind : int32_t { kConformal = 0, kConformalDiagonal = 1, kTable = 2 };
enum ShearRelax : int32_t { kTauPiDefault = 0, kTauPiGubser = 1, kTauPiMinval = 2 };
enum ZetaMode : int32_t { kZetaDefault = 0, kZetaConstant = 1, kZetaCs2 = 2, kZetaPeaked = 3 };

// Run configuration (the subset of the reference Settings the hot path reads).
// Layout is mirrored by a ctypes Structure in the tests.
struct Config {
  int32_t dim;               // 2 or 3 (spatial dimensions)
  int32_t coord;             // 0 = Milne ("hyperbolic", EoM_default); 1 = Cartesian
  int32_t eos_kind;          // EosKind
  int32_t using_shear;       // settings.h:263-270 (eta/s > 1e-10)
  int32_t using_vorticity;
  int32_t shear_relax_mode;  // ShearRelax
  int32_t zeta_mode;         // ZetaMode
  int32_t factorized_kernel; // D=3 W2D(r_perp)*W1D(deta) kernel
  int32_t input_as_entropy;
  int32_t modulate_zeta_with_tanh;
  int32_t thermo_mode;       // 0 = reference Schur-complement chain, 1 = exact Hessian inverse
  int32_t pad1;
  double hT, hEta, t0, dt;
  double eos_c, eos_T0, eos_muB0, eos_muQ0, eos_muS0;
  double eta_over_s, zeta_over_s, zeta_cs2_A, zeta_cs2_p;
  double zeta_peak_T, zeta_peak_width;   // peaked zeta/s mode (config 4)
  double xmin, ymin, etamin;              // lower corner of the IC grid
  double freeze_out_T;                    // fm^-1
  int32_t particlization;                 // freeze-out status machine after every step
  int32_t surface;                        // with particlization: the freeze-out hypersurface
  // diffusion sector (include/settings.h; src/transport_coefficients.cpp:82-115)
  int32_t using_diffusion;                // diffusionMode != "disabled"
  int32_t diffusion_mode;                 // 0 constant_over_T2, 2 kappaB_coth
  int32_t diffusion_relax_mode;           // 0 tau_q = 0.2/T, 1 tau_q = C_B/T (kappaB_coth)
  int32_t diffusion_regulator;            // regulate_diffusion enabled
  int32_t critical_scaling_diffusion;     // Gaussian suppression of kappa near (T_c, muB_c)
  int32_t pad2;
  double kappa_over_T2[9];                // constant_kappa_over_T2 (row-major B, S, Q)
  double C_B;
  double reg_chi0, reg_e0, reg_xi0, reg_rq_max;   // regulator; e0, xi0 in GeV/fm^3
  double crit_T, crit_muB, crit_wT, crit_wmuB;    // critical point and widths, MeV
  // second-order coefficients (src/transport_coefficients.cpp:117-278):
  // 0 the *_DEFAULT function, 1 israel-stewart (the two deltas), 2 disabled
  int32_t delta_pipi_mode, tau_pipi_mode, lambda_piPi_mode, phi6_mode, phi7_mode;
  int32_t delta_PiPi_mode, lambda_Pipi_mode, phi1_mode, phi3_mode;
  int32_t restrict_mu_T_ratios;           // src/eos.cpp:781-786 (settings, off by default)
};

// Freeze-out snapshot of one step (FreezeOut::freeze_array,
// include/freeze_out.h:20-80): per particle r[3] u[3] gradP[3] gradE[3]
// s e rhoB rhoS rhoQ T muB muS muQ theta bulk sigma_lab pi^{mu nu}[10]
// pi^{33} shv_nabla_u w cs2 q^mu[3][4].
enum SnapField : int { SF_R = 0, SF_U = 3, SF_GP = 6, SF_GE = 9, SF_S = 12, SF_E, SF_RB, SF_RS, SF_RQ, SF_T, SF_MUB,
                       SF_MUS, SF_MUQ, SF_THETA, SF_BULK, SF_SLAB, SF_SHV, SF_SHV33 = SF_SHV + 10, SF_SNU, SF_W, SF_CS2,
                       SF_Q, NSF = SF_Q + 12 };

// Per-particle state, struct of arrays.
struct System {
  Config cfg;
  int n = 0;
  double t = 0;
  // evolved state
  std::vector<double> r[3], u[3];
  std::vector<double> ext[4];       // extensive s, rhoB, rhoS, rhoQ (per sph mass)
  std::vector<double> mass[4];      // sph_mass (1 after init)
  std::vector<double> ext_bulk;
  std::vector<double> ext_shv[6];   // (0,0),(0,1),(0,2),(1,1),(1,2) of the 2x3 block; [5] unused
  std::vector<double> Ez;           // contribution_to_total_Ez
  std::vector<int32_t> freeze, btrack;
  // freeze-out status machine: energy snapshot of the previous step, steps
  // seen, freeze-out energy density e(T_FO, 0, 0, 0)
  std::vector<double> frz1_e;
  int frzc = 0;
  double efcheck = 0;
  // hypersurface (cfg.surface): snapshots frz1, frz2, fback, fback2, fback3,
  // fback4 (NSF x n each), the times of the last two steps, the step count,
  // and the rows of freeze_out.dat in the order they are written (each with
  // its step and particle index in front)
  std::vector<double> snap[6];
  double taup = 0, taupp = 0;
  int nstep = 0;
  std::vector<std::vector<double>> fo_rows;
  // input
  std::vector<double> in_e, in_s, in_rho[3], in_bulk;
  std::vector<double> in_shv[6];    // pi^{xx},xy,xeta,yy,yeta,etaeta (fm^-4..)
  // use the input bulk as the trace of bulk_from_trace / the input pi^{ij}
  // as with input_initial_shear (set_bulk_Pi, calculate_extensive_shv)
  int use_in_bulk = 0, use_in_shv = 0;
  // derived
  std::vector<double> gamma, v[3], sigma_lab, sigma, smoothed[4];
  // thermo: T, muB, muS, muQ, p, s, rhoB, rhoS, rhoQ, e, w, cs2, dwds, dwdB, dwdS, dwdQ
  std::vector<double> th[16];
  std::vector<int32_t> eos_id;      // index into the EoS chain of the last solution
  std::vector<int32_t> eos_status;  // 0 ok, >0 number of failed attempts, <0 no solution
  std::vector<double> bulk;
  std::vector<double> shv[16];      // 4x4 pi^{mu nu}
  // transport
  std::vector<double> eta_pi, tau_pi, zeta_Pi, tau_Pi, delta_PiPi, delta_pipi,
      lambda_piPi, lambda_Pipi, phi1, phi3, phi6, phi7, tau_pipi;
  // gradients
  std::vector<double> gradP[3], gradE[3], gradBulk[3], gradshear[3], divshear[3], gradV[9];
  // time derivatives
  std::vector<double> du_dt[3], d_ext[4], d_ext_bulk, d_ext_shv[6], dEz, theta, shv_nabla_u;
  // src/eom_default.cpp:1831-1985 (with shear): sigma^{11,12,13,22,23},
  // shear / bulk Knudsen and inverse Reynolds numbers
  std::vector<double> sigma_t[5], kn_shear, kn_bulk, ire_shear, ire_bulk;
  // diffusion sector: extensive q (charge c = B, S, Q; direction i) at 3c + i,
  // q^mu of the last reset_pi_tensor at 4c + mu, the initial q^mu, the twelve
  // alpha derivatives (eos_alpha_derivs order), tau_q and kappa_q (3c + d),
  // grad alpha (direction i, charge c at 3i + c), div q_a, v.grad q^0_a,
  // d(ext q)/dt, and the diffusion Knudsen / inverse Reynolds numbers
  std::vector<double> ext_q[9], q[12], in_q[12], dalpha[12], tau_q[9], kappa_q[9];
  std::vector<double> grad_alpha[9], div_qa[3], grad_qa[3], d_ext_q[9], kn_diff[3], ire_diff[3];
  // evolver cache
  std::vector<double> r0[3], u0[3], ext0[4], ext_bulk0, ext_shv0[6], Ez0, ext_q0[9];
  // table EoS (optional)
  struct Table* table = nullptr;
};

enum ThermoIdx { kT = 0, kMuB, kMuS, kMuQ, kP, kS, kRhoB, kRhoS, kRhoQ, kE, kW, kCs2,
                 kDwds, kDwdB, kDwdS, kDwdQ };

// --- SPH kernel (src/kernel.cpp) ---------------------------------------------
double kernel_W(int D, double r, double h);
void kernel_gradW(int D, const double* rel, double r, double h, double* grad);
double kernel_W_factorized(const double* r1, const double* r2, double hT, double hEta);
void kernel_gradW_factorized(const double* rel, double hT, double hEta, double* grad);

// --- neighbours --------------------------------------------------------------
// Full neighbour list, CSR, predicate dx^2+dy^2+dz^2 <= (2h)^2, self excluded.
void neighbours_bruteforce(const System& s, std::vector<int32_t>& off, std::vector<int32_t>& idx);
void neighbours_celllist(const System& s, std::vector<int32_t>& off, std::vector<int32_t>& idx);

// --- the step pieces ----------------------------------------------------------
struct NbrList { std::vector<int32_t> off, idx; };
void build_neighbours(System& s, NbrList& nl);
void update_velocity(System& s);
void smooth_fields(System& s, const NbrList& nl);
void calculate_initial_sigma(System& s, const NbrList& nl, double t);
int update_thermodynamics(System& s);
void reset_pi_tensor(System& s);
void regulate_diffusion(System& s);
void update_viscosities(System& s);
void smooth_gradients(System& s, const NbrList& nl);
void evaluate_time_derivatives(System& s);
void get_time_derivatives(System& s, NbrList& nl);
void rk2_step(System& s, NbrList& nl);
void freeze_out_status(System& s);
// returns the number of particles without an EoS solution (the reference throws)
int initialize(System& s, NbrList& nl);

struct Totals { double S, B, Sq, Q, E, Ez; };
Totals conservation(const System& s);

// --- equation of state ---------------------------------------------------------
struct Table;
// 17-field thermo at (T, muB, muQ, muS): p s B S Q e cs2 chiBB chiQQ chiSS chiBQ
// chiBS chiQS chiTB chiTQ chiTS chiTT (include/eos_base.h get_full_thermo order)
void eos_full_thermo(const Config& c, const Table* tab, int model, const double tbqs[4], double out[17]);
// Invert (e or s, B, S, Q) -> (T, muB, muQ, muS) with the reference's seed chain.
// Returns the chain index of the model used, or -1 when no solution was found.
int eos_invert(const Config& c, const Table* tab, int mode_entropy, const double target[4],
               int start_model, double tbqs_inout[4], int* iterations);
// Derived thermodynamics after a solution (include/eos.h:121-175 set_thermo subset).
void eos_set_thermo(const Config& c, const Table* tab, int model, const double tbqs[4], double th16[16]);
// dalpha_a/ds (out[a]) and dalpha_a/drho_b (out[3 + 3a + b]), a, b = B, S, Q
// (src/eos.cpp:337-493).
void eos_alpha_derivs(const Config& c, const Table* tab, int model, const double tbqs[4], double out12[12]);
int eos_chain_length(const Config& c);

}  // namespace orc
