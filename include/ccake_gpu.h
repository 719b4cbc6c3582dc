/*
 * ccake_gpu.h -- C ABI of the GB300-native CCAKE SPH hot path (libccake_gpu.so).
 *
 * One context holds one hydro event resident in the device memory of the
 * current CUDA device: particle state, neighbour cell lists, EoS seeds.
 * Plain C, no exceptions cross this boundary, every call returns a
 * ccake_status_t. A context is used by one host thread at a time.
 *
 * The reference (the-nuclear-confectionery/CCAKE) exposes this path only as
 * C++ templates; each entry below names the reference member function it
 * replaces (paths are within the reference project).
 *
 * Units are the reference's internal units: positions fm (eta dimensionless),
 * energy density fm^-4, entropy and charge densities fm^-3, T and mu fm^-1.
 */
#ifndef CCAKE_GPU_H
#define CCAKE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ccake_status {
  CCAKE_OK = 0,
  CCAKE_ERR_INVALID = 1,        /* bad argument or unsupported configuration */
  CCAKE_ERR_CUDA = 2,           /* a CUDA runtime call failed */
  CCAKE_ERR_EOS = 3,            /* the EoS root finder found no solution (src/eos.cpp:790-801) */
  CCAKE_ERR_NEG_ENTROPY = 4,    /* negative extensive entropy (src/evolver.cpp:437-450) */
  CCAKE_ERR_CAPACITY = 5,       /* an output buffer is too small */
  CCAKE_ERR_STATE = 6,          /* call out of order (e.g. step before initialize) */
  CCAKE_ERR_NOMEM = 7,          /* device allocation failed */
  CCAKE_ERR_NONFINITE = 8       /* a non-finite value appeared in the evolved state */
} ccake_status_t;

/* Run configuration: the subset of the reference Settings
 * (include/settings.h:23-287) that the hot path reads. */
typedef struct ccake_config {
  int32_t dim;               /* spatial dimensions: 2 or 3 */
  int32_t coord;             /* 0 Milne ("hyperbolic", EoM_default), 1 Cartesian (EoM_cartesian) */
  int32_t eos_kind;          /* 0 conformal, 1 conformal_diagonal, 2 table */
  int32_t using_shear;       /* include/settings.h:263-270 */
  int32_t using_vorticity;
  int32_t shear_relax_mode;  /* 0 default max(5 eta/w, 0.005), 1 "Gubser" 5 eta/w, 2 minVal */
  int32_t zeta_mode;         /* 0 default 0.005 w/T, 1 constant, 2 cs2-dependent, 3 peaked */
  int32_t factorized_kernel; /* D=3 W2D(r_perp, hT)*W1D(deta, hEta) (src/kernel.cpp:130-170); FP64
                                form (precision 0) only, CCAKE_ERR_INVALID otherwise */
  int32_t input_as_entropy;  /* input column is s instead of e */
  int32_t modulate_zeta_with_tanh;
  int32_t thermo_mode;       /* 0 reference dw/ds chain (src/eos.cpp:276-344), 1 exact Hessian inverse */
  int32_t precision;         /* 0 FP64 throughout; 1 FP32-compensated pair sums */
  double hT, hEta, t0, dt;
  double eos_c, eos_T0, eos_muB0, eos_muQ0, eos_muS0;
  double eta_over_s, zeta_over_s, zeta_cs2_A, zeta_cs2_p;
  double zeta_peak_T, zeta_peak_width;
  double xmin, ymin, etamin;  /* lower corner of the IC grid (IC header, src/BSQHydro.cpp:241-249) */
  double freeze_out_T;        /* fm^-1 */
  double skin_frac;           /* candidate-list skin as a fraction of 2h (0: 0.1); the
                                 list is rebuilt every R steps, R = floor(skin / (2 dt vmax)),
                                 vmax = max(1, 1/tau) in Milne (x, y, eta_s) coordinates */
  int32_t particlization;     /* run the freeze-out status machine after every step
                                 (include/settings.h particlization_enabled) */
  int32_t surface;            /* with particlization: interpolate the freeze-out
                                 hypersurface (FreezeOut::bsqsvinterpolate), rows
                                 of freeze_out.dat, ccake_freeze_out_rows */
  /* diffusion sector (include/settings.h diffusionMode != "disabled";
   * src/eom_default.cpp:1415-1817, src/eom_cartesian.cpp:1327-1722): FP64
   * form (precision 0), Newton EoS (no pre-inverted tables) */
  int32_t using_diffusion;
  int32_t diffusion_mode;       /* 0 constant_over_T2 (kappa = kappa_over_T2 T^2), 2 kappaB_coth */
  int32_t diffusion_relax_mode; /* 0 tau_q = 0.2/T; 1 tau_q = C_B/T (kappaB_coth) */
  int32_t diffusion_regulator;  /* regulate_diffusion (src/sph_workstation.cpp:132-218) */
  int32_t critical_scaling_diffusion;  /* Gaussian suppression of kappa near the critical point */
  int32_t pad2;
  double kappa_over_T2[9];      /* constant_kappa_over_T2, row-major over (B, S, Q) */
  double C_B;
  double reg_chi0, reg_e0, reg_xi0, reg_rq_max;   /* regulator; e0, xi0 in GeV/fm^3 */
  double crit_T, crit_muB, crit_wT, crit_wmuB;    /* critical point and widths, MeV */
  /* second-order transport coefficients, the reference's *_mode settings
   * (include/settings.h:172-190, src/transport_coefficients.cpp:117-278 and
   * :704-912): CCAKE_COEF_DEFAULT takes the reference's *_DEFAULT function
   * (delta_pipi 4/3 tau_pi, tau_pipi 10/7 tau_pi, lambda_piPi 6/5 tau_pi,
   * phi6 0, phi7 9/(70 p), delta_PiPi 2/3 tau_Pi, lambda_Pipi
   * 8/5 (1/3 - cs2) tau_Pi, phi1 0, phi3 0); CCAKE_COEF_IS ("israel-stewart",
   * delta_pipi and delta_PiPi only) takes tau_pi / tau_Pi; CCAKE_COEF_DISABLED
   * takes 0. A zeroed config is all DEFAULT; the reference's own setting
   * defaults (include/defaults.h:48-52) are IS for delta_pipi and DISABLED for
   * tau_pipi, lambda_piPi, phi6 and phi7. */
  int32_t delta_pipi_mode, tau_pipi_mode, lambda_piPi_mode, phi6_mode, phi7_mode;
  int32_t delta_PiPi_mode, lambda_Pipi_mode, phi1_mode, phi3_mode;
  int32_t pad3;
  /* seed of the initial e -> (T, mu) inversion (ccake_initialize; the
   * reference's s_out, src/sph_workstation.cpp:1791-1851):
   * CCAKE_SEED_REFERENCE (0) the reference's 580 MeV forced seed,
   * CCAKE_SEED_LEARNED (2) the trained seed network (ccake_mlp_train /
   * ccake_mlp_set_params; table EoS only), then the reference's seeds. The
   * step's entropy-mode inversions always start from each particle's
   * previous (T, mu), as the reference's do. */
  int32_t seed_mode;
  /* restrict_mu_T_ratios (src/eos.cpp:781-786; off by default): a table
   * solution with max(|muB|, |muS|, |muQ|) > 3.5 T is refused and the row
   * goes down the EoS chain */
  int32_t restrict_mu_T_ratios;
} ccake_config;

enum { CCAKE_COEF_DEFAULT = 0, CCAKE_COEF_IS = 1, CCAKE_COEF_DISABLED = 2 };

/* Host struct-of-arrays particle input, the columns of the reference's
 * "ccake" IC format (src/BSQHydro.cpp:206-330) already in internal units.
 * eta/ueta may be NULL for dim = 2; rhoB/rhoS/rhoQ may be NULL (zero). */
typedef struct ccake_particles_soa {
  int64_t n;
  const double *x, *y, *eta;
  const double *e_or_s;
  const double *rhoB, *rhoS, *rhoQ;
  const double *ux, *uy, *ueta;
} ccake_particles_soa;

/* ---- on-disk formats --------------------------------------------------
 * The "ccake" initial-condition text format, src/BSQHydro.cpp:206-425
 * (BSQHydro::read_ccake; the IC_file setting): a header line
 * "#<n> dx dy deta <n> xmin ymin etamin", then one cell a line,
 *   x y eta e|s rhoB rhoS rhoQ ux uy ueta bulk pixx pixy pixeta piyy piyeta pietaeta
 * plus qB^0..3 qS^0..3 qQ^0..3 with initial diffusion. Blank and '#' lines
 * after the header are skipped. */
typedef struct ccake_ic ccake_ic;
typedef struct ccake_ic_options {
  int32_t input_as_entropy;         /* column 4 is s (1/fm^3), else e (GeV/fm^3) */
  int32_t input_initial_diffusion;  /* 29 columns instead of 17 */
  int32_t baryon, strange, electric;/* charges enabled (settings *_charge_enabled);
                                       disabled ones read as zero */
  int32_t reserved;
  double e_cutoff;                  /* GeV/fm^3: a cell is kept when e (with entropy
                                       input, the ideal pion gas e(s)) is above it */
} ccake_ic_options;

/* Reads and converts the file (e, bulk and pi^{ij} divided by hbar c);
 * CCAKE_ERR_INVALID for a missing file, a header without '#' and eight
 * numbers, or a data line with fewer numbers than the format has. */
ccake_status_t ccake_ic_read_ccake(const char* path, const ccake_ic_options* opt, ccake_ic** out);
/* Number of cells kept; grid6 (may be NULL) = dx, dy, deta, xmin, ymin, etamin. */
ccake_status_t ccake_ic_info(const ccake_ic* ic, int64_t* n, double* grid6);
/* One column by name (x y eta e s rhoB rhoS rhoQ ux uy ueta bulk pixx pixy
 * pixeta piyy piyeta pietaeta qB0..qB3 qS0..qS3 qQ0..qQ3) into dst[n]. */
ccake_status_t ccake_ic_column(const ccake_ic* ic, const char* name, double* dst);
/* Points soa at the cells (valid until ccake_ic_free), for ccake_load_particles. */
ccake_status_t ccake_ic_particles(const ccake_ic* ic, ccake_particles_soa* soa);
void ccake_ic_free(ccake_ic* ic);

/* Conserved totals, src/system_state.cpp:738-885. */
typedef struct ccake_totals {
  double S, B, Sq, Q, E, Ez;
} ccake_totals;

typedef struct ccake_ctx ccake_ctx;

/* Human-readable name of a status code. */
const char* ccake_status_string(ccake_status_t s);

/* Last error message of a context (never NULL). */
const char* ccake_last_error(const ccake_ctx* ctx);

/* Creates a context on the current CUDA device.
 * Replaces BSQHydro<D,TEOM>::BSQHydro and SPHWorkstation::initialize
 * (include/BSQHydro.h:48-54, src/sph_workstation.cpp:37-84). */
ccake_status_t ccake_ctx_create(const ccake_config* cfg, ccake_ctx** out);
ccake_status_t ccake_ctx_destroy(ccake_ctx* ctx);

/* Copies host particles into device memory, reordered by neighbour cell.
 * Replaces SPHWorkstation::process_initial_conditions and
 * SystemState::allocate_cabana_particles (src/sph_workstation.cpp:1228-1340,
 * src/system_state.cpp:57-326). */
ccake_status_t ccake_load_particles(ccake_ctx* ctx, const ccake_particles_soa* host);

/* Initial viscous state of the loaded particles (src/sph_workstation.cpp:
 * 1350-1430; the IC file's bulk and pi columns, internal units, the caller's
 * particle order). trace (n doubles, may be NULL): the bulk column as the
 * trace input of bulk_from_trace, ext Pi = (trace - p) / sigma
 * (SPHWorkstation::set_bulk_Pi). pi (6 rows of n, may be NULL): pi^{xx},
 * pi^{xy}, pi^{x eta}, pi^{yy}, pi^{y eta}, pi^{eta eta} as with
 * input_initial_shear, ext pi^{ij} = pi^{ij} / sigma for the five stored
 * entries (calculate_extensive_shv; pi^{eta eta} follows from
 * tracelessness). sigma is that of the initial smoothing. Without this call
 * both start at zero. Call between ccake_load_particles and
 * ccake_initialize. */
ccake_status_t ccake_set_initial_viscous(ccake_ctx* ctx, const double* trace, const double* pi);

/* Initial diffusion currents of the loaded particles (the reference's
 * input_initial_diffusion columns, src/BSQHydro.cpp:345-375): q has 12 rows
 * of n doubles in the caller's particle order, row 4c + mu = q^mu of charge
 * c (B, S, Q). Only the spatial q^i are used: ccake_initialize sets the
 * extensive current q^i / sigma (SPHWorkstation::set_diffusion,
 * src/sph_workstation.cpp:1441-1458) and q^0 follows from orthogonality to u.
 * Needs using_diffusion; call between ccake_load_particles and
 * ccake_initialize (without it the currents start at zero). */
ccake_status_t ccake_set_initial_diffusion(ccake_ctx* ctx, const double* q);

/* e -> s inversion, initial sigma, extensive densities and initial smoothing.
 * Replaces BSQHydro::initialize_hydrodynamics (src/BSQHydro.cpp:568-646). */
ccake_status_t ccake_initialize(ccake_ctx* ctx);

/* Step building blocks, each runnable alone on the current state for parity
 * checks; together they are one derivative evaluation
 * (SPHWorkstation::get_time_derivatives, src/sph_workstation.cpp:1509-1612). */
/* SystemState::reset_neighbour_list (src/system_state.cpp:650-719) */
ccake_status_t ccake_build_neighbours(ccake_ctx* ctx);
/* SPHWorkstation::smooth_all_particle_fields (src/sph_workstation.cpp:494-578),
 * preceded by TEOM::update_velocity (src/eom_default.cpp:17-38) */
ccake_status_t ccake_smooth_fields(ccake_ctx* ctx);
/* SPHWorkstation::update_all_particle_thermodynamics (src/sph_workstation.cpp:1713-1772)
 * followed by TEOM::reset_pi_tensor (src/eom_default.cpp:56-172) */
ccake_status_t ccake_update_thermo(ccake_ctx* ctx);
/* SPHWorkstation::update_all_particle_viscosities (src/sph_workstation.cpp:1622-1699) */
ccake_status_t ccake_update_viscosities(ccake_ctx* ctx);
/* SPHWorkstation::smooth_all_particle_gradients (src/sph_workstation.cpp:796-986) */
ccake_status_t ccake_smooth_gradients(ccake_ctx* ctx);
/* TEOM::evaluate_time_derivatives (src/eom_default.cpp:211-869) */
ccake_status_t ccake_time_derivatives(ccake_ctx* ctx);

/* Advances n_steps midpoint-RK2 steps with the fused device path (graph
 * captured). Replaces SPHWorkstation::advance_timestep ->
 * Evolver::execute_timestep (src/sph_workstation.cpp:2042-2073,
 * src/evolver.cpp:97-117, :344-517). */
ccake_status_t ccake_step(ccake_ctx* ctx, int32_t n_steps);

/* Stop rule: *keep_going = 0 once every particle is frozen out (freeze >= 4,
 * with particlization) or tau > max_tau. Replaces
 * SPHWorkstation::continue_evolution (src/sph_workstation.cpp:1992-2024). */
ccake_status_t ccake_continue_evolution(ccake_ctx* ctx, double max_tau, int32_t* keep_going);

/* ccake_step with its device time: CUDA events recorded on the context's
 * stream around the n_steps graph launches (milliseconds in *device_ms).
 * Measurement entry point; no reference counterpart. */
ccake_status_t ccake_step_timed(ccake_ctx* ctx, int32_t n_steps, float* device_ms);

/* Kernels launched by ccake_step / ccake_step_timed on this context so far:
 * the kernel nodes of the step graph and of the candidate-list build graph,
 * times their launches. Measurement entry point; no reference counterpart. */
ccake_status_t ccake_kernel_launches(const ccake_ctx* ctx, int64_t* launches);

/* Runs n_steps RK2 steps kernel by kernel (no graph) with CUDA events between
 * the launches and returns the average device time per launch, in ms, of:
 * ms[0] the four cell-list kernels together, ms[1] the smoothing+EoS pass,
 * ms[2] the gradient+EoM+RK2 pass. Measurement entry point; no reference
 * counterpart (the reference's phase timers are src/sph_workstation.cpp:1543-1583). */
ccake_status_t ccake_profile_phases(ccake_ctx* ctx, int32_t n_steps, double* ms3);

/* Bytes of device memory the context holds. */
ccake_status_t ccake_device_bytes(const ccake_ctx* ctx, int64_t* bytes);

/* Current time tau (fm/c) and particle count. */
ccake_status_t ccake_get_time(const ccake_ctx* ctx, double* t);
ccake_status_t ccake_get_count(const ccake_ctx* ctx, int64_t* n);

/* Conservation sums (src/system_state.cpp:738-885). */
ccake_status_t ccake_conservation(ccake_ctx* ctx, ccake_totals* out);

/* Copies one named per-particle field, in the caller's input order, to host
 * memory (n doubles). Names: x y eta u0 u1 u2 v0.. ext_s ext_B ext_S ext_Q
 * ext_bulk ext_shv0..4 Ez gamma sigma_lab sigma T muB muS muQ p s rhoB rhoS
 * rhoQ e w cs2 dwds dwdB dwdS dwdQ bulk shvIJ (I,J in 0..3) gradP0.. gradE0..
 * gradBulk0.. gradshear0.. divshear0.. gradV0..8 du_dt0.. d_ext_s d_ext_bulk
 * d_ext_shv0..4 dEz eta_pi tau_pi zeta_Pi tau_Pi. */
ccake_status_t ccake_copy_out(ccake_ctx* ctx, const char* field, double* host_out);
/* Integer fields: btrack eos_id eos_iters freeze. */
ccake_status_t ccake_copy_out_int(ccake_ctx* ctx, const char* field, int32_t* host_out);

/* Diagnostics of the last derivative evaluation (the second substep of the
 * last RK2 step) into the copy-out fields theta, sigma_tensor0..4
 * (sigma^{11,12,13,22,23}), shear_knudsen, bulk_knudsen,
 * inverse_reynolds_shear, inverse_reynolds_bulk and the transport
 * coefficients eta_pi, zeta_Pi, tau_Pi, tau_pi: theta and sigma^{ij} of
 * src/eom_default.cpp:774-807, the numbers of compute_hydro_numbers
 * (:1831-1985, computed with shear only). All zero before the first step. */
ccake_status_t ccake_hydro_numbers(ccake_ctx* ctx);

/* The reference's text output system_state_<n>.dat (src/output.cpp:102-181,
 * Output::print_system_state_to_txt) at path: the time, then one row a
 * particle in input order: index, t, position (3), p, T, muB, muS, muQ, e
 * (GeV units), rhoB, rhoS, rhoQ, s, eta_pi, zeta_Pi, tau_Pi, tau_pi, theta,
 * inverse Reynolds and Knudsen numbers (shear, bulk), pi^{00,11,22,01,02,12,
 * 13,23,33}, u (3), gamma, freeze status, EoS name, causality (0: not
 * checked), the diffusion Knudsen numbers (B, S, Q) and inverse Reynolds
 * numbers (B, S, Q) (0 without the diffusion sector). */
ccake_status_t ccake_write_system_state(ccake_ctx* ctx, const char* path);

/* Freeze-out hypersurface rows (cfg.particlization and cfg.surface), one
 * for each particle interpolated so far (FreezeOut::bsqsvinterpolate,
 * include/freeze_out.h:617-936): step, particle (input index), then the
 * fields of a freeze_out.dat row (src/output.cpp:433-475; 40 in 2-D, 45 in
 * 3-D), ordered by step, then particle. width = fields + 2; rows may be NULL
 * (count and width only). */
ccake_status_t ccake_freeze_out_rows(ccake_ctx* ctx, int64_t* count, int32_t* width, double* rows);
/* freeze_out.dat (Output::flush_freeze_out): "# B S Q", then the rows. */
ccake_status_t ccake_write_freeze_out(ccake_ctx* ctx, const char* path, double B, double S, double Q);

/* ---- pre-inverted (s, rhoB, rhoS, rhoQ) -> thermodynamics tables ---------
 * The reference's EoS_Interpolator (include/eos_interpolator.h:33-165,
 * src/eos_interpolator.cpp:531-739) and its generator
 * (utilities/generate_eos_table.cpp): one tile a decade [10^e, 10^(e+1)) of
 * each density, N^4 nodes a tile at min + i * 10^(e+1)/N, 11 values a node:
 * T, muB, muQ, muS, e, p, cs2, dw/ds, dw/drhoB, dw/drhoQ, dw/drhoS. */
typedef struct ccake_preinv_config {
  int32_t exp_lo[4];   /* first decade exponent of s, rhoB, rhoS, rhoQ (generator: -3 -3 -3 -3) */
  int32_t exp_hi[4];   /* last decade exponent (generator: 1 0 0 0); at most 8 decades an axis */
  int32_t nodes;       /* nodes a tile axis, 2..64 (generator: 20) */
  int32_t reserved;
} ccake_preinv_config;

/* Generates the tables on the device from the context's EoS (every node by
 * the entropy-mode inversion from T = 750/197 fm^-1, mu = 0);
 * CCAKE_ERR_EOS if a node has no solution (the generator aborts there). */
ccake_status_t ccake_preinverted_build(ccake_ctx* ctx, const ccake_preinv_config* cfg);
/* on != 0: the step takes its thermodynamics from the tables
 * (fill_thermodynamics) instead of the inversion. */
ccake_status_t ccake_preinverted_use(ccake_ctx* ctx, int32_t on);
/* Lookups of n rows (s, rhoB, rhoS, rhoQ) into out11[n][11], host arrays. */
ccake_status_t ccake_preinverted_lookup(ccake_ctx* ctx, int64_t n, const double* sBSQ, double* out11);
/* The same on device arrays, enqueued on stream (a cudaStream_t; NULL is
 * the default stream), as ccake_eos_invert_device. */
ccake_status_t ccake_preinverted_lookup_device(ccake_ctx* ctx, int64_t n, const double* d_sBSQ, double* d_out11,
                                               void* stream);
/* count = number of nodes; host (may be NULL) receives count x 11 values,
 * tiles in order (rhoQ decade fastest), nodes row-major (rhoQ fastest). */
ccake_status_t ccake_preinverted_copy(ccake_ctx* ctx, int64_t* count, double* host);



/* Neighbour list of the current positions in CSR form, input order, each row
 * sorted by index (parity checks only). offsets has n+1 entries; returns
 * CCAKE_ERR_CAPACITY with *count set when idx_cap is too small. */
ccake_status_t ccake_get_neighbours(ccake_ctx* ctx, int32_t* offsets, int32_t* idx, int64_t idx_cap,
                                    int64_t* count);

/* Batch EoS inversion on host arrays: in4 rows (e|s, rhoB, rhoS, rhoQ);
 * tbqs rows (T, muB, muQ, muS) hold the seeds on entry and the solution on
 * exit; th16 rows receive T muB muS muQ p s rhoB rhoS rhoQ e w cs2 dwds dwdB
 * dwdS dwdQ (may be NULL); status = EoS chain index used or -1.
 * Replaces EquationOfState::update_s / s_out (src/eos.cpp:574-975). */
ccake_status_t ccake_eos_invert_batch(ccake_ctx* ctx, int32_t entropy_mode, int64_t n, const double* in4,
                                      double* tbqs, double* th16, int32_t* status, int32_t* iters);

/* Tabulated EoS (eos_kind 2): uniform grid in (T, muB, muQ, muS) (fm^-1),
 * n[k] points from lo[k] with spacing d[k], nodes row-major with muS fastest,
 * 17 FP64 fields per node in the order p s rhoB rhoS rhoQ e cs2 chiBB chiQQ
 * chiSS chiBQ chiBS chiQS chiTB chiTQ chiTS chiTT (fm units). The EoS chain
 * is then table -> tanh_conformal -> conformal -> conformal_diagonal (eos_id
 * 0..3). conf5 / cdiag5: (c, T0, muB0, muQ0, muS0) of the conformal (and
 * tanh-conformal) and of the conformal-diagonal fallbacks; NULL takes the
 * reference's matching to the table (ccake_eos_table_fallback_scales at the
 * config's freeze_out_T). Copied to device memory; call after
 * ccake_ctx_create and before ccake_initialize. Replaces the table loader of
 * EquationOfState::init (src/eos_table.cpp:12-100,
 * src/eos_initialization.cpp:216-501). */
ccake_status_t ccake_set_eos_table(ccake_ctx* ctx, const int32_t* n, const double* lo, const double* d,
                                   const double* fields, const double* conf5, const double* cdiag5);

/* Fallback scales matched to a table as the reference does
 * (src/eos_initialization.cpp:276-464): with Tmax = 1.1 freeze_out_T and the
 * grid maxima mu_max, c = p(Tmax, 0, 0, 0) / Tmax^4 and T0 = 1 for both;
 * tanh-conformal / conformal mu0 = c^(1/4) mu_max / sqrt(sqrt(p(Tmax, mu_max))
 * - sqrt(p(Tmax, 0))); conformal-diagonal mu0 = (c / (p(Tmax, mu_max) -
 * p(Tmax, 0)))^(1/4) mu_max; an axis whose maximum is 0 gets mu0 = 1. Host
 * computation, no context. CCAKE_ERR_INVALID when a scale is not finite and
 * positive. */
ccake_status_t ccake_eos_table_fallback_scales(const int32_t* n, const double* lo, const double* d,
                                              const double* fields, double freeze_out_T, double* conf5,
                                              double* cdiag5);

/* Tabulated EoS from the reference's text format: eos_path is a thermo.dat
 * file or a directory holding one; line 1 the 4 grid sizes, then one line
 * per node "T muB muQ muS p s B S Q e cs2 chiBB chiQQ chiSS chiBQ chiBS chiQS
 * chiTB chiTQ chiTS chiTT" (axes in MeV, nodes row-major with muS fastest).
 * Axes are converted to fm^-1 and each grid rebuilt from its extremes; with
 * normalize_by_T the fields are ratios p/T^4 ... chi/T^2, else MeV powers.
 * Then as ccake_set_eos_table (NULL scales: matched to the table).
 * Replaces EoS_table::EoS_table
 * (src/eos_table.cpp:14-100) with InterpolatorND<4>::load_data_from_dat
 * (src/interpolatorND.cpp:125-228). */
ccake_status_t ccake_set_eos_table_file(ccake_ctx* ctx, const char* eos_path, int32_t normalize_by_T,
                                        const double* conf5, const double* cdiag5);

/* Model thermodynamics at n host rows tbqs (T, muB, muQ, muS) for EoS chain
 * index chain_index (0 = first model of the chain), 17 values per row in the
 * table's field order (NaN outside a table). Replaces
 * EquationOfState::tbqs + get_full_thermo (include/eos.h:121-175). */
ccake_status_t ccake_eos_thermo_batch(ccake_ctx* ctx, int32_t chain_index, int64_t n, const double* tbqs,
                                      double* out17);

/* Seed rules of the batch inversion (seed_mode of ccake_eos_invert_batch_ex). */
enum {
  CCAKE_SEED_REFERENCE = 0, /* the reference's seed chain from the tbqs rows */
  CCAKE_SEED_ANALYTIC = 1,  /* entropy mode, conformal models: the exact inverse,
                               accepted when max|F| < 1e-10, else Newton from it,
                               then the reference's seed chain */
  CCAKE_SEED_LEARNED = 2    /* the learned seed (ccake_mlp_train) for the first
                               model of the chain, then the reference's seed chain */
};

/* ccake_eos_invert_batch with a seed rule. No reference counterpart: the
 * reference always seeds from the previous solution. */
ccake_status_t ccake_eos_invert_batch_ex(ccake_ctx* ctx, int32_t entropy_mode, int32_t seed_mode, int64_t n,
                                         const double* in4, double* tbqs, double* th16, int32_t* status,
                                         int32_t* iters);

/* The same inversion on DEVICE arrays (same row layouts; th16 and iters may
 * be NULL), launched on `stream` (a cudaStream_t, NULL for the default
 * stream) without synchronising. No reference counterpart (batch form of
 * EquationOfState::update_s for callers whose states live on the GPU). */
ccake_status_t ccake_eos_invert_device(ccake_ctx* ctx, int32_t entropy_mode, int32_t seed_mode, int64_t n,
                                       const double* d_in4, double* d_tbqs, double* d_th16, int32_t* d_status,
                                       int32_t* d_iters, void* stream);

/* The SPH cubic-spline kernel the FP64 pair loops evaluate, on the GPU: for
 * each squared distance r2[i] (finite, >= 0) in a run of dim (2 or 3)
 * dimensions with smoothing length h, w[i] = W(sqrt(r2[i]), h) and fg[i] the
 * radial factor of its gradient, grad_a W = fg (r_a - r_b); both 0 beyond
 * r = 2h. Host arrays of n values; synchronous. Replaces
 * SPHkernel<D>::kernel(distance, hT) and SPHkernel<D>::gradKernel(rel,
 * distance, hT) (include/kernel.h:22-30, src/kernel.cpp:36-118) for a batch
 * of pairs. */
ccake_status_t ccake_sph_kernel(int32_t dim, double h, int64_t n, const double* r2, double* w, double* fg);

/* ------------------------------------------------------------------------
 * Event server: continuous batching of independent hydro events on one GPU.
 * No reference counterpart (the reference runs one event per process).
 *
 * Submitted events wait in a FIFO queue; an internal thread admits them while
 * the device bytes of the resident events stay within hbm_budget_bytes (and
 * at most max_active run at once) and keeps their state resident. An event
 * stops once every particle is frozen out (particlization in its config; the
 * freeze-out status machine at freeze_out_T) or tau reaches its tau_max.
 *  - Mixed-form events (precision 1, without the hypersurface output) of one
 *    dimension are advanced together: one CUDA-graph launch runs a
 *    candidate-list period of RK2 steps for all of them, each step kernel a
 *    single grouped launch over every event's particles; the stop rule is
 *    applied on the device before every step, and events join and leave the
 *    group between periods. Their results are those of the same event run
 *    alone (ccake_step), bit for bit.
 *  - Other events advance each on its own stream in quanta of
 *    steps_per_launch RK2 steps (CUDA-graph launches); their stop rule is
 *    applied after each quantum.
 * Events admitted while others run share the GPU.
 * ------------------------------------------------------------------------ */
typedef struct ccake_server ccake_server;

typedef struct ccake_server_config {
  int64_t hbm_budget_bytes; /* device bytes for resident events (0: 80 % of the free memory) */
  int32_t max_active;       /* events advanced concurrently (0: 32) */
  int32_t steps_per_launch; /* RK2 steps per quantum (0: 20) */
} ccake_server_config;

typedef struct ccake_event_result {
  int64_t ticket;
  int64_t particles;
  int32_t state;     /* 0 queued, 1 running, 2 done, 3 failed */
  int32_t status;    /* ccake_status_t of a failed event, else 0 */
  int32_t steps;     /* RK2 steps taken */
  int32_t frozen;    /* 1 if it stopped because every particle froze out */
  double tau;        /* final tau (fm/c) */
  double queue_s;    /* submit -> admission */
  double latency_s;  /* submit -> done */
  int64_t device_bytes;
  int32_t grouped;   /* 1: advanced with the other mixed-form events of its dimension by grouped launches */
  int32_t reserved;
} ccake_event_result;

ccake_status_t ccake_server_create(const ccake_server_config* cfg, ccake_server** out);
/* Stops the internal thread (events still running are abandoned) and frees everything. */
ccake_status_t ccake_server_destroy(ccake_server* srv);
/* Device bytes the server reserves for an event of n particles with this
 * config when it admits it (the admission rule compares these with
 * hbm_budget_bytes). No reference counterpart. */
ccake_status_t ccake_estimate_device_bytes(const ccake_config* cfg, int64_t n, int64_t* bytes);
/* Copies the event (config and host arrays) into the queue; *ticket identifies it.
 * CCAKE_ERR_CAPACITY (ticket 0, nothing queued) for an event whose device
 * bytes alone exceed the server's budget. */
ccake_status_t ccake_server_submit(ccake_server* srv, const ccake_config* cfg, const ccake_particles_soa* p,
                                   double tau_max, int64_t* ticket);
/* Current state of an event (CCAKE_ERR_INVALID for an unknown or released ticket). */
ccake_status_t ccake_server_poll(ccake_server* srv, int64_t ticket, ccake_event_result* out);
/* Blocks until no event is queued or running. */
ccake_status_t ccake_server_wait_all(ccake_server* srv);
/* A field of a finished event, caller's particle order (as ccake_copy_out). */
ccake_status_t ccake_server_copy_out(ccake_server* srv, int64_t ticket, const char* field, double* host_out);
/* Frees a finished event's device memory and forgets it. */
ccake_status_t ccake_server_release(ccake_server* srv, int64_t ticket);

/* Learned Newton seed for the tabulated EoS: a 4-64-64-64-4 tanh MLP from
 * (log e, rho_i / e^(3/4)) to (log T, mu_i / T), both standardised, trained
 * and evaluated with BF16 tensor-core kernels. No reference counterpart (the
 * reference seeds from fixed values and the previous solution).
 *
 * ccake_mlp_train: n_samples states uniform in the table's box (seeded),
 * mapped forward through the table, epochs of Adam (learning rate lr, cosine
 * decay to lr/20) on minibatches of `batch` rows; *final_mse = mean squared
 * error of the last epoch (standardised units). Needs the table. */
ccake_status_t ccake_mlp_train(ccake_ctx* ctx, int64_t n_samples, int32_t epochs, int32_t batch, double lr,
                               uint64_t seed, double* final_mse);
/* Parameters (8900 FP32: W1 [64][4], b1, W2 [64][64], b2, W3, b3, W4 [4][64],
 * b4) and standardisation (16 FP32: input mean[4], std[4], output mean[4],
 * std[4]) of the context's network. */
ccake_status_t ccake_mlp_get_params(ccake_ctx* ctx, float* params, float* norm16);
ccake_status_t ccake_mlp_set_params(ccake_ctx* ctx, const float* params, const float* norm16);
/* Network on n host rows of standardised features (4 floats each) ->
 * standardised outputs (4 floats each). */
ccake_status_t ccake_mlp_forward(ccake_ctx* ctx, int64_t n, const float* feat, float* out);
/* Gradient of the mean squared error over n host rows (standardised features
 * and targets) with respect to the 8900 parameters; *sse = sum of squared
 * errors. */
ccake_status_t ccake_mlp_gradient(ccake_ctx* ctx, int64_t n, const float* feat, const float* tgt, float* grad,
                                  double* sse);

/* Neighbour counts (the number of b != a with |r_a - r_b|^2 <= (2h)^2, the
 * same exact predicate as every other entry point) of n particles whose
 * positions are already in device memory, written to d_counts (device, n
 * int32), launched on `stream` (a cudaStream_t, NULL for the default stream).
 * No counterpart in the reference: an allocation-free entry point for callers
 * that cannot call cudaMalloc while they run (inside another library's
 * allocation-free section, from a stream callback, or under an allocator they
 * do not own). It allocates nothing: its cell-list scratch is one file-scope
 * device array for at most 262,144 particles and 262,144 cells (about 5.2 MB,
 * held by every device that loads the library until exit); larger inputs are
 * rejected with CCAKE_ERR_CAPACITY. lo3/hi3 (host, 3 doubles) bound the cell
 * grid (particles outside are clamped to edge cells; the counts do not depend
 * on the box). The first call on a device looks up the scratch address; make
 * it before any stream capture. That address is cached for the life of the
 * process, which assumes the device's primary context lives as long: do not
 * call this entry point on a device after cudaDeviceReset. Calls share the
 * scratch: calls that overlap on the GPU race and must be serialised by the
 * caller. Returns once the kernels are enqueued. */
ccake_status_t ccake_neighbour_counts_noalloc(const double* d_x, const double* d_y, const double* d_eta, int64_t n,
                                              int32_t dim, double h, const double* lo3, const double* hi3,
                                              int32_t* d_counts, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CCAKE_GPU_H */
