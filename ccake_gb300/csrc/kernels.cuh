// Device buffers and kernel launchers of the SPH hot path.
#pragma once
#include "common.cuh"
#include "eos.cuh"

namespace ccake {

// Threads a block of the per-particle kernels (also the block size of the
// grouped launches' per-event block decomposition).
constexpr int kBlock = 128;

// Device pointers of one event (struct-of-arrays slabs of length n).
struct Ptrs {
  int n;
  double* y;        // NY * n   current state
  double* y0;       // NY * n   state at the start of the RK2 step
  double* m;        // n        sph mass
  double* th;       // NTH * n  thermodynamics (LRF densities before the EoS, solution after)
  double* gam;      // n
  double* v;        // 3 * n
  double* slab;     // n        sigma_lab
  double* sig;      // n        sigma (local rest frame)
  double* bulk;     // n        Pi
  double* pi;       // NPI * n  pi^{mu nu}
  double* recA;     // RA * n   neighbour record of the smoothing pass
  double* recB;     // RB * n   neighbour record of the gradient pass
  double* grads;    // NGRAD * n (parity checks)
  double* derivs;   // NDER * n  (parity checks)
  double* in_e;     // n  input energy (or entropy) density
  double* in_s;     // n  entropy density found at initialisation
  double* in_rho;   // 3 * n input charge densities
  int32_t* eos_id;
  int32_t* eos_iters;
  int32_t* btrack;
  int32_t* freeze;
  int32_t* cell_of;
  int32_t* cell_rank;
  int32_t* cell_count;
  int32_t* cell_start;   // ncell + 1
  int32_t* cell_idx;     // n
  int32_t* scan_aux;     // 2 * scan_tiles(ncell) + 1: tile totals, tile offsets, ticket (zeroed)
  int32_t* err;          // NERR
  Clock* clock;
  double* partials;      // reduction scratch
  // per-substep neighbour list written by pass A, read by pass B (k-major:
  // entry k of particle i at k * n + i); nbr_f is the radial factor of grad W
  double* frz1_e;        // n  energy snapshot of the freeze-out status machine
  double* fz;            // 6 * NSF * n  freeze-out snapshots (with surface), else null
  double* fo_rows;       // n * kFoRow   hypersurface rows appended on the device
  int32_t* fo_count;     // 1            rows written
  float4* posf;          // FP32 copy of the positions (candidate prefilter)
  int32_t* nbr_idx;      // K * n
  double* nbr_f;         // K * n
  // factorised 3-D kernel only (else null): grad_a W = (nbr_f dx, nbr_f dy,
  // nbr_fe d eta), nbr_f = dW_2D factor x W_1D, nbr_fe = W_2D x dW_1D factor
  double* nbr_fe;        // K * n
  int K;                 // list capacity per particle
  // candidate (Verlet) list: every b within 2h + skin of a at the last
  // build, k-major like the neighbour list; rebuilt every few steps
  int32_t* cand_idx;     // Kc * n
  int32_t* cand_cnt;     // n
  int32_t* cand_max;     // 1: the largest candidate count of the last build
  int Kc;
  // mixed-precision form (precision = 1): FP32 neighbour records
  float* recAf;          // RAF * n
  float* recBf;          // RBF * n
  // diffusion sector (null when off)
  double* dif;           // NDIF * n
  double* recQ;          // RQ * n   neighbour record of the diffusion sums
};

// Grouped launches (the mixed form's step kernels). One launch covers up to
// kGroupMax events: event e owns blocks first_block[e] .. first_block[e + 1]
// - 1, kBlock particles each in the event's own block decomposition, so each
// event runs the same code on the same particles as when it is launched alone
// (a group of one) and gives the same bits. The events' constants, EoS and
// array pointers travel in the launch's parameter space (GroupArgs is passed
// by value, read as __grid_constant__), as the single-event kernels' did;
// what the kernels change between steps lives in device memory (EventState).
constexpr int kGroupMax = 16;
// eos_iters of a particle the analytic EoS pass left to the full inversion
constexpr int32_t kEosPending = -1;

struct EventDesc {
  RunConst rc;
  EosDev eos;
  Ptrs p;
};

// Mutable per-event state of a group in device memory. active = 0 (the
// device-side stop rule fired, or the event failed): its blocks return at once.
struct EventState {
  double tau_max;        // stop rule: no step starts at tau >= tau_max - dt/2
  double tau;            // tau at the last stop-rule check
  int32_t active;
  int32_t frozen_stop;   // 1: stopped because every particle froze out
  int32_t steps;         // RK2 steps taken (counted by the substep-2 clock)
  int32_t status;        // ccake_status_t of a failure seen by the stop rule
};

struct GroupArgs {
  int32_t nev;
  int32_t first_block[kGroupMax + 1];
  EventState* state;     // device, nev entries
  EventDesc ev[kGroupMax];
};

// Mixed-precision neighbour records. A position x is carried as the float
// pair (hi, lo), hi = fl(x), lo = fl(x - hi), so a difference of nearby
// positions keeps full FP32 precision. Record B (96 bytes) and the 3-D record
// A (64 bytes, padded) are 32-byte aligned, so that each pair of float4 is
// one 32-byte gather; the 2-D record A keeps 48 bytes (three 16-byte
// gathers), which holds more neighbours in L1 than the padded form.
//   A: xhi0 xhi1 xhi2 m | xlo0 xlo1 xlo2 0 | m*ext_s m*ext_B m*ext_S m*ext_Q [| 0 0 0 0 in 3-D]
//   B: xhi0 xhi1 xhi2 m | xlo0 xlo1 xlo2 p/sl^2 | e Pi/sl^2 v0 v1 |
//      v2 pi01/sl^2 pi02/sl^2 pi03/sl^2 | pi11 pi12 pi13 pi22 | pi23 pi33 0 0
//      (the pi^{ij} entries divided by sl^2 as well)
constexpr int RAF = 16;   // slab floats a particle (the 3-D stride)
template <int D>
constexpr int raf_stride() { return D == 3 ? 16 : 12; }
constexpr int RBF = 24;

// Pass A modes
enum : int { A_SMOOTH_ONLY = 0, A_WITH_THERMO = 1 };
// Pass B mode bits
enum : int { B_GRADS = 1, B_EOM = 2, B_DERIVS = 4, B_UPDATE = 8, B_WRITE_Y0 = 16 };

void launch_build_cells(const RunConst& rc, const Ptrs& p, cudaStream_t s);
void launch_candidates(const RunConst& rc, const Ptrs& p, cudaStream_t s);
void launch_passA(const RunConst& rc, const EosDev& eos, const Ptrs& p, int mode, cudaStream_t s);
void launch_thermo(const RunConst& rc, const EosDev& eos, const Ptrs& p, cudaStream_t s);
void launch_passB(const RunConst& rc, const Ptrs& p, int mode, double dt_sub, cudaStream_t s);
void launch_visc(const RunConst& rc, const Ptrs& p, cudaStream_t s);
void launch_clock(const Ptrs& p, int substep, double dt, cudaStream_t s);
void launch_init_state(const RunConst& rc, const Ptrs& p, cudaStream_t s);
// seeds: n rows (T, muB, muQ, muS) of learned seeds, or null for the reference's
void launch_init_invert(const RunConst& rc, const EosDev& eos, const Ptrs& p, const double* seeds, cudaStream_t s);
void launch_pack_inputs(const Ptrs& p, double* in4, cudaStream_t s);
void launch_sph_kernel(const RunConst& rc, int64_t n, const double* r2, double* w, double* fg, cudaStream_t s);
void launch_init_ext(const RunConst& rc, const Ptrs& p, cudaStream_t s);
void launch_init_diffusion(const Ptrs& p, const double* iq, cudaStream_t s);
void launch_init_viscous(const Ptrs& p, const double* iv, int bulk, int shear, cudaStream_t s);
void launch_totals(const RunConst& rc, const Ptrs& p, int nblocks, cudaStream_t s);
void launch_neighbour_counts(const RunConst& rc, const Ptrs& p, int32_t* counts, cudaStream_t s);
void launch_neighbour_fill(const RunConst& rc, const Ptrs& p, const int32_t* offsets, int32_t* idx,
                           cudaStream_t s);
void launch_pack_fp64(const RunConst& rc, const Ptrs& p, cudaStream_t s);
void launch_pack_mixed(const RunConst& rc, const Ptrs& p, cudaStream_t s);
// The mixed form's step kernels as grouped launches (see GroupArgs): pass A
// (smoothing sums and neighbour list, then the FP64 EoS), pass B (gradient
// sums, then the equations of motion and the RK2 update of substep `sub`, dt
// from each event's config), the clock, the freeze-out status machine, and
// the stop rule (before a step: retire events that are all frozen out with
// particlization, that reached tau_max, or that raised an error). The
// events' EoS must carry jac32 = 1 (FP32 table Newton Jacobians).
void launch_passA_mixed(const GroupArgs& g, int dim, cudaStream_t s);
void launch_passB_mixed(const GroupArgs& g, int dim, int mode, int sub, cudaStream_t s);
void launch_clock_group(const GroupArgs& g, int sub, cudaStream_t s);
void launch_freeze_group(const GroupArgs& g, cudaStream_t s);
void launch_stop_group(const GroupArgs& g, cudaStream_t s);
void launch_eos_thermo(const EosDev& eos, int chain_index, int64_t n, const double* tbqs, double* out17,
                       cudaStream_t s);
// Batch inversion. With scratch (n + 1 int32, device) and seed_mode 0 or 2,
// two passes: the first attempt of every row with a Newton budget of
// kEosFirstIters, then the full inversion of the rows it left (same results
// as one pass).
constexpr int kEosFirstIters = 8;
void launch_table_f32(const double* f, float* fd, int64_t nodes, cudaStream_t s);
void launch_preinv_grid(const PreinvView& P, int64_t tile0, int64_t count, double* in4, double* tbqs, cudaStream_t s);
void launch_preinv_pack(int64_t count, const double* th16, const int32_t* status, double* out, int32_t* nfail,
                        cudaStream_t s);
void launch_preinv_lookup(const PreinvView* P, int64_t n, const double* sBSQ, double* out, cudaStream_t s);
void launch_diagnostics(const RunConst& rc, const Ptrs& p, int grads_f32, cudaStream_t s);
// status machine, snapshots and hypersurface rows after a step (cfg.surface)
void launch_freeze_surface(const RunConst& rc, const Ptrs& p, int grads_f32, double dt, cudaStream_t s);
// the gradient sums of the mixed pass B alone (no equations of motion)
void launch_gradients_mixed(const GroupArgs& g, int dim, cudaStream_t s);
void launch_eos_batch(const EosDev& eos, int entropy, int seed_mode, int64_t n, const double* in4, double* tbqs,
                      double* th16, int32_t* status, int32_t* iters, int32_t* scratch, cudaStream_t s);

// Stop-rule probe of an event: the largest temperature, the current tau and
// the error counters (filled by launch_probe).
struct Probe {
  double maxT;
  double tau;
  int32_t err[NERR];
  int32_t frozen;   // particles with freeze >= 4
  int32_t pad;
};
void launch_freeze(const RunConst& rc, const Ptrs& p, cudaStream_t s);
void launch_count_frozen(const Ptrs& p, int32_t* out, cudaStream_t s);
void launch_probe(const Ptrs& p, Probe* out, cudaStream_t s);

constexpr int kTotBlocks = 608;   // 4 x 152 SMs; fixed so the sums are reproducible

// CTAs of the cell-count scan (1024 cells each)
inline int scan_tiles(int ncell) { return (ncell + 1023) / 1024; }

}  // namespace ccake
