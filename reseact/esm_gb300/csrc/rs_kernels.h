// rs_kernels.h -- host-visible launch interface of the device kernels (no CUDA types beyond
// cudaStream_t cross it, so the C-ABI layer in rs_api.cpp stays plain C++).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "rs_device.cuh"

namespace rs {

// Per-thread work-array capacities of the two chemistry kernel instantiations.
constexpr int kSmallMS = 16, kSmallMR = 40, kSmallMLU = 160, kSmallMP = 80;
constexpr int kLargeMS = 64, kLargeMR = 128, kLargeMLU = 1600, kLargeMP = 256;
constexpr int kMaxProgStack = 32;

struct JitChem;
struct MixedTmaps;  // tensor maps of the mixed-precision split planes (rs_transport.cu)

struct LaunchCtx {
  cudaStream_t stream;
  DevMech mech;
  int nc;          // cells
  int nsp;         // species per cell in the state (chemistry species + air mass)
  int size_class;  // 0 small, 1 large
  const JitChem* jit = nullptr;  // mechanism-specialised kernels, or null: table-walking ones
};

struct PerCellArgs {
  double t0, t1, dt0, rtol, atol, maxiters;
  double beta1, beta2, invqmin, invqmax, gamma, qsmin, qsmax, qoldinit;
  int clamp;
  double* totals;  // [accepted substeps, attempts] summed over cells, or null
};

// Transport geometry and forcing on the device (grid SoA, lon fastest).
template <typename R>
struct DevTransport {
  int nlon, nlat, nlev, ntr, nsp, lon_bc, lat_bc;
  double omega;
  const double* gx;    // [nlat]
  const double* gylo;  // [nlat]
  const double* gyhi;  // [nlat]
  const double* mx;    // [nlev][nlat][nlon+1]
  const double* my;    // [nlev][nlat+1][nlon]
  const double* mz;    // [nlev+1][nlat][nlon]
  const double* qw;    // [ntr][nlev][nlat]
  const double* qe;
  const double* qs;    // [ntr][nlev][nlon]
  const double* qn;
  const double* vsA;   // [(nlev+2)][ncol] slope coefficients, cells -1..nlev
  const double* vsB;
  const double* veAB;  // [(nlev+1)][ncol] edge coefficients, edges 0..nlev
  const double* veC;
  const double* veD;
  R* fx;               // [ntr][nlev][nlat][nlon+1]
  R* fy;               // [ntr][nlev][nlat+1][nlon]
  R* fz;               // [ntr][nlev+1][nlat][nlon]
  // mixed precision (compensated FP32): the RHS input split into hi, lo planes [ntr][nc]
  // (hi + lo = q to 2^-47), the metric factors and vertical coefficients as (hi, lo) pairs, and
  // the per-cell accumulator of m dq/dt as pairs [ntr][nc] (in the memory of fx)
  float* qhi;
  float* qlo;
  const float2* gx2;    // [nlat]
  const float2* gylo2;  // [nlat]
  const float2* gyhi2;  // [nlat]
  const float2* vsA2;   // as vsA / vsB / veAB / veC / veD
  const float2* vsB2;
  const float2* veAB2;
  const float2* veC2;
  const float2* veD2;
  float2* acc;
  const float2* mx2;    // the air-mass face fluxes as pairs (shapes of mx, my, mz)
  const float2* my2;
  const float2* mz2;
  int mixed;
  // full PBL mixing (transport half): per-layer fraction f and weight w = dp*f, the column
  // normaliser max(sum_k w, 1 Pa), scratch for the per-tracer column means, 1/tau
  int pbl;
  const double* pbl_f;     // [nlev][nlat][nlon]
  const double* pbl_w;     // [nlev][nlat][nlon]
  const double* pbl_den;   // [nlat][nlon]
  double* pbl_qbar;        // [ntr][nlat][nlon]
  double pbl_tau, pbl_rtau;
  // pressure fixer: per-cell correction of the horizontal divergence in the air-mass equation,
  // dm/dt = -(((DxM + DyM) + mcorr) + DzM); null when off
  const double* mcorr;     // [nlev][nlat][nlon]
  // launch shape of the FP64 pencil flux kernels (chosen by rs_autotune)
  int pencil;    // pencils per block in the lat / vertical kernels: 8, 16 or 32
  int rows;      // threads along the pencil (blockDim.y): 4 .. 32
  int xthreads;  // threads per lon row: 64 .. 256 in steps of 32
  int xgroups, yzgroups;  // tracer groups (blockIdx.y) of the lon / lat and vertical pencils
  // launch shape of the mixed-precision pencil kernels (chosen by rs_autotune)
  int mpencil, mrows, mxthreads;
  int msper_x, msper_yz;  // tracers per block (blockIdx.y selects the group)
  // bulk-copy staging of the mixed pencils: host-side tensor maps (null: plain loads) and the
  // device word a pencil kernel sets when a staging wait runs out (1) -- the solve then stops
  const MixedTmaps* tma;
  int* tma_err;
  int mbulk_x, mbulk_yz;  // use the bulk copies for lon rows / lat and vertical pencils
  // streaming forms instead of the pencils (no shared memory): a warp of shuffles per lon row
  // segment, one thread per lat / vertical line
  int mstream_x, mstream_yz;
};

// chemistry (rs_chem.cu)
void launch_rates(const LaunchCtx& L, const double* T, const double* P, double* kr);
// F0/F1 (optional, the specialised kernels only): per-cell f(U0)/f(U1) planes [ns][nc] that
// let an attempt reuse the previous accepted attempt's last RHS evaluation.
void launch_ros23_attempt(const LaunchCtx& L, const Ctl* ctl, double* U0, double* U1,
                          const double* kr, const double* em, double* part, double rtol,
                          double atol, int clamp, double* F0 = nullptr, double* F1 = nullptr);
// One step at the controller's dtc that is accepted whatever its error (the replay of a
// recorded step): the specialised kernels skip the error estimate; the table kernels run the
// full attempt (part: its block partials, unused).  Same new state as launch_ros23_attempt.
void launch_ros23_step(const LaunchCtx& L, const Ctl* ctl, double* U0, double* U1,
                       const double* kr, const double* em, double* part, double rtol,
                       double atol, int clamp);
void launch_chem_rhs(const LaunchCtx& L, const double* U, const double* kr, const double* em,
                     double* dU);
void launch_block_jac(const LaunchCtx& L, const double* U, const double* kr, const int* srow,
                      const int* scol, double* J);
// regcap: the form capped at 32 registers (2048 resident threads per SM)
void launch_chem_per_cell(const LaunchCtx& L, int nblocks, int threads, double* U,
                          const double* kr, const double* em, double* dtc, double* steps,
                          unsigned long long* queue, int* status, const PerCellArgs& a,
                          bool regcap = false);
// the per-cell form with G lanes per cell (G = 4, 8, 16; table mechanisms, minimum-fill order):
// doubles of shared memory per cell, the threads per block that fit (0: none), resident blocks
// per SM, and the launch
int group_cell_doubles(const DevMech& M);
int chem_group_threads(const LaunchCtx& L, int G);
int chem_group_blocks_per_sm(const LaunchCtx& L, int G, int threads);
void launch_chem_per_cell_group(const LaunchCtx& L, int G, int nblocks, int threads, double* U,
                                const double* kr, const double* em, double* dtc, double* steps,
                                unsigned long long* queue, int* status, const PerCellArgs& a);

// transport (rs_transport.cu).  Stage s in 1..4 of one SSPRK43 attempt; buffers:
// U0/U1 accepted/candidate (selected by ctl->cur), S1..S3 stage scratch.
struct TransportBufs {
  double* U0;
  double* U1;
  double* S1;
  double* S2;
  double* S3;
  double* partial;
};
void launch_ssprk43_attempt(cudaStream_t st, const DevTransport<double>& T, const Ctl* ctl,
                            const TransportBufs& B, double rtol, double atol, int clamp);
// du = f_transport(u) with flux time factor g for a grid-SoA state (single evaluation hook)
// dUadv (optional): the same tendency without the PBL mixing term (the adjoint's air-mass
// derivative uses the advective part only)
void launch_transport_rhs(cudaStream_t st, const DevTransport<double>& T, const double* U,
                          double g, double* dU, double* dUadv = nullptr);

// Tensor maps for the bulk-copy staging of the mixed pencils over T.qhi / T.qlo; null (and the
// reason in *why) where the grid does not meet the copy engine's alignment and size rules.
MixedTmaps* mixed_tmaps_create(const DevTransport<double>& T, const char** why);
// Dynamic shared memory of a mixed-precision pencil block (pw = 1: a lon row) and the cap.
size_t mixed_pencil_bytes(int n, int pw, bool tma);
size_t mixed_pencil_cap();
void mixed_tmaps_destroy(MixedTmaps* m);
bool mixed_tmaps_dir_ok(const MixedTmaps* m, int dir);  // dir 0 lon rows, 1 lat, 2 vertical
void launch_flux_dir(cudaStream_t st, const DevTransport<double>& T, const double* Q, int dir);
// (hi, lo) float pairs of n doubles (the mixed kernels' face fluxes)
void launch_make_pairs(cudaStream_t st, const double* src, float2* dst, size_t n);
void launch_flux_dir_mixed(cudaStream_t st, const DevTransport<double>& T, const double* Q, int dir,
                           bool split);

// control (rs_control.cu)
void launch_ctl_init(cudaStream_t st, Ctl* ctl, const Ctl& init);
void launch_replay_accept(cudaStream_t st, Ctl* ctl);
// adjoint tape: after an attempt's controller, store the pre-step state of an accepted step
// (two launches; no-ops unless the controller carries a tape)
void launch_tape_store(cudaStream_t st, const Ctl* ctl, const double* U0, const double* U1,
                       size_t n);
void launch_clamp_mask(cudaStream_t st, size_t n, double* lam, const double* out);

// discrete adjoint (rs_adjoint.cu)
// kz (optional, the specialised kernels only): the step's k1 and z2 from the stage tape
void launch_ros23_vjp(const LaunchCtx& L, const double* U, const double* Uout, const double* lam,
                      double* lam_out, const double* kr, const double* em, double* ebar,
                      double dt, int clamp, const double* kz = nullptr);
void launch_transport_rhs_vjp(cudaStream_t st, const DevTransport<double>& T, const double* U,
                              const double* F, const double* fbar, double* ubar, double* G,
                              double* Cf, double g);
void launch_lincomb(cudaStream_t st, size_t n, double* out, double a, const double* x, double b,
                    const double* y, double c, const double* z);
void launch_finalize(cudaStream_t st, Ctl* ctl, const double* partial, int nparts);
void launch_finalize_graph(cudaStream_t st, Ctl* ctl, const double* partial, int nparts,
                           cudaGraphConditionalHandle loop);
void launch_nonfinite(cudaStream_t st, const double* U, size_t n, int* flag);
void launch_to_soa(cudaStream_t st, const double* cm, double* soa, int nlon, int nlat, int nlev,
                   int nsp);
void launch_to_cellmajor(cudaStream_t st, const double* soa, double* cm, int nlon, int nlat,
                         int nlev, int nsp);

}  // namespace rs
