/*
 * reseact_gb300.h -- C ABI of the GB300 operator-split step (libreseact_gb300.so).
 *
 * One Lie-Trotter macro step of ReSEACT: SSPRK43 flux-form PPM transport over [t0, t1]
 * followed by Rosenbrock23 block-diagonal chemistry over [t0, t1], each with its own
 * adaptive PI controller and a clamp to >= 0 of every accepted state.
 *
 * Reference interfaces this ABI replaces (paths relative to the reference repository):
 *   rs_macro_step      <- OpSplit.lie_trotter_solve            tools/reactant_handoff/op_split.jl:100-164
 *                         and the device-resident twin adv(...)  run_reseact_reactant.jl:310-355
 *                         (dtT/dtC carried in and out exactly as adv returns dtTend/dtCend)
 *   rs_set_forcing     <- refresh_forcing + sync_forcing!       run_reseact_reactant.jl:360-366,434-440
 *   rs_set_state /     <- the cell-major state vector u[(c-1)*NS+s]
 *   rs_get_state          (cellmajor_perm, prototypes/reseact_3d_chem/block_jac.jl:18-40;
 *                          state dump layout run_reseact.jl:378-391)
 *   rs_rhs_transport   <- f_trans! (transport half of the split, split_common.jl:530-533)
 *   rs_rhs_chem        <- f_chem!  (chemistry half, split_common.jl:530-533)
 *   rs_block_jac       <- block_ad_jac / symbolic block Jacobian
 *                         prototypes/reseact_3d_chem/block_jac.jl:108-136,
 *                         tools/reactant_handoff/rx_sym_block_jac.jl:205-233
 *   rs_single_step     <- ssprk43_step / ros23_step             rx_traced_integrator.jl:362-400 / 279-349
 *   rs_record / rs_backward_macro_step / rs_adjoint_*  <- forward_pass (checkpoints +
 *                         recorded (t,dt)), backward_sweep / backward_stage!, ros23_step_vjp and
 *                         ssprk43_step_vjp (tools/adjoint_gradient.jl:609-835,
 *                         rx_traced_integrator.jl:610-623)
 *   rs_get_rate_constants <- the per-cell rate constants of the .esm mechanism
 *                         (prototypes/g2_depsink/g2_nodep.esm:450-1780,1861)
 *
 * Conventions
 *   - Every entry point returns rs_status (0 = RS_OK); no C++ exception crosses the ABI.
 *     rs_last_error(h) returns the text of the handle's last failure.
 *   - Host pointers are borrowed for the duration of the call only; the handle owns all
 *     device memory and its CUDA stream.  Calls are synchronous on return.
 *   - One handle per host thread.
 *   - Gridded host arrays use the reference's Julia array order (lon fastest):
 *     a field of shape (NLON, NLAT, NLEV) is the C array [NLEV][NLAT][NLON].
 *   - The state is CELL-MAJOR as in the reference: u[c*NS + s] with cells sorted by
 *     (i_lon, j_lat, k_lev) tuples, i.e. c = (i*NLAT + j)*NLEV + k (0-based), and species
 *     sorted by name with the air mass "m" last (when has_air_mass = 1).
 */
#ifndef RESEACT_GB300_H
#define RESEACT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RS_API_VERSION 1

typedef enum rs_status {
  RS_OK = 0,
  RS_ERR_INVALID = 1,     /* bad argument or configuration */
  RS_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  RS_ERR_MAXITERS = 3,    /* adaptive loop hit maxiters before t1 (reference: maxiters cap) */
  RS_ERR_NONFINITE = 4,   /* non-finite state after a macro step */
  RS_ERR_NOMEM = 5,       /* device allocation failed */
  RS_ERR_STATE = 6,       /* call out of order (e.g. no forcing set) */
  RS_ERR_UNSUPPORTED = 7  /* feature not available (library, device or configuration) */
} rs_status;

/* lateral boundary kinds */
enum { RS_BC_PERIODIC = 0, RS_BC_OPEN = 1, RS_BC_CLOSED = 2 };
/* arithmetic of the transport half: FP64, or MIXED = compensated FP32 (the PPM reconstruction
 * and face terms in double-float pairs on the FP32 pipe, about 48 significant bits; the state,
 * air mass, stage updates and error norm in FP64) */
enum { RS_PREC_FP64 = 0, RS_PREC_MIXED = 1 };
/* chemistry step-size control: one global dt (reference) or per-cell adaptive substeps */
enum { RS_CHEM_GLOBAL_DT = 0, RS_CHEM_PER_CELL = 1 };
/* rs_single_step operators */
enum { RS_OP_TRANSPORT = 0, RS_OP_CHEMISTRY = 1 };

/* rate-program opcodes (postfix), one program per reaction */
enum {
  RS_OP_CONST = 0, RS_OP_TEMP = 1, RS_OP_PRES = 2, RS_OP_PARAM = 3,
  RS_OP_ADD = 10, RS_OP_SUB = 11, RS_OP_MUL = 12, RS_OP_DIV = 13, RS_OP_POW = 14, RS_OP_NEG = 15,
  RS_OP_EXP = 20, RS_OP_LOG = 21, RS_OP_LOG10 = 22, RS_OP_SQRT = 23
};

/* A mass-action mechanism, lowered from an .esm reaction_systems entry.
 * Species are the n_species non-constant species (sorted by name); constant species are
 * folded into the rate programs.  Reaction r consumes react_species[react_ptr[r]..react_ptr[r+1])
 * with integer stoichiometry react_nu and produces prod_species with coefficients prod_coef.
 * Its rate constant is the postfix program prog_op/prog_val[prog_ptr[r]..prog_ptr[r+1]),
 * evaluated per cell from T, P and params[].  combinatoric = 1 divides the mass-action
 * product by prod(nu!) (Catalyst's default rate law). */
typedef struct rs_mechanism {
  int32_t n_species;
  int32_t n_reactions;
  int32_t n_params;
  int32_t combinatoric;
  const int32_t* react_ptr;     /* [n_reactions+1] */
  const int32_t* react_species; /* [react_ptr[n_reactions]] */
  const int32_t* react_nu;
  const int32_t* prod_ptr;      /* [n_reactions+1] */
  const int32_t* prod_species;
  const double* prod_coef;
  const int32_t* prog_ptr;      /* [n_reactions+1] */
  const int32_t* prog_op;
  const double* prog_val;
  const double* params;         /* [n_params] */
} rs_mechanism;

/* Lat-lon grid.  Cell centres lon0 + i*dlon, lat0 + j*dlat (degrees); latitude edges are
 * centre +- dlat/2 clamped to [-90, 90] (half-width polar caps for pole-centred grids). */
typedef struct rs_grid {
  int32_t nlon, nlat, nlev;
  int32_t lon_bc;  /* RS_BC_PERIODIC (global) or RS_BC_OPEN (regional inflow/outflow) */
  int32_t lat_bc;  /* RS_BC_CLOSED (poles, zero flux) or RS_BC_OPEN (regional) */
  double lon0_deg, dlon_deg;
  double lat0_deg, dlat_deg;
} rs_grid;

/* PI controller constants (rx_traced_integrator.jl:86-99). */
typedef struct rs_controller {
  double beta1, beta2, qmin, qmax, gamma, qsteady_min, qsteady_max, qoldinit;
} rs_controller;

typedef struct rs_config {
  int32_t api_version;     /* RS_API_VERSION */
  int32_t device;          /* CUDA device ordinal */
  rs_grid grid;
  int32_t has_air_mass;    /* 1: state carries a trailing air-mass species m (transport) */
  int32_t do_transport;    /* 1: run the SSPRK43 half */
  int32_t do_chemistry;    /* 1: run the Rosenbrock23 half */
  rs_mechanism mech;
  double rtol_T, atol_T;   /* transport tolerances (reference: 1e-4, 1e-6) */
  double rtol_C, atol_C;   /* chemistry tolerances (reference: 1e-4, 1e-9) */
  rs_controller ctrl_T;    /* SSPRK43: beta1 7/30, beta2 2/15, qsteady_max 1 */
  rs_controller ctrl_C;    /* ROS23:   beta1 7/20, beta2 1/5,  qsteady_max 6/5 */
  double maxiters;         /* per adaptive solve (reference: 2e4) */
  int32_t clamp_nonneg;    /* clamp accepted states to >= 0 (reference: true) */
  int32_t precision;       /* RS_PREC_FP64 or RS_PREC_MIXED */
  int32_t chem_mode;       /* RS_CHEM_GLOBAL_DT or RS_CHEM_PER_CELL */
} rs_config;

/* Forcing for one macro step (refresh_forcing).  NULL members keep their previous value
 * (zero before the first call).  Horizontal air-mass fluxes are on the unit sphere
 * (Mx = dp_face*U_face/a, Pa/s); Mz (Pa/s) is at the LOWER edge of each level, +ve upward,
 * level 0 at the surface.  All three scale in time by cos(flux_omega*t); flux_omega is taken
 * only from a call that passes at least one flux field. */
typedef struct rs_forcing {
  const double* mx;          /* [nlev][nlat][nlon+1] west-face zonal flux */
  const double* my;          /* [nlev][nlat+1][nlon] south-face meridional flux */
  const double* mz;          /* [nlev+1][nlat][nlon] */
  double flux_omega;         /* rad/s; 0 = steady fluxes */
  const double* dp;          /* [nlev][nlat][nlon] pressure thickness (vertical PPM geometry) */
  const double* qbc_w;       /* [n_species][nlev][nlat] west-halo mixing ratios (open lon BC) */
  const double* qbc_e;       /* [n_species][nlev][nlat] */
  const double* qbc_s;       /* [n_species][nlev][nlon] south-halo mixing ratios (open lat BC) */
  const double* qbc_n;       /* [n_species][nlev][nlon] */
  const double* temperature; /* [nlev][nlat][nlon] K */
  const double* pressure;    /* [nlev][nlat][nlon] Pa */
  const double* emission;    /* [n_species][nlev][nlat][nlon] source added to d(species)/dt */
  /* GEOS-Chem-style full PBL mixing, a transport-half term (reseact.esm Transport3D equations
   * p_pbl_top, pbl_f, pbl_wt, pbl_sum_*, pbl_mean_*; tracer tendency
   * pbl_f*(pbl_mean - q)/tau_pblmix).  p_pbl_top = PS*exp(-PBLH*g/(Rd*T_surface)) with
   * g = 9.80665, Rd = 287.05 and T_surface the temperature of level 0; pbl_f is the clamped
   * overlap of each layer's pressure interval with [p_pbl_top, PS] over dp; the mean is
   * sum_k (dp*pbl_f)_k q_k / max(sum_k (dp*pbl_f)_k, 1 Pa).  Active once pblh, ps, hyb_a,
   * hyb_b and the temperature have been given and tau_pblmix > 0; tau_pblmix is taken from a
   * call that passes pblh.  Exactly mass-conserving: sum_k dp_k * tendency_k = 0. */
  const double* pblh;        /* [nlat][nlon] PBL height (m) */
  const double* ps;          /* [nlat][nlon] surface pressure (Pa) */
  const double* hyb_a;       /* [nlev+1] interface pressure coefficient A (Pa), 0 = surface */
  const double* hyb_b;       /* [nlev+1] interface coefficient B: p_k = A_k + B_k * PS */
  double tau_pblmix;         /* relaxation time (s); the reference's default is 900 */
  /* Pressure fixer with diagnosed vertical mass flux (reseact.esm Transport3D divh, divh_col,
   * dp_col, divh_fix, Mz, dm/dt): with dps_dt and hyb_b given, the horizontal divergence is
   * corrected to the surface-pressure tendency, divh_fix = divh + (-dPSdt - sum_k divh_k) *
   * dp_k / sum_k dp_k; Mz is diagnosed as sum over the layers below of -(dB_k dPSdt +
   * divh_fix_k) (the mz field is then ignored); the air mass obeys dm/dt = -(divh_fix + D(Mz))
   * = dB_k dPSdt; tracers keep the raw horizontal fluxes with the diagnosed Mz.  Needs steady
   * fluxes (flux_omega = 0). */
  const double* dps_dt;      /* [nlat][nlon] surface-pressure tendency (Pa/s) */
} rs_forcing;

/* Per-macro-step statistics (op_split.jl:159-163 return tuple plus the carried dts). */
typedef struct rs_stats {
  double naT, nrT;       /* transport accepted / rejected attempts */
  double naC, nrC;       /* chemistry accepted / rejected attempts (global-dt mode); in
                            per-cell mode the accepted / rejected substeps summed over cells */
  double dtT_end, dtC_end;
  double tT_end, tC_end; /* time reached by each half (== t1 on success) */
  double chem_cell_steps;  /* per-cell mode: sum over cells of accepted substeps */
  double kernel_launches;  /* CUDA kernels this call launched (device loop + checks) */
  int32_t status;
} rs_stats;

typedef struct rs_handle rs_handle;

/* Fill *cfg with the reference defaults (tolerances, controllers, clamp, maxiters). */
void rs_default_config(rs_config* cfg);

rs_status rs_create(const rs_config* cfg, rs_handle** out);
void rs_destroy(rs_handle* h);
const char* rs_last_error(const rs_handle* h);

/* Number of state values (cells * species) and of species per cell. */
size_t rs_state_size(const rs_handle* h);
int32_t rs_species_per_cell(const rs_handle* h);

rs_status rs_set_state(rs_handle* h, const double* u_cellmajor, size_t n);
rs_status rs_get_state(rs_handle* h, double* u_cellmajor, size_t n);
rs_status rs_set_forcing(rs_handle* h, const rs_forcing* f);

/* Rate constants k[r][cell] (cell in grid order [nlev][nlat][nlon]).  rs_rates recomputes
 * them from T/P/params; rs_set_rate_constants installs caller-provided values (e.g. per-cell
 * photolysis) until the next forcing change of T or P. */
rs_status rs_get_rate_constants(rs_handle* h, double* k, size_t n);
rs_status rs_set_rate_constants(rs_handle* h, const double* k, size_t n);

/* Per-cell chemistry (RS_CHEM_PER_CELL) diagnostics, cell in grid order: the accepted substeps
 * of each cell in the last macro step (steps, may be NULL) and the step size each cell carries
 * into the next (dt, may be NULL; 0 before the first window).  n = the cell count.  No
 * reference counterpart (the reference has one global step size). */
rs_status rs_get_cell_steps(rs_handle* h, double* steps, double* dt, size_t n);

/* One Lie-Trotter macro step over [t0, t1] on the resident state.  *dtT / *dtC are the
 * carried step sizes in and out.  Returns RS_ERR_MAXITERS / RS_ERR_NONFINITE on failure
 * (the state then holds whatever the halves reached; bisection stays with the caller, as
 * in op_split.jl:219-241). */
rs_status rs_macro_step(rs_handle* h, double t0, double t1, double* dtT, double* dtC,
                        rs_stats* out);

/* Single evaluations for parity tests (host arrays in the cell-major state layout). */
rs_status rs_rhs_transport(rs_handle* h, double t, const double* u, double* du, size_t n);
rs_status rs_rhs_chem(rs_handle* h, double t, const double* u, double* du, size_t n);
/* J[c][r][s] = d f_chem(cell c, species r) / d u(cell c, species s) */
rs_status rs_block_jac(rs_handle* h, const double* u, double* jac, size_t n_jac);
/* One unclamped attempt of the chosen integrator from u_in; writes u_out and the hairer
 * error estimate. */
rs_status rs_single_step(rs_handle* h, int32_t op, double t, double dt, const double* u_in,
                         double* u_out, double* eest, size_t n);

/* Device view of the resident state for zero-copy callers: species-major planes
 * [species][nlev][nlat][nlon] of doubles.  Valid until the next rs_macro_step. */
rs_status rs_state_device_ptr(rs_handle* h, void** d_state);
/* The handle's CUDA stream (cudaStream_t), for callers timing with CUDA events. */
void* rs_stream(rs_handle* h);

/* Project-written autotuner (no reference counterpart): times candidate launch shapes on the
 * handle's current state and forcing -- threads per block x blocks per SM ("cells per block")
 * of the per-cell chemistry kernel (three attempts per cell on scratch copies) and, for the
 * table-walking kernels of the production build, the form with G = 4, 8 or 16 lanes per cell
 * and its work arrays in shared memory; threads per lon row and pencil width x rows per block
 * (the halo tile) of the transport kernels -- keeps the fastest for this handle and writes a
 * JSON report of every candidate into buf. */
rs_status rs_autotune(rs_handle* h, char* buf, size_t buf_len);

/* Set one launch shape that rs_autotune would choose, e.g. to replay an earlier tuning without
 * timing again (no reference counterpart).  Keys: "xthreads", "pencil", "rows",
 * "x_tracer_groups", "yz_tracer_groups" (FP64 pencils);
 * "mixed_xthreads", "mixed_x_tracers", "mixed_pencil", "mixed_rows", "mixed_yz_tracers",
 * "mixed_x_bulk", "mixed_yz_bulk" (mixed pencils); "mixed_x_stream", "mixed_yz_stream" (1: the
 * streaming forms of the mixed kernels instead of the pencils); "per_cell_threads",
 * "per_cell_blocks_per_sm", "per_cell_group" (per-cell chemistry; group 0 = one thread per
 * cell, 4 / 8 / 16 = lanes per cell, production build only), "per_cell_regcap" (1: the
 * table-walking per-cell kernel at 32 registers); "chem_attempt_variant" (0 "regs", 1 "smem",
 * 2 "regs2", 3 "split": how the specialised attempt kernel keeps W, where built).  Values outside a key's
 * candidates are RS_ERR_INVALID.  Every shape gives bit-identical results. */
rs_status rs_set_launch_shape(rs_handle* h, const char* key, int32_t value);

/* Chemistry kernel selection (no reference counterpart; the reference compiles its RHS and
 * Jacobian from the .esm system into native code, which the SPECIALIZED kernels mirror).
 * SPECIALIZED: the mechanism's rate products, RHS, Jacobian, LU and solves are generated as
 *   straight-line CUDA at rs_create and compiled for the device with NVRTC (mechanisms of up
 *   to 32 species and 256 LU slots);
 * TABLE: one kernel for every mechanism that walks the sparse tables;
 * AUTO (the default): SPECIALIZED when it could be built, else TABLE.
 * Both compute the same arithmetic in the same order.  rs_set_chem_kernel returns
 * RS_ERR_UNSUPPORTED for SPECIALIZED when it could not be built (reason in rs_last_error). */
enum { RS_CHEM_KERNEL_AUTO = 0, RS_CHEM_KERNEL_TABLE = 1, RS_CHEM_KERNEL_SPECIALIZED = 2 };
rs_status rs_set_chem_kernel(rs_handle* h, int32_t kind);
/* The kernel kind in use (TABLE or SPECIALIZED) and a one-line JSON description of it. */
rs_status rs_get_chem_kernel(rs_handle* h, int32_t* kind, char* info, size_t info_len);
/* Staging of the mixed-precision transport pencils (no reference counterpart).  Beside the
 * pencils, the mixed transport has streaming forms without shared memory (a warp of shuffles
 * per lon-row segment, one thread per lat / vertical line with a register window) that form the
 * same pairs in the same order; in AUTO mode rs_autotune picks per direction among all of them,
 * PLAIN and BULK select the pencils.
 * BULK: the interior of every lat / vertical pencil is copied into shared memory by one
 *   tensor-map bulk copy (TMA) per split plane and every lon row by a 1-D bulk copy, double
 *   buffered across tracers; the ghost cells are loaded by the threads.  Used where the grid
 *   meets the copy engine's rules (nlon % 4 == 0, nlat and nlev <= 256 for the pencils);
 * PLAIN: the threads load every cell;
 * AUTO (the default): BULK where available (rs_autotune may pick PLAIN when it is faster).
 * Both give bit-identical fluxes.  A bulk-copy wait that runs out stops the solve with
 * RS_ERR_CUDA.  rs_get_transport_staging reports the mode in use and a one-line JSON of the
 * directions that can use bulk copies. */
enum { RS_STAGING_AUTO = 0, RS_STAGING_PLAIN = 1, RS_STAGING_BULK = 2 };
rs_status rs_set_transport_staging(rs_handle* h, int32_t mode);
rs_status rs_get_transport_staging(rs_handle* h, int32_t* mode, char* info, size_t info_len);
/* The generated CUDA source of a mechanism's specialised kernels, and an NVRTC compile of it
 * for sm_103a with ptxas's resource report in log; neither needs a device.  *len_out (may be
 * NULL) receives the source length + 1; buf may be NULL to query it. */
/* Elimination order of the pivot-free LU of W = I - gamma h J: ord[k] is the species
 * eliminated at pivot k.  The strict build keeps the reference's natural order (blocksolve,
 * rx_traced_integrator.jl:110-135); the production build eliminates in a greedy minimum-fill
 * order (same symmetric permutation of rows and columns, fewer fill-in slots and updates).
 * rs_mechanism_lu_order gives either order for a mechanism without a device. */
rs_status rs_lu_order(rs_handle* h, int32_t* ord, int32_t n);
rs_status rs_mechanism_lu_order(const rs_mechanism* mech, int32_t natural, int32_t* ord,
                                int32_t n);
/* Lie-Trotter window solve inside the library (op_split.jl:100-164 lie_trotter_solve and
 * :219-241 lie_trotter_solve_bisect): the stop grid is the macro-dt lattice joined with the
 * forcing cadence boundaries in the half-open interval (t0, t1] and t1 itself; each stop
 * interval is one rs_macro_step; refresh(user, t) fires after a stop that lands on a cadence
 * boundary (the callback may call rs_set_forcing); with min_macro_dt > 0 a failed window
 * restarts from its initial state (kept on the device) as two halves, down to min_macro_dt,
 * calling on_bisect(user, t0, t1) first.  Works on the device-resident state (rs_set_state /
 * rs_get_state around it); *dtT / *dtC carry the inner step sizes in and out.  The counts in
 * the result are summed over the windows that succeeded (a failed window's attempts are not
 * counted, as in the reference). */
typedef void (*rs_refresh_fn)(void* user, double t);
typedef void (*rs_bisect_fn)(void* user, double t0, double t1);
typedef struct rs_solve_opts {
  double macro_dt;              /* > 0 */
  double min_macro_dt;          /* bisection floor (reference default 9 s); <= 0: no bisection */
  const double* forcing_tstops; /* cadence boundaries (may be NULL) */
  size_t n_tstops;
  rs_refresh_fn refresh;        /* may be NULL */
  rs_bisect_fn on_bisect;       /* may be NULL */
  void* user;
} rs_solve_opts;
typedef struct rs_solve_result {
  double naT, nrT, naC, nrC;    /* accepted / rejected inner attempts */
  double nmacro;                /* macro steps taken */
  double nbisect;               /* windows split */
  double nrefresh;              /* refresh calls */
  int32_t status;               /* RS_OK or the status of the window that failed */
  int32_t pad;
} rs_solve_result;
rs_status rs_lie_trotter_solve(rs_handle* h, double t0, double t1, double* dtT, double* dtC,
                               const rs_solve_opts* opts, rs_solve_result* out);

/* Air-mass continuity drift (run_reseact.jl:297-324): r = (m - dp(PS)) / dp(PS) per cell with
 * dp(PS) = dA_k + dB_k PS from the hybrid coefficients and the caller's surface pressure ps
 * [nlat][nlon] at the state's time; out[0] = RMS over interior cells, out[1] = RMS over the
 * lateral wall cells, out[2] = the interior value of largest magnitude. */
rs_status rs_continuity_drift(rs_handle* h, const double* ps, double* out3);
/* The reciprocal the production build's specialised kernels use in place of IEEE division
 * (Newton-Raphson from the hardware approximation; the strict build divides), applied to n
 * host values on the handle's device: a numerics check, r[i] ~ 1/x[i] within a few ulp. */
rs_status rs_chem_kernel_reciprocal(rs_handle* h, const double* x, double* r, size_t n);
rs_status rs_chem_kernel_source(const rs_mechanism* mech, int32_t strict, char* buf,
                                size_t buf_len, size_t* len_out);
rs_status rs_chem_kernel_compile(const rs_mechanism* mech, int32_t strict, char* log,
                                 size_t log_len);

/* Discrete adjoint (tools/adjoint_gradient.jl:609-835; step VJPs rx_traced_integrator.jl:610-623).
 * rs_record(h, 1) clears and starts recording: every rs_macro_step then keeps a device
 * checkpoint of its input state and the accepted (t, dt) of both halves; rs_record(h, 0) stops.
 * rs_adjoint_set_lambda loads dJ/du_end (cell-major); rs_backward_macro_step(h, k) replays
 * recorded step k from its checkpoint with the FIXED step sequence and propagates lambda back
 * through its chemistry steps, then its transport steps (clamp masks applied), accumulating
 * dJ/d(emission) of every chemistry step; call it for k = count-1 ... 0 with the forcing of
 * step k installed (the reference refreshes forcing per checkpoint the same way).  The
 * adjoint differentiates the FP64 scheme; per-cell chemistry cannot be recorded. */
rs_status rs_record(rs_handle* h, int32_t on);
int32_t rs_record_count(const rs_handle* h);
/* Device tape of the recording (no reference counterpart; the reference replays from its
 * checkpoints).  While recording, the forward also stores the state before every accepted
 * step and each macro step's end state; with the specialised chemistry kernels the stage
 * vectors k1, z2 of every accepted chemistry step; and for the FP64 scheme without PBL
 * mixing the stage tendencies and states of every accepted transport step.  The step VJPs
 * read the stages instead of recomputing them.  The three share budget_bytes of device
 * memory in fixed proportions, in arenas reserved by rs_record(h, 1): -1 (the default) for a
 * quarter of the free device memory, 0 for none.  A recorded macro step whose tape is complete is swept back
 * without the replay -- the same bits, since the replay reproduces the forward's states and
 * stages exactly; one that did not fit (or any step, with budget 0) is replayed from its
 * checkpoint.  Takes effect at the next rs_record(h, 1).  rs_record_taped counts the recorded
 * macro steps with a complete tape. */
rs_status rs_set_adjoint_tape(rs_handle* h, int64_t budget_bytes);
int32_t rs_record_taped(const rs_handle* h);
rs_status rs_adjoint_set_lambda(rs_handle* h, const double* lambda, size_t n);
rs_status rs_adjoint_get_lambda(rs_handle* h, double* lambda, size_t n);
rs_status rs_backward_macro_step(rs_handle* h, int32_t k);
/* Frozen-dt replay (replay_fixed, tools/adjoint_gradient.jl:647-669): re-run recorded macro
 * step k on the resident state with its recorded accepted (t, dt) sequence of both halves
 * (every step accepted, the clamp as recorded) and the forcing installed now -- the map
 * whose derivative the discrete adjoint computes.  Central differences of a chain of these
 * replays from a perturbed input check the adjoint (the reference's fdtape stage,
 * tools/adjoint_gradient.jl:116-132).  FP64 global-dt handles only (RS_ERR_UNSUPPORTED). */
rs_status rs_replay_macro_step(rs_handle* h, int32_t k);
/* dJ/d(emission) accumulated so far, [n_species][nlev][nlat][nlon] (grid order) */
rs_status rs_adjoint_get_grad_emission(rs_handle* h, double* grad, size_t n);
rs_status rs_adjoint_reset_grad(rs_handle* h);

/* One unclamped Rosenbrock23 attempt of step dt over all cells, reading d_u_in and writing
 * d_u_out (DEVICE pointers, the grid-SoA layout of rs_state_device_ptr, n = the handle's
 * state size), returning the hairer error estimate in *eest (host pointer, may be NULL).
 * No counterpart in the reference.  It allocates nothing, for callers that cannot allocate
 * device memory when they step (a host whose own memory pool owns the device, or a loop that
 * must not synchronise on an allocation): its scratch is a 524,800-byte array fixed in the
 * library, whose device address rs_create resolves for the handle's device (rs_create fails
 * if it cannot).  Limit: 16,777,216 cells (RS_ERR_INVALID beyond).
 * Ordering: the attempt runs on the handle's stream (rs_stream).  d_u_in must be complete on
 * the device before the call -- synchronise the stream that wrote it, or make rs_stream wait
 * on an event recorded after the write; the call returns after the handle's stream has
 * finished, so d_u_out and *eest are ready on return.  The first call after a forcing change
 * of temperature or pressure also launches the rate-constant kernel on that stream (into the
 * handle's own buffers, allocated at rs_create).  All calls share the scratch, so calls that
 * overlap on the GPU (other threads or streams) race; serialise them.  After cudaDeviceReset
 * the library must be reloaded before this entry point is used again. */
rs_status rs_ros23_attempt_noalloc(rs_handle* h, double dt, const double* d_u_in,
                                   double* d_u_out, double* eest);

/* Per-kernel launch statistics, collected while profiling is on. */
rs_status rs_set_profiling(rs_handle* h, int32_t on);
/* names: ';'-separated kernel family names written into buf (size buf_len); counts and
 * milliseconds per family into the arrays (length max_kernels).  Returns the family count
 * in *n_out. */
rs_status rs_get_profile(rs_handle* h, char* buf, size_t buf_len, double* launches,
                         double* total_ms, int32_t max_kernels, int32_t* n_out);
rs_status rs_reset_profile(rs_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* RESEACT_GB300_H */
