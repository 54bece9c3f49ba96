// rs_chem.cu -- chemistry kernels: per-cell rate constants, the Rosenbrock23 attempt on the
// block-diagonal Jacobian (one thread per grid cell), single-evaluation hooks, and the
// persistent per-cell adaptive kernel fed by a device work queue.
//
// GB300 design note: FP64 issues at ~2 lane-ops per clock per SM on this part (measured
// 1.19 TFLOP/s vs 74 TFLOP/s FP32), so chemistry is FP64-issue bound.  One thread per cell
// walking the mechanism's sparse tables executes only the structurally nonzero FP64 work
// (82-slot LU for SuperFast instead of 144 dense, no idle lanes); index and load traffic rides
// the otherwise idle integer/LSU pipes.  Reference algorithm: ros23_step,
// tools/reactant_handoff/rx_traced_integrator.jl:279-349.
#include <cuda_runtime.h>

#include "rs_device.cuh"
#include "rs_jit.h"
#include "rs_kernels.h"

namespace rs {

// ------------------------------------------------------------------ rate constants
__global__ void k_rates(DevMech M, int nc, const double* __restrict__ T,
                        const double* __restrict__ P, double* __restrict__ krates) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double Tc = T ? T[c] : 298.0, Pc = P ? P[c] : 101325.0;
  double st[kMaxProgStack];
  for (int r = 0; r < M.nr; ++r) {
    int sp = 0;
    int e1 = ldi(M.prog_ptr + r + 1);
    for (int e = ldi(M.prog_ptr + r); e < e1; ++e) {
      int op = ldi(M.prog_op + e);
      double v = ld(M.prog_val + e);
      switch (op) {
        case 0: st[sp++] = v; break;
        case 1: st[sp++] = Tc; break;
        case 2: st[sp++] = Pc; break;
        case 3: st[sp++] = ld(M.params + (int)v); break;
        case 10: --sp; st[sp - 1] = st[sp - 1] + st[sp]; break;
        case 11: --sp; st[sp - 1] = st[sp - 1] - st[sp]; break;
        case 12: --sp; st[sp - 1] = st[sp - 1] * st[sp]; break;
        case 13: --sp; st[sp - 1] = st[sp - 1] / st[sp]; break;
        case 14: --sp; st[sp - 1] = pow(st[sp - 1], st[sp]); break;
        case 15: st[sp - 1] = -st[sp - 1]; break;
        case 20: st[sp - 1] = exp(st[sp - 1]); break;
        case 21: st[sp - 1] = log(st[sp - 1]); break;
        case 22: st[sp - 1] = log10(st[sp - 1]); break;
        case 23: st[sp - 1] = sqrt(st[sp - 1]); break;
        default: st[0] = __longlong_as_double(0x7ff8000000000000ULL); sp = 1; e = e1; break;
      }
    }
    double k = st[0];
    if (M.combinatoric) {
      int q1 = ldi(M.rptr + r + 1);
      for (int q = ldi(M.rptr + r); q < q1; ++q) {
        double f = 1.0;
        for (int t = 2; t <= ldi(M.rnu + q); ++t) f *= t;
        if (f != 1.0) k = k * (1.0 / f);
      }
    }
    krates[(size_t)r * nc + c] = k;
  }
}

// ------------------------------------------------------------------ one ROS23 attempt
// Per-cell work arrays live in thread-local memory (L1-resident at the occupancy used).
template <int MS, int MR, int MLU, int MP>
struct RosWork {
  double x[MS], f0[MS], k1[MS], f1[MS], k2[MS], xn[MS], b[MS], piv[MS], em[MS], f2[MS];
  double kc[MR], v[MR], P[MP], W[MLU];
};

// A scaled error term ut / (max(|x|, |xn|) rtol + atol); the production build multiplies by a
// one-Newton-step reciprocal and takes the magnitude max on the bit patterns (the norm only
// steers the controller), the strict build divides as the reference does.
__device__ __forceinline__ double norm_term(double ut, double x, double xn, double rtol,
                                            double atol) {
#if RS_STRICT
  double am = fmax(fabs(x), fabs(xn));
  double den = am * rtol + atol;
  return ut / den;
#else
  return ut * rcp_nr1(fma(amax_bits(x, xn), rtol, atol));  // den >= atol > 0
#endif
}

// One attempt for one cell from x with step dt: xn (unclamped) and the cell's sum of squared
// scaled errors over its chemistry species (the inert air-mass row contributes 0).  have_f0:
// w.f0 already holds f(x); have_p: w.P already holds the partials at x (the per-cell loop
// after a rejected attempt, or after an accepted one whose clamp left the candidate as it
// was: f(x) is then the attempt's f2) -- the same bits as evaluating them again.
struct StepScalars {
  double dt, dto2, dto6, dtgamma;
};
__device__ __forceinline__ StepScalars step_scalars(const DevMech& M, double dt) {
  return StepScalars{dt, dt / 2, dt / 6, dt * M.ros_d};
}

template <int MS, int MR, int MLU, int MP>
__device__ __forceinline__ double ros23_cell(const DevMech& M, RosWork<MS, MR, MLU, MP>& w,
                                             const double* emis, const StepScalars& h,
                                             double rtol, double atol, bool have_f0 = false,
                                             bool have_p = false) {
  const int n = M.ns;
  const double dt = h.dt;
  if (!have_f0) {
    velocities(M, w.kc, w.x, w.v);
    rhs_from_v(M, w.v, emis, w.f0);
  }
  if (!have_p) partials(M, w.kc, w.x, w.P);
  build_w(M, w.P, h.dtgamma, w.W);
  lu_factor(M, w.W, w.piv);
  for (int s = 0; s < n; ++s) w.k1[s] = w.f0[s];
  lu_solve(M, w.W, w.piv, w.k1);  // k1 = W \ f0
  for (int s = 0; s < n; ++s) w.xn[s] = w.x[s] + h.dto2 * w.k1[s];  // u1
  velocities(M, w.kc, w.xn, w.v);
  rhs_from_v(M, w.v, emis, w.f1);  // f1 = f(u1)
  for (int s = 0; s < n; ++s) w.k2[s] = w.f1[s] - w.k1[s];
  lu_solve(M, w.W, w.piv, w.k2);
  for (int s = 0; s < n; ++s) w.k2[s] = w.k2[s] + w.k1[s];  // k2 = W\(f1-k1) + k1
  for (int s = 0; s < n; ++s) w.xn[s] = w.x[s] + dt * w.k2[s];  // unew
  velocities(M, w.kc, w.xn, w.v);
  rhs_from_v(M, w.v, emis, w.f2);  // f2 = f(unew)
  for (int s = 0; s < n; ++s) {
    double a = M.ros_c32 * (w.k2[s] - w.f1[s]);
    double c = 2.0 * (w.k1[s] - w.f0[s]);
    w.b[s] = (w.f2[s] - a) - c;
  }
  lu_solve(M, w.W, w.piv, w.b);  // k3
  double acc = 0.0;
  for (int s = 0; s < n; ++s) {
    double ut = h.dto6 * ((w.k1[s] - 2.0 * w.k2[s]) + w.b[s]);
    double at = norm_term(ut, w.x[s], w.xn[s], rtol, atol);
    acc = acc + at * at;
  }
  return acc;
}

// Global-dt attempt (reference mode): every cell steps with the controller's dtc; block
// partial sums of the error norm over 256-cell chunks (fixed tree).  Input state U[cur],
// candidate (clamped) into U[cur^1].
template <int MS, int MR, int MLU, int MP>
__global__ void __launch_bounds__(256) k_ros23_attempt(
    DevMech M, int nc, int nsp, const Ctl* __restrict__ ctl, double* __restrict__ U0,
    double* __restrict__ U1, const double* __restrict__ krates,
    const double* __restrict__ emission, double* __restrict__ partial, double rtol,
    double atol, int clamp) {
  __shared__ double sm[kRedThreads];
  if (ctl->done) return;
  const StepScalars hs{ctl->dtc, ctl->dto2, ctl->dto6, ctl->dtgamma};
  const int cur = ctl->cur;
  const double* U = cur ? U1 : U0;
  double* Un = cur ? U0 : U1;
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (c < nc) {
    RosWork<MS, MR, MLU, MP> w;
    for (int s = 0; s < M.ns; ++s) w.x[s] = U[(size_t)s * nc + c];
    for (int r = 0; r < M.nr; ++r) w.kc[r] = krates[(size_t)r * nc + c];
    const double* em = nullptr;
    if (emission) {
      for (int s = 0; s < M.ns; ++s) w.em[s] = emission[(size_t)s * nc + c];
      em = w.em;
    }
    e = ros23_cell(M, w, em, hs, rtol, atol);
    for (int s = 0; s < M.ns; ++s) {
      double xv = w.xn[s];
      Un[(size_t)s * nc + c] = clamp ? fmax(xv, 0.0) : xv;
    }
    for (int s = M.ns; s < nsp; ++s) {  // inert air mass
      double xv = U[(size_t)s * nc + c];
      Un[(size_t)s * nc + c] = clamp ? fmax(xv, 0.0) : xv;
    }
  }
  double tot = block_tree256(e, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// Single-evaluation hooks (rs_rhs_chem, rs_block_jac) on a grid-SoA state.
template <int MS, int MR, int MLU, int MP>
__global__ void k_chem_rhs(DevMech M, int nc, int nsp, const double* __restrict__ U,
                           const double* __restrict__ krates, const double* __restrict__ emission,
                           double* __restrict__ dU) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double x[MS], kc[MR], v[MR], f[MS], em[MS];
  for (int s = 0; s < M.ns; ++s) x[s] = U[(size_t)s * nc + c];
  for (int r = 0; r < M.nr; ++r) kc[r] = krates[(size_t)r * nc + c];
  if (emission)
    for (int s = 0; s < M.ns; ++s) em[s] = emission[(size_t)s * nc + c];
  velocities(M, kc, x, v);
  rhs_from_v(M, v, emission ? em : nullptr, f);
  for (int s = 0; s < M.ns; ++s) dU[(size_t)s * nc + c] = f[s];
  for (int s = M.ns; s < nsp; ++s) dU[(size_t)s * nc + c] = 0.0;
}

// J[c][r][s] over the nsp x nsp block (air-mass row/column zero)
template <int MS, int MR, int MLU, int MP>
__global__ void k_block_jac(DevMech M, int nc, int nsp, const double* __restrict__ U,
                            const double* __restrict__ krates, const int* __restrict__ slot_row,
                            const int* __restrict__ slot_col, double* __restrict__ J) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double x[MS], kc[MR], P[MP];
  for (int s = 0; s < M.ns; ++s) x[s] = U[(size_t)s * nc + c];
  for (int r = 0; r < M.nr; ++r) kc[r] = krates[(size_t)r * nc + c];
  partials(M, kc, x, P);
  double* out = J + (size_t)c * nsp * nsp;
  for (int e = 0; e < nsp * nsp; ++e) out[e] = 0.0;
  for (int e = 0; e < M.njac; ++e) {
    double acc = 0.0;
    int t1 = ldi(M.jac_ptr + e + 1);
    for (int t = ldi(M.jac_ptr + e); t < t1; ++t)
      acc = acc + ld(M.jac_coef + t) * P[ldi(M.jac_part + t)];
    int sl = ldi(M.jac_slot + e);
    out[slot_row[sl] * nsp + slot_col[sl]] = acc;
  }
}

// ------------------------------------------------------------------ per-cell adaptive form
// Persistent kernel: each thread pulls cells from a device work queue and integrates each with
// its own ROS23 + PI controller over [t0, t1] (the reference controller,
// rx_traced_integrator.jl:455-507, applied per cell with the cell's own hairer norm).  Lanes
// of a warp run the same attempt code on different cells, so uneven step counts do not idle
// lanes: a lane whose cell finishes takes the next one from the queue.  Step sizes are rounded
// down to 4 fraction bits (quant_dt), which keeps per-cell trajectories insensitive to
// roundoff-sized input changes.  MINB bounds the registers: 5 blocks of 256 threads (51
// registers, 1280 resident threads per SM) or 8 (32 registers, 2048 threads: more local-memory
// requests in flight for large mechanisms); the same arithmetic.
template <int MS, int MR, int MLU, int MP, int MINB>
__global__ void __launch_bounds__(256, MINB) k_chem_per_cell(
    DevMech M, int nc, int nsp, double* __restrict__ U, const double* __restrict__ krates,
    const double* __restrict__ emission, double* __restrict__ dt_cell,
    double* __restrict__ steps_cell, unsigned long long* __restrict__ queue,
    int* __restrict__ status, PerCellArgs a) {
  RosWork<MS, MR, MLU, MP> w;
  double my_steps = 0.0, my_attempts = 0.0;  // this thread's totals (exact small integers)
  double t = 0, dt = 0, qold = 0, iters = 0, nacc = 0;
  bool have_f0 = false, have_p = false;  // w.f0 == f(x), w.P == partials at x
  int c = -1;
  const double tlim = a.t1 - 1.0e-9;
  for (;;) {
    if (c < 0) {
      unsigned long long nxt = atomicAdd(queue, 1ull);
      if (nxt >= (unsigned long long)nc) break;
      c = (int)nxt;
      for (int s = 0; s < M.ns; ++s) w.x[s] = U[(size_t)s * nc + c];
      for (int r = 0; r < M.nr; ++r) w.kc[r] = krates[(size_t)r * nc + c];
      if (emission)
        for (int s = 0; s < M.ns; ++s) w.em[s] = emission[(size_t)s * nc + c];
      t = a.t0;
      dt = quant_dt(dt_cell[c] > 0.0 ? dt_cell[c] : a.dt0);
      qold = a.qoldinit;
      iters = 0;
      nacc = 0;
      have_f0 = have_p = false;
    }
    if ((t < tlim) && (iters < a.maxiters)) {
      double dtc = fmin(dt, a.t1 - t);
      double sse = ros23_cell(M, w, emission ? w.em : nullptr, step_scalars(M, dtc), a.rtol,
                              a.atol, have_f0, have_p);
      have_f0 = have_p = true;  // for x; replaced below if x moves
      double EEst = sqrt(sse / (double)nsp);
      if (isnan(EEst)) EEst = 1.0e10;
      double q11 = pow(fmax(EEst, 1.0e-35), a.beta1);
      double q = q11 / pow(qold, a.beta2);
      q = fmax(a.invqmax, fmin(a.invqmin, q / a.gamma));
      if (EEst <= 1.0) {
        bool same = true;  // the clamp left the candidate as it was: f(x) is f2
        for (int s = 0; s < M.ns; ++s) {
          const double xs = a.clamp ? fmax(w.xn[s], 0.0) : w.xn[s];
          same = same && (__double_as_longlong(xs) == __double_as_longlong(w.xn[s]));
          w.x[s] = xs;
        }
        if (same)
          for (int s = 0; s < M.ns; ++s) w.f0[s] = w.f2[s];
        have_f0 = same;
        have_p = false;
        t = t + dtc;
        bool insteady = (a.qsmin <= q) && (q <= a.qsmax);
        dt = quant_dt(dtc / (insteady ? 1.0 : q));
        qold = fmax(EEst, a.qoldinit);
        nacc += 1.0;
      } else {
        dt = quant_dt(dtc / fmin(a.invqmin, q11 / a.gamma));
      }
      iters += 1.0;
    } else {
      if (t < tlim) atomicOr(status, 1);
      for (int s = 0; s < M.ns; ++s) U[(size_t)s * nc + c] = w.x[s];
      dt_cell[c] = dt;
      if (steps_cell) steps_cell[c] = nacc;
      my_steps += nacc;
      my_attempts += iters;
      c = -1;
    }
  }
  // integer-valued totals: atomic double adds are exact (far below 2^53), order-free
  if (a.totals) {
    atomicAdd(a.totals, my_steps);
    atomicAdd(a.totals + 1, my_attempts);
  }
}

// ------------------------------------------------------------------ per-cell, G lanes per cell
// The per-cell adaptive form with one cell spread over G lanes (G = 4, 8, 16) and its work
// arrays in shared memory instead of thread-local memory: the lanes split the rate products,
// RHS sums, partials and Jacobian entries, each pivot's multipliers and updates (every update
// of one pivot writes a different slot), each column of the forward solve, and the back
// substitution as a column sweep (descending columns: see the table derivation).  Every value
// is formed by the same operations in the same order as in k_chem_per_cell, so both give the
// same bits; rs_autotune times both.  Scalars that all lanes need (pivot reciprocals, the
// error norm, the controller) are formed redundantly by every lane of the group: this GPU
// charges an FP64 warp instruction the same time whatever the number of active lanes.
// Shared memory per cell (doubles): x, xn, f0, k1, f1, k2, b, em, piv, norm terms, f2 [ns each],
// rate constants [nr], velocities / partials (never live together) [max(nr, npart)], W [nlu].
struct GroupOff {
  int x, xn, f0, k1, f1, k2, b, em, piv, at, f2, kc, pv, w;
};
__device__ __forceinline__ GroupOff group_off(const DevMech& M) {
  const int n = M.ns;
  GroupOff o;
  o.x = 0; o.xn = n; o.f0 = 2 * n; o.k1 = 3 * n; o.f1 = 4 * n; o.k2 = 5 * n; o.b = 6 * n;
  o.em = 7 * n; o.piv = 8 * n; o.at = 9 * n; o.f2 = 10 * n; o.kc = 11 * n; o.pv = 11 * n + M.nr;
  o.w = o.pv + (M.nr > M.npart ? M.nr : M.npart);
  return o;
}

template <int G>
struct Grp {
  int l;        // lane within the group
  unsigned m;   // the group's lanes in the warp
  __device__ __forceinline__ void sync() const { __syncwarp(m); }
};

// v[r] = k_r prod x^nu (velocities), lanes split the reactions
template <int G>
__device__ __forceinline__ void g_velocities(const DevMech& M, const Grp<G>& g, const double* kc,
                                             const double* x, double* v) {
  for (int r = g.l; r < M.nr; r += G) {
    double a = kc[r];
    int e1 = ldi(M.rptr + r + 1);
    for (int e = ldi(M.rptr + r); e < e1; ++e) {
      double xs = x[ldi(M.rsp + e)];
      int nu = ldi(M.rnu + e);
      for (int t = 0; t < nu; ++t) a = a * xs;
    }
    v[r] = a;
  }
}
template <int G>
__device__ __forceinline__ void g_rhs(const DevMech& M, const Grp<G>& g, const double* v,
                                      const double* emis, double* f) {
  for (int s = g.l; s < M.ns; s += G) {
    double acc = 0.0;
    int e1 = ldi(M.rhs_ptr + s + 1);
    for (int e = ldi(M.rhs_ptr + s); e < e1; ++e) acc = acc + ld(M.rhs_c + e) * v[ldi(M.rhs_r + e)];
    f[s] = emis ? acc + emis[s] : acc;
  }
}
template <int G>
__device__ __forceinline__ void g_partials(const DevMech& M, const Grp<G>& g, const double* k,
                                           const double* x, double* P) {
  for (int p = g.l; p < M.npart; p += G) {
    int r = ldi(M.part_r + p), q = ldi(M.part_q + p);
    double d = k[r];
    int e1 = ldi(M.rptr + r + 1);
    for (int e = ldi(M.rptr + r); e < e1; ++e) {
      int s = ldi(M.rsp + e), nu = ldi(M.rnu + e);
      double xs = x[s];
      if (s == q) {
        if (nu >= 2) {
          double f = (double)nu;
          for (int t = 1; t < nu; ++t) f = f * xs;
          d = d * f;
        }
      } else {
        for (int t = 0; t < nu; ++t) d = d * xs;
      }
    }
    P[p] = d;
  }
}
template <int G>
__device__ __forceinline__ void g_build_w(const DevMech& M, const Grp<G>& g, const double* P,
                                          double dtgamma, double* W) {
  for (int e = g.l; e < M.nlu; e += G) W[e] = 0.0;
  g.sync();
  for (int i = g.l; i < M.ns; i += G) W[ldi(M.lu_diag + i)] = 1.0;
  g.sync();
  for (int e = g.l; e < M.njac; e += G) {
    double acc = 0.0;
    int t1 = ldi(M.jac_ptr + e + 1);
    for (int t = ldi(M.jac_ptr + e); t < t1; ++t)
      acc = acc + ld(M.jac_coef + t) * P[ldi(M.jac_part + t)];
    double tmp = dtgamma * acc;
    W[ldi(M.jac_slot + e)] = (ldi(M.jac_diag + e) ? 1.0 : 0.0) - tmp;
  }
  g.sync();
}
template <int G>
__device__ __forceinline__ void g_lu_factor(const DevMech& M, const Grp<G>& g, double* W,
                                            double* piv) {
  for (int k = 0; k < M.ns; ++k) {
#if RS_STRICT
    const double pk = 1.0 / W[ldi(M.lu_diag + k)];
#else
    const double pk = rcp_nr(W[ldi(M.lu_diag + k)]);
#endif
    if (g.l == 0) piv[k] = pk;
    const int i1 = ldi(M.elim_ptr + k + 1);
    for (int ii = ldi(M.elim_ptr + k) + g.l; ii < i1; ii += G) {
      const int sl = ldi(M.elim_lik + ii);
      W[sl] = W[sl] * pk;
    }
    g.sync();
    const int u1 = ldi(M.pupd_ptr + k + 1);
    for (int u = ldi(M.pupd_ptr + k) + g.l; u < u1; u += G) {
      const int dst = ldi(M.upd_dst + u);
      double mw = W[ldi(M.upd_lik + u)] * W[ldi(M.upd_src + u)];
      W[dst] = W[dst] - mw;
    }
    g.sync();
  }
}
// in place b -> x; entry at the group's sync state, leaves synced
template <int G>
__device__ __forceinline__ void g_lu_solve(const DevMech& M, const Grp<G>& g, const double* W,
                                           const double* piv, double* b) {
  for (int k = 0; k < M.ns; ++k) {
    const double bk = b[ldi(M.ord + k)];
    const int e1 = ldi(M.low_ptr + k + 1);
    for (int e = ldi(M.low_ptr + k) + g.l; e < e1; e += G) {
      const int i = ldi(M.low_row + e);
      double mb = W[ldi(M.low_slot + e)] * bk;
      b[i] = b[i] - mb;
    }
    g.sync();
  }
  for (int j = M.ns - 1; j >= 0; --j) {
    const int sj = ldi(M.ord + j);
#if RS_STRICT
    const double xj = b[sj] / W[ldi(M.lu_diag + j)];
#else
    const double xj = b[sj] * piv[j];
#endif
    const int e1 = ldi(M.upc_ptr + j + 1);
    for (int e = ldi(M.upc_ptr + j) + g.l; e < e1; e += G) {
      const int i = ldi(M.upc_row + e);
      double wx = W[ldi(M.upc_slot + e)] * xj;
      b[i] = b[i] - wx;
    }
    g.sync();
    if (g.l == 0) b[sj] = xj;  // nobody reads b[sj] again in this sweep
  }
  g.sync();
}

// One attempt from S[x] with step sizes h: S[xn] (unclamped); returns the sum of squared scaled
// errors (the same value in every lane of the group).
template <int G>
__device__ __forceinline__ double ros23_group(const DevMech& M, const Grp<G>& g, double* S,
                                              const GroupOff& o, bool emis,
                                              const StepScalars& h, double rtol, double atol,
                                              bool have_f0) {
  const int n = M.ns;
  const double dt = h.dt;
  double *x = S + o.x, *xn = S + o.xn, *f0 = S + o.f0, *k1 = S + o.k1, *f1 = S + o.f1,
         *k2 = S + o.k2, *b = S + o.b, *piv = S + o.piv, *at = S + o.at, *f2 = S + o.f2,
         *kc = S + o.kc, *pv = S + o.pv, *W = S + o.w;
  const double* em = emis ? S + o.em : nullptr;
  if (!have_f0) {
    g_velocities(M, g, kc, x, pv);
    g.sync();
    g_rhs(M, g, pv, em, f0);
    g.sync();
  }
  g_partials(M, g, kc, x, pv);
  g.sync();
  g_build_w(M, g, pv, h.dtgamma, W);
  g_lu_factor(M, g, W, piv);
  for (int s = g.l; s < n; s += G) k1[s] = f0[s];
  g.sync();
  g_lu_solve(M, g, W, piv, k1);  // k1 = W \ f0
  for (int s = g.l; s < n; s += G) xn[s] = x[s] + h.dto2 * k1[s];  // u1
  g.sync();
  g_velocities(M, g, kc, xn, pv);
  g.sync();
  g_rhs(M, g, pv, em, f1);  // f1 = f(u1)
  for (int s = g.l; s < n; s += G) k2[s] = f1[s] - k1[s];
  g.sync();
  g_lu_solve(M, g, W, piv, k2);
  for (int s = g.l; s < n; s += G) k2[s] = k2[s] + k1[s];  // k2 = W\(f1-k1) + k1
  for (int s = g.l; s < n; s += G) xn[s] = x[s] + dt * k2[s];  // unew
  g.sync();
  g_velocities(M, g, kc, xn, pv);
  g.sync();
  g_rhs(M, g, pv, em, f2);  // f2 = f(unew)
  for (int s = g.l; s < n; s += G) {
    double a = M.ros_c32 * (k2[s] - f1[s]);
    double c = 2.0 * (k1[s] - f0[s]);
    b[s] = (f2[s] - a) - c;
  }
  g.sync();
  g_lu_solve(M, g, W, piv, b);  // k3
  for (int s = g.l; s < n; s += G) {
    double ut = h.dto6 * ((k1[s] - 2.0 * k2[s]) + b[s]);
    at[s] = norm_term(ut, x[s], xn[s], rtol, atol);
  }
  g.sync();
  double acc = 0.0;
  for (int s = 0; s < n; ++s) {
    const double a = at[s];
    acc = acc + a * a;
  }
  return acc;
}

template <int G>
__global__ void __launch_bounds__(128) k_chem_per_cell_group(
    DevMech M, int nc, int nsp, double* __restrict__ U, const double* __restrict__ krates,
    const double* __restrict__ emission, double* __restrict__ dt_cell,
    double* __restrict__ steps_cell, unsigned long long* __restrict__ queue,
    int* __restrict__ status, PerCellArgs a, int cell_doubles) {
  extern __shared__ double gsm[];
  const int wl = threadIdx.x & 31;
  Grp<G> g;
  g.l = threadIdx.x % G;
  g.m = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (wl & ~(G - 1));
  const int lead = wl & ~(G - 1);
  double* S = gsm + (size_t)(threadIdx.x / G) * cell_doubles;
  const GroupOff o = group_off(M);
  const bool emis = emission != nullptr;
  double my_steps = 0.0, my_attempts = 0.0;
  double t = 0, dt = 0, qold = 0, iters = 0, nacc = 0;
  bool have_f0 = false;  // S[f0] == f(S[x])
  int c = -1;
  const double tlim = a.t1 - 1.0e-9;
  for (;;) {
    if (c < 0) {
      unsigned long long nxt = 0;
      if (g.l == 0) nxt = atomicAdd(queue, 1ull);
      nxt = __shfl_sync(g.m, nxt, lead);
      if (nxt >= (unsigned long long)nc) break;
      c = (int)nxt;
      for (int s = g.l; s < M.ns; s += G) S[o.x + s] = U[(size_t)s * nc + c];
      for (int r = g.l; r < M.nr; r += G) S[o.kc + r] = krates[(size_t)r * nc + c];
      if (emis)
        for (int s = g.l; s < M.ns; s += G) S[o.em + s] = emission[(size_t)s * nc + c];
      g.sync();
      t = a.t0;
      dt = quant_dt(dt_cell[c] > 0.0 ? dt_cell[c] : a.dt0);
      qold = a.qoldinit;
      iters = 0;
      nacc = 0;
      have_f0 = false;
    }
    if ((t < tlim) && (iters < a.maxiters)) {
      double dtc = fmin(dt, a.t1 - t);
      double sse = ros23_group(M, g, S, o, emis, step_scalars(M, dtc), a.rtol, a.atol, have_f0);
      have_f0 = true;
      double EEst = sqrt(sse / (double)nsp);
      if (isnan(EEst)) EEst = 1.0e10;
      double q11 = pow(fmax(EEst, 1.0e-35), a.beta1);
      double q = q11 / pow(qold, a.beta2);
      q = fmax(a.invqmax, fmin(a.invqmin, q / a.gamma));
      if (EEst <= 1.0) {
        bool same = true;  // the clamp left the candidate as it was: f(x) is f2
        for (int s = g.l; s < M.ns; s += G) {
          const double xv = S[o.xn + s];
          const double xs = a.clamp ? fmax(xv, 0.0) : xv;
          same = same && (__double_as_longlong(xs) == __double_as_longlong(xv));
          S[o.x + s] = xs;
        }
        have_f0 = __all_sync(g.m, same);
        if (have_f0)
          for (int s = g.l; s < M.ns; s += G) S[o.f0 + s] = S[o.f2 + s];
        g.sync();
        t = t + dtc;
        bool insteady = (a.qsmin <= q) && (q <= a.qsmax);
        dt = quant_dt(dtc / (insteady ? 1.0 : q));
        qold = fmax(EEst, a.qoldinit);
        nacc += 1.0;
      } else {
        dt = quant_dt(dtc / fmin(a.invqmin, q11 / a.gamma));
      }
      iters += 1.0;
    } else {
      if (g.l == 0 && t < tlim) atomicOr(status, 1);
      for (int s = g.l; s < M.ns; s += G) U[(size_t)s * nc + c] = S[o.x + s];
      if (g.l == 0) {
        dt_cell[c] = dt;
        if (steps_cell) steps_cell[c] = nacc;
        my_steps += nacc;
        my_attempts += iters;
      }
      g.sync();  // the next cell's loads overwrite S
      c = -1;
    }
  }
  if (a.totals && g.l == 0) {
    atomicAdd(a.totals, my_steps);
    atomicAdd(a.totals + 1, my_attempts);
  }
}

// ------------------------------------------------------------------ launch helpers
template <int MS, int MR, int MLU, int MP>
struct ChemLaunch {
  static void attempt(const LaunchCtx& L, const Ctl* ctl, double* U0, double* U1,
                      const double* kr, const double* em, double* part, double rtol,
                      double atol, int clamp) {
    int nb = (L.nc + kRedThreads - 1) / kRedThreads;
    k_ros23_attempt<MS, MR, MLU, MP><<<nb, kRedThreads, 0, L.stream>>>(
        L.mech, L.nc, L.nsp, ctl, U0, U1, kr, em, part, rtol, atol, clamp);
  }
  static void rhs(const LaunchCtx& L, const double* U, const double* kr, const double* em,
                  double* dU) {
    int nb = (L.nc + 127) / 128;
    k_chem_rhs<MS, MR, MLU, MP><<<nb, 128, 0, L.stream>>>(L.mech, L.nc, L.nsp, U, kr, em, dU);
  }
  static void jac(const LaunchCtx& L, const double* U, const double* kr, const int* srow,
                  const int* scol, double* J) {
    int nb = (L.nc + 127) / 128;
    k_block_jac<MS, MR, MLU, MP><<<nb, 128, 0, L.stream>>>(L.mech, L.nc, L.nsp, U, kr, srow,
                                                           scol, J);
  }
  static void per_cell(const LaunchCtx& L, int nblocks, int threads, double* U,
                       const double* kr, const double* em, double* dtc, double* steps,
                       unsigned long long* queue, int* status, const PerCellArgs& a,
                       bool regcap) {
    if (regcap)
      k_chem_per_cell<MS, MR, MLU, MP, 8><<<nblocks, threads, 0, L.stream>>>(
          L.mech, L.nc, L.nsp, U, kr, em, dtc, steps, queue, status, a);
    else
      k_chem_per_cell<MS, MR, MLU, MP, 5><<<nblocks, threads, 0, L.stream>>>(
          L.mech, L.nc, L.nsp, U, kr, em, dtc, steps, queue, status, a);
  }
};

using Small = ChemLaunch<kSmallMS, kSmallMR, kSmallMLU, kSmallMP>;
using Large = ChemLaunch<kLargeMS, kLargeMR, kLargeMLU, kLargeMP>;

void launch_rates(const LaunchCtx& L, const double* T, const double* P, double* kr) {
  int nb = (L.nc + 127) / 128;
  k_rates<<<nb, 128, 0, L.stream>>>(L.mech, L.nc, T, P, kr);
}
void launch_ros23_attempt(const LaunchCtx& L, const Ctl* ctl, double* U0, double* U1,
                          const double* kr, const double* em, double* part, double rtol,
                          double atol, int clamp, double* F0, double* F1) {
  if (L.jit) {
    jit_launch_attempt(*L.jit, L.stream, L.nc, L.nsp, ctl, U0, U1, kr, em, part, rtol, atol,
                       clamp, F0, F1);
    return;
  }
  if (L.size_class == 0) Small::attempt(L, ctl, U0, U1, kr, em, part, rtol, atol, clamp);
  else Large::attempt(L, ctl, U0, U1, kr, em, part, rtol, atol, clamp);
}
void launch_ros23_step(const LaunchCtx& L, const Ctl* ctl, double* U0, double* U1,
                       const double* kr, const double* em, double* part, double rtol,
                       double atol, int clamp) {
  if (L.jit && L.jit->step[em ? 1 : 0]) {
    jit_launch_step(*L.jit, L.stream, L.nc, L.nsp, ctl, U0, U1, kr, em, clamp);
    return;
  }
  launch_ros23_attempt(L, ctl, U0, U1, kr, em, part, rtol, atol, clamp);
}
void launch_chem_rhs(const LaunchCtx& L, const double* U, const double* kr, const double* em,
                     double* dU) {
  if (L.size_class == 0) Small::rhs(L, U, kr, em, dU);
  else Large::rhs(L, U, kr, em, dU);
}
void launch_block_jac(const LaunchCtx& L, const double* U, const double* kr, const int* srow,
                      const int* scol, double* J) {
  if (L.size_class == 0) Small::jac(L, U, kr, srow, scol, J);
  else Large::jac(L, U, kr, srow, scol, J);
}
int group_cell_doubles(const DevMech& M) {
  int d = 11 * M.ns + M.nr + (M.nr > M.npart ? M.nr : M.npart) + M.nlu;
  return d + (d & 1);  // even: 16-byte aligned cells
}
template <int G>
static int group_threads_t(const DevMech& M) {
  int maxdyn = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&maxdyn, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return 0;
  for (int thr : {128, 64, 32})
    if (thr >= G && (size_t)(thr / G) * group_cell_doubles(M) * sizeof(double) <= (size_t)maxdyn)
      return thr;
  return 0;
}
int chem_group_threads(const LaunchCtx& L, int G) {
  switch (G) {
    case 4: return group_threads_t<4>(L.mech);
    case 8: return group_threads_t<8>(L.mech);
    case 16: return group_threads_t<16>(L.mech);
    default: return 0;
  }
}
template <int G>
static int group_occupancy_t(const DevMech& M, int thr) {
  const size_t smem = (size_t)(thr / G) * group_cell_doubles(M) * sizeof(double);
  if (cudaFuncSetAttribute(k_chem_per_cell_group<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_chem_per_cell_group<G>, thr, smem) !=
      cudaSuccess)
    return 0;
  return nb;
}
int chem_group_blocks_per_sm(const LaunchCtx& L, int G, int thr) {
  switch (G) {
    case 4: return group_occupancy_t<4>(L.mech, thr);
    case 8: return group_occupancy_t<8>(L.mech, thr);
    case 16: return group_occupancy_t<16>(L.mech, thr);
    default: return 0;
  }
}
void launch_chem_per_cell_group(const LaunchCtx& L, int G, int nblocks, int thr, double* U,
                                const double* kr, const double* em, double* dtc, double* steps,
                                unsigned long long* queue, int* status, const PerCellArgs& a) {
  const int cd = group_cell_doubles(L.mech);
  const size_t smem = (size_t)(thr / G) * cd * sizeof(double);
#define RS_GROUP_LAUNCH(GG)                                                                    \
  cudaFuncSetAttribute(k_chem_per_cell_group<GG>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                       (int)smem);                                                             \
  k_chem_per_cell_group<GG><<<nblocks, thr, smem, L.stream>>>(L.mech, L.nc, L.nsp, U, kr, em, \
                                                              dtc, steps, queue, status, a, cd)
  switch (G) {
    case 4: RS_GROUP_LAUNCH(4); break;
    case 8: RS_GROUP_LAUNCH(8); break;
    case 16: RS_GROUP_LAUNCH(16); break;
    default: break;
  }
#undef RS_GROUP_LAUNCH
}
void launch_chem_per_cell(const LaunchCtx& L, int nblocks, int threads, double* U,
                          const double* kr, const double* em, double* dtc, double* steps,
                          unsigned long long* queue, int* status, const PerCellArgs& a,
                          bool regcap) {
  if (L.jit) {
    jit_launch_per_cell(*L.jit, L.stream, L.nc, L.nsp, nblocks, threads, U, kr, em, dtc, steps,
                        queue, status, a);
    return;
  }
  if (L.size_class == 0)
    Small::per_cell(L, nblocks, threads, U, kr, em, dtc, steps, queue, status, a, regcap);
  else
    Large::per_cell(L, nblocks, threads, U, kr, em, dtc, steps, queue, status, a, regcap);
}

}  // namespace rs
