// rs_device.cuh -- device-side building blocks shared by the chemistry and transport kernels.
//
// Arithmetic order contract: every floating-point expression below associates exactly like the
// CPU restatement of the reference (ROS23 rx_traced_integrator.jl:279-349, blocksolve :110-135,
// SSPRK43 :362-400, hairer norm :329-347), so the strict build (--fmad=false, RS_STRICT)
// reproduces it bit for bit given the same rate constants; the fast build differs only by FMA
// contraction, by multiplying with precomputed reciprocals where the reference divides, and by
// the LU elimination order (minimum fill instead of natural; the same solution to roundoff).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#ifndef RS_STRICT
#define RS_STRICT 0
#endif

namespace rs {

constexpr int kRedThreads = 256;  // fixed reduction chunk (cells per level-1 partial)

// Step sizes of the per-cell adaptive form are rounded down to 4 fraction bits (16 sizes per
// octave).  The per-cell controller alone decides each cell's step sequence, and on stiff
// mechanisms a roundoff-sized input change flips some cells' accept / reject decisions and moves
// them by up to the integration tolerance (a 1-ulp change of dt0 moves ~0.4 % of the C3 cells
// by more than 1e-6 relative).  On the lattice a sequence changes only where a proposal lies
// within the perturbation of a lattice point, at the price of ~3 % more steps.  The global-dt
// (reference) controller is not rounded.
__host__ __device__ inline double quant_dt(double d) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(__double_as_longlong(d) & ~((1ll << 48) - 1));
#else
  unsigned long long b;
  __builtin_memcpy(&b, &d, sizeof b);
  b &= ~((1ull << 48) - 1);
  __builtin_memcpy(&d, &b, sizeof b);
  return d;
#endif
}

// ------------------------------------------------------------------ mechanism tables
// Derived on the host from rs_mechanism (derive_tables in rs_api.cu); all index arrays are warp-uniform
// reads (every thread walks the same table), served by the L1/texture path.
struct DevMech {
  int ns, nr, nlu, npart, njac;
  const int* rptr;      // [nr+1] reactant entries of reaction r
  const int* rsp;       // reactant species
  const int* rnu;       // reactant stoichiometry
  const int* rhs_ptr;   // [ns+1] RHS terms of species s (reactions ascending)
  const int* rhs_r;
  const double* rhs_c;
  const int* part_r;    // partial p = d v_{part_r} / d x_{part_q}
  const int* part_q;
  const int* part_e;    // reactant entry index of the partial
  const int* jac_ptr;   // [njac+1] terms of Jacobian entry e
  const int* jac_slot;  // LU slot of entry e
  const int* jac_diag;  // 1 if entry e is on the diagonal
  const int* jac_part;
  const double* jac_coef;
  const int* lu_diag;   // [ns] slot of pivot k (elimination position k)
  const int* ord;       // [ns] species eliminated at position k (identity: natural order)
  const int* elim_ptr;  // [ns+1] per pivot k: range of (i,k) multipliers
  const int* elim_lik;  // slot of (i,k)
  const int* upd_ptr;   // [n_elim+1] per multiplier: range of updates
  const int* upd_dst;
  const int* upd_src;
  const int* low_ptr;   // [ns+1] forward solve, pivot column k: rows after k
  const int* low_row;   //   (species index of the row)
  const int* low_slot;
  const int* up_ptr;    // [ns+1] backward solve, pivot row i: columns after i ascending
  const int* up_col;    //   (species index of the column)
  const int* up_slot;
  const int* pupd_ptr;  // [ns+1] updates of pivot k (ranges of upd_dst / upd_src)
  const int* upd_lik;   // multiplier slot (i,k) of each update
  const int* upc_ptr;   // [ns+1] upper factor by columns: column j's entries (rows i < j)
  const int* upc_row;   //   (species index of the row)
  const int* upc_slot;
  const int* prog_ptr;  // rate programs
  const int* prog_op;
  const double* prog_val;
  const double* params;
  int combinatoric;     // 1: divide k by prod(nu!) (entry by entry, as the oracle does)
  double ros_d;         // ROS23 d = 1/(2+sqrt(2))  (rx_traced_integrator.jl:256)
  double ros_c32;       // ROS23 c32 = 6+sqrt(2)    (rx_traced_integrator.jl:257)
};

// ------------------------------------------------------------------ controller state
// One per adaptive solve, resident in device memory: the host launches attempts, the
// finalize kernel applies the PI controller (rx_traced_integrator.jl:480-505) and raises
// `done`; every attempt kernel returns immediately once `done` is set.
struct Ctl {
  double t, dt, tend, qold, nacc, nrej, iters, dtc, eest, maxiters;
  double beta1, beta2, invqmin, invqmax, gamma, qsmin, qsmax, qoldinit;
  double ntot;     // number of states in the norm
  double omega;    // flux time factor g(t) = cos(omega t)
  double g[4];     // SSPRK43 stage factors of the next attempt: t, t+dt/2, t+dt, t+dt/2
  double dto2, dto6, dtgamma;  // dtc/2, dtc/6, dtc*d of the next attempt (shared by all cells)
  double ros_d;    // ROS23 d, for dtgamma
  double* seq;     // if set: accepted (t, dt) pairs are appended here (adjoint recording)
  int* nseq;
  int seqcap;
  int cur;         // state buffer holding the accepted state (0/1)
  int done;
  int accept;
  int pad;
  // if set: the state before each accepted step is copied to tape + k * n, k the accepted
  // count, while k < tapecap (adjoint tape); ntape[0] counts stored states, ntape[1] is raised
  // when a step found no slot
  double* tape;
  int* ntape;
  int tapecap;
  int pad2;
  // if set (specialised chemistry kernels): every attempt writes its stage vectors k1 and z2
  // (the second solve's result before k1 is added), [2][ns][n] doubles, to kz + slot * 2 ns n
  // with slot = the accepted count, while slot < kzcap -- the adjoint's stage tape
  double* kz;
  int kzcap;
  int pad3;
  // if set (transport, FP64 scheme without PBL mixing): every attempt's stage kernels write
  // the stage tendencies F0..F3 and the stage states V1, V2, V4 ([7][nsp][nc] doubles) to
  // ftape + slot * 7 nsp nc, slot = the accepted count, while slot < fcap -- the transport
  // stage tape
  double* ftape;
  int fcap;
  int pad4;
};

__device__ __forceinline__ double ld(const double* p) { return __ldg(p); }
__device__ __forceinline__ int ldi(const int* p) { return __ldg(p); }

// Reciprocal from the hardware approximation r (PTX rcp.approx.ftz.f64) by one third-order
// correction: with e = 1 - d r, 1/d = r / (1 - e) = r (1 + e + e^2 + ...), so r (1 + e + e^2)
// leaves e^3 -- below an ulp for the approximation's |e| -- in three FMAs (two Newton steps
// take four).  The production build uses it where d > 0 and normal (LU pivots, m, error-norm
// denominators >= atol).
__device__ __forceinline__ double rcp_nr(double d) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  const double e = fma(-d, r, 1.0);
  return fma(r, fma(e, e, e), r);
}

// One Newton step (relative error ~1e-12 or better) and max(|a|, |b|) on the magnitude bits:
// the production build's forms for error-norm terms, whose only use is the step-size controller.
__device__ __forceinline__ double rcp_nr1(double d) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  return fma(r, fma(-d, r, 1.0), r);
}
__device__ __forceinline__ double amax_bits(double a, double b) {  // on 32-bit halves
  const unsigned ha = (unsigned)__double2hiint(a) & 0x7fffffffu, la = (unsigned)__double2loint(a);
  const unsigned hb = (unsigned)__double2hiint(b) & 0x7fffffffu, lb = (unsigned)__double2loint(b);
  const bool bl = ha < hb || (ha == hb && la < lb);
  return __hiloint2double((int)(bl ? hb : ha), (int)(bl ? lb : la));
}

// ------------------------------------------------------------------ chemistry core
// v_r = k_r * prod x^nu over the reactant entries, in table order
__device__ __forceinline__ void velocities(const DevMech& M, const double* k, const double* x,
                                           double* v) {
  for (int r = 0; r < M.nr; ++r) {
    double a = k[r];
    int e1 = ldi(M.rptr + r + 1);
    for (int e = ldi(M.rptr + r); e < e1; ++e) {
      double xs = x[ldi(M.rsp + e)];
      int nu = ldi(M.rnu + e);
      for (int t = 0; t < nu; ++t) a = a * xs;
    }
    v[r] = a;
  }
}

// f_s = sum_r net[r,s] v_r (+ emission)
__device__ __forceinline__ void rhs_from_v(const DevMech& M, const double* v, const double* emis,
                                           double* f) {
  for (int s = 0; s < M.ns; ++s) {
    double acc = 0.0;
    int e1 = ldi(M.rhs_ptr + s + 1);
    for (int e = ldi(M.rhs_ptr + s); e < e1; ++e) acc = acc + ld(M.rhs_c + e) * v[ldi(M.rhs_r + e)];
    f[s] = emis ? acc + emis[s] : acc;
  }
}

// partial derivatives d v_r / d x_q
__device__ __forceinline__ void partials(const DevMech& M, const double* k, const double* x,
                                         double* P) {
  for (int p = 0; p < M.npart; ++p) {
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

// W = I - dtgamma * J on the LU fill pattern (W[r,s] = (r==s ? 1.0 : 0.0) - dtgamma*J[r,s])
__device__ __forceinline__ void build_w(const DevMech& M, const double* P, double dtgamma,
                                        double* W) {
  for (int e = 0; e < M.nlu; ++e) W[e] = 0.0;
  for (int i = 0; i < M.ns; ++i) W[ldi(M.lu_diag + i)] = 1.0;
  for (int e = 0; e < M.njac; ++e) {
    double acc = 0.0;
    int t1 = ldi(M.jac_ptr + e + 1);
    for (int t = ldi(M.jac_ptr + e); t < t1; ++t)
      acc = acc + ld(M.jac_coef + t) * P[ldi(M.jac_part + t)];
    double tmp = dtgamma * acc;
    W[ldi(M.jac_slot + e)] = (ldi(M.jac_diag + e) ? 1.0 : 0.0) - tmp;
  }
}

// Pivot-free sparse LU in elimination order (natural, as blocksolve, in the strict build; zero
// updates skipped); L multipliers overwrite their slots, piv[k] = 1 / U[k,k] for pivot k (the
// production build's reciprocal rcp_nr).
__device__ __forceinline__ void lu_factor(const DevMech& M, double* W, double* piv) {
  int m = 0;
  for (int k = 0; k < M.ns; ++k) {
#if RS_STRICT
    double pk = 1.0 / W[ldi(M.lu_diag + k)];
#else
    double pk = rcp_nr(W[ldi(M.lu_diag + k)]);  // within 2 ulp of 1/U_kk
#endif
    piv[k] = pk;
    int i1 = ldi(M.elim_ptr + k + 1);
    for (int ii = ldi(M.elim_ptr + k); ii < i1; ++ii, ++m) {
      int sl = ldi(M.elim_lik + ii);
      double mult = W[sl] * pk;
      int u1 = ldi(M.upd_ptr + m + 1);
      for (int u = ldi(M.upd_ptr + m); u < u1; ++u) {
        int dst = ldi(M.upd_dst + u);
        double mw = mult * W[ldi(M.upd_src + u)];
        W[dst] = W[dst] - mw;
      }
      W[sl] = mult;
    }
  }
}

// Solve (LU) x = b in place (b -> x, indexed by species): forward replay of the multipliers
// in elimination order, then back substitution x_i = (b_i - sum_{j after i} U_ij x_j) / U_ii.
__device__ __forceinline__ void lu_solve(const DevMech& M, const double* W, const double* piv,
                                         double* b) {
  for (int k = 0; k < M.ns; ++k) {
    double bk = b[ldi(M.ord + k)];
    int e1 = ldi(M.low_ptr + k + 1);
    for (int e = ldi(M.low_ptr + k); e < e1; ++e) {
      int i = ldi(M.low_row + e);
      double mb = W[ldi(M.low_slot + e)] * bk;
      b[i] = b[i] - mb;
    }
  }
  for (int i = M.ns - 1; i >= 0; --i) {
    const int si = ldi(M.ord + i);
    double acc = b[si];
    int e1 = ldi(M.up_ptr + i + 1);
    for (int e = ldi(M.up_ptr + i); e < e1; ++e) {
      double wx = W[ldi(M.up_slot + e)] * b[ldi(M.up_col + e)];
      acc = acc - wx;
    }
#if RS_STRICT
    b[si] = acc / W[ldi(M.lu_diag + i)];
#else
    b[si] = acc * piv[i];
#endif
  }
}

// ------------------------------------------------------------------ integer-pipe FP64 helpers
// Sign tests, magnitude compares and selects of doubles on their bit patterns (the integer
// pipes; FP64 issues at ~2 lanes per SM per clock on this GPU).
// d0, d1 nonzero with equal signs: d1*d0 > 0 unless the product underflows
__device__ __forceinline__ bool sgn_same_nz(double a, double b) {
  const int ha = __double2hiint(a), hb = __double2hiint(b);
  const bool nza = ((ha & 0x7fffffff) | __double2loint(a)) != 0;
  const bool nzb = ((hb & 0x7fffffff) | __double2loint(b)) != 0;
  return ((ha ^ hb) >= 0) & nza & nzb;
}
constexpr long long kMagMask = 0x7fffffffffffffffLL, kSignBit = (long long)0x8000000000000000ULL,
                    kExpOne = 1LL << 52;
__device__ __forceinline__ double sel_d(bool c, double x, double y) {
  return __longlong_as_double(c ? __double_as_longlong(x) : __double_as_longlong(y));
}
// |x| < |y| for magnitude bit patterns given as (hi & 0x7fffffff, lo) halves.  The integer
// helpers work on 32-bit halves: 64-bit masks of reinterpreted doubles were partly emitted as
// FP64 instructions.
__device__ __forceinline__ bool mag_lt(unsigned h0, unsigned l0, unsigned h1, unsigned l1) {
  return h0 < h1 || (h0 == h1 && l0 < l1);
}
// Biased exponent field of x (0 for zero and subnormals).
__device__ __forceinline__ int bexp(double x) { return (__double2hiint(x) >> 20) & 0x7ff; }
__device__ __forceinline__ bool is_zero_d(double x) {
  return ((__double2hiint(x) & 0x7fffffff) | __double2loint(x)) == 0;
}
// The integer forms reproduce the FP forms' products d0*d1 only while those cannot underflow:
// for nonzero normal d0, d1 the product is >= 2^(e0 + e1 - 2046), nonzero when e0 + e1 >= 972.
// Where a product could underflow (or an operand is subnormal) the FP form decides instead.
__device__ __forceinline__ bool prod_may_underflow(double d0, double d1) {
  if (is_zero_d(d0) || is_zero_d(d1)) return false;  // exact zero either way
  const int e0 = bexp(d0), e1 = bexp(d1);
  return e0 == 0 || e1 == 0 || e0 + e1 < 980;
}
// Any nonzero difference of doubles >= 2^-484 in magnitude (or zero) is >= 2^-537, so
// products of two such differences do not underflow; tiny operands use the FP form.
__device__ __forceinline__ bool tiny_operand(double x) {
  return !is_zero_d(x) && bexp(x) < 539;
}
// Order-preserving integer key of a finite double (-0 and +0 both map to 0, key(-x) = -key(x)):
// the sign of the rounded difference x - y is the sign of key(x) - key(y) (gradual underflow
// makes x - y == 0 exactly when x == y), so the limiter's sign tests need no subtraction.
__device__ __forceinline__ long long ord_key(double x) {
  const long long b = __double_as_longlong(x);
  const long long sgn = b >> 63;  // 0 or -1
  return (b ^ (sgn & kMagMask)) - sgn;
}

// ------------------------------------------------------------------ fixed-tree reductions
// Pairwise tree over 256 lanes: v[t] += v[t+s] for s = 128 ... 1 (identical to the CPU
// restatement's tree256).  Returns the total in thread 0.
__device__ __forceinline__ double block_tree256(double v, double* sm) {
  int t = threadIdx.x;
  sm[t] = v;
  __syncthreads();
  for (int s = 128; s >= 32; s >>= 1) {
    if (t < s) sm[t] = sm[t] + sm[t + s];
    __syncthreads();
  }
  double a = sm[t];
  if (t < 32) {
    for (int s = 16; s > 0; s >>= 1) {
      double o = __shfl_down_sync(0xffffffffu, a, s);
      if (t < s) a = a + o;
    }
  }
  __syncthreads();
  return a;
}

}  // namespace rs
