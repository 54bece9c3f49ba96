// rs_adjoint.cu -- discrete-adjoint kernels of the split step (K4 transport, K5 chemistry).
//
// One-step VJPs at a fixed, recorded dt: lambda_in = (d u_out / d u_in)^T lambda_out and, for
// chemistry, d J / d emission.  The controller's accept/reject and dt choices and the clamp are
// the discrete decisions the adjoint is taken along (rx_traced_integrator.jl:540-547,
// tools/adjoint_gradient.jl:736).  The exact ROS23 adjoint needs d(J v)/du because W is built
// from J(u); for mass action that Hessian is exact and sparse (only reactant pairs of one
// reaction), which is what replaces the reference's Enzyme second derivative.  PPM limiter
// branches are frozen at the primal: the face value is then linear in its five stencil values
// and its weights are assembled from the linear forms of the same reconstruction.
// Sums are gathered per cell in a fixed order (no atomics): results are deterministic.
#include <cuda_runtime.h>

#include <algorithm>

#include "rs_device.cuh"
#include "rs_jit.h"
#include "rs_kernels.h"

namespace rs {

// ------------------------------------------------------------------ chemistry (K5)
// Sparse transposed solve W^T x = b in place with the factors of lu_factor:
// W^T = U^T L^T; U^T forward (right-looking over the rows of U), then L^T backward.
__device__ __forceinline__ void lu_solve_T(const DevMech& M, const double* W, const double* piv,
                                           double* b) {
  for (int j = 0; j < M.ns; ++j) {
    const int sj = ldi(M.ord + j);
#if RS_STRICT
    double tj = b[sj] / W[ldi(M.lu_diag + j)];
#else
    double tj = b[sj] * piv[j];
#endif
    b[sj] = tj;
    int e1 = ldi(M.up_ptr + j + 1);
    for (int e = ldi(M.up_ptr + j); e < e1; ++e) {
      int i = ldi(M.up_col + e);
      b[i] = b[i] - W[ldi(M.up_slot + e)] * tj;
    }
  }
  for (int k = M.ns - 1; k >= 0; --k) {
    const int sk = ldi(M.ord + k);
    double acc = b[sk];
    int e1 = ldi(M.low_ptr + k + 1);
    for (int e = ldi(M.low_ptr + k); e < e1; ++e)
      acc = acc - W[ldi(M.low_slot + e)] * b[ldi(M.low_row + e)];
    b[sk] = acc;
  }
}

// a_r = sum_s net[r,s] y_s (through the per-species RHS term lists)
template <int MR>
__device__ __forceinline__ void reaction_sums(const DevMech& M, const double* y, double* a) {
  for (int r = 0; r < M.nr; ++r) a[r] = 0.0;
  for (int s = 0; s < M.ns; ++s) {
    double ys = y[s];
    int e1 = ldi(M.rhs_ptr + s + 1);
    for (int e = ldi(M.rhs_ptr + s); e < e1; ++e) {
      int r = ldi(M.rhs_r + e);
      a[r] = a[r] + ld(M.rhs_c + e) * ys;
    }
  }
}

// out += J(x)^T y  given the partials P at x (P[p] = d v_{r_p} / d x_{q_p})
template <int MR>
__device__ __forceinline__ void jt_apply(const DevMech& M, const double* P, const double* y,
                                         double* a, double* out) {
  reaction_sums<MR>(M, y, a);
  for (int p = 0; p < M.npart; ++p) {
    int r = ldi(M.part_r + p), q = ldi(M.part_q + p);
    out[q] = out[q] + a[r] * P[p];
  }
}

// d^2 v_r / dx_a dx_b
__device__ __forceinline__ double d2vel(const DevMech& M, int r, double k, const double* x, int a,
                                        int b) {
  double d = k;
  int e1 = ldi(M.rptr + r + 1);
  for (int e = ldi(M.rptr + r); e < e1; ++e) {
    int s = ldi(M.rsp + e), nu = ldi(M.rnu + e);
    int order = (s == a) + (s == b);
    if (order > nu) return 0.0;
    double c = 1.0;
    for (int t = 0; t < order; ++t) c *= (double)(nu - t);
    for (int t = 0; t < nu - order; ++t) c *= x[s];
    d *= c;
  }
  return d;
}

template <int MS, int MR, int MLU, int MP>
struct VjpWork {
  double x[MS], f0[MS], k1[MS], u1[MS], f1[MS], z2[MS], bb[MS], f0b[MS], f1b[MS], ub[MS],
      piv[MS], em[MS];
  double kc[MR], v[MR], a0[MR], a1[MR], P[MP], P1[MP], W[MLU];
};

template <int MS, int MR, int MLU, int MP>
__global__ void __launch_bounds__(128) k_ros23_vjp(
    DevMech M, int nc, int nsp, const double* __restrict__ U, const double* __restrict__ Uout,
    const double* __restrict__ lam, double* __restrict__ lam_out,
    const double* __restrict__ krates, const double* __restrict__ emission,
    double* __restrict__ ebar, double dt, int clamp) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  VjpWork<MS, MR, MLU, MP> w;
  const int n = M.ns;
  const double dto2 = dt / 2, dtgamma = dt * M.ros_d;
  for (int s = 0; s < n; ++s) w.x[s] = U[(size_t)s * nc + c];
  for (int r = 0; r < M.nr; ++r) w.kc[r] = krates[(size_t)r * nc + c];
  const double* em = nullptr;
  if (emission) {
    for (int s = 0; s < n; ++s) w.em[s] = emission[(size_t)s * nc + c];
    em = w.em;
  }
  // ---- forward recompute (the live part of ros23: unew = u + dt k2)
  velocities(M, w.kc, w.x, w.v);
  rhs_from_v(M, w.v, em, w.f0);
  partials(M, w.kc, w.x, w.P);
  build_w(M, w.P, dtgamma, w.W);
  lu_factor(M, w.W, w.piv);
  for (int s = 0; s < n; ++s) w.k1[s] = w.f0[s];
  lu_solve(M, w.W, w.piv, w.k1);
  for (int s = 0; s < n; ++s) w.u1[s] = w.x[s] + dto2 * w.k1[s];
  velocities(M, w.kc, w.u1, w.v);
  rhs_from_v(M, w.v, em, w.f1);
  partials(M, w.kc, w.u1, w.P1);
  for (int s = 0; s < n; ++s) w.z2[s] = w.f1[s] - w.k1[s];
  lu_solve(M, w.W, w.piv, w.z2);
  // ---- backward; lambda masked by the clamp of this step's output
  for (int s = 0; s < n; ++s) {
    double l = lam[(size_t)s * nc + c];
    if (clamp && Uout && !(Uout[(size_t)s * nc + c] > 0.0)) l = 0.0;
    w.ub[s] = l;
    w.bb[s] = dt * l;  // k2bar
  }
  lu_solve_T(M, w.W, w.piv, w.bb);  // b2bar = W^-T k2bar
  for (int s = 0; s < n; ++s) {
    w.f1b[s] = w.bb[s];
    w.f0b[s] = dt * w.ub[s] - w.bb[s];  // k1bar = k2bar - b2bar (held in f0b)
  }
  for (int s = 0; s < n; ++s) w.u1[s] = 0.0;  // u1bar = J(u1)^T f1bar
  jt_apply<MR>(M, w.P1, w.f1b, w.a0, w.u1);
  for (int s = 0; s < n; ++s) {
    w.ub[s] = w.ub[s] + w.u1[s];
    w.f0b[s] = w.f0b[s] + dto2 * w.u1[s];
  }
  lu_solve_T(M, w.W, w.piv, w.f0b);  // f0bar = W^-T k1bar
  jt_apply<MR>(M, w.P, w.f0b, w.a0, w.ub);
  // Hessian term: Jbar_ij = dtgamma (b2bar_i z2_j + f0bar_i k1_j)
  reaction_sums<MR>(M, w.bb, w.a1);
  reaction_sums<MR>(M, w.f0b, w.a0);
  for (int r = 0; r < M.nr; ++r) {
    int e1 = ldi(M.rptr + r + 1);
    for (int ea = ldi(M.rptr + r); ea < e1; ++ea) {
      int j = ldi(M.rsp + ea);
      double gj = dtgamma * (w.a1[r] * w.z2[j] + w.a0[r] * w.k1[j]);
      if (gj == 0.0) continue;
      for (int eb = ldi(M.rptr + r); eb < e1; ++eb) {
        int q = ldi(M.rsp + eb);
        w.ub[q] = w.ub[q] + gj * d2vel(M, r, w.kc[r], w.x, j, q);
      }
    }
  }
  for (int s = 0; s < n; ++s) {
    lam_out[(size_t)s * nc + c] = w.ub[s];
    if (ebar) ebar[(size_t)s * nc + c] += w.f0b[s] + w.f1b[s];
  }
  for (int s = n; s < nsp; ++s) {  // inert air mass: identity, clamp mask only
    double l = lam[(size_t)s * nc + c];
    if (clamp && Uout && !(Uout[(size_t)s * nc + c] > 0.0)) l = 0.0;
    lam_out[(size_t)s * nc + c] = l;
  }
}

void launch_ros23_vjp(const LaunchCtx& L, const double* U, const double* Uout, const double* lam,
                      double* lam_out, const double* kr, const double* em, double* ebar,
                      double dt, int clamp, const double* kz) {
  if (L.jit) {
    jit_launch_vjp(*L.jit, L.stream, L.nc, L.nsp, U, Uout, lam, lam_out, kr, em, ebar, dt, clamp,
                   kz);
    return;
  }
  int nb = (L.nc + 127) / 128;
  if (L.size_class == 0)
    k_ros23_vjp<kSmallMS, kSmallMR, kSmallMLU, kSmallMP><<<nb, 128, 0, L.stream>>>(
        L.mech, L.nc, L.nsp, U, Uout, lam, lam_out, kr, em, ebar, dt, clamp);
  else
    k_ros23_vjp<kLargeMS, kLargeMR, kLargeMLU, kLargeMP><<<nb, 128, 0, L.stream>>>(
        L.mech, L.nc, L.nsp, U, Uout, lam, lam_out, kr, em, ebar, dt, clamp);
}

// ------------------------------------------------------------------ transport (K4)
// Weights of the upwind face value w.r.t. the five stencil values (uniform horizontally,
// dp-weighted vertically).  With the branch decisions frozen at the forward state, every
// quantity of the reconstruction is a linear form in the five stencil values: a limited slope
// is 0 (extremum) or exactly one of da, +-2 d0, +-2 d1 (the smallest, with da's sign); the
// edges and the CW84 limiter combine those.  The value-level decisions use the forward
// kernels' expressions; only the coefficients are carried, about a quarter of the FP64 work of
// a forward-mode pass with five tangents (the oracle's restatement, which the tests compare).
__device__ __forceinline__ void slope_form(double am, double a, double ap, double sA, double sB,
                                           bool uniform, double& val, double c[3]) {
  c[0] = c[1] = c[2] = 0.0;
  val = 0.0;
  const double d0 = a - am, d1 = ap - a;
  if (!(d1 * d0 > 0.0)) return;
  double da, f[3];
  if (uniform) {
    da = 0.5 * (ap - am);
    f[0] = -0.5; f[1] = 0.0; f[2] = 0.5;
  } else {
    da = sA * d1 + sB * d0;
    f[0] = -sB; f[1] = sB - sA; f[2] = sA;
  }
  const double a0 = d0 < 0.0 ? -d0 : d0, a1 = d1 < 0.0 ? -d1 : d1, ada = da < 0.0 ? -da : da;
  const double l0 = 2.0 * a0, l1 = 2.0 * a1;
  const bool pick1 = l1 < l0;                    // lim = min(2|d0|, 2|d1|) as lmin5
  const double lim = pick1 ? l1 : l0;
  const double sg = signbit(da) ? -1.0 : 1.0;     // copysign onto da
  if (lim < ada) {                                // the limit binds
    if (pick1) {
      const double m = (d1 < 0.0 ? -2.0 : 2.0) * sg;
      c[1] = -m; c[2] = m;
    } else {
      const double m = (d0 < 0.0 ? -2.0 : 2.0) * sg;
      c[0] = -m; c[1] = m;
    }
    val = sg * lim;
  } else {
    const double m = (da < 0.0 ? -1.0 : 1.0) * sg;  // |da| carried back onto da's sign
    c[0] = m * f[0]; c[1] = m * f[1]; c[2] = m * f[2];
    val = sg * ada;
  }
}
// slope_form without branches: the same value and coefficients for every input.  Each
// coefficient of a limited slope is an exact constant (0, +-1/2, +-2) or a sign flip of a
// vertical coefficient, so the frozen branch is picked by integer compares of the magnitude
// bits (2|d| = |d| with the exponent field + 1 for the nonzero d of a live slope) and selects;
// the fused adjoint pencils' lanes then issue the same 4-5 FP64 instructions whatever branch
// their cell took.
__device__ __forceinline__ void slope_form_bf(double am, double a, double ap, double sA, double sB,
                                              bool uniform, double& val, double c[3]) {
  const double d0 = a - am, d1 = ap - a;
  if (prod_may_underflow(d0, d1)) {  // tiny or subnormal differences: the FP form, as forward
    slope_form(am, a, ap, sA, sB, uniform, val, c);
    return;
  }
#if RS_STRICT
  const bool live = d1 * d0 > 0.0;
#else
  const bool live = sgn_same_nz(d0, d1);  // the forward kernels' test
#endif
  const double da = uniform ? 0.5 * (ap - am) : sA * d1 + sB * d0;
  const int s0 = __double2hiint(d0), s1 = __double2hiint(d1), sd = __double2hiint(da);
  const unsigned h0 = (unsigned)s0 & 0x7fffffffu, l0 = (unsigned)__double2loint(d0);
  const unsigned h1 = (unsigned)s1 & 0x7fffffffu, l1 = (unsigned)__double2loint(d1);
  const unsigned hd = (unsigned)sd & 0x7fffffffu, ld = (unsigned)__double2loint(da);
  const bool pick1 = mag_lt(h1, l1, h0, l0);                              // 2|d1| < 2|d0|
  const unsigned hm = (pick1 ? h1 : h0) + (1u << 20), lm = pick1 ? l1 : l0;  // 2 min(|d0|, |d1|)
  const bool binds = mag_lt(hm, lm, hd, ld);                              // the limit binds
  const bool dneg = sd < 0;                                               // signbit(da)
  val = live ? __hiloint2double((int)((binds ? hm : hd) | ((unsigned)sd & 0x80000000u)),
                                (int)(binds ? lm : ld))
             : 0.0;
  // limited: c = (0, -m, m) or (-m, m, 0) with m = (d < 0 ? -2 : 2) * sg, d the picked difference
  const bool mneg = (pick1 ? (s1 < 0) : (s0 < 0)) != dneg;
  const double m = mneg ? -2.0 : 2.0;
  // unlimited: c = (da < 0 ? -1 : 1) * sg * f, which is -f only for da == -0
  double f0 = -0.5, f1 = 0.0, f2 = 0.5;
  if (!uniform) {
    f0 = -sB;
    f1 = sB - sA;
    f2 = sA;
  }
  const bool flip = (unsigned)sd == 0x80000000u && ld == 0u;  // da == -0.0
  const double u0 = flip ? -f0 : f0, u1 = flip ? -f1 : f1, u2 = flip ? -f2 : f2;
  const double q0 = pick1 ? 0.0 : -m, q1 = pick1 ? -m : m, q2 = pick1 ? m : 0.0;
  c[0] = live ? sel_d(binds, q0, u0) : 0.0;
  c[1] = live ? sel_d(binds, q1, u1) : 0.0;
  c[2] = live ? sel_d(binds, q2, u2) : 0.0;
}

__device__ __forceinline__ void face_weights_lin(const double* v, bool right, bool uniform,
                                                 const double* sA, const double* sB,
                                                 const double* eL, const double* eR, double* w) {
  double vm1, vd0, vp1, cm1[3], c0[3], cp1[3];
  slope_form(v[0], v[1], v[2], sA[0], sB[0], uniform, vm1, cm1);  // cell up-1: positions 0..2
  slope_form(v[1], v[2], v[3], sA[1], sB[1], uniform, vd0, c0);   // cell up:   positions 1..3
  slope_form(v[2], v[3], v[4], sA[2], sB[2], uniform, vp1, cp1);  // cell up+1: positions 2..4
  const double k6 = 1.0 / 6.0;
  double L[5] = {0, 0, 0, 0, 0}, R[5] = {0, 0, 0, 0, 0}, aLv, aRv;
  if (uniform) {
    aLv = (v[1] + 0.5 * (v[2] - v[1])) - k6 * (vd0 - vm1);
    aRv = (v[2] + 0.5 * (v[3] - v[2])) - k6 * (vp1 - vd0);
    L[1] = 0.5; L[2] = 0.5;
    R[2] = 0.5; R[3] = 0.5;
    for (int o = 0; o < 3; ++o) {
      L[1 + o] -= k6 * c0[o];
      L[o] += k6 * cm1[o];
      R[2 + o] -= k6 * cp1[o];
      R[1 + o] += k6 * c0[o];
    }
  } else {
    aLv = ((v[1] + eL[0] * (v[2] - v[1])) + eL[1] * vd0) + eL[2] * vm1;
    aRv = ((v[2] + eR[0] * (v[3] - v[2])) + eR[1] * vp1) + eR[2] * vd0;
    L[1] = 1.0 - eL[0]; L[2] = eL[0];
    R[2] = 1.0 - eR[0]; R[3] = eR[0];
    for (int o = 0; o < 3; ++o) {
      L[1 + o] += eL[1] * c0[o];
      L[o] += eL[2] * cm1[o];
      R[2 + o] += eR[1] * cp1[o];
      R[1 + o] += eR[2] * c0[o];
    }
  }
  const double a = v[2];
  if ((aRv - a) * (a - aLv) <= 0.0) {  // extremum: flat at the cell value
    for (int o = 0; o < 5; ++o) w[o] = o == 2 ? 1.0 : 0.0;
    return;
  }
  const double dA = aRv - aLv;
  const double a6 = 6.0 * (a - 0.5 * (aLv + aRv));
  if (dA * a6 > dA * dA) {             // aL = 3a - 2aR
    for (int o = 0; o < 5; ++o) L[o] = (o == 2 ? 3.0 : 0.0) - 2.0 * R[o];
  } else if (-(dA * dA) > dA * a6) {   // aR = 3a - 2aL
    for (int o = 0; o < 5; ++o) R[o] = (o == 2 ? 3.0 : 0.0) - 2.0 * L[o];
  }
  const double* r = right ? R : L;
  for (int o = 0; o < 5; ++o) w[o] = r[o];
}


// index maps of a stencil position p along a direction -> position in range, or -1 (open ghost)
__device__ __forceinline__ int map_pos(int p, int n, int bc) {
  if (p >= 0 && p < n) return p;
  if (bc == 0) return p < 0 ? p + n : p - n;  // periodic (stencil positions lie in [-3, n+2])
  if (bc == 1) return -1;                  // open: boundary data, no state
  return p < 0 ? -1 - p : 2 * n - 1 - p;   // mirror (closed walls, vertical)
}

// per cell: g = fbar/m, ubar_direct = g divM, mbar = -sum g f
__global__ void __launch_bounds__(256) k_adj_cell(DevTransport<double> T, const double* __restrict__ U,
                                                  const double* __restrict__ F,
                                                  const double* __restrict__ fbar,
                                                  double* __restrict__ ubar,
                                                  double* __restrict__ G, double g) {
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  int i = (int)(c % T.nlon);
  int j = (int)((c / T.nlon) % T.nlat);
  int k = (int)(c / ((size_t)T.nlon * T.nlat));
  const int nf = T.nlon + 1;
  const size_t ncol = (size_t)T.nlon * T.nlat, col = (size_t)j * T.nlon + i;
  double mxw = g * T.mx[((size_t)k * T.nlat + j) * nf + i];
  double mxe = g * T.mx[((size_t)k * T.nlat + j) * nf + i + 1];
  double mys = (T.lat_bc != 1 && j == 0) ? 0.0 : g * T.my[((size_t)k * (T.nlat + 1) + j) * T.nlon + i];
  double myn = (T.lat_bc != 1 && j + 1 == T.nlat) ? 0.0
             : g * T.my[((size_t)k * (T.nlat + 1) + j + 1) * T.nlon + i];
  double mzb = (k == 0) ? 0.0 : g * T.mz[(size_t)k * ncol + col];
  double mzt = (k + 1 == T.nlev) ? 0.0 : g * T.mz[(size_t)(k + 1) * ncol + col];
  double divM = ((mxe - mxw) * T.gx[j] + (myn * T.gyhi[j] - mys * T.gylo[j])) + (mzt - mzb);
  double m = U[(size_t)T.ntr * nc + c];
  double mb = 0.0;
  for (int s = 0; s < T.ntr; ++s) {
    double gs = fbar[(size_t)s * nc + c] / m;
    G[(size_t)s * nc + c] = gs;
    ubar[(size_t)s * nc + c] = gs * divM;
    mb = mb - gs * F[(size_t)s * nc + c];
  }
  ubar[(size_t)T.ntr * nc + c] = mb;
}

// per face (direction DIR): contributions C[s][face][o] = Fbar * M * w_o
template <int DIR>
__global__ void __launch_bounds__(256) k_adj_face(DevTransport<double> T, const double* __restrict__ U,
                                                  const double* __restrict__ G,
                                                  double* __restrict__ Cf, double g) {
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  const size_t ncol = (size_t)T.nlon * T.nlat;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int n = DIR == 0 ? T.nlon : (DIR == 1 ? T.nlat : T.nlev);
  int bc = DIR == 0 ? T.lon_bc : (DIR == 1 ? (T.lat_bc == 1 ? 1 : 2) : 2);
  long long total = DIR == 0 ? (long long)(T.nlon + 1) * T.nlat * T.nlev
                  : DIR == 1 ? (long long)T.nlon * (T.nlat + 1) * T.nlev
                             : (long long)ncol * (T.nlev + 1);
  if (idx >= total) return;
  int i, j, k, f;
  if (DIR == 0) {
    f = (int)(idx % (T.nlon + 1)); j = (int)((idx / (T.nlon + 1)) % T.nlat);
    k = (int)(idx / ((long long)(T.nlon + 1) * T.nlat)); i = f;
  } else if (DIR == 1) {
    i = (int)(idx % T.nlon); f = (int)((idx / T.nlon) % (T.nlat + 1));
    k = (int)(idx / ((long long)T.nlon * (T.nlat + 1))); j = f;
  } else {
    i = (int)(idx % T.nlon); j = (int)((idx / T.nlon) % T.nlat); f = (int)(idx / (long long)ncol);
    k = f;
  }
  const size_t fplane = (size_t)total;
  bool wall = (DIR == 1 && T.lat_bc != 1 && (f == 0 || f == T.nlat)) ||
              (DIR == 2 && (f == 0 || f == T.nlev));
  double M = 0.0;
  if (!wall) {
    if (DIR == 0) M = g * T.mx[((size_t)k * T.nlat + j) * (T.nlon + 1) + f];
    else if (DIR == 1) M = g * T.my[((size_t)k * (T.nlat + 1) + f) * T.nlon + i];
    else M = g * T.mz[(size_t)f * ncol + (size_t)j * T.nlon + i];
  }
  bool right = M > 0.0;
  int up = right ? f - 1 : f;
  // cell index of position p along this direction (or -1 for a ghost)
  auto cell_of = [&](int p) -> long long {
    int q = map_pos(p, n, bc);
    if (q < 0) return -1;
    if (DIR == 0) return ((long long)k * T.nlat + j) * T.nlon + q;
    if (DIR == 1) return ((long long)k * T.nlat + q) * T.nlon + i;
    return (long long)q * ncol + (size_t)j * T.nlon + i;
  };
  // neighbours: cell before the face (f-1) sees +F, cell after (f) sees -F in D
  long long cb = (f >= 1) ? cell_of(f - 1) : -1;
  long long ca = (f < n) ? cell_of(f) : -1;
  double cbw = DIR == 0 ? T.gx[j] : (DIR == 1 ? (f >= 1 ? T.gyhi[f - 1] : 0.0) : 1.0);
  double caw = DIR == 0 ? T.gx[j] : (DIR == 1 ? (f < n ? T.gylo[f] : 0.0) : 1.0);
  double sA[3] = {0, 0, 0}, sB[3] = {0, 0, 0}, eL[3] = {0, 0, 0}, eR[3] = {0, 0, 0};
  if (DIR == 2 && !wall) {
    size_t col = (size_t)j * T.nlon + i;
    for (int o = 0; o < 3; ++o) {
      sA[o] = T.vsA[(size_t)(up + o) * ncol + col];
      sB[o] = T.vsB[(size_t)(up + o) * ncol + col];
    }
    eL[0] = T.veAB[(size_t)up * ncol + col]; eL[1] = T.veC[(size_t)up * ncol + col];
    eL[2] = T.veD[(size_t)up * ncol + col];
    eR[0] = T.veAB[(size_t)(up + 1) * ncol + col]; eR[1] = T.veC[(size_t)(up + 1) * ncol + col];
    eR[2] = T.veD[(size_t)(up + 1) * ncol + col];
  }
  for (int s = 0; s < T.ntr; ++s) {
    double* out = Cf + ((size_t)s * fplane + (size_t)idx) * 5;
    if (wall) {
      for (int o = 0; o < 5; ++o) out[o] = 0.0;
      continue;
    }
    double v[5], w[5];
    for (int o = 0; o < 5; ++o) {
      long long cc = cell_of(up - 2 + o);
      if (cc >= 0) {
        v[o] = U[(size_t)s * nc + cc];
      } else {  // open-wall ghost: the prescribed boundary value
        int p = up - 2 + o;
        if (DIR == 0) v[o] = (p < 0 ? T.qw : T.qe)[((size_t)s * T.nlev + k) * T.nlat + j];
        else v[o] = (p < 0 ? T.qs : T.qn)[((size_t)s * T.nlev + k) * T.nlon + i];
      }
    }
    face_weights_lin(v, right, DIR != 2, sA, sB, eL, eR, w);
    double Fb = 0.0;
    if (cb >= 0) Fb = Fb - G[(size_t)s * nc + cb] * cbw;
    if (ca >= 0) Fb = Fb + G[(size_t)s * nc + ca] * caw;
    for (int o = 0; o < 5; ++o) out[o] = Fb * M * w[o];
  }
}

// per cell: gather the face contributions whose stencil position maps to this cell
template <int DIR>
__global__ void __launch_bounds__(256) k_adj_gather(DevTransport<double> T, const double* __restrict__ U,
                                                    const double* __restrict__ Cf,
                                                    double* __restrict__ ubar, double g) {
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  const size_t ncol = (size_t)T.nlon * T.nlat;
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  int i = (int)(c % T.nlon);
  int j = (int)((c / T.nlon) % T.nlat);
  int k = (int)(c / ncol);
  int n = DIR == 0 ? T.nlon : (DIR == 1 ? T.nlat : T.nlev);
  int bc = DIR == 0 ? T.lon_bc : (DIR == 1 ? (T.lat_bc == 1 ? 1 : 2) : 2);
  int pos = DIR == 0 ? i : (DIR == 1 ? j : k);
  long long total = DIR == 0 ? (long long)(T.nlon + 1) * T.nlat * T.nlev
                  : DIR == 1 ? (long long)T.nlon * (T.nlat + 1) * T.nlev
                             : (long long)ncol * (T.nlev + 1);
  auto face_index = [&](int f) -> long long {
    if (DIR == 0) return ((long long)k * T.nlat + j) * (T.nlon + 1) + f;
    if (DIR == 1) return ((long long)k * (T.nlat + 1) + f) * T.nlon + i;
    return (long long)f * ncol + (size_t)j * T.nlon + i;
  };
  auto mface = [&](int f) -> double {
    if (DIR == 0) return g * T.mx[((size_t)k * T.nlat + j) * (T.nlon + 1) + f];
    if (DIR == 1) return g * T.my[((size_t)k * (T.nlat + 1) + f) * T.nlon + i];
    return g * T.mz[(size_t)f * ncol + (size_t)j * T.nlon + i];
  };
  // candidate faces: windows around pos (and around pos -+ n for a periodic seam), visited
  // once each in a fixed order
  int lo[3], hi[3], nw = 0;
  if (bc == 0) {
    lo[nw] = pos - n - 5; hi[nw] = pos - n + 5; ++nw;
  }
  lo[nw] = pos - 5; hi[nw] = pos + 5; ++nw;
  if (bc == 0) {
    lo[nw] = pos + n - 5; hi[nw] = pos + n + 5; ++nw;
  }
  for (int s = 0; s < T.ntr; ++s) {
    double acc = 0.0;
    int last = -1;
    for (int wdw = 0; wdw < nw; ++wdw) {
      int a = lo[wdw] < 0 ? 0 : lo[wdw];
      int b = hi[wdw] > n ? n : hi[wdw];
      for (int f = a; f <= b; ++f) {
        if (f <= last) continue;
        last = f;
        double M = mface(f);
        int up = (M > 0.0) ? f - 1 : f;
        const double* cf = Cf + ((size_t)s * (size_t)total + (size_t)face_index(f)) * 5;
        for (int o = 0; o < 5; ++o)
          if (map_pos(up - 2 + o, n, bc) == pos) acc = acc + cf[o];
      }
    }
    ubar[(size_t)s * nc + c] += acc;
  }
}

// ------------------------------------------------------------------ fused adjoint pencils
// One block per pencil (a lon row; or PW adjacent lat lines / vertical columns), looping over
// the tracers.  The same arithmetic as face_weights_lin + the per-cell gather, reorganised:
//   1. the tracer values (3-cell halo) and the cell adjoints g = fbar / m go to shared memory;
//   2. each cell's linearised slope (value + 3 coefficients) once per cell;
//   3. each edge's value and weights over its 4 stencil positions once per edge -- the aL of
//      the cell right of the edge and the aR of the cell left of it are the same expression;
//   4. per face: the frozen-branch limiter on (a, aL, aR) with those weights, the face
//      adjoint Fbar (from the two adjacent cells' g) and the contributions Fbar M w_o;
//   5. per cell: the contributions of every face whose stencil covers it, faces ascending and
//      positions ascending (the fixed order of the per-cell gather), added to ubar.
// Per face the old path evaluated three slope forms and both edges' weights and went through
// a global slab; here each is done once and stays on chip.  Bit-identical to that path.
template <int DIR>
__device__ __forceinline__ void adj_pencil_geometry(const DevTransport<double>& T, int& n, int& bc) {
  n = DIR == 0 ? T.nlon : (DIR == 1 ? T.nlat : T.nlev);
  bc = DIR == 0 ? T.lon_bc : (DIR == 1 ? (T.lat_bc == 1 ? 1 : 2) : 2);
}
// doubles of shared memory per pencil (and the int upwind indices) for a direction of length n
__host__ __device__ inline int adj_pencil_doubles(int n) {
  return (n + 6) + n + 4 * (n + 4) + 5 * (n + 3) + 5 * (n + 1) + (n + 1);
}

template <int DIR, int PW>
__global__ void __launch_bounds__(256) k_adj_pencil(DevTransport<double> T,
                                                    const double* __restrict__ U,
                                                    const double* __restrict__ G,
                                                    double* __restrict__ ubar, double g) {
  const int s_blk = blockIdx.y;  // one tracer per block row of the grid
  int n, bc;
  adj_pencil_geometry<DIR>(T, n, bc);
  extern __shared__ double sma[];
  const int tx = threadIdx.x, ty = threadIdx.y, ny = blockDim.y;
  // per-pencil arrays, [index][PW] with the pencil's lane fastest
  double* V = sma;                           // [n+6]: stencil positions -3 .. n+2
  double* Gc = V + (n + 6) * PW;             // [n]:   cell adjoints 0 .. n-1
  double* SV = Gc + n * PW;                  // [n+4]: slope values of cells -2 .. n+1
  double* SC = SV + (n + 4) * PW;            // [3][n+4]: slope coefficients
  double* EV = SC + 3 * (n + 4) * PW;        // [n+3]: edge values, edges -1 .. n+1
  double* EW = EV + (n + 3) * PW;            // [4][n+3]: edge weights on positions e-2 .. e+1
  double* C = EW + 4 * (n + 3) * PW;         // [5][n+1]: face contributions
  double* Mf = C + 5 * (n + 1) * PW;         // [n+1]: face air-mass flux (0 on walls)
  int* upf = reinterpret_cast<int*>(Mf + (n + 1) * PW);  // [n+1]
  const int ln = DIR == 0 ? 0 : tx;  // lane of this thread's pencil in the [index][PW] arrays
#define AV(a, i) a[(i) * PW + ln]
  const size_t ncol = (size_t)T.nlon * T.nlat, nc = ncol * T.nlev;
  // the pencil: fixed (j, k) for x; (i, k) for y; (i, j) for z
  int i = 0, j = 0, k = 0;
  bool live = true;
  if (DIR == 0) {
    j = blockIdx.x % T.nlat;
    k = blockIdx.x / T.nlat;
  } else if (DIR == 1) {
    const int ntile = (T.nlon + PW - 1) / PW;
    k = blockIdx.x / ntile;
    i = (blockIdx.x % ntile) * PW + tx;
    live = i < T.nlon;
  } else {
    const size_t col = (size_t)blockIdx.x * PW + tx;
    live = col < ncol;
    i = live ? (int)(col % T.nlon) : 0;
    j = live ? (int)(col / T.nlon) : 0;
  }
  auto cell = [&](int q) -> size_t {  // flat cell index of position q (0 <= q < n)
    if (DIR == 0) return ((size_t)k * T.nlat + j) * T.nlon + q;
    if (DIR == 1) return ((size_t)k * T.nlat + q) * T.nlon + i;
    return (size_t)q * ncol + (size_t)j * T.nlon + i;
  };
  const size_t colz = (size_t)j * T.nlon + i;
  // x rows: one lane per position (PW == 1); y / z: one lane per pencil, ty strides positions
  const int lane0 = DIR == 0 ? threadIdx.x : ty;
  const int lstride = DIR == 0 ? blockDim.x : ny;
  for (int f = lane0; f <= n; f += lstride) {
    const bool wall = (DIR == 1 && T.lat_bc != 1 && (f == 0 || f == n)) || (DIR == 2 && (f == 0 || f == n));
    double M = 0.0;
    if (live && !wall) {
      if (DIR == 0) M = g * T.mx[((size_t)k * T.nlat + j) * (T.nlon + 1) + f];
      else if (DIR == 1) M = g * T.my[((size_t)k * (T.nlat + 1) + f) * T.nlon + i];
      else M = g * T.mz[(size_t)f * ncol + colz];
    }
    AV(Mf, f) = M;
    AV(upf, f) = (M > 0.0) ? f - 1 : f;
  }
  {
    const int s = s_blk;
    const double* q = U + (size_t)s * nc;
    // 1. values and cell adjoints
    for (int p = lane0 - 3; p <= n + 2; p += lstride) {
      double v = 0.0;
      if (live) {
        const int qq = map_pos(p, n, bc);
        if (qq >= 0) {
          v = q[cell(qq)];
        } else if (DIR == 0) {
          v = (p < 0 ? T.qw : T.qe)[((size_t)s * T.nlev + k) * T.nlat + j];
        } else {
          v = (p < 0 ? T.qs : T.qn)[((size_t)s * T.nlev + k) * T.nlon + i];
        }
      }
      AV(V, p + 3) = v;
      if (p >= 0 && p < n) AV(Gc, p) = live ? G[(size_t)s * nc + cell(p)] : 0.0;
    }
    __syncthreads();
    // 2. slopes of cells -2 .. n+1 (vertical coefficient rows p+1, as the forward kernels)
    for (int p = lane0 - 2; p <= n + 1; p += lstride) {
      double sA = 0.0, sB = 0.0;
      if (DIR == 2 && live && p >= -1 && p <= n) {
        sA = T.vsA[(size_t)(p + 1) * ncol + colz];
        sB = T.vsB[(size_t)(p + 1) * ncol + colz];
      }
      double val, c[3];
      slope_form_bf(AV(V, p + 2), AV(V, p + 3), AV(V, p + 4), sA, sB, DIR != 2, val, c);
      AV(SV, p + 2) = val;
      for (int o = 0; o < 3; ++o) AV(SC, o * (n + 4) + p + 2) = c[o];
    }
    __syncthreads();
    // 3. edges -1 .. n+1 between cells e-1 and e: value and weights on positions e-2 .. e+1,
    //    built in face_weights_lin's order (the aL of cell e, the aR of cell e-1)
    for (int e = lane0 - 1; e <= n + 1; e += lstride) {
      const double vm = AV(V, e + 2), vc = AV(V, e + 3);  // cells e-1, e
      const double sm_ = AV(SV, e + 1), sc_ = AV(SV, e + 2);  // slopes of cells e-1, e
      double w[4] = {0.0, 0.0, 0.0, 0.0}, ev;
      if (DIR != 2) {
        const double k6 = 1.0 / 6.0;
        ev = (vm + 0.5 * (vc - vm)) - k6 * (sc_ - sm_);
        w[1] = 0.5; w[2] = 0.5;
        for (int o = 0; o < 3; ++o) {
          w[1 + o] -= k6 * AV(SC, o * (n + 4) + e + 2);
          w[o] += k6 * AV(SC, o * (n + 4) + e + 1);
        }
      } else {
        double eab = 0.0, ec = 0.0, ed = 0.0;
        if (live && e >= 0 && e <= n) {
          eab = T.veAB[(size_t)e * ncol + colz];
          ec = T.veC[(size_t)e * ncol + colz];
          ed = T.veD[(size_t)e * ncol + colz];
        }
        ev = ((vm + eab * (vc - vm)) + ec * sc_) + ed * sm_;
        w[1] = 1.0 - eab; w[2] = eab;
        for (int o = 0; o < 3; ++o) {
          w[1 + o] += ec * AV(SC, o * (n + 4) + e + 2);
          w[o] += ed * AV(SC, o * (n + 4) + e + 1);
        }
      }
      AV(EV, e + 1) = ev;
      for (int o = 0; o < 4; ++o) AV(EW, o * (n + 3) + e + 1) = w[o];
    }
    __syncthreads();
    // 4. faces: limiter with frozen branches, face adjoint, contributions
    for (int f = lane0; f <= n; f += lstride) {
      const double M = AV(Mf, f);
      double* out = &AV(C, f);  // C[o][f] at out[o * (n+1) * PW]
      const size_t cstr = (size_t)(n + 1) * PW;
      const bool wall = (DIR == 1 && T.lat_bc != 1 && (f == 0 || f == n)) || (DIR == 2 && (f == 0 || f == n));
      if (wall) {
        for (int o = 0; o < 5; ++o) out[o * cstr] = 0.0;
        continue;
      }
      const int up = AV(upf, f);
      const bool right = M > 0.0;
      double L[5], R[5];
      L[4] = 0.0; R[0] = 0.0;
      for (int o = 0; o < 4; ++o) {
        L[o] = AV(EW, o * (n + 3) + up + 1);      // edge up: positions up-2 .. up+1
        R[1 + o] = AV(EW, o * (n + 3) + up + 2);  // edge up+1: positions up-1 .. up+2
      }
      const double aLv = AV(EV, up + 1), aRv = AV(EV, up + 2), a = AV(V, up + 3);
      // the limiter's decisions as the forward kernels take them, then one set of weights
      // per lane by selects: flat -> e_2; steepened side -> 3 e_2 - 2 (other side); else the side
      const double dA = aRv - aLv;
      const double a6 = 6.0 * (a - 0.5 * (aLv + aRv));
      bool flat, stl, str;
#if !RS_STRICT
      if (!(tiny_operand(a) || tiny_operand(aLv) || tiny_operand(aRv))) {
        const long long ka = ord_key(a), kl = ord_key(aLv), kr = ord_key(aRv);
        flat = !((kr > ka && ka > kl) || (kr < ka && ka < kl));
        const long long kd = ord_key(dA), k6 = ord_key(a6);
        stl = (kd > 0 && k6 > kd) || (kd < 0 && k6 < kd);
        str = !stl && ((kd > 0 && k6 < -kd) || (kd < 0 && k6 > -kd));
      } else
#endif
      {
        flat = (aRv - a) * (a - aLv) <= 0.0;
        stl = dA * a6 > dA * dA;                      // aL <- 3a - 2aR
        str = !stl && (-(dA * dA) > dA * a6);         // aR <- 3a - 2aL
      }
      const bool need = (stl && !right) || (str && right);
      double w[5];
      for (int o = 0; o < 5; ++o) {
        const double st = (o == 2 ? 3.0 : 0.0) - 2.0 * sel_d(stl, R[o], L[o]);
        const double side = sel_d(right, R[o], L[o]);
        w[o] = sel_d(flat, o == 2 ? 1.0 : 0.0, sel_d(need, st, side));
      }
      double cbw, caw;
      if (DIR == 0) cbw = caw = T.gx[j];
      else if (DIR == 1) {
        cbw = f >= 1 ? T.gyhi[f - 1] : 0.0;
        caw = f < n ? T.gylo[f] : 0.0;
      } else cbw = caw = 1.0;
      double Fb = 0.0;
      if (f >= 1) Fb = Fb - AV(Gc, f - 1) * cbw;
      if (f < n) Fb = Fb + AV(Gc, f) * caw;
      for (int o = 0; o < 5; ++o) out[o * cstr] = Fb * M * w[o];
    }
    __syncthreads();
    // 5. gather (faces ascending, positions ascending; periodic seam windows as before).  The
    //    stencil positions that map to cell pos are pos itself and, on a periodic seam, its
    //    images pos -+ n (open walls map ghosts to the boundary values, not to cells).  Face f
    //    covers positions f-3 .. f+2, so each image p is reached only by faces p-2 .. p+3; for
    //    n >= 6 these face ranges are disjoint and ascending with the images, and each face
    //    reaches pos through exactly one position -- the same faces in the same order as the
    //    general loop below, without its divergent window scan at the row ends.  Next to a
    //    mirror wall a face can reach the cell twice (itself and its reflection); those cells
    //    scan the faces that reach either, and short pencils take the general loop.
    for (int pos = lane0; pos < n; pos += lstride) {
      if (!live) break;
      const bool end = pos < 3 || pos > n - 4;
      if (!end || (bc != 2 && n >= 6)) {
        const int nimg = (bc == 0 && end) ? 3 : 1;
        double acc = 0.0;
        for (int m = 0; m < nimg; ++m) {
          const int img = nimg == 3 ? pos + (m - 1) * n : pos;
          const int fa = img - 2 < 0 ? 0 : img - 2, fb = img + 3 > n ? n : img + 3;
          for (int f = fa; f <= fb; ++f) {
            const int o = img - AV(upf, f) + 2;
            if (o >= 0 && o <= 4) acc = acc + AV(C, o * (n + 1) + f);
          }
        }
        ubar[(size_t)s * nc + cell(pos)] += acc;
        continue;
      }
      if (bc == 2 && n >= 6) {
        // mirror walls: positions pos and its reflection r (-1-pos below, 2n-1-pos above) map
        // to this cell.  Faces ascending over those that can reach either, and per face the
        // two candidate positions ascending (r < pos below the wall, pos < r above): the
        // general loop's terms in its order.
        const int r = pos < 3 ? -1 - pos : 2 * n - 1 - pos;
        const int p0 = r < pos ? r : pos, p1 = r < pos ? pos : r;
        const int fa = p0 - 2 < 0 ? 0 : p0 - 2, fb = p1 + 3 > n ? n : p1 + 3;
        double acc = 0.0;
        for (int f = fa; f <= fb; ++f) {
          const int up = AV(upf, f);
          const int o0 = p0 - up + 2, o1 = p1 - up + 2;
          if (o0 >= 0 && o0 <= 4) acc = acc + AV(C, o0 * (n + 1) + f);
          if (o1 >= 0 && o1 <= 4) acc = acc + AV(C, o1 * (n + 1) + f);
        }
        ubar[(size_t)s * nc + cell(pos)] += acc;
        continue;
      }
      int lo[3], hi[3], nw = 0;
      if (bc == 0) { lo[nw] = pos - n - 5; hi[nw] = pos - n + 5; ++nw; }
      lo[nw] = pos - 5; hi[nw] = pos + 5; ++nw;
      if (bc == 0) { lo[nw] = pos + n - 5; hi[nw] = pos + n + 5; ++nw; }
      double acc = 0.0;
      int last = -1;
      for (int wdw = 0; wdw < nw; ++wdw) {
        const int a0 = lo[wdw] < 0 ? 0 : lo[wdw];
        const int b0 = hi[wdw] > n ? n : hi[wdw];
        for (int f = a0; f <= b0; ++f) {
          if (f <= last) continue;
          last = f;
          const int up = AV(upf, f);
          for (int o = 0; o < 5; ++o)
            if (map_pos(up - 2 + o, n, bc) == pos) acc = acc + AV(C, o * (n + 1) + f);
        }
      }
      ubar[(size_t)s * nc + cell(pos)] += acc;
    }
    __syncthreads();
  }
#undef AV
}

// ubar = (d f_T / du)^T fbar at stage state U (whose RHS value is F), time factor g
// VJP of the PBL mixing term t_k = f_k (qbar - q_k) / tau with qbar = sum_j w_j q_j / den:
// ubar_j += (w_j / den) * (sum_k fbar_k f_k) / tau - fbar_j f_j / tau, per tracer and column
// (the term does not depend on the air mass).
__global__ void k_pbl_vjp(DevTransport<double> T, const double* __restrict__ fbar,
                          double* __restrict__ ubar) {
  const size_t ncol = (size_t)T.nlon * T.nlat, nc = ncol * T.nlev;
  const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (size_t)T.ntr * ncol) return;
  const size_t s = id / ncol, col = id % ncol;
  const double* fb = fbar + s * nc + col;
  double* ub = ubar + s * nc + col;
  double a = 0.0;
  for (int k = 0; k < T.nlev; ++k) a = a + fb[(size_t)k * ncol] * T.pbl_f[(size_t)k * ncol + col];
  const double at = a / T.pbl_tau, den = T.pbl_den[col];
  for (int k = 0; k < T.nlev; ++k) {
    const size_t x = (size_t)k * ncol + col;
    ub[(size_t)k * ncol] += (T.pbl_w[x] / den) * at - (fb[(size_t)k * ncol] * T.pbl_f[x]) / T.pbl_tau;
  }
}

// The fused adjoint pencils for all three directions, or false (nothing launched) when a
// direction's pencils do not fit in shared memory -- the caller then uses the face + gather
// kernels, which compute the same bits.
constexpr size_t kAdjSmemCap = 110 * 1024;  // two blocks per SM
static size_t adj_pencil_bytes(int n, int pw) {
  return ((size_t)adj_pencil_doubles(n) * sizeof(double) + (size_t)(n + 1) * sizeof(int)) * pw;
}
template <int DIR, int PW>
static void adj_pencil_launch(cudaStream_t st, const DevTransport<double>& T, const double* U,
                              const double* G, double* ubar, double g, size_t smem) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_adj_pencil<DIR, PW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kAdjSmemCap);
    attr = true;
  }
  const size_t ncol = (size_t)T.nlon * T.nlat;
  if constexpr (DIR == 0) {
    const int thr = std::min(256, (T.nlon + 6 + 31) / 32 * 32);
    k_adj_pencil<0, 1><<<dim3((unsigned)(T.nlat * T.nlev), (unsigned)T.ntr), thr, smem, st>>>(T, U, G, ubar, g);
  } else if constexpr (DIR == 1) {
    const unsigned ntile = (unsigned)((T.nlon + PW - 1) / PW);
    k_adj_pencil<1, PW><<<dim3(ntile * (unsigned)T.nlev, (unsigned)T.ntr), dim3(PW, 256 / PW), smem, st>>>(T, U, G, ubar, g);
  } else {
    k_adj_pencil<2, PW><<<dim3((unsigned)((ncol + PW - 1) / PW), (unsigned)T.ntr), dim3(PW, 256 / PW), smem, st>>>(T, U, G, ubar, g);
  }
}
template <int DIR>
static bool adj_pencil_dir(cudaStream_t st, const DevTransport<double>& T, const double* U,
                           const double* G, double* ubar, double g, bool dry) {
  const int n = DIR == 0 ? T.nlon : (DIR == 1 ? T.nlat : T.nlev);
  if constexpr (DIR == 0) {
    const size_t b = adj_pencil_bytes(n, 1);
    if (b > kAdjSmemCap) return false;
    if (!dry) adj_pencil_launch<0, 1>(st, T, U, G, ubar, g, b);
    return true;
  } else {
    // the widest pencil tile that leaves room for four blocks per SM, else for two
    int pick = 0;
    for (int pw : {16, 8, 4})
      if (!pick && adj_pencil_bytes(n, pw) <= kAdjSmemCap / 2) pick = pw;
    for (int pw : {16, 8, 4})
      if (!pick && adj_pencil_bytes(n, pw) <= kAdjSmemCap) pick = pw;
    if (!pick) return false;
    const size_t b = adj_pencil_bytes(n, pick);
    if (!dry) {
      if (pick == 16) adj_pencil_launch<DIR, 16>(st, T, U, G, ubar, g, b);
      else if (pick == 8) adj_pencil_launch<DIR, 8>(st, T, U, G, ubar, g, b);
      else adj_pencil_launch<DIR, 4>(st, T, U, G, ubar, g, b);
    }
    return true;
  }
}
static bool launch_adj_pencils(cudaStream_t st, const DevTransport<double>& T, const double* U,
                               const double* G, double* ubar, double g) {
  if (!adj_pencil_dir<0>(st, T, U, G, ubar, g, true) || !adj_pencil_dir<1>(st, T, U, G, ubar, g, true) ||
      !adj_pencil_dir<2>(st, T, U, G, ubar, g, true))
    return false;
  adj_pencil_dir<0>(st, T, U, G, ubar, g, false);
  adj_pencil_dir<1>(st, T, U, G, ubar, g, false);
  adj_pencil_dir<2>(st, T, U, G, ubar, g, false);
  return true;
}

void launch_transport_rhs_vjp(cudaStream_t st, const DevTransport<double>& T, const double* U,
                              const double* F, const double* fbar, double* ubar, double* G,
                              double* Cf, double g) {
  size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  unsigned nb = (unsigned)((nc + 255) / 256);
  k_adj_cell<<<nb, 256, 0, st>>>(T, U, F, fbar, ubar, G, g);
  if (!launch_adj_pencils(st, T, U, G, ubar, g)) {  // pencils too long for shared memory
    long long nx = (long long)(T.nlon + 1) * T.nlat * T.nlev;
    long long ny = (long long)T.nlon * (T.nlat + 1) * T.nlev;
    long long nz = (long long)T.nlon * T.nlat * (T.nlev + 1);
    k_adj_face<0><<<(unsigned)((nx + 255) / 256), 256, 0, st>>>(T, U, G, Cf, g);
    k_adj_gather<0><<<nb, 256, 0, st>>>(T, U, Cf, ubar, g);
    k_adj_face<1><<<(unsigned)((ny + 255) / 256), 256, 0, st>>>(T, U, G, Cf, g);
    k_adj_gather<1><<<nb, 256, 0, st>>>(T, U, Cf, ubar, g);
    k_adj_face<2><<<(unsigned)((nz + 255) / 256), 256, 0, st>>>(T, U, G, Cf, g);
    k_adj_gather<2><<<nb, 256, 0, st>>>(T, U, Cf, ubar, g);
  }
  if (T.pbl) {
    size_t n = (size_t)T.ntr * T.nlon * T.nlat;
    k_pbl_vjp<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(T, fbar, ubar);
  }
}

// out = a*x + b*y + c*z over n elements (null operands skipped)
__global__ void k_lincomb(size_t n, double* __restrict__ out, double a, const double* x, double b,
                          const double* y, double c, const double* z) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double r = 0.0;
  if (x) r = a * x[e];
  if (y) r = r + b * y[e];
  if (z) r = r + c * z[e];
  out[e] = r;
}
void launch_lincomb(cudaStream_t st, size_t n, double* out, double a, const double* x, double b,
                    const double* y, double c, const double* z) {
  k_lincomb<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, out, a, x, b, y, c, z);
}

}  // namespace rs
