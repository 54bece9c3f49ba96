// ORACLE -- CPU FP64 restatement of ReSEACT's operator-split step.  TEST INFRASTRUCTURE ONLY:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this library,
// and only as the parity reference / the timed CPU baseline.  The product (libreseact_gb300.so) never
// links, loads or calls it.
//
// The reference is Julia and cannot run here (no julia, un-vendored EarthSciAST /
// OrdinaryDiffEq stack).  This file restates, in plain C++ FP64 with -ffp-contract=off:
//   * ROS23 attempt           tools/reactant_handoff/rx_traced_integrator.jl:255-349
//   * pivot-free blocksolve   rx_traced_integrator.jl:101-135  (dense, natural order)
//     (optionally on the symmetric permutation a production build eliminates in: or_set_lu_order)
//   * SSPRK43 attempt         rx_traced_integrator.jl:351-437
//   * PI controller + loop    rx_traced_integrator.jl:85-99, 439-507
//   * Lie-Trotter macro step  run_reseact_reactant.jl:310-355 (adv), op_split.jl:100-164
//   * mass-action chemistry   prototypes/g2_depsink/g2_nodep.esm:450-1780 (tables built by
//                             reseact/esm_gb300/mechanism.py from that schema)
//   * CWC flux-form transport reseact.esm:1535 (continuity), :2083 (species, mixing-ratio
//                             form), prototypes/transport_3d/transport_3d.esm (analytic winds)
//   * CW84 monotone PPM       Colella & Woodward 1984 eqs. 1.6-1.8, 1.10 (the reference's PPM
//                             rule files are absent; only their slope form is quoted in
//                             tools/diag/ppm_limiter_kink_repro.jl:3-8 and the extremum test
//                             in tools/diag/rhs_kink_probe.jl:9-14) -- PARITY FOR THE PPM
//                             ARITHMETIC IS UNPINNED against the reference; it is pinned by the
//                             CWC freestream invariant (transport_3d.esm tests, tools/cwc_gate.jl).
//
// Layout: grid SoA, u[s*NC + c] with c = (k*nlat + j)*nlon + i.  The global hairer norm uses
// the fixed two-level reduction tree documented at reduce_fixed() below.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/reseact_gb300.h"

namespace {

constexpr double kD2R = 0.017453292519943295;
constexpr double kOneSixth = 1.0 / 6.0;

// ------------------------------------------------------------------ mechanism (dense form)
struct Mech {
  int ns = 0, nr = 0, np = 0, comb = 1;
  std::vector<int> rptr, rsp, rnu, pptr, pops;
  std::vector<double> pvals, params, net;  // net[r*ns + s]
  std::vector<int> prptr, prsp;
  std::vector<double> prcoef;
};

Mech make_mech(const rs_mechanism* m) {
  Mech M;
  M.ns = m->n_species; M.nr = m->n_reactions; M.np = m->n_params; M.comb = m->combinatoric;
  M.rptr.assign(m->react_ptr, m->react_ptr + M.nr + 1);
  M.rsp.assign(m->react_species, m->react_species + M.rptr[M.nr]);
  M.rnu.assign(m->react_nu, m->react_nu + M.rptr[M.nr]);
  M.prptr.assign(m->prod_ptr, m->prod_ptr + M.nr + 1);
  M.prsp.assign(m->prod_species, m->prod_species + M.prptr[M.nr]);
  M.prcoef.assign(m->prod_coef, m->prod_coef + M.prptr[M.nr]);
  M.pptr.assign(m->prog_ptr, m->prog_ptr + M.nr + 1);
  M.pops.assign(m->prog_op, m->prog_op + M.pptr[M.nr]);
  M.pvals.assign(m->prog_val, m->prog_val + M.pptr[M.nr]);
  M.params.assign(m->params, m->params + M.np);
  M.net.assign((size_t)M.nr * M.ns, 0.0);
  for (int r = 0; r < M.nr; ++r) {
    for (int e = M.rptr[r]; e < M.rptr[r + 1]; ++e) M.net[(size_t)r * M.ns + M.rsp[e]] -= M.rnu[e];
    for (int e = M.prptr[r]; e < M.prptr[r + 1]; ++e) M.net[(size_t)r * M.ns + M.prsp[e]] += M.prcoef[e];
  }
  return M;
}

// Postfix rate program (one per reaction), evaluated per cell.
double eval_prog(const Mech& M, int r, double T, double P) {
  double st[64];
  int sp = 0;
  for (int e = M.pptr[r]; e < M.pptr[r + 1]; ++e) {
    int op = M.pops[e];
    double v = M.pvals[e];
    switch (op) {
      case RS_OP_CONST: st[sp++] = v; break;
      case RS_OP_TEMP: st[sp++] = T; break;
      case RS_OP_PRES: st[sp++] = P; break;
      case RS_OP_PARAM: st[sp++] = M.params[(int)v]; break;
      case RS_OP_ADD: --sp; st[sp - 1] = st[sp - 1] + st[sp]; break;
      case RS_OP_SUB: --sp; st[sp - 1] = st[sp - 1] - st[sp]; break;
      case RS_OP_MUL: --sp; st[sp - 1] = st[sp - 1] * st[sp]; break;
      case RS_OP_DIV: --sp; st[sp - 1] = st[sp - 1] / st[sp]; break;
      case RS_OP_POW: --sp; st[sp - 1] = std::pow(st[sp - 1], st[sp]); break;
      case RS_OP_NEG: st[sp - 1] = -st[sp - 1]; break;
      case RS_OP_EXP: st[sp - 1] = std::exp(st[sp - 1]); break;
      case RS_OP_LOG: st[sp - 1] = std::log(st[sp - 1]); break;
      case RS_OP_LOG10: st[sp - 1] = std::log10(st[sp - 1]); break;
      case RS_OP_SQRT: st[sp - 1] = std::sqrt(st[sp - 1]); break;
      default: return NAN;
    }
  }
  double k = st[0];
  if (M.comb) {  // mass-action product divided by prod(nu!)
    for (int e = M.rptr[r]; e < M.rptr[r + 1]; ++e) {
      double f = 1.0;
      for (int t = 2; t <= M.rnu[e]; ++t) f *= t;
      if (f != 1.0) k = k * (1.0 / f);
    }
  }
  return k;
}

// reaction velocity v_r = k * prod x^nu (reactant entries in table order)
inline double velocity(const Mech& M, int r, double k, const double* x) {
  double v = k;
  for (int e = M.rptr[r]; e < M.rptr[r + 1]; ++e)
    for (int t = 0; t < M.rnu[e]; ++t) v = v * x[M.rsp[e]];
  return v;
}

// d v_r / d x_q
inline double dvel(const Mech& M, int r, double k, const double* x, int q) {
  double d = k;
  for (int e = M.rptr[r]; e < M.rptr[r + 1]; ++e) {
    int s = M.rsp[e], nu = M.rnu[e];
    if (s == q) {
      if (nu >= 2) {
        double f = (double)nu;
        for (int t = 1; t < nu; ++t) f = f * x[s];
        d = d * f;
      }
    } else {
      for (int t = 0; t < nu; ++t) d = d * x[s];
    }
  }
  return d;
}

// chemistry RHS of one cell: f_s = sum_r net[r,s] v_r (+ emission)
void chem_rhs_cell(const Mech& M, const double* k, const double* x, const double* emis,
                   double* f, double* vbuf) {
  for (int r = 0; r < M.nr; ++r) vbuf[r] = velocity(M, r, k[r], x);
  for (int s = 0; s < M.ns; ++s) {
    double acc = 0.0;
    for (int r = 0; r < M.nr; ++r) {
      double c = M.net[(size_t)r * M.ns + s];
      if (c != 0.0) acc = acc + c * vbuf[r];
    }
    f[s] = emis ? acc + emis[s] : acc;
  }
}

// dense analytic block Jacobian J[s*ns+q] (the exact Jacobian the reference obtains by
// forward-mode AD / symbolic differentiation, block_jac.jl:108-136)
void chem_jac_cell(const Mech& M, const double* k, const double* x, double* J) {
  // Reaction-major accumulation: each entry J[s,q] still receives its contributions in
  // increasing reaction order, starting from 0.0, so the sums associate exactly as in the
  // entry-by-entry form sum_r net[r,s] dv_r/dx_q.
  int ns = M.ns;
  std::fill(J, J + ns * ns, 0.0);
  for (int r = 0; r < M.nr; ++r) {
    const double* net = M.net.data() + (size_t)r * ns;
    for (int e = M.rptr[r]; e < M.rptr[r + 1]; ++e) {
      int q = M.rsp[e];
      double d = dvel(M, r, k[r], x, q);
      for (int s = 0; s < ns; ++s) {
        double c = net[s];
        if (c != 0.0) J[s * ns + q] = J[s * ns + q] + c * d;
      }
    }
  }
}

// Pivot-free Gaussian elimination (rx_traced_integrator.jl:110-135): factor W in place,
// recording the multipliers in the lower triangle; solve() replays the same elimination on b.
void lu_factor(int n, double* W) {
  for (int k = 0; k < n; ++k) {
    double piv = 1.0 / W[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double m = W[i * n + k] * piv;
      for (int j = k + 1; j < n; ++j) {
        double mw = m * W[k * n + j];
        W[i * n + j] = W[i * n + j] - mw;
      }
      W[i * n + k] = m;
    }
  }
}
void lu_solve(int n, const double* LU, const double* b, double* x) {
  double y[64];
  for (int i = 0; i < n; ++i) y[i] = b[i];
  for (int k = 0; k < n; ++k)
    for (int i = k + 1; i < n; ++i) {
      double mb = LU[i * n + k] * y[k];
      y[i] = y[i] - mb;
    }
  for (int i = n - 1; i >= 0; --i) {
    double acc = y[i];
    for (int j = i + 1; j < n; ++j) {
      double wx = LU[i * n + j] * x[j];
      acc = acc - wx;
    }
    x[i] = acc / LU[i * n + i];
  }
}

// The same elimination on the symmetric permutation P W P^T, rows and columns in the order
// `ord` (species eliminated at each pivot); with an empty order this is blocksolve exactly.
// Used to check a production build that eliminates in a fill-reducing order.
void lu_factor_ord(const std::vector<int>& ord, int n, std::vector<double>& W) {
  if (!ord.empty()) {
    std::vector<double> P((size_t)n * n);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) P[(size_t)i * n + j] = W[(size_t)ord[i] * n + ord[j]];
    W.swap(P);
  }
  lu_factor(n, W.data());
}
void lu_solve_ord(const std::vector<int>& ord, int n, const double* LU, const double* b,
                  double* x) {
  if (ord.empty()) {
    lu_solve(n, LU, b, x);
    return;
  }
  double bp[64], xp[64];
  for (int i = 0; i < n; ++i) bp[i] = b[ord[i]];
  lu_solve(n, LU, bp, xp);
  for (int i = 0; i < n; ++i) x[ord[i]] = xp[i];
}

// ------------------------------------------------------------------ fixed reduction tree
// Level 1: chunks of 256 cells, v[t] = e[b*256 + t] (0.0 past the end), then the pairwise
// tree v[t] += v[t+s] for s = 128, 64, ..., 1.  Level 2: one chunk of 256 lanes, lane t sums
// partial[t + 256*q] for q = 0, 1, ... in order from 0.0, then the same tree.  The CUDA
// kernels reduce with exactly this tree, so the global error norm is bitwise reproducible.
double tree256(double* v) {
  for (int s = 128; s > 0; s >>= 1)
    for (int t = 0; t < s; ++t) v[t] = v[t] + v[t + s];
  return v[0];
}
double reduce_fixed(const double* e, size_t n) {
  size_t nb = (n + 255) / 256;
  std::vector<double> part(nb);
  for (size_t b = 0; b < nb; ++b) {
    double v[256];
    for (int t = 0; t < 256; ++t) {
      size_t idx = b * 256 + t;
      v[t] = idx < n ? e[idx] : 0.0;
    }
    part[b] = tree256(v);
  }
  double v[256];
  for (int t = 0; t < 256; ++t) {
    double acc = 0.0;
    for (size_t q = t; q < nb; q += 256) acc = acc + part[q];
    v[t] = acc;
  }
  return tree256(v);
}

// ------------------------------------------------------------------ grid + transport
struct Grid {
  int nlon, nlat, nlev, lon_bc, lat_bc;
  size_t nc;
  std::vector<double> gx, gylo, gyhi;  // per lat row
};

Grid make_grid(const rs_grid* g) {
  Grid G;
  G.nlon = g->nlon; G.nlat = g->nlat; G.nlev = g->nlev;
  G.lon_bc = g->lon_bc; G.lat_bc = g->lat_bc;
  G.nc = (size_t)g->nlon * g->nlat * g->nlev;
  std::vector<double> phie(g->nlat + 1), ce(g->nlat + 1);
  for (int j = 0; j <= g->nlat; ++j) {
    double p = g->lat0_deg + (j - 0.5) * g->dlat_deg;
    p = std::min(90.0, std::max(-90.0, p));
    phie[j] = p;
    ce[j] = (std::fabs(p) >= 90.0) ? 0.0 : std::cos(p * kD2R);
  }
  double dlon = g->dlon_deg * kD2R;
  G.gx.resize(g->nlat); G.gylo.resize(g->nlat); G.gyhi.resize(g->nlat);
  for (int j = 0; j < g->nlat; ++j) {
    double dS = std::sin(phie[j + 1] * kD2R) - std::sin(phie[j] * kD2R);
    double dphi = (phie[j + 1] - phie[j]) * kD2R;
    G.gx[j] = dphi / (dlon * dS);
    G.gylo[j] = ce[j] / dS;
    G.gyhi[j] = ce[j + 1] / dS;
  }
  return G;
}

struct Forcing {
  std::vector<double> mx, my, mz, dp, qw, qe, qs, qn, T, P, emis;
  double omega = 0.0;
  // full PBL mixing (reseact.esm Transport3D p_pbl_top, pbl_f, pbl_wt, pbl_mean_*): inputs,
  // and per layer the fraction f and weight w = dp f, per column den = max(sum w, 1 Pa)
  std::vector<double> pblh, ps, hyb_a, hyb_b, pbl_f, pbl_w, pbl_den;
  double tau_pbl = 0.0;
  bool pbl = false;
  // pressure fixer (reseact.esm Transport3D divh_fix / diagnosed Mz): dPS/dt per column and
  // the per-cell correction of the horizontal divergence in the air-mass equation
  std::vector<double> dpsdt, mcorr;
  // vertical PPM coefficients per column: slope (sA,sB) for cells -1..nlev, edge (eAB,eC,eD)
  // for edges 0..nlev (edge e lies between cells e-1 and e)
  std::vector<double> vs, ve;
};

inline double dp_mirror(const double* dpcol_stride, int nlev, size_t stride, int k) {
  int kk = k < 0 ? -1 - k : (k >= nlev ? 2 * nlev - 1 - k : k);
  return dpcol_stride[(size_t)kk * stride];
}

void vertical_coefs(const Grid& G, Forcing& F) {
  int nlev = G.nlev;
  size_t ncol = (size_t)G.nlon * G.nlat;
  F.vs.assign(ncol * (nlev + 2) * 2, 0.0);
  F.ve.assign(ncol * (nlev + 1) * 3, 0.0);
  for (size_t col = 0; col < ncol; ++col) {
    const double* d = F.dp.data() + col;
    size_t st = ncol;
    for (int k = -1; k <= nlev; ++k) {  // slope coefficients (CW84 eq. 1.7)
      double D0 = dp_mirror(d, nlev, st, k - 1), D1 = dp_mirror(d, nlev, st, k),
             D2 = dp_mirror(d, nlev, st, k + 1);
      double c = D1 / (D0 + D1 + D2);
      double sA = c * (2.0 * D0 + D1) / (D2 + D1);
      double sB = c * (D1 + 2.0 * D2) / (D0 + D1);
      F.vs[(col * (nlev + 2) + (k + 1)) * 2 + 0] = sA;
      F.vs[(col * (nlev + 2) + (k + 1)) * 2 + 1] = sB;
    }
    for (int e = 0; e <= nlev; ++e) {  // edge coefficients (CW84 eq. 1.6), cells e-1 | e
      int k = e - 1;
      double Dm = dp_mirror(d, nlev, st, k - 1), D0 = dp_mirror(d, nlev, st, k),
             D1 = dp_mirror(d, nlev, st, k + 1), D2 = dp_mirror(d, nlev, st, k + 2);
      double S = Dm + D0 + D1 + D2;
      double eA = D0 / (D0 + D1);
      double t1 = (Dm + D0) / (2.0 * D0 + D1);
      double t2 = (D2 + D1) / (2.0 * D1 + D0);
      double eB = (2.0 * D1 * D0 / (D0 + D1)) * (t1 - t2) / S;
      double eC = -(D0 * t1) / S;
      double eD = D1 * (D1 + D2) / (D0 + 2.0 * D1) / S;
      F.ve[(col * (nlev + 1) + e) * 3 + 0] = eA + eB;
      F.ve[(col * (nlev + 1) + e) * 3 + 1] = eC;
      F.ve[(col * (nlev + 1) + e) * 3 + 2] = eD;
    }
  }
}

// uniform-grid monotonised slope (CW84 eq. 1.7-1.8)
inline double slope_u(double am, double a, double ap) {
  double d0 = a - am, d1 = ap - a;
  if (d1 * d0 > 0.0) {
    double da = 0.5 * (ap - am);
    double lim = std::min(2.0 * std::fabs(d0), 2.0 * std::fabs(d1));
    return std::copysign(std::min(std::fabs(da), lim), da);
  }
  return 0.0;
}
inline double slope_n(double am, double a, double ap, double sA, double sB) {
  double d0 = a - am, d1 = ap - a;
  if (d1 * d0 > 0.0) {
    double da = sA * d1 + sB * d0;
    double lim = std::min(2.0 * std::fabs(d0), 2.0 * std::fabs(d1));
    return std::copysign(std::min(std::fabs(da), lim), da);
  }
  return 0.0;
}
// CW84 eq. 1.10 parabola limiter; returns (aL, aR) of cell with mean a
inline void limit(double a, double& aL, double& aR) {
  if ((aR - a) * (a - aL) <= 0.0) {
    aL = a; aR = a;
  } else {
    double dA = aR - aL;
    double a6 = 6.0 * (a - 0.5 * (aL + aR));
    if (dA * a6 > dA * dA) aL = 3.0 * a - 2.0 * aR;
    else if (-(dA * dA) > dA * a6) aR = 3.0 * a - 2.0 * aL;
  }
}
// Uniform PPM face value from the upwind cell: vals[0..4] = a_{u-2..u+2}; side = +1 takes the
// right edge (flow in +direction), -1 the left edge.
inline double ppm_face_u(const double* v, int right) {
  double dm1 = slope_u(v[0], v[1], v[2]);
  double d0 = slope_u(v[1], v[2], v[3]);
  double dp1 = slope_u(v[2], v[3], v[4]);
  double aL = v[1] + 0.5 * (v[2] - v[1]) - (d0 - dm1) * kOneSixth;
  double aR = v[2] + 0.5 * (v[3] - v[2]) - (dp1 - d0) * kOneSixth;
  limit(v[2], aL, aR);
  return right ? aR : aL;
}

// ---- frozen-branch linearisation of the PPM face value (for the discrete adjoint) --------
// The reconstruction is piecewise linear in the five stencil values: every branch (monotone
// slope test, min/abs/copysign selections, CW84 limiter cases) is decided on VALUES, so with
// the branches frozen at the primal the face value is v . w for a weight vector w.  Lin5
// carries (value, d/dv_0..4) through the same operations to produce w.
struct Lin5 {
  double v, g[5];
};
inline Lin5 L5(double v) { Lin5 r{v, {0, 0, 0, 0, 0}}; return r; }
inline Lin5 operator+(const Lin5& a, const Lin5& b) {
  Lin5 r{a.v + b.v, {}}; for (int o = 0; o < 5; ++o) r.g[o] = a.g[o] + b.g[o]; return r; }
inline Lin5 operator-(const Lin5& a, const Lin5& b) {
  Lin5 r{a.v - b.v, {}}; for (int o = 0; o < 5; ++o) r.g[o] = a.g[o] - b.g[o]; return r; }
inline Lin5 operator*(double c, const Lin5& a) {
  Lin5 r{c * a.v, {}}; for (int o = 0; o < 5; ++o) r.g[o] = c * a.g[o]; return r; }
inline Lin5 neg(const Lin5& a) { return (-1.0) * a; }
inline Lin5 labs(const Lin5& a) { return a.v < 0.0 ? neg(a) : a; }
inline Lin5 lmin(const Lin5& a, const Lin5& b) { return (b.v < a.v) ? b : a; }
inline Lin5 lcopysign(const Lin5& mag, const Lin5& sgn) {
  bool negs = std::signbit(sgn.v), negm = std::signbit(mag.v);
  return negs == negm ? mag : neg(mag);
}
inline Lin5 slope_lu(const Lin5& am, const Lin5& a, const Lin5& ap) {
  Lin5 d0 = a - am, d1 = ap - a;
  if (d1.v * d0.v > 0.0) {
    Lin5 da = 0.5 * (ap - am);
    Lin5 lim = lmin(2.0 * labs(d0), 2.0 * labs(d1));
    return lcopysign(lmin(labs(da), lim), da);
  }
  return L5(0.0);
}
inline Lin5 slope_ln(const Lin5& am, const Lin5& a, const Lin5& ap, double sA, double sB) {
  Lin5 d0 = a - am, d1 = ap - a;
  if (d1.v * d0.v > 0.0) {
    Lin5 da = sA * d1 + sB * d0;
    Lin5 lim = lmin(2.0 * labs(d0), 2.0 * labs(d1));
    return lcopysign(lmin(labs(da), lim), da);
  }
  return L5(0.0);
}
inline void limit_l(const Lin5& a, Lin5& aL, Lin5& aR) {
  if ((aR.v - a.v) * (a.v - aL.v) <= 0.0) {
    aL = a; aR = a;
  } else {
    double dA = aR.v - aL.v;
    double a6 = 6.0 * (a.v - 0.5 * (aL.v + aR.v));
    if (dA * a6 > dA * dA) aL = 3.0 * a - 2.0 * aR;
    else if (-(dA * dA) > dA * a6) aR = 3.0 * a - 2.0 * aL;
  }
}
inline Lin5 seed(const double* v, int o) { Lin5 r = L5(v[o]); r.g[o] = 1.0; return r; }
// weights of the uniform-grid upwind face value w.r.t. v[0..4]
inline void face_weights_u(const double* v, bool right, double* w) {
  Lin5 x[5];
  for (int o = 0; o < 5; ++o) x[o] = seed(v, o);
  Lin5 dm1 = slope_lu(x[0], x[1], x[2]), d0 = slope_lu(x[1], x[2], x[3]),
       dp1 = slope_lu(x[2], x[3], x[4]);
  Lin5 aL = x[1] + 0.5 * (x[2] - x[1]) - kOneSixth * (d0 - dm1);
  Lin5 aR = x[2] + 0.5 * (x[3] - x[2]) - kOneSixth * (dp1 - d0);
  limit_l(x[2], aL, aR);
  const Lin5& r = right ? aR : aL;
  for (int o = 0; o < 5; ++o) w[o] = r.g[o];
}

struct MacroRec {  // one recorded macro step (Ckpt of tools/adjoint_gradient.jl:621)
  std::vector<double> u;
  double t0, t1;
  std::vector<std::pair<double, double>> seqT, seqC;
};

struct Model {
  std::vector<MacroRec> recs;
  Grid G;
  Mech M;
  int nsp;  // species per cell in the state (chem species + air mass)
  int has_m;
  rs_config cfg;
  Forcing F;
  std::vector<double> krates;  // [nr][nc]
  std::vector<int> ord;        // LU elimination order (species per pivot); empty: natural
};

// value of species s (state plane q) at lon index i (ghosts per BC), lat j, lev k
inline double qx(const Model& md, const double* q, int s, int i, int j, int k) {
  const Grid& G = md.G;
  if (i < 0 || i >= G.nlon) {
    if (G.lon_bc == RS_BC_PERIODIC) i = ((i % G.nlon) + G.nlon) % G.nlon;
    else {
      const std::vector<double>& b = (i < 0) ? md.F.qw : md.F.qe;
      return b[((size_t)s * G.nlev + k) * G.nlat + j];
    }
  }
  return q[((size_t)k * G.nlat + j) * G.nlon + i];
}
inline double qy(const Model& md, const double* q, int s, int i, int j, int k) {
  const Grid& G = md.G;
  if (j < 0 || j >= G.nlat) {
    if (G.lat_bc == RS_BC_OPEN) {
      const std::vector<double>& b = (j < 0) ? md.F.qs : md.F.qn;
      return b[((size_t)s * G.nlev + k) * G.nlon + i];
    }
    j = j < 0 ? -1 - j : 2 * G.nlat - 1 - j;
  }
  return q[((size_t)k * G.nlat + j) * G.nlon + i];
}
inline double qz(const Model& md, const double* q, int i, int j, int k) {
  const Grid& G = md.G;
  int kk = k < 0 ? -1 - k : (k >= G.nlev ? 2 * G.nlev - 1 - k : k);
  return q[((size_t)kk * G.nlat + j) * G.nlon + i];
}

// face fluxes of tracer s at cell (i,j,k): west/east, south/north, bottom/top
// PBL fraction and weights of every layer, as the reseact.esm Transport3D equations define them:
// p_top = PS exp(-(PBLH g)/(Rd T_surface)); f_k = max(0, min(1, (min(PS, p_k) - max(p_top,
// p_k+1))/dp_k)) with interface p_k = A_k + B_k PS (k = 0 at the surface); den = max(sum w, 1).
void build_pbl(const Grid& G, Forcing& F) {
  size_t ncol = (size_t)G.nlon * G.nlat;
  F.pbl = F.tau_pbl > 0.0 && F.pblh.size() == ncol && F.ps.size() == ncol && !F.T.empty() &&
          F.hyb_a.size() == (size_t)G.nlev + 1 && F.hyb_b.size() == (size_t)G.nlev + 1;
  if (!F.pbl) return;
  const double g_acc = 9.80665, rd_air = 287.05;
  F.pbl_f.assign(G.nc, 0.0);
  F.pbl_w.assign(G.nc, 0.0);
  F.pbl_den.assign(ncol, 0.0);
  for (size_t col = 0; col < ncol; ++col) {
    double PS = F.ps[col];
    double ptop = PS * std::exp(-1.0 * ((F.pblh[col] * g_acc) / (rd_air * F.T[col])));
    double wt = 0.0;
    for (int k = 0; k < G.nlev; ++k) {
      size_t c = (size_t)k * ncol + col;
      double lo = F.hyb_a[k] + F.hyb_b[k] * PS, up = F.hyb_a[k + 1] + F.hyb_b[k + 1] * PS;
      double f = std::max(0.0, std::min(1.0, (std::min(PS, lo) - std::max(ptop, up)) / F.dp[c]));
      F.pbl_f[c] = f;
      F.pbl_w[c] = F.dp[c] * f;
      wt = wt + F.pbl_w[c];
    }
    F.pbl_den[col] = std::max(wt, 1.0);
  }
}

// Pressure fixer, per column with sums from the surface up (reseact.esm Transport3D divh,
// divh_col, dp_col, divh_fix, Mz): corr_k = (-dPSdt - sum_k divh_k) * (dp_k / sum_k dp_k),
// Mz_{k+1} = Mz_k + -(dB_k dPSdt + (divh_k + corr_k)) with Mz_0 = 0; Mz replaces the given mz.
void build_fixer(const Grid& G, Forcing& F) {
  size_t ncol = (size_t)G.nlon * G.nlat, nf = (size_t)G.nlon + 1;
  F.mcorr.clear();
  if (F.dpsdt.size() != ncol || F.hyb_b.size() != (size_t)G.nlev + 1 || F.mx.empty() ||
      F.my.empty())
    return;
  bool open_lat = G.lat_bc == RS_BC_OPEN;
  std::vector<double> divh(G.nc);
  F.mcorr.assign(G.nc, 0.0);
  F.mz.assign((size_t)(G.nlev + 1) * ncol, 0.0);
  for (int j = 0; j < G.nlat; ++j)
    for (int i = 0; i < G.nlon; ++i) {
      size_t col = (size_t)j * G.nlon + i;
      double hcol = 0.0, dcol = 0.0;
      for (int k = 0; k < G.nlev; ++k) {
        size_t c = (size_t)k * ncol + col;
        double mxw = F.mx[((size_t)k * G.nlat + j) * nf + i];
        double mxe = F.mx[((size_t)k * G.nlat + j) * nf + i + 1];
        double mys = (!open_lat && j == 0) ? 0.0 : F.my[((size_t)k * (G.nlat + 1) + j) * G.nlon + i];
        double myn = (!open_lat && j + 1 == G.nlat) ? 0.0
                   : F.my[((size_t)k * (G.nlat + 1) + j + 1) * G.nlon + i];
        double DxM = (mxe - mxw) * G.gx[j];
        double DyM = myn * G.gyhi[j] - mys * G.gylo[j];
        divh[c] = DxM + DyM;
        hcol = hcol + divh[c];
        dcol = dcol + F.dp[c];
      }
      double dps = F.dpsdt[col], acc = 0.0;
      for (int k = 0; k < G.nlev; ++k) {
        size_t c = (size_t)k * ncol + col;
        F.mcorr[c] = (-dps - hcol) * (F.dp[c] / dcol);
        double fix = divh[c] + F.mcorr[c];
        acc = acc + -((F.hyb_b[k] - F.hyb_b[k + 1]) * dps + fix);
        F.mz[(size_t)(k + 1) * ncol + col] = acc;
      }
    }
}

double xflux(const Model& md, const double* q, int s, int i, int j, int k, double g) {
  const Grid& G = md.G;
  double M = g * md.F.mx[((size_t)k * G.nlat + j) * (G.nlon + 1) + i];
  int up = M > 0.0 ? i - 1 : i;
  double v[5];
  for (int o = 0; o < 5; ++o) v[o] = qx(md, q, s, up - 2 + o, j, k);
  return M * ppm_face_u(v, M > 0.0);
}
double yflux(const Model& md, const double* q, int s, int i, int j, int k, double g) {
  const Grid& G = md.G;
  if (G.lat_bc != RS_BC_OPEN && (j == 0 || j == G.nlat)) return 0.0;
  double M = g * md.F.my[((size_t)k * (G.nlat + 1) + j) * G.nlon + i];
  int up = M > 0.0 ? j - 1 : j;
  double v[5];
  for (int o = 0; o < 5; ++o) v[o] = qy(md, q, s, i, up - 2 + o, k);
  return M * ppm_face_u(v, M > 0.0);
}
double zflux(const Model& md, const double* q, int i, int j, int kf, double g) {
  const Grid& G = md.G;
  if (kf == 0 || kf == G.nlev) return 0.0;
  size_t ncol = (size_t)G.nlon * G.nlat, col = (size_t)j * G.nlon + i;
  double M = g * md.F.mz[(size_t)kf * ncol + col];
  int up = M > 0.0 ? kf - 1 : kf;
  double v[5];
  for (int o = 0; o < 5; ++o) v[o] = qz(md, q, i, j, up - 2 + o);
  const double* vs = md.F.vs.data() + col * (G.nlev + 2) * 2;
  const double* ve = md.F.ve.data() + col * (G.nlev + 1) * 3;
  auto sl = [&](int c, double am, double a, double ap) {
    return slope_n(am, a, ap, vs[(c + 1) * 2], vs[(c + 1) * 2 + 1]);
  };
  double dm1 = sl(up - 1, v[0], v[1], v[2]);
  double d0 = sl(up, v[1], v[2], v[3]);
  double dp1 = sl(up + 1, v[2], v[3], v[4]);
  const double* eL = ve + (size_t)up * 3;        // edge between up-1 | up
  const double* eR = ve + (size_t)(up + 1) * 3;  // edge between up | up+1
  double aL = v[1] + eL[0] * (v[2] - v[1]) + eL[1] * d0 + eL[2] * dm1;
  double aR = v[2] + eR[0] * (v[3] - v[2]) + eR[1] * dp1 + eR[2] * d0;
  limit(v[2], aL, aR);
  return M * (M > 0.0 ? aR : aL);
}

// Transport RHS (CWC mixing-ratio form, reseact.esm:2083; continuity reseact.esm:1535).
// with_pbl = false gives the advective tendency alone (the adjoint's air-mass derivative)
void transport_rhs(const Model& md, const double* u, double t, double* du, bool with_pbl = true) {
  const Grid& G = md.G;
  double g = md.F.omega != 0.0 ? std::cos(md.F.omega * t) : 1.0;
  size_t nc = G.nc;
  int ntr = md.has_m ? md.nsp - 1 : md.nsp;
  const double* m = md.has_m ? u + (size_t)(md.nsp - 1) * nc : nullptr;
  const bool pbl = with_pbl && md.F.pbl;
  const size_t ncol0 = (size_t)G.nlon * G.nlat;
  std::vector<double> qbar;
  if (pbl) {  // PBL mean of every tracer and column, summed from the surface up
    qbar.assign((size_t)ntr * ncol0, 0.0);
    for (int s = 0; s < ntr; ++s)
      for (size_t col = 0; col < ncol0; ++col) {
        double acc = 0.0;
        for (int k = 0; k < G.nlev; ++k)
          acc = acc + md.F.pbl_w[(size_t)k * ncol0 + col] * u[(size_t)s * nc + (size_t)k * ncol0 + col];
        qbar[(size_t)s * ncol0 + col] = acc / md.F.pbl_den[col];
      }
  }
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < G.nlev; ++k)
    for (int j = 0; j < G.nlat; ++j)
      for (int i = 0; i < G.nlon; ++i) {
        size_t c = ((size_t)k * G.nlat + j) * G.nlon + i;
        size_t ncol = (size_t)G.nlon * G.nlat, col = (size_t)j * G.nlon + i;
        double mxw = g * md.F.mx[((size_t)k * G.nlat + j) * (G.nlon + 1) + i];
        double mxe = g * md.F.mx[((size_t)k * G.nlat + j) * (G.nlon + 1) + i + 1];
        double mys = (G.lat_bc != RS_BC_OPEN && j == 0) ? 0.0
                   : g * md.F.my[((size_t)k * (G.nlat + 1) + j) * G.nlon + i];
        double myn = (G.lat_bc != RS_BC_OPEN && j + 1 == G.nlat) ? 0.0
                   : g * md.F.my[((size_t)k * (G.nlat + 1) + j + 1) * G.nlon + i];
        double mzb = (k == 0) ? 0.0 : g * md.F.mz[(size_t)k * ncol + col];
        double mzt = (k + 1 == G.nlev) ? 0.0 : g * md.F.mz[(size_t)(k + 1) * ncol + col];
        double DxM = (mxe - mxw) * G.gx[j];
        double DyM = myn * G.gyhi[j] - mys * G.gylo[j];
        double DzM = mzt - mzb;
        double divM = (DxM + DyM) + DzM;
        for (int s = 0; s < ntr; ++s) {
          const double* q = u + (size_t)s * nc;
          double fw = xflux(md, q, s, i, j, k, g), fe = xflux(md, q, s, i + 1, j, k, g);
          double fs = yflux(md, q, s, i, j, k, g), fn = yflux(md, q, s, i, j + 1, k, g);
          double fb = zflux(md, q, i, j, k, g), ft = zflux(md, q, i, j, k + 1, g);
          double Dx = (fe - fw) * G.gx[j];
          double Dy = fn * G.gyhi[j] - fs * G.gylo[j];
          double Dz = ft - fb;
          double a = -((Dx + Dy) + Dz);
          double b = q[c] * divM;
          double adv = m ? (a + b) / m[c] : a + b;
          if (pbl)  // full PBL mixing: pbl_f * (pbl_mean - q) / tau_pblmix
            adv = adv + (md.F.pbl_f[c] * (qbar[(size_t)s * ncol0 + col] - q[c])) / md.F.tau_pbl;
          du[(size_t)s * nc + c] = adv;
        }
        if (md.has_m)  // with the pressure fixer: -((divh + corr) + DzM)
          du[(size_t)(md.nsp - 1) * nc + c] =
              md.F.mcorr.empty() ? -divM : -(((DxM + DyM) + md.F.mcorr[c]) + DzM);
      }
}

// per-cell contribution to the hairer norm: sum over species of (err/den)^2
inline double cell_err(const Model& md, const double* u, const double* unew, const double* err,
                       size_t c, double atol, double rtol) {
  double acc = 0.0;
  for (int s = 0; s < md.nsp; ++s) {
    size_t x = (size_t)s * md.G.nc + c;
    double am = std::max(std::fabs(u[x]), std::fabs(unew[x]));
    double den = am * rtol + atol;
    double at = err[x] / den;
    acc = acc + at * at;
  }
  return acc;
}

// SSPRK43 attempt (rx_traced_integrator.jl:362-400).  Returns EEst.
double ssprk43_step(const Model& md, const double* u, double t, double dt, double* unew,
                    std::vector<double>& w) {
  size_t n = (size_t)md.nsp * md.G.nc;
  w.resize(3 * n);
  double* u3 = w.data();
  double* k = w.data() + n;
  double* ut = w.data() + 2 * n;
  double dt_2 = dt / 2;
  std::copy(u, u + n, u3);
  for (int i = 1; i <= 3; ++i) {
    double ci = 0.5 * (i - 1);
    transport_rhs(md, u3, t + ci * dt, k);
#pragma omp parallel for schedule(static)
    for (size_t x = 0; x < n; ++x) u3[x] = u3[x] + dt_2 * k[x];
  }
  std::vector<double> u4(n);
#pragma omp parallel for schedule(static)
  for (size_t x = 0; x < n; ++x) {
    ut[x] = (1.0 / 3.0) * u[x] + (2.0 / 3.0) * u3[x];
    u4[x] = (2.0 / 3.0) * u[x] + (1.0 / 3.0) * u3[x];
  }
  transport_rhs(md, u4.data(), t + dt_2, k);
#pragma omp parallel for schedule(static)
  for (size_t x = 0; x < n; ++x) {
    unew[x] = u4[x] + dt_2 * k[x];
    ut[x] = 0.5 * (ut[x] - unew[x]);
  }
  std::vector<double> e(md.G.nc);
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < md.G.nc; ++c) e[c] = cell_err(md, u, unew, ut, c, md.cfg.atol_T, md.cfg.rtol_T);
  double sse = reduce_fixed(e.data(), md.G.nc);
  return std::sqrt(sse / (double)n);
}

const double kRosD = 1.0 / (2.0 + std::sqrt(2.0));
const double kRosC32 = 6.0 + std::sqrt(2.0);

// ROS23 attempt of one cell (rx_traced_integrator.jl:279-349), writes unew and the cell's
// error residual utilde; chemistry never couples cells.
void ros23_cell(const Model& md, const double* kr, const double* x, const double* emis, double t,
                double dt, double* unew, double* ut) {
  const Mech& M = md.M;
  int n = M.ns;
  double f0[64], f1[64], f2[64], k1[64], k2[64], k3[64], b[64], u1[64], xn[64], vb[256];
  std::vector<double> J(n * n), W(n * n);
  chem_rhs_cell(M, kr, x, emis, f0, vb);
  chem_jac_cell(M, kr, x, J.data());
  double dtgamma = dt * kRosD;
  for (int r = 0; r < n; ++r)
    for (int s = 0; s < n; ++s) {
      double tmp = dtgamma * J[r * n + s];
      W[r * n + s] = r == s ? 1.0 - tmp : 0.0 - tmp;
    }
  lu_factor_ord(md.ord, n, W);
  lu_solve_ord(md.ord, n, W.data(), f0, k1);
  double dto2 = dt / 2;
  for (int s = 0; s < n; ++s) u1[s] = x[s] + dto2 * k1[s];
  chem_rhs_cell(M, kr, u1, emis, f1, vb);
  for (int s = 0; s < n; ++s) b[s] = f1[s] - k1[s];
  lu_solve_ord(md.ord, n, W.data(), b, k2);
  for (int s = 0; s < n; ++s) k2[s] = k2[s] + k1[s];
  for (int s = 0; s < n; ++s) xn[s] = x[s] + dt * k2[s];
  chem_rhs_cell(M, kr, xn, emis, f2, vb);
  for (int s = 0; s < n; ++s) {
    double a = kRosC32 * (k2[s] - f1[s]);
    double c = 2.0 * (k1[s] - f0[s]);
    b[s] = (f2[s] - a) - c;
  }
  lu_solve_ord(md.ord, n, W.data(), b, k3);
  double dto6 = dt / 6;
  for (int s = 0; s < n; ++s) {
    unew[s] = xn[s];
    ut[s] = dto6 * ((k1[s] - 2.0 * k2[s]) + k3[s]);
  }
  (void)t;
}

double ros23_step(const Model& md, const double* u, double t, double dt, double* unew,
                  std::vector<double>& w) {
  size_t nc = md.G.nc, n = (size_t)md.nsp * nc;
  int ns = md.M.ns;
  w.resize(n);
  double* ut = w.data();
  const bool has_emis = !md.F.emis.empty();
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < nc; ++c) {
    double x[64], xn[64], e[64], kr[256], em[64];
    for (int s = 0; s < ns; ++s) x[s] = u[(size_t)s * nc + c];
    for (int r = 0; r < md.M.nr; ++r) kr[r] = md.krates[(size_t)r * nc + c];
    if (has_emis)
      for (int s = 0; s < ns; ++s) em[s] = md.F.emis[(size_t)s * nc + c];
    ros23_cell(md, kr, x, has_emis ? em : nullptr, t, dt, xn, e);
    for (int s = 0; s < ns; ++s) {
      unew[(size_t)s * nc + c] = xn[s];
      ut[(size_t)s * nc + c] = e[s];
    }
    for (int s = ns; s < md.nsp; ++s) {  // inert air mass: f = 0, J row = 0
      unew[(size_t)s * nc + c] = u[(size_t)s * nc + c];
      ut[(size_t)s * nc + c] = 0.0;
    }
  }
  std::vector<double> e(nc);
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < nc; ++c) e[c] = cell_err(md, u, unew, ut, c, md.cfg.atol_C, md.cfg.rtol_C);
  double sse = reduce_fixed(e.data(), nc);
  return std::sqrt(sse / (double)n);
}

// adaptive_solve (rx_traced_integrator.jl:455-507)
struct SolveOut { double t, dt, nacc, nrej, iters; };
using StepSeq = std::vector<std::pair<double, double>>;  // accepted (t, dt)

template <class Step>
SolveOut adaptive_solve(Step step, std::vector<double>& u, double t0, double tend, double dt0,
                        const rs_controller& c, double maxiters, bool clamp,
                        StepSeq* seq = nullptr) {
  size_t n = u.size();
  std::vector<double> unew(n);
  double beta1 = c.beta1, beta2 = c.beta2;
  double invqmax = 1.0 / c.qmax, invqmin = 1.0 / c.qmin, gamma = c.gamma;
  double t = t0, dt = dt0, qold = c.qoldinit, nacc = 0, nrej = 0, iters = 0;
  double tlim = tend - 1.0e-9;
  while ((t < tlim) && (iters < maxiters)) {
    double dtc = std::min(dt, tend - t);
    double EEst = step(u.data(), t, dtc, unew.data());
    if (clamp)
      for (size_t x = 0; x < n; ++x) unew[x] = std::max(unew[x], 0.0);
    if (std::isnan(EEst)) EEst = 1.0e10;
    double q11 = std::pow(std::max(EEst, 1.0e-35), beta1);
    double qden = std::pow(qold, beta2);
    double q = q11 / qden;
    q = std::max(invqmax, std::min(invqmin, q / gamma));
    bool accept = EEst <= 1.0;
    bool insteady = (c.qsteady_min <= q) && (q <= c.qsteady_max);
    double qa = insteady ? 1.0 : q;
    double dt_acc = dtc / qa;
    double qr = std::min(invqmin, q11 / gamma);
    double dt_rej = dtc / qr;
    if (accept) {
      if (seq) seq->push_back({t, dtc});
      u.swap(unew);
      t = t + dtc;
      dt = dt_acc;
      qold = std::max(EEst, c.qoldinit);
      nacc += 1.0;
    } else {
      dt = dt_rej;
      nrej += 1.0;
    }
    iters += 1.0;
  }
  return {t, dt, nacc, nrej, iters};
}

// ====================================================================== discrete adjoint
// One-step VJPs at fixed dt with the clamp and the controller treated as the discrete
// decisions they are (rx_traced_integrator.jl:509-623; tools/adjoint_gradient.jl:731-835):
// lambda_in = (du_out/du_in)^T lambda_out, plus d/d(emission) for the chemistry steps.

// stencil position p along x/y/z of cell (i,j,k) -> state cell index, or -1 for a boundary
// ghost that carries no state (open walls)
inline long map_x(const Grid& G, int p, int j, int k) {
  if (p < 0 || p >= G.nlon) {
    if (G.lon_bc != RS_BC_PERIODIC) return -1;
    p = ((p % G.nlon) + G.nlon) % G.nlon;
  }
  return ((long)k * G.nlat + j) * G.nlon + p;
}
inline long map_y(const Grid& G, int i, int p, int k) {
  if (p < 0 || p >= G.nlat) {
    if (G.lat_bc == RS_BC_OPEN) return -1;
    p = p < 0 ? -1 - p : 2 * G.nlat - 1 - p;
  }
  return ((long)k * G.nlat + p) * G.nlon + i;
}
inline long map_z(const Grid& G, int i, int j, int p) {
  if (p < 0 || p >= G.nlev) p = p < 0 ? -1 - p : 2 * G.nlev - 1 - p;
  return ((long)p * G.nlat + j) * G.nlon + i;
}

// ubar = (d f_transport / du)^T fbar at state u, time t (all species incl. air mass)
void transport_rhs_vjp(const Model& md, const double* u, double t, const double* fbar,
                       double* ubar) {
  const Grid& G = md.G;
  double g = md.F.omega != 0.0 ? std::cos(md.F.omega * t) : 1.0;
  size_t nc = G.nc;
  int ntr = md.nsp - 1;
  const double* m = u + (size_t)ntr * nc;
  std::vector<double> f((size_t)md.nsp * nc);
  transport_rhs(md, u, t, f.data(), false);  // advective part: the air mass enters only there
  std::fill(ubar, ubar + (size_t)md.nsp * nc, 0.0);
  if (md.F.pbl) {  // PBL mixing: ubar_j += (w_j/den) (sum_k fbar_k f_k)/tau - fbar_j f_j/tau
    size_t ncol0 = (size_t)G.nlon * G.nlat;
    for (int s = 0; s < ntr; ++s)
      for (size_t col = 0; col < ncol0; ++col) {
        double a = 0.0;
        for (int k = 0; k < G.nlev; ++k) {
          size_t x = (size_t)k * ncol0 + col;
          a = a + fbar[(size_t)s * nc + x] * md.F.pbl_f[x];
        }
        double at = a / md.F.tau_pbl, den = md.F.pbl_den[col];
        for (int k = 0; k < G.nlev; ++k) {
          size_t x = (size_t)k * ncol0 + col;
          ubar[(size_t)s * nc + x] += (md.F.pbl_w[x] / den) * at -
                                      (fbar[(size_t)s * nc + x] * md.F.pbl_f[x]) / md.F.tau_pbl;
        }
      }
  }
  std::vector<double> gq((size_t)ntr * nc);
  size_t ncol = (size_t)G.nlon * G.nlat;
  for (int k = 0; k < G.nlev; ++k)
    for (int j = 0; j < G.nlat; ++j)
      for (int i = 0; i < G.nlon; ++i) {
        size_t c = ((size_t)k * G.nlat + j) * G.nlon + i, col = (size_t)j * G.nlon + i;
        double mxw = g * md.F.mx[((size_t)k * G.nlat + j) * (G.nlon + 1) + i];
        double mxe = g * md.F.mx[((size_t)k * G.nlat + j) * (G.nlon + 1) + i + 1];
        double mys = (G.lat_bc != RS_BC_OPEN && j == 0) ? 0.0
                   : g * md.F.my[((size_t)k * (G.nlat + 1) + j) * G.nlon + i];
        double myn = (G.lat_bc != RS_BC_OPEN && j + 1 == G.nlat) ? 0.0
                   : g * md.F.my[((size_t)k * (G.nlat + 1) + j + 1) * G.nlon + i];
        double mzb = (k == 0) ? 0.0 : g * md.F.mz[(size_t)k * ncol + col];
        double mzt = (k + 1 == G.nlev) ? 0.0 : g * md.F.mz[(size_t)(k + 1) * ncol + col];
        double divM = ((mxe - mxw) * G.gx[j] + (myn * G.gyhi[j] - mys * G.gylo[j])) + (mzt - mzb);
        double mb = 0.0;
        for (int s = 0; s < ntr; ++s) {
          double gs = fbar[(size_t)s * nc + c] / m[c];
          gq[(size_t)s * nc + c] = gs;
          ubar[(size_t)s * nc + c] += gs * divM;
          mb -= gs * f[(size_t)s * nc + c];
        }
        ubar[(size_t)ntr * nc + c] += mb;
      }
  // x faces
  for (int k = 0; k < G.nlev; ++k)
    for (int j = 0; j < G.nlat; ++j)
      for (int fi = 0; fi <= G.nlon; ++fi) {
        double M = g * md.F.mx[((size_t)k * G.nlat + j) * (G.nlon + 1) + fi];
        bool right = M > 0.0;
        int up = right ? fi - 1 : fi;
        for (int s = 0; s < ntr; ++s) {
          const double* q = u + (size_t)s * nc;
          double v[5], w[5];
          for (int o = 0; o < 5; ++o) v[o] = qx(md, q, s, up - 2 + o, j, k);
          face_weights_u(v, right, w);
          double Fb = 0.0;
          if (fi >= 1) Fb -= gq[(size_t)s * nc + ((size_t)k * G.nlat + j) * G.nlon + fi - 1] * G.gx[j];
          if (fi < G.nlon) Fb += gq[(size_t)s * nc + ((size_t)k * G.nlat + j) * G.nlon + fi] * G.gx[j];
          for (int o = 0; o < 5; ++o) {
            long cc = map_x(G, up - 2 + o, j, k);
            if (cc >= 0) ubar[(size_t)s * nc + cc] += Fb * M * w[o];
          }
        }
      }
  // y faces
  for (int k = 0; k < G.nlev; ++k)
    for (int fj = 0; fj <= G.nlat; ++fj) {
      if (G.lat_bc != RS_BC_OPEN && (fj == 0 || fj == G.nlat)) continue;
      for (int i = 0; i < G.nlon; ++i) {
        double M = g * md.F.my[((size_t)k * (G.nlat + 1) + fj) * G.nlon + i];
        bool right = M > 0.0;
        int up = right ? fj - 1 : fj;
        for (int s = 0; s < ntr; ++s) {
          const double* q = u + (size_t)s * nc;
          double v[5], w[5];
          for (int o = 0; o < 5; ++o) v[o] = qy(md, q, s, i, up - 2 + o, k);
          face_weights_u(v, right, w);
          double Fb = 0.0;
          if (fj >= 1) Fb -= gq[(size_t)s * nc + ((size_t)k * G.nlat + fj - 1) * G.nlon + i] * G.gyhi[fj - 1];
          if (fj < G.nlat) Fb += gq[(size_t)s * nc + ((size_t)k * G.nlat + fj) * G.nlon + i] * G.gylo[fj];
          for (int o = 0; o < 5; ++o) {
            long cc = map_y(G, i, up - 2 + o, k);
            if (cc >= 0) ubar[(size_t)s * nc + cc] += Fb * M * w[o];
          }
        }
      }
    }
  // z faces (walls carry no flux)
  for (int kf = 1; kf < G.nlev; ++kf)
    for (int j = 0; j < G.nlat; ++j)
      for (int i = 0; i < G.nlon; ++i) {
        size_t col = (size_t)j * G.nlon + i;
        double M = g * md.F.mz[(size_t)kf * ncol + col];
        bool right = M > 0.0;
        int up = right ? kf - 1 : kf;
        const double* vs = md.F.vs.data() + col * (G.nlev + 2) * 2;
        const double* ve = md.F.ve.data() + col * (G.nlev + 1) * 3;
        for (int s = 0; s < ntr; ++s) {
          const double* q = u + (size_t)s * nc;
          Lin5 x[5];
          for (int o = 0; o < 5; ++o) {
            double vo = qz(md, q, i, j, up - 2 + o);
            x[o] = L5(vo);
            x[o].g[o] = 1.0;
          }
          auto sl = [&](int cidx, const Lin5& a0, const Lin5& a1, const Lin5& a2) {
            return slope_ln(a0, a1, a2, vs[(cidx + 1) * 2], vs[(cidx + 1) * 2 + 1]);
          };
          Lin5 dm1 = sl(up - 1, x[0], x[1], x[2]), d0 = sl(up, x[1], x[2], x[3]),
               dp1 = sl(up + 1, x[2], x[3], x[4]);
          const double* eL = ve + (size_t)up * 3;
          const double* eR = ve + (size_t)(up + 1) * 3;
          Lin5 aL = x[1] + eL[0] * (x[2] - x[1]) + eL[1] * d0 + eL[2] * dm1;
          Lin5 aR = x[2] + eR[0] * (x[3] - x[2]) + eR[1] * dp1 + eR[2] * d0;
          limit_l(x[2], aL, aR);
          const Lin5& r = right ? aR : aL;
          double Fb = -gq[(size_t)s * nc + (size_t)(kf - 1) * ncol + col] +
                      gq[(size_t)s * nc + (size_t)kf * ncol + col];
          for (int o = 0; o < 5; ++o) {
            long cc = map_z(G, i, j, up - 2 + o);
            ubar[(size_t)s * nc + cc] += Fb * M * r.g[o];
          }
        }
      }
}

// lam_in = (d unew / du)^T lam for one SSPRK43 step at fixed (t, dt)
void ssprk43_vjp(const Model& md, const double* u, double t, double dt, const double* lam,
                 double* lam_in) {
  size_t n = (size_t)md.nsp * md.G.nc;
  double h = dt / 2;
  std::vector<double> f(n), u1(n), u2(n), u4(n), a(n), b(n), w(n);
  transport_rhs(md, u, t, f.data());
  for (size_t x = 0; x < n; ++x) u1[x] = u[x] + h * f[x];
  transport_rhs(md, u1.data(), t + 0.5 * dt, f.data());
  for (size_t x = 0; x < n; ++x) u2[x] = u1[x] + h * f[x];
  transport_rhs(md, u2.data(), t + 1.0 * dt, f.data());
  for (size_t x = 0; x < n; ++x) u4[x] = (2.0 / 3.0) * u[x] + (1.0 / 3.0) * (u2[x] + h * f[x]);
  // unew = u4 + h f(u4)
  for (size_t x = 0; x < n; ++x) w[x] = h * lam[x];
  transport_rhs_vjp(md, u4.data(), t + h, w.data(), a.data());
  for (size_t x = 0; x < n; ++x) a[x] += lam[x];          // ubar4
  for (size_t x = 0; x < n; ++x) {
    lam_in[x] = (2.0 / 3.0) * a[x];                        // via u4 = 2/3 u + 1/3 u3
    b[x] = (1.0 / 3.0) * a[x];                             // ubar3 = ubar2 (+ f2 path)
    w[x] = h * b[x];
  }
  transport_rhs_vjp(md, u2.data(), t + 1.0 * dt, w.data(), a.data());
  for (size_t x = 0; x < n; ++x) { b[x] += a[x]; w[x] = h * b[x]; }   // ubar2 -> ubar1
  transport_rhs_vjp(md, u1.data(), t + 0.5 * dt, w.data(), a.data());
  for (size_t x = 0; x < n; ++x) { b[x] += a[x]; w[x] = h * b[x]; }   // ubar1 -> ubar0
  transport_rhs_vjp(md, u, t, w.data(), a.data());
  for (size_t x = 0; x < n; ++x) lam_in[x] += b[x] + a[x];
}

// d^2 v_r / dx_a dx_b (a, b species of reactant entries of r)
inline double d2vel(const Mech& M, int r, double k, const double* x, int a, int b) {
  double d = k;
  for (int e = M.rptr[r]; e < M.rptr[r + 1]; ++e) {
    int s = M.rsp[e], nu = M.rnu[e];
    int order = (s == a) + (s == b);
    if (order > nu) return 0.0;
    double c = 1.0;
    for (int t = 0; t < order; ++t) c *= (double)(nu - t);
    for (int t = 0; t < nu - order; ++t) c *= x[s];
    d *= c;
  }
  return d;
}

// one ROS23 step VJP of one cell: lam (d J / d unew) -> ubar (d J / d u), ebar += d J / d emis
void ros23_vjp_cell(const Model& md, const double* kr, const double* x, const double* emis,
                    double dt, const double* lam, double* ubar, double* ebar) {
  const Mech& M = md.M;
  int n = M.ns;
  double f0[64], k1[64], u1[64], f1[64], b2[64], z2[64], vb[256];
  std::vector<double> J(n * n), W(n * n), J1(n * n);
  chem_rhs_cell(M, kr, x, emis, f0, vb);
  chem_jac_cell(M, kr, x, J.data());
  double dtgamma = dt * kRosD;
  for (int r = 0; r < n; ++r)
    for (int s = 0; s < n; ++s) W[r * n + s] = (r == s ? 1.0 : 0.0) - dtgamma * J[r * n + s];
  std::vector<double> LU(W);
  const std::vector<int>& ord = md.ord;
  lu_factor_ord(ord, n, LU);
  lu_solve_ord(ord, n, LU.data(), f0, k1);
  for (int s = 0; s < n; ++s) u1[s] = x[s] + (dt / 2) * k1[s];
  chem_rhs_cell(M, kr, u1, emis, f1, vb);
  for (int s = 0; s < n; ++s) b2[s] = f1[s] - k1[s];
  lu_solve_ord(ord, n, LU.data(), b2, z2);
  // transposed solves with the same factors: W^T y = c
  auto solveT = [&](const double* cs, double* ys) {
    // P W P^T = L U (unit L); W^T = P^T U^T L^T P: forward with U^T, then backward with L^T,
    // on the permuted vectors
    double c[64], y[64], t1[64];
    for (int i = 0; i < n; ++i) c[i] = ord.empty() ? cs[i] : cs[ord[i]];
    for (int i = 0; i < n; ++i) {
      double acc = c[i];
      for (int j = 0; j < i; ++j) acc -= LU[j * n + i] * t1[j];
      t1[i] = acc / LU[i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double acc = t1[i];
      for (int j = i + 1; j < n; ++j) acc -= LU[j * n + i] * y[j];
      y[i] = acc;
    }
    for (int i = 0; i < n; ++i) ys[ord.empty() ? i : ord[i]] = y[i];
  };
  double k2b[64], k1b[64], b2b[64], f1b[64], u1b[64], f0b[64];
  for (int s = 0; s < n; ++s) { ubar[s] = lam[s]; k2b[s] = dt * lam[s]; k1b[s] = k2b[s]; }
  solveT(k2b, b2b);                       // b2bar = W^-T k2bar  (z2bar = k2bar)
  for (int s = 0; s < n; ++s) { f1b[s] = b2b[s]; k1b[s] -= b2b[s]; }
  chem_jac_cell(M, kr, u1, J1.data());
  for (int q = 0; q < n; ++q) {           // u1bar = J(u1)^T f1bar
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc += J1[i * n + q] * f1b[i];
    u1b[q] = acc;
  }
  for (int s = 0; s < n; ++s) { ubar[s] += u1b[s]; k1b[s] += (dt / 2) * u1b[s]; }
  solveT(k1b, f0b);                       // f0bar = W^-T k1bar
  for (int q = 0; q < n; ++q) {           // u += J(u)^T f0bar
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc += J[i * n + q] * f0b[i];
    ubar[q] += acc;
  }
  if (ebar)
    for (int s = 0; s < n; ++s) ebar[s] += f0b[s] + f1b[s];
  // Jbar = -dtgamma * Wbar, Wbar = -(b2bar z2^T + f0bar k1^T)  =>  Jbar = dtgamma (...)
  // u_q += sum_r sum_j (sum_i Jbar_ij net_ri) d2v_r/dx_j dx_q
  for (int r = 0; r < M.nr; ++r) {
    for (int ea = M.rptr[r]; ea < M.rptr[r + 1]; ++ea) {
      int j = M.rsp[ea];
      double gj = 0.0;
      for (int i = 0; i < n; ++i) {
        double c = M.net[(size_t)r * n + i];
        if (c != 0.0) gj += c * dtgamma * (b2b[i] * z2[j] + f0b[i] * k1[j]);
      }
      if (gj == 0.0) continue;
      for (int eb = M.rptr[r]; eb < M.rptr[r + 1]; ++eb) {
        int q = M.rsp[eb];
        ubar[q] += gj * d2vel(M, r, kr[r], x, j, q);
      }
    }
  }
}

void ros23_vjp(const Model& md, const double* u, double dt, const double* lam, double* lam_in,
               double* ebar) {
  size_t nc = md.G.nc;
  int ns = md.M.ns;
  bool he = !md.F.emis.empty();
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < nc; ++c) {
    double x[64], kr[256], em[64], l[64], ub[64], eb[64];
    for (int s = 0; s < ns; ++s) {
      x[s] = u[(size_t)s * nc + c];
      l[s] = lam[(size_t)s * nc + c];
      eb[s] = 0.0;
    }
    for (int r = 0; r < md.M.nr; ++r) kr[r] = md.krates[(size_t)r * nc + c];
    if (he)
      for (int s = 0; s < ns; ++s) em[s] = md.F.emis[(size_t)s * nc + c];
    ros23_vjp_cell(md, kr, x, he ? em : nullptr, dt, l, ub, eb);
    for (int s = 0; s < ns; ++s) {
      lam_in[(size_t)s * nc + c] = ub[s];
      if (ebar) ebar[(size_t)s * nc + c] += eb[s];
    }
    for (int s = ns; s < md.nsp; ++s) lam_in[(size_t)s * nc + c] = lam[(size_t)s * nc + c];
  }
}

void compute_rates(Model& md) {
  size_t nc = md.G.nc;
  md.krates.assign((size_t)md.M.nr * nc, 0.0);
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < nc; ++c) {
    double T = md.F.T.empty() ? 298.0 : md.F.T[c];
    double P = md.F.P.empty() ? 101325.0 : md.F.P[c];
    for (int r = 0; r < md.M.nr; ++r) md.krates[(size_t)r * nc + c] = eval_prog(md.M, r, T, P);
  }
}

void copy_opt(std::vector<double>& dst, const double* src, size_t n) {
  if (src) dst.assign(src, src + n);
  else if (dst.empty()) dst.assign(n, 0.0);
}

}  // namespace

// ====================================================================== C API (oracle)
extern "C" {

struct or_model;

or_model* or_create(const rs_config* cfg) {
  Model* md = new Model();
  md->cfg = *cfg;
  md->G = make_grid(&cfg->grid);
  md->M = make_mech(&cfg->mech);
  md->has_m = cfg->has_air_mass;
  md->nsp = md->M.ns + (cfg->has_air_mass ? 1 : 0);
  return reinterpret_cast<or_model*>(md);
}

void or_destroy(or_model* h) { delete reinterpret_cast<Model*>(h); }

// LU elimination order (species eliminated at each pivot; null restores natural order)
void or_set_lu_order(or_model* h, const int32_t* ord) {
  Model& md = *reinterpret_cast<Model*>(h);
  if (ord) md.ord.assign(ord, ord + md.M.ns);
  else md.ord.clear();
}

int or_set_forcing(or_model* h, const rs_forcing* f) {
  Model& md = *reinterpret_cast<Model*>(h);
  const Grid& G = md.G;
  size_t nc = G.nc;
  int ns = md.M.ns;
  copy_opt(md.F.mx, f->mx, (size_t)G.nlev * G.nlat * (G.nlon + 1));
  copy_opt(md.F.my, f->my, (size_t)G.nlev * (G.nlat + 1) * G.nlon);
  copy_opt(md.F.mz, f->mz, (size_t)(G.nlev + 1) * G.nlat * G.nlon);
  if (f->mx || f->my || f->mz || md.F.mx.empty()) md.F.omega = f->flux_omega;
  if (f->dp) md.F.dp.assign(f->dp, f->dp + nc);
  else if (md.F.dp.empty()) md.F.dp.assign(nc, 1.0);
  copy_opt(md.F.qw, f->qbc_w, (size_t)ns * G.nlev * G.nlat);
  copy_opt(md.F.qe, f->qbc_e, (size_t)ns * G.nlev * G.nlat);
  copy_opt(md.F.qs, f->qbc_s, (size_t)ns * G.nlev * G.nlon);
  copy_opt(md.F.qn, f->qbc_n, (size_t)ns * G.nlev * G.nlon);
  bool tp = f->temperature || f->pressure || md.krates.empty();
  if (f->temperature) md.F.T.assign(f->temperature, f->temperature + nc);
  if (f->pressure) md.F.P.assign(f->pressure, f->pressure + nc);
  if (f->emission) md.F.emis.assign(f->emission, f->emission + (size_t)ns * nc);
  vertical_coefs(G, md.F);
  size_t ncol = (size_t)G.nlon * G.nlat;
  if (f->pblh) {
    md.F.pblh.assign(f->pblh, f->pblh + ncol);
    md.F.tau_pbl = f->tau_pblmix;
  }
  if (f->ps) md.F.ps.assign(f->ps, f->ps + ncol);
  if (f->hyb_a) md.F.hyb_a.assign(f->hyb_a, f->hyb_a + G.nlev + 1);
  if (f->hyb_b) md.F.hyb_b.assign(f->hyb_b, f->hyb_b + G.nlev + 1);
  if (md.cfg.do_transport) build_pbl(G, md.F);
  if (f->dps_dt) md.F.dpsdt.assign(f->dps_dt, f->dps_dt + ncol);
  if (md.cfg.do_transport && (f->dps_dt || f->hyb_b || f->mx || f->my || f->mz || f->dp))
    build_fixer(G, md.F);
  if (tp) compute_rates(md);
  return 0;
}

void or_set_rates(or_model* h, const double* k) {
  Model& md = *reinterpret_cast<Model*>(h);
  md.krates.assign(k, k + (size_t)md.M.nr * md.G.nc);
}
void or_get_rates(or_model* h, double* k) {
  Model& md = *reinterpret_cast<Model*>(h);
  std::copy(md.krates.begin(), md.krates.end(), k);
}

// single-cell chemistry helpers (box model / golden tests): k from T, P
void or_cell_rates(or_model* h, double T, double P, double* k) {
  Model& md = *reinterpret_cast<Model*>(h);
  for (int r = 0; r < md.M.nr; ++r) k[r] = eval_prog(md.M, r, T, P);
}

// state arrays below are grid SoA [species][nlev][nlat][nlon]
void or_rhs_transport(or_model* h, double t, const double* u, double* du) {
  transport_rhs(*reinterpret_cast<Model*>(h), u, t, du);
}

void or_rhs_chem(or_model* h, const double* u, double* du) {
  Model& md = *reinterpret_cast<Model*>(h);
  size_t nc = md.G.nc;
  int ns = md.M.ns;
  bool he = !md.F.emis.empty();
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < nc; ++c) {
    double x[64], f[64], kr[256], vb[256], em[64];
    for (int s = 0; s < ns; ++s) x[s] = u[(size_t)s * nc + c];
    for (int r = 0; r < md.M.nr; ++r) kr[r] = md.krates[(size_t)r * nc + c];
    if (he)
      for (int s = 0; s < ns; ++s) em[s] = md.F.emis[(size_t)s * nc + c];
    chem_rhs_cell(md.M, kr, x, he ? em : nullptr, f, vb);
    for (int s = 0; s < ns; ++s) du[(size_t)s * nc + c] = f[s];
    for (int s = ns; s < md.nsp; ++s) du[(size_t)s * nc + c] = 0.0;
  }
}

// J[c][r][s], ns_state x ns_state per cell (air-mass row/column zero)
void or_block_jac(or_model* h, const double* u, double* J) {
  Model& md = *reinterpret_cast<Model*>(h);
  size_t nc = md.G.nc;
  int ns = md.M.ns, nsp = md.nsp;
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < nc; ++c) {
    double x[64], kr[256];
    std::vector<double> Jc(ns * ns);
    for (int s = 0; s < ns; ++s) x[s] = u[(size_t)s * nc + c];
    for (int r = 0; r < md.M.nr; ++r) kr[r] = md.krates[(size_t)r * nc + c];
    chem_jac_cell(md.M, kr, x, Jc.data());
    double* out = J + c * nsp * nsp;
    std::fill(out, out + nsp * nsp, 0.0);
    for (int r = 0; r < ns; ++r)
      for (int s = 0; s < ns; ++s) out[r * nsp + s] = Jc[r * ns + s];
  }
}

double or_single_step(or_model* h, int op, double t, double dt, const double* u, double* unew) {
  Model& md = *reinterpret_cast<Model*>(h);
  std::vector<double> w;
  return op == RS_OP_TRANSPORT ? ssprk43_step(md, u, t, dt, unew, w)
                               : ros23_step(md, u, t, dt, unew, w);
}

// One Lie-Trotter macro step (adv, run_reseact_reactant.jl:310-355): transport adaptive
// solve over [t0,t1] then chemistry adaptive solve over [t0,t1], clamp inside both.
// stats: naT, nrT, naC, nrC, dtT_end, dtC_end, tT_end, tC_end
int or_macro_step(or_model* h, double* u, double t0, double t1, double* dtT, double* dtC,
                  double* stats) {
  Model& md = *reinterpret_cast<Model*>(h);
  size_t n = (size_t)md.nsp * md.G.nc;
  std::vector<double> uv(u, u + n), w;
  bool clamp = md.cfg.clamp_nonneg != 0;
  SolveOut oT{t1, *dtT, 0, 0, 0}, oC{t1, *dtC, 0, 0, 0};
  if (md.cfg.do_transport) {
    oT = adaptive_solve([&](const double* x, double t, double dt, double* xn) {
      return ssprk43_step(md, x, t, dt, xn, w); }, uv, t0, t1, *dtT, md.cfg.ctrl_T,
      md.cfg.maxiters, clamp);
  }
  if (md.cfg.do_chemistry) {
    oC = adaptive_solve([&](const double* x, double t, double dt, double* xn) {
      return ros23_step(md, x, t, dt, xn, w); }, uv, t0, t1, *dtC, md.cfg.ctrl_C,
      md.cfg.maxiters, clamp);
  }
  std::copy(uv.begin(), uv.end(), u);
  *dtT = oT.dt; *dtC = oC.dt;
  stats[0] = oT.nacc; stats[1] = oT.nrej; stats[2] = oC.nacc; stats[3] = oC.nrej;
  stats[4] = oT.dt; stats[5] = oC.dt; stats[6] = oT.t; stats[7] = oC.t;
  bool okT = !md.cfg.do_transport || oT.t >= t1 - 1e-9;
  bool okC = !md.cfg.do_chemistry || oC.t >= t1 - 1e-9;
  if (!okT || !okC) return RS_ERR_MAXITERS;
  for (size_t x = 0; x < n; ++x)
    if (!std::isfinite(u[x])) return RS_ERR_NONFINITE;
  return 0;
}

// Step sizes of the per-cell form rounded down to 4 fraction bits (16 sizes per octave), as the
// batched kernel does: the per-cell trajectories then move by roundoff, not by the integration
// tolerance, under roundoff-sized input changes.  No reference counterpart (the reference has
// one global dt).
static double quant_dt(double d) {
  uint64_t b;
  std::memcpy(&b, &d, sizeof b);
  b &= ~((uint64_t(1) << 48) - 1);
  std::memcpy(&d, &b, sizeof b);
  return d;
}

// Per-cell adaptive chemistry (each cell its own ROS23 + PI controller over [t0,t1]), the
// algorithm of the batched persistent kernel; error norm over the cell's own states.
// dt_io (may be null): per-cell step sizes carried in (a cell with dt_io <= 0 starts from dt0)
// and out, as the batched kernel carries them from one macro step to the next.
int or_chem_per_cell(or_model* h, double* u, double t0, double t1, double dt0, double* dt_io,
                     double* steps_out) {
  const double* dt_in = dt_io;
  double* dt_out = dt_io;
  Model& md = *reinterpret_cast<Model*>(h);
  size_t nc = md.G.nc;
  int ns = md.M.ns, nsp = md.nsp;
  const rs_controller c = md.cfg.ctrl_C;
  int fail = 0;
  bool he = !md.F.emis.empty();
#pragma omp parallel for schedule(dynamic, 64) reduction(| : fail)
  for (size_t cell = 0; cell < nc; ++cell) {
    double x[64], xn[64], e[64], kr[256], em[64];
    for (int s = 0; s < ns; ++s) x[s] = u[(size_t)s * nc + cell];
    for (int r = 0; r < md.M.nr; ++r) kr[r] = md.krates[(size_t)r * nc + cell];
    if (he)
      for (int s = 0; s < ns; ++s) em[s] = md.F.emis[(size_t)s * nc + cell];
    double t = t0, dt = quant_dt(dt_in && dt_in[cell] > 0.0 ? dt_in[cell] : dt0), qold = c.qoldinit,
           iters = 0, nacc = 0;
    double tlim = t1 - 1.0e-9;
    double invqmax = 1.0 / c.qmax, invqmin = 1.0 / c.qmin;
    while ((t < tlim) && (iters < md.cfg.maxiters)) {
      double dtc = std::min(dt, t1 - t);
      ros23_cell(md, kr, x, he ? em : nullptr, t, dtc, xn, e);
      double sse = 0.0;
      for (int s = 0; s < ns; ++s) {
        double am = std::max(std::fabs(x[s]), std::fabs(xn[s]));
        double den = am * md.cfg.rtol_C + md.cfg.atol_C;
        double at = e[s] / den;
        sse = sse + at * at;
      }
      double EEst = std::sqrt(sse / (double)nsp);
      if (std::isnan(EEst)) EEst = 1.0e10;
      double q11 = std::pow(std::max(EEst, 1.0e-35), c.beta1);
      double q = q11 / std::pow(qold, c.beta2);
      q = std::max(invqmax, std::min(invqmin, q / c.gamma));
      if (EEst <= 1.0) {
        for (int s = 0; s < ns; ++s) x[s] = md.cfg.clamp_nonneg ? std::max(xn[s], 0.0) : xn[s];
        t = t + dtc;
        bool insteady = (c.qsteady_min <= q) && (q <= c.qsteady_max);
        dt = quant_dt(dtc / (insteady ? 1.0 : q));
        qold = std::max(EEst, c.qoldinit);
        nacc += 1.0;
      } else {
        dt = quant_dt(dtc / std::min(invqmin, q11 / c.gamma));
      }
      iters += 1.0;
    }
    if (t < tlim) fail |= 1;
    for (int s = 0; s < ns; ++s) u[(size_t)s * nc + cell] = x[s];
    if (dt_out) dt_out[cell] = dt;
    if (steps_out) steps_out[cell] = nacc;
  }
  return fail ? RS_ERR_MAXITERS : 0;
}

double or_reduce_fixed(const double* e, size_t n) { return reduce_fixed(e, n); }

// ---- discrete adjoint (tools/adjoint_gradient.jl:609-835) --------------------------------
void or_record_clear(or_model* h) { reinterpret_cast<Model*>(h)->recs.clear(); }
int or_record_count(or_model* h) { return (int)reinterpret_cast<Model*>(h)->recs.size(); }

// macro step that also checkpoints its input and the accepted (t, dt) of both halves
int or_record_macro_step(or_model* h, double* u, double t0, double t1, double* dtT, double* dtC,
                         double* stats) {
  Model& md = *reinterpret_cast<Model*>(h);
  size_t n = (size_t)md.nsp * md.G.nc;
  MacroRec rec;
  rec.u.assign(u, u + n);
  rec.t0 = t0;
  rec.t1 = t1;
  std::vector<double> uv(u, u + n), w;
  bool clamp = md.cfg.clamp_nonneg != 0;
  SolveOut oT{t1, *dtT, 0, 0, 0}, oC{t1, *dtC, 0, 0, 0};
  if (md.cfg.do_transport)
    oT = adaptive_solve([&](const double* x, double t, double dt, double* xn) {
      return ssprk43_step(md, x, t, dt, xn, w); }, uv, t0, t1, *dtT, md.cfg.ctrl_T,
      md.cfg.maxiters, clamp, &rec.seqT);
  if (md.cfg.do_chemistry)
    oC = adaptive_solve([&](const double* x, double t, double dt, double* xn) {
      return ros23_step(md, x, t, dt, xn, w); }, uv, t0, t1, *dtC, md.cfg.ctrl_C,
      md.cfg.maxiters, clamp, &rec.seqC);
  std::copy(uv.begin(), uv.end(), u);
  *dtT = oT.dt; *dtC = oC.dt;
  stats[0] = oT.nacc; stats[1] = oT.nrej; stats[2] = oC.nacc; stats[3] = oC.nrej;
  md.recs.push_back(std::move(rec));
  return 0;
}

// replay one recorded macro step from u with its fixed sequences; optionally keep the tape
// (input state of every accepted step) -- the fixed-sequence replay of
// tools/adjoint_gradient.jl:647-669
static void replay_rec(Model& md, const MacroRec& rec, std::vector<double>& u,
                       std::vector<std::vector<double>>* tapeT,
                       std::vector<std::vector<double>>* tapeC) {
  size_t n = u.size();
  std::vector<double> raw(n), w;
  bool clamp = md.cfg.clamp_nonneg != 0;
  for (auto& st : rec.seqT) {
    if (tapeT) tapeT->push_back(u);
    ssprk43_step(md, u.data(), st.first, st.second, raw.data(), w);
    for (size_t x = 0; x < n; ++x) u[x] = clamp ? std::max(raw[x], 0.0) : raw[x];
  }
  for (auto& st : rec.seqC) {
    if (tapeC) tapeC->push_back(u);
    ros23_step(md, u.data(), st.first, st.second, raw.data(), w);
    for (size_t x = 0; x < n; ++x) u[x] = clamp ? std::max(raw[x], 0.0) : raw[x];
  }
}

// replay every recorded macro step (fixed step sequences) from u, in place
void or_replay(or_model* h, double* u) {
  Model& md = *reinterpret_cast<Model*>(h);
  size_t n = (size_t)md.nsp * md.G.nc;
  std::vector<double> uv(u, u + n);
  for (auto& rec : md.recs) replay_rec(md, rec, uv, nullptr, nullptr);
  std::copy(uv.begin(), uv.end(), u);
}

// backward sweep over all recorded macro steps: lam (d J / d u_end, in) -> d J / d u_0 (out);
// ebar (grid SoA [ns][nc]) accumulates d J / d emission
void or_adjoint_backward(or_model* h, double* lam, double* ebar) {
  Model& md = *reinterpret_cast<Model*>(h);
  size_t n = (size_t)md.nsp * md.G.nc;
  std::vector<double> L(lam, lam + n), Lin(n), out;
  bool clamp = md.cfg.clamp_nonneg != 0;
  for (int k = (int)md.recs.size() - 1; k >= 0; --k) {
    const MacroRec& rec = md.recs[k];
    std::vector<std::vector<double>> tT, tC;
    std::vector<double> u = rec.u;
    replay_rec(md, rec, u, &tT, &tC);
    // chemistry steps in reverse: clamp mask of each step's output, then the step VJP
    for (int j = (int)rec.seqC.size() - 1; j >= 0; --j) {
      const std::vector<double>& out_j = (j + 1 < (int)tC.size()) ? tC[j + 1] : u;
      if (clamp)
        for (size_t x = 0; x < n; ++x) if (!(out_j[x] > 0.0)) L[x] = 0.0;
      ros23_vjp(md, tC[j].data(), rec.seqC[j].second, L.data(), Lin.data(), ebar);
      L.swap(Lin);
    }
    for (int j = (int)rec.seqT.size() - 1; j >= 0; --j) {
      const std::vector<double>& out_j =
          (j + 1 < (int)tT.size()) ? tT[j + 1] : (tC.empty() ? u : tC[0]);
      if (clamp)
        for (size_t x = 0; x < n; ++x) if (!(out_j[x] > 0.0)) L[x] = 0.0;
      ssprk43_vjp(md, tT[j].data(), rec.seqT[j].first, rec.seqT[j].second, L.data(), Lin.data());
      L.swap(Lin);
    }
  }
  std::copy(L.begin(), L.end(), lam);
}

// single-step VJPs (unit tests)
void or_ssprk43_vjp(or_model* h, const double* u, double t, double dt, const double* lam,
                    double* lam_in) {
  ssprk43_vjp(*reinterpret_cast<Model*>(h), u, t, dt, lam, lam_in);
}
void or_ros23_vjp(or_model* h, const double* u, double dt, const double* lam, double* lam_in,
                  double* ebar) {
  ros23_vjp(*reinterpret_cast<Model*>(h), u, dt, lam, lam_in, ebar);
}
void or_transport_rhs_vjp(or_model* h, const double* u, double t, const double* fbar,
                          double* ubar) {
  transport_rhs_vjp(*reinterpret_cast<Model*>(h), u, t, fbar, ubar);
}

}  // extern "C"
