// rs_transport.cu -- SSPRK43 flux-form transport: monotone PPM face fluxes and the stage kernel.
//
// Transport RHS (CWC mixing-ratio form of reseact.esm:2083, continuity reseact.esm:1535):
//   dq/dt = ( -(Dx(Mx q) + Dy(My q) + Dz(Mz q)) + q * (Dx Mx + Dy My + Dz Mz) ) / m
//   dm/dt = -(Dx Mx + Dy My + Dz Mz)
// with finite-volume divergences on the unit sphere (Dx = (F_e - F_w) dphi/(dlon dS),
// Dy = (F_n cos phi_n - F_s cos phi_s)/dS, Dz = F_top - F_bottom) and face values from the
// upwind cell's CW84-limited parabola (eqs. 1.6-1.8, 1.10; nonuniform-dp form vertically).
// At q == 1 every slope is 0, every face value is exactly 1 and each tracer flux equals the
// air-mass flux bit for bit, so dq/dt == 0 exactly (the CWC freestream gate of
// prototypes/transport_3d/transport_3d.esm and tools/cwc_gate.jl).
//
// SSPRK43 attempt (rx_traced_integrator.jl:362-400): 4 stages, each = 3 face-flux kernels
// (x, y, z) + 1 stage kernel; the 4th stage kernel also forms the embedded error and the
// fixed-tree partial sums of the hairer norm.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "rs_device.cuh"
#include "rs_kernels.h"

namespace rs {

constexpr double kOneSixth = 1.0 / 6.0;
constexpr int kFluxThreads = 256;

// (the limit 2 min(|d0|, |d1|) equals min(2|d0|, 2|d1|) exactly: scaling by 2 is exact)
__device__ __forceinline__ double slope_u(double am, double a, double ap) {
  double d0 = a - am, d1 = ap - a;
  if (d1 * d0 > 0.0) {
    double da = 0.5 * (ap - am);
    double lim = 2.0 * fmin(fabs(d0), fabs(d1));
    return copysign(fmin(fabs(da), lim), da);
  }
  return 0.0;
}
__device__ __forceinline__ double slope_n(double am, double a, double ap, double sA, double sB) {
  double d0 = a - am, d1 = ap - a;
  if (d1 * d0 > 0.0) {
    double da = sA * d1 + sB * d0;
    double lim = 2.0 * fmin(fabs(d0), fabs(d1));
    return copysign(fmin(fabs(da), lim), da);
  }
  return 0.0;
}
__device__ __forceinline__ void limit(double a, double& aL, double& aR) {
  if ((aR - a) * (a - aL) <= 0.0) {
    aL = a;
    aR = a;
  } else {
    double dA = aR - aL;
    double a6 = 6.0 * (a - 0.5 * (aL + aR));
    if (dA * a6 > dA * dA) aL = 3.0 * a - 2.0 * aR;
    else if (-(dA * dA) > dA * a6) aR = 3.0 * a - 2.0 * aL;
  }
}
// ---- production-build forms of slope_u / slope_n / limit.  The same slopes, edges and limiter
// decisions, with the sign tests and the exact power-of-two scalings done on the sign and
// exponent bits in the integer pipes (FP64 issues at ~2 lanes per SM per clock on this GPU):
//   d1*d0 > 0            <=>  d0, d1 nonzero with equal signs       (unless the product underflows)
//   0.5*s, 2*m           =    exponent field -1 / +1                 (normal operands)
//   fmin of magnitudes   =    integer min of the magnitude bits
// so slopes and the extremum test are bit-identical to the FP forms for normal operands (where a
// product of differences could underflow, or an operand is subnormal, the FP form decides).  The
// steepening tests dA*a6 > dA*dA and -(dA*dA) > dA*a6 become sign tests of dA and a6 -+ dA,
// which can differ from the FP forms only where a6 = +-dA to roundoff -- where the limiter is
// continuous (the steepened edge equals the unsteepened one), so a face moves by roundoff only.
// copysign(min(|da|, 2 min(|d0|, |d1|)), da), or 0 where d0, d1 are not nonzero with equal
// signs, on the 32-bit halves of the bit patterns.  (Written on 64-bit masks of reinterpreted
// doubles, the same arithmetic was partly emitted as FP64 adds -- three per slope, measured with
// ncu -- so everything here stays in 32-bit integer operations.)  `half`: |da| = |span| / 2.
__device__ __forceinline__ double slope_pick32(double d0, double d1, double da, bool half) {
  const unsigned hs = (unsigned)__double2hiint(da);
  const unsigned hd = (hs & 0x7fffffffu) - (half ? (1u << 20) : 0u), ld = (unsigned)__double2loint(da);
  const unsigned h0 = (unsigned)__double2hiint(d0) & 0x7fffffffu, l0 = (unsigned)__double2loint(d0);
  const unsigned h1 = (unsigned)__double2hiint(d1) & 0x7fffffffu, l1 = (unsigned)__double2loint(d1);
  const bool p1 = mag_lt(h1, l1, h0, l0);
  const unsigned hm = (p1 ? h1 : h0) + (1u << 20), lm = p1 ? l1 : l0;  // 2 min(|d0|, |d1|)
  const bool binds = mag_lt(hm, lm, hd, ld);
  const unsigned hr = (binds ? hm : hd) | (hs & 0x80000000u), lr = binds ? lm : ld;
  const bool live = ((__double2hiint(d0) ^ __double2hiint(d1)) >= 0) & ((h0 | l0) != 0u) &
                    ((h1 | l1) != 0u);
  return __hiloint2double(live ? (int)hr : 0, live ? (int)lr : 0);
}
__device__ __forceinline__ double slope_u_fast(double am, double a, double ap) {
  const double d0 = a - am, d1 = ap - a;
  if (prod_may_underflow(d0, d1)) return slope_u(am, a, ap);
  return slope_pick32(d0, d1, ap - am, true);  // nonzero span where live; |da| = |ap - am| / 2
}
__device__ __forceinline__ double slope_n_fast(double am, double a, double ap, double sA, double sB) {
  const double d0 = a - am, d1 = ap - a;
  if (prod_may_underflow(d0, d1)) return slope_n(am, a, ap, sA, sB);
  return slope_pick32(d0, d1, sA * d1 + sB * d0, false);
}
// Branch-free: every lane issues the same six FP64 instructions (dA, a6, one steepened edge) and
// picks its result with integer selects -- with the limiter's data-dependent branches, a warp
// issued both sides and the FP64 pipe (16 cycles per warp instruction) ran with about half its
// lanes idle.
__device__ __forceinline__ void limit_fast(double a, double& aL, double& aR) {
  if (tiny_operand(a) || tiny_operand(aL) || tiny_operand(aR)) {
    limit(a, aL, aR);
    return;
  }
  const long long ka = ord_key(a), kl = ord_key(aL), kr = ord_key(aR);
  // extremum: (aR - a)(a - aL) <= 0
  const bool flat = !((kr > ka && ka > kl) || (kr < ka && ka < kl));
  const double dA = aR - aL;
  const double a6 = 6.0 * (a - 0.5 * (aL + aR));
  const long long kd = ord_key(dA), k6 = ord_key(a6);
  // dA (a6 - dA) > 0 and dA (a6 + dA) < 0 as comparisons of a6 with +-dA
  const bool stl = (kd > 0 && k6 > kd) || (kd < 0 && k6 < kd);             // aL <- 3a - 2aR
  const bool str = !stl && ((kd > 0 && k6 < -kd) || (kd < 0 && k6 > -kd));  // aR <- 3a - 2aL
  const double st = fma(-2.0, sel_d(stl, aR, aL), 3.0 * a);
  const double nL = sel_d(stl, st, aL), nR = sel_d(str, st, aR);
  aL = sel_d(flat, a, nL);
  aR = sel_d(flat, a, nR);
}
// the forms the transport kernels use: the oracle's in the strict build, the integer-pipe forms
// in the production build
__device__ __forceinline__ double slope_u_p(double am, double a, double ap) {
#if RS_STRICT
  return slope_u(am, a, ap);
#else
  return slope_u_fast(am, a, ap);
#endif
}
__device__ __forceinline__ double slope_n_p(double am, double a, double ap, double sA, double sB) {
#if RS_STRICT
  return slope_n(am, a, ap, sA, sB);
#else
  return slope_n_fast(am, a, ap, sA, sB);
#endif
}
__device__ __forceinline__ void limit_p(double a, double& aL, double& aR) {
#if RS_STRICT
  limit(a, aL, aR);
#else
  limit_fast(a, aL, aR);
#endif
}

// slopes from the neighbour differences d0 = a - am, d1 = ap - a (computed once per cell by the
// pencil kernels) -- the same operations as slope_u / slope_n, so bit-identical to them
__device__ __forceinline__ double slope_ud(double d0, double d1, double am, double ap) {
#if RS_STRICT
  if (d1 * d0 > 0.0) {
    double da = 0.5 * (ap - am);
    double lim = 2.0 * fmin(fabs(d0), fabs(d1));
    return copysign(fmin(fabs(da), lim), da);
  }
  return 0.0;
#else
  if (prod_may_underflow(d0, d1)) {
    if (d1 * d0 > 0.0) {
      double da = 0.5 * (ap - am);
      double lim = 2.0 * fmin(fabs(d0), fabs(d1));
      return copysign(fmin(fabs(da), lim), da);
    }
    return 0.0;
  }
  return slope_pick32(d0, d1, ap - am, true);
#endif
}
__device__ __forceinline__ double slope_nd(double d0, double d1, double sA, double sB) {
#if RS_STRICT
  if (d1 * d0 > 0.0) {
    double da = sA * d1 + sB * d0;
    double lim = 2.0 * fmin(fabs(d0), fabs(d1));
    return copysign(fmin(fabs(da), lim), da);
  }
  return 0.0;
#else
  if (prod_may_underflow(d0, d1)) {
    if (d1 * d0 > 0.0) {
      double da = sA * d1 + sB * d0;
      double lim = 2.0 * fmin(fabs(d0), fabs(d1));
      return copysign(fmin(fabs(da), lim), da);
    }
    return 0.0;
  }
  return slope_pick32(d0, d1, sA * d1 + sB * d0, false);
#endif
}

__device__ __forceinline__ double ppm_face_u(const double* v, bool right) {
  double dm1 = slope_u_p(v[0], v[1], v[2]);
  double d0 = slope_u_p(v[1], v[2], v[3]);
  double dp1 = slope_u_p(v[2], v[3], v[4]);
  double aL = v[1] + 0.5 * (v[2] - v[1]) - (d0 - dm1) * kOneSixth;
  double aR = v[2] + 0.5 * (v[3] - v[2]) - (dp1 - d0) * kOneSixth;
  limit_p(v[2], aL, aR);
  return right ? aR : aL;
}

// ---- mixed precision: the same reconstruction in FP32 on deviations from the upwind cell.
// PPM is translation-equivariant (slopes, edges and limiter tests use differences only), so
// subtracting the upwind value a2 from the stencil changes nothing in exact arithmetic; the
// deviations d_o = (hi_o - hi_2) + (lo_o - lo_2) come from the split (hi, lo) state planes
// without any FP64 instruction, FP32 then carries ~1e-7 relative error of the DEVIATION (not
// of q), and the face value is a2 + dev in FP64.  q == 1 gives d == 0 and a face of exactly 1.
__device__ __forceinline__ float slope_uf(float am, float a, float ap) {
  float d0 = a - am, d1 = ap - a;
  if (d1 * d0 > 0.0f) {
    float da = 0.5f * (ap - am);
    float lim = fminf(2.0f * fabsf(d0), 2.0f * fabsf(d1));
    return copysignf(fminf(fabsf(da), lim), da);
  }
  return 0.0f;
}
__device__ __forceinline__ float slope_nf(float am, float a, float ap, float sA, float sB) {
  float d0 = a - am, d1 = ap - a;
  if (d1 * d0 > 0.0f) {
    float da = sA * d1 + sB * d0;
    float lim = fminf(2.0f * fabsf(d0), 2.0f * fabsf(d1));
    return copysignf(fminf(fabsf(da), lim), da);
  }
  return 0.0f;
}
__device__ __forceinline__ void limitf(float a, float& aL, float& aR) {
  if ((aR - a) * (a - aL) <= 0.0f) {
    aL = a;
    aR = a;
  } else {
    float dA = aR - aL;
    float a6 = 6.0f * (a - 0.5f * (aL + aR));
    if (dA * a6 > dA * dA) aL = 3.0f * a - 2.0f * aR;
    else if (-(dA * dA) > dA * a6) aR = 3.0f * a - 2.0f * aL;
  }
}
__device__ __forceinline__ float ppm_face_uf(const float* v, bool right) {
  float dm1 = slope_uf(v[0], v[1], v[2]);
  float d0 = slope_uf(v[1], v[2], v[3]);
  float dp1 = slope_uf(v[2], v[3], v[4]);
  float aL = v[1] + 0.5f * (v[2] - v[1]) - (d0 - dm1) * (1.0f / 6.0f);
  float aR = v[2] + 0.5f * (v[3] - v[2]) - (dp1 - d0) * (1.0f / 6.0f);
  limitf(v[2], aL, aR);
  return right ? aR : aL;
}
// split a double into hi + lo floats (used only for boundary ghosts in the flux kernels)
__device__ __forceinline__ void split_d(double x, float& hi, float& lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

// Stage input selection: inside an adaptive attempt the field and the time factor come from
// the device-resident controller (input U[cur] for stage 1, S1/S2/S3 for stages 2-4, g from
// ctl->g[stage-1]); for a single RHS evaluation they are given directly.
struct StageSel {
  const Ctl* ctl;
  int stage;
  const double* U0;
  const double* U1;
  const double* S1;
  const double* S2;
  const double* S3;
  const double* Q;  // direct evaluation
  double g;
};
__device__ __forceinline__ bool resolve_stage(const StageSel& s, const double*& Q, double& g) {
  if (!s.ctl) {
    Q = s.Q;
    g = s.g;
    return true;
  }
  if (s.ctl->done) return false;
  g = s.ctl->g[s.stage - 1];
  Q = s.stage == 1 ? (s.ctl->cur ? s.U1 : s.U0)
                   : (s.stage == 2 ? s.S1 : (s.stage == 3 ? s.S2 : s.S3));
  return true;
}

// ------------------------------------------------------------------ face fluxes
// x faces: (i_f in 0..nlon, j, k), i_f fastest
__global__ void __launch_bounds__(kFluxThreads) k_flux_x(DevTransport<double> T, StageSel sel) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  const int nf = T.nlon + 1;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)nf * T.nlat * T.nlev;
  if (idx >= total) return;
  int i = (int)(idx % nf);
  int j = (int)((idx / nf) % T.nlat);
  int k = (int)(idx / ((long long)nf * T.nlat));
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  const size_t row = ((size_t)k * T.nlat + j) * T.nlon;
  double M = g * T.mx[((size_t)k * T.nlat + j) * nf + i];
  bool right = M > 0.0;
  int up = right ? i - 1 : i;
  int ii[5];
  bool ghost[5];
  for (int o = 0; o < 5; ++o) {
    int q = up - 2 + o;
    ghost[o] = false;
    if (q < 0 || q >= T.nlon) {
      if (T.lon_bc == 0) q = ((q % T.nlon) + T.nlon) % T.nlon;
      else ghost[o] = true;
    }
    ii[o] = q;
  }
  if (T.mixed) {
    for (int s = 0; s < T.ntr; ++s) {
      const size_t pb = (size_t)s * nc + row;
      float hi[5], lo[5];
      for (int o = 0; o < 5; ++o) {
        if (ghost[o]) {
          const double* b = ii[o] < 0 ? T.qw : T.qe;
          split_d(b[((size_t)s * T.nlev + k) * T.nlat + j], hi[o], lo[o]);
        } else {
          hi[o] = T.qhi[pb + ii[o]];
          lo[o] = T.qlo[pb + ii[o]];
        }
      }
      float d[5];
      for (int o = 0; o < 5; ++o) d[o] = (hi[o] - hi[2]) + (lo[o] - lo[2]);
      double a2 = ghost[2] ? (double)hi[2] + (double)lo[2] : Q[pb + ii[2]];
      T.fx[((size_t)s * T.nlev * T.nlat + (size_t)k * T.nlat + j) * nf + i] =
          M * (a2 + (double)ppm_face_uf(d, right));
    }
    return;
  }
  for (int s = 0; s < T.ntr; ++s) {
    const double* q = Q + (size_t)s * nc + row;
    double v[5];
    for (int o = 0; o < 5; ++o) {
      if (ghost[o]) {
        const double* b = ii[o] < 0 ? T.qw : T.qe;
        v[o] = b[((size_t)s * T.nlev + k) * T.nlat + j];
      } else {
        v[o] = q[ii[o]];
      }
    }
    T.fx[((size_t)s * T.nlev * T.nlat + (size_t)k * T.nlat + j) * nf + i] = M * ppm_face_u(v, right);
  }
}

// y faces: (i, j_f in 0..nlat, k), i fastest
__global__ void __launch_bounds__(kFluxThreads) k_flux_y(DevTransport<double> T, StageSel sel) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  const int nf = T.nlat + 1;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)T.nlon * nf * T.nlev;
  if (idx >= total) return;
  int i = (int)(idx % T.nlon);
  int j = (int)((idx / T.nlon) % nf);
  int k = (int)(idx / ((long long)T.nlon * nf));
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  const size_t fbase = ((size_t)k * nf + j) * T.nlon + i;
  const size_t fplane = (size_t)T.nlev * nf * T.nlon;
  if (T.lat_bc != 1 && (j == 0 || j == T.nlat)) {
    for (int s = 0; s < T.ntr; ++s) T.fy[(size_t)s * fplane + fbase] = 0.0;
    return;
  }
  double M = g * T.my[fbase];
  bool right = M > 0.0;
  int up = right ? j - 1 : j;
  int jj[5];
  bool ghost[5];
  for (int o = 0; o < 5; ++o) {
    int q = up - 2 + o;
    ghost[o] = false;
    if (q < 0 || q >= T.nlat) {
      if (T.lat_bc == 1) ghost[o] = true;
      else q = q < 0 ? -1 - q : 2 * T.nlat - 1 - q;
    }
    jj[o] = q;
  }
  if (T.mixed) {
    for (int s = 0; s < T.ntr; ++s) {
      const size_t pb = (size_t)s * nc + (size_t)k * T.nlat * T.nlon + i;
      float hi[5], lo[5];
      for (int o = 0; o < 5; ++o) {
        if (ghost[o]) {
          const double* b = jj[o] < 0 ? T.qs : T.qn;
          split_d(b[((size_t)s * T.nlev + k) * T.nlon + i], hi[o], lo[o]);
        } else {
          hi[o] = T.qhi[pb + (size_t)jj[o] * T.nlon];
          lo[o] = T.qlo[pb + (size_t)jj[o] * T.nlon];
        }
      }
      float d[5];
      for (int o = 0; o < 5; ++o) d[o] = (hi[o] - hi[2]) + (lo[o] - lo[2]);
      double a2 = ghost[2] ? (double)hi[2] + (double)lo[2] : Q[pb + (size_t)jj[2] * T.nlon];
      T.fy[(size_t)s * fplane + fbase] = M * (a2 + (double)ppm_face_uf(d, right));
    }
    return;
  }
  for (int s = 0; s < T.ntr; ++s) {
    const double* q = Q + (size_t)s * nc + (size_t)k * T.nlat * T.nlon + i;
    double v[5];
    for (int o = 0; o < 5; ++o) {
      if (ghost[o]) {
        const double* b = jj[o] < 0 ? T.qs : T.qn;
        v[o] = b[((size_t)s * T.nlev + k) * T.nlon + i];
      } else {
        v[o] = q[(size_t)jj[o] * T.nlon];
      }
    }
    T.fy[(size_t)s * fplane + fbase] = M * ppm_face_u(v, right);
  }
}

// z faces: (i, j, k_f in 0..nlev), i fastest; nonuniform (dp-weighted) CW84 reconstruction
__global__ void __launch_bounds__(kFluxThreads) k_flux_z(DevTransport<double> T, StageSel sel) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  const int nf = T.nlev + 1;
  const size_t ncol = (size_t)T.nlon * T.nlat;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)ncol * nf;
  if (idx >= total) return;
  size_t col = (size_t)(idx % (long long)ncol);
  int kf = (int)(idx / (long long)ncol);
  const size_t nc = ncol * T.nlev;
  const size_t fplane = ncol * nf;
  if (kf == 0 || kf == T.nlev) {
    for (int s = 0; s < T.ntr; ++s) T.fz[(size_t)s * fplane + (size_t)kf * ncol + col] = 0.0;
    return;
  }
  double M = g * T.mz[(size_t)kf * ncol + col];
  bool right = M > 0.0;
  int up = right ? kf - 1 : kf;
  int kk[5];
  for (int o = 0; o < 5; ++o) {
    int q = up - 2 + o;
    kk[o] = q < 0 ? -1 - q : (q >= T.nlev ? 2 * T.nlev - 1 - q : q);
  }
  // coefficient rows: slope cells up-1..up+1 (stored from cell -1), edges up and up+1
  double sA0 = T.vsA[(size_t)(up) * ncol + col], sB0 = T.vsB[(size_t)(up) * ncol + col];
  double sA1 = T.vsA[(size_t)(up + 1) * ncol + col], sB1 = T.vsB[(size_t)(up + 1) * ncol + col];
  double sA2 = T.vsA[(size_t)(up + 2) * ncol + col], sB2 = T.vsB[(size_t)(up + 2) * ncol + col];
  double eLab = T.veAB[(size_t)up * ncol + col], eLc = T.veC[(size_t)up * ncol + col],
         eLd = T.veD[(size_t)up * ncol + col];
  double eRab = T.veAB[(size_t)(up + 1) * ncol + col], eRc = T.veC[(size_t)(up + 1) * ncol + col],
         eRd = T.veD[(size_t)(up + 1) * ncol + col];
  if (T.mixed) {
    float fA0 = T.vsA32[(size_t)(up) * ncol + col], fB0 = T.vsB32[(size_t)(up) * ncol + col];
    float fA1 = T.vsA32[(size_t)(up + 1) * ncol + col], fB1 = T.vsB32[(size_t)(up + 1) * ncol + col];
    float fA2 = T.vsA32[(size_t)(up + 2) * ncol + col], fB2 = T.vsB32[(size_t)(up + 2) * ncol + col];
    float fLab = T.veAB32[(size_t)up * ncol + col], fLc = T.veC32[(size_t)up * ncol + col],
          fLd = T.veD32[(size_t)up * ncol + col];
    float fRab = T.veAB32[(size_t)(up + 1) * ncol + col],
          fRc = T.veC32[(size_t)(up + 1) * ncol + col], fRd = T.veD32[(size_t)(up + 1) * ncol + col];
    for (int s = 0; s < T.ntr; ++s) {
      const size_t pb = (size_t)s * nc + col;
      float hi[5], lo[5];
      for (int o = 0; o < 5; ++o) {
        hi[o] = T.qhi[pb + (size_t)kk[o] * ncol];
        lo[o] = T.qlo[pb + (size_t)kk[o] * ncol];
      }
      float d[5];
      for (int o = 0; o < 5; ++o) d[o] = (hi[o] - hi[2]) + (lo[o] - lo[2]);
      float dm1 = slope_nf(d[0], d[1], d[2], fA0, fB0);
      float d0 = slope_nf(d[1], d[2], d[3], fA1, fB1);
      float dp1 = slope_nf(d[2], d[3], d[4], fA2, fB2);
      float aL = d[1] + fLab * (d[2] - d[1]) + fLc * d0 + fLd * dm1;
      float aR = d[2] + fRab * (d[3] - d[2]) + fRc * dp1 + fRd * d0;
      limitf(d[2], aL, aR);
      double a2 = Q[pb + (size_t)kk[2] * ncol];
      T.fz[(size_t)s * fplane + (size_t)kf * ncol + col] = M * (a2 + (double)(right ? aR : aL));
    }
    return;
  }
  for (int s = 0; s < T.ntr; ++s) {
    const double* q = Q + (size_t)s * nc + col;
    double v[5];
    for (int o = 0; o < 5; ++o) v[o] = q[(size_t)kk[o] * ncol];
    double dm1 = slope_n_p(v[0], v[1], v[2], sA0, sB0);
    double d0 = slope_n_p(v[1], v[2], v[3], sA1, sB1);
    double dp1 = slope_n_p(v[2], v[3], v[4], sA2, sB2);
    double aL = v[1] + eLab * (v[2] - v[1]) + eLc * d0 + eLd * dm1;
    double aR = v[2] + eRab * (v[3] - v[2]) + eRc * dp1 + eRd * d0;
    limit_p(v[2], aL, aR);
    T.fz[(size_t)s * fplane + (size_t)kf * ncol + col] = M * (right ? aR : aL);
  }
}

// ------------------------------------------------------------------ fused pencil kernels
// FP64 face fluxes with each cell's monotone slope and each edge value computed ONCE per
// stage (the per-face kernels above recompute three slopes and two edges for every face):
// a block stages whole pencils (a lon row; or 32 adjacent columns of a lat line / vertical
// column) in shared memory, then slopes, then edges, then the upwind limiter and flux of
// each face.  Same expressions in the same order as ppm_face_u / the vertical branch, so the
// fluxes are bit-identical to the per-face kernels.
__global__ void __launch_bounds__(256) k_flux_x_fused(DevTransport<double> T, StageSel sel) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  extern __shared__ double smx[];
  const int n = T.nlon, nf = n + 1, L = n + 6;
  double* V = smx;            // V[p+3], p in [-3, n+2]
  double* Dd = smx + L;       // Dd[p+3] = v(p+1) - v(p), p in [-3, n+1]
  double* D = smx + 2 * L;    // D[p+3], slopes p in [-2, n+1]
  double* E = smx + 3 * L;    // E[f+3], edge between f-1 and f, f in [-1, n+1]
  double* Mf = smx + 4 * L;   // Mf[f], the face's air-mass flux g*mx (shared by all tracers)
  const int row = blockIdx.x;  // (k, j)
  const int j = row % T.nlat, k = row / T.nlat;
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  const size_t rbase = ((size_t)k * T.nlat + j) * n;
  for (int f = threadIdx.x; f <= n; f += blockDim.x) Mf[f] = g * T.mx[((size_t)k * T.nlat + j) * nf + f];
  const int s0 = (int)((long long)blockIdx.y * T.ntr / gridDim.y);  // this block's tracers
  const int s1 = (int)((long long)(blockIdx.y + 1) * T.ntr / gridDim.y);
  for (int s = s0; s < s1; ++s) {
    const double* q = Q + (size_t)s * nc + rbase;
    auto val = [&](int p) -> double {
      if (p < 0 || p >= n) {
        if (T.lon_bc == 0) return q[((p % n) + n) % n];
        return (p < 0 ? T.qw : T.qe)[((size_t)s * T.nlev + k) * T.nlat + j];
      }
      return q[p];
    };
    for (int p = threadIdx.x - 3; p <= n + 2; p += blockDim.x) {
      const double v = val(p);
      V[p + 3] = v;
      if (p <= n + 1) Dd[p + 3] = val(p + 1) - v;
    }
    __syncthreads();
    for (int p = threadIdx.x - 2; p <= n + 1; p += blockDim.x)
      D[p + 3] = slope_ud(Dd[p + 2], Dd[p + 3], V[p + 2], V[p + 4]);
    __syncthreads();
    for (int f = threadIdx.x - 1; f <= n + 1; f += blockDim.x)
      E[f + 3] = V[f + 2] + 0.5 * Dd[f + 2] - (D[f + 3] - D[f + 2]) * kOneSixth;
    __syncthreads();
    for (int f = threadIdx.x; f <= n; f += blockDim.x) {
      const double M = Mf[f];
      const bool right = __double_as_longlong(M) > 0;  // M > 0 for every non-NaN M
      int up = right ? f - 1 : f;
      double aL = E[up + 3], aR = E[up + 4];
      limit_p(V[up + 3], aL, aR);
      T.fx[((size_t)s * T.nlev * T.nlat + (size_t)k * T.nlat + j) * nf + f] = M * (right ? aR : aL);
    }
    __syncthreads();
  }
}

// y: block = PW adjacent i at one level, all j; threads (PW, rows)
template <int kPencil>
__global__ void __launch_bounds__(512) k_flux_y_fused(DevTransport<double> T, StageSel sel) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  extern __shared__ double smy[];
  const int n = T.nlat, nfj = n + 1, L = n + 6;
  double* V = smy;                    // [L][kPencil]
  double* Dd = smy + L * kPencil;     // neighbour differences v(p+1) - v(p)
  double* D = smy + 2 * L * kPencil;
  double* E = smy + 3 * L * kPencil;
  double* Mf = smy + 4 * L * kPencil;  // [n+1][kPencil] face air-mass fluxes g*my
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int ntile = (T.nlon + kPencil - 1) / kPencil;
  const int k = blockIdx.x / ntile;
  const int i = (blockIdx.x % ntile) * kPencil + tx;
  const bool live = i < T.nlon;
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  const size_t fplane = (size_t)T.nlev * nfj * T.nlon;
  const bool open = T.lat_bc == 1;
  if (live)
    for (int f = ty; f <= n; f += blockDim.y)
      Mf[f * kPencil + tx] = g * T.my[((size_t)k * nfj + f) * T.nlon + i];
#define RS_P(a, p) a[((p) + 3) * kPencil + tx]
  const int s0 = (int)((long long)blockIdx.y * T.ntr / gridDim.y);  // this block's tracers
  const int s1 = (int)((long long)(blockIdx.y + 1) * T.ntr / gridDim.y);
  for (int s = s0; s < s1; ++s) {
    const double* q = Q + (size_t)s * nc + (size_t)k * T.nlat * T.nlon;
    auto val = [&](int p) -> double {
      if (!live) return 0.0;
      if (p < 0 || p >= n) {
        if (open) return (p < 0 ? T.qs : T.qn)[((size_t)s * T.nlev + k) * T.nlon + i];
        return q[(size_t)(p < 0 ? -1 - p : 2 * n - 1 - p) * T.nlon + i];
      }
      return q[(size_t)p * T.nlon + i];
    };
    for (int p = (int)ty - 3; p <= n + 2; p += blockDim.y) {
      const double v = val(p);
      RS_P(V, p) = v;
      if (p <= n + 1) RS_P(Dd, p) = val(p + 1) - v;
    }
    __syncthreads();
    for (int p = (int)ty - 2; p <= n + 1; p += blockDim.y)
      RS_P(D, p) = slope_ud(RS_P(Dd, p - 1), RS_P(Dd, p), RS_P(V, p - 1), RS_P(V, p + 1));
    __syncthreads();
    for (int f = (int)ty - 1; f <= n + 1; f += blockDim.y)
      RS_P(E, f) = RS_P(V, f - 1) + 0.5 * RS_P(Dd, f - 1) - (RS_P(D, f) - RS_P(D, f - 1)) * kOneSixth;
    __syncthreads();
    if (live) {
      for (int f = ty; f <= n; f += blockDim.y) {
        size_t fb = ((size_t)k * nfj + f) * T.nlon + i;
        if (!open && (f == 0 || f == n)) {
          T.fy[(size_t)s * fplane + fb] = 0.0;
          continue;
        }
        const double M = Mf[f * kPencil + tx];
        const bool right = __double_as_longlong(M) > 0;
        int up = right ? f - 1 : f;
        double aL = RS_P(E, up), aR = RS_P(E, up + 1);
        limit_p(RS_P(V, up), aL, aR);
        T.fy[(size_t)s * fplane + fb] = M * (right ? aR : aL);
      }
    }
    __syncthreads();
  }
}

// z: block = PW adjacent columns, all levels; dp-weighted coefficients
template <int kPencil>
__global__ void __launch_bounds__(512) k_flux_z_fused(DevTransport<double> T, StageSel sel) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  extern __shared__ double smz[];
  const int n = T.nlev, L = n + 6;
  double* V = smz;
  double* Dd = smz + L * kPencil;
  double* D = smz + 2 * L * kPencil;
  double* E = smz + 3 * L * kPencil;
  double* Mf = smz + 4 * L * kPencil;  // [n+1][kPencil] face air-mass fluxes g*mz
  const int tx = threadIdx.x, ty = threadIdx.y;
  const size_t ncol = (size_t)T.nlon * T.nlat;
  const size_t col = (size_t)blockIdx.x * kPencil + tx;
  const bool live = col < ncol;
  const size_t nc = ncol * n;
  const size_t fplane = ncol * (n + 1);
  if (live)
    for (int kf = ty; kf <= n; kf += blockDim.y) Mf[kf * kPencil + tx] = g * T.mz[(size_t)kf * ncol + col];
  const int s0 = (int)((long long)blockIdx.y * T.ntr / gridDim.y);  // this block's tracers
  const int s1 = (int)((long long)(blockIdx.y + 1) * T.ntr / gridDim.y);
  for (int s = s0; s < s1; ++s) {
    const double* q = Q + (size_t)s * nc;
    auto val = [&](int p) -> double {
      const int pp = p < 0 ? -1 - p : (p >= n ? 2 * n - 1 - p : p);
      return live ? q[(size_t)pp * ncol + col] : 0.0;
    };
    for (int p = (int)ty - 3; p <= n + 2; p += blockDim.y) {
      const double v = val(p);
      RS_P(V, p) = v;
      if (p <= n + 1) RS_P(Dd, p) = val(p + 1) - v;
    }
    __syncthreads();
    for (int p = (int)ty - 1; p <= n; p += blockDim.y) {  // slopes of cells -1..n
      double sA = live ? T.vsA[(size_t)(p + 1) * ncol + col] : 0.0;
      double sB = live ? T.vsB[(size_t)(p + 1) * ncol + col] : 0.0;
      RS_P(D, p) = slope_nd(RS_P(Dd, p - 1), RS_P(Dd, p), sA, sB);
    }
    __syncthreads();
    for (int e = ty; e <= n; e += blockDim.y) {  // edges 0..n (cells e-1 | e)
      double eab = live ? T.veAB[(size_t)e * ncol + col] : 0.0;
      double ec = live ? T.veC[(size_t)e * ncol + col] : 0.0;
      double ed = live ? T.veD[(size_t)e * ncol + col] : 0.0;
      RS_P(E, e) = RS_P(V, e - 1) + eab * RS_P(Dd, e - 1) + ec * RS_P(D, e) + ed * RS_P(D, e - 1);
    }
    __syncthreads();
    if (live) {
      for (int kf = ty; kf <= n; kf += blockDim.y) {
        if (kf == 0 || kf == n) {
          T.fz[(size_t)s * fplane + (size_t)kf * ncol + col] = 0.0;
          continue;
        }
        const double M = Mf[kf * kPencil + tx];
        const bool right = __double_as_longlong(M) > 0;
        int up = right ? kf - 1 : kf;
        double aL = RS_P(E, up), aR = RS_P(E, up + 1);
        limit_p(RS_P(V, up), aL, aR);
        T.fz[(size_t)s * fplane + (size_t)kf * ncol + col] = M * (right ? aR : aL);
      }
    }
    __syncthreads();
  }
#undef RS_P
}

// ------------------------------------------------------------------ mixed-precision pencils
// FP32 reconstruction once per cell (instead of per face): a pencil stages the split state
// (hi, lo planes) in shared memory, forms the neighbour differences
//   dl_p = (hi_{p+1} - hi_p) + (lo_{p+1} - lo_p)          (exact hi differences of nearby values)
// and each cell's monotone slope from them; a face then needs only the upwind cell's two edge
// DEVIATIONS (translation invariance of PPM: the value of the upwind cell is 0)
//   uniform:  aL = -dl_{up-1}/2 - (S_up - S_{up-1})/6,  aR = dl_up/2 - (S_{up+1} - S_up)/6
//   dp-weighted (edge e between cells e-1, e with coefficients ab, c, d):
//             aL = (ab_up - 1) dl_{up-1} + c_up S_up + d_up S_{up-1}
//             aR = ab_{up+1} dl_up + c_{up+1} S_{up+1} + d_{up+1} S_up
// the CW84 limiter on (0, aL, aR), and the face value a_up + dev in FP64.  q == 1 gives dl = 0,
// S = 0, dev = 0 and a face of exactly 1 (the freestream stays exact).  blockIdx.y selects a
// group of sper tracers, so short pencil grids still fill the 152 SMs.
__device__ __forceinline__ float slope_from_diff(float d0, float d1) {
  if (d1 * d0 > 0.0f) {
    const float da = 0.5f * (d0 + d1);
    const float lim = 2.0f * fminf(fabsf(d0), fabsf(d1));
    return copysignf(fminf(fabsf(da), lim), da);
  }
  return 0.0f;
}
__device__ __forceinline__ float slope_from_diff_n(float d0, float d1, float sA, float sB) {
  if (d1 * d0 > 0.0f) {
    const float da = sA * d1 + sB * d0;
    const float lim = 2.0f * fminf(fabsf(d0), fabsf(d1));
    return copysignf(fminf(fabsf(da), lim), da);
  }
  return 0.0f;
}

// Shared-memory layout of the mixed pencils (floats first, 128-byte aligned rows so that bulk
// copies can land in them): the H, Lo rows (two sets when staged by bulk copies, so the next
// tracer's copy overlaps this tracer's work), then Dl, S rows of L entries (interior cell p at
// row p + kHo), then the face air-mass flux as float and as double.
constexpr int kHoX = 32;  // lon rows: interior starts 128 bytes into each row
constexpr int kHoP = 8;   // lat / vertical pencils: interior starts 8 pencil rows in
__host__ __device__ inline int mixed_rows_x(int n) { return (n + kHoX + 3 + 31) / 32 * 32; }
__host__ __device__ inline int mixed_rows_p(int n) { return (n + kHoP + 3 + 1) / 2 * 2; }

// The face flux is M a2 + M dev: a2 the upwind cell's FP64 value, the deviation product in FP32
// (one FMA in FP64); q == 1 gives exactly M.
// float -> double by re-biasing the exponent in the integer pipes (exact; zero kept, subnormal,
// inf and NaN convert)
__device__ __forceinline__ double f2d_bits(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned fe = (u >> 23) & 0xffu;
  if ((u << 1) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  if (fe == 0u || fe == 255u) return (double)x;
  return __hiloint2double((int)((u & 0x80000000u) | ((fe + 896u) << 20) | ((u & 0x7fffffu) >> 3)),
                          (int)(u << 29));
}
__device__ __forceinline__ double mixed_flux(double M, float Mf, double a2, float dev) {
#if RS_STRICT
  return fma(M, a2, (double)(Mf * dev));
#else
  return fma(M, a2, f2d_bits(Mf * dev));
#endif
}

// ---- bulk-copy staging (TMA): mbarrier with a transaction count, one elected issuing thread.
// Every wait is bounded: after kSpinLimit polls the block records the failure, stops the
// adaptive solve it belongs to, waits (bounded again) for its own copies and returns.
struct MixedTmaps {
  CUtensorMap yh[2], yl[2];  // lat pencils over qhi / qlo, box {pw, nlat, 1}; [0]: pw 16, [1]: 32
  CUtensorMap zh[2], zl[2];  // vertical pencils, box {pw, nlev, 1}
  bool x_ok, y_ok, z_ok;
};
constexpr int kSpinLimit = 1 << 24;
constexpr size_t kSmemAlignPad = 128;  // the launch adds this so the layout can start 128-aligned

__device__ __forceinline__ float* align128(unsigned char* p) {
  return reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(p) + 127) & ~(uintptr_t)127);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* b, uint32_t parity) {
  for (int i = 0; i < kSpinLimit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* m, int c0, int c1, int c2,
                                            unsigned long long* b) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(b))
      : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          unsigned long long* b) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(b))
      : "memory");
}
// A staging wait ran out: flag it, stop the solve (every later kernel of the attempt returns on
// `done` and the controller ends the loop), then give this block's copies a bounded chance to
// land before the block's shared memory is released.
__device__ __noinline__ void staging_abort(int* err, const Ctl* ctl, unsigned long long* bar,
                                           int uses0, int uses1) {
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    atomicOr(err, 1);
    if (ctl) atomicExch(const_cast<int*>(&ctl->done), 1);
    if (uses0 > 0) mbar_wait_bounded(bar, (uint32_t)((uses0 - 1) & 1));
    if (uses1 > 0) mbar_wait_bounded(bar + 1, (uint32_t)((uses1 - 1) & 1));
  }
}

template <bool kTma>
__global__ void __launch_bounds__(256) k_flux_x_mixed(DevTransport<double> T, StageSel sel, int sper) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  const int s0 = blockIdx.y * sper, s1 = min(T.ntr, s0 + sper);  // this block's tracers
  extern __shared__ __align__(16) unsigned char smx32_raw[];
  float* smx32 = align128(smx32_raw);
  __shared__ __align__(8) unsigned long long bar[2];
  const int n = T.nlon, nf = n + 1, L = mixed_rows_x(n);
  float* const H0 = smx32;  // H[p + kHoX], p in [-3, n+2]
  float* const L0 = smx32 + L;
  float* const H1 = smx32 + (kTma ? 2 * L : 0);
  float* const L1 = smx32 + (kTma ? 3 * L : L);
  float* Dl = smx32 + (kTma ? 4 : 2) * L;  // Dl[p + kHoX] = v(p+1) - v(p), p in [-3, n+1]
  float* S = Dl + L;                       // S[p + kHoX], slopes of cells p in [-2, n+1]
  float* Mf32 = S + L;                     // [n+1]
  double* Mf = reinterpret_cast<double*>(Mf32 + (nf + 1) / 2 * 2);  // [n+1]
  const int row = blockIdx.x;
  const int j = row % T.nlat, k = row / T.nlat;
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  const size_t rbase = ((size_t)k * T.nlat + j) * n;
  const bool periodic = T.lon_bc == 0;
  const int tid = threadIdx.x;
  int uses0 = 0, uses1 = 0;  // copies issued per buffer
  auto issue = [&](int s, int b) {  // one tracer's interior hi / lo rows (n floats each)
    const size_t pb = (size_t)s * nc + rbase;
    fence_proxy_async();
    mbar_expect_tx(bar + b, (uint32_t)(2 * n * sizeof(float)));
    bulk_load((b ? H1 : H0) + kHoX, T.qhi + pb, (uint32_t)(n * sizeof(float)), bar + b);
    bulk_load((b ? L1 : L0) + kHoX, T.qlo + pb, (uint32_t)(n * sizeof(float)), bar + b);
  };
  if (kTma) {
    if (tid == 0) {
      mbar_init(bar);
      mbar_init(bar + 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0 && s0 < s1) issue(s0, 0);
    uses0 = s0 < s1;
  }
  for (int f = tid; f <= n; f += blockDim.x) {
    const double M = g * T.mx[((size_t)k * T.nlat + j) * nf + f];
    Mf[f] = M;
    Mf32[f] = (float)M;
  }
  for (int s = s0; s < s1; ++s) {
    const int it = s - s0, b = kTma ? (it & 1) : 0;
    float* H = b ? H1 : H0;
    float* Lo = b ? L1 : L0;
    const size_t pb = (size_t)s * nc + rbase;
    if (kTma) {
      if (s + 1 < s1) {
        if (tid == 0) issue(s + 1, b ^ 1);
        if (b) uses0 += 1;
        else uses1 += 1;
      }
      if (tid < 6) {  // the three ghost cells on each side
        const int p = tid < 3 ? tid - 3 : n + tid - 3;
        float h, l;
        if (periodic) {
          const int q = p < 0 ? p + n : p - n;
          h = T.qhi[pb + q];
          l = T.qlo[pb + q];
        } else {
          split_d((p < 0 ? T.qw : T.qe)[((size_t)s * T.nlev + k) * T.nlat + j], h, l);
        }
        H[p + kHoX] = h;
        Lo[p + kHoX] = l;
      }
      const bool ok = mbar_wait_bounded(bar + b, (uint32_t)(((it >> 1)) & 1));
      if (__syncthreads_or(!ok)) {
        staging_abort(T.tma_err, sel.ctl, bar, uses0, uses1);
        return;
      }
    } else {
      for (int p = tid - 3; p <= n + 2; p += blockDim.x) {
        float h, l;
        if (p < 0 || p >= n) {
          if (periodic) {
            const int q = ((p % n) + n) % n;
            h = T.qhi[pb + q];
            l = T.qlo[pb + q];
          } else {
            split_d((p < 0 ? T.qw : T.qe)[((size_t)s * T.nlev + k) * T.nlat + j], h, l);
          }
        } else {
          h = T.qhi[pb + p];
          l = T.qlo[pb + p];
        }
        H[p + kHoX] = h;
        Lo[p + kHoX] = l;
      }
      __syncthreads();
    }
    for (int p = tid - 3; p <= n + 1; p += blockDim.x)
      Dl[p + kHoX] = (H[p + kHoX + 1] - H[p + kHoX]) + (Lo[p + kHoX + 1] - Lo[p + kHoX]);
    __syncthreads();
    for (int p = tid - 2; p <= n + 1; p += blockDim.x)
      S[p + kHoX] = slope_from_diff(Dl[p + kHoX - 1], Dl[p + kHoX]);
    __syncthreads();
    auto face = [&](int f, bool ghosts) {
      const double M = Mf[f];
      const bool right = __double_as_longlong(M) > 0;
      const int up = right ? f - 1 : f;
      const int u = up + kHoX;
      float aL = -0.5f * Dl[u - 1] - (S[u] - S[u - 1]) * (1.0f / 6.0f);
      float aR = 0.5f * Dl[u] - (S[u + 1] - S[u]) * (1.0f / 6.0f);
      limitf(0.0f, aL, aR);
      double a2;
      if (!ghosts) a2 = Q[pb + (up < 0 ? n - 1 : (up >= n ? 0 : up))];
      else if (up >= 0 && up < n) a2 = Q[pb + up];
      else a2 = (double)H[u] + (double)Lo[u];
      T.fx[((size_t)s * T.nlev * T.nlat + (size_t)k * T.nlat + j) * nf + f] =
          mixed_flux(M, Mf32[f], a2, right ? aR : aL);
    };
    if (periodic)
      for (int f = tid; f <= n; f += blockDim.x) face(f, false);
    else
      for (int f = tid; f <= n; f += blockDim.x) face(f, true);
    __syncthreads();
  }
}

template <int kPencil, bool kTma>
__global__ void __launch_bounds__(512) k_flux_y_mixed(DevTransport<double> T, StageSel sel, int sper,
                                                      const __grid_constant__ CUtensorMap mh,
                                                      const __grid_constant__ CUtensorMap ml) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  const int s0 = blockIdx.y * sper, s1 = min(T.ntr, s0 + sper);  // this block's tracers
  extern __shared__ __align__(16) unsigned char smy32_raw[];
  float* smy32 = align128(smy32_raw);
  __shared__ __align__(8) unsigned long long bar[2];
  const int n = T.nlat, nfj = n + 1, L = mixed_rows_p(n);
  const int R = L * kPencil;  // one row set [L][kPencil], cell p at row p + kHoP
  float* const H0 = smy32;
  float* const L0 = smy32 + R;
  float* const H1 = smy32 + (kTma ? 2 * R : 0);
  float* const L1 = smy32 + (kTma ? 3 * R : R);
  float* Dl = smy32 + (kTma ? 4 : 2) * R;
  float* S = Dl + R;
  float* Mf32 = S + R;  // [n+1][kPencil]
  double* Mf = reinterpret_cast<double*>(Mf32 + nfj * kPencil);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool lead = tx == 0 && ty == 0;
  const int ntile = (T.nlon + kPencil - 1) / kPencil;
  const int k = blockIdx.x / ntile;
  const int i0 = (blockIdx.x % ntile) * kPencil;
  const int i = i0 + tx;
  const bool live = i < T.nlon;
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  const size_t fplane = (size_t)T.nlev * nfj * T.nlon;
  const bool open = T.lat_bc == 1;
  int uses0 = 0, uses1 = 0;  // copies issued per buffer
  auto issue = [&](int s, int b) {  // interior rows 0..n-1 of (i0.., k, s): box {kPencil, n, 1}
    fence_proxy_async();
    mbar_expect_tx(bar + b, (uint32_t)(2 * n * kPencil * sizeof(float)));
    tma_load_3d((b ? H1 : H0) + kHoP * kPencil, &mh, i0, 0, k + s * T.nlev, bar + b);
    tma_load_3d((b ? L1 : L0) + kHoP * kPencil, &ml, i0, 0, k + s * T.nlev, bar + b);
  };
  if (kTma) {
    if (lead) {
      mbar_init(bar);
      mbar_init(bar + 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (lead && s0 < s1) issue(s0, 0);
    uses0 = s0 < s1;
  }
  if (live)
    for (int f = ty; f <= n; f += blockDim.y) {
      const double M = g * T.my[((size_t)k * nfj + f) * T.nlon + i];
      Mf[f * kPencil + tx] = M;
      Mf32[f * kPencil + tx] = (float)M;
    }
#define RS_Y(a, p) a[((p) + kHoP) * kPencil + tx]
  for (int s = s0; s < s1; ++s) {
    const int it = s - s0, b = kTma ? (it & 1) : 0;
    float* H = b ? H1 : H0;
    float* Lo = b ? L1 : L0;
    const size_t pb = (size_t)s * nc + (size_t)k * T.nlat * T.nlon;
    auto cell = [&](int p, float& h, float& l) {  // a ghost (p outside 0..n-1) or interior cell
      h = 0.0f;
      l = 0.0f;
      if (!live) return;
      if (p < 0 || p >= n) {
        if (open) {
          split_d((p < 0 ? T.qs : T.qn)[((size_t)s * T.nlev + k) * T.nlon + i], h, l);
          return;
        }
        p = p < 0 ? -1 - p : 2 * n - 1 - p;
      }
      h = T.qhi[pb + (size_t)p * T.nlon + i];
      l = T.qlo[pb + (size_t)p * T.nlon + i];
    };
    if (kTma) {
      if (s + 1 < s1) {
        if (lead) issue(s + 1, b ^ 1);
        if (b) uses0 += 1;
        else uses1 += 1;
      }
      for (int r = ty; r < 6; r += blockDim.y) {
        const int p = r < 3 ? r - 3 : n + r - 3;
        float h, l;
        cell(p, h, l);
        RS_Y(H, p) = h;
        RS_Y(Lo, p) = l;
      }
      const bool ok = mbar_wait_bounded(bar + b, (uint32_t)((it >> 1) & 1));
      if (__syncthreads_or(!ok)) {
        staging_abort(T.tma_err, sel.ctl, bar, uses0, uses1);
        return;
      }
    } else {
      for (int p = (int)ty - 3; p <= n + 2; p += blockDim.y) {
        float h, l;
        cell(p, h, l);
        RS_Y(H, p) = h;
        RS_Y(Lo, p) = l;
      }
      __syncthreads();
    }
    for (int p = (int)ty - 3; p <= n + 1; p += blockDim.y)
      RS_Y(Dl, p) = (RS_Y(H, p + 1) - RS_Y(H, p)) + (RS_Y(Lo, p + 1) - RS_Y(Lo, p));
    __syncthreads();
    for (int p = (int)ty - 2; p <= n + 1; p += blockDim.y)
      RS_Y(S, p) = slope_from_diff(RS_Y(Dl, p - 1), RS_Y(Dl, p));
    __syncthreads();
    auto face = [&](int f, bool ghosts) {
      const size_t fb = ((size_t)k * nfj + f) * T.nlon + i;
      const double M = Mf[f * kPencil + tx];
      const bool right = __double_as_longlong(M) > 0;
      const int up = right ? f - 1 : f;
      float aL = -0.5f * RS_Y(Dl, up - 1) - (RS_Y(S, up) - RS_Y(S, up - 1)) * (1.0f / 6.0f);
      float aR = 0.5f * RS_Y(Dl, up) - (RS_Y(S, up + 1) - RS_Y(S, up)) * (1.0f / 6.0f);
      limitf(0.0f, aL, aR);
      double a2;
      if (!ghosts || (up >= 0 && up < n)) a2 = Q[pb + (size_t)up * T.nlon + i];
      else a2 = (double)RS_Y(H, up) + (double)RS_Y(Lo, up);
      T.fy[(size_t)s * fplane + fb] = mixed_flux(M, Mf32[f * kPencil + tx], a2, right ? aR : aL);
    };
    if (live) {
      if (open) {
        for (int f = ty; f <= n; f += blockDim.y) face(f, true);
      } else {  // walls: zero flux on the two boundary faces, interior faces have no ghosts
        for (int f = ty; f <= n; f += blockDim.y) {
          if (f == 0 || f == n) T.fy[(size_t)s * fplane + ((size_t)k * nfj + f) * T.nlon + i] = 0.0;
          else face(f, false);
        }
      }
    }
    __syncthreads();
  }
#undef RS_Y
}

template <int kPencil, bool kTma>
__global__ void __launch_bounds__(512) k_flux_z_mixed(DevTransport<double> T, StageSel sel, int sper,
                                                      const __grid_constant__ CUtensorMap mh,
                                                      const __grid_constant__ CUtensorMap ml) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  const int s0 = blockIdx.y * sper, s1 = min(T.ntr, s0 + sper);  // this block's tracers
  extern __shared__ __align__(16) unsigned char smz32_raw[];
  float* smz32 = align128(smz32_raw);
  __shared__ __align__(8) unsigned long long bar[2];
  const int n = T.nlev, L = mixed_rows_p(n);
  const int R = L * kPencil;
  float* const H0 = smz32;
  float* const L0 = smz32 + R;
  float* const H1 = smz32 + (kTma ? 2 * R : 0);
  float* const L1 = smz32 + (kTma ? 3 * R : R);
  float* Dl = smz32 + (kTma ? 4 : 2) * R;
  float* S = Dl + R;
  float* Mf32 = S + R;  // [n+1][kPencil]
  double* Mf = reinterpret_cast<double*>(Mf32 + (n + 1) * kPencil);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool lead = tx == 0 && ty == 0;
  const size_t ncol = (size_t)T.nlon * T.nlat;
  const size_t col0 = (size_t)blockIdx.x * kPencil;
  const size_t col = col0 + tx;
  const bool live = col < ncol;
  const size_t nc = ncol * n;
  const size_t fplane = ncol * (n + 1);
  int uses0 = 0, uses1 = 0;  // copies issued per buffer
  auto issue = [&](int s, int b) {  // levels 0..n-1 of columns col0..: box {kPencil, n, 1}
    fence_proxy_async();
    mbar_expect_tx(bar + b, (uint32_t)(2 * n * kPencil * sizeof(float)));
    tma_load_3d((b ? H1 : H0) + kHoP * kPencil, &mh, (int)col0, 0, s, bar + b);
    tma_load_3d((b ? L1 : L0) + kHoP * kPencil, &ml, (int)col0, 0, s, bar + b);
  };
  if (kTma) {
    if (lead) {
      mbar_init(bar);
      mbar_init(bar + 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (lead && s0 < s1) issue(s0, 0);
    uses0 = s0 < s1;
  }
  if (live)
    for (int kf = ty; kf <= n; kf += blockDim.y) {
      const double M = g * T.mz[(size_t)kf * ncol + col];
      Mf[kf * kPencil + tx] = M;
      Mf32[kf * kPencil + tx] = (float)M;
    }
#define RS_Z(a, p) a[((p) + kHoP) * kPencil + tx]
  for (int s = s0; s < s1; ++s) {
    const int it = s - s0, b = kTma ? (it & 1) : 0;
    float* H = b ? H1 : H0;
    float* Lo = b ? L1 : L0;
    const size_t pb = (size_t)s * nc + col;
    if (kTma) {
      if (s + 1 < s1) {
        if (lead) issue(s + 1, b ^ 1);
        if (b) uses0 += 1;
        else uses1 += 1;
      }
      for (int r = ty; r < 6; r += blockDim.y) {  // mirrored ghost levels
        const int p = r < 3 ? r - 3 : n + r - 3;
        const int pp = p < 0 ? -1 - p : 2 * n - 1 - p;
        RS_Z(H, p) = live ? T.qhi[pb + (size_t)pp * ncol] : 0.0f;
        RS_Z(Lo, p) = live ? T.qlo[pb + (size_t)pp * ncol] : 0.0f;
      }
      const bool ok = mbar_wait_bounded(bar + b, (uint32_t)((it >> 1) & 1));
      if (__syncthreads_or(!ok)) {
        staging_abort(T.tma_err, sel.ctl, bar, uses0, uses1);
        return;
      }
    } else {
      for (int p = (int)ty - 3; p <= n + 2; p += blockDim.y) {
        const int pp = p < 0 ? -1 - p : (p >= n ? 2 * n - 1 - p : p);
        RS_Z(H, p) = live ? T.qhi[pb + (size_t)pp * ncol] : 0.0f;
        RS_Z(Lo, p) = live ? T.qlo[pb + (size_t)pp * ncol] : 0.0f;
      }
      __syncthreads();
    }
    for (int p = (int)ty - 3; p <= n + 1; p += blockDim.y)
      RS_Z(Dl, p) = (RS_Z(H, p + 1) - RS_Z(H, p)) + (RS_Z(Lo, p + 1) - RS_Z(Lo, p));
    __syncthreads();
    for (int p = (int)ty - 1; p <= n; p += blockDim.y) {  // slopes of cells -1..n (coefficient row p+1)
      const float sA = live ? T.vsA32[(size_t)(p + 1) * ncol + col] : 0.0f;
      const float sB = live ? T.vsB32[(size_t)(p + 1) * ncol + col] : 0.0f;
      RS_Z(S, p) = slope_from_diff_n(RS_Z(Dl, p - 1), RS_Z(Dl, p), sA, sB);
    }
    __syncthreads();
    if (live) {
      for (int kf = ty; kf <= n; kf += blockDim.y) {
        if (kf == 0 || kf == n) {
          T.fz[(size_t)s * fplane + (size_t)kf * ncol + col] = 0.0;
          continue;
        }
        const double M = Mf[kf * kPencil + tx];
        const bool right = __double_as_longlong(M) > 0;
        const int up = right ? kf - 1 : kf;
        const float lab = T.veAB32[(size_t)up * ncol + col], lc = T.veC32[(size_t)up * ncol + col],
                    ld = T.veD32[(size_t)up * ncol + col];
        const float rab = T.veAB32[(size_t)(up + 1) * ncol + col],
                    rc = T.veC32[(size_t)(up + 1) * ncol + col],
                    rd = T.veD32[(size_t)(up + 1) * ncol + col];
        float aL = (lab - 1.0f) * RS_Z(Dl, up - 1) + lc * RS_Z(S, up) + ld * RS_Z(S, up - 1);
        float aR = rab * RS_Z(Dl, up) + rc * RS_Z(S, up + 1) + rd * RS_Z(S, up);
        limitf(0.0f, aL, aR);
        const double a2 = Q[pb + (size_t)up * ncol];
        T.fz[(size_t)s * fplane + (size_t)kf * ncol + col] =
            mixed_flux(M, Mf32[kf * kPencil + tx], a2, right ? aR : aL);
      }
    }
    __syncthreads();
  }
#undef RS_Z
}

// ------------------------------------------------------------------ stage kernel
#if !RS_STRICT
// hi + lo split without FP64-pipe conversions (production build): hi = v truncated to 24
// significant bits, lo = the next 24 bits of the remainder, truncated -- hi + lo = v to 2^-47
// relative.  Values outside [2^-74, 2^127) (zero, subnormals, inf, NaN included) convert.
__device__ __forceinline__ void split_bits(double v, float& hi, float& lo) {
  const unsigned h = (unsigned)__double2hiint(v), l = (unsigned)__double2loint(v);
  const int e = (int)((h >> 20) & 0x7ff);
  if (e < 949 || e > 1150) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
    return;
  }
  const unsigned sign = h & 0x80000000u;
  hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((h & 0xfffffu) << 3) | (l >> 29));
  const unsigned r = l & 0x1fffffffu;  // the 29 mantissa bits below hi
  if (r == 0) {
    lo = 0.0f;
    return;
  }
  const int t = 31 - __clz((int)r);  // leading bit of r, 0..28
  const unsigned mant = t >= 23 ? (r >> (t - 23)) : (r << (23 - t));
  lo = __uint_as_float(sign | ((unsigned)(e - 948 + t) << 23) | (mant & 0x7fffffu));
}
#endif
__device__ __forceinline__ void split_store(const DevTransport<double>& T, size_t x, double v) {
  float hi, lo;
#if RS_STRICT
  hi = (float)v;
  lo = (float)(v - (double)hi);
#else
  split_bits(v, hi, lo);
#endif
  T.qhi[x] = hi;
  T.qlo[x] = lo;
}

// split the attempt's input state U[cur] (stage 1's RHS argument) into hi/lo planes
__global__ void __launch_bounds__(kRedThreads) k_split_input(DevTransport<double> T,
                                                             const Ctl* __restrict__ ctl,
                                                             const double* __restrict__ U0,
                                                             const double* __restrict__ U1,
                                                             const double* __restrict__ Qd) {
  const double* U;
  if (ctl) {
    if (ctl->done) return;
    U = ctl->cur ? U1 : U0;
  } else {
    U = Qd;
  }
  size_t n = (size_t)T.ntr * T.nlon * T.nlat * T.nlev;
  size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < n) split_store(T, x, U[x]);
}
// Divergence of the air-mass flux at cell (i,j,k) at time factor g.
struct CellGeo {
  double gx, gylo, gyhi;
};
// The six air-mass face fluxes of cell (i,j,k) at time factor g, zero through closed walls.
struct MassFluxes {
  double w, e, s, n, b, t;
};
__device__ __forceinline__ MassFluxes mass_fluxes(const DevTransport<double>& T, int i, int j,
                                                  int k, double g) {
  const int nf = T.nlon + 1;
  const size_t ncol = (size_t)T.nlon * T.nlat, col = (size_t)j * T.nlon + i;
  MassFluxes F;
  F.w = g * T.mx[((size_t)k * T.nlat + j) * nf + i];
  F.e = g * T.mx[((size_t)k * T.nlat + j) * nf + i + 1];
  F.s = (T.lat_bc != 1 && j == 0) ? 0.0 : g * T.my[((size_t)k * (T.nlat + 1) + j) * T.nlon + i];
  F.n = (T.lat_bc != 1 && j + 1 == T.nlat) ? 0.0
      : g * T.my[((size_t)k * (T.nlat + 1) + j + 1) * T.nlon + i];
  F.b = (k == 0) ? 0.0 : g * T.mz[(size_t)k * ncol + col];
  F.t = (k + 1 == T.nlev) ? 0.0 : g * T.mz[(size_t)(k + 1) * ncol + col];
  return F;
}
// horizontal (DxM + DyM) and vertical (DzM) parts of the air-mass flux divergence
__device__ __forceinline__ void div_parts(const MassFluxes& F, const CellGeo& G, double& hz,
                                          double& vz) {
  double DxM = (F.e - F.w) * G.gx;
  double DyM = F.n * G.gyhi - F.s * G.gylo;
  hz = DxM + DyM;
  vz = F.t - F.b;
}
__device__ __forceinline__ void div_parts(const DevTransport<double>& T, int i, int j, int k,
                                          double g, const CellGeo& G, double& hz, double& vz) {
  div_parts(mass_fluxes(T, i, j, k, g), G, hz, vz);
}
// Production form of a flux divergence, (e - w) gx + n gyhi - s gylo + (t - b), as one FMA
// chain (five FP64 operations).  k_stage applies it to the air-mass fluxes and to every tracer's
// fluxes alike, so a tracer whose fluxes equal the air-mass fluxes bit for bit (a uniform
// field) still cancels exactly.
__device__ __forceinline__ double div_chain(double w, double e, double s, double n, double b,
                                            double t, const CellGeo& G) {
  return fma(e - w, G.gx, fma(n, G.gyhi, fma(-s, G.gylo, t - b)));
}
__device__ __forceinline__ double div_m(const DevTransport<double>& T, int i, int j, int k,
                                        double g, const CellGeo& G) {
  double hz, vz;
  div_parts(T, i, j, k, g, G, hz, vz);
  return hz + vz;
}
// air-mass tendency: -divM, or with the pressure fixer -((divh + corr) + DzM)
__device__ __forceinline__ double dm_dt(const DevTransport<double>& T, int i, int j, int k,
                                        double g, const CellGeo& G, size_t c) {
  double hz, vz;
  div_parts(T, i, j, k, g, G, hz, vz);
  return T.mcorr ? -((hz + T.mcorr[c]) + vz) : -(hz + vz);
}

// Full PBL mixing (reseact.esm Transport3D pbl_sum_* / pbl_mean_*): per tracer and column the
// PBL mean qbar = sum_k w_k q_k / den, summed from the surface up as the reference's column
// aggregate; the stage kernels add pbl_f * (qbar - q) / tau to each tracer tendency.
__global__ void __launch_bounds__(kRedThreads) k_pbl_mean(DevTransport<double> T, StageSel sel) {
  const double* Q;
  double g;
  if (!resolve_stage(sel, Q, g)) return;
  const size_t ncol = (size_t)T.nlon * T.nlat, nc = ncol * T.nlev;
  const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (size_t)T.ntr * ncol) return;
  const size_t s = id / ncol, col = id % ncol;
  const double* q = Q + s * nc + col;
  double acc = 0.0;
  for (int k = 0; k < T.nlev; ++k) acc = acc + T.pbl_w[(size_t)k * ncol + col] * q[(size_t)k * ncol];
  T.pbl_qbar[id] = acc / T.pbl_den[col];
}

__device__ __forceinline__ double pbl_term(const DevTransport<double>& T, size_t c, size_t col,
                                           int s, double q) {
  const double pb = T.pbl_f[c] * (T.pbl_qbar[(size_t)s * T.nlon * T.nlat + col] - q);
#if RS_STRICT
  return pb / T.pbl_tau;
#else
  return pb * T.pbl_rtau;
#endif
}

static void launch_pbl_mean(cudaStream_t st, const DevTransport<double>& T, const StageSel& sel) {
  size_t n = (size_t)T.ntr * T.nlon * T.nlat;
  k_pbl_mean<<<(unsigned)((n + kRedThreads - 1) / kRedThreads), kRedThreads, 0, st>>>(T, sel);
}

// stage in 1..4.  Qin: the field whose fluxes were computed (RHS argument).
//   1: S1 = U + dt/2 f(U)           2: S2 = S1 + dt/2 f(S1)
//   3: S1 = u3 = S2 + dt/2 f(S2), S3 = u4 = 2/3 U + 1/3 u3
//   4: unew = S3 + dt/2 f(S3); err = 1/2 (1/3 U + 2/3 u3 - unew); candidate = clamp(unew)
template <int STAGE>
__global__ void __launch_bounds__(kRedThreads) k_stage(DevTransport<double> T,
                                                       const Ctl* __restrict__ ctl,
                                                       TransportBufs B, double rtol,
                                                       double atol, int clamp) {
  __shared__ double sm[kRedThreads];
  if (ctl->done) return;
  const double g = ctl->g[STAGE - 1];
  const int cur = ctl->cur;
  const double* U = cur ? B.U1 : B.U0;
  double* Un = cur ? B.U0 : B.U1;
  const double dt = ctl->dtc;
  const double dt_2 = dt / 2;
  const double* Qin = STAGE == 1 ? U : (STAGE == 2 ? B.S1 : (STAGE == 3 ? B.S2 : B.S3));
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  // transport stage tape (recording): this stage's tendency at Fo, its output state (stages
  // 1-3: V1, V2, V4) at Vo, in the slot of the accepted count
  double* Fo = nullptr;
  double* Vo = nullptr;
  if (ctl->ftape) {
    const int slot = (int)ctl->nacc;
    if (slot >= 0 && slot < ctl->fcap) {
      const size_t nst = nc * (size_t)T.nsp;
      double* rec = ctl->ftape + (size_t)slot * 7 * nst;
      Fo = rec + (size_t)(STAGE - 1) * nst;
      if (STAGE < 4) Vo = rec + (size_t)(3 + STAGE) * nst;
    }
  }
  double e = 0.0;
  if (c < nc) {
    int i = (int)(c % T.nlon);
    int j = (int)((c / T.nlon) % T.nlat);
    int k = (int)(c / ((size_t)T.nlon * T.nlat));
    CellGeo G{T.gx[j], T.gylo[j], T.gyhi[j]};
    // the air-mass divergence, once per cell: tracers and the air-mass row
    const MassFluxes F = mass_fluxes(T, i, j, k, g);
#if RS_STRICT
    double hz, vz;
    div_parts(F, G, hz, vz);
    const double divM = hz + vz;
    const double dmdt = T.mcorr ? -((hz + T.mcorr[c]) + vz) : -(hz + vz);  // = dm_dt(...)
#else
    const double divM = div_chain(F.w, F.e, F.s, F.n, F.b, F.t, G);  // the tracers' own chain
    double dmdt = -divM;
    if (T.mcorr) {  // the pressure fixer's -((divh + corr) + DzM)
      double hz, vz;
      div_parts(F, G, hz, vz);
      dmdt = -((hz + T.mcorr[c]) + vz);
    }
#endif
    double m = Qin[(size_t)(T.nsp - 1) * nc + c];
#if !RS_STRICT
    double rm = rcp_nr(m);  // m > 0
#endif
    const int nfx = T.nlon + 1, nfy = T.nlat + 1;
    const size_t ncol = (size_t)T.nlon * T.nlat, col = (size_t)j * T.nlon + i;
    const size_t fxp = (size_t)T.nlev * T.nlat * nfx, fyp = (size_t)T.nlev * nfy * T.nlon,
                 fzp = ncol * (T.nlev + 1);
    const size_t fxi = ((size_t)k * T.nlat + j) * nfx + i;
    const size_t fyi = ((size_t)k * nfy + j) * T.nlon + i;
    const size_t fzi = (size_t)k * ncol + col;
#if !RS_STRICT
    const double sc = dt_2 * rm;  // the tracer increment is (a + q divM) * sc without PBL mixing
#endif
    for (int s = 0; s < T.nsp; ++s) {
      size_t x = (size_t)s * nc + c;
      double q = Qin[x];
      // the stage's new value is q + dt/2 * f: nx = q + dt_2 * du (strict: the oracle's
      // expression order); the production build forms it as fma(du, scale, q), folding 1/m
      // into the scale when no PBL term is added
      double du;
#if !RS_STRICT
      double scale = dt_2;
      bool per_m = false;  // du is the tendency times m (1/m folded into the scale)
#endif
      if (s < T.ntr) {
        double fw = T.fx[s * fxp + fxi], fe = T.fx[s * fxp + fxi + 1];
        double fs = T.fy[s * fyp + fyi], fn = T.fy[s * fyp + fyi + T.nlon];
        double fb = T.fz[s * fzp + fzi], ft = T.fz[s * fzp + fzi + ncol];
#if RS_STRICT
        double Dx = (fe - fw) * G.gx;
        double Dy = fn * G.gyhi - fs * G.gylo;
        double Dz = ft - fb;
        double a = -((Dx + Dy) + Dz);
        double b = q * divM;
        du = (a + b) / m;
        if (T.pbl) du = du + pbl_term(T, c, col, s, q);
#else
        const double ab = fma(q, divM, -div_chain(fw, fe, fs, fn, fb, ft, G));
        if (T.pbl) {
          du = fma(ab, rm, pbl_term(T, c, col, s, q));
        } else {
          du = ab;
          scale = sc;
          per_m = true;
        }
#endif
      } else {
        du = dmdt;
      }
#if RS_STRICT
      const double nx = q + dt_2 * du;
      if (Fo) Fo[x] = du;
#else
      const double nx = fma(du, scale, q);
      if (Fo) Fo[x] = per_m ? du * rm : du;
#endif
      if (STAGE == 1) {
        B.S1[x] = nx;
        if (Vo) Vo[x] = nx;
        if (T.mixed && s < T.ntr) split_store(T, x, nx);
      } else if (STAGE == 2) {
        B.S2[x] = nx;
        if (Vo) Vo[x] = nx;
        if (T.mixed && s < T.ntr) split_store(T, x, nx);
      } else if (STAGE == 3) {
        double u3 = nx;
        double u0 = U[x];
        B.S1[x] = u3;
        double u4 = (2.0 / 3.0) * u0 + (1.0 / 3.0) * u3;
        B.S3[x] = u4;
        if (Vo) Vo[x] = u4;
        if (T.mixed && s < T.ntr) split_store(T, x, u4);
      } else {
        double u0 = U[x];
        double u3 = B.S1[x];
        double un = nx;
#if RS_STRICT
        double ut = (1.0 / 3.0) * u0 + (2.0 / 3.0) * u3;
        double err = 0.5 * (ut - un);
        double am = fmax(fabs(u0), fabs(un));
        double den = am * rtol + atol;
        double at = err / den;
        e = e + at * at;
        Un[x] = clamp ? fmax(un, 0.0) : un;
#else
        // (1/3 u0 + 2/3 u3) - un in two FMAs; the factor 1/2 of the error goes onto the
        // cell's sum as an exact 1/4
        const double err = fma(2.0 / 3.0, u3, fma(1.0 / 3.0, u0, -un));
        const double den = fma(amax_bits(u0, un), rtol, atol);
        const double at = err * rcp_nr1(den);  // den >= atol > 0
        e = fma(at, at, e);
        // clamp at 0 on the sign bit (integer pipe); a NaN candidate fails the norm anyway
        Un[x] = (clamp && __double2hiint(un) < 0) ? 0.0 : un;
#endif
      }
    }
  }
#if !RS_STRICT
  if (STAGE == 4) e = 0.25 * e;
#endif
  if (STAGE == 4) {
    double tot = block_tree256(e, sm);
    if (threadIdx.x == 0) B.partial[blockIdx.x] = tot;
  }
}

// Plain RHS evaluation for the rs_rhs_transport hook: du = f(U) at time factor g.
__global__ void __launch_bounds__(kRedThreads) k_rhs_eval(DevTransport<double> T,
                                                          const double* __restrict__ Qin,
                                                          double* __restrict__ dU, double g,
                                                          double* __restrict__ dUadv) {
  const size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  int i = (int)(c % T.nlon);
  int j = (int)((c / T.nlon) % T.nlat);
  int k = (int)(c / ((size_t)T.nlon * T.nlat));
  CellGeo G{T.gx[j], T.gylo[j], T.gyhi[j]};
  double divM = div_m(T, i, j, k, g, G);
  const bool has_m = T.nsp > T.ntr;
  double m = has_m ? Qin[(size_t)(T.nsp - 1) * nc + c] : 1.0;
  const int nfx = T.nlon + 1, nfy = T.nlat + 1;
  const size_t ncol = (size_t)T.nlon * T.nlat, col = (size_t)j * T.nlon + i;
  const size_t fxp = (size_t)T.nlev * T.nlat * nfx, fyp = (size_t)T.nlev * nfy * T.nlon,
               fzp = ncol * (T.nlev + 1);
  const size_t fxi = ((size_t)k * T.nlat + j) * nfx + i;
  const size_t fyi = ((size_t)k * nfy + j) * T.nlon + i;
  const size_t fzi = (size_t)k * ncol + col;
  for (int s = 0; s < T.nsp; ++s) {
    size_t x = (size_t)s * nc + c;
    if (s < T.ntr) {
      double fw = T.fx[s * fxp + fxi], fe = T.fx[s * fxp + fxi + 1];
      double fs = T.fy[s * fyp + fyi], fn = T.fy[s * fyp + fyi + T.nlon];
      double fb = T.fz[s * fzp + fzi], ft = T.fz[s * fzp + fzi + ncol];
      double Dx = (fe - fw) * G.gx;
      double Dy = fn * G.gyhi - fs * G.gylo;
      double Dz = ft - fb;
      double a = -((Dx + Dy) + Dz);
      double b = Qin[x] * divM;
      const double adv = has_m ? (a + b) / m : a + b;
      dU[x] = T.pbl ? adv + pbl_term(T, c, col, s, Qin[x]) : adv;
      if (dUadv) dUadv[x] = adv;
    } else {
      const double dm = dm_dt(T, i, j, k, g, G, c);
      dU[x] = dm;
      if (dUadv) dUadv[x] = dm;
    }
  }
}

// allow > 48 KB of dynamic shared memory for long pencils (once per process)
constexpr int kPencilSmemCap = 200 * 1024;
static void allow_big_smem() {
  static bool done = false;
  if (done) return;
  const int cap = kPencilSmemCap;
  cudaFuncSetAttribute(k_flux_x_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_y_fused<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_y_fused<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_y_fused<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_z_fused<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_z_fused<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_z_fused<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_x_mixed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_x_mixed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_y_mixed<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_y_mixed<32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_y_mixed<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_y_mixed<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_z_mixed<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_z_mixed<32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_z_mixed<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(k_flux_z_mixed<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  done = true;
}

// Launch shape of the fused pencil kernels: V, Dd, D, E rows (n+6 each) plus the n+1 face fluxes,
// per pencil.  Lat / vertical blocks are (pencil width 8, 16 or 32) x rows threads, at most 512;
// the tuned width drops to 16 where 32 does not fit; a direction whose pencils do not fit even
// at 16 uses the per-face FP64 kernel (the same fluxes, bit for bit).  Lon rows take 64..256
// threads in steps of 32.
struct FluxShape {
  int pw, rows, xt;
  int gx, gyz;  // tracer groups (grid y) of the lon and of the lat / vertical pencils
  size_t shx, shy, shz;
  bool fx, fy, fz;  // fused kernel used for x / y / z
};
static size_t pencil_bytes(int n, int pw) { return (size_t)(4 * (n + 6) + (n + 1)) * pw * sizeof(double); }
static FluxShape flux_shape(const DevTransport<double>& T) {
  FluxShape f;
  f.pw = (T.pencil == 8 || T.pencil == 16) ? T.pencil : 32;
  if (f.pw == 32 && (pencil_bytes(T.nlat, f.pw) > (size_t)kPencilSmemCap ||
                     pencil_bytes(T.nlev, f.pw) > (size_t)kPencilSmemCap))
    f.pw = 16;
  f.rows = (T.rows == 4 || T.rows == 16 || T.rows == 32) ? T.rows : 8;
  if (f.pw * f.rows > 512) f.rows = 512 / f.pw;
  f.xt = (T.xthreads >= 64 && T.xthreads <= 256 && T.xthreads % 32 == 0) ? T.xthreads : 128;
  const int ntr = T.ntr > 0 ? T.ntr : 1;
  f.gx = T.xgroups < 1 ? 1 : (T.xgroups > ntr ? ntr : T.xgroups);
  f.gyz = T.yzgroups < 1 ? 1 : (T.yzgroups > ntr ? ntr : T.yzgroups);
  f.shx = pencil_bytes(T.nlon, 1);
  f.shy = pencil_bytes(T.nlat, f.pw);
  f.shz = pencil_bytes(T.nlev, f.pw);
  f.fx = f.shx <= (size_t)kPencilSmemCap;
  f.fy = f.shy <= (size_t)kPencilSmemCap;
  f.fz = f.shz <= (size_t)kPencilSmemCap;
  return f;
}

static void launch_flux_one(cudaStream_t st, const DevTransport<double>& T, const StageSel& sel,
                            const FluxShape& f, int dir) {
  size_t ncol = (size_t)T.nlon * T.nlat;
  if (dir == 0) {
    if (f.fx) {
      k_flux_x_fused<<<dim3((unsigned)(T.nlat * T.nlev), (unsigned)f.gx), f.xt, f.shx, st>>>(T, sel);
    } else {
      long long nx = (long long)(T.nlon + 1) * T.nlat * T.nlev;
      k_flux_x<<<(unsigned)((nx + kFluxThreads - 1) / kFluxThreads), kFluxThreads, 0, st>>>(T, sel);
    }
  } else if (dir == 1) {
    if (f.fy) {
      unsigned ntile = (unsigned)((T.nlon + f.pw - 1) / f.pw);
      const dim3 grid(ntile * (unsigned)T.nlev, (unsigned)f.gyz);
      if (f.pw == 8) k_flux_y_fused<8><<<grid, dim3(8, f.rows), f.shy, st>>>(T, sel);
      else if (f.pw == 16) k_flux_y_fused<16><<<grid, dim3(16, f.rows), f.shy, st>>>(T, sel);
      else k_flux_y_fused<32><<<grid, dim3(32, f.rows), f.shy, st>>>(T, sel);
    } else {
      long long ny = (long long)T.nlon * (T.nlat + 1) * T.nlev;
      k_flux_y<<<(unsigned)((ny + kFluxThreads - 1) / kFluxThreads), kFluxThreads, 0, st>>>(T, sel);
    }
  } else {
    if (f.fz) {
      const dim3 grid((unsigned)((ncol + f.pw - 1) / f.pw), (unsigned)f.gyz);
      if (f.pw == 8) k_flux_z_fused<8><<<grid, dim3(8, f.rows), f.shz, st>>>(T, sel);
      else if (f.pw == 16) k_flux_z_fused<16><<<grid, dim3(16, f.rows), f.shz, st>>>(T, sel);
      else k_flux_z_fused<32><<<grid, dim3(32, f.rows), f.shz, st>>>(T, sel);
    } else {
      long long nz = (long long)T.nlon * T.nlat * (T.nlev + 1);
      k_flux_z<<<(unsigned)((nz + kFluxThreads - 1) / kFluxThreads), kFluxThreads, 0, st>>>(T, sel);
    }
  }
}

// Mixed-precision pencils: four FP32 rows (hi, lo, neighbour differences, slopes; six with the
// second hi / lo set of the bulk-copy staging) plus the n+1 face fluxes as float and double, per
// pencil.  A direction that does not fit uses the per-face FP32 kernel (the same deviation-form
// reconstruction, evaluated per face).
static size_t mixed_pencil_bytes(int n, int pw, bool tma) {
  const int rows = tma ? 6 : 4;
  if (pw == 1) {
    const int L = mixed_rows_x(n);
    return (size_t)rows * L * sizeof(float) + (size_t)((n + 2) / 2 * 2) * sizeof(float) +
           (size_t)(n + 1) * sizeof(double) + kSmemAlignPad;
  }
  const int L = mixed_rows_p(n);
  return ((size_t)rows * L * sizeof(float) + (size_t)(n + 1) * (sizeof(float) + sizeof(double))) * pw +
         kSmemAlignPad;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the driver
// library); null when the entry point is unavailable.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

// 3-D FP32 tensor {d0, d1, d2} (d0 contiguous) with box {b0, b1, 1}; false if rejected.
static bool encode_f32_3d(CUtensorMap* m, float* base, uint64_t d0, uint64_t d1, uint64_t d2,
                          uint32_t b0, uint32_t b1) {
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {d0, d1, d2};
  const cuuint64_t strides[2] = {d0 * sizeof(float), d0 * d1 * sizeof(float)};
  const cuuint32_t box[3] = {b0, b1, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

MixedTmaps* mixed_tmaps_create(const DevTransport<double>& T, const char** why) {
  *why = nullptr;
  if (!T.qhi || !T.qlo) {
    *why = "no split planes (FP64 transport)";
    return nullptr;
  }
  auto* m = new MixedTmaps();
  const uint64_t ncol = (uint64_t)T.nlon * T.nlat;
  // 1-D bulk copies of lon rows: 16-byte aligned starts and sizes need nlon % 4 == 0
  m->x_ok = T.nlon % 4 == 0;
  // tensor strides must be multiples of 16 bytes; boxes at most 256 rows
  m->y_ok = T.nlon % 4 == 0 && T.nlat <= 256;
  m->z_ok = ncol % 4 == 0 && T.nlev <= 256;
  for (int w = 0; w < 2 && m->y_ok; ++w) {
    const uint32_t pw = w ? 32 : 16;
    m->y_ok = encode_f32_3d(&m->yh[w], T.qhi, T.nlon, T.nlat, (uint64_t)T.nlev * T.ntr, pw, T.nlat) &&
              encode_f32_3d(&m->yl[w], T.qlo, T.nlon, T.nlat, (uint64_t)T.nlev * T.ntr, pw, T.nlat);
  }
  for (int w = 0; w < 2 && m->z_ok; ++w) {
    const uint32_t pw = w ? 32 : 16;
    m->z_ok = encode_f32_3d(&m->zh[w], T.qhi, ncol, T.nlev, T.ntr, pw, T.nlev) &&
              encode_f32_3d(&m->zl[w], T.qlo, ncol, T.nlev, T.ntr, pw, T.nlev);
  }
  if (!m->x_ok && !m->y_ok && !m->z_ok) {
    *why = "grid does not meet the bulk-copy alignment rules";
    delete m;
    return nullptr;
  }
  return m;
}

void mixed_tmaps_destroy(MixedTmaps* m) { delete m; }
bool mixed_tmaps_dir_ok(const MixedTmaps* m, int dir) {
  return m && (dir == 0 ? m->x_ok : (dir == 1 ? m->y_ok : m->z_ok));
}

static void launch_fluxes_mixed(cudaStream_t st, const DevTransport<double>& T, const StageSel& sel,
                                int only_dir = -1) {
  int pw = T.mpencil == 16 ? 16 : 32;
  const MixedTmaps* tm = T.tma;
  const bool tx = tm && tm->x_ok && T.mbulk_x, ty = tm && tm->y_ok && T.mbulk_yz,
             tz = tm && tm->z_ok && T.mbulk_yz;
  if (mixed_pencil_bytes(T.nlat, pw, ty) > (size_t)kPencilSmemCap ||
      mixed_pencil_bytes(T.nlev, pw, tz) > (size_t)kPencilSmemCap)
    pw = 16;
  const int w = pw == 32;
  const int rows = (T.mrows == 4 || T.mrows == 16) ? T.mrows : 8;
  const int xt = (T.mxthreads == 64 || T.mxthreads == 256) ? T.mxthreads : 128;
  auto groups = [&](int sper) { return (unsigned)((T.ntr + sper - 1) / sper); };
  const int sx = std::max(1, std::min(T.ntr, T.msper_x)), syz = std::max(1, std::min(T.ntr, T.msper_yz));
  const size_t ncol = (size_t)T.nlon * T.nlat;
  const size_t shx = mixed_pencil_bytes(T.nlon, 1, tx), shy = mixed_pencil_bytes(T.nlat, pw, ty),
               shz = mixed_pencil_bytes(T.nlev, pw, tz);
  static const CUtensorMap kNoMap{};  // placeholder argument of the plain-load variants
  if (only_dir < 0 || only_dir == 0) {
    if (shx <= (size_t)kPencilSmemCap) {
      dim3 grid((unsigned)(T.nlat * T.nlev), groups(sx));
      if (tx) k_flux_x_mixed<true><<<grid, xt, shx, st>>>(T, sel, sx);
      else k_flux_x_mixed<false><<<grid, xt, shx, st>>>(T, sel, sx);
    } else {
      long long nx = (long long)(T.nlon + 1) * T.nlat * T.nlev;
      k_flux_x<<<(unsigned)((nx + kFluxThreads - 1) / kFluxThreads), kFluxThreads, 0, st>>>(T, sel);
    }
  }
  if (only_dir < 0 || only_dir == 1) {
    if (shy <= (size_t)kPencilSmemCap) {
      dim3 grid((unsigned)((T.nlon + pw - 1) / pw) * (unsigned)T.nlev, groups(syz));
      const CUtensorMap& mh = ty ? tm->yh[w] : kNoMap;
      const CUtensorMap& ml = ty ? tm->yl[w] : kNoMap;
      if (pw == 16) {
        if (ty) k_flux_y_mixed<16, true><<<grid, dim3(16, rows), shy, st>>>(T, sel, syz, mh, ml);
        else k_flux_y_mixed<16, false><<<grid, dim3(16, rows), shy, st>>>(T, sel, syz, mh, ml);
      } else {
        if (ty) k_flux_y_mixed<32, true><<<grid, dim3(32, rows), shy, st>>>(T, sel, syz, mh, ml);
        else k_flux_y_mixed<32, false><<<grid, dim3(32, rows), shy, st>>>(T, sel, syz, mh, ml);
      }
    } else {
      long long ny = (long long)T.nlon * (T.nlat + 1) * T.nlev;
      k_flux_y<<<(unsigned)((ny + kFluxThreads - 1) / kFluxThreads), kFluxThreads, 0, st>>>(T, sel);
    }
  }
  if (only_dir < 0 || only_dir == 2) {
    if (shz <= (size_t)kPencilSmemCap) {
      dim3 grid((unsigned)((ncol + pw - 1) / pw), groups(syz));
      const CUtensorMap& mh = tz ? tm->zh[w] : kNoMap;
      const CUtensorMap& ml = tz ? tm->zl[w] : kNoMap;
      if (pw == 16) {
        if (tz) k_flux_z_mixed<16, true><<<grid, dim3(16, rows), shz, st>>>(T, sel, syz, mh, ml);
        else k_flux_z_mixed<16, false><<<grid, dim3(16, rows), shz, st>>>(T, sel, syz, mh, ml);
      } else {
        if (tz) k_flux_z_mixed<32, true><<<grid, dim3(32, rows), shz, st>>>(T, sel, syz, mh, ml);
        else k_flux_z_mixed<32, false><<<grid, dim3(32, rows), shz, st>>>(T, sel, syz, mh, ml);
      }
    } else {
      long long nz = (long long)T.nlon * T.nlat * (T.nlev + 1);
      k_flux_z<<<(unsigned)((nz + kFluxThreads - 1) / kFluxThreads), kFluxThreads, 0, st>>>(T, sel);
    }
  }
}

static void launch_fluxes(cudaStream_t st, const DevTransport<double>& T, const StageSel& sel) {
  allow_big_smem();
  if (T.mixed) {
    launch_fluxes_mixed(st, T, sel);
    return;
  }
  const FluxShape f = flux_shape(T);
  for (int dir = 0; dir < 3; ++dir) launch_flux_one(st, T, sel, f, dir);
}

// one direction of the mixed-precision flux computation on a given field (used by the
// autotuner); the hi/lo planes of Q are split first
void launch_flux_dir_mixed(cudaStream_t st, const DevTransport<double>& T, const double* Q, int dir,
                           bool split) {
  StageSel sel{nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, Q, 1.0};
  allow_big_smem();
  if (split) {
    size_t n = (size_t)T.ntr * T.nlon * T.nlat * T.nlev;
    k_split_input<<<(unsigned)((n + kRedThreads - 1) / kRedThreads), kRedThreads, 0, st>>>(
        T, nullptr, nullptr, nullptr, Q);
  }
  launch_fluxes_mixed(st, T, sel, dir);
}

// one direction of the flux computation on a given field (used by the autotuner)
void launch_flux_dir(cudaStream_t st, const DevTransport<double>& T, const double* Q, int dir) {
  StageSel sel{nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, Q, 1.0};
  DevTransport<double> T1 = T;
  T1.mixed = 0;
  allow_big_smem();
  launch_flux_one(st, T1, sel, flux_shape(T1), dir);
}

void launch_ssprk43_attempt(cudaStream_t st, const DevTransport<double>& T, const Ctl* ctl,
                            const TransportBufs& B, double rtol, double atol, int clamp) {
  size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  unsigned nb = (unsigned)((nc + kRedThreads - 1) / kRedThreads);
  StageSel sel{ctl, 1, B.U0, B.U1, B.S1, B.S2, B.S3, nullptr, 1.0};
  if (T.mixed) {
    size_t n = (size_t)T.ntr * nc;
    k_split_input<<<(unsigned)((n + kRedThreads - 1) / kRedThreads), kRedThreads, 0, st>>>(
        T, ctl, B.U0, B.U1, nullptr);
  }
  launch_fluxes(st, T, sel);
  if (T.pbl) launch_pbl_mean(st, T, sel);
  k_stage<1><<<nb, kRedThreads, 0, st>>>(T, ctl, B, rtol, atol, clamp);
  sel.stage = 2;
  launch_fluxes(st, T, sel);
  if (T.pbl) launch_pbl_mean(st, T, sel);
  k_stage<2><<<nb, kRedThreads, 0, st>>>(T, ctl, B, rtol, atol, clamp);
  sel.stage = 3;
  launch_fluxes(st, T, sel);
  if (T.pbl) launch_pbl_mean(st, T, sel);
  k_stage<3><<<nb, kRedThreads, 0, st>>>(T, ctl, B, rtol, atol, clamp);
  sel.stage = 4;
  launch_fluxes(st, T, sel);
  if (T.pbl) launch_pbl_mean(st, T, sel);
  k_stage<4><<<nb, kRedThreads, 0, st>>>(T, ctl, B, rtol, atol, clamp);
}

void launch_transport_rhs(cudaStream_t st, const DevTransport<double>& T, const double* U,
                          double g, double* dU, double* dUadv) {
  StageSel sel{nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, U, g};
  size_t nc = (size_t)T.nlon * T.nlat * T.nlev;
  if (T.mixed) {
    size_t n = (size_t)T.ntr * nc;
    k_split_input<<<(unsigned)((n + kRedThreads - 1) / kRedThreads), kRedThreads, 0, st>>>(
        T, nullptr, nullptr, nullptr, U);
  }
  launch_fluxes(st, T, sel);
  if (T.pbl) launch_pbl_mean(st, T, sel);
  k_rhs_eval<<<(unsigned)((nc + kRedThreads - 1) / kRedThreads), kRedThreads, 0, st>>>(T, U, dU, g,
                                                                                     dUadv);
}

}  // namespace rs
