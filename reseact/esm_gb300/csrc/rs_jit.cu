// rs_jit.cu -- generator and NVRTC loader of the mechanism-specialised chemistry kernels.
//
// The generated kernels compute exactly what the table-walking kernels of rs_chem.cu compute
// (ROS23 attempt, rx_traced_integrator.jl:279-349; blocksolve :110-135; hairer norm
// :329-347; per-cell PI controller :455-507), term for term in the same association:
//   v_r   = k_r * x_a * x_a * x_b ...             (reactant entries in table order)
//   f_s   = sum_r net[r,s] v_r (+ emission_s)     (reactions ascending; x*1 and x*(-1) folded)
//   P_p   = d v_r / d x_q                          (same product order as the tables)
//   W     = I - dtgamma * J on the LU fill pattern
//   LU    natural-order pivot-free elimination, zero updates skipped
// so that a strict build (no FMA contraction, divides where the reference divides) is still
// bit-compatible with the CPU restatement.  The only freedom taken is the sign of an exact
// zero (an off-diagonal W entry is written -(dtgamma*acc) instead of 0.0 - dtgamma*acc).
//
// NVRTC is loaded with dlopen so that the library itself loads without it; a handle whose
// kernels cannot be generated keeps the table-walking kernels (also CUDA).
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include "rs_jit.h"
#include "rs_kernels.h"

namespace rs {

static_assert(sizeof(PerCellArgs) == 128 && offsetof(PerCellArgs, clamp) == 112 &&
                  offsetof(PerCellArgs, totals) == 120,
              "PerCellArgs layout is restated in the generated source");

namespace {

// ------------------------------------------------------------------ NVRTC entry points
struct Nvrtc {
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcGetErrorString) err = nullptr;
  std::string why;
  bool ok() const { return why.empty(); }
};

const Nvrtc& nvrtc() {
  static const Nvrtc api = [] {
    Nvrtc a;
    std::vector<std::string> names = {"libnvrtc.so.13", "libnvrtc.so"};
    if (const char* ch = std::getenv("CUDA_HOME")) names.push_back(std::string(ch) + "/lib64/libnvrtc.so.13");
    names.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
    void* h = nullptr;
    for (const auto& n : names)
      if ((h = dlopen(n.c_str(), RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) {
      a.why = "libnvrtc.so.13 not found";
      return a;
    }
    auto sym = [&](auto& fp, const char* name) {
      fp = reinterpret_cast<std::remove_reference_t<decltype(fp)>>(dlsym(h, name));
      if (!fp && a.why.empty()) a.why = std::string("libnvrtc lacks ") + name;
    };
    sym(a.create, "nvrtcCreateProgram");
    sym(a.compile, "nvrtcCompileProgram");
    sym(a.log_size, "nvrtcGetProgramLogSize");
    sym(a.log, "nvrtcGetProgramLog");
    sym(a.cubin_size, "nvrtcGetCUBINSize");
    sym(a.cubin, "nvrtcGetCUBIN");
    sym(a.destroy, "nvrtcDestroyProgram");
    sym(a.err, "nvrtcGetErrorString");
    return a;
  }();
  return api;
}

// ------------------------------------------------------------------ source generation
std::string lit(double v) {  // exact hex-float literal
  char b[64];
  std::snprintf(b, sizeof b, "%a", v);
  return std::signbit(v) ? "(" + std::string(b) + ")" : std::string(b);
}

// W storage: shared-memory variant only while NLU doubles per thread x 256 threads fit
constexpr int kBlock = 256;
constexpr size_t kSmemCap = 227 * 1024 - kBlock * sizeof(double);

size_t smem_bytes(const MechTables& T) { return (size_t)T.nlu * kBlock * sizeof(double); }
// "split" variant: the last split_slots(T) LU slots of W in shared memory, the others in
// registers, two 256-thread blocks per SM (each block's shared part within half an SM's
// 228 KB, its static reduction array and the per-block reserve included)
int split_slots(const MechTables& T) {
  const int cap = (int)((113 * 1024 - 3 * 1024) / (kBlock * sizeof(double)));  // 55
  return T.nlu >= 16 ? (T.nlu < cap ? T.nlu : cap) : 0;
}

struct Gen {
  const MechTables& T;
  bool strict;
  std::ostringstream o;

  void vel(const char* x) {
    for (int r = 0; r < T.nr; ++r) {
      std::ostringstream e;
      e << "K(" << r << ")";
      for (int q = T.rptr[r]; q < T.rptr[r + 1]; ++q)
        for (int t = 0; t < T.rnu[q]; ++t) e << "*" << x << "[" << T.rsp[q] << "]";
      o << "  v[" << r << "] = " << e.str() << ";\n";
    }
  }
  // acc = sum c_t * a[i_t], first term without the leading 0.0 +, +-1 coefficients folded
  static void sum_terms(std::ostringstream& e, bool first, double c, const std::string& term) {
    if (first) {
      if (c == 1.0) e << term;
      else if (c == -1.0) e << "-" << term;
      else e << lit(c) << "*" << term;
    } else {
      // fold into the running sum: e is rebuilt around the previous expression
      std::string prev = e.str();
      e.str("");
      if (c == 1.0) e << prev << " + " << term;
      else if (c == -1.0) e << prev << " - " << term;
      else e << "RS_FMA(" << lit(c) << ", " << term << ", " << prev << ")";
    }
  }
  void rhs(const char* f) {
    for (int s = 0; s < T.ns; ++s) {
      std::ostringstream e;
      bool first = true;
      for (int t = T.rhs_ptr[s]; t < T.rhs_ptr[s + 1]; ++t) {
        sum_terms(e, first, T.rhs_c[t], "v[" + std::to_string(T.rhs_r[t]) + "]");
        first = false;
      }
      std::string ex = first ? std::string("0.0") : e.str();
      o << "  { const double a_ = " << ex << "; " << f << "[" << s << "] = HE ? a_ + EM(" << s
        << ") : a_; }\n";
    }
  }
  // f = RHS at state x.  Strict build: the rates v_r, then each species' sum of c * v_r (the
  // oracle's order).  Production build: per reaction the head u_r = K_r * (all factors but
  // the last) once, and each term as one FMA of u_r with the last factor into the species'
  // sum -- one instruction fewer per reaction than a rate product followed by adds.
  void rates_rhs(const char* x, const char* f) {
    if (strict) {
      vel(x);
      rhs(f);
      return;
    }
    o << "  {\n";  // the heads are local to this evaluation
    std::vector<std::string> last(T.nr);
    for (int r = 0; r < T.nr; ++r) {
      std::vector<int> fac;
      for (int q = T.rptr[r]; q < T.rptr[r + 1]; ++q)
        for (int t = 0; t < T.rnu[q]; ++t) fac.push_back(T.rsp[q]);
      std::ostringstream h;
      h << "K(" << r << ")";
      for (size_t i = 0; i + 1 < fac.size(); ++i) h << "*" << x << "[" << fac[i] << "]";
      o << "  const double u" << r << "_ = " << h.str() << ";\n";
      last[r] = fac.empty() ? std::string() : std::string(x) + "[" + std::to_string(fac.back()) + "]";
    }
    for (int sp = 0; sp < T.ns; ++sp) {
      std::string acc;
      for (int t = T.rhs_ptr[sp]; t < T.rhs_ptr[sp + 1]; ++t) {
        const int r = T.rhs_r[t];
        const double cf = T.rhs_c[t];
        const std::string u = "u" + std::to_string(r) + "_";
        std::string term;  // the product c * v_r, for a first term
        if (last[r].empty()) term = cf == 1.0 ? u : (cf == -1.0 ? "(-" + u + ")" : lit(cf) + "*" + u);
        else if (cf == 1.0) term = u + "*" + last[r];
        else if (cf == -1.0) term = "(-" + u + ")*" + last[r];
        else term = lit(cf) + "*(" + u + "*" + last[r] + ")";
        if (acc.empty()) {
          acc = term;
        } else if (last[r].empty()) {
          acc = cf == 1.0 ? acc + " + " + u : (cf == -1.0 ? acc + " - " + u : "RS_FMA(" + lit(cf) + ", " + u + ", " + acc + ")");
        } else if (cf == 1.0) {
          acc = "RS_FMA(" + u + ", " + last[r] + ", " + acc + ")";
        } else if (cf == -1.0) {
          acc = "RS_FMA(-" + u + ", " + last[r] + ", " + acc + ")";
        } else {
          acc = "RS_FMA(" + lit(cf) + ", " + u + "*" + last[r] + ", " + acc + ")";
        }
      }
      if (acc.empty()) acc = "0.0";
      o << "  { const double a_ = " << acc << "; " << f << "[" << sp << "] = HE ? a_ + EM(" << sp
        << ") : a_; }\n";
    }
    o << "  }\n";
  }
  // Partial derivatives dv_r/dx_q of the rates at xa; `scaled` forms them from kd<r>_ =
  // -dtg * K_r (declared by build_w_scaled) instead of K_r.
  void partials(const char* xa = "x", const char* Pa = "P", bool scaled = false) {
    for (int p = 0; p < T.npart; ++p) {
      int r = T.part_r[p], qs = T.part_q[p];
      std::ostringstream d;
      if (scaled) d << "kd" << r << "_";
      else d << "K(" << r << ")";
      for (int q = T.rptr[r]; q < T.rptr[r + 1]; ++q) {
        int s = T.rsp[q], nu = T.rnu[q];
        if (s == qs) {
          if (nu >= 2) {
            std::ostringstream f;
            f << lit((double)nu);
            for (int t = 1; t < nu; ++t) f << "*" << xa << "[" << s << "]";
            d << "*(" << f.str() << ")";
          }
        } else {
          for (int t = 0; t < nu; ++t) d << "*" << xa << "[" << s << "]";
        }
      }
      o << "  " << Pa << "[" << p << "] = " << d.str() << ";\n";
    }
  }
  void build_w() {
    std::vector<std::string> w(T.nlu, "0.0");
    for (int i = 0; i < T.ns; ++i) w[T.lu_diag[i]] = "1.0";
    for (int e = 0; e < T.njac; ++e) {
      std::ostringstream acc;
      bool first = true;
      for (int t = T.jac_ptr[e]; t < T.jac_ptr[e + 1]; ++t) {
        sum_terms(acc, first, T.jac_coef[t], "P[" + std::to_string(T.jac_part[t]) + "]");
        first = false;
      }
      std::string a = first ? std::string("0.0") : acc.str();
      w[T.jac_slot[e]] = T.jac_diag[e] ? "RS_FMA(-dtg, (" + a + "), 1.0)" : "-(dtg*(" + a + "))";
    }
    for (int e = 0; e < T.nlu; ++e) o << "  WV(" << e << ") = " << w[e] << ";\n";
  }
  // Production attempt: W = I - dtg*J with -dtg folded once into each reaction's rate
  // constant (kd_r = -dtg * K_r) before the partials at x are formed, so each Jacobian entry of
  // W is its plain sum of scaled partials (plus 1 on the diagonal): one multiply per reaction
  // instead of one per entry.
  void build_w_scaled() {
    std::vector<char> used(T.nr, 0);
    for (int p = 0; p < T.npart; ++p) used[T.part_r[p]] = 1;
    o << "  {\n";
    for (int r = 0; r < T.nr; ++r)
      if (used[r]) o << "  const double kd" << r << "_ = -dtg * K(" << r << ");\n";
    partials("x", "P", true);
    std::vector<std::string> w(T.nlu, "0.0");
    for (int i = 0; i < T.ns; ++i) w[T.lu_diag[i]] = "1.0";
    for (int e = 0; e < T.njac; ++e) {
      std::ostringstream acc;
      bool first = true;
      for (int t = T.jac_ptr[e]; t < T.jac_ptr[e + 1]; ++t) {
        sum_terms(acc, first, T.jac_coef[t], "P[" + std::to_string(T.jac_part[t]) + "]");
        first = false;
      }
      if (first) continue;
      w[T.jac_slot[e]] = T.jac_diag[e] ? "1.0 + (" + acc.str() + ")" : acc.str();
    }
    for (int e = 0; e < T.nlu; ++e) o << "  WV(" << e << ") = " << w[e] << ";\n";
    o << "  }\n";
  }
  void lu_factor() {
    int m = 0;
    for (int k = 0; k < T.ns; ++k) {
      if (strict)
        o << "  pv[" << k << "] = 1.0 / WV(" << T.lu_diag[k] << ");\n";
      else
        o << "  pv[" << k << "] = rcp_nr(WV(" << T.lu_diag[k] << "));\n";
      for (int ii = T.elim_ptr[k]; ii < T.elim_ptr[k + 1]; ++ii, ++m) {
        int sl = T.elim_lik[ii];
        o << "  { const double mu_ = WV(" << sl << ") * pv[" << k << "];\n";
        for (int u = T.upd_ptr[m]; u < T.upd_ptr[m + 1]; ++u)
          o << "    WV(" << T.upd_dst[u] << ") = RS_FMA(-mu_, WV(" << T.upd_src[u] << "), WV("
            << T.upd_dst[u] << "));\n";
        o << "    WV(" << sl << ") = mu_; }\n";
      }
    }
  }
  // W^T x = b in place with the same factors: U^T then L^T (the table kernels' lu_solve_T)
  void lu_solve_T(const char* b) {
    for (int j = 0; j < T.ns; ++j) {
      const int sj = T.ord[j];
      if (strict)
        o << "  { const double tj = " << b << "[" << sj << "] / WV(" << T.lu_diag[j] << ");\n";
      else
        o << "  { const double tj = " << b << "[" << sj << "] * pv[" << j << "];\n";
      o << "    " << b << "[" << sj << "] = tj;\n";
      for (int e = T.up_ptr[j]; e < T.up_ptr[j + 1]; ++e)
        o << "    " << b << "[" << T.up_col[e] << "] = RS_FMA(-WV(" << T.up_slot[e] << "), tj, " << b
          << "[" << T.up_col[e] << "]);\n";
      o << "  }\n";
    }
    for (int k = T.ns - 1; k >= 0; --k) {
      const int sk = T.ord[k];
      std::string acc = std::string(b) + "[" + std::to_string(sk) + "]";
      for (int e = T.low_ptr[k]; e < T.low_ptr[k + 1]; ++e)
        acc = "RS_FMA(-WV(" + std::to_string(T.low_slot[e]) + "), " + b + "[" +
              std::to_string(T.low_row[e]) + "], " + acc + ")";
      o << "  " << b << "[" << sk << "] = " << acc << ";\n";
    }
  }
  // a_r = sum_s net[r,s] y_s, species ascending within each reaction (the tables' order)
  void reaction_sums(const char* y, const char* a) {
    std::vector<std::vector<std::pair<int, double>>> per(T.nr);
    for (int sp = 0; sp < T.ns; ++sp)
      for (int t = T.rhs_ptr[sp]; t < T.rhs_ptr[sp + 1]; ++t)
        per[T.rhs_r[t]].push_back({sp, T.rhs_c[t]});
    for (int r = 0; r < T.nr; ++r) {
      std::ostringstream e;
      bool first = true;
      for (auto& tc : per[r]) {
        sum_terms(e, first, tc.second, std::string(y) + "[" + std::to_string(tc.first) + "]");
        first = false;
      }
      o << "  " << a << "[" << r << "] = " << (first ? std::string("0.0") : e.str()) << ";\n";
    }
  }
  // out += J^T y from the partials Pa (a: scratch for the reaction sums)
  void jt_apply(const char* Pa, const char* y, const char* a, const char* out) {
    reaction_sums(y, a);
    for (int p = 0; p < T.npart; ++p)
      o << "  " << out << "[" << T.part_q[p] << "] = RS_FMA(" << a << "[" << T.part_r[p] << "], "
        << Pa << "[" << p << "], " << out << "[" << T.part_q[p] << "]);\n";
  }
  // exact mass-action Hessian term of the ROS23 VJP: for every reaction r and reactant entries
  // j, q: ub_q += dtg (a1_r z2_j + a0_r k1_j) d2v_r/dx_j dx_q (structural zeros skipped)
  void hessian() {
    for (int r = 0; r < T.nr; ++r)
      for (int ea = T.rptr[r]; ea < T.rptr[r + 1]; ++ea) {
        const int j = T.rsp[ea];
        bool any = false;
        std::ostringstream body;
        for (int eb = T.rptr[r]; eb < T.rptr[r + 1]; ++eb) {
          const int q = T.rsp[eb];
          std::ostringstream d;
          d << "K(" << r << ")";
          bool zero = false;
          for (int e = T.rptr[r]; e < T.rptr[r + 1]; ++e) {
            const int sp = T.rsp[e], nu = T.rnu[e];
            const int order = (sp == j) + (sp == q);
            if (order > nu) { zero = true; break; }
            double cst = 1.0;
            for (int t = 0; t < order; ++t) cst *= (double)(nu - t);
            const int m = nu - order;
            if (cst == 1.0 && m == 0) continue;
            std::ostringstream c;
            if (cst != 1.0) c << lit(cst);
            for (int t = 0; t < m; ++t) c << ((cst != 1.0 || t > 0) ? "*" : "") << "x[" << sp << "]";
            d << "*(" << c.str() << ")";
          }
          if (zero) continue;
          any = true;
          body << "    ub[" << q << "] = RS_FMA(gj, " << d.str() << ", ub[" << q << "]);\n";
        }
        if (!any) continue;
        o << "  { const double gj = dtg * RS_FMA(a0[" << r << "], k1[" << j << "], a1[" << r
          << "] * z2[" << j << "]);\n" << body.str() << "  }\n";
      }
  }

  // pivots in elimination order, vector entries by species index (T.ord maps the two)
  void lu_solve(const char* b) {
    for (int k = 0; k < T.ns; ++k)
      for (int e = T.low_ptr[k]; e < T.low_ptr[k + 1]; ++e)
        o << "  " << b << "[" << T.low_row[e] << "] = RS_FMA(-WV(" << T.low_slot[e] << "), " << b
          << "[" << T.ord[k] << "], " << b << "[" << T.low_row[e] << "]);\n";
    for (int i = T.ns - 1; i >= 0; --i) {
      const int si = T.ord[i];
      std::string acc = std::string(b) + "[" + std::to_string(si) + "]";
      for (int e = T.up_ptr[i]; e < T.up_ptr[i + 1]; ++e)
        acc = "RS_FMA(-WV(" + std::to_string(T.up_slot[e]) + "), " + b + "[" +
              std::to_string(T.up_col[e]) + "], " + acc + ")";
      if (strict)
        o << "  " << b << "[" << si << "] = (" << acc << ") / WV(" << T.lu_diag[i] << ");\n";
      else
        o << "  " << b << "[" << si << "] = (" << acc << ") * pv[" << i << "];\n";
    }
  }
};

const char* kPrelude = R"(
typedef unsigned long long u64;
struct PCA {
  double t0, t1, dt0, rtol, atol, maxiters;
  double beta1, beta2, invqmin, invqmax, gamma, qsmin, qsmax, qoldinit;
  int clamp;
  double* totals;
};
static_assert(sizeof(PCA) == 128, "PerCellArgs layout");

// Reciprocal from the hardware approximation r (PTX rcp.approx.ftz.f64) by one third-order
// correction: with e = 1 - d r, 1/d = r / (1 - e) = r (1 + e + e^2 + ...), so r (1 + e + e^2)
// leaves e^3 -- below an ulp for the approximation's |e| -- in three FMAs.  Used by the
// production build in place of IEEE division; d > 0 and normal on every call site (LU pivots
// 1 - dtgamma*J_ii, error-norm denominators >= atol).
__device__ __forceinline__ double rcp_nr(double d) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  const double e = fma(-d, r, 1.0);
  return fma(r, fma(e, e, e), r);
}
// one Newton step: relative error ~1e-12 or better -- enough for error-norm denominators, whose
// only use is the step-size controller
__device__ __forceinline__ double rcp_nr1(double d) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  return fma(r, fma(-d, r, 1.0), r);
}
// max(|a|, |b|) as the larger magnitude bit pattern, on 32-bit halves (integer pipe; NaN stays
// NaN)
__device__ __forceinline__ double amax_bits(double a, double b) {
  const unsigned ha = (unsigned)__double2hiint(a) & 0x7fffffffu, la = (unsigned)__double2loint(a);
  const unsigned hb = (unsigned)__double2hiint(b) & 0x7fffffffu, lb = (unsigned)__double2loint(b);
  const bool bl = ha < hb || (ha == hb && la < lb);
  return __hiloint2double((int)(bl ? hb : ha), (int)(bl ? lb : la));
}

// Per-cell step sizes are rounded down to 4 fraction bits (16 sizes per octave): a perturbation
// of the inputs then changes a cell's step sequence only where a proposal sits within the
// perturbation of a lattice point, so per-cell trajectories stay within roundoff of each other
// under roundoff-sized changes.
__device__ __forceinline__ double quant_dt(double d) {
  return __longlong_as_double(__double_as_longlong(d) & ~((1ll << 48) - 1));
}

// pairwise tree over 256 lanes, v[t] += v[t+s] for s = 128 ... 1; total in thread 0
__device__ __forceinline__ double tree256(double v, double* sm) {
  const int t = threadIdx.x;
  sm[t] = v;
  __syncthreads();
  for (int s = 128; s >= 32; s >>= 1) {
    if (t < s) sm[t] = sm[t] + sm[t + s];
    __syncthreads();
  }
  double a = sm[t];
  if (t < 32) {
    for (int s = 16; s > 0; s >>= 1) {
      const double o = __shfl_down_sync(0xffffffffu, a, s);
      if (t < s) a = a + o;
    }
  }
  __syncthreads();
  return a;
}
)";

std::string generate(const MechTables& T, double ros_d, double ros_c32, bool strict,
                     bool with_smem) {
  const int nsplit = split_slots(T);
  Gen g{T, strict, {}};
  auto& o = g.o;
  o << "// generated: " << T.ns << " species, " << T.nr << " reactions, " << T.nlu
    << " LU slots\n";
  o << "#define NS " << T.ns << "\n#define NRA " << (T.nr > 0 ? T.nr : 1) << "\n#define NPA "
    << (T.npart > 0 ? T.npart : 1) << "\n#define NLU " << T.nlu << "\n#define NLU_R "
    << (T.nlu - nsplit) << "  // LU slots in registers in the split variant\n";
  o << "#define ROS_D " << lit(ros_d) << "\n#define ROS_C32 " << lit(ros_c32) << "\n";
  o << "#define OFF_DONE " << offsetof(Ctl, done) << "\n#define OFF_CUR " << offsetof(Ctl, cur)
    << "\n#define OFF_DTC " << offsetof(Ctl, dtc) << "\n#define OFF_DTO2 "
    << offsetof(Ctl, dto2) << "\n#define OFF_DTO6 " << offsetof(Ctl, dto6)
    << "\n#define OFF_DTG " << offsetof(Ctl, dtgamma) << "\n#define OFF_ITERS "
    << offsetof(Ctl, iters) << "\n#define OFF_NACC " << offsetof(Ctl, nacc)
    << "\n#define OFF_KZ " << offsetof(Ctl, kz) << "\n#define OFF_KZCAP "
    << offsetof(Ctl, kzcap) << "\n";
  o << kPrelude;
  // Every multiply-add is written out: RS_FMA fuses in the production build and keeps the
  // multiply and the add separate in the strict build; both builds compile with --fmad=false,
  // so no compiler contraction decides anything and all variants compute the same bits.
  // RS_NQUOT / RS_AMAX serve the error norm only (its value steers the controller and nothing
  // else): a one-step reciprocal and an integer magnitude max in the production build.
  o << (strict ? "#define RS_QUOT(a, b) ((a) / (b))\n#define RS_FMA(a, b, c) ((a) * (b) + (c))\n"
                 "#define RS_NQUOT(a, b) ((a) / (b))\n#define RS_AMAX(a, b) fmax(fabs(a), fabs(b))\n"
                 "#define RS_VDECL double v[NRA];  // the rates of the oracle-order RHS\n"
               : "#define RS_QUOT(a, b) ((a) * rcp_nr(b))\n#define RS_FMA(a, b, c) fma((a), (b), (c))\n"
                 "#define RS_NQUOT(a, b) ((a) * rcp_nr1(b))\n#define RS_AMAX(a, b) amax_bits((a), (b))\n"
                 "#define RS_VDECL  // the fused RHS keeps no rate array\n");
  // One ROS23 attempt of one cell: xn (unclamped) and the cell's sum of squared scaled errors.
  // f0 = f(x) is computed here unless the caller already holds it (have_f0): after an
  // accepted attempt whose clamp left the state bit for bit unchanged, f(x_new) is exactly
  // the third RHS evaluation f2 of that attempt.  fout (global layout, may be null) receives
  // f2 when the clamp leaves xn unchanged and a NaN marker in plane 0 otherwise; with KEEP
  // the caller also gets f2 in registers.
  o << R"(
// the stage-tape slot of the attempt a controller is running (null when it keeps no tape):
// slot = the accepted count, [2][NS][N] doubles per slot, slots below the controller's kzcap
__device__ __forceinline__ double* stage_slot(const unsigned char* __restrict__ ctl, u64 N) {
  double* kz = *(double* const*)(ctl + OFF_KZ);
  const int cap = *(const int*)(ctl + OFF_KZCAP);
  const int slot = (int)*(const double*)(ctl + OFF_NACC);
  return (kz && slot >= 0 && slot < cap) ? kz + (u64)slot * 2 * NS * N : nullptr;
}
// SOL: the step's solution only (a replay along recorded accepted steps needs no error norm).
// W storage: LU slots e < KR in the register array W, the others in shared memory at
// WSM[(e - KR) * 256] (this thread's column of a [slot][thread] array); every slot index is a
// compile-time constant, so each access resolves to one of the two when compiled.
template <bool HE, int KR, bool KEEP, bool SOL = false>
__device__ __forceinline__ double ros23_cell(const double* __restrict__ kr,
    const double* __restrict__ em, u64 N, int c, const double* x, double* xn, double* W,
    double* WSM, double* f0, bool have_f0, double* __restrict__ fout, int clamp, double* f2,
    double dt, double dto2, double dto6, double dtg, double rtol, double atol,
    double* __restrict__ kzo) {
#define K(r) __ldg(kr + (u64)(r) * N + c)
#define EM(s) __ldg(em + (u64)(s) * N + c)
#define WV(e) (*((e) < KR ? &W[(e)] : &WSM[((e) - KR) * 256]))
  RS_VDECL
  double P[NPA], k1[NS], f1[NS], k2[NS], b[NS], pv[NS];
  if (!have_f0) {
)";
  g.rates_rhs("x", "f0");
  o << "  }\n";
  if (g.strict) {
    g.partials();
    g.build_w();
  } else {
    g.build_w_scaled();
  }
  g.lu_factor();
  o << "#pragma unroll\n  for (int s = 0; s < NS; ++s) k1[s] = f0[s];\n";
  g.lu_solve("k1");
  o << "  if (kzo) {  // stage tape: k1\n#pragma unroll\n    for (int s = 0; s < NS; ++s) "
       "kzo[(u64)s * N + c] = k1[s];\n  }\n";
  o << "#pragma unroll\n  for (int s = 0; s < NS; ++s) xn[s] = RS_FMA(dto2, k1[s], x[s]);\n";
  g.rates_rhs("xn", "f1");
  o << "#pragma unroll\n  for (int s = 0; s < NS; ++s) k2[s] = f1[s] - k1[s];\n";
  g.lu_solve("k2");
  o << "  if (kzo) {  // stage tape: z2, the solve's result before k1 is added\n#pragma unroll\n"
       "    for (int s = 0; s < NS; ++s) kzo[(u64)(NS + s) * N + c] = k2[s];\n  }\n";
  o << "#pragma unroll\n  for (int s = 0; s < NS; ++s) k2[s] = k2[s] + k1[s];\n";
  o << "#pragma unroll\n  for (int s = 0; s < NS; ++s) xn[s] = RS_FMA(dt, k2[s], x[s]);\n";
  o << "  if constexpr (SOL) return 0.0;\n";
  g.rates_rhs("xn", "b");
  o << R"(  if (fout) {
    bool same = true;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const double cl = clamp ? fmax(xn[s], 0.0) : xn[s];
      same = same && (__double_as_longlong(cl) == __double_as_longlong(xn[s]));
    }
    if (same) {
#pragma unroll
      for (int s = 0; s < NS; ++s) fout[(u64)s * N + c] = b[s];
    } else {
      fout[c] = __longlong_as_double(0x7ff8000000000000LL);
    }
  }
  if constexpr (KEEP) {
#pragma unroll
    for (int s = 0; s < NS; ++s) f2[s] = b[s];
  }
#pragma unroll
  for (int s = 0; s < NS; ++s)  // y - 2d as fma(-2, d, y): exact doubling, one rounding either way
    b[s] = RS_FMA(-2.0, k1[s] - f0[s], RS_FMA(-ROS_C32, (k2[s] - f1[s]), b[s]));
)";
  g.lu_solve("b");
  // error norm sum_s (dto6 * e_s / den_s)^2; the production build takes dto6^2 out of the sum
  const char* ut = g.strict ? "dto6 * (RS_FMA(-2.0, k2[s], k1[s]) + b[s])" : "RS_FMA(-2.0, k2[s], k1[s]) + b[s]";
  o << R"(  double acc = 0.0;
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const double ut = )" << ut << R"(;
    const double am = RS_AMAX(x[s], xn[s]);
    const double den = RS_FMA(am, rtol, atol);
    const double at = RS_NQUOT(ut, den);
    acc = RS_FMA(at, at, acc);
  }
)";
  o << (g.strict ? "  return acc;\n" : "  return acc * (dto6 * dto6);\n");
  o << R"(#undef K
#undef EM
#undef WV
}

// global-dt attempt: every cell steps with the controller's dtc; 256-cell block partials.
// F0/F1 (may be null) pair with U0/U1: F[cur] holds f(U[cur]) per cell (NaN in plane 0 where
// unknown); from the second attempt of a solve on, a cell reuses it instead of evaluating
// f(x) again (the first attempt of a solve starts from a state written elsewhere).
// MODE 0: W in registers; 1: W in shared memory; 2: split (NLU_R slots in registers)
template <bool HE, int MODE>
__device__ __forceinline__ void attempt_body(const unsigned char* __restrict__ ctl,
    double* __restrict__ U0, double* __restrict__ U1, const double* __restrict__ kr,
    const double* __restrict__ em, double* __restrict__ partial, int nc, int nsp,
    double rtol, double atol, int clamp, double* __restrict__ F0, double* __restrict__ F1) {
  __shared__ double red[256];
  if (*(const int*)(ctl + OFF_DONE)) return;
  const double dt = *(const double*)(ctl + OFF_DTC);
  const double dto2 = *(const double*)(ctl + OFF_DTO2);
  const double dto6 = *(const double*)(ctl + OFF_DTO6);
  const double dtg = *(const double*)(ctl + OFF_DTG);
  const int cur = *(const int*)(ctl + OFF_CUR);
  const double iters = *(const double*)(ctl + OFF_ITERS);
  const double* __restrict__ U = cur ? U1 : U0;
  double* __restrict__ Un = cur ? U0 : U1;
  double* __restrict__ Fin = cur ? F1 : F0;
  double* __restrict__ Fout = cur ? F0 : F1;
  double* __restrict__ kzo = stage_slot(ctl, (u64)nc);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const u64 N = (u64)nc;
  double e = 0.0;
  if (c < nc) {
    double x[NS], xn[NS], f0[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) x[s] = U[(u64)s * N + c];
    bool have = false;
    if (F0 && iters > 0.0) {
#pragma unroll
      for (int s = 0; s < NS; ++s) f0[s] = Fin[(u64)s * N + c];
      have = f0[0] == f0[0];
    }
    if constexpr (MODE == 1) {
      extern __shared__ double wsm[];
      e = ros23_cell<HE, 0, false>(kr, em, N, c, x, xn, nullptr, wsm + threadIdx.x, f0, have,
                                   F0 ? Fout : nullptr, clamp, nullptr, dt, dto2, dto6, dtg,
                                   rtol, atol, kzo);
    } else if constexpr (MODE == 2) {
      extern __shared__ double wsm[];
      double W[NLU_R > 0 ? NLU_R : 1];
      e = ros23_cell<HE, NLU_R, false>(kr, em, N, c, x, xn, W, wsm + threadIdx.x, f0, have,
                                       F0 ? Fout : nullptr, clamp, nullptr, dt, dto2, dto6,
                                       dtg, rtol, atol, kzo);
    } else {
      double W[NLU];
      e = ros23_cell<HE, NLU, false>(kr, em, N, c, x, xn, W, nullptr, f0, have,
                                     F0 ? Fout : nullptr, clamp, nullptr, dt, dto2, dto6, dtg,
                                     rtol, atol, kzo);
    }
    if (F0 && !have) {  // keep f(x) for a retry of this state after a rejection
#pragma unroll
      for (int s = 0; s < NS; ++s) Fin[(u64)s * N + c] = f0[s];
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) Un[(u64)s * N + c] = clamp ? fmax(xn[s], 0.0) : xn[s];
    for (int s = NS; s < nsp; ++s) {
      const double xv = U[(u64)s * N + c];
      Un[(u64)s * N + c] = clamp ? fmax(xv, 0.0) : xv;
    }
  }
  const double tot = tree256(e, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// per-cell adaptive form: persistent threads pull cells from a device work queue and
// integrate each over [t0, t1] with its own PI controller
template <bool HE>
__device__ __forceinline__ void per_cell_body(int nc, int nsp, double* __restrict__ U,
    const double* __restrict__ kr, const double* __restrict__ em,
    double* __restrict__ dt_cell, double* __restrict__ steps_cell,
    unsigned long long* __restrict__ queue, int* __restrict__ status, PCA a) {
  double x[NS], xn[NS], W[NLU], f0[NS], f2[NS];
  bool have = false;  // f0 == f(x) for the current cell
  double my_steps = 0.0, my_attempts = 0.0;
  double t = 0, dt = 0, qold = 0, iters = 0, nacc = 0;
  int c = -1;
  const u64 N = (u64)nc;
  const double tlim = a.t1 - 1.0e-9;
  for (;;) {
    if (c < 0) {
      const unsigned long long nxt = atomicAdd(queue, 1ull);
      if (nxt >= (unsigned long long)nc) break;
      c = (int)nxt;
#pragma unroll
      for (int s = 0; s < NS; ++s) x[s] = U[(u64)s * N + c];
      have = false;
      t = a.t0;
      dt = quant_dt(dt_cell[c] > 0.0 ? dt_cell[c] : a.dt0);
      qold = a.qoldinit;
      iters = 0;
      nacc = 0;
    }
    if ((t < tlim) && (iters < a.maxiters)) {
      const double dtc = fmin(dt, a.t1 - t);
      const double sse = ros23_cell<HE, NLU, true>(kr, em, N, c, x, xn, W, nullptr, f0, have, nullptr,
                                                 a.clamp, f2, dtc, dtc / 2, dtc / 6,
                                                 dtc * ROS_D, a.rtol, a.atol, nullptr);
      have = true;  // f0 == f(x) after the call; replaced below if x moves
      double EEst = sqrt(sse / (double)nsp);
      if (EEst != EEst) EEst = 1.0e10;
      const double q11 = pow(fmax(EEst, 1.0e-35), a.beta1);
      double q = q11 / pow(qold, a.beta2);
      q = fmax(a.invqmax, fmin(a.invqmin, q / a.gamma));
      if (EEst <= 1.0) {
        bool same = true;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          const double xs = a.clamp ? fmax(xn[s], 0.0) : xn[s];
          same = same && (__double_as_longlong(xs) == __double_as_longlong(xn[s]));
          x[s] = xs;
        }
        if (same) {
#pragma unroll
          for (int s = 0; s < NS; ++s) f0[s] = f2[s];
        }
        have = same;
        t = t + dtc;
        const bool insteady = (a.qsmin <= q) && (q <= a.qsmax);
        dt = quant_dt(dtc / (insteady ? 1.0 : q));
        qold = fmax(EEst, a.qoldinit);
        nacc += 1.0;
      } else {
        dt = quant_dt(dtc / fmin(a.invqmin, q11 / a.gamma));
      }
      iters += 1.0;
    } else {
      if (t < tlim) atomicOr(status, 1);
#pragma unroll
      for (int s = 0; s < NS; ++s) U[(u64)s * N + c] = x[s];
      dt_cell[c] = dt;
      if (steps_cell) steps_cell[c] = nacc;
      my_steps += nacc;
      my_attempts += iters;
      c = -1;
    }
  }
  if (a.totals) {
    atomicAdd(a.totals, my_steps);
    atomicAdd(a.totals + 1, my_attempts);
  }
}

#define RS_ATTEMPT(NAME, HE, MODE, MINB)                                                    \
  extern "C" __global__ void __launch_bounds__(256, MINB) NAME(                             \
      const unsigned char* __restrict__ ctl, double* __restrict__ U0,                       \
      double* __restrict__ U1, const double* __restrict__ kr,                               \
      const double* __restrict__ em, double* __restrict__ partial, int nc, int nsp,         \
      double rtol, double atol, int clamp, double* __restrict__ F0,                         \
      double* __restrict__ F1) {                                                            \
    attempt_body<HE, MODE>(ctl, U0, U1, kr, em, partial, nc, nsp, rtol, atol, clamp, F0,    \
                           F1);                                                             \
  }
RS_ATTEMPT(rs_jit_attempt_r0, false, 0, 1)
RS_ATTEMPT(rs_jit_attempt_r1, true, 0, 1)
RS_ATTEMPT(rs_jit_attempt_q0, false, 0, 2)
RS_ATTEMPT(rs_jit_attempt_q1, true, 0, 2)

// one accepted step at the controller's dtc without the error estimate: the attempt's own
// arithmetic up to the new state (the same bits), for the fixed-sequence replay of a recorded
// macro step
template <bool HE>
__device__ __forceinline__ void step_body(const unsigned char* __restrict__ ctl,
    double* __restrict__ U0, double* __restrict__ U1, const double* __restrict__ kr,
    const double* __restrict__ em, int nc, int nsp, int clamp) {
  if (*(const int*)(ctl + OFF_DONE)) return;
  const double dt = *(const double*)(ctl + OFF_DTC);
  const double dto2 = *(const double*)(ctl + OFF_DTO2);
  const double dtg = *(const double*)(ctl + OFF_DTG);
  const int cur = *(const int*)(ctl + OFF_CUR);
  const double* __restrict__ U = cur ? U1 : U0;
  double* __restrict__ Un = cur ? U0 : U1;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const u64 N = (u64)nc;
  double x[NS], xn[NS], f0[NS], W[NLU];
#pragma unroll
  for (int s = 0; s < NS; ++s) x[s] = U[(u64)s * N + c];
  ros23_cell<HE, NLU, false, true>(kr, em, N, c, x, xn, W, nullptr, f0, false, nullptr, clamp, nullptr,
                                 dt, dto2, 0.0, dtg, 0.0, 0.0, stage_slot(ctl, N));
#pragma unroll
  for (int s = 0; s < NS; ++s) Un[(u64)s * N + c] = clamp ? fmax(xn[s], 0.0) : xn[s];
  for (int s = NS; s < nsp; ++s) {
    const double xv = U[(u64)s * N + c];
    Un[(u64)s * N + c] = clamp ? fmax(xv, 0.0) : xv;
  }
}
#define RS_STEP(NAME, HE)                                                                   \
  extern "C" __global__ void __launch_bounds__(256, 2) NAME(                                \
      const unsigned char* __restrict__ ctl, double* __restrict__ U0,                       \
      double* __restrict__ U1, const double* __restrict__ kr,                               \
      const double* __restrict__ em, int nc, int nsp, int clamp) {                          \
    step_body<HE>(ctl, U0, U1, kr, em, nc, nsp, clamp);                                     \
  }
RS_STEP(rs_jit_step_0, false)
RS_STEP(rs_jit_step_1, true)
)";
  if (with_smem)
    o << "RS_ATTEMPT(rs_jit_attempt_s0, false, 1, 1)\nRS_ATTEMPT(rs_jit_attempt_s1, true, 1, 1)\n";
  if (nsplit > 0)
    o << "RS_ATTEMPT(rs_jit_attempt_h0, false, 2, 2)\nRS_ATTEMPT(rs_jit_attempt_h1, true, 2, 2)\n";
  o << R"(
#define RS_PER_CELL(NAME, HE)                                                                \
  extern "C" __global__ void __launch_bounds__(256) NAME(int nc, int nsp,                   \
      double* __restrict__ U, const double* __restrict__ kr, const double* __restrict__ em,  \
      double* __restrict__ dt_cell, double* __restrict__ steps_cell,                         \
      unsigned long long* __restrict__ queue, int* __restrict__ status, PCA a) {             \
    per_cell_body<HE>(nc, nsp, U, kr, em, dt_cell, steps_cell, queue, status, a);            \
  }
RS_PER_CELL(rs_jit_per_cell_0, false)
RS_PER_CELL(rs_jit_per_cell_1, true)

// VJP of one ROS23 step at a recorded dt (the table kernel k_ros23_vjp, specialised): forward
// recompute of the live stages, then lam_out = (d unew / d u)^T lam and ebar += d J / d emission.
// KZ: k1 and z2 come from the stage tape (kzi, [2][NS][nc]) written by the step's forward, so
// the two RHS evaluations and forward solves are skipped; the partials, W and its LU are
// recomputed either way.
template <bool HE, bool KZ>
__device__ __forceinline__ void vjp_body(int nc, int nsp, const double* __restrict__ U,
    const double* __restrict__ Uout, const double* __restrict__ lam,
    double* __restrict__ lam_out, const double* __restrict__ kr,
    const double* __restrict__ em, double* __restrict__ ebar, double dt, int clamp,
    const double* __restrict__ kzi) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const u64 N = (u64)nc;
  const double dto2 = dt / 2, dtg = dt * ROS_D;
#define K(r) __ldg(kr + (u64)(r) * N + c)
#define EM(s) __ldg(em + (u64)(s) * N + c)
#define WV(e) W[(e)]
  double x[NS], f0[NS], k1[NS], u1[NS], f1[NS], z2[NS], bb[NS], f0b[NS], f1b[NS], ub[NS], pv[NS];
  RS_VDECL
  double a0[NRA], a1[NRA], P[NPA], P1[NPA], W[NLU];
#pragma unroll
  for (int s = 0; s < NS; ++s) x[s] = U[(u64)s * N + c];
)";
  o << "  if constexpr (!KZ) {\n";
  g.rates_rhs("x", "f0");
  o << "  }\n";
  g.partials("x", "P");
  g.build_w();
  g.lu_factor();
  o << "  if constexpr (KZ) {\n#pragma unroll\n    for (int s = 0; s < NS; ++s) k1[s] = "
       "kzi[(u64)s * N + c];\n  } else {\n";
  o << "#pragma unroll\n  for (int s = 0; s < NS; ++s) k1[s] = f0[s];\n";
  g.lu_solve("k1");
  o << "  }\n";
  o << "#pragma unroll\n  for (int s = 0; s < NS; ++s) u1[s] = RS_FMA(dto2, k1[s], x[s]);\n";
  o << "  if constexpr (!KZ) {\n";
  g.rates_rhs("u1", "f1");
  o << "  }\n";
  g.partials("u1", "P1");
  o << "  if constexpr (KZ) {\n#pragma unroll\n    for (int s = 0; s < NS; ++s) z2[s] = "
       "kzi[(u64)(NS + s) * N + c];\n  } else {\n";
  o << "#pragma unroll\n  for (int s = 0; s < NS; ++s) z2[s] = f1[s] - k1[s];\n";
  g.lu_solve("z2");
  o << "  }\n";
  o << R"(#pragma unroll
  for (int s = 0; s < NS; ++s) {
    double l = lam[(u64)s * N + c];
    if (clamp && Uout && !(Uout[(u64)s * N + c] > 0.0)) l = 0.0;
    ub[s] = l;
    bb[s] = dt * l;
  }
)";
  g.lu_solve_T("bb");
  o << R"(#pragma unroll
  for (int s = 0; s < NS; ++s) {
    f1b[s] = bb[s];
    f0b[s] = RS_FMA(dt, ub[s], -bb[s]);
  }
  {
    double u1b[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) u1b[s] = 0.0;
)";
  g.jt_apply("P1", "f1b", "a0", "u1b");
  o << R"(#pragma unroll
    for (int s = 0; s < NS; ++s) {
      ub[s] = ub[s] + u1b[s];
      f0b[s] = RS_FMA(dto2, u1b[s], f0b[s]);
    }
  }
)";
  g.lu_solve_T("f0b");
  g.jt_apply("P", "f0b", "a0", "ub");
  g.reaction_sums("bb", "a1");
  g.reaction_sums("f0b", "a0");
  g.hessian();
  o << R"(#pragma unroll
  for (int s = 0; s < NS; ++s) {
    lam_out[(u64)s * N + c] = ub[s];
    if (ebar) ebar[(u64)s * N + c] += f0b[s] + f1b[s];
  }
  for (int s = NS; s < nsp; ++s) {
    double l = lam[(u64)s * N + c];
    if (clamp && Uout && !(Uout[(u64)s * N + c] > 0.0)) l = 0.0;
    lam_out[(u64)s * N + c] = l;
  }
#undef K
#undef EM
#undef WV
}
#define RS_VJP(NAME, HE, KZ)                                                                 \
  extern "C" __global__ void __launch_bounds__(128) NAME(int nc, int nsp,                   \
      const double* __restrict__ U, const double* __restrict__ Uout,                        \
      const double* __restrict__ lam, double* __restrict__ lam_out,                         \
      const double* __restrict__ kr, const double* __restrict__ em,                         \
      double* __restrict__ ebar, double dt, int clamp, const double* __restrict__ kzi) {     \
    vjp_body<HE, KZ>(nc, nsp, U, Uout, lam, lam_out, kr, em, ebar, dt, clamp, kzi);          \
  }
RS_VJP(rs_jit_vjp_0, false, false)
RS_VJP(rs_jit_vjp_1, true, false)
RS_VJP(rs_jit_vjpk_0, false, true)
RS_VJP(rs_jit_vjpk_1, true, true)

// the production reciprocal applied elementwise (accuracy check against IEEE division)
extern "C" __global__ void rs_jit_rcp(const double* __restrict__ x, double* __restrict__ r,
                                      int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = rcp_nr(x[i]);
}
)";
  return o.str();
}

// ------------------------------------------------------------------ compile cache
struct Compiled {
  cudaLibrary_t lib = nullptr;
  double ms = 0;
};
std::mutex g_mu;
std::map<std::string, Compiled> g_cache;  // source + options -> loaded library (process life)

}  // namespace

// NVRTC compile of generated source to an sm_103a cubin (no device needed).  With verbose
// the log carries ptxas's resource usage (registers, spill stores/loads, shared memory).
bool jit_compile(const std::string& src, bool strict, bool verbose, std::vector<char>* cubin,
                 std::string* log) {
  const Nvrtc& N = nvrtc();
  if (!N.ok()) {
    *log = N.why;
    return false;
  }
  nvrtcProgram prog = nullptr;
  nvrtcResult r = N.create(&prog, src.c_str(), "rs_chem_jit.cu", 0, nullptr, nullptr);
  if (r != NVRTC_SUCCESS) {
    *log = std::string("nvrtcCreateProgram: ") + N.err(r);
    return false;
  }
  (void)strict;  // the source itself differs between the builds (RS_FMA, RS_QUOT)
  std::vector<const char*> opts = {"-arch=sm_103a", "-std=c++17", "--fmad=false"};
  if (verbose) opts.push_back("--ptxas-options=-v");
  r = N.compile(prog, (int)opts.size(), opts.data());
  size_t n = 0;
  N.log_size(prog, &n);
  std::string text(n, '\0');
  if (n) N.log(prog, &text[0]);
  while (!text.empty() && text.back() == '\0') text.pop_back();
  if (r != NVRTC_SUCCESS) {
    *log = std::string("nvrtcCompileProgram: ") + N.err(r) + "\n" + text;
    N.destroy(&prog);
    return false;
  }
  *log = text;
  if (cubin) {
    size_t nb = 0;
    N.cubin_size(prog, &nb);
    cubin->resize(nb);
    N.cubin(prog, cubin->data());
  }
  N.destroy(&prog);
  return true;
}

namespace {

bool compile_and_load(const std::string& src, bool strict, Compiled* out, std::string* why) {
  auto t0 = std::chrono::steady_clock::now();
  std::vector<char> cubin;
  std::string log;
  if (!jit_compile(src, strict, false, &cubin, &log)) {
    *why = log.substr(0, 4000);
    return false;
  }
  cudaError_t e = cudaLibraryLoadData(&out->lib, cubin.data(), nullptr, nullptr, 0, nullptr,
                                      nullptr, 0);
  if (e != cudaSuccess) {
    *why = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
    return false;
  }
  out->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                .count();
  return true;
}

}  // namespace

const char* const kJitVariantNames[kJitVariants] = {"regs", "smem", "regs2", "split"};

bool jit_chem_eligible(const MechTables& T) {
  return T.ns >= 1 && T.ns <= 32 && T.nlu <= 256 && T.nr <= 160 && T.npart <= 320;
}

std::string jit_chem_source(const MechTables& T, bool strict) {
  return generate(T, 1.0 / (2.0 + std::sqrt(2.0)), 6.0 + std::sqrt(2.0), strict,
                  smem_bytes(T) <= kSmemCap);
}

std::shared_ptr<JitChem> jit_chem_build(const MechTables& T, double ros_d, double ros_c32,
                                        bool strict, std::string* why) {
  if (!jit_chem_eligible(T)) {
    *why = "mechanism too large for straight-line kernels";
    return nullptr;
  }
  const bool with_smem = smem_bytes(T) <= kSmemCap;
  std::string src = generate(T, ros_d, ros_c32, strict, with_smem);
  std::string key = src + (strict ? "|strict" : "|fast");
  Compiled cmp;
  double ms = 0;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      cmp = it->second;
    } else {
      if (!compile_and_load(src, strict, &cmp, why)) return nullptr;
      g_cache[key] = cmp;
      ms = cmp.ms;
    }
  }
  auto J = std::make_shared<JitChem>();
  J->compile_ms = ms;
  auto get = [&](cudaKernel_t* k, const char* name) {
    cudaError_t e = cudaLibraryGetKernel(k, cmp.lib, name);
    if (e != cudaSuccess && why->empty())
      *why = std::string("cudaLibraryGetKernel(") + name + "): " + cudaGetErrorString(e);
    return e == cudaSuccess;
  };
  bool ok = get(&J->attempt[0][0], "rs_jit_attempt_r0") && get(&J->attempt[0][1], "rs_jit_attempt_r1") &&
            get(&J->attempt[2][0], "rs_jit_attempt_q0") && get(&J->attempt[2][1], "rs_jit_attempt_q1") &&
            get(&J->per_cell[0], "rs_jit_per_cell_0") && get(&J->per_cell[1], "rs_jit_per_cell_1") &&
            get(&J->rcp, "rs_jit_rcp") && get(&J->vjp[0], "rs_jit_vjp_0") &&
            get(&J->vjp[1], "rs_jit_vjp_1") && get(&J->step[0], "rs_jit_step_0") &&
            get(&J->step[1], "rs_jit_step_1") && get(&J->vjpk[0], "rs_jit_vjpk_0") &&
            get(&J->vjpk[1], "rs_jit_vjpk_1");
  if (!ok) return nullptr;
  // the shared-memory variants: their dynamic shared memory, or dropped where it cannot be set
  auto shared_variant = [&](int v, const char* n0, const char* n1, size_t bytes) {
    if (!get(&J->attempt[v][0], n0) || !get(&J->attempt[v][1], n1)) {
      J->attempt[v][0] = J->attempt[v][1] = nullptr;
      return;
    }
    J->attempt_smem[v] = bytes;
    for (int he = 0; he < 2; ++he) {
      cudaError_t e = cudaFuncSetAttribute((const void*)J->attempt[v][he],
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes);
      if (e != cudaSuccess) {
        cudaGetLastError();
        J->attempt[v][0] = J->attempt[v][1] = nullptr;
        J->attempt_smem[v] = 0;
        return;
      }
    }
  };
  if (with_smem) shared_variant(1, "rs_jit_attempt_s0", "rs_jit_attempt_s1", smem_bytes(T));
  if (split_slots(T) > 0)
    shared_variant(3, "rs_jit_attempt_h0", "rs_jit_attempt_h1",
                   (size_t)split_slots(T) * kBlock * sizeof(double));
  for (int v = 0; v < kJitVariants; ++v) {
    cudaFuncAttributes fa{};
    if (J->attempt[v][0] && cudaFuncGetAttributes(&fa, (const void*)J->attempt[v][0]) == cudaSuccess)
      J->regs[v] = fa.numRegs;
    else
      cudaGetLastError();
  }
  why->clear();
  return J;
}

void jit_launch_attempt(const JitChem& J, cudaStream_t st, int nc, int nsp, const Ctl* ctl,
                        double* U0, double* U1, const double* kr, const double* em,
                        double* part, double rtol, double atol, int clamp, double* F0,
                        double* F1) {
  const int v = J.attempt[J.variant][0] ? J.variant : 0;
  cudaKernel_t k = J.attempt[v][em ? 1 : 0];
  const unsigned char* c = reinterpret_cast<const unsigned char*>(ctl);
  if (!F0 || !F1) F0 = F1 = nullptr;
  void* args[] = {&c, &U0, &U1, &kr, &em, &part, &nc, &nsp, &rtol, &atol, &clamp, &F0, &F1};
  int nb = (nc + kBlock - 1) / kBlock;
  cudaLaunchKernel((const void*)k, dim3(nb), dim3(kBlock), args, J.attempt_smem[v], st);
}

void jit_launch_step(const JitChem& J, cudaStream_t st, int nc, int nsp, const Ctl* ctl,
                     double* U0, double* U1, const double* kr, const double* em, int clamp) {
  cudaKernel_t k = J.step[em ? 1 : 0];
  const unsigned char* c = reinterpret_cast<const unsigned char*>(ctl);
  void* args[] = {&c, &U0, &U1, &kr, &em, &nc, &nsp, &clamp};
  cudaLaunchKernel((const void*)k, dim3((nc + kBlock - 1) / kBlock), dim3(kBlock), args, 0, st);
}

void jit_launch_rcp(const JitChem& J, cudaStream_t st, const double* x, double* r, int n) {
  void* args[] = {&x, &r, &n};
  cudaLaunchKernel((const void*)J.rcp, dim3((n + 255) / 256), dim3(256), args, 0, st);
}

void jit_launch_vjp(const JitChem& J, cudaStream_t st, int nc, int nsp, const double* U,
                    const double* Uout, const double* lam, double* lam_out, const double* kr,
                    const double* em, double* ebar, double dt, int clamp, const double* kz) {
  cudaKernel_t k = kz ? J.vjpk[em ? 1 : 0] : J.vjp[em ? 1 : 0];
  void* args[] = {&nc, &nsp, &U, &Uout, &lam, &lam_out, &kr, &em, &ebar, &dt, &clamp, &kz};
  cudaLaunchKernel((const void*)k, dim3((nc + 127) / 128), dim3(128), args, 0, st);
}

void jit_launch_per_cell(const JitChem& J, cudaStream_t st, int nc, int nsp, int nblocks,
                         int threads, double* U, const double* kr, const double* em,
                         double* dtc, double* steps, unsigned long long* queue, int* status,
                         const PerCellArgs& a) {
  cudaKernel_t k = J.per_cell[em ? 1 : 0];
  PerCellArgs av = a;
  void* args[] = {&nc, &nsp, &U, &kr, &em, &dtc, &steps, &queue, &status, &av};
  cudaLaunchKernel((const void*)k, dim3(nblocks), dim3(threads), args, 0, st);
}

}  // namespace rs
