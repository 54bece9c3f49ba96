// rs_api.cu -- the C ABI of libreseact_gb300.so (declared in include/reseact_gb300.h).
//
// Host side only: validates the configuration, derives the sparse mechanism tables, owns all
// device memory and the CUDA stream, uploads forcing, and drives the device-resident adaptive
// loops of one Lie-Trotter macro step (transport SSPRK43 then chemistry ROS23 over the same
// window, op_split.jl:100-164 / run_reseact_reactant.jl:310-355).  No C++ exception crosses
// the ABI; failures return rs_status and leave their text in rs_last_error.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/reseact_gb300.h"
#include "rs_device.cuh"
#include "rs_kernels.h"
#include "rs_jit.h"
#include "rs_mech.h"

namespace {

using rs::Ctl;

struct RsError : std::runtime_error {
  rs_status code;
  RsError(rs_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      throw RsError(e_ == cudaErrorMemoryAllocation ? RS_ERR_NOMEM : RS_ERR_CUDA,       \
                    std::string(#call) + ": " + cudaGetErrorString(e_));                \
  } while (0)

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  void alloc(size_t count) {
    if (p && n >= count) return;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count == 0) return;
    CK(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void upload(const T* h, size_t count, cudaStream_t st) {
    alloc(count);
    if (count) CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, st));
  }
  void zero(cudaStream_t st) {
    if (p) CK(cudaMemsetAsync(p, 0, n * sizeof(T), st));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// ------------------------------------------------------------------ mechanism tables
using rs::MechTables;

MechTables derive_tables(const rs_mechanism& m, bool natural_order) {
  MechTables T;
  if (m.n_species <= 0 || m.n_reactions < 0) throw RsError(RS_ERR_INVALID, "empty mechanism");
  if (!m.react_ptr || !m.prod_ptr || !m.prog_ptr) throw RsError(RS_ERR_INVALID, "null tables");
  T.ns = m.n_species;
  T.nr = m.n_reactions;
  T.comb = m.combinatoric;
  int ns = T.ns, nr = T.nr;
  T.rptr.assign(m.react_ptr, m.react_ptr + nr + 1);
  int nre = T.rptr[nr];
  T.rsp.assign(m.react_species, m.react_species + nre);
  T.rnu.assign(m.react_nu, m.react_nu + nre);
  for (int e = 0; e < nre; ++e)
    if (T.rsp[e] < 0 || T.rsp[e] >= ns || T.rnu[e] < 1 || T.rnu[e] > 8)
      throw RsError(RS_ERR_INVALID, "bad reactant entry");
  std::vector<double> net((size_t)nr * ns, 0.0);
  for (int r = 0; r < nr; ++r) {
    std::set<int> seen;
    for (int e = T.rptr[r]; e < T.rptr[r + 1]; ++e) {
      if (!seen.insert(T.rsp[e]).second)
        throw RsError(RS_ERR_INVALID, "species repeated among the reactants of one reaction");
      net[(size_t)r * ns + T.rsp[e]] -= T.rnu[e];
    }
    for (int e = m.prod_ptr[r]; e < m.prod_ptr[r + 1]; ++e) {
      int s = m.prod_species[e];
      if (s < 0 || s >= ns) throw RsError(RS_ERR_INVALID, "bad product species");
      net[(size_t)r * ns + s] += m.prod_coef[e];
    }
  }
  // RHS terms per species, reactions ascending
  T.rhs_ptr.push_back(0);
  for (int s = 0; s < ns; ++s) {
    for (int r = 0; r < nr; ++r)
      if (net[(size_t)r * ns + s] != 0.0) {
        T.rhs_r.push_back(r);
        T.rhs_c.push_back(net[(size_t)r * ns + s]);
      }
    T.rhs_ptr.push_back((int)T.rhs_r.size());
  }
  // partials, reaction order then reactant-entry order
  for (int r = 0; r < nr; ++r)
    for (int e = T.rptr[r]; e < T.rptr[r + 1]; ++e) {
      T.part_r.push_back(r);
      T.part_q.push_back(T.rsp[e]);
      T.part_e.push_back(e);
    }
  T.npart = (int)T.part_r.size();
  std::set<std::pair<int, int>> jpat;
  for (int p = 0; p < T.npart; ++p)
    for (int s = 0; s < ns; ++s)
      if (net[(size_t)T.part_r[p] * ns + s] != 0.0) jpat.insert({s, T.part_q[p]});
  // Elimination order of the pivot-free LU of W = I - gamma h J.  The reference's blocksolve
  // eliminates in natural species order; the strict build keeps that order (bit-compatible
  // with the CPU restatement).  The production build eliminates in a greedy minimum-fill
  // order (ties: fewest multiply-adds, then species index): the same symmetric permutation
  // of rows and columns, so the diagonal stays the pivot, and the same solution to roundoff,
  // with fewer fill slots and updates (SuperFast 82 -> 71 slots, 131 -> 83 updates; the
  // 30-species synthetic mechanism 532 -> 290 slots, 2631 -> 619 updates).
  std::vector<int> ord(ns);
  for (int i = 0; i < ns; ++i) ord[i] = i;
  if (!natural_order) {
    std::set<std::pair<int, int>> P = jpat;
    for (int i = 0; i < ns; ++i) P.insert({i, i});
    std::vector<int> left(ord), chosen;
    while (!left.empty()) {
      long best_fill = -1, best_cost = 0;
      size_t best_at = 0;
      for (size_t a = 0; a < left.size(); ++a) {
        int k = left[a];
        long nrow = 0, ncol = 0, nfill = 0;
        for (int i : left)
          if (i != k && P.count({i, k})) ++nrow;
        for (int j : left)
          if (j != k && P.count({k, j})) ++ncol;
        for (int i : left)
          if (i != k && P.count({i, k}))
            for (int j : left)
              if (j != k && P.count({k, j}) && !P.count({i, j})) ++nfill;
        long cost = nrow * ncol;
        if (best_fill < 0 || nfill < best_fill || (nfill == best_fill && cost < best_cost)) {
          best_fill = nfill;
          best_cost = cost;
          best_at = a;
        }
      }
      int k = left[best_at];
      for (int i : left)
        if (i != k && P.count({i, k}))
          for (int j : left)
            if (j != k && P.count({k, j})) P.insert({i, j});
      chosen.push_back(k);
      left.erase(left.begin() + best_at);
    }
    ord = chosen;
  }
  std::vector<int> pos(ns);
  for (int k = 0; k < ns; ++k) pos[ord[k]] = k;
  T.ord = ord;
  // symbolic elimination in pivot-position space
  std::set<std::pair<int, int>> fill;
  for (auto& e : jpat) fill.insert({pos[e.first], pos[e.second]});
  for (int i = 0; i < ns; ++i) fill.insert({i, i});
  for (int k = 0; k < ns; ++k) {
    std::vector<int> rows, cols;
    for (int i = k + 1; i < ns; ++i)
      if (fill.count({i, k})) rows.push_back(i);
    for (int j = k + 1; j < ns; ++j)
      if (fill.count({k, j})) cols.push_back(j);
    for (int i : rows)
      for (int j : cols) fill.insert({i, j});
  }
  std::map<std::pair<int, int>, int> slot;  // keyed by (row, col) positions
  for (auto& e : fill) {  // std::set orders row-major
    int id = (int)slot.size();
    slot[e] = id;
    T.slot_row.push_back(ord[e.first]);  // species indices
    T.slot_col.push_back(ord[e.second]);
  }
  T.nlu = (int)slot.size();
  for (int k = 0; k < ns; ++k) T.lu_diag.push_back(slot[{k, k}]);  // pivot k (position)
  // Jacobian entries (row-major in species), terms in partial (= reaction) order
  T.jac_ptr.push_back(0);
  for (auto& e : jpat) {
    int s = e.first, q = e.second;
    for (int p = 0; p < T.npart; ++p) {
      double c = net[(size_t)T.part_r[p] * ns + s];
      if (T.part_q[p] == q && c != 0.0) {
        T.jac_part.push_back(p);
        T.jac_coef.push_back(c);
      }
    }
    T.jac_slot.push_back(slot[{pos[s], pos[q]}]);
    T.jac_diag.push_back(s == q ? 1 : 0);
    T.jac_ptr.push_back((int)T.jac_part.size());
  }
  T.njac = (int)jpat.size();
  // elimination schedule (positions)
  T.elim_ptr.push_back(0);
  T.upd_ptr.push_back(0);
  for (int k = 0; k < ns; ++k) {
    std::vector<int> rows, cols;
    for (int i = k + 1; i < ns; ++i)
      if (fill.count({i, k})) rows.push_back(i);
    for (int j = k + 1; j < ns; ++j)
      if (fill.count({k, j})) cols.push_back(j);
    for (int i : rows) {
      T.elim_lik.push_back(slot[{i, k}]);
      for (int j : cols) {
        T.upd_dst.push_back(slot[{i, j}]);
        T.upd_src.push_back(slot[{k, j}]);
      }
      T.upd_ptr.push_back((int)T.upd_dst.size());
    }
    T.elim_ptr.push_back((int)T.elim_lik.size());
  }
  // triangular solves: pivots in position order, vector entries by species index
  T.low_ptr.push_back(0);
  for (int k = 0; k < ns; ++k) {
    for (int i = k + 1; i < ns; ++i)
      if (fill.count({i, k})) {
        T.low_row.push_back(ord[i]);
        T.low_slot.push_back(slot[{i, k}]);
      }
    T.low_ptr.push_back((int)T.low_row.size());
  }
  // Back substitution, row i: x_i = (b_i - sum_j U_ij x_j) U_ii^-1.  The natural order (the
  // strict build) sums in ascending j, as blocksolve; the production order in descending j, the
  // order in which the x_j become known, so that a column sweep (the G-lanes-per-cell kernels:
  // subtract U_ij x_j from every row of column j as soon as x_j is known) adds each row's terms
  // in the same order as the row loop of the thread-per-cell kernels -- the same bits.
  T.up_ptr.push_back(0);
  for (int i = 0; i < ns; ++i) {
    for (int jj = i + 1; jj < ns; ++jj) {
      const int j = natural_order ? jj : ns - 1 - (jj - i - 1);
      if (fill.count({i, j})) {
        T.up_col.push_back(ord[j]);
        T.up_slot.push_back(slot[{i, j}]);
      }
    }
    T.up_ptr.push_back((int)T.up_col.size());
  }
  // the same schedule for kernels that spread one cell over several lanes: the updates of
  // pivot k (each dst slot at most once per pivot) with their multiplier slots, and the
  // upper factor by columns
  for (int k = 0; k <= ns; ++k) T.pupd_ptr.push_back(T.upd_ptr[T.elim_ptr[k]]);
  T.upd_lik.assign(T.upd_dst.size(), 0);
  for (size_t mm = 0; mm < T.elim_lik.size(); ++mm)
    for (int u = T.upd_ptr[mm]; u < T.upd_ptr[mm + 1]; ++u) T.upd_lik[u] = T.elim_lik[mm];
  T.upc_ptr.push_back(0);
  for (int j = 0; j < ns; ++j) {
    for (int i = 0; i < j; ++i)
      if (fill.count({i, j})) {
        T.upc_row.push_back(ord[i]);
        T.upc_slot.push_back(slot[{i, j}]);
      }
    T.upc_ptr.push_back((int)T.upc_row.size());
  }
  // rate programs: validate stack discipline
  T.prog_ptr.assign(m.prog_ptr, m.prog_ptr + nr + 1);
  int np = T.prog_ptr[nr];
  T.prog_op.assign(m.prog_op, m.prog_op + np);
  T.prog_val.assign(m.prog_val, m.prog_val + np);
  T.params.assign(m.params ? m.params : nullptr, m.params ? m.params + m.n_params : nullptr);
  if (T.params.empty()) T.params.push_back(0.0);
  for (int r = 0; r < nr; ++r) {
    int sp = 0;
    for (int e = T.prog_ptr[r]; e < T.prog_ptr[r + 1]; ++e) {
      int op = T.prog_op[e];
      if (op <= 3) {
        ++sp;
        if (op == 3 && ((int)T.prog_val[e] < 0 || (int)T.prog_val[e] >= m.n_params))
          throw RsError(RS_ERR_INVALID, "rate program parameter out of range");
      } else if (op >= 10 && op <= 14) {
        --sp;
      } else if (!(op == 15 || (op >= 20 && op <= 23))) {
        throw RsError(RS_ERR_INVALID, "unknown rate-program opcode");
      }
      if (sp < 1 || sp > rs::kMaxProgStack) throw RsError(RS_ERR_INVALID, "rate program stack");
    }
    if (sp != 1) throw RsError(RS_ERR_INVALID, "rate program leaves a stack depth != 1");
  }
  return T;
}

// ------------------------------------------------------------------ handle
struct Profile {
  std::vector<std::string> names;
  std::vector<double> launches, ms;
  struct Pending {
    int fam;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  bool on = false;
};

}  // namespace

struct rs_handle {
  rs_config cfg{};
  std::string err;
  cudaStream_t st = nullptr;
  int nlon = 0, nlat = 0, nlev = 0, nsp = 0, ntr = 0;
  size_t nc = 0;
  MechTables mt;
  rs::DevMech dm{};
  rs::LaunchCtx lc{};
  // mechanism tables on device
  std::vector<DevBuf<int>> itabs;
  std::vector<DevBuf<double>> dtabs;
  DevBuf<int> slot_row, slot_col;
  // state and scratch
  DevBuf<double> U[2], S1, S2, S3, fx, fy, fz, partial, krates, T, P, emis, io, io2;
  DevBuf<double> mx, my, mz, qw, qe, qs, qn, gx, gylo, gyhi, vsA, vsB, veAB, veC, veD, dtcell,
      stepcell, totals;
  DevBuf<float> qhi, qlo;  // mixed-precision transport: split planes
  DevBuf<float> gx2, gylo2, gyhi2, vsA2, vsB2, veAB2, veC2, veD2;  // (hi, lo) pairs
  DevBuf<float> mx2, my2, mz2;  // the face fluxes as (hi, lo) pairs (mixed precision)
  rs::MixedTmaps* tmaps = nullptr;  // bulk-copy staging of the mixed pencils (null: unavailable)
  void* noalloc_base = nullptr;     // this device's scratch of rs_ros23_attempt_noalloc
  std::string tmaps_why;
  int staging = RS_STAGING_AUTO;
  DevBuf<int> tma_err;              // set by a pencil kernel whose staging wait ran out
  DevBuf<Ctl> ctl;  // [0] transport, [1] chemistry, [2] single-step scratch
  DevBuf<int> flag;
  DevBuf<unsigned long long> queue;
  Ctl* hctl = nullptr;  // pinned mirror
  int* hflag = nullptr;
  int cur = 0;
  double launches = 0;  // kernels launched by the current rs_macro_step
  bool have_forcing = false, rates_dirty = true, rates_override = false, have_emis = false;
  double omega = 0.0;
  std::vector<double> dp_host;
  Profile prof;
  rs::DevTransport<double> dt{};
  // discrete adjoint: recorded macro steps (checkpoint + accepted (t, dt) of both halves)
  struct Rec {
    DevBuf<double> ck;
    double t0 = 0, t1 = 0;
    std::vector<double> seqT, seqC;  // flattened (t, dt) pairs
    // device tape: the state before every accepted step, then the end state, at
    // tape_arena + tape_off (complete: the backward needs no replay)
    size_t tape_off = 0;
    size_t tape_cap = 0;  // states available to this macro step
    bool tape_ok = false;
    size_t kz_off = 0, kz_cap = 0;  // its chemistry stage slots (k1, z2 per accepted step)
    bool kz_ok = false;             // the forward wrote every chemistry step's stages
    size_t f_off = 0, f_cap = 0;    // its transport stage slots (F0..F3, V1, V2, V4)
    bool f_set = false, f_ok = false;
  };
  bool rec_on = false;
  // tape budget in bytes (-1: a quarter of the free device memory when recording starts,
  // 0: always replay), the arena reserved for it and the doubles the recorded steps use
  long long tape_budget = -1;
  DevBuf<double> tape_arena;
  size_t tape_limit = 0, tape_used = 0;
  DevBuf<int> ntape;  // per half: states stored, slot overflow
  // the stage tape (specialised chemistry kernels): k1 and z2 of every accepted chemistry
  // step, [2][ns][nc] doubles each, in its own arena (its share of the tape budget), and the
  // replay's scratch of the same layout
  DevBuf<double> kz_arena, kzs;
  size_t kz_limit = 0, kz_used = 0;
  // the transport stage tape (FP64 scheme without PBL mixing): per accepted transport step
  // the stage tendencies F0..F3 and stage states V1, V2, V4, [7][nsp][nc] doubles; its arena,
  // and the replay's scratch of the same layout
  DevBuf<double> f_arena, fs;
  size_t f_limit = 0, f_used = 0;
  std::vector<Rec> recs;
  std::vector<DevBuf<double>> ck_pool;  // checkpoint buffers kept for reuse across recordings
  DevBuf<double> seqbuf, lam, lam2, ebar, tape, adj, G, Cf;
  DevBuf<int> nseq;
  // device-driven adaptive loops: one CUDA graph per half, a conditional WHILE node whose body
  // is one attempt + the controller; rebuilt when forcing or rate constants change
  struct LoopGraph {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    bool valid = false;
    bool with_tape = false;  // body stores the adjoint tape after the controller (recording)
  };
  LoopGraph loops[2];
  cudaStream_t cap = nullptr;
  bool use_graphs = true;
  // launch shapes picked by rs_autotune (defaults until it runs)
  struct Tune {
    int pc_threads = 128, pc_blocks_per_sm = 4;      // per-cell chemistry kernel
    int pc_group = 0;  // lanes per cell of the table-walking per-cell kernel (0: one thread)
    int pc_regcap = 0;  // 1: the table-walking per-cell kernel capped at 32 registers
    int pencil = 32, rows = 8, xthreads = 128;        // transport pencil kernels
    int xgroups = 1, yzgroups = 1;                    // their tracer groups
    int mpencil = 16, mrows = 16, mxthreads = 128;    // mixed-precision pencil kernels
    int msper_x = 1 << 20, msper_yz = 1;             // tracers per block (clamped to ntr)
    int mbulk_x = 1, mbulk_yz = 1;                    // bulk-copy staging per direction
    int mstream_x = 1, mstream_yz = 1;                // streaming kernels instead of pencils
  } tune;
  // mechanism-specialised chemistry kernels (null: not built) and the kind in use
  // full PBL mixing: host inputs, and the derived per-layer fraction / weight and column
  // normaliser on the device (recomputed when an input changes)
  std::vector<double> pblh_host, ps_host, hyb_a_host, hyb_b_host, tsfc_host;
  double tau_pbl = 0.0;
  bool pbl_on = false;
  DevBuf<double> pbl_f, pbl_w, pbl_den, pbl_qbar;
  // pressure fixer: host inputs (horizontal fluxes, geometry, dPS/dt) and the air-mass
  // divergence correction on the device; the diagnosed Mz replaces the mz field
  std::vector<double> mx_host, my_host, gx_host, gylo_host, gyhi_host, dpsdt_host;
  bool fixer_on = false;
  DevBuf<double> mcorr;
  std::shared_ptr<rs::JitChem> jit;
  DevBuf<double> fsal[2];  // f(U[b]) planes [ns][nc] for the specialised global-dt attempts
  std::string jit_why;
  int chem_kernel = RS_CHEM_KERNEL_AUTO;
};

namespace {

void set_err(rs_handle* h, const std::string& s) {
  if (h) h->err = s;
}

// --- profiling helpers: events bracket each launch group while profiling is on
int fam_id(rs_handle* h, const char* name) {
  auto& P = h->prof;
  for (size_t i = 0; i < P.names.size(); ++i)
    if (P.names[i] == name) return (int)i;
  P.names.push_back(name);
  P.launches.push_back(0);
  P.ms.push_back(0);
  return (int)P.names.size() - 1;
}
cudaEvent_t get_event(rs_handle* h) {
  auto& P = h->prof;
  if (!P.pool.empty()) {
    cudaEvent_t e = P.pool.back();
    P.pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  CK(cudaEventCreate(&e));
  return e;
}
struct Scope {
  rs_handle* h;
  int fam = -1;
  cudaEvent_t a = nullptr;
  Scope(rs_handle* hh, const char* name) : h(hh) {
    if (!h->prof.on) return;
    fam = fam_id(h, name);
    a = get_event(h);
    CK(cudaEventRecord(a, h->st));
  }
  ~Scope() {
    if (fam < 0) return;
    cudaEvent_t b = get_event(h);
    cudaEventRecord(b, h->st);
    h->prof.pending.push_back({fam, a, b});
  }
};
void collect_profile(rs_handle* h) {
  auto& P = h->prof;
  if (P.pending.empty()) return;
  CK(cudaStreamSynchronize(h->st));
  for (auto& p : P.pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, p.a, p.b));
    P.launches[p.fam] += 1;
    P.ms[p.fam] += ms;
    P.pool.push_back(p.a);
    P.pool.push_back(p.b);
  }
  P.pending.clear();
}

template <typename T>
const T* upload_tab(rs_handle* h, std::vector<DevBuf<T>>& store, const std::vector<T>& v) {
  store.emplace_back();
  std::vector<T> w = v;
  if (w.empty()) w.push_back(T(0));
  store.back().upload(w.data(), w.size(), h->st);
  return store.back().p;
}

void build_device_mech(rs_handle* h) {
  auto& T = h->mt;
  auto& D = h->dm;
  auto ui = [&](const std::vector<int>& v) { return upload_tab(h, h->itabs, v); };
  auto ud = [&](const std::vector<double>& v) { return upload_tab(h, h->dtabs, v); };
  h->itabs.reserve(40);
  h->dtabs.reserve(8);
  D.ns = T.ns;
  D.nr = T.nr;
  D.nlu = T.nlu;
  D.npart = T.npart;
  D.njac = T.njac;
  D.rptr = ui(T.rptr); D.rsp = ui(T.rsp); D.rnu = ui(T.rnu);
  D.rhs_ptr = ui(T.rhs_ptr); D.rhs_r = ui(T.rhs_r); D.rhs_c = ud(T.rhs_c);
  D.part_r = ui(T.part_r); D.part_q = ui(T.part_q); D.part_e = ui(T.part_e);
  D.jac_ptr = ui(T.jac_ptr); D.jac_slot = ui(T.jac_slot); D.jac_diag = ui(T.jac_diag);
  D.jac_part = ui(T.jac_part); D.jac_coef = ud(T.jac_coef);
  D.lu_diag = ui(T.lu_diag);
  D.ord = ui(T.ord);
  D.elim_ptr = ui(T.elim_ptr); D.elim_lik = ui(T.elim_lik); D.upd_ptr = ui(T.upd_ptr);
  D.upd_dst = ui(T.upd_dst); D.upd_src = ui(T.upd_src);
  D.low_ptr = ui(T.low_ptr); D.low_row = ui(T.low_row); D.low_slot = ui(T.low_slot);
  D.up_ptr = ui(T.up_ptr); D.up_col = ui(T.up_col); D.up_slot = ui(T.up_slot);
  D.pupd_ptr = ui(T.pupd_ptr); D.upd_lik = ui(T.upd_lik);
  D.upc_ptr = ui(T.upc_ptr); D.upc_row = ui(T.upc_row); D.upc_slot = ui(T.upc_slot);
  D.prog_ptr = ui(T.prog_ptr); D.prog_op = ui(T.prog_op); D.prog_val = ud(T.prog_val);
  D.params = ud(T.params);
  D.combinatoric = T.comb;
  D.ros_d = 1.0 / (2.0 + std::sqrt(2.0));
  D.ros_c32 = 6.0 + std::sqrt(2.0);
  h->slot_row.upload(T.slot_row.data(), T.slot_row.size(), h->st);
  h->slot_col.upload(T.slot_col.data(), T.slot_col.size(), h->st);
}

// (hi, lo) float pairs of a double array for the compensated FP32 transport:
// hi = fl32(v), lo = fl32(v - hi); hi + lo = v to about 2^-48 relative
void upload_pairs(const std::vector<double>& v, DevBuf<float>& d, cudaStream_t st) {
  std::vector<float> w(2 * v.size());
  for (size_t i = 0; i < v.size(); ++i) {
    const float hi = (float)v[i];
    w[2 * i] = hi;
    w[2 * i + 1] = (float)(v[i] - (double)hi);
  }
  d.upload(w.data(), w.size(), st);
  CK(cudaStreamSynchronize(st));  // w is a temporary
}

// The air-mass face fluxes as (hi, lo) pairs for the compensated FP32 kernels (after every
// flux change, including the pressure fixer's diagnosed Mz).
void make_flux_pairs(rs_handle* h) {
  h->mx2.alloc(2 * h->mx.n);
  h->my2.alloc(2 * h->my.n);
  h->mz2.alloc(2 * h->mz.n);
  rs::launch_make_pairs(h->st, h->mx.p, reinterpret_cast<float2*>(h->mx2.p), h->mx.n);
  rs::launch_make_pairs(h->st, h->my.p, reinterpret_cast<float2*>(h->my2.p), h->my.n);
  rs::launch_make_pairs(h->st, h->mz.p, reinterpret_cast<float2*>(h->mz2.p), h->mz.n);
  CK(cudaGetLastError());
}

// Lat-lon geometry on the unit sphere (same formulas and order as the CPU restatement).
void build_geometry(rs_handle* h) {
  const rs_grid& g = h->cfg.grid;
  const double d2r = 0.017453292519943295;
  std::vector<double> phie(g.nlat + 1), ce(g.nlat + 1), gx(g.nlat), gl(g.nlat), gh(g.nlat);
  for (int j = 0; j <= g.nlat; ++j) {
    double p = g.lat0_deg + (j - 0.5) * g.dlat_deg;
    p = std::min(90.0, std::max(-90.0, p));
    phie[j] = p;
    ce[j] = (std::fabs(p) >= 90.0) ? 0.0 : std::cos(p * d2r);
  }
  double dlon = g.dlon_deg * d2r;
  for (int j = 0; j < g.nlat; ++j) {
    double dS = std::sin(phie[j + 1] * d2r) - std::sin(phie[j] * d2r);
    double dphi = (phie[j + 1] - phie[j]) * d2r;
    gx[j] = dphi / (dlon * dS);
    gl[j] = ce[j] / dS;
    gh[j] = ce[j + 1] / dS;
  }
  h->gx.upload(gx.data(), gx.size(), h->st);
  h->gylo.upload(gl.data(), gl.size(), h->st);
  h->gyhi.upload(gh.data(), gh.size(), h->st);
  h->gx_host = gx;
  h->gylo_host = gl;
  h->gyhi_host = gh;
  if (h->cfg.precision == RS_PREC_MIXED) {
    upload_pairs(gx, h->gx2, h->st);
    upload_pairs(gl, h->gylo2, h->st);
    upload_pairs(gh, h->gyhi2, h->st);
  }
}

// CW84 nonuniform coefficients from dp (eqs. 1.6-1.7), mirror ghosts at the no-flux walls.
void build_vertical(rs_handle* h) {
  int nlev = h->nlev;
  size_t ncol = (size_t)h->nlon * h->nlat;
  std::vector<double> sA((nlev + 2) * ncol), sB((nlev + 2) * ncol), eAB((nlev + 1) * ncol),
      eC((nlev + 1) * ncol), eD((nlev + 1) * ncol);
  const std::vector<double>& dp = h->dp_host;
  auto D = [&](size_t col, int k) {
    int kk = k < 0 ? -1 - k : (k >= nlev ? 2 * nlev - 1 - k : k);
    return dp[(size_t)kk * ncol + col];
  };
  for (size_t col = 0; col < ncol; ++col) {
    for (int k = -1; k <= nlev; ++k) {
      double D0 = D(col, k - 1), D1 = D(col, k), D2 = D(col, k + 1);
      double c = D1 / (D0 + D1 + D2);
      sA[(size_t)(k + 1) * ncol + col] = c * (2.0 * D0 + D1) / (D2 + D1);
      sB[(size_t)(k + 1) * ncol + col] = c * (D1 + 2.0 * D2) / (D0 + D1);
    }
    for (int e = 0; e <= nlev; ++e) {
      int k = e - 1;
      double Dm = D(col, k - 1), D0 = D(col, k), D1 = D(col, k + 1), D2 = D(col, k + 2);
      double S = Dm + D0 + D1 + D2;
      double eA = D0 / (D0 + D1);
      double t1 = (Dm + D0) / (2.0 * D0 + D1);
      double t2 = (D2 + D1) / (2.0 * D1 + D0);
      double eB = (2.0 * D1 * D0 / (D0 + D1)) * (t1 - t2) / S;
      eAB[(size_t)e * ncol + col] = eA + eB;
      eC[(size_t)e * ncol + col] = -(D0 * t1) / S;
      eD[(size_t)e * ncol + col] = D1 * (D1 + D2) / (D0 + 2.0 * D1) / S;
    }
  }
  h->vsA.upload(sA.data(), sA.size(), h->st);
  h->vsB.upload(sB.data(), sB.size(), h->st);
  h->veAB.upload(eAB.data(), eAB.size(), h->st);
  h->veC.upload(eC.data(), eC.size(), h->st);
  h->veD.upload(eD.data(), eD.size(), h->st);
  if (h->cfg.precision == RS_PREC_MIXED) {
    upload_pairs(sA, h->vsA2, h->st);
    upload_pairs(sB, h->vsB2, h->st);
    upload_pairs(eAB, h->veAB2, h->st);
    upload_pairs(eC, h->veC2, h->st);
    upload_pairs(eD, h->veD2, h->st);
  }
  CK(cudaStreamSynchronize(h->st));  // the host vectors above are temporaries
}

void refresh_dt(rs_handle* h) {
  auto& T = h->dt;
  T.nlon = h->nlon; T.nlat = h->nlat; T.nlev = h->nlev;
  T.ntr = h->ntr; T.nsp = h->nsp;
  T.lon_bc = h->cfg.grid.lon_bc; T.lat_bc = h->cfg.grid.lat_bc;
  T.omega = h->omega;
  T.gx = h->gx.p; T.gylo = h->gylo.p; T.gyhi = h->gyhi.p;
  T.mx = h->mx.p; T.my = h->my.p; T.mz = h->mz.p;
  T.qw = h->qw.p; T.qe = h->qe.p; T.qs = h->qs.p; T.qn = h->qn.p;
  T.vsA = h->vsA.p; T.vsB = h->vsB.p; T.veAB = h->veAB.p; T.veC = h->veC.p; T.veD = h->veD.p;
  T.fx = h->fx.p; T.fy = h->fy.p; T.fz = h->fz.p;
  T.mixed = h->cfg.precision == RS_PREC_MIXED;
  T.qhi = h->qhi.p; T.qlo = h->qlo.p;
  auto f2 = [](const DevBuf<float>& b) { return reinterpret_cast<const float2*>(b.p); };
  T.gx2 = f2(h->gx2); T.gylo2 = f2(h->gylo2); T.gyhi2 = f2(h->gyhi2);
  T.vsA2 = f2(h->vsA2); T.vsB2 = f2(h->vsB2); T.veAB2 = f2(h->veAB2); T.veC2 = f2(h->veC2);
  T.veD2 = f2(h->veD2);
  T.acc = T.mixed ? reinterpret_cast<float2*>(h->fx.p) : nullptr;  // ntr*nc pairs fit in fx
  T.mx2 = f2(h->mx2); T.my2 = f2(h->my2); T.mz2 = f2(h->mz2);
  T.pencil = h->tune.pencil;
  T.rows = h->tune.rows;
  T.xthreads = h->tune.xthreads;
  T.xgroups = h->tune.xgroups;
  T.yzgroups = h->tune.yzgroups;
  T.mpencil = h->tune.mpencil;
  T.mrows = h->tune.mrows;
  T.mxthreads = h->tune.mxthreads;
  T.msper_x = h->tune.msper_x;
  T.msper_yz = h->tune.msper_yz;
  T.tma = (h->staging != RS_STAGING_PLAIN) ? h->tmaps : nullptr;
  T.tma_err = h->tma_err.p;
  T.mbulk_x = h->staging == RS_STAGING_BULK ? 1 : h->tune.mbulk_x;
  T.mbulk_yz = h->staging == RS_STAGING_BULK ? 1 : h->tune.mbulk_yz;
  // a staging mode set by rs_set_transport_staging selects the pencils
  T.mstream_x = h->staging == RS_STAGING_AUTO ? h->tune.mstream_x : 0;
  T.mstream_yz = h->staging == RS_STAGING_AUTO ? h->tune.mstream_yz : 0;
  T.pbl = h->pbl_on;
  T.pbl_f = h->pbl_f.p; T.pbl_w = h->pbl_w.p; T.pbl_den = h->pbl_den.p; T.pbl_qbar = h->pbl_qbar.p;
  T.pbl_tau = h->tau_pbl;
  T.pbl_rtau = h->tau_pbl > 0.0 ? 1.0 / h->tau_pbl : 0.0;
  T.mcorr = h->fixer_on ? h->mcorr.p : nullptr;
}

// Pressure fixer (reseact.esm Transport3D divh, divh_col, dp_col, divh_fix, Mz), per column:
//   divh_k = DxM + DyM (the kernels' expressions, steady fluxes), corr_k = (-dPSdt - sum divh)
//   * (dp_k / sum dp), Mz_0 = 0, Mz_{k+1} = Mz_k + -(dB_k dPSdt + (divh_k + corr_k)),
// sums from the surface up; corr goes to the air-mass equation, Mz replaces the mz field.
void build_fixer(rs_handle* h) {
  const rs_grid& g = h->cfg.grid;
  const size_t ncol = (size_t)g.nlon * g.nlat, nf = (size_t)g.nlon + 1;
  h->fixer_on = h->cfg.do_transport && h->dpsdt_host.size() == ncol &&
                h->hyb_b_host.size() == (size_t)g.nlev + 1 &&
                h->mx_host.size() == (size_t)g.nlev * g.nlat * nf &&
                h->my_host.size() == (size_t)g.nlev * (g.nlat + 1) * g.nlon;
  if (!h->fixer_on) return;
  if (h->omega != 0.0)
    throw RsError(RS_ERR_UNSUPPORTED, "the pressure fixer needs steady fluxes (flux_omega = 0)");
  const bool open_lat = g.lat_bc == RS_BC_OPEN;
  const double* dp = h->dp_host.data();
  const double* B = h->hyb_b_host.data();
  std::vector<double> divh(h->nc), corr(h->nc), mz((size_t)(g.nlev + 1) * ncol, 0.0);
  for (int j = 0; j < g.nlat; ++j)
    for (int i = 0; i < g.nlon; ++i) {
      const size_t col = (size_t)j * g.nlon + i;
      double hcol = 0.0, dcol = 0.0;
      for (int k = 0; k < g.nlev; ++k) {
        const size_t c = (size_t)k * ncol + col;
        const double mxw = h->mx_host[((size_t)k * g.nlat + j) * nf + i];
        const double mxe = h->mx_host[((size_t)k * g.nlat + j) * nf + i + 1];
        const double mys = (!open_lat && j == 0) ? 0.0
                         : h->my_host[((size_t)k * (g.nlat + 1) + j) * g.nlon + i];
        const double myn = (!open_lat && j + 1 == g.nlat) ? 0.0
                         : h->my_host[((size_t)k * (g.nlat + 1) + j + 1) * g.nlon + i];
        const double DxM = (mxe - mxw) * h->gx_host[j];
        const double DyM = myn * h->gyhi_host[j] - mys * h->gylo_host[j];
        divh[c] = DxM + DyM;
        hcol = hcol + divh[c];
        dcol = dcol + dp[c];
      }
      const double dps = h->dpsdt_host[col];
      double acc = 0.0;
      for (int k = 0; k < g.nlev; ++k) {
        const size_t c = (size_t)k * ncol + col;
        corr[c] = (-dps - hcol) * (dp[c] / dcol);
        const double fix = divh[c] + corr[c];
        acc = acc + -((B[k] - B[k + 1]) * dps + fix);
        mz[(size_t)(k + 1) * ncol + col] = acc;
      }
    }
  h->mz.upload(mz.data(), mz.size(), h->st);
  h->mcorr.upload(corr.data(), corr.size(), h->st);
}

// PBL fraction and weights of every layer (reseact.esm Transport3D p_pbl_top, pbl_f, pbl_wt):
//   p_top = PS exp(-(PBLH g) / (Rd T_surface)),  p_k = A_k + B_k PS (interface k, 0 = surface)
//   f_k = max(0, min(1, (min(PS, p_k) - max(p_top, p_k+1)) / dp_k)),  w_k = dp_k f_k,
//   den = max(sum_k w_k, 1 Pa), summed from the surface up.
void build_pbl(rs_handle* h) {
  const rs_grid& g = h->cfg.grid;
  const size_t ncol = (size_t)g.nlon * g.nlat;
  h->pbl_on = h->cfg.do_transport && h->tau_pbl > 0.0 && h->pblh_host.size() == ncol &&
              h->ps_host.size() == ncol && h->tsfc_host.size() == ncol &&
              h->hyb_a_host.size() == (size_t)g.nlev + 1 && h->hyb_b_host.size() == (size_t)g.nlev + 1;
  if (!h->pbl_on) return;
  const double g_acc = 9.80665, rd_air = 287.05;
  std::vector<double> F(h->nc), W(h->nc), D(ncol);
  const double* dp = h->dp_host.data();
  const double* A = h->hyb_a_host.data();
  const double* B = h->hyb_b_host.data();
  for (size_t col = 0; col < ncol; ++col) {
    const double PS = h->ps_host[col];
    const double ptop = PS * std::exp(-1.0 * ((h->pblh_host[col] * g_acc) / (rd_air * h->tsfc_host[col])));
    double wt = 0.0;
    for (int k = 0; k < g.nlev; ++k) {
      const size_t c = (size_t)k * ncol + col;
      const double lo = A[k] + B[k] * PS, up = A[k + 1] + B[k + 1] * PS;
      const double f = std::max(0.0, std::min(1.0, (std::min(PS, lo) - std::max(ptop, up)) / dp[c]));
      F[c] = f;
      W[c] = dp[c] * f;
      wt = wt + W[c];
    }
    D[col] = std::max(wt, 1.0);
  }
  h->pbl_f.upload(F.data(), F.size(), h->st);
  h->pbl_w.upload(W.data(), W.size(), h->st);
  h->pbl_den.upload(D.data(), D.size(), h->st);
  h->pbl_qbar.alloc((size_t)h->ntr * ncol);
}

// The transport stage tape applies to the FP64 scheme the adjoint differentiates, without PBL
// mixing (whose VJP needs the advective tendency on its own).
bool transport_stage_tape(const rs_handle* h) {
  return h->cfg.do_transport && !h->pbl_on && h->cfg.precision == RS_PREC_FP64;
}

Ctl make_ctl(rs_handle* h, double t0, double t1, double dt0, const rs_controller& c,
             double ntot) {
  Ctl k{};
  k.t = t0; k.dt = dt0; k.tend = t1; k.qold = c.qoldinit;
  k.nacc = 0; k.nrej = 0; k.iters = 0; k.eest = 0; k.maxiters = h->cfg.maxiters;
  k.beta1 = c.beta1; k.beta2 = c.beta2;
  k.invqmin = 1.0 / c.qmin; k.invqmax = 1.0 / c.qmax; k.gamma = c.gamma;
  k.qsmin = c.qsteady_min; k.qsmax = c.qsteady_max; k.qoldinit = c.qoldinit;
  k.ntot = ntot; k.omega = h->omega;
  k.ros_d = h->dm.ros_d;
  k.seq = nullptr;
  k.nseq = nullptr;
  k.seqcap = 0;
  return k;
}

void ensure_rates(rs_handle* h) {
  if (!h->rates_dirty || h->rates_override) return;
  Scope s(h, "rates");
  rs::launch_rates(h->lc, h->T.p, h->P.p, h->krates.p);
  CK(cudaGetLastError());
  h->rates_dirty = false;
}

// Run the adaptive loop whose controller sits in ctl slot `slot` until it raises done.
// Attempts are queued in growing batches; every attempt kernel is a no-op once done is set,
// so only the batch boundary needs a host check of the pinned flag.
template <class Attempt>
void run_adaptive(rs_handle* h, int slot, Attempt attempt) {
  Ctl* dctl = h->ctl.p + slot;
  int batch = 1;
  double launched = 0;
  for (;;) {
    for (int b = 0; b < batch; ++b) attempt(dctl);
    launched += batch;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&h->hctl[slot], dctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (h->hctl[slot].done) break;
    if (launched > h->cfg.maxiters + 8) break;  // safety: the device loop is capped by maxiters
    if (!h->prof.on) batch = std::min(batch * 2, 64);
  }
}

void transport_attempt(rs_handle* h, Ctl* c) {
  rs::TransportBufs B{h->U[0].p, h->U[1].p, h->S1.p, h->S2.p, h->S3.p, h->partial.p};
  {
    Scope s(h, "ssprk43_stages");
    rs::launch_ssprk43_attempt(h->st, h->dt, c, B, h->cfg.rtol_T, h->cfg.atol_T,
                               h->cfg.clamp_nonneg);
  }
  Scope s(h, "finalize");
  rs::launch_finalize(h->st, c, h->partial.p, (int)((h->nc + 255) / 256));
  if (h->rec_on) rs::launch_tape_store(h->st, c, h->U[0].p, h->U[1].p, h->nc * h->nsp);
  h->launches += h->cfg.precision == RS_PREC_MIXED ? 18 : 17;
}

void chem_attempt(rs_handle* h, Ctl* c) {
  {
    Scope s(h, "ros23_attempt");
    rs::launch_ros23_attempt(h->lc, c, h->U[0].p, h->U[1].p, h->krates.p,
                             h->have_emis ? h->emis.p : nullptr, h->partial.p, h->cfg.rtol_C,
                             h->cfg.atol_C, h->cfg.clamp_nonneg, h->fsal[0].p, h->fsal[1].p);
  }
  Scope s(h, "finalize");
  rs::launch_finalize(h->st, c, h->partial.p, (int)((h->nc + 255) / 256));
  if (h->rec_on) rs::launch_tape_store(h->st, c, h->U[0].p, h->U[1].p, h->nc * h->nsp);
  h->launches += 2;
}

void drop_graph(rs_handle::LoopGraph& L) {
  if (L.ex) cudaGraphExecDestroy(L.ex);
  if (L.g) cudaGraphDestroy(L.g);
  L.ex = nullptr;
  L.g = nullptr;
  L.valid = false;
}

void invalidate_graphs(rs_handle* h) {
  for (auto& L : h->loops) L.valid = false;
}

// Build the device loop of one half: WHILE(cond) { attempt kernels; finalize + set cond }.
void build_loop_graph(rs_handle* h, int slot) {
  auto& L = h->loops[slot];
  drop_graph(L);
  if (!h->cap) CK(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking));
  CK(cudaGraphCreate(&L.g, 0));
  cudaGraphConditionalHandle cond;
  CK(cudaGraphConditionalHandleCreate(&cond, L.g, 1, cudaGraphCondAssignDefault));
  // cudaGraphNodeParams has no default constructor (a union of non-trivial members):
  // zero-initialised raw storage, then the conditional member
  alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
  std::memset(raw, 0, sizeof(raw));
  cudaGraphNodeParams* np = reinterpret_cast<cudaGraphNodeParams*>(raw);
  np->type = cudaGraphNodeTypeConditional;
  np->conditional.handle = cond;
  np->conditional.type = cudaGraphCondTypeWhile;
  np->conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, L.g, nullptr, nullptr, 0, np));
  cudaGraph_t body = np->conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(h->cap, body, nullptr, nullptr, 0,
                                   cudaStreamCaptureModeRelaxed));
  Ctl* c = h->ctl.p + slot;
  int nparts = (int)((h->nc + 255) / 256);
  if (slot == 0) {
    rs::TransportBufs B{h->U[0].p, h->U[1].p, h->S1.p, h->S2.p, h->S3.p, h->partial.p};
    rs::launch_ssprk43_attempt(h->cap, h->dt, c, B, h->cfg.rtol_T, h->cfg.atol_T,
                               h->cfg.clamp_nonneg);
  } else {
    rs::LaunchCtx lc = h->lc;
    lc.stream = h->cap;
    rs::launch_ros23_attempt(lc, c, h->U[0].p, h->U[1].p, h->krates.p,
                             h->have_emis ? h->emis.p : nullptr, h->partial.p, h->cfg.rtol_C,
                             h->cfg.atol_C, h->cfg.clamp_nonneg, h->fsal[0].p, h->fsal[1].p);
  }
  rs::launch_finalize_graph(h->cap, c, h->partial.p, nparts, cond);
  // while recording, the tape kernels follow the controller (no-ops for a controller without
  // a tape: a macro step the arena has no room for)
  if (h->rec_on) rs::launch_tape_store(h->cap, c, h->U[0].p, h->U[1].p, h->nc * h->nsp);
  L.with_tape = h->rec_on;
  cudaGraph_t captured = nullptr;
  CK(cudaStreamEndCapture(h->cap, &captured));
  CK(cudaGraphInstantiate(&L.ex, L.g, 0));
  L.valid = true;
}

// Run one adaptive solve of half `slot` as a single graph launch; the host reads the
// controller once at the end.
void run_adaptive_graph(rs_handle* h, int slot) {
  auto& L = h->loops[slot];
  if (!L.valid || L.with_tape != h->rec_on) build_loop_graph(h, slot);
  CK(cudaGraphLaunch(L.ex, h->st));
  CK(cudaMemcpyAsync(&h->hctl[slot], h->ctl.p + slot, sizeof(Ctl), cudaMemcpyDeviceToHost,
                     h->st));
  CK(cudaStreamSynchronize(h->st));
  h->launches += h->hctl[slot].iters *
                 (slot == 0 ? (h->cfg.precision == RS_PREC_MIXED ? 18 : 17) : 2);
}

rs_status guard(rs_handle* h, const std::function<void()>& fn);

}  // namespace

// ====================================================================== C ABI
extern "C" {

void rs_default_config(rs_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->api_version = RS_API_VERSION;
  c->has_air_mass = 1;
  c->do_transport = 1;
  c->do_chemistry = 1;
  c->rtol_T = 1e-4; c->atol_T = 1e-6;
  c->rtol_C = 1e-4; c->atol_C = 1e-9;
  c->ctrl_T = {7.0 / 30.0, 2.0 / 15.0, 1.0 / 5.0, 10.0, 9.0 / 10.0, 1.0, 1.0, 1e-4};
  c->ctrl_C = {7.0 / 20.0, 1.0 / 5.0, 1.0 / 5.0, 10.0, 9.0 / 10.0, 1.0, 6.0 / 5.0, 1e-4};
  c->maxiters = 2.0e4;
  c->clamp_nonneg = 1;
  c->precision = RS_PREC_FP64;
  c->chem_mode = RS_CHEM_GLOBAL_DT;
  c->grid.lon_bc = RS_BC_PERIODIC;
  c->grid.lat_bc = RS_BC_CLOSED;
}

}  // extern "C"

namespace {
rs_status guard(rs_handle* h, const std::function<void()>& fn) {
  try {
    fn();
    return RS_OK;
  } catch (const RsError& e) {
    set_err(h, e.what());
    return e.code;
  } catch (const std::exception& e) {
    set_err(h, e.what());
    return RS_ERR_INVALID;
  } catch (...) {
    set_err(h, "unknown error");
    return RS_ERR_INVALID;
  }
}
thread_local std::string g_create_err;
// Device address of the allocation-free attempt's scratch array on a device (defined with it
// at the end of this file); rs_create resolves it for its device.
void* noalloc_scratch(int dev);
}  // namespace

extern "C" {

rs_status rs_create(const rs_config* cfg, rs_handle** out) {
  if (!cfg || !out) return RS_ERR_INVALID;
  *out = nullptr;
  rs_handle* h = new rs_handle();
  rs_status st = guard(h, [&] {
    if (cfg->api_version != RS_API_VERSION) throw RsError(RS_ERR_INVALID, "api_version mismatch");
    h->cfg = *cfg;
    const rs_grid& g = cfg->grid;
    if (g.nlon < 1 || g.nlat < 1 || g.nlev < 1) throw RsError(RS_ERR_INVALID, "grid size");
    if (cfg->do_transport) {
      if (!cfg->has_air_mass) throw RsError(RS_ERR_INVALID, "transport needs the air-mass species");
      if (g.nlat < 3 || g.nlev < 3 || g.nlon < 3)
        throw RsError(RS_ERR_INVALID, "transport needs nlon, nlat, nlev >= 3");
      if (cfg->precision != RS_PREC_FP64 && cfg->precision != RS_PREC_MIXED)
        throw RsError(RS_ERR_INVALID, "precision");
      // the compensated FP32 pencils keep a whole lon row / 16 lat or vertical pencils in
      // shared memory
      if (cfg->precision == RS_PREC_MIXED &&
          (rs::mixed_pencil_bytes(g.nlon, 1, false) > rs::mixed_pencil_cap() ||
           rs::mixed_pencil_bytes(g.nlat, 16, false) > rs::mixed_pencil_cap() ||
           rs::mixed_pencil_bytes(g.nlev, 16, false) > rs::mixed_pencil_cap()))
        throw RsError(RS_ERR_UNSUPPORTED,
                      "mixed precision needs lon rows and 16-wide lat / vertical pencils that fit "
                      "in shared memory (nlon <= 6365, nlat and nlev <= 391)");
    }
    if (cfg->maxiters < 1) throw RsError(RS_ERR_INVALID, "maxiters");
    CK(cudaSetDevice(cfg->device));
    // Resolve the scratch array of rs_ros23_attempt_noalloc on this device now: with lazy
    // module loading the first lookup loads the module that holds the array (allocating and
    // possibly synchronising), which must not happen inside the allocation-free call.
    h->noalloc_base = noalloc_scratch(cfg->device);
    CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    h->mt = derive_tables(cfg->mech, RS_STRICT != 0);
    auto& T = h->mt;
    int cls = -1;
    if (T.ns <= rs::kSmallMS && T.nr <= rs::kSmallMR && T.nlu <= rs::kSmallMLU &&
        T.npart <= rs::kSmallMP)
      cls = 0;
    else if (T.ns <= rs::kLargeMS && T.nr <= rs::kLargeMR && T.nlu <= rs::kLargeMLU &&
             T.npart <= rs::kLargeMP)
      cls = 1;
    if (cls < 0) throw RsError(RS_ERR_UNSUPPORTED, "mechanism exceeds the kernel capacities");
    h->nlon = g.nlon; h->nlat = g.nlat; h->nlev = g.nlev;
    h->nc = (size_t)g.nlon * g.nlat * g.nlev;
    if (h->nc > (size_t)0x7fffffff) throw RsError(RS_ERR_INVALID, "too many cells");
    h->nsp = T.ns + (cfg->has_air_mass ? 1 : 0);
    h->ntr = T.ns;
    build_device_mech(h);
    h->lc = rs::LaunchCtx{h->st, h->dm, (int)h->nc, h->nsp, cls};
    h->jit = rs::jit_chem_build(h->mt, h->dm.ros_d, h->dm.ros_c32, RS_STRICT != 0, &h->jit_why);
    h->lc.jit = h->jit.get();
    if (h->jit && cfg->do_chemistry && cfg->chem_mode == RS_CHEM_GLOBAL_DT) {
      h->fsal[0].alloc((size_t)T.ns * h->nc);
      h->fsal[1].alloc((size_t)T.ns * h->nc);
    }
    size_t n = h->nc * h->nsp;
    h->U[0].alloc(n); h->U[1].alloc(n);
    h->U[0].zero(h->st); h->U[1].zero(h->st);
    h->partial.alloc((h->nc + 255) / 256 + 1);
    h->krates.alloc(std::max<size_t>(1, (size_t)T.nr * h->nc));
    h->krates.zero(h->st);
    h->ctl.alloc(3);
    h->ctl.zero(h->st);
    h->flag.alloc(1);
    h->queue.alloc(1);
    CK(cudaMallocHost(&h->hctl, 3 * sizeof(Ctl)));
    CK(cudaMallocHost(&h->hflag, sizeof(int)));
    if (cfg->chem_mode == RS_CHEM_PER_CELL) {
      h->dtcell.alloc(h->nc);
      h->dtcell.zero(h->st);
      h->stepcell.alloc(h->nc);
    }
    if (cfg->do_transport) {
      h->S1.alloc(n); h->S2.alloc(n); h->S3.alloc(n);
      h->fx.alloc((size_t)h->ntr * g.nlev * g.nlat * (g.nlon + 1));
      h->fy.alloc((size_t)h->ntr * g.nlev * (g.nlat + 1) * g.nlon);
      h->fz.alloc((size_t)h->ntr * (g.nlev + 1) * g.nlat * g.nlon);
      h->mx.alloc((size_t)g.nlev * g.nlat * (g.nlon + 1)); h->mx.zero(h->st);
      h->my.alloc((size_t)g.nlev * (g.nlat + 1) * g.nlon); h->my.zero(h->st);
      h->mz.alloc((size_t)(g.nlev + 1) * g.nlat * g.nlon); h->mz.zero(h->st);
      h->qw.alloc((size_t)h->ntr * g.nlev * g.nlat); h->qw.zero(h->st);
      h->qe.alloc((size_t)h->ntr * g.nlev * g.nlat); h->qe.zero(h->st);
      h->qs.alloc((size_t)h->ntr * g.nlev * g.nlon); h->qs.zero(h->st);
      h->qn.alloc((size_t)h->ntr * g.nlev * g.nlon); h->qn.zero(h->st);
      if (cfg->precision == RS_PREC_MIXED) {
        h->qhi.alloc((size_t)h->ntr * h->nc);
        h->qlo.alloc((size_t)h->ntr * h->nc);
      }
      h->tma_err.alloc(1);
      h->tma_err.zero(h->st);
      build_geometry(h);
      h->dp_host.assign(h->nc, 1.0);
      build_vertical(h);
    }
    if (cfg->do_transport && cfg->precision == RS_PREC_MIXED) make_flux_pairs(h);  // zero fluxes
    refresh_dt(h);
    if (cfg->do_transport && cfg->precision == RS_PREC_MIXED) {
      const char* why = nullptr;
      h->tmaps = rs::mixed_tmaps_create(h->dt, &why);
      if (!h->tmaps) h->tmaps_why = why ? why : "";
      refresh_dt(h);
    }
    CK(cudaStreamSynchronize(h->st));
  });
  if (st != RS_OK) {
    g_create_err = h->err;
    rs_destroy(h);
    return st;
  }
  *out = h;
  return RS_OK;
}

void rs_destroy(rs_handle* h) {
  if (!h) return;
  if (h->st) cudaStreamSynchronize(h->st);
  for (auto& L : h->loops) drop_graph(L);
  if (h->cap) cudaStreamDestroy(h->cap);
  for (auto& b : h->itabs) b.release();
  for (auto& b : h->dtabs) b.release();
  DevBuf<float>* fbufs[] = {&h->qhi, &h->qlo, &h->gx2, &h->gylo2, &h->gyhi2, &h->vsA2,
                            &h->vsB2, &h->veAB2, &h->veC2, &h->veD2, &h->mx2, &h->my2, &h->mz2};
  for (auto* b : fbufs) b->release();
  DevBuf<double>* bufs[] = {&h->U[0], &h->U[1], &h->S1, &h->S2, &h->S3, &h->fx, &h->fy, &h->fz,
                            &h->partial, &h->krates, &h->T, &h->P, &h->emis, &h->io, &h->io2,
                            &h->mx, &h->my, &h->mz, &h->qw, &h->qe, &h->qs, &h->qn, &h->gx,
                            &h->gylo, &h->gyhi, &h->vsA, &h->vsB, &h->veAB, &h->veC, &h->veD,
                            &h->dtcell, &h->stepcell, &h->totals, &h->fsal[0], &h->fsal[1],
                            &h->pbl_f, &h->pbl_w, &h->pbl_den, &h->pbl_qbar, &h->mcorr};
  for (auto* b : bufs) b->release();
  h->slot_row.release();
  h->slot_col.release();
  for (auto& r : h->recs) r.ck.release();
  for (auto& b : h->ck_pool) b.release();
  DevBuf<double>* abufs[] = {&h->seqbuf, &h->lam, &h->lam2, &h->ebar, &h->tape, &h->adj, &h->G,
                             &h->Cf, &h->tape_arena, &h->kz_arena, &h->kzs, &h->f_arena,
                             &h->fs};
  for (auto* b : abufs) b->release();
  h->nseq.release();
  h->ntape.release();
  h->tma_err.release();
  rs::mixed_tmaps_destroy(h->tmaps);
  h->ctl.release();
  h->flag.release();
  h->queue.release();
  if (h->hctl) cudaFreeHost(h->hctl);
  if (h->hflag) cudaFreeHost(h->hflag);
  for (auto& p : h->prof.pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : h->prof.pool) cudaEventDestroy(e);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
}

const char* rs_last_error(const rs_handle* h) {
  return h ? h->err.c_str() : g_create_err.c_str();
}

size_t rs_state_size(const rs_handle* h) { return h ? h->nc * h->nsp : 0; }
int32_t rs_species_per_cell(const rs_handle* h) { return h ? h->nsp : 0; }
void* rs_stream(rs_handle* h) { return h ? (void*)h->st : nullptr; }

rs_status rs_set_state(rs_handle* h, const double* u, size_t n) {
  if (!h || !u) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != h->nc * h->nsp) throw RsError(RS_ERR_INVALID, "state size mismatch");
    Scope s(h, "h2d_state");
    h->io.upload(u, n, h->st);
    rs::launch_to_soa(h->st, h->io.p, h->U[h->cur].p, h->nlon, h->nlat, h->nlev, h->nsp);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
  });
}

rs_status rs_get_state(rs_handle* h, double* u, size_t n) {
  if (!h || !u) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != h->nc * h->nsp) throw RsError(RS_ERR_INVALID, "state size mismatch");
    Scope s(h, "d2h_state");
    h->io.alloc(n);
    rs::launch_to_cellmajor(h->st, h->U[h->cur].p, h->io.p, h->nlon, h->nlat, h->nlev, h->nsp);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(u, h->io.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  });
}

rs_status rs_state_device_ptr(rs_handle* h, void** d) {
  if (!h || !d) return RS_ERR_INVALID;
  *d = h->U[h->cur].p;
  return RS_OK;
}

rs_status rs_set_forcing(rs_handle* h, const rs_forcing* f) {
  if (!h || !f) return RS_ERR_INVALID;
  return guard(h, [&] {
    const rs_grid& g = h->cfg.grid;
    cudaStream_t st = h->st;
    size_t nc = h->nc;
    if (h->cfg.do_transport) {
      if (f->mx) {
        h->mx.upload(f->mx, (size_t)g.nlev * g.nlat * (g.nlon + 1), st);
        h->mx_host.assign(f->mx, f->mx + (size_t)g.nlev * g.nlat * (g.nlon + 1));
      }
      if (f->my) {
        h->my.upload(f->my, (size_t)g.nlev * (g.nlat + 1) * g.nlon, st);
        h->my_host.assign(f->my, f->my + (size_t)g.nlev * (g.nlat + 1) * g.nlon);
      }
      if (f->mz) h->mz.upload(f->mz, (size_t)(g.nlev + 1) * g.nlat * g.nlon, st);
      if (f->qbc_w) h->qw.upload(f->qbc_w, (size_t)h->ntr * g.nlev * g.nlat, st);
      if (f->qbc_e) h->qe.upload(f->qbc_e, (size_t)h->ntr * g.nlev * g.nlat, st);
      if (f->qbc_s) h->qs.upload(f->qbc_s, (size_t)h->ntr * g.nlev * g.nlon, st);
      if (f->qbc_n) h->qn.upload(f->qbc_n, (size_t)h->ntr * g.nlev * g.nlon, st);
      if (f->dp) {
        for (size_t c = 0; c < nc; ++c)
          if (!(f->dp[c] > 0.0)) throw RsError(RS_ERR_INVALID, "dp must be positive");
        h->dp_host.assign(f->dp, f->dp + nc);
        build_vertical(h);
      }
      if (f->mx || f->my || f->mz) h->omega = f->flux_omega;
      const size_t ncol = (size_t)g.nlon * g.nlat;
      bool pbl_inputs = f->dp != nullptr || f->temperature != nullptr;
      if (f->pblh) {
        if (!(f->tau_pblmix >= 0.0)) throw RsError(RS_ERR_INVALID, "tau_pblmix must be >= 0");
        h->pblh_host.assign(f->pblh, f->pblh + ncol);
        h->tau_pbl = f->tau_pblmix;
        pbl_inputs = true;
      }
      if (f->ps) {
        for (size_t c = 0; c < ncol; ++c)
          if (!(f->ps[c] > 0.0)) throw RsError(RS_ERR_INVALID, "ps must be positive");
        h->ps_host.assign(f->ps, f->ps + ncol);
        pbl_inputs = true;
      }
      if (f->hyb_a) { h->hyb_a_host.assign(f->hyb_a, f->hyb_a + g.nlev + 1); pbl_inputs = true; }
      if (f->hyb_b) { h->hyb_b_host.assign(f->hyb_b, f->hyb_b + g.nlev + 1); pbl_inputs = true; }
      if (f->temperature) h->tsfc_host.assign(f->temperature, f->temperature + ncol);
      if (pbl_inputs) build_pbl(h);
      if (f->dps_dt) h->dpsdt_host.assign(f->dps_dt, f->dps_dt + ncol);
      if (f->dps_dt || f->hyb_b || f->mx || f->my || f->mz || f->dp) build_fixer(h);
      if (h->cfg.precision == RS_PREC_MIXED) make_flux_pairs(h);
    }
    if (f->temperature) {
      h->T.upload(f->temperature, nc, st);
      h->rates_dirty = true;
      h->rates_override = false;
    }
    if (f->pressure) {
      h->P.upload(f->pressure, nc, st);
      h->rates_dirty = true;
      h->rates_override = false;
    }
    if (f->emission) {
      h->emis.upload(f->emission, (size_t)h->mt.ns * nc, st);
      h->have_emis = true;
    }
    h->have_forcing = true;
    refresh_dt(h);
    invalidate_graphs(h);
    CK(cudaStreamSynchronize(st));
  });
}

rs_status rs_get_rate_constants(rs_handle* h, double* k, size_t n) {
  if (!h || !k) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != (size_t)h->mt.nr * h->nc) throw RsError(RS_ERR_INVALID, "rate array size");
    ensure_rates(h);
    CK(cudaMemcpyAsync(k, h->krates.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  });
}

rs_status rs_get_cell_steps(rs_handle* h, double* steps, double* dt, size_t n) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != h->nc) throw RsError(RS_ERR_INVALID, "cell array size");
    if (h->cfg.chem_mode != RS_CHEM_PER_CELL)
      throw RsError(RS_ERR_UNSUPPORTED, "per-cell step counts exist in the per-cell mode only");
    if (steps) CK(cudaMemcpyAsync(steps, h->stepcell.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    if (dt) CK(cudaMemcpyAsync(dt, h->dtcell.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  });
}

rs_status rs_set_rate_constants(rs_handle* h, const double* k, size_t n) {
  if (!h || !k) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != (size_t)h->mt.nr * h->nc) throw RsError(RS_ERR_INVALID, "rate array size");
    h->krates.upload(k, n, h->st);
    h->rates_dirty = false;
    h->rates_override = true;
    invalidate_graphs(h);
    CK(cudaStreamSynchronize(h->st));
  });
}

#ifndef RS_BOUNDS_CHECK
#define RS_BOUNDS_CHECK 0
#endif
// A mixed pencil kernel whose bulk-copy wait ran out sets bit 1 of tma_err and stops the
// solve; in the bounds-check build a pencil kernel whose index check failed sets bit 2.
static void check_staging(rs_handle* h) {
  if (!h->tma_err.p) return;
  int e = 0;
  CK(cudaMemcpyAsync(h->hflag, h->tma_err.p, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  e = *h->hflag;
  if (e) {
    CK(cudaMemsetAsync(h->tma_err.p, 0, sizeof(int), h->st));
    if (e & 2)
      throw RsError(RS_ERR_INVALID, "a transport kernel's index check failed (bounds-check build)");
    throw RsError(RS_ERR_CUDA, "a transport pencil's bulk-copy wait timed out; solve stopped");
  }
}

rs_status rs_macro_step(rs_handle* h, double t0, double t1, double* dtT, double* dtC,
                        rs_stats* out) {
  if (!h || !dtT || !dtC) return RS_ERR_INVALID;
  rs_stats stats{};
  rs_status rc = guard(h, [&] {
    if (!(t1 > t0)) throw RsError(RS_ERR_INVALID, "t1 must exceed t0");
    if (!(*dtT > 0.0) || !(*dtC > 0.0)) throw RsError(RS_ERR_INVALID, "dt must be positive");
    h->launches = 0;
    if (h->rates_dirty && !h->rates_override) h->launches += 1;
    ensure_rates(h);
    double ntot = (double)h->nc * h->nsp;
    bool okT = true, okC = true;
    stats.dtT_end = *dtT;
    stats.dtC_end = *dtC;
    stats.tT_end = t1;
    stats.tC_end = t1;
    const int seqcap = (int)std::min(h->cfg.maxiters + 1.0, 1.0e6);
    if (h->rec_on) {
      if (h->cfg.chem_mode != RS_CHEM_GLOBAL_DT)
        throw RsError(RS_ERR_UNSUPPORTED, "the adjoint records global-dt chemistry only");
      h->recs.emplace_back();
      auto& r = h->recs.back();
      r.t0 = t0;
      r.t1 = t1;
      size_t n = h->nc * h->nsp;
      if (!h->ck_pool.empty()) {
        r.ck = h->ck_pool.back();
        h->ck_pool.pop_back();
      }
      r.ck.alloc(n);
      CK(cudaMemcpyAsync(r.ck.p, h->U[h->cur].p, n * sizeof(double), cudaMemcpyDeviceToDevice,
                         h->st));
      h->seqbuf.alloc((size_t)4 * seqcap);
      h->nseq.alloc(2);
      CK(cudaMemsetAsync(h->nseq.p, 0, 2 * sizeof(int), h->st));
      r.tape_off = h->tape_used;
      r.tape_cap = h->tape_limit > h->tape_used ? (h->tape_limit - h->tape_used) / n : 0;
      const size_t nkz = (size_t)2 * h->mt.ns * h->nc;
      r.kz_off = h->kz_used;
      r.kz_cap = h->kz_limit > h->kz_used ? (h->kz_limit - h->kz_used) / nkz : 0;
      r.f_off = h->f_used;
      r.f_cap = h->f_limit > h->f_used ? (h->f_limit - h->f_used) / (7 * n) : 0;
      h->ntape.alloc(4);
      CK(cudaMemsetAsync(h->ntape.p, 0, 4 * sizeof(int), h->st));
    }
    // device-tape slots for the half about to run: its steps' inputs from slot `first` on
    // (the transport half's steps come first), one slot kept for the macro step's end state
    auto tape_half = [&](Ctl& init, size_t first, int half) {
      if (!h->rec_on) return;
      const auto& r = h->recs.back();
      const size_t n = h->nc * h->nsp;
      if (r.tape_cap < first + 2) return;
      init.tape = h->tape_arena.p + r.tape_off + first * n;
      init.ntape = h->ntape.p + 2 * half;
      init.tapecap = (int)std::min<size_t>(r.tape_cap - 1 - first, 1u << 30);
    };
    if (h->cfg.do_transport) {
      Ctl init = make_ctl(h, t0, t1, *dtT, h->cfg.ctrl_T, ntot);
      init.cur = h->cur;
      if (h->rec_on) {
        init.seq = h->seqbuf.p;
        init.nseq = h->nseq.p;
        init.seqcap = seqcap;
      }
      tape_half(init, 0, 0);
      if (h->rec_on && transport_stage_tape(h) && h->recs.back().f_cap > 0) {
        init.ftape = h->f_arena.p + h->recs.back().f_off;
        init.fcap = (int)std::min<size_t>(h->recs.back().f_cap, 1u << 30);
        h->recs.back().f_set = true;
      }
      rs::launch_ctl_init(h->st, h->ctl.p + 0, init);
      h->launches += 1;
      if (h->use_graphs && !h->prof.on) run_adaptive_graph(h, 0);
      else run_adaptive(h, 0, [&](Ctl* c) { transport_attempt(h, c); });
      const Ctl& c = h->hctl[0];
      h->cur = c.cur;
      stats.naT = c.nacc; stats.nrT = c.nrej; stats.dtT_end = c.dt; stats.tT_end = c.t;
      okT = c.t >= t1 - 1e-9;
      *dtT = c.dt;
    }
    if (h->cfg.do_chemistry && okT) {
      if (h->cfg.chem_mode == RS_CHEM_GLOBAL_DT) {
        Ctl init = make_ctl(h, t0, t1, *dtC, h->cfg.ctrl_C, ntot);
        init.cur = h->cur;
        if (h->rec_on) {
          init.seq = h->seqbuf.p + (size_t)2 * seqcap;
          init.nseq = h->nseq.p + 1;
          init.seqcap = seqcap;
        }
        tape_half(init, h->cfg.do_transport ? (size_t)stats.naT : 0, 1);
        if (h->rec_on && h->lc.jit && h->recs.back().kz_cap > 0) {  // the stage tape
          init.kz = h->kz_arena.p + h->recs.back().kz_off;
          init.kzcap = (int)std::min<size_t>(h->recs.back().kz_cap, 1u << 30);
        }
        rs::launch_ctl_init(h->st, h->ctl.p + 1, init);
        h->launches += 1;
        if (h->use_graphs && !h->prof.on) run_adaptive_graph(h, 1);
        else run_adaptive(h, 1, [&](Ctl* c) { chem_attempt(h, c); });
        const Ctl& c = h->hctl[1];
        h->cur = c.cur;
        stats.naC = c.nacc; stats.nrC = c.nrej; stats.dtC_end = c.dt; stats.tC_end = c.t;
        okC = c.t >= t1 - 1e-9;
        *dtC = c.dt;
      } else {
        const rs_controller& c = h->cfg.ctrl_C;
        h->totals.alloc(2);
        h->totals.zero(h->st);
        rs::PerCellArgs a{t0, t1, *dtC, h->cfg.rtol_C, h->cfg.atol_C, h->cfg.maxiters,
                          c.beta1, c.beta2, 1.0 / c.qmin, 1.0 / c.qmax, c.gamma,
                          c.qsteady_min, c.qsteady_max, c.qoldinit, h->cfg.clamp_nonneg,
                          h->totals.p};
        CK(cudaMemsetAsync(h->queue.p, 0, sizeof(unsigned long long), h->st));
        CK(cudaMemsetAsync(h->flag.p, 0, sizeof(int), h->st));
        int dev = 0, nsm = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        int thr = h->tune.pc_threads;
        int nblocks = std::max(1, std::min(nsm * h->tune.pc_blocks_per_sm,
                                           (int)((h->nc + thr - 1) / thr)));
        const int G = h->lc.jit ? 0 : h->tune.pc_group;
        if (G > 0) {  // a persistent grid of resident blocks, one cell per G lanes
          thr = rs::chem_group_threads(h->lc, G);
          const int bps = rs::chem_group_blocks_per_sm(h->lc, G, thr);
          if (thr == 0 || bps == 0) throw RsError(RS_ERR_UNSUPPORTED, "per-cell group kernel does not fit");
          nblocks = std::max(1, std::min(nsm * bps, (int)((h->nc + thr / G - 1) / (thr / G))));
        }
        {
          Scope s(h, "chem_per_cell");
          if (G > 0)
            rs::launch_chem_per_cell_group(h->lc, G, nblocks, thr, h->U[h->cur].p, h->krates.p,
                                           h->have_emis ? h->emis.p : nullptr, h->dtcell.p,
                                           h->stepcell.p, h->queue.p, h->flag.p, a);
          else
            rs::launch_chem_per_cell(h->lc, nblocks, thr, h->U[h->cur].p, h->krates.p,
                                     h->have_emis ? h->emis.p : nullptr, h->dtcell.p,
                                     h->stepcell.p, h->queue.p, h->flag.p, a,
                                     h->tune.pc_regcap != 0);
        }
        h->launches += 1;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h->hflag, h->flag.p, sizeof(int), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        okC = *h->hflag == 0;
        double tot[2] = {0, 0};
        CK(cudaMemcpy(tot, h->totals.p, sizeof(tot), cudaMemcpyDeviceToHost));
        stats.chem_cell_steps = tot[0];
        stats.naC = tot[0];                 // per-cell mode: cell-steps, summed over cells
        stats.nrC = tot[1] - tot[0];
      }
    }
    collect_profile(h);
    if (h->rec_on) {
      int ns_h[2] = {0, 0};
      CK(cudaMemcpyAsync(ns_h, h->nseq.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      auto& r = h->recs.back();
      if (ns_h[0] > seqcap || ns_h[1] > seqcap) throw RsError(RS_ERR_INVALID, "step record overflow");
      r.seqT.resize((size_t)2 * ns_h[0]);
      r.seqC.resize((size_t)2 * ns_h[1]);
      if (ns_h[0])
        CK(cudaMemcpy(r.seqT.data(), h->seqbuf.p, r.seqT.size() * sizeof(double),
                      cudaMemcpyDeviceToHost));
      if (ns_h[1])
        CK(cudaMemcpy(r.seqC.data(), h->seqbuf.p + (size_t)2 * seqcap,
                      r.seqC.size() * sizeof(double), cudaMemcpyDeviceToHost));
      // the tape is complete when both halves stored every accepted step's input (a half
      // that did not run stored none); the end state closes it
      int nt[4] = {0, 0, 0, 0};
      CK(cudaMemcpy(nt, h->ntape.p, sizeof(nt), cudaMemcpyDeviceToHost));
      const size_t n = h->nc * h->nsp, used = (size_t)ns_h[0] + ns_h[1] + 1;
      // with the specialised kernels the chemistry stages must be complete too, so that every
      // step VJP reads its k1, z2 from a forward pass (the tape's or the replay's)
      const bool need_kz = h->lc.jit && ns_h[1] > 0;
      const bool need_f = r.f_set && ns_h[0] > 0;
      r.tape_ok = h->tape_limit > 0 && nt[1] == 0 && nt[3] == 0 && nt[0] == ns_h[0] &&
                  nt[2] == ns_h[1] && used <= r.tape_cap &&
                  (ns_h[0] == 0 || h->cfg.do_transport) && (ns_h[1] == 0 || h->cfg.do_chemistry) &&
                  (!need_kz || (size_t)ns_h[1] <= r.kz_cap) &&
                  (!need_f || (size_t)ns_h[0] <= r.f_cap);
      if (r.tape_ok) {
        CK(cudaMemcpyAsync(h->tape_arena.p + r.tape_off + (used - 1) * n, h->U[h->cur].p,
                           n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
        h->tape_used += used * n;
        if (need_kz) h->kz_used += (size_t)ns_h[1] * 2 * h->mt.ns * h->nc;
        r.kz_ok = need_kz;
        if (need_f) h->f_used += (size_t)ns_h[0] * 7 * n;
        r.f_ok = need_f;
      }
    }
    if (!okT || !okC) {
      check_staging(h);
      throw RsError(RS_ERR_MAXITERS, "adaptive solve stopped before t1 (maxiters)");
    }
    CK(cudaMemsetAsync(h->flag.p, 0, sizeof(int), h->st));
    rs::launch_nonfinite(h->st, h->U[h->cur].p, h->nc * h->nsp, h->flag.p);
    h->launches += 1;
    CK(cudaMemcpyAsync(h->hflag, h->flag.p, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (*h->hflag) throw RsError(RS_ERR_NONFINITE, "non-finite state after the macro step");
    if (RS_BOUNDS_CHECK) check_staging(h);
  });
  stats.status = rc;
  stats.kernel_launches = h->launches;
  if (out) *out = stats;
  return rc;
}

rs_status rs_rhs_transport(rs_handle* h, double t, const double* u, double* du, size_t n) {
  if (!h || !u || !du) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (!h->cfg.do_transport) throw RsError(RS_ERR_STATE, "transport disabled");
    if (n != h->nc * h->nsp) throw RsError(RS_ERR_INVALID, "state size mismatch");
    h->io.upload(u, n, h->st);
    h->io2.alloc(n);
    rs::launch_to_soa(h->st, h->io.p, h->S1.p, h->nlon, h->nlat, h->nlev, h->nsp);
    double g = h->omega != 0.0 ? std::cos(h->omega * t) : 1.0;
    rs::launch_transport_rhs(h->st, h->dt, h->S1.p, g, h->S2.p);
    rs::launch_to_cellmajor(h->st, h->S2.p, h->io2.p, h->nlon, h->nlat, h->nlev, h->nsp);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(du, h->io2.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (h->tmaps || RS_BOUNDS_CHECK) check_staging(h);
  });
}

rs_status rs_rhs_chem(rs_handle* h, double t, const double* u, double* du, size_t n) {
  (void)t;
  if (!h || !u || !du) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != h->nc * h->nsp) throw RsError(RS_ERR_INVALID, "state size mismatch");
    ensure_rates(h);
    h->io.upload(u, n, h->st);
    h->io2.alloc(2 * n);
    double* soa = h->io2.p;
    double* dsoa = h->io2.p + n;
    rs::launch_to_soa(h->st, h->io.p, soa, h->nlon, h->nlat, h->nlev, h->nsp);
    rs::launch_chem_rhs(h->lc, soa, h->krates.p, h->have_emis ? h->emis.p : nullptr, dsoa);
    rs::launch_to_cellmajor(h->st, dsoa, h->io.p, h->nlon, h->nlat, h->nlev, h->nsp);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(du, h->io.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  });
}

rs_status rs_block_jac(rs_handle* h, const double* u, double* J, size_t n_jac) {
  if (!h || !u || !J) return RS_ERR_INVALID;
  return guard(h, [&] {
    size_t n = h->nc * h->nsp;
    if (n_jac != h->nc * h->nsp * h->nsp) throw RsError(RS_ERR_INVALID, "jacobian size");
    ensure_rates(h);
    h->io.upload(u, n, h->st);
    h->io2.alloc(n + n_jac);
    double* soa = h->io2.p;
    double* dJ = h->io2.p + n;
    rs::launch_to_soa(h->st, h->io.p, soa, h->nlon, h->nlat, h->nlev, h->nsp);
    rs::launch_block_jac(h->lc, soa, h->krates.p, h->slot_row.p, h->slot_col.p, dJ);
    CK(cudaGetLastError());
    // device J is [grid cell][r][s]; reorder to the cell-major cell index on the host
    std::vector<double> tmp(n_jac);
    CK(cudaMemcpyAsync(tmp.data(), dJ, n_jac * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    size_t bs = (size_t)h->nsp * h->nsp;
    for (int k = 0; k < h->nlev; ++k)
      for (int j = 0; j < h->nlat; ++j)
        for (int i = 0; i < h->nlon; ++i) {
          size_t gcell = ((size_t)k * h->nlat + j) * h->nlon + i;
          size_t ccell = ((size_t)i * h->nlat + j) * h->nlev + k;
          std::memcpy(J + ccell * bs, tmp.data() + gcell * bs, bs * sizeof(double));
        }
  });
}

rs_status rs_single_step(rs_handle* h, int32_t op, double t, double dt, const double* u_in,
                         double* u_out, double* eest, size_t n) {
  if (!h || !u_in || !u_out) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != h->nc * h->nsp) throw RsError(RS_ERR_INVALID, "state size mismatch");
    if (!(dt > 0.0)) throw RsError(RS_ERR_INVALID, "dt must be positive");
    if (op == RS_OP_TRANSPORT && !h->cfg.do_transport) throw RsError(RS_ERR_STATE, "transport disabled");
    if (op != RS_OP_TRANSPORT && op != RS_OP_CHEMISTRY) throw RsError(RS_ERR_INVALID, "op");
    ensure_rates(h);
    const rs_controller& cc = op == RS_OP_TRANSPORT ? h->cfg.ctrl_T : h->cfg.ctrl_C;
    Ctl init = make_ctl(h, t, t + dt, dt, cc, (double)n);
    init.cur = 0;
    init.maxiters = 1.0;
    h->io.upload(u_in, n, h->st);
    h->io2.alloc(2 * n);
    double* a = h->io2.p;
    double* b = h->io2.p + n;
    rs::launch_to_soa(h->st, h->io.p, a, h->nlon, h->nlat, h->nlev, h->nsp);
    rs::launch_ctl_init(h->st, h->ctl.p + 2, init);
    Ctl* c = h->ctl.p + 2;
    if (op == RS_OP_TRANSPORT) {
      rs::TransportBufs B{a, b, h->S1.p, h->S2.p, h->S3.p, h->partial.p};
      rs::launch_ssprk43_attempt(h->st, h->dt, c, B, h->cfg.rtol_T, h->cfg.atol_T, 0);
    } else {
      rs::launch_ros23_attempt(h->lc, c, a, b, h->krates.p, h->have_emis ? h->emis.p : nullptr,
                               h->partial.p, h->cfg.rtol_C, h->cfg.atol_C, 0);
    }
    rs::launch_finalize(h->st, c, h->partial.p, (int)((h->nc + 255) / 256));
    rs::launch_to_cellmajor(h->st, b, h->io.p, h->nlon, h->nlat, h->nlev, h->nsp);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(u_out, h->io.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaMemcpyAsync(&h->hctl[2], c, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (eest) *eest = h->hctl[2].eest;
  });
}

rs_status rs_set_profiling(rs_handle* h, int32_t on) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    collect_profile(h);
    h->prof.on = on != 0;
  });
}

rs_status rs_reset_profile(rs_handle* h) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    collect_profile(h);
    std::fill(h->prof.launches.begin(), h->prof.launches.end(), 0.0);
    std::fill(h->prof.ms.begin(), h->prof.ms.end(), 0.0);
  });
}

rs_status rs_get_profile(rs_handle* h, char* buf, size_t buf_len, double* launches,
                         double* total_ms, int32_t max_kernels, int32_t* n_out) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    collect_profile(h);
    auto& P = h->prof;
    std::string names;
    int n = std::min<int>((int)P.names.size(), max_kernels);
    for (int i = 0; i < n; ++i) {
      if (i) names += ";";
      names += P.names[i];
      if (launches) launches[i] = P.launches[i];
      if (total_ms) total_ms[i] = P.ms[i];
    }
    if (buf && buf_len) {
      std::strncpy(buf, names.c_str(), buf_len - 1);
      buf[buf_len - 1] = 0;
    }
    if (n_out) *n_out = n;
  });
}

}  // extern "C"

// ====================================================================== discrete adjoint
namespace {

// SSPRK43 step VJP at fixed (t, dt): recompute the stage states, then walk the stages back
// (the transpose of rx_traced_integrator.jl:404-437).  Buffers: adj = 11 state-sized slabs.
// rec (optional): the step's transport stage record from the forward or the replay --
// F0..F3 and V1, V2, V4, [7][n] -- in place of recomputing the stages here
void transport_step_vjp(rs_handle* h, const double* u, double t, double dt, const double* lam,
                        double* out, const double* rec = nullptr) {
  size_t n = h->nc * h->nsp;
  double* V1 = h->adj.p + 0 * n;
  double* V2 = h->adj.p + 1 * n;
  double* V4 = h->adj.p + 2 * n;
  double* F0 = h->adj.p + 3 * n;
  double* F1 = h->adj.p + 4 * n;
  double* F2 = h->adj.p + 5 * n;
  double* F3 = h->adj.p + 6 * n;
  double* A = h->adj.p + 7 * n;
  double* B = h->adj.p + 8 * n;
  double* Wb = h->adj.p + 9 * n;
  // the air-mass derivative of the VJP takes the advective tendency alone (PBL mixing does not
  // depend on the air mass): with PBL mixing it is kept in four more slabs
  double* Fa[4] = {F0, F1, F2, F3};
  if (h->pbl_on)
    for (int q = 0; q < 4; ++q) Fa[q] = h->adj.p + (11 + q) * n;
  rs::DevTransport<double> T = h->dt;
  T.mixed = 0;  // the adjoint differentiates the FP64 scheme
  auto gf = [&](double tt) { return h->omega != 0.0 ? std::cos(h->omega * tt) : 1.0; };
  double h2 = dt / 2;
  cudaStream_t st = h->st;
  const double* Fr[4] = {Fa[0], Fa[1], Fa[2], Fa[3]};
  const double* Vr[3] = {V1, V2, V4};
  if (rec) {
    for (int q = 0; q < 4; ++q) Fr[q] = rec + (size_t)q * n;
    for (int q = 0; q < 3; ++q) Vr[q] = rec + (size_t)(4 + q) * n;
  } else {
    rs::launch_transport_rhs(st, T, u, gf(t), F0, h->pbl_on ? Fa[0] : nullptr);
    rs::launch_lincomb(st, n, V1, 1.0, u, h2, F0, 0.0, nullptr);
    rs::launch_transport_rhs(st, T, V1, gf(t + 0.5 * dt), F1, h->pbl_on ? Fa[1] : nullptr);
    rs::launch_lincomb(st, n, V2, 1.0, V1, h2, F1, 0.0, nullptr);
    rs::launch_transport_rhs(st, T, V2, gf(t + 1.0 * dt), F2, h->pbl_on ? Fa[2] : nullptr);
    rs::launch_lincomb(st, n, V4, 1.0, V2, h2, F2, 0.0, nullptr);        // u3
    rs::launch_lincomb(st, n, V4, 2.0 / 3.0, u, 1.0 / 3.0, V4, 0.0, nullptr);  // u4
    rs::launch_transport_rhs(st, T, V4, gf(t + h2), F3, h->pbl_on ? Fa[3] : nullptr);
  }
  auto vjp = [&](const double* Us, const double* Fs, double g, const double* fbar, double* ub) {
    rs::launch_transport_rhs_vjp(st, T, Us, Fs, fbar, ub, h->G.p, h->Cf.p, g);
  };
  rs::launch_lincomb(st, n, Wb, h2, lam, 0.0, nullptr, 0.0, nullptr);
  vjp(Vr[2], Fr[3], gf(t + h2), Wb, A);
  rs::launch_lincomb(st, n, A, 1.0, A, 1.0, lam, 0.0, nullptr);           // ubar4
  rs::launch_lincomb(st, n, out, 2.0 / 3.0, A, 0.0, nullptr, 0.0, nullptr);
  rs::launch_lincomb(st, n, B, 1.0 / 3.0, A, 0.0, nullptr, 0.0, nullptr);  // ubar3 = ubar2
  rs::launch_lincomb(st, n, Wb, h2, B, 0.0, nullptr, 0.0, nullptr);
  vjp(Vr[1], Fr[2], gf(t + 1.0 * dt), Wb, A);
  rs::launch_lincomb(st, n, B, 1.0, B, 1.0, A, 0.0, nullptr);             // ubar2 -> ubar1
  rs::launch_lincomb(st, n, Wb, h2, B, 0.0, nullptr, 0.0, nullptr);
  vjp(Vr[0], Fr[1], gf(t + 0.5 * dt), Wb, A);
  rs::launch_lincomb(st, n, B, 1.0, B, 1.0, A, 0.0, nullptr);             // ubar1 -> ubar0
  rs::launch_lincomb(st, n, Wb, h2, B, 0.0, nullptr, 0.0, nullptr);
  vjp(u, Fr[0], gf(t), Wb, A);
  rs::launch_lincomb(st, n, out, 1.0, out, 1.0, B, 1.0, A);
}

void ensure_adjoint_buffers(rs_handle* h) {
  size_t n = h->nc * h->nsp;
  h->lam.alloc(n);
  h->lam2.alloc(n);
  if (!h->ebar.p) {
    h->ebar.alloc((size_t)h->mt.ns * h->nc);
    h->ebar.zero(h->st);
  }
  if (h->cfg.do_transport) {
    h->adj.alloc((h->pbl_on ? 15 : 11) * n);  // + 4 advection-only tendencies with PBL mixing
    h->G.alloc((size_t)h->ntr * h->nc);
    const rs_grid& g = h->cfg.grid;
    size_t fx = (size_t)(g.nlon + 1) * g.nlat * g.nlev, fy = (size_t)g.nlon * (g.nlat + 1) * g.nlev,
           fz = (size_t)g.nlon * g.nlat * (g.nlev + 1);
    h->Cf.alloc((size_t)h->ntr * std::max(fx, std::max(fy, fz)) * 5);
  }
}

}  // namespace

extern "C" {

rs_status rs_record(rs_handle* h, int32_t on) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (on) {
      if (h->cfg.chem_mode != RS_CHEM_GLOBAL_DT)
        throw RsError(RS_ERR_UNSUPPORTED, "the adjoint records global-dt chemistry only");
      for (auto& r : h->recs) {
        h->ck_pool.push_back(r.ck);
        r.ck.p = nullptr;
        r.ck.n = 0;
      }
      h->recs.clear();
      // the device tape's arena, reserved here so that recorded macro steps allocate nothing
      size_t want = 0;
      if (h->tape_budget < 0) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        want = (fr + (h->tape_arena.n + h->kz_arena.n + h->f_arena.n) * sizeof(double)) / 4;
      } else {
        want = (size_t)h->tape_budget;
      }
      // states, chemistry stages and transport stages share the budget in fixed proportions:
      // their sizes per step, weighted for six chemistry steps per transport step (states:
      // one per step, 7 per transport step; the chemistry stages only with the specialised
      // kernels, the only ones that write them; the transport stages only for the FP64
      // scheme without PBL mixing).  A macro step that overruns any of them is replayed.
      const double ws = 7.0 * h->nsp;
      const double wk = (h->lc.jit && h->cfg.do_chemistry) ? 12.0 * h->mt.ns : 0.0;
      const double wf = transport_stage_tape(h) ? 7.0 * h->nsp : 0.0;
      const size_t want_kz = (size_t)((double)want * wk / (ws + wk + wf));
      const size_t want_f = (size_t)((double)want * wf / (ws + wk + wf));
      h->tape_limit = (want - want_kz - want_f) / sizeof(double);
      h->kz_limit = want_kz / sizeof(double);
      h->f_limit = want_f / sizeof(double);
      if (h->f_limit > h->f_arena.n) {
        h->f_arena.release();
        h->f_arena.alloc(h->f_limit);
      }
      if (h->tape_limit > h->tape_arena.n) {
        h->tape_arena.release();
        h->tape_arena.alloc(h->tape_limit);
      }
      if (h->kz_limit > h->kz_arena.n) {
        h->kz_arena.release();
        h->kz_arena.alloc(h->kz_limit);
      }
      h->tape_used = 0;
      h->kz_used = 0;
      h->f_used = 0;
    }
    h->rec_on = on != 0;
    // the device loops with the tape kernels, built now rather than in the first recorded
    // macro step
    if (h->rec_on && h->use_graphs) {
      if (h->cfg.do_transport) build_loop_graph(h, 0);
      if (h->cfg.do_chemistry && h->cfg.chem_mode == RS_CHEM_GLOBAL_DT) build_loop_graph(h, 1);
    }
  });
}

int32_t rs_record_count(const rs_handle* h) { return h ? (int32_t)h->recs.size() : 0; }

rs_status rs_set_adjoint_tape(rs_handle* h, int64_t budget_bytes) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (budget_bytes < -1) throw RsError(RS_ERR_INVALID, "tape budget must be >= -1");
    h->tape_budget = budget_bytes;
  });
}

int32_t rs_record_taped(const rs_handle* h) {
  if (!h) return 0;
  int32_t k = 0;
  for (const auto& r : h->recs) k += r.tape_ok ? 1 : 0;
  return k;
}

rs_status rs_adjoint_set_lambda(rs_handle* h, const double* lam, size_t n) {
  if (!h || !lam) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != h->nc * h->nsp) throw RsError(RS_ERR_INVALID, "state size mismatch");
    ensure_adjoint_buffers(h);
    h->io.upload(lam, n, h->st);
    rs::launch_to_soa(h->st, h->io.p, h->lam.p, h->nlon, h->nlat, h->nlev, h->nsp);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
  });
}

rs_status rs_adjoint_get_lambda(rs_handle* h, double* lam, size_t n) {
  if (!h || !lam) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != h->nc * h->nsp) throw RsError(RS_ERR_INVALID, "state size mismatch");
    if (!h->lam.p) throw RsError(RS_ERR_STATE, "no adjoint state (rs_adjoint_set_lambda first)");
    h->io.alloc(n);
    rs::launch_to_cellmajor(h->st, h->lam.p, h->io.p, h->nlon, h->nlat, h->nlev, h->nsp);
    CK(cudaMemcpyAsync(lam, h->io.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  });
}

rs_status rs_adjoint_get_grad_emission(rs_handle* h, double* g, size_t n) {
  if (!h || !g) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n != (size_t)h->mt.ns * h->nc) throw RsError(RS_ERR_INVALID, "gradient size mismatch");
    ensure_adjoint_buffers(h);
    CK(cudaMemcpyAsync(g, h->ebar.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  });
}

rs_status rs_adjoint_reset_grad(rs_handle* h) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    ensure_adjoint_buffers(h);
    h->ebar.zero(h->st);
    CK(cudaStreamSynchronize(h->st));
  });
}

// Frozen-dt replay of recorded macro step k on the RESIDENT state (replay_fixed,
// tools/adjoint_gradient.jl:647-669): the recorded accepted (t, dt) of both halves, each step
// accepted whatever its error, clamp as in the forward, with the forcing installed now.  The
// composed map of these replays is the map the discrete adjoint differentiates; the reference
// checks its gradient against central differences of it (the fdtape stage,
// adjoint_gradient.jl:116-132).
rs_status rs_replay_macro_step(rs_handle* h, int32_t k) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (k < 0 || k >= (int)h->recs.size()) throw RsError(RS_ERR_INVALID, "no such recorded step");
    if (h->cfg.precision != RS_PREC_FP64 || h->cfg.chem_mode != RS_CHEM_GLOBAL_DT)
      throw RsError(RS_ERR_UNSUPPORTED, "the replay is of the FP64 global-dt scheme");
    ensure_rates(h);
    const auto& r = h->recs[k];
    const int nT = (int)(r.seqT.size() / 2), nC = (int)(r.seqC.size() / 2);
    cudaStream_t st = h->st;
    const int clamp = h->cfg.clamp_nonneg;
    Ctl* c = h->ctl.p + 2;
    const double ntot = (double)(h->nc * h->nsp);
    int cur = h->cur;
    for (int j = 0; j < nT + nC; ++j) {
      const bool tr = j < nT;
      const double tj = tr ? r.seqT[2 * j] : r.seqC[2 * (j - nT)];
      const double dj = tr ? r.seqT[2 * j + 1] : r.seqC[2 * (j - nT) + 1];
      // tend well past t + dt so that dtc = min(dt, tend - t) is the recorded dt exactly
      Ctl init = make_ctl(h, tj, tj + 4.0 * dj + 1.0, dj, tr ? h->cfg.ctrl_T : h->cfg.ctrl_C, ntot);
      init.cur = cur;
      rs::launch_ctl_init(st, c, init);
      if (tr) {
        rs::TransportBufs B{h->U[0].p, h->U[1].p, h->S1.p, h->S2.p, h->S3.p, h->partial.p};
        rs::launch_ssprk43_attempt(st, h->dt, c, B, h->cfg.rtol_T, h->cfg.atol_T, clamp);
      } else {
        rs::launch_ros23_step(h->lc, c, h->U[0].p, h->U[1].p, h->krates.p,
                              h->have_emis ? h->emis.p : nullptr, h->partial.p,
                              h->cfg.rtol_C, h->cfg.atol_C, clamp);
      }
      rs::launch_replay_accept(st, c);
      cur ^= 1;
    }
    h->cur = cur;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
  });
}

rs_status rs_backward_macro_step(rs_handle* h, int32_t k) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (k < 0 || k >= (int)h->recs.size()) throw RsError(RS_ERR_INVALID, "no such recorded step");
    if (!h->lam.p) throw RsError(RS_ERR_STATE, "no adjoint state (rs_adjoint_set_lambda first)");
    ensure_adjoint_buffers(h);
    ensure_rates(h);
    const auto& r = h->recs[k];
    size_t n = h->nc * h->nsp;
    int nT = (int)(r.seqT.size() / 2), nC = (int)(r.seqC.size() / 2);
    cudaStream_t st = h->st;
    const int clamp = h->cfg.clamp_nonneg;
    double* tape = nullptr;
    double* fin = nullptr;
    // k1, z2 of every chemistry step (specialised kernels): the forward's stage tape, or the
    // replay's scratch; the step VJPs read them instead of recomputing both stages
    const size_t nkz = (size_t)2 * h->mt.ns * h->nc;
    const bool use_kz = h->lc.jit != nullptr && nC > 0;
    double* kzb = nullptr;
    // F0..F3, V1, V2, V4 of every transport step: the forward's stage tape, or the replay's
    const bool use_f = transport_stage_tape(h) && nT > 0;
    double* fb = nullptr;
    if (r.tape_ok) {  // the forward stored every step's input and the end state
      tape = h->tape_arena.p + r.tape_off;
      fin = tape + (size_t)(nT + nC) * n;
      if (use_kz && r.kz_ok) kzb = h->kz_arena.p + r.kz_off;
      if (use_f && r.f_ok) fb = h->f_arena.p + r.f_off;
    } else {
    if (use_kz) {
      size_t mostC = 0;
      for (const auto& q : h->recs) mostC = std::max(mostC, q.seqC.size() / 2);
      h->kzs.alloc(mostC * nkz);
      kzb = h->kzs.p;
    }
    if (use_f) {
      size_t mostT = 0;
      for (const auto& q : h->recs) mostT = std::max(mostT, q.seqT.size() / 2);
      h->fs.alloc(mostT * 7 * n);
      fb = h->fs.p;
    }
    // one tape for the largest recorded macro step (no reallocation during a sweep)
    size_t most = 0;
    for (const auto& q : h->recs) most = std::max(most, (q.seqT.size() + q.seqC.size()) / 2);
    h->tape.alloc((most + 2) * n);
    tape = h->tape.p;
    double* R[2] = {tape + (size_t)(nT + nC) * n, tape + (size_t)(nT + nC + 1) * n};
    // ---- fixed-sequence replay from the checkpoint, keeping every step's input
    int cur = 0;
    {
    Scope sc_replay(h, "adj_replay");
    CK(cudaMemcpyAsync(R[0], r.ck.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    Ctl* c = h->ctl.p + 2;
    double ntot = (double)n;
    for (int j = 0; j < nT + nC; ++j) {
      bool tr = j < nT;
      double tj = tr ? r.seqT[2 * j] : r.seqC[2 * (j - nT)];
      double dj = tr ? r.seqT[2 * j + 1] : r.seqC[2 * (j - nT) + 1];
      CK(cudaMemcpyAsync(tape + (size_t)j * n, R[cur], n * sizeof(double),
                         cudaMemcpyDeviceToDevice, st));
      // tend well past t + dt so that dtc = min(dt, tend - t) is the recorded dt exactly
      Ctl init = make_ctl(h, tj, tj + 4.0 * dj + 1.0, dj, tr ? h->cfg.ctrl_T : h->cfg.ctrl_C, ntot);
      init.cur = cur;
      if (!tr && kzb) {  // the step writes its k1, z2 to its own slot (accepted count 0)
        init.kz = kzb + (size_t)(j - nT) * nkz;
        init.kzcap = 1;
      }
      if (tr && fb) {  // the step writes its stage record to its own slot
        init.ftape = fb + (size_t)j * 7 * n;
        init.fcap = 1;
      }
      rs::launch_ctl_init(st, c, init);
      if (tr) {
        rs::TransportBufs B{R[0], R[1], h->S1.p, h->S2.p, h->S3.p, h->partial.p};
        rs::launch_ssprk43_attempt(st, h->dt, c, B, h->cfg.rtol_T, h->cfg.atol_T, clamp);
      } else {
        rs::launch_ros23_step(h->lc, c, R[0], R[1], h->krates.p,
                              h->have_emis ? h->emis.p : nullptr, h->partial.p,
                              h->cfg.rtol_C, h->cfg.atol_C, clamp);
      }
      rs::launch_replay_accept(st, c);
      cur ^= 1;
    }
    }
    // the final replayed state closes the tape (output of the last step)
    fin = R[cur];
    }
    auto out_of = [&](int j) -> const double* {
      return (j + 1 < nT + nC) ? tape + (size_t)(j + 1) * n : fin;
    };
    // ---- chemistry steps in reverse, then transport steps in reverse
    { Scope sc_vjp(h, "adj_chem_vjp");
    for (int j = nC - 1; j >= 0; --j) {
      int jj = nT + j;
      rs::launch_ros23_vjp(h->lc, tape + (size_t)jj * n, clamp ? out_of(jj) : nullptr, h->lam.p,
                           h->lam2.p, h->krates.p, h->have_emis ? h->emis.p : nullptr,
                           h->ebar.p, r.seqC[2 * j + 1], clamp,
                           kzb ? kzb + (size_t)j * nkz : nullptr);
      std::swap(h->lam.p, h->lam2.p);
    }
    }
    Scope sc_tvjp(h, "adj_transport_vjp");
    for (int j = nT - 1; j >= 0; --j) {
      if (clamp) rs::launch_clamp_mask(st, n, h->lam.p, out_of(j));
      transport_step_vjp(h, tape + (size_t)j * n, r.seqT[2 * j], r.seqT[2 * j + 1], h->lam.p,
                         h->lam2.p, fb ? fb + (size_t)j * 7 * n : nullptr);
      std::swap(h->lam.p, h->lam2.p);
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
  });
}

}  // extern "C"

// ====================================================================== chemistry kernel kind
extern "C" rs_status rs_set_chem_kernel(rs_handle* h, int32_t kind) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (kind != RS_CHEM_KERNEL_AUTO && kind != RS_CHEM_KERNEL_TABLE &&
        kind != RS_CHEM_KERNEL_SPECIALIZED)
      throw RsError(RS_ERR_INVALID, "unknown chemistry kernel kind");
    if (kind == RS_CHEM_KERNEL_SPECIALIZED && !h->jit)
      throw RsError(RS_ERR_UNSUPPORTED, "specialised chemistry kernels unavailable: " + h->jit_why);
    h->chem_kernel = kind;
    h->lc.jit = (kind == RS_CHEM_KERNEL_TABLE) ? nullptr : h->jit.get();
    invalidate_graphs(h);
  });
}

extern "C" rs_status rs_get_chem_kernel(rs_handle* h, int32_t* kind, char* info, size_t info_len) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    const bool spec = h->lc.jit != nullptr;
    if (kind) *kind = spec ? RS_CHEM_KERNEL_SPECIALIZED : RS_CHEM_KERNEL_TABLE;
    if (info && info_len) {
      std::string why = h->jit_why;
      for (char& ch : why)
        if (ch == '"' || ch == '\\' || ch == '\n') ch = ' ';
      char line[768];
      if (h->jit)
        std::snprintf(line, sizeof line,
                      "{\"kind\": \"%s\", \"variant\": \"%s\", \"regs\": [%d, %d, %d, %d], "
                      "\"smem_bytes\": %zu, \"split_smem_bytes\": %zu, \"compile_ms\": %.1f}",
                      spec ? "specialized" : "table", rs::kJitVariantNames[h->jit->variant],
                      h->jit->regs[0], h->jit->regs[1], h->jit->regs[2], h->jit->regs[3],
                      h->jit->attempt_smem[1], h->jit->attempt_smem[3], h->jit->compile_ms);
      else
        std::snprintf(line, sizeof line, "{\"kind\": \"table\", \"why\": \"%.600s\"}", why.c_str());
      std::strncpy(info, line, info_len - 1);
      info[info_len - 1] = 0;
    }
  });
}

// ====================================================================== launch shapes
extern "C" rs_status rs_set_launch_shape(rs_handle* h, const char* key, int32_t value) {
  if (!h || !key) return RS_ERR_INVALID;
  return guard(h, [&] {
    const std::string k(key);
    auto in = [&](std::initializer_list<int> c) {
      for (int v : c)
        if (v == value) return true;
      return false;
    };
    auto& t = h->tune;
    const int ntr = std::max(1, h->dt.ntr);
    bool ok = true;
    if (k == "xthreads") ok = in({64, 96, 128, 160, 192, 224, 256}) && (t.xthreads = value, true);
    else if (k == "pencil") ok = in({8, 16, 32}) && (t.pencil = value, true);
    else if (k == "rows") ok = in({4, 8, 16, 32}) && (t.rows = value, true);
    else if (k == "x_tracer_groups") ok = value >= 1 && value <= ntr && (t.xgroups = value, true);
    else if (k == "yz_tracer_groups") ok = value >= 1 && value <= ntr && (t.yzgroups = value, true);
    else if (k == "mixed_xthreads") ok = in({64, 128, 256}) && (t.mxthreads = value, true);
    else if (k == "mixed_x_tracers") ok = value >= 1 && value <= ntr && (t.msper_x = value, true);
    else if (k == "mixed_pencil") ok = in({16, 32}) && (t.mpencil = value, true);
    else if (k == "mixed_rows") ok = in({4, 8, 16}) && (t.mrows = value, true);
    else if (k == "mixed_yz_tracers") ok = value >= 1 && value <= ntr && (t.msper_yz = value, true);
    else if (k == "mixed_x_bulk") ok = in({0, 1}) && (t.mbulk_x = value, true);
    else if (k == "mixed_yz_bulk") ok = in({0, 1}) && (t.mbulk_yz = value, true);
    else if (k == "mixed_x_stream") ok = in({0, 1}) && (t.mstream_x = value, true);
    else if (k == "mixed_yz_stream") ok = in({0, 1}) && (t.mstream_yz = value, true);
    else if (k == "per_cell_threads") ok = in({64, 128, 256}) && (t.pc_threads = value, true);
    else if (k == "per_cell_blocks_per_sm") ok = in({1, 2, 4, 8, 16}) && (t.pc_blocks_per_sm = value, true);
    else if (k == "per_cell_regcap") ok = in({0, 1}) && (t.pc_regcap = value, true);
    else if (k == "chem_attempt_variant") {  // the specialised attempt kernel's variant
      ok = value >= 0 && value < rs::kJitVariants && h->jit && h->jit->attempt[value][0];
      if (ok) h->jit->variant = value;
    }
    else if (k == "per_cell_group") {
      // G lanes per cell: the production build's (minimum-fill, descending back substitution)
      // table-walking kernels only, and only where a block of them fits in shared memory
      ok = in({0, 4, 8, 16}) && (value == 0 || (!RS_STRICT && rs::chem_group_threads(h->lc, value) > 0));
      if (ok) t.pc_group = value;
    }
    else throw RsError(RS_ERR_INVALID, "unknown launch-shape key: " + k);
    if (!ok) throw RsError(RS_ERR_INVALID, "value out of range for " + k);
    refresh_dt(h);
    invalidate_graphs(h);
  });
}

// ====================================================================== transport staging
extern "C" rs_status rs_set_transport_staging(rs_handle* h, int32_t mode) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (mode != RS_STAGING_AUTO && mode != RS_STAGING_PLAIN && mode != RS_STAGING_BULK)
      throw RsError(RS_ERR_INVALID, "unknown staging mode");
    if (mode == RS_STAGING_BULK && !h->tmaps)
      throw RsError(RS_ERR_UNSUPPORTED,
                    "bulk-copy staging unavailable: " +
                        (h->tmaps_why.empty() ? std::string("mixed-precision transport only")
                                              : h->tmaps_why));
    h->staging = mode;
    refresh_dt(h);
    invalidate_graphs(h);
  });
}

extern "C" rs_status rs_get_transport_staging(rs_handle* h, int32_t* mode, char* info,
                                              size_t info_len) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    const bool bulk = h->tmaps && h->staging != RS_STAGING_PLAIN &&
                      (h->staging == RS_STAGING_BULK || h->tune.mbulk_x || h->tune.mbulk_yz);
    if (mode) *mode = bulk ? RS_STAGING_BULK : RS_STAGING_PLAIN;
    if (info && info_len) {
      char line[256];
      const rs::DevTransport<double>& T = h->dt;
      auto use = [&](int d) {
        if (!rs::mixed_tmaps_dir_ok(h->tmaps, d)) return "unavailable";
        return (T.tma && (d == 0 ? T.mbulk_x : T.mbulk_yz)) ? "bulk" : "plain";
      };
      if (h->tmaps)
        std::snprintf(line, sizeof line,
                      "{\"mode\": \"%s\", \"lon_rows\": \"%s\", \"lat_pencils\": \"%s\", "
                      "\"vertical_pencils\": \"%s\"}",
                      bulk ? "bulk" : "plain", use(0), use(1), use(2));
      else
        std::snprintf(line, sizeof line, "{\"mode\": \"plain\", \"why\": \"%.180s\"}",
                      h->tmaps_why.c_str());
      std::strncpy(info, line, info_len - 1);
      info[info_len - 1] = 0;
    }
  });
}

extern "C" rs_status rs_chem_kernel_reciprocal(rs_handle* h, const double* x, double* r,
                                               size_t n) {
  if (!h || (n && (!x || !r))) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (!h->jit) throw RsError(RS_ERR_UNSUPPORTED, "no specialised kernels: " + h->jit_why);
    if (n > (size_t)0x7fffffff) throw RsError(RS_ERR_INVALID, "n");
    if (!n) return;
    h->io.alloc(2 * n);
    CK(cudaMemcpyAsync(h->io.p, x, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
    rs::jit_launch_rcp(*h->jit, h->st, h->io.p, h->io.p + n, (int)n);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(r, h->io.p + n, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  });
}

extern "C" rs_status rs_lu_order(rs_handle* h, int32_t* ord, int32_t n) {
  if (!h || !ord) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (n < h->mt.ns) throw RsError(RS_ERR_INVALID, "ord holds fewer entries than species");
    for (int k = 0; k < h->mt.ns; ++k) ord[k] = h->mt.ord[k];
  });
}

extern "C" rs_status rs_continuity_drift(rs_handle* h, const double* ps, double* out3) {
  if (!h || !ps || !out3) return RS_ERR_INVALID;
  return guard(h, [&] {
    const rs_grid& g = h->cfg.grid;
    if (!h->cfg.has_air_mass) throw RsError(RS_ERR_INVALID, "the state carries no air mass");
    if (h->hyb_a_host.size() != (size_t)g.nlev + 1 || h->hyb_b_host.size() != (size_t)g.nlev + 1)
      throw RsError(RS_ERR_STATE, "hybrid coefficients not given (rs_forcing hyb_a, hyb_b)");
    const size_t ncol = (size_t)g.nlon * g.nlat;
    std::vector<double> m(h->nc);
    CK(cudaMemcpyAsync(m.data(), h->U[h->cur].p + (size_t)(h->nsp - 1) * h->nc,
                       h->nc * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const double* A = h->hyb_a_host.data();
    const double* B = h->hyb_b_host.data();
    double s2i = 0.0, s2w = 0.0, worst = 0.0;
    size_t ni = 0, nw = 0;
    for (int k = 0; k < g.nlev; ++k)
      for (int j = 0; j < g.nlat; ++j)
        for (int i = 0; i < g.nlon; ++i) {
          const size_t col = (size_t)j * g.nlon + i;
          const double dpk = (A[k] - A[k + 1]) + (B[k] - B[k + 1]) * ps[col];
          const double r = (m[(size_t)k * ncol + col] - dpk) / dpk;
          if (i == 0 || i == g.nlon - 1 || j == 0 || j == g.nlat - 1) {
            s2w += r * r;
            ++nw;
          } else {
            s2i += r * r;
            ++ni;
            if (std::fabs(r) > std::fabs(worst)) worst = r;
          }
        }
    out3[0] = std::sqrt(s2i / (double)std::max<size_t>(ni, 1));
    out3[1] = std::sqrt(s2w / (double)std::max<size_t>(nw, 1));
    out3[2] = worst;
  });
}

// ====================================================================== window solve
namespace {

double round6(double t) { return std::round(t * 1.0e6) / 1.0e6; }

struct WindowSolve {
  rs_handle* h;
  const rs_solve_opts& o;
  rs_solve_result r{};
  std::vector<DevBuf<double>> ck;  // window start states, one per bisection depth

  // one window with the reference's stop grid; counts of a failed window are dropped
  rs_status plain(double t0, double tf, double macro_dt, double& dtT, double& dtC) {
    std::vector<double> stops;
    std::set<double> fstops;
    for (size_t q = 0; q < o.n_tstops; ++q) {
      const double t = o.forcing_tstops[q];
      if (t0 + 1e-6 < t && t <= tf + 1e-6) fstops.insert(round6(t));
    }
    for (long i = 1;; ++i) {
      const double x = t0 + macro_dt * (double)i;
      if (x > tf - 1e-9) break;
      stops.push_back(x);
    }
    for (double t : fstops) stops.push_back(t);
    stops.push_back(tf);
    std::sort(stops.begin(), stops.end());
    stops.erase(std::unique(stops.begin(), stops.end()), stops.end());
    rs_solve_result part{};
    double tcur = t0;
    for (double tnext : stops) {
      if (tnext <= tcur + 1e-9) continue;
      rs_stats st{};
      rs_status rc = rs_macro_step(h, tcur, tnext, &dtT, &dtC, &st);
      if (rc != RS_OK) return rc;
      part.naT += st.naT; part.nrT += st.nrT; part.naC += st.naC; part.nrC += st.nrC;
      part.nmacro += 1.0;
      tcur = tnext;
      if (fstops.count(round6(tcur))) {
        part.nrefresh += 1.0;
        if (o.refresh) o.refresh(o.user, tcur);
      }
    }
    r.naT += part.naT; r.nrT += part.nrT; r.naC += part.naC; r.nrC += part.nrC;
    r.nmacro += part.nmacro;
    r.nrefresh += part.nrefresh;
    return RS_OK;
  }

  rs_status bisect(double t0, double tf, double macro_dt, double& dtT, double& dtC, int depth) {
    const bool can_split = o.min_macro_dt > 0.0 && (tf - t0) > o.min_macro_dt + 1e-9;
    const size_t n = h->nc * h->nsp;
    if (can_split) {  // the window's start state, for a restart
      if ((int)ck.size() <= depth) ck.resize(depth + 1);
      ck[depth].alloc(n);
      CK(cudaMemcpyAsync(ck[depth].p, h->U[h->cur].p, n * sizeof(double),
                         cudaMemcpyDeviceToDevice, h->st));
    }
    const double dtT0 = dtT, dtC0 = dtC;
    rs_status rc = plain(t0, tf, macro_dt, dtT, dtC);
    if (rc == RS_OK || !can_split) return rc;
    CK(cudaMemcpyAsync(h->U[h->cur].p, ck[depth].p, n * sizeof(double),
                       cudaMemcpyDeviceToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    const double tm = 0.5 * (t0 + tf);
    r.nbisect += 1.0;
    if (o.on_bisect) o.on_bisect(o.user, t0, tf);
    dtT = dtT0;
    dtC = dtC0;
    rc = bisect(t0, tm, std::min(macro_dt, tm - t0), dtT, dtC, depth + 1);
    if (rc != RS_OK) return rc;
    return bisect(tm, tf, std::min(macro_dt, tf - tm), dtT, dtC, depth + 1);
  }
};

}  // namespace

extern "C" rs_status rs_lie_trotter_solve(rs_handle* h, double t0, double t1, double* dtT,
                                          double* dtC, const rs_solve_opts* opts,
                                          rs_solve_result* out) {
  if (!h || !dtT || !dtC || !opts) return RS_ERR_INVALID;
  WindowSolve ws{h, *opts};
  rs_status rc = guard(h, [&] {
    if (!(t1 > t0)) throw RsError(RS_ERR_INVALID, "t1 must exceed t0");
    if (!(opts->macro_dt > 0.0)) throw RsError(RS_ERR_INVALID, "macro_dt must be positive");
    if (opts->n_tstops && !opts->forcing_tstops) throw RsError(RS_ERR_INVALID, "forcing_tstops");
    rs_status w = ws.bisect(t0, t1, opts->macro_dt, *dtT, *dtC, 0);
    if (w != RS_OK) throw RsError(w, std::string("window failed: ") + h->err);
  });
  for (auto& b : ws.ck) b.release();
  ws.r.status = rc;
  if (out) *out = ws.r;
  return rc;
}

// Source and compile check of the specialised kernels for a mechanism (no device needed).
namespace {
rs_status nohandle(const std::function<void()>& fn) {
  try {
    fn();
    g_create_err.clear();
    return RS_OK;
  } catch (const RsError& e) {
    g_create_err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_create_err = e.what();
    return RS_ERR_INVALID;
  }
}
void copy_out(const std::string& s, char* buf, size_t len) {
  if (!buf || !len) return;
  size_t n = std::min(len - 1, s.size());
  std::memcpy(buf, s.data(), n);
  buf[n] = 0;
}
}  // namespace

extern "C" rs_status rs_chem_kernel_source(const rs_mechanism* mech, int32_t strict, char* buf,
                                           size_t buf_len, size_t* len_out) {
  if (!mech) return RS_ERR_INVALID;
  return nohandle([&] {
    MechTables T = derive_tables(*mech, strict != 0);
    if (!rs::jit_chem_eligible(T))
      throw RsError(RS_ERR_UNSUPPORTED, "mechanism too large for straight-line kernels");
    std::string src = rs::jit_chem_source(T, strict != 0);
    if (len_out) *len_out = src.size() + 1;
    copy_out(src, buf, buf_len);
  });
}

extern "C" rs_status rs_mechanism_lu_order(const rs_mechanism* mech, int32_t natural,
                                           int32_t* ord, int32_t n) {
  if (!mech || !ord) return RS_ERR_INVALID;
  return nohandle([&] {
    MechTables T = derive_tables(*mech, natural != 0);
    if (n < T.ns) throw RsError(RS_ERR_INVALID, "ord holds fewer entries than species");
    for (int k = 0; k < T.ns; ++k) ord[k] = T.ord[k];
  });
}

extern "C" rs_status rs_chem_kernel_compile(const rs_mechanism* mech, int32_t strict, char* log,
                                            size_t log_len) {
  if (!mech) return RS_ERR_INVALID;
  return nohandle([&] {
    MechTables T = derive_tables(*mech, strict != 0);
    if (!rs::jit_chem_eligible(T))
      throw RsError(RS_ERR_UNSUPPORTED, "mechanism too large for straight-line kernels");
    std::string text;
    bool ok = rs::jit_compile(rs::jit_chem_source(T, strict != 0), strict != 0, true, nullptr, &text);
    copy_out(text, log, log_len);
    if (!ok) throw RsError(RS_ERR_UNSUPPORTED, text.substr(0, 2000));
  });
}

// ====================================================================== autotuner
namespace {

template <class F>
float time_min(cudaStream_t st, int reps, F&& launch) {
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  float best = 1e30f;
  for (int r = 0; r < reps; ++r) {
    CK(cudaEventRecord(a, st));
    launch();
    CK(cudaEventRecord(b, st));
    CK(cudaEventSynchronize(b));
    CK(cudaGetLastError());
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, a, b));
    best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

}  // namespace

extern "C" rs_status rs_autotune(rs_handle* h, char* buf, size_t buf_len) {
  if (!h) return RS_ERR_INVALID;
  return guard(h, [&] {
    ensure_rates(h);
    std::string rep = "{";
    char line[256];
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    if (h->cfg.do_chemistry && h->cfg.chem_mode == RS_CHEM_PER_CELL) {
      // three attempts per cell on scratch copies: the state and the carried dts are untouched
      size_t n = h->nc * h->nsp;
      h->io2.alloc(n);
      h->io.alloc(h->nc);
      h->totals.alloc(2);
      const rs_controller& c = h->cfg.ctrl_C;
      rs::PerCellArgs a{0.0, 1.0e30, 1.0, h->cfg.rtol_C, h->cfg.atol_C, 3.0, c.beta1, c.beta2,
                        1.0 / c.qmin, 1.0 / c.qmax, c.gamma, c.qsteady_min, c.qsteady_max,
                        c.qoldinit, h->cfg.clamp_nonneg, nullptr};
      float best = 1e30f;
      rep += "\"per_cell\": [";
      bool first = true;
      for (int thr : {64, 128, 256})
        for (int bps : {1, 2, 4, 8}) {
          int nb = std::max(1, std::min(nsm * bps, (int)((h->nc + thr - 1) / thr)));
          float ms = time_min(h->st, 2, [&] {
            cudaMemcpyAsync(h->io2.p, h->U[h->cur].p, n * sizeof(double),
                            cudaMemcpyDeviceToDevice, h->st);
            cudaMemsetAsync(h->io.p, 0, h->nc * sizeof(double), h->st);
            cudaMemsetAsync(h->queue.p, 0, sizeof(unsigned long long), h->st);
            rs::launch_chem_per_cell(h->lc, nb, thr, h->io2.p, h->krates.p,
                                     h->have_emis ? h->emis.p : nullptr, h->io.p, nullptr,
                                     h->queue.p, h->flag.p, a);
          });
          std::snprintf(line, sizeof line, "%s{\"threads\": %d, \"blocks_per_sm\": %d, \"ms\": %.4f}",
                        first ? "" : ", ", thr, bps, ms);
          rep += line;
          first = false;
          if (ms < best) {
            best = ms;
            h->tune.pc_threads = thr;
            h->tune.pc_blocks_per_sm = bps;
            h->tune.pc_group = 0;
            h->tune.pc_regcap = 0;
          }
        }
      // the table-walking kernel capped at 32 registers, at full occupancy
      if (!h->lc.jit)
        for (int thr : {128, 256}) {
          const int bps = 2048 / thr;
          int nb = std::max(1, std::min(nsm * bps, (int)((h->nc + thr - 1) / thr)));
          float ms = time_min(h->st, 2, [&] {
            cudaMemcpyAsync(h->io2.p, h->U[h->cur].p, n * sizeof(double),
                            cudaMemcpyDeviceToDevice, h->st);
            cudaMemsetAsync(h->io.p, 0, h->nc * sizeof(double), h->st);
            cudaMemsetAsync(h->queue.p, 0, sizeof(unsigned long long), h->st);
            rs::launch_chem_per_cell(h->lc, nb, thr, h->io2.p, h->krates.p,
                                     h->have_emis ? h->emis.p : nullptr, h->io.p, nullptr,
                                     h->queue.p, h->flag.p, a, true);
          });
          std::snprintf(line, sizeof line,
                        ", {\"threads\": %d, \"blocks_per_sm\": %d, \"regcap\": 1, \"ms\": %.4f}",
                        thr, bps, ms);
          rep += line;
          if (ms < best) {
            best = ms;
            h->tune.pc_threads = thr;
            h->tune.pc_blocks_per_sm = bps;
            h->tune.pc_group = 0;
            h->tune.pc_regcap = 1;
          }
        }
      // G lanes per cell (table-walking kernels of the production build): every resident
      // block of the persistent grid
      if (!RS_STRICT && !h->lc.jit)
        for (int G : {4, 8, 16}) {
          const int thr = rs::chem_group_threads(h->lc, G);
          const int bps = thr ? rs::chem_group_blocks_per_sm(h->lc, G, thr) : 0;
          if (bps == 0) continue;
          const int cpb = thr / G;
          int nb = std::max(1, std::min(nsm * bps, (int)((h->nc + cpb - 1) / cpb)));
          float ms = time_min(h->st, 2, [&] {
            cudaMemcpyAsync(h->io2.p, h->U[h->cur].p, n * sizeof(double),
                            cudaMemcpyDeviceToDevice, h->st);
            cudaMemsetAsync(h->io.p, 0, h->nc * sizeof(double), h->st);
            cudaMemsetAsync(h->queue.p, 0, sizeof(unsigned long long), h->st);
            rs::launch_chem_per_cell_group(h->lc, G, nb, thr, h->io2.p, h->krates.p,
                                           h->have_emis ? h->emis.p : nullptr, h->io.p, nullptr,
                                           h->queue.p, h->flag.p, a);
          });
          std::snprintf(line, sizeof line,
                        ", {\"group\": %d, \"threads\": %d, \"blocks_per_sm\": %d, \"ms\": %.4f}",
                        G, thr, bps, ms);
          rep += line;
          if (ms < best) {
            best = ms;
            h->tune.pc_group = G;
            h->tune.pc_regcap = 0;
          }
        }
      std::snprintf(line, sizeof line,
                    "], \"per_cell_choice\": {\"threads\": %d, \"blocks_per_sm\": %d, \"group\": %d, "
                    "\"regcap\": %d}",
                    h->tune.pc_threads, h->tune.pc_blocks_per_sm, h->tune.pc_group, h->tune.pc_regcap);
      rep += line;
    }
    if (h->cfg.do_chemistry && h->cfg.chem_mode == RS_CHEM_GLOBAL_DT && h->lc.jit) {
      // variants of the specialised attempt kernel: one attempt from the accepted state into
      // the candidate buffer (the accepted state is untouched)
      Ctl init = make_ctl(h, 0.0, 600.0, 60.0, h->cfg.ctrl_C, (double)h->nc * h->nsp);
      init.cur = h->cur;
      Ctl* c = h->ctl.p + 2;
      rs::launch_ctl_init(h->st, c, init);
      float best = 1e30f;
      int pick = 0;
      bool first = true;
      rep += std::string(rep.size() > 1 ? ", " : "") + "\"chem_attempt\": [";
      for (int v = 0; v < rs::kJitVariants; ++v) {
        if (!h->jit->attempt[v][0]) continue;
        h->jit->variant = v;
        float ms = time_min(h->st, 3, [&] {
          rs::launch_ros23_attempt(h->lc, c, h->U[0].p, h->U[1].p, h->krates.p,
                                   h->have_emis ? h->emis.p : nullptr, h->partial.p,
                                   h->cfg.rtol_C, h->cfg.atol_C, h->cfg.clamp_nonneg);
        });
        std::snprintf(line, sizeof line, "%s{\"variant\": \"%s\", \"regs\": %d, \"ms\": %.4f}",
                      first ? "" : ", ", rs::kJitVariantNames[v], h->jit->regs[v], ms);
        rep += line;
        first = false;
        if (ms < best) {
          best = ms;
          pick = v;
        }
      }
      h->jit->variant = pick;
      std::snprintf(line, sizeof line, "], \"chem_choice\": \"%s\"", rs::kJitVariantNames[pick]);
      rep += line;
      invalidate_graphs(h);
    }
    if (h->cfg.do_transport) {
      const double* Q = h->U[h->cur].p;
      rs::DevTransport<double> T = h->dt;
      float bx = 1e30f;
      rep += std::string(rep.size() > 1 ? ", " : "") + "\"lon_rows\": [";
      bool first = true;
      // the row (n + 6 cells) in one pass of whole warps, and the fixed sizes around it
      const int fit = (h->nlon + 6 + 31) / 32 * 32;
      std::vector<int> xts{64, 128, 256};
      if (fit > 128 && fit < 256) xts.push_back(fit);
      for (int xt : xts) {
        T.xthreads = xt;
        float ms = time_min(h->st, 3, [&] { rs::launch_flux_dir(h->st, T, Q, 0); });
        std::snprintf(line, sizeof line, "%s{\"threads\": %d, \"ms\": %.4f}", first ? "" : ", ", xt, ms);
        rep += line;
        first = false;
        if (ms < bx) {
          bx = ms;
          h->tune.xthreads = xt;
        }
      }
      rep += "], \"pencils\": [";
      first = true;
      float byz = 1e30f;
      T.xthreads = h->tune.xthreads;
      for (int pw : {8, 16, 32})
        for (int rows : {4, 8, 16, 32}) {
          if (pw * rows < 64 || pw * rows > 512) continue;
          T.pencil = pw;
          T.rows = rows;
          float ms = time_min(h->st, 3, [&] {
            rs::launch_flux_dir(h->st, T, Q, 1);
            rs::launch_flux_dir(h->st, T, Q, 2);
          });
          std::snprintf(line, sizeof line, "%s{\"pencil\": %d, \"rows\": %d, \"ms\": %.4f}",
                        first ? "" : ", ", pw, rows, ms);
          rep += line;
          first = false;
          if (ms < byz) {
            byz = ms;
            h->tune.pencil = pw;
            h->tune.rows = rows;
          }
        }
      T.pencil = h->tune.pencil;
      T.rows = h->tune.rows;
      // tracer groups per launch (grid y): more, shorter blocks fill the last wave of the grid
      auto sweep_groups = [&](const char* key, int& best_g, int& Tg, std::function<void()> run) {
        rep += std::string("], \"") + key + "\": [";
        bool first_g = true;
        float bg = 1e30f;
        for (int gsz : {1, 2, 3, 4, 6, 8, 12}) {
          if (gsz > std::max(1, h->dt.ntr)) continue;
          Tg = gsz;
          float ms = time_min(h->st, 3, run);
          std::snprintf(line, sizeof line, "%s{\"groups\": %d, \"ms\": %.4f}",
                        first_g ? "" : ", ", gsz, ms);
          rep += line;
          first_g = false;
          if (ms < bg) {
            bg = ms;
            best_g = gsz;
          }
        }
        Tg = best_g;
      };
      sweep_groups("x_tracer_groups", h->tune.xgroups, T.xgroups,
                   [&] { rs::launch_flux_dir(h->st, T, Q, 0); });
      sweep_groups("yz_tracer_groups", h->tune.yzgroups, T.yzgroups, [&] {
        rs::launch_flux_dir(h->st, T, Q, 1);
        rs::launch_flux_dir(h->st, T, Q, 2);
      });
      std::snprintf(line, sizeof line,
                    "], \"transport_choice\": {\"xthreads\": %d, \"pencil\": %d, \"rows\": %d, "
                    "\"x_tracer_groups\": %d, \"yz_tracer_groups\": %d}",
                    h->tune.xthreads, h->tune.pencil, h->tune.rows, h->tune.xgroups,
                    h->tune.yzgroups);
      rep += line;
      if (h->cfg.precision == RS_PREC_MIXED) {
        // the FP32 deviation-form pencils: threads per lon row and tracers per block for x,
        // pencil width, rows and tracers per block for y and z, each with bulk-copy and with
        // plain-load staging when the mode is AUTO (one split of Q, then timings)
        const int ntr = h->dt.ntr;
        std::vector<int> spers{1, 2, ntr};
        std::vector<int> modes;
        if (h->tmaps && h->staging != RS_STAGING_PLAIN) modes.push_back(RS_STAGING_BULK);
        if (!h->tmaps || h->staging != RS_STAGING_BULK) modes.push_back(RS_STAGING_PLAIN);
        rs::launch_flux_dir_mixed(h->st, T, Q, -1, true);
        rep += ", \"mixed_lon_rows\": [";
        first = true;
        float bmx = 1e30f, bmyz = 1e30f;
        int mode_x = modes[0], mode_yz = modes[0];
        T.tma = h->tmaps;
        const bool auto_mode = h->staging == RS_STAGING_AUTO;
        bool stream_x = false, stream_yz = false;
        if (auto_mode) {  // the streaming forms first: a warp per lon row segment, x tracers
          T.mstream_x = 1;
          for (int sp : spers) {
            T.msper_x = sp;
            float ms = time_min(h->st, 3, [&] { rs::launch_flux_dir_mixed(h->st, T, Q, 0, false); });
            std::snprintf(line, sizeof line, "%s{\"staging\": \"stream\", \"tracers\": %d, \"ms\": %.4f}",
                          first ? "" : ", ", sp, ms);
            rep += line;
            first = false;
            if (ms < bmx) {
              bmx = ms;
              stream_x = true;
              h->tune.msper_x = sp;
            }
          }
        }
        T.mstream_x = 0;
        for (int md : modes) {
          T.mbulk_x = md == RS_STAGING_BULK;
          for (int xt : {64, 128, 256})
            for (int sp : spers) {
              T.mxthreads = xt;
              T.msper_x = sp;
              float ms = time_min(h->st, 3, [&] { rs::launch_flux_dir_mixed(h->st, T, Q, 0, false); });
              std::snprintf(line, sizeof line,
                            "%s{\"staging\": \"%s\", \"threads\": %d, \"tracers\": %d, \"ms\": %.4f}",
                            first ? "" : ", ", md == RS_STAGING_BULK ? "bulk" : "plain", xt, sp, ms);
              rep += line;
              first = false;
              if (ms < bmx) {
                bmx = ms;
                mode_x = md;
                stream_x = false;
                h->tune.mxthreads = xt;
                h->tune.msper_x = sp;
              }
            }
        }
        rep += "], \"mixed_pencils\": [";
        first = true;
        if (auto_mode) {  // the streaming forms: one thread per lat / vertical line
          T.mstream_yz = 1;
          for (int sp : spers) {
            T.msper_yz = sp;
            float ms = time_min(h->st, 3, [&] {
              rs::launch_flux_dir_mixed(h->st, T, Q, 1, false);
              rs::launch_flux_dir_mixed(h->st, T, Q, 2, false);
            });
            std::snprintf(line, sizeof line, "%s{\"staging\": \"stream\", \"tracers\": %d, \"ms\": %.4f}",
                          first ? "" : ", ", sp, ms);
            rep += line;
            first = false;
            if (ms < bmyz) {
              bmyz = ms;
              stream_yz = true;
              h->tune.msper_yz = sp;
            }
          }
        }
        T.mstream_yz = 0;
        for (int md : modes) {
          T.mbulk_yz = md == RS_STAGING_BULK;
          for (int pw : {16, 32})
            for (int rows : {4, 8, 16})
              for (int sp : spers) {
                T.mpencil = pw;
                T.mrows = rows;
                T.msper_yz = sp;
                float ms = time_min(h->st, 3, [&] {
                  rs::launch_flux_dir_mixed(h->st, T, Q, 1, false);
                  rs::launch_flux_dir_mixed(h->st, T, Q, 2, false);
                });
                std::snprintf(line, sizeof line,
                              "%s{\"staging\": \"%s\", \"pencil\": %d, \"rows\": %d, "
                              "\"tracers\": %d, \"ms\": %.4f}",
                              first ? "" : ", ", md == RS_STAGING_BULK ? "bulk" : "plain", pw, rows,
                              sp, ms);
                rep += line;
                first = false;
                if (ms < bmyz) {
                  bmyz = ms;
                  mode_yz = md;
                  stream_yz = false;
                  h->tune.mpencil = pw;
                  h->tune.mrows = rows;
                  h->tune.msper_yz = sp;
                }
              }
        }
        h->tune.mbulk_x = mode_x == RS_STAGING_BULK;
        h->tune.mbulk_yz = mode_yz == RS_STAGING_BULK;
        h->tune.mstream_x = stream_x;
        h->tune.mstream_yz = stream_yz;
        std::snprintf(line, sizeof line,
                      "], \"mixed_choice\": {\"xthreads\": %d, \"x_tracers\": %d, \"x_staging\": "
                      "\"%s\", \"pencil\": %d, \"rows\": %d, \"yz_tracers\": %d, "
                      "\"yz_staging\": \"%s\"}",
                      h->tune.mxthreads, std::min(h->tune.msper_x, ntr),
                      stream_x ? "stream" : (mode_x == RS_STAGING_BULK ? "bulk" : "plain"),
                      h->tune.mpencil, h->tune.mrows, h->tune.msper_yz,
                      stream_yz ? "stream" : (mode_yz == RS_STAGING_BULK ? "bulk" : "plain"));
        rep += line;
      }
      refresh_dt(h);
      invalidate_graphs(h);
    }
    rep += "}";
    CK(cudaStreamSynchronize(h->st));
    if (buf && buf_len) {
      std::strncpy(buf, rep.c_str(), buf_len - 1);
      buf[buf_len - 1] = 0;
    }
  });
}

// ====================================================================== allocation-free attempt
// Some callers cannot allocate device memory at the point where they want to step the
// chemistry: a host that runs its own memory pool (a Julia CUDA.jl or PyTorch caching
// allocator that has already reserved the device), or a latency-critical loop where an
// allocation would synchronise the device.  rs_ros23_attempt_noalloc serves them: its
// scratch (the 256-cell partial sums of the error norm and the controller record) lives in
// one file-scope device array that every GPU loading this library holds until exit.
namespace {

constexpr size_t kNoAllocMaxCells = (size_t)1 << 24;  // 16,777,216 cells
constexpr size_t kNoAllocParts = kNoAllocMaxCells / rs::kRedThreads;  // 65,536 partial sums
constexpr size_t kNoAllocCtlBytes = 512;  // room for one controller record
static_assert(sizeof(Ctl) <= kNoAllocCtlBytes, "controller record outgrew its scratch slot");
constexpr size_t kNoAllocBytes = kNoAllocParts * sizeof(double) + kNoAllocCtlBytes;  // 524,800 B

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
void* g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};
std::mutex g_noalloc_mu;

// Device address of the scratch array for device `dev`, resolved once per device by rs_create
// with that device current (a failed lookup fails rs_create).  Host code must not take the
// array's address directly: on the host the symbol is only a stand-in.  The cached address
// belongs to the device's primary context; after cudaDeviceReset the library must be
// reloaded before the entry point is used again.
void* noalloc_scratch(int dev) {
  if (dev < 0 || dev >= kNoAllocMaxDevices) throw RsError(RS_ERR_INVALID, "device ordinal");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[dev] = p;
  }
  return g_noalloc_addr[dev];
}

}  // namespace

extern "C" rs_status rs_ros23_attempt_noalloc(rs_handle* h, double dt, const double* d_u_in,
                                              double* d_u_out, double* eest) {
  if (!h || !d_u_in || !d_u_out) return RS_ERR_INVALID;
  return guard(h, [&] {
    if (!(dt > 0.0)) throw RsError(RS_ERR_INVALID, "dt must be positive");
    if (h->nc > kNoAllocMaxCells)
      throw RsError(RS_ERR_INVALID, "rs_ros23_attempt_noalloc handles at most 16,777,216 cells; "
                                    "this grid has " + std::to_string(h->nc));
    int prev = -1;
    CK(cudaGetDevice(&prev));
    if (prev != h->cfg.device) CK(cudaSetDevice(h->cfg.device));
    struct Restore {
      int d, p;
      ~Restore() {
        if (p >= 0 && p != d) cudaSetDevice(p);
      }
    } restore{h->cfg.device, prev};
    unsigned char* base = static_cast<unsigned char*>(h->noalloc_base);  // resolved by rs_create
    double* part = reinterpret_cast<double*>(base);
    Ctl* ctl = reinterpret_cast<Ctl*>(base + kNoAllocParts * sizeof(double));
    ensure_rates(h);
    Ctl init = make_ctl(h, 0.0, dt, dt, h->cfg.ctrl_C, (double)h->nc * h->nsp);
    init.cur = 0;
    init.maxiters = 1.0;
    rs::launch_ctl_init(h->st, ctl, init);  // every field of the record is rewritten
    rs::launch_ros23_attempt(h->lc, ctl, const_cast<double*>(d_u_in), d_u_out, h->krates.p,
                             h->have_emis ? h->emis.p : nullptr, part, h->cfg.rtol_C,
                             h->cfg.atol_C, 0);
    rs::launch_finalize(h->st, ctl, part, (int)((h->nc + rs::kRedThreads - 1) / rs::kRedThreads));
    CK(cudaGetLastError());
    if (eest) {
      CK(cudaMemcpyAsync(&h->hctl[2], ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      *eest = h->hctl[2].eest;
    } else {
      CK(cudaStreamSynchronize(h->st));
    }
  });
}
