// rs_jit.h -- mechanism-specialised chemistry kernels (rs_jit.cu).
//
// At rs_create the host writes the mechanism's rate products, RHS sums, exact Jacobian, the
// pivot-free LU of W = I - dt*d*J and its triangular solves out as straight-line CUDA C++
// (constant indices, constant stoichiometric coefficients) and compiles it for sm_103a with
// NVRTC.  Every work array then lives in registers (or, for W, in shared memory) and no
// thread walks an index table, which removes the table loads and the local-memory traffic of
// the table-walking kernels in rs_chem.cu.  The arithmetic follows the same association as
// those kernels, so a strict-build handle stays bit-compatible with the CPU restatement.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "rs_device.cuh"
#include "rs_mech.h"

namespace rs {

struct PerCellArgs;

// Variants of the global-dt attempt kernel (the autotuner picks one by timing):
//   0 "regs"   W in registers (spilled by ptxas where needed), one 256-thread block per SM
//   1 "smem"   W in dynamic shared memory, [slot][thread] so a warp's accesses are contiguous
//   2 "regs2"  as 0 but capped at 128 registers for two blocks per SM
//   3 "split"  the last half of W's LU slots (at most 55) in shared memory, the rest in
//              registers, capped at 128 registers for two blocks per SM
constexpr int kJitVariants = 4;
extern const char* const kJitVariantNames[kJitVariants];

struct JitChem {
  cudaKernel_t attempt[kJitVariants][2] = {};  // [variant][has emission]; null: not built
  cudaKernel_t per_cell[2] = {};               // [has emission]
  cudaKernel_t rcp = nullptr;                  // elementwise production reciprocal
  cudaKernel_t vjp[2] = {};                    // ROS23 step VJP [has emission]
  cudaKernel_t step[2] = {};                   // accepted step, no error estimate [has emission]
  cudaKernel_t vjpk[2] = {};                   // step VJP reading k1, z2 from the stage tape
  size_t attempt_smem[kJitVariants] = {};  // dynamic shared bytes of each attempt variant
  int variant = 0;          // variant used for global-dt attempts
  double compile_ms = 0;    // NVRTC time (0 when the compiled image came from cache)
  int regs[kJitVariants] = {};  // registers per thread of each attempt variant
};

// True when the mechanism is small enough for straight-line code (all work arrays of one
// attempt fit the register file without a table walk).
bool jit_chem_eligible(const MechTables& T);

// Generate, compile (or fetch from the process-wide cache) and load the specialised kernels
// for the current device.  Returns null and sets *why when NVRTC is unavailable or fails.
std::shared_ptr<JitChem> jit_chem_build(const MechTables& T, double ros_d, double ros_c32,
                                        bool strict, std::string* why);

// The generated source (for inspection and tests).
std::string jit_chem_source(const MechTables& T, bool strict);

// NVRTC compile of generated source to an sm_103a cubin; needs no device.  With verbose the
// log carries ptxas's resource usage.  Returns false with the error text in *log.
bool jit_compile(const std::string& src, bool strict, bool verbose, std::vector<char>* cubin,
                 std::string* log);

// Same contracts as launch_ros23_attempt / launch_chem_per_cell in rs_kernels.h.
void jit_launch_attempt(const JitChem& J, cudaStream_t st, int nc, int nsp, const Ctl* ctl,
                        double* U0, double* U1, const double* kr, const double* em,
                        double* part, double rtol, double atol, int clamp, double* F0,
                        double* F1);
// same contract as launch_ros23_step in rs_kernels.h
void jit_launch_step(const JitChem& J, cudaStream_t st, int nc, int nsp, const Ctl* ctl,
                     double* U0, double* U1, const double* kr, const double* em, int clamp);
void jit_launch_rcp(const JitChem& J, cudaStream_t st, const double* x, double* r, int n);
// same contract as launch_ros23_vjp in rs_kernels.h
void jit_launch_vjp(const JitChem& J, cudaStream_t st, int nc, int nsp, const double* U,
                    const double* Uout, const double* lam, double* lam_out, const double* kr,
                    const double* em, double* ebar, double dt, int clamp,
                    const double* kz = nullptr);
void jit_launch_per_cell(const JitChem& J, cudaStream_t st, int nc, int nsp, int nblocks,
                         int threads, double* U, const double* kr, const double* em,
                         double* dtc, double* steps, unsigned long long* queue, int* status,
                         const PerCellArgs& a);

}  // namespace rs
