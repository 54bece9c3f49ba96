// rs_control.cu -- device-resident step-size control and layout kernels.
//
// k_finalize closes one attempt: level-2 fixed-tree sum of the 256-cell partials, the hairer
// norm EEst = sqrt(sse/N) (rx_traced_integrator.jl:347,398), then the PI controller exactly as
// adaptive_solve's loop body (rx_traced_integrator.jl:480-505): NaN -> reject, q11 = EEst^b1,
// q = q11/qold^b2 clamped to [1/qmax, 1/qmin] after /gamma, accept iff EEst <= 1 with the
// steady band snapped to 1, reject dt <- dtc/min(1/qmin, q11/gamma).  It also prepares the
// next attempt (dtc = min(dt, tend - t), SSPRK43 stage factors) and raises `done` when the
// loop condition (t < tend - 1e-9) & (iters < maxiters) fails, so the host never has to
// read anything back between attempts.
#include <cuda_runtime.h>

#include "rs_device.cuh"
#include "rs_kernels.h"

namespace rs {

__device__ void prepare_next(Ctl* c) {
  c->dtc = fmin(c->dt, c->tend - c->t);
  c->dto2 = c->dtc / 2;
  c->dto6 = c->dtc / 6;
  c->dtgamma = c->dtc * c->ros_d;
  double tlim = c->tend - 1.0e-9;
  c->done = !((c->t < tlim) && (c->iters < c->maxiters));
  if (c->omega != 0.0) {
    double dt_2 = c->dtc / 2;
    c->g[0] = cos(c->omega * (c->t + 0.0 * c->dtc));
    c->g[1] = cos(c->omega * (c->t + 0.5 * c->dtc));
    c->g[2] = cos(c->omega * (c->t + 1.0 * c->dtc));
    c->g[3] = cos(c->omega * (c->t + dt_2));
  } else {
    c->g[0] = c->g[1] = c->g[2] = c->g[3] = 1.0;
  }
}

// One attempt's close-out (all threads of one 256-thread block); returns in every thread.
__device__ void finalize_body(Ctl* __restrict__ c, const double* __restrict__ partial,
                              int nparts, double* sm) {
  if (c->done) return;
  double acc = 0.0;
  for (int q = threadIdx.x; q < nparts; q += kRedThreads) acc = acc + partial[q];
  double sse = block_tree256(acc, sm);
  if (threadIdx.x != 0) return;
  double EEst = sqrt(sse / c->ntot);
  if (isnan(EEst)) EEst = 1.0e10;
  double q11 = pow(fmax(EEst, 1.0e-35), c->beta1);
  double qden = pow(c->qold, c->beta2);
  double q = q11 / qden;
  q = fmax(c->invqmax, fmin(c->invqmin, q / c->gamma));
  bool accept = EEst <= 1.0;
  bool insteady = (c->qsmin <= q) && (q <= c->qsmax);
  double qa = insteady ? 1.0 : q;
  double dtc = c->dtc;
  double dt_acc = dtc / qa;
  double qr = fmin(c->invqmin, q11 / c->gamma);
  double dt_rej = dtc / qr;
  c->eest = EEst;
  c->accept = accept;
  if (accept) {
    if (c->seq) {
      int k = *c->nseq;
      if (k < c->seqcap) {
        c->seq[2 * k] = c->t;
        c->seq[2 * k + 1] = dtc;
      }
      *c->nseq = k + 1;
    }
    c->cur ^= 1;
    c->t = c->t + dtc;
    c->dt = dt_acc;
    c->qold = fmax(EEst, c->qoldinit);
    c->nacc += 1.0;
  } else {
    c->dt = dt_rej;
    c->nrej += 1.0;
  }
  c->iters += 1.0;
  prepare_next(c);
}

__global__ void __launch_bounds__(kRedThreads) k_finalize(Ctl* __restrict__ c,
                                                          const double* __restrict__ partial,
                                                          int nparts) {
  __shared__ double sm[kRedThreads];
  finalize_body(c, partial, nparts, sm);
}

// Graph-resident variant: also drives the conditional WHILE node of the device loop.  It sets
// the loop condition on EVERY path (0 once the controller is done), and the controller raises
// done after at most maxiters attempts, so the graph loop always terminates.
__global__ void __launch_bounds__(kRedThreads) k_finalize_graph(
    Ctl* __restrict__ c, const double* __restrict__ partial, int nparts,
    cudaGraphConditionalHandle loop) {
  __shared__ double sm[kRedThreads];
  finalize_body(c, partial, nparts, sm);
  __syncthreads();
  if (threadIdx.x == 0) cudaGraphSetConditional(loop, c->done ? 0u : 1u);
}

__global__ void k_ctl_init(Ctl* __restrict__ c, Ctl init) {
  *c = init;
  prepare_next(c);
}

__global__ void k_nonfinite(const double* __restrict__ U, size_t n, int* __restrict__ flag) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  int bad = 0;
  for (; i < n; i += stride) bad |= !isfinite(U[i]);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// cell-major (c = (i*nlat + j)*nlev + k, species fastest) <-> grid SoA planes
__global__ void k_to_soa(const double* __restrict__ cm, double* __restrict__ soa, int nlon,
                         int nlat, int nlev, int nsp) {
  size_t nc = (size_t)nlon * nlat * nlev;
  size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;  // index into soa
  if (x >= nc * nsp) return;
  int s = (int)(x / nc);
  size_t g = x % nc;
  int i = (int)(g % nlon);
  int j = (int)((g / nlon) % nlat);
  int k = (int)(g / ((size_t)nlon * nlat));
  size_t c = ((size_t)i * nlat + j) * nlev + k;
  soa[x] = cm[c * nsp + s];
}
__global__ void k_to_cellmajor(const double* __restrict__ soa, double* __restrict__ cm, int nlon,
                               int nlat, int nlev, int nsp) {
  size_t nc = (size_t)nlon * nlat * nlev;
  size_t y = (size_t)blockIdx.x * blockDim.x + threadIdx.x;  // index into cm
  if (y >= nc * nsp) return;
  int s = (int)(y % nsp);
  size_t c = y / nsp;
  int k = (int)(c % nlev);
  int j = (int)((c / nlev) % nlat);
  int i = (int)(c / ((size_t)nlev * nlat));
  cm[y] = soa[(size_t)s * nc + ((size_t)k * nlat + j) * nlon + i];
}

// Adjoint tape, one attempt's close-out after the controller's: when the attempt was accepted
// (the accepted count passed the stored count) the state before the step -- the buffer the
// accepted candidate did not go to -- is copied to its slot; k_tape_bump then records it.
__global__ void k_tape_store(const Ctl* __restrict__ c, const double* __restrict__ U0,
                             const double* __restrict__ U1, size_t n) {
  if (!c->tape) return;
  const int k = (int)c->nacc - 1;
  if (k < c->ntape[0] || k >= c->tapecap) return;
  const double* __restrict__ src = c->cur ? U0 : U1;
  double* __restrict__ dst = c->tape + (size_t)k * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    dst[e] = src[e];
}
__global__ void k_tape_bump(const Ctl* __restrict__ c) {
  if (!c->tape) return;
  const int k = (int)c->nacc;
  if (k <= c->ntape[0]) return;
  if (k > c->tapecap) c->ntape[1] = 1;
  else c->ntape[0] = k;
}
void launch_tape_store(cudaStream_t st, const Ctl* ctl, const double* U0, const double* U1,
                       size_t n) {
  k_tape_store<<<1024, 256, 0, st>>>(ctl, U0, U1, n);  // grid-stride copy
  k_tape_bump<<<1, 1, 0, st>>>(ctl);
}

// fixed-sequence replay: accept the attempt unconditionally (tools/adjoint_gradient.jl:647-669)
__global__ void k_replay_accept(Ctl* __restrict__ c) {
  c->cur ^= 1;
  c->t = c->t + c->dtc;
}
// lam *= (out > 0): adjoint of the clamp max(raw, 0) (tools/adjoint_gradient.jl:736)
__global__ void k_clamp_mask(size_t n, double* __restrict__ lam, const double* __restrict__ out) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n && !(out[e] > 0.0)) lam[e] = 0.0;
}
void launch_replay_accept(cudaStream_t st, Ctl* ctl) { k_replay_accept<<<1, 1, 0, st>>>(ctl); }
void launch_clamp_mask(cudaStream_t st, size_t n, double* lam, const double* out) {
  k_clamp_mask<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, lam, out);
}

void launch_finalize(cudaStream_t st, Ctl* ctl, const double* partial, int nparts) {
  k_finalize<<<1, kRedThreads, 0, st>>>(ctl, partial, nparts);
}
void launch_finalize_graph(cudaStream_t st, Ctl* ctl, const double* partial, int nparts,
                           cudaGraphConditionalHandle loop) {
  k_finalize_graph<<<1, kRedThreads, 0, st>>>(ctl, partial, nparts, loop);
}
void launch_ctl_init(cudaStream_t st, Ctl* ctl, const Ctl& init) {
  k_ctl_init<<<1, 1, 0, st>>>(ctl, init);
}
void launch_nonfinite(cudaStream_t st, const double* U, size_t n, int* flag) {
  k_nonfinite<<<1216, 256, 0, st>>>(U, n, flag);
}
void launch_to_soa(cudaStream_t st, const double* cm, double* soa, int nlon, int nlat, int nlev,
                   int nsp) {
  size_t n = (size_t)nlon * nlat * nlev * nsp;
  k_to_soa<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cm, soa, nlon, nlat, nlev, nsp);
}
void launch_to_cellmajor(cudaStream_t st, const double* soa, double* cm, int nlon, int nlat,
                         int nlev, int nsp) {
  size_t n = (size_t)nlon * nlat * nlev * nsp;
  k_to_cellmajor<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(soa, cm, nlon, nlat, nlev, nsp);
}

}  // namespace rs
