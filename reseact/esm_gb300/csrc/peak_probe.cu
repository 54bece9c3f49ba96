// peak_probe.cu -- measures the FP64 and FP32 FMA issue rate of the device (the roofline
// denominators for the FP64-bound chemistry and transport kernels; the HBM and bf16
// denominators come from the measured peaks file).  Independent FMA chains, 8 per thread,
// 2 CTAs of 1024 threads per SM; in-bounds writes only; bounded loops.
// Prints one JSON line: {"fp64_tflops": ..., "fp32_tflops": ..., "sm_count": ..., ...}
// With the argument "lanes": the FP64 chains run on only 1, 4, 8, 16 or 32 lanes of each warp,
// with 1..32 warps per SM, and the line lists the warp FMA instructions per SM per clock of
// each case (whether an FP64 warp instruction costs the same time whatever its active lanes).
#include <cuda_runtime.h>

#include <cstdio>

template <typename T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
  T acc[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) acc[c] = (T)(threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = fma(acc[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += acc[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// the chains of fma_chains on lanes < active of each warp only
__global__ void fma_chains_lanes(double* out, int iters, int active, double a, double b) {
  double acc[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) acc[c] = (double)(threadIdx.x + c);
  if ((int)(threadIdx.x & 31) < active) {
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] = fma(acc[c], a, b);
    }
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += acc[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

static int lanes_sweep(const cudaDeviceProp& p) {
  const int nsm = p.multiProcessorCount, iters = 2000;
  int khz = 0;
  cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, 0);  // the maximum SM clock
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * nsm * 1024) != cudaSuccess) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  printf("{\"fp64_lanes\": [");
  bool first = true;
  for (int warps : {1, 2, 4, 8, 16, 32})
    for (int active : {1, 4, 8, 16, 32}) {
      float best = 1e30f;
      for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        fma_chains_lanes<<<nsm, 32 * warps>>>(out, iters, active, 0.999, 0.001);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
      }
      const double winstr = 8.0 * iters * warps, clk = best * 1e-3 * khz * 1e3;
      printf("%s{\"warps_per_sm\": %d, \"active_lanes\": %d, \"ms\": %.4f, "
             "\"warp_fma_per_sm_clk\": %.5f}",
             first ? "" : ", ", warps, active, best, winstr / clk);
      first = false;
    }
  printf("], \"clock_mhz\": %d, \"name\": \"%s\"}\n", khz / 1000, p.name);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

template <typename T>
static double measure(int blocks, int threads, int iters) {
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    double tf = 2.0 * 8 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
    if (rep > 0 && tf > best) best = tf;
  }
  cudaFree(out);
  return best;
}

int main(int argc, char** argv) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) {
    printf("{\"error\": \"no device\"}\n");
    return 1;
  }
  if (argc > 1 && argv[1][0] == 'l') return lanes_sweep(p);
  int blocks = p.multiProcessorCount * 2;
  double f64 = measure<double>(blocks, 1024, 2000);
  double f32 = measure<float>(blocks, 1024, 40000);
  printf("{\"fp64_tflops\": %.4f, \"fp32_tflops\": %.4f, \"sm_count\": %d, \"name\": \"%s\", "
         "\"how\": \"8 independent FMA chains per thread, %d CTAs x 1024 threads, best of 3\"}\n",
         f64, f32, p.multiProcessorCount, p.name, blocks);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
