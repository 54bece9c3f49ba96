// peak_probe.cu -- measures the FP64 and FP32 FMA issue rate of the device (the roofline
// denominators for the FP64-bound chemistry and transport kernels; the HBM and bf16
// denominators come from the measured peaks file).  Independent FMA chains, 8 per thread,
// 2 CTAs of 1024 threads per SM; in-bounds writes only; bounded loops.
// Prints one JSON line: {"fp64_tflops": ..., "fp32_tflops": ..., "sm_count": ..., ...}
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

int main() {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) {
    printf("{\"error\": \"no device\"}\n");
    return 1;
  }
  int blocks = p.multiProcessorCount * 2;
  double f64 = measure<double>(blocks, 1024, 2000);
  double f32 = measure<float>(blocks, 1024, 40000);
  printf("{\"fp64_tflops\": %.4f, \"fp32_tflops\": %.4f, \"sm_count\": %d, \"name\": \"%s\", "
         "\"how\": \"8 independent FMA chains per thread, %d CTAs x 1024 threads, best of 3\"}\n",
         f64, f32, p.multiProcessorCount, p.name, blocks);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
