// probe.cu -- FP32 FMA throughput of the device, the peak for the FP32 Lanczos roofline.
//
// Every thread runs 8 independent FMA chains in registers (no memory traffic inside the
// timed loop); 4 CTAs of 256 threads per SM keep all four SM sub-partitions busy.
#include <cuda_runtime.h>

#include "sq_kernels.hpp"

namespace sq {

namespace {

constexpr int kChains = 8;
constexpr int kIters = 8192;

__global__ void __launch_bounds__(256) fma_probe_kernel(float *sink, float seed) {
  float v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) v[c] = seed + threadIdx.x * 1e-7f + c;
  const float a = 0.999999f, b = 1e-7f;
  for (int i = 0; i < kIters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = fmaf(v[c], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += v[c];
  if (s == 12345.678f) sink[blockIdx.x] = s;  // keeps the chains live, never true in practice
}

}  // namespace

cudaError_t measure_fp32_peak(int device, double *tflops) {
  int sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 4, threads = 256;
  float *sink = nullptr;
  if ((e = cudaMalloc(&sink, sizeof(float) * blocks)) != cudaSuccess) return e;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  fma_probe_kernel<<<blocks, threads>>>(sink, 1.0f);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    cudaEventRecord(t0);
    fma_probe_kernel<<<blocks, threads>>>(sink, 1.0f + r);
    cudaEventRecord(t1);
    cudaEventSynchronize(t1);
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    if (ms < best) best = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(sink);
  if (e != cudaSuccess) return e;
  const double flops = 2.0 * kChains * (double)kIters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return cudaSuccess;
}

}  // namespace sq
