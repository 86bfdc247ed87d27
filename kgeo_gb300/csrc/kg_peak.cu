// FP64 pipe throughput probe (measurement helper for the roofline denominator).
#include <cuda_runtime.h>

#include "../../include/kgeo_gb300.h"

namespace {

__global__ void fp64_fma_loop(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-7, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int kgeo_measure_fp64_peak(double* tflops, void* stream) {
  if (!tflops) return KGEO_ERR_NULL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KGEO_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return KGEO_ERR_CUDA;
  const int blocks = sms * 8, threads = 256, iters = 40;
  double* out = nullptr;
  if (cudaMallocAsync(&out, sizeof(double) * blocks * threads, s) != cudaSuccess) return KGEO_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int w = 0; w < 2; ++w) fp64_fma_loop<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-6);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, s);
    fp64_fma_loop<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-6);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaFreeAsync(out, s);
  cudaStreamSynchronize(s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return cudaGetLastError() == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}
