// FP32 FMA throughput probe: the roofline denominator for the CUDA-core
// bound intersection kernels (register-resident FMA chains, no memory).
#include <cuda_runtime.h>

#include "horender.h"

namespace {
constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) fma_loop(float* out, float a, float b) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-7f + c;
  for (int i = 0; i < kIters; ++i)
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 123.456f) out[0] = s;  // keeps the chains live; never true in practice
}
}  // namespace

extern "C" int ho_measure_fp32_peak(int device, double* tflops) {
  if (!tflops) return HO_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return HO_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  float* out = nullptr;
  if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return HO_ERR_CUDA;
  const int blocks = sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_loop<<<blocks, 256>>>(out, 0.999999f, 1e-7f);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    fma_loop<<<blocks, 256>>>(out, 0.999999f, 1e-7f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return HO_ERR_CUDA;
  const double flops = 2.0 * kChains * kIters * static_cast<double>(blocks) * 256.0;
  *tflops = flops / (best * 1e-3) / 1e12;
  return HO_OK;
}
