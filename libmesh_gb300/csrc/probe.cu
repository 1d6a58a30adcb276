// FP64 pipe throughput probe: independent DFMA chains on every SM, timed with
// CUDA events.  Gives the FP64 roofline denominator the assembly kernels are
// measured against (GB300 FP64 is not among the measured peaks).
#include <cuda_runtime.h>

#include "../../include/libmesh_gb300.h"

namespace {
constexpr int CHAINS = 8;
__global__ void k_dfma(int iters, double a, double b, double *sink) {
  double x[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
  double s = 0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += x[c];
  if (s == 1234.5678) sink[0] = s;  // keeps the chains live
}
}  // namespace

extern "C" lmg_status lmg_probe_fp64(int32_t device, double *tflops) {
  if (!tflops) return LMG_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return LMG_ERR_CUDA;
  int n_sm = 0;
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device);
  double *sink = nullptr;
  if (cudaMalloc((void **)&sink, sizeof(double)) != cudaSuccess) return LMG_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = n_sm * 4, threads = 256, iters = 4096;
  k_dfma<<<blocks, threads>>>(64, 0.999999, 1e-7, sink);  // warm-up
  cudaEventRecord(e0);
  k_dfma<<<blocks, threads>>>(iters, 0.999999, 1e-7, sink);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess || ms <= 0) return LMG_ERR_CUDA;
  const double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return LMG_OK;
}
