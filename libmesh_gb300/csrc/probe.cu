// FP64 throughput probes, timed with CUDA events: independent DFMA chains on
// every SM (the FP64 roofline denominator the assembly kernels are measured
// against; the copy-bandwidth and BF16 peaks measured beside it say nothing
// about FP64), and the same
// with FP64 tensor-core products (mma.sync m8n8k4 f64, DMMA), to compare the
// two routes an FP64 contraction could take.
#include <cuda_runtime.h>

#include "../../include/libmesh_gb300.h"
#include "df.cuh"

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
// CHAINS independent accumulators per warp, each a chain of m8n8k4 FP64
// products (512 flops per warp-wide instruction).
__global__ void k_dmma(int iters, double *sink) {
  const double a = 1.0 + threadIdx.x * 1e-6, b = 0.5;
  double d[CHAINS][2];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) d[c][0] = d[c][1] = c;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CHAINS; ++c)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(d[c][0]), "+d"(d[c][1])
                   : "d"(a), "d"(b));
  double s = 0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += d[c][0] + d[c][1];
  if (s == 1234.5678) sink[0] = s;
}

template <typename Launch>
lmg_status time_probe(int32_t device, double flops_per_launch, Launch &&launch, double *tflops) {
  if (cudaSetDevice(device) != cudaSuccess) return LMG_ERR_CUDA;
  double *sink = nullptr;
  if (cudaMalloc((void **)&sink, sizeof(double)) != cudaSuccess) return LMG_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch(64, sink);  // warm-up
  cudaEventRecord(e0);
  launch(4096, sink);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess || ms <= 0) return LMG_ERR_CUDA;
  *tflops = flops_per_launch / (ms * 1e-3) / 1e12;
  return LMG_OK;
}
}  // namespace

extern "C" lmg_status lmg_probe_fp64_tensor(int32_t device, double *tflops) {
  if (!tflops) return LMG_ERR_ARG;
  int n_sm = 0;
  if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return LMG_ERR_CUDA;
  const int blocks = n_sm * 4, threads = 256;
  const double flops = 512.0 * CHAINS * 4096.0 * blocks * (threads / 32);
  return time_probe(
      device, flops, [&](int iters, double *sink) { k_dmma<<<blocks, threads>>>(iters, sink); }, tflops);
}

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

// The exact float -> double conversion the kernels use (lmg::f2d), applied on
// the device to n values: out[i] = f2d(in[i]).
namespace {
__global__ void k_f2d(int64_t n, const float *in, double *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = lmg::f2d(in[i]);
}
}  // namespace

extern "C" lmg_status lmg_probe_f2d(int32_t device, int64_t n, const float *in, double *out) {
  if (n < 0 || (n > 0 && (!in || !out))) return LMG_ERR_ARG;
  if (n == 0) return LMG_OK;
  if (cudaSetDevice(device) != cudaSuccess) return LMG_ERR_CUDA;
  float *din = nullptr;
  double *dout = nullptr;
  cudaError_t e = cudaMalloc((void **)&din, sizeof(float) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc((void **)&dout, sizeof(double) * (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpy(din, in, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_f2d<<<256, 256>>>(n, din, dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
  if (din) cudaFree(din);
  if (dout) cudaFree(dout);
  return e == cudaSuccess ? LMG_OK : LMG_ERR_CUDA;
}
