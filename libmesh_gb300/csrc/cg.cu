// Jacobi-preconditioned conjugate gradients on the assembled CSR (FP64), the
// solve behind LinearImplicitSystem::solve for the symmetric forms
// (src/systems/linear_implicit_system.C:122-165; KSPCG as set up in
// systems_of_equations_ex6.C:90-100; Eigen CG semantics in
// src/solvers/eigen_sparse_linear_solver.C:132-170).  Stops when
// ||r||_2 <= rtol ||b||_2.  Every reduction is a fixed two-stage tree, so
// repeated solves give identical iterates.  Scalars stay on the device; the
// host reads the residual every few iterations.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "assemble.cuh"

namespace lmg {

namespace {

constexpr int RT = 256;      // threads per reduction block
constexpr int RBLK = 1024;   // reduction blocks

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double w[RT / 32];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = (threadIdx.x < RT / 32) ? w[threadIdx.x] : 0.0;
    s = warp_sum(s);
  }
  __syncthreads();
  return s;  // valid in thread 0
}

__global__ void k_spmv(int64_t n, const int32_t *rp, const int32_t *col, const double *val, const double *x,
                       double *y) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    double s = 0.0;
    for (int32_t k = rp[r] + lane; k < rp[r + 1]; k += 32) s += val[k] * x[col[k]];
    s = warp_sum(s);
    if (lane == 0) y[r] = s;
  }
}

// partial[b] for two dot products at once: (x1.y1, x2.y2)
__global__ void k_dot2(int64_t n, const double *x1, const double *y1, const double *x2, const double *y2,
                       double *partial) {
  double s1 = 0.0, s2 = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n; i += (int64_t)gridDim.x * RT) {
    s1 += x1[i] * y1[i];
    if (x2) s2 += x2[i] * y2[i];
  }
  s1 = block_sum(s1);
  s2 = block_sum(s2);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = s1;
    partial[2 * blockIdx.x + 1] = s2;
  }
}

__global__ void k_dot2_final(int nblk, const double *partial, double *out) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = threadIdx.x; i < nblk; i += RT) {
    s1 += partial[2 * i];
    s2 += partial[2 * i + 1];
  }
  s1 = block_sum(s1);
  s2 = block_sum(s2);
  if (threadIdx.x == 0) {
    out[0] = s1;
    out[1] = s2;
  }
}

__global__ void k_diag_inv(int64_t n, const int32_t *rp, const int32_t *col, const double *val, double *dinv) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int32_t k = rp[r]; k < rp[r + 1]; ++k)
      if (col[k] == r) d = val[k];
    dinv[r] = (d != 0.0) ? 1.0 / d : 1.0;
  }
}

// x += a p; r -= a q; z = dinv r   with a = rz / pq read from the device
__global__ void k_update_xr(int64_t n, const double *sc, double *x, double *r, double *z, const double *p,
                            const double *q, const double *dinv) {
  const double a = sc[0] / sc[2];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    const double ri = r[i] - a * q[i];
    r[i] = ri;
    z[i] = dinv[i] * ri;
  }
}

// p = z + (rz_new / rz) p ; rz <- rz_new
__global__ void k_update_p(int64_t n, double *sc, double *p, const double *z) {
  const double b = sc[3] / sc[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + b * p[i];
}

__global__ void k_init(int64_t n, const double *b, double *x, double *r, double *z, double *p, const double *dinv) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = 0.0;
    r[i] = b[i];
    z[i] = dinv[i] * b[i];
    p[i] = z[i];
  }
}

__global__ void k_copy2(double *dst, const double *src) {
  dst[0] = src[0];
}

}  // namespace

// sc layout: [0] rz, [1] rr, [2] pq, [3] rz_new, [4] rr_new
int cg_solve(int64_t n, const int32_t *rp, const int32_t *col, const double *val, const double *b, double *x,
             double rtol, int maxit, cudaStream_t s, int n_sm, int *iters, double *relres, int64_t *launches) {
  double *r, *z, *p, *q, *dinv, *partial, *sc;
  const size_t bytes = sizeof(double) * (size_t)n;
  if (cudaMalloc(&r, bytes) || cudaMalloc(&z, bytes) || cudaMalloc(&p, bytes) || cudaMalloc(&q, bytes) ||
      cudaMalloc(&dinv, bytes) || cudaMalloc(&partial, sizeof(double) * 2 * RBLK) || cudaMalloc(&sc, sizeof(double) * 8))
    return 7;
  const int g1 = n_sm * 8, gs = n_sm * 16;
  int nblk = (int)std::min<int64_t>(RBLK, (n + RT - 1) / RT);
  int64_t L = 0;
  k_diag_inv<<<g1, 256, 0, s>>>(n, rp, col, val, dinv);
  k_init<<<g1, 256, 0, s>>>(n, b, x, r, z, p, dinv);
  k_dot2<<<nblk, RT, 0, s>>>(n, r, z, r, r, partial);
  k_dot2_final<<<1, RT, 0, s>>>(nblk, partial, sc);  // sc[0] = rz, sc[1] = rr
  L += 4;
  double h[2];
  cudaMemcpyAsync(h, sc, sizeof(double) * 2, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const double bnorm = std::sqrt(h[1]);
  double rn = bnorm;
  int it = 0;
  if (bnorm == 0.0) {
    *iters = 0;
    *relres = 0.0;
  } else {
    for (it = 0; it < maxit; ++it) {
      k_spmv<<<gs, 256, 0, s>>>(n, rp, col, val, p, q);
      k_dot2<<<nblk, RT, 0, s>>>(n, p, q, nullptr, nullptr, partial);
      k_dot2_final<<<1, RT, 0, s>>>(nblk, partial, sc + 2);  // sc[2] = pq
      k_update_xr<<<g1, 256, 0, s>>>(n, sc, x, r, z, p, q, dinv);
      k_dot2<<<nblk, RT, 0, s>>>(n, r, z, r, r, partial);
      k_dot2_final<<<1, RT, 0, s>>>(nblk, partial, sc + 3);  // sc[3] = rz_new, sc[4] = rr
      k_update_p<<<g1, 256, 0, s>>>(n, sc, p, z);
      k_copy2<<<1, 1, 0, s>>>(sc, sc + 3);                   // rz <- rz_new
      L += 8;
      if ((it + 1) % 16 == 0 || it + 1 == maxit) {
        cudaMemcpyAsync(h, sc + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        rn = std::sqrt(h[0]);
        if (!(rn > rtol * bnorm)) { ++it; break; }
      }
    }
    *iters = it;
    *relres = rn / bnorm;
  }
  *launches += L;
  cudaError_t e = cudaStreamSynchronize(s);
  cudaFree(r); cudaFree(z); cudaFree(p); cudaFree(q); cudaFree(dinv); cudaFree(partial); cudaFree(sc);
  return e == cudaSuccess ? 0 : 2;
}

}  // namespace lmg
