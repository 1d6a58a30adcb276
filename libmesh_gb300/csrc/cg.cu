// Jacobi-preconditioned conjugate gradients on the assembled CSR (FP64), the
// solve behind LinearImplicitSystem::solve for the symmetric forms
// (src/systems/linear_implicit_system.C:122-165; KSPCG as set up in
// systems_of_equations_ex6.C:90-100; Eigen CG semantics in
// src/solvers/eigen_sparse_linear_solver.C:132-170).  Stops when
// ||r||_2 <= rtol ||b||_2.  An iteration is three launches: the product
// q = A p fused with p.q, the x / r / z update fused with r.z and r.r, and the
// p update.  Every reduction is a fixed two-stage tree (block sums, then the
// last block to finish sums the partials in block order), so repeated solves
// give identical iterates.  Scalars stay on the device; the host reads the
// residual every 16 iterations.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "assemble.cuh"
#include "../../include/libmesh_gb300.h"

namespace lmg {

namespace {

constexpr int RT = 256;      // threads per reduction block
constexpr int RBLK = 16384;  // reduction blocks (largest grid of a reducing kernel)

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

// The last block to finish a reducing kernel sums the per-block partials in
// block order (the order does not depend on which block came last), so the
// reductions stay deterministic without a second launch.
__device__ __forceinline__ bool last_block(unsigned int *cnt) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(cnt, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  return last;
}

// q = A p (G lanes per row) and pq = p.q: per-block partials, the last block
// writes sc[2] = pq and resets the counter.
template <int G>
__global__ void __launch_bounds__(RT) k_spmv_pq(int64_t n, const int32_t *__restrict__ rp,
                                                 const int32_t *__restrict__ col, const double *__restrict__ val,
                                                 const double *__restrict__ p, double *__restrict__ q,
                                                 double *partial, double *sc, unsigned int *cnt) {
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), grp = lane / G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double pq = 0.0;
  for (int64_t w0 = warp * RPW; w0 < n; w0 += n_warps * RPW) {
    const int64_t r = w0 + grp;
    double s = 0.0;
    if (r < n) {
      const int32_t b = __ldg(rp + r), e = __ldg(rp + r + 1);
#pragma unroll 4
      for (int32_t k = b + sub; k < e; k += G) s += __ldg(val + k) * __ldg(p + __ldg(col + k));
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
    if (r < n && sub == 0) {
      q[r] = s;
      pq += p[r] * s;
    }
  }
  pq = block_sum(pq);
  if (threadIdx.x == 0) partial[blockIdx.x] = pq;
  if (last_block(cnt)) {
    double t = 0.0;
    const volatile double *vp = partial;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += RT) t += vp[i];
    t = block_sum(t);
    if (threadIdx.x == 0) {
      sc[2] = t;
      *cnt = 0u;
    }
  }
}

// x += a p; r -= a q; z = dinv r with a = rz / pq, rz = sc[cur]; then
// rz_new = r.z into sc[1 - cur] and rr = r.r into sc[3] (last block).
__global__ void __launch_bounds__(RT) k_update_xr_dots(int64_t n, double *sc, int cur, double *x, double *r,
                                                        double *z, const double *p, const double *q,
                                                        const double *dinv, double *partial, unsigned int *cnt) {
  const double a = sc[cur] / sc[2];
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    const double ri = r[i] - a * q[i];
    r[i] = ri;
    const double zi = dinv[i] * ri;
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  rz = block_sum(rz);
  rr = block_sum(rr);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = rz;
    partial[2 * blockIdx.x + 1] = rr;
  }
  if (last_block(cnt)) {
    double t1 = 0.0, t2 = 0.0;
    const volatile double *vp = partial;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += RT) {
      t1 += vp[2 * i];
      t2 += vp[2 * i + 1];
    }
    t1 = block_sum(t1);
    t2 = block_sum(t2);
    if (threadIdx.x == 0) {
      sc[1 - cur] = t1;
      sc[3] = t2;
      *cnt = 0u;
    }
  }
}

// p = z + (rz_new / rz) p with rz = sc[cur], rz_new = sc[1 - cur]
__global__ void k_update_p2(int64_t n, const double *sc, int cur, double *p, const double *z) {
  const double b = sc[1 - cur] / sc[cur];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + b * p[i];
}

// Lanes per row of the product for a mean row length (measured on the
// 27-point Q1 pattern of 129^3 nodes: 4 lanes 152 us, 8 lanes 322 us, 32 lanes
// 846 us per product).
inline int spmv_lanes(int64_t n, int64_t nnz) {
  const int64_t m = n > 0 ? nnz / n : 0;
  return m <= 48 ? 4 : (m <= 128 ? 8 : 16);
}

// One CG iteration in three launches, shared by both solvers.
void cg_iteration(int sg, int gs, int g1, cudaStream_t s, int64_t n, const int32_t *rp, const int32_t *col,
                  const double *val, double *x, double *r, double *z, double *p, double *q, const double *dinv,
                  double *partial, double *sc, unsigned int *cnt, int cur) {
  switch (sg) {
    case 4: k_spmv_pq<4><<<gs, RT, 0, s>>>(n, rp, col, val, p, q, partial, sc, cnt); break;
    case 8: k_spmv_pq<8><<<gs, RT, 0, s>>>(n, rp, col, val, p, q, partial, sc, cnt); break;
    default: k_spmv_pq<16><<<gs, RT, 0, s>>>(n, rp, col, val, p, q, partial, sc, cnt); break;
  }
  k_update_xr_dots<<<g1, RT, 0, s>>>(n, sc, cur, x, r, z, p, q, dinv, partial, cnt + 1);
  k_update_p2<<<g1, 256, 0, s>>>(n, sc, cur, p, z);
}

__global__ void k_init(int64_t n, const double *b, double *x, double *r, double *z, double *p, const double *dinv) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = 0.0;
    r[i] = b[i];
    z[i] = dinv[i] * b[i];
    p[i] = z[i];
  }
}

}  // namespace

// sc layout: [0], [1] rz of the current / next iteration (the initial rr in
// [1]), [2] pq, [3] rr, [4] two block counters of the reducing kernels
namespace {
// The solver's work vectors, freed on every return path.
struct CgWork {
  double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr, *partial = nullptr,
         *sc = nullptr;
  ~CgWork() {
    for (double *v : {r, z, p, q, dinv, partial, sc})
      if (v) cudaFree(v);
  }
};
}  // namespace

int cg_solve(int64_t n, const int32_t *rp, const int32_t *col, const double *val, const double *b, double *x,
             double rtol, int maxit, cudaStream_t s, int n_sm, int *iters, double *relres, int64_t *launches) {
  CgWork w;
  const size_t bytes = sizeof(double) * (size_t)n;
  if (cudaMalloc(&w.r, bytes) || cudaMalloc(&w.z, bytes) || cudaMalloc(&w.p, bytes) || cudaMalloc(&w.q, bytes) ||
      cudaMalloc(&w.dinv, bytes) || cudaMalloc(&w.partial, sizeof(double) * 2 * RBLK) ||
      cudaMalloc(&w.sc, sizeof(double) * 8))
    return 7;
  double *r = w.r, *z = w.z, *p = w.p, *q = w.q, *dinv = w.dinv, *partial = w.partial, *sc = w.sc;
  cudaMemsetAsync(sc, 0, sizeof(double) * 8, s);  // sc[4] holds the two block counters
  unsigned int *cnt = reinterpret_cast<unsigned int *>(sc + 4);
  const int g1 = n_sm * 8, gs = n_sm * 64;
  int nblk = (int)std::min<int64_t>(RBLK, (n + RT - 1) / RT);
  int64_t L = 0;
  int32_t nnz = 0;
  cudaMemcpyAsync(&nnz, rp + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const int sg = spmv_lanes(n, nnz);
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
  if (!std::isfinite(bnorm)) {  // NaN or Inf in the right-hand side: nothing to iterate on
    *launches += L;
    return cudaStreamSynchronize(s) == cudaSuccess ? 3 : 2;
  }
  if (bnorm == 0.0) {
    *iters = 0;
    *relres = 0.0;
  } else {
    for (it = 0; it < maxit; ++it) {
      cg_iteration(sg, gs, g1, s, n, rp, col, val, x, r, z, p, q, dinv, partial, sc, cnt, it & 1);
      L += 3;
      if ((it + 1) % 16 == 0 || it + 1 == maxit) {
        cudaMemcpyAsync(h, sc + 3, sizeof(double), cudaMemcpyDeviceToHost, s);
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
  return e == cudaSuccess ? 0 : 2;
}

}  // namespace lmg

// ---------------------------------------------------------------------------
// lmg_cg_solve_noalloc: the solve above on caller-owned device arrays, with
// its work vectors in one fixed device array of this file instead of memory
// from cudaMalloc.  Same kernels, same launch shapes, same reduction order,
// so the iterates equal lmg_cg_solve's.
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t NA_DOFS = LMG_CG_NOALLOC_MAX_DOFS;
constexpr int NA_DEVICES = 64;

// r, z, p, q, dinv (NA_DOFS each), the reduction partials (2 RBLK), the scalar slots (8).
// Shared by every call on a device.
static __device__ __align__(256) double g_cg_scratch[5 * NA_DOFS + 2 * lmg::RBLK + 8];

std::mutex g_na_mutex;
double *g_na_base[NA_DEVICES] = {};
int g_na_sm[NA_DEVICES] = {};
unsigned long long g_na_ctx[NA_DEVICES] = {};  // driver context the cached address belongs to

lmg_status na_fail(char *msg, int32_t len, lmg_status code, const char *text) {
  if (msg && len > 0) std::snprintf(msg, (size_t)len, "%s", text);
  return code;
}

// Unique id of the calling thread's current driver context (cuCtxGetId ids
// are never reused, so a context re-created by cudaDeviceReset gets a new one).
// The two driver calls are looked up through the runtime; 0 if unavailable.
unsigned long long na_context_id() {
  using GetCur = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCur get_cur = nullptr;
  static GetId get_id = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = reinterpret_cast<GetCur>(f);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_cur || !get_id || get_cur(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Set-up, with the device current: the array's device address on that device.
// Done on the first call on each device and again whenever the current
// context differs from the one the address was taken in (after
// cudaDeviceReset, or under a context the caller made current); when the
// context id cannot be read, the address is looked up on every call.
cudaError_t na_setup(int dev, double **base, int *n_sm) {
  std::lock_guard<std::mutex> lock(g_na_mutex);
  const unsigned long long ctx = na_context_id();
  if (!g_na_base[dev] || ctx == 0 || ctx != g_na_ctx[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_cg_scratch);
    if (e != cudaSuccess) return e;
    int sm = 0;
    e = cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_na_sm[dev] = sm;
    g_na_base[dev] = static_cast<double *>(p);
    g_na_ctx[dev] = ctx;
  }
  *base = g_na_base[dev];
  *n_sm = g_na_sm[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" lmg_status lmg_cg_solve_noalloc(int64_t n, const int32_t *rp, const int32_t *col, const double *val,
                                           const double *b, double *x, double rtol, int32_t maxit, void *stream,
                                           int32_t *iters, double *relres, char *msg, int32_t msg_len) {
  using namespace lmg;
  na_fail(msg, msg_len, LMG_OK, "");
  if (n <= 0 || !rp || !col || !val || !b || !x || !(rtol > 0.0) || maxit <= 0)
    return na_fail(msg, msg_len, LMG_ERR_ARG, "cg_solve_noalloc: bad argument");
  if (n > NA_DOFS) {
    char t[160];
    std::snprintf(t, sizeof t, "cg_solve_noalloc: n_dofs = %lld exceeds the fixed work space of %lld dofs",
                  (long long)n, (long long)NA_DOFS);
    return na_fail(msg, msg_len, LMG_ERR_ARG, t);
  }
  int dev = 0, n_sm = 0;
  double *base = nullptr;
  if (cudaGetDevice(&dev) != cudaSuccess) return na_fail(msg, msg_len, LMG_ERR_CUDA, "cg_solve_noalloc: no device");
  if (dev >= NA_DEVICES) return na_fail(msg, msg_len, LMG_ERR_ARG, "cg_solve_noalloc: device ordinal too large");
  if (na_setup(dev, &base, &n_sm) != cudaSuccess)
    return na_fail(msg, msg_len, LMG_ERR_CUDA, "cg_solve_noalloc: cudaGetSymbolAddress of the work space failed");
  double *r = base, *z = base + NA_DOFS, *p = base + 2 * NA_DOFS, *q = base + 3 * NA_DOFS,
         *dinv = base + 4 * NA_DOFS, *partial = base + 5 * NA_DOFS, *sc = partial + 2 * RBLK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The scalar slots start every call at zero; every other word is written before it is read.
  if (cudaMemsetAsync(sc, 0, sizeof(double) * 8, s) != cudaSuccess)
    return na_fail(msg, msg_len, LMG_ERR_CUDA, "cg_solve_noalloc: clearing the scalar slots failed");
  const int g1 = n_sm * 8, gs = n_sm * 64;
  const int nblk = (int)std::min<int64_t>(RBLK, (n + RT - 1) / RT);
  int32_t nnz = 0;  // the row pointer's last entry sets the SpMV lane count
  if (cudaMemcpyAsync(&nnz, rp + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return na_fail(msg, msg_len, LMG_ERR_CUDA, "cg_solve_noalloc: reading the row pointer failed");
  const int sg = spmv_lanes(n, nnz);
  k_diag_inv<<<g1, 256, 0, s>>>(n, rp, col, val, dinv);
  k_init<<<g1, 256, 0, s>>>(n, b, x, r, z, p, dinv);
  k_dot2<<<nblk, RT, 0, s>>>(n, r, z, r, r, partial);
  k_dot2_final<<<1, RT, 0, s>>>(nblk, partial, sc);  // sc[0] = rz, sc[1] = rr
  double h[2] = {0.0, 0.0};
  if (cudaMemcpyAsync(h, sc, sizeof(double) * 2, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return na_fail(msg, msg_len, LMG_ERR_CUDA, "cg_solve_noalloc: device failure");
  const double bnorm = std::sqrt(h[1]);
  double rn = bnorm;
  int it = 0;
  if (!std::isfinite(bnorm))  // the same status lmg_cg_solve returns
    return na_fail(msg, msg_len, LMG_ERR_ARG, "cg_solve_noalloc: the right-hand side is not finite");
  if (bnorm > 0.0) {
    unsigned int *cnt = reinterpret_cast<unsigned int *>(sc + 4);  // cleared with the scalar slots
    for (it = 0; it < maxit; ++it) {
      cg_iteration(sg, gs, g1, s, n, rp, col, val, x, r, z, p, q, dinv, partial, sc, cnt, it & 1);
      if ((it + 1) % 16 == 0 || it + 1 == maxit) {
        if (cudaMemcpyAsync(h, sc + 3, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
          return na_fail(msg, msg_len, LMG_ERR_CUDA, "cg_solve_noalloc: device failure");
        rn = std::sqrt(h[0]);
        if (!(rn > rtol * bnorm)) { ++it; break; }
      }
    }
  }
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
    return na_fail(msg, msg_len, LMG_ERR_CUDA, "cg_solve_noalloc: device failure");
  if (iters) *iters = it;
  if (relres) *relres = bnorm > 0.0 ? rn / bnorm : 0.0;
  return LMG_OK;
}
