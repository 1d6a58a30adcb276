// Global insertion without floating-point atomics.
//
// libMesh adds each element block into the PETSc matrix in element order
// (SparseMatrix::add_matrix -> MatSetValues(ADD_VALUES), src/numerics/petsc_matrix.C:735-755;
// NumericVector::add_vector, src/numerics/petsc_vector.C:174-195), so every CSR
// value is ((0 + c_e1) + c_e2) + ... over the elements touching it, in element
// order.  Here the scatter is inverted into a gather: the plan lists, for every
// block slot of the CSR, the element blocks that land on it in ascending element
// order, and one warp per block row sums them.  The result is deterministic and
// the summation order is the reference's.
//
// Lanes walk the bs*bs values of consecutive block slots, so the bs*bs values of
// one stored element block are read by bs*bs neighbouring lanes (one contiguous
// chunk); each lane loads its contribution indices four at a time before
// summing, to keep several independent loads in flight.  Sums run in
// double-float (df.cuh) on the FP32 pipe; GB300's FP64 pipe would otherwise
// bound this memory-streaming kernel.
#include <cuda_runtime.h>

#include <algorithm>

#include "assemble.cuh"
#include "df.cuh"

namespace lmg {

namespace {

// Load vector F: thread per block row, the element entries of each of its BS
// dofs summed in element order (NumericVector::add_vector's order over the
// elements, src/numerics/petsc_vector.C:174-195) in double-float from the
// first term on, rounded once to FP64.  One kernel for every insertion (FP64,
// mixed, fused, QoI load), so the forms give the same F bit for bit.
template <int BS>
__global__ void __launch_bounds__(256) k_load_vec(int64_t r0, int64_t r1, const int32_t *fptr,
                                                  const int32_t *fcontrib, const float2 *Fe2, double *F) {
  for (int64_t P = r0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; P < r1;
       P += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c0 = fptr[P], c1 = fptr[P + 1];
    DFAcc s[BS];
#pragma unroll
    for (int q = 0; q < BS; ++q) s[q] = {0.f, 0.f};
    int32_t c = c0;
    for (; c + 1 < c1; c += 2) {  // two incidences' loads in flight
      const int64_t b0 = (int64_t)__ldg(fcontrib + c) * BS, b1 = (int64_t)__ldg(fcontrib + c + 1) * BS;
      float2 v0[BS], v1[BS];
#pragma unroll
      for (int q = 0; q < BS; ++q) {
        v0[q] = __ldg(Fe2 + b0 + q);
        v1[q] = __ldg(Fe2 + b1 + q);
      }
#pragma unroll
      for (int q = 0; q < BS; ++q) {
        acc_add(s[q], v0[q]);
        acc_add(s[q], v1[q]);
      }
    }
    if (c < c1) {
      const int64_t b0 = (int64_t)__ldg(fcontrib + c) * BS;
#pragma unroll
      for (int q = 0; q < BS; ++q) acc_add(s[q], __ldg(Fe2 + b0 + q));
    }
#pragma unroll
    for (int q = 0; q < BS; ++q) F[BS * P + q] = f2d(s[q].hi) + f2d(s[q].lo);
  }
}


// FP64 drop-in insertion, warp per block row P.  Lane l < (32/BS)*BS owns row
// i = l % BS of the slots jj = l / BS + (32/BS) t, i.e. the BS entries
// K[BS P + i][BS Q + k], k < BS: one decoded contribution index serves BS
// loads, and the row's values are written contiguously.  Every slot of the row
// is summed (a lower slot reads the stored upper element block transposed), so
// each row of K is written contiguously: writing the upper values into their
// transposed slots instead scatters 8-byte stores over other rows and measured
// slower.  Both forms are symmetric and a slot and its transpose sum the same
// entries in the same element order, so K_QP = K_PQ^T bit for bit.  Each value
// is the double-float sum, in element order, of the double-float element
// entries that land on it, rounded once to FP64.
//
// The row's plan is staged in shared memory first (slot offsets, then the
// contribution indices, each one coalesced load), so that the element-block
// loads of all its slots are independent of one another; rows larger than the
// staging buffers read the plan from global memory (same sums).  The load
// vector's first 32 contributions are fetched before the slots.
constexpr int GW = 8;      // warps per CTA
constexpr int RG = 4;      // consecutive block rows per warp step (their plans are contiguous)
constexpr int DCAP = 192;  // staged slots per warp step
constexpr int CCAP = 768;  // staged contributions per warp step

// Slots jj = js, js + SPI, ... of block row P; `ptr[jj]` is the slot's first
// contribution relative to `con`.
template <int BS>
__device__ __forceinline__ void row_slots(const GatherArgs &g, const int32_t *ptr, const int32_t *con, int deg,
                                          int jdiag, int js, int i, int32_t rowp) {
  constexpr int B2 = BS * BS, SPI = 32 / BS;
  for (int jj = js; jj < deg; jj += SPI) {
    const int32_t a0 = ptr[jj], a1 = ptr[jj + 1];
    const bool diag = jj == jdiag;
    const float2 *Kp = diag ? g.Kdiag2 : g.Koff2;
    DFAcc s[BS];
#pragma unroll
    for (int k = 0; k < BS; ++k) s[k] = {0.f, 0.f};
    if (a0 < a1) {  // the first term starts the sum
      const int32_t x = con[a0];
      const int64_t b = diag ? (int64_t)x * B2 : (int64_t)(x >> 1) * B2;
      const bool t = !diag && (x & 1);
#pragma unroll
      for (int k = 0; k < BS; ++k) {
        const float2 v = __ldg(Kp + b + (t ? k * BS + i : i * BS + k));
        s[k] = {v.x, v.y};
      }
    }
    for (int32_t u = a0 + 1; u < a1; u += 2) {
      const bool two = u + 1 < a1;
      const int32_t x0 = con[u], x1 = two ? con[u + 1] : x0;
      // diagonal slots list e*nb + a (no transpose), the others 2*(e*no + o) + t
      const int64_t b0 = diag ? (int64_t)x0 * B2 : (int64_t)(x0 >> 1) * B2;
      const int64_t b1 = diag ? (int64_t)x1 * B2 : (int64_t)(x1 >> 1) * B2;
      const bool t0 = !diag && (x0 & 1), t1 = !diag && (x1 & 1);
      float2 v0[BS], v1[BS];
#pragma unroll
      for (int k = 0; k < BS; ++k) {
        v0[k] = __ldg(Kp + b0 + (t0 ? k * BS + i : i * BS + k));
        v1[k] = two ? __ldg(Kp + b1 + (t1 ? k * BS + i : i * BS + k)) : float2{0.f, 0.f};
      }
#pragma unroll
      for (int k = 0; k < BS; ++k) {
        acc_add(s[k], v0[k]);
        if (two) acc_add(s[k], v1[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < BS; ++k) g.K[rowp + jj * BS + k] = f2d(s[k].hi) + f2d(s[k].lo);
  }
}

template <int BS>
__global__ void __launch_bounds__(GW * 32, 6) k_gather(GatherArgs g) {
  constexpr int SPI = 32 / BS;
  __shared__ int32_t s_ptr[GW][DCAP + 1];
  __shared__ int32_t s_con[GW][CCAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int js = lane / BS, i = lane - js * BS;
  const bool act = lane < SPI * BS;
  int32_t *sp = s_ptr[warp], *sc = s_con[warp];
  // A warp takes RG consecutive block rows at a time: their slot offsets and
  // contribution lists are contiguous, so one round of loads stages all of
  // them; the rows' sums then read the plan from shared memory.  A step whose
  // plan outgrows the buffers reads it from global memory (same sums).
  for (int64_t P0 = g.row_begin + ((int64_t)blockIdx.x * GW + warp) * RG; P0 < g.row_end;
       P0 += (int64_t)gridDim.x * GW * RG) {
    const int nr = (int)(g.row_end - P0 < RG ? g.row_end - P0 : RG);
    const int64_t hb = lane <= nr ? g.brow_ptr[P0 + lane] : 0;  // the step's row offsets
    const int32_t hd = (g.bdiag && lane < nr) ? g.bdiag[P0 + lane] : -1;  // and diagonal slots
    const int64_t rb0 = __shfl_sync(0xffffffffu, hb, 0), rbn = __shfl_sync(0xffffffffu, hb, nr);
    const int ns = (int)(rbn - rb0);
    bool staged = false;
    if (ns <= DCAP) {
      for (int t = lane; t <= ns; t += 32) sp[t] = __ldg(g.bptr + rb0 + t);
      __syncwarp();
      const int32_t cb = sp[0], nc = sp[ns] - cb;
      __syncwarp();  // every lane has read cb before sp is rebased
      if (nc <= CCAP) {
        staged = true;
        for (int t = lane; t < nc; t += 32) sc[t] = __ldg(g.bcontrib + cb + t);
        for (int t = lane; t <= ns; t += 32) sp[t] -= cb;
      }
      __syncwarp();
    }
    for (int r = 0; r < nr; ++r) {
      const int64_t P = P0 + r;
      const int64_t rb = __shfl_sync(0xffffffffu, hb, r);
      const int deg = (int)(__shfl_sync(0xffffffffu, hb, r + 1) - rb);
      // dof row BS P + i of the block CSR starts at BS^2 brow_ptr[P] + i BS deg
      const int32_t rowp = act ? (int32_t)(BS * BS * rb + (int64_t)i * BS * deg) : 0;
      int jdiag = __shfl_sync(0xffffffffu, hd, r);
      if (!g.bdiag) {
        for (int t = lane; t < deg; t += 32)
          if (g.bcol[rb + t] == (int32_t)P) jdiag = t;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) jdiag = max(jdiag, __shfl_xor_sync(0xffffffffu, jdiag, o));
      }
      if (act) {
        if (staged) row_slots<BS>(g, sp + (rb - rb0), sc, deg, jdiag, js, i, rowp);
        else row_slots<BS>(g, g.bptr + rb, g.bcontrib, deg, jdiag, js, i, rowp);
      }
    }
    __syncwarp();  // the step's plan is read before the next step stages its own
  }
}

// Mixed insertion, warp per block row P, same lane layout.  Off-diagonal
// entries: FP32 contributions summed in FP32 in element order, masked by the
// Dirichlet rows and columns.  Diagonal blocks: minus the double-float sum of
// the row's stored (unmasked) off-diagonal entries, so K t = 0 holds to FP64
// roundoff for every rigid translation t on unconstrained rows; a constrained
// dof gets the reference's value (one 1 per element touching it).
template <int BS>
__global__ void __launch_bounds__(256) k_gather_mixed(GatherArgs g) {
  constexpr int B2 = BS * BS, SPL = 32 / B2;
  const int lane = threadIdx.x & 31;
  const int js = lane / B2, rem = lane - js * B2;
  const bool act = lane < SPL * B2;
  const int i = rem / BS, k = rem - i * BS, tr = k * BS + i;
  for (int64_t P = g.row_begin + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); P < g.row_end;
       P += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t rb = g.brow_ptr[P];
    const int deg = (int)(g.brow_ptr[P + 1] - rb);
    const int32_t rowp = act ? g.row_ptr[BS * P + i] : 0;
    const bool rc = act && g.constrained[BS * P + i] != 0;
    DF acc = {0.f, 0.f};
    int jdiag = -1;
    for (int jj = js; act && jj < deg; jj += SPL) {
      const int64_t j = rb + jj;
      const int32_t Q = g.bcol[j];
      if (Q == (int32_t)P) { jdiag = jj; continue; }
      // FP32 sum of the FP32 contributions, in element order (32-bit offsets:
      // the plan guarantees n_contributions * bs^2 < 2^31)
      const int32_t c0 = g.bptr[j], c1 = g.bptr[j + 1];
      float kv = 0.f;
      for (int32_t c = c0; c < c1; c += 4) {
        float v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int32_t x = (c + u < c1) ? __ldg(g.bcontrib + c + u) : -1;
          v[u] = (x >= 0) ? __ldg(g.Koff32 + (x >> 1) * B2 + ((x & 1) ? tr : rem)) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (c + u < c1) kv = __fadd_rn(kv, v[u]);
      }
      acc = df_add1(acc, kv);  // row sums stay double-float over the stored entries
      const bool masked = rc || g.constrained[(int64_t)BS * Q + k] != 0;
      g.K[rowp + jj * BS + k] = masked ? 0.0 : f2d(kv);
    }
    // row sums: lanes rem, rem + B2, ... hold partial sums of the same entry
    if constexpr (B2 == 1) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        DF y;
        y.hi = __shfl_xor_sync(0xffffffffu, acc.hi, o);
        y.lo = __shfl_xor_sync(0xffffffffu, acc.lo, o);
        acc = (lane & o) ? df_add(y, acc) : df_add(acc, y);
      }
    } else {
#pragma unroll
      for (int t = 1; t < SPL; ++t) {
        DF y;
        y.hi = __shfl_sync(0xffffffffu, acc.hi, (lane + t * B2) & 31);
        y.lo = __shfl_sync(0xffffffffu, acc.lo, (lane + t * B2) & 31);
        if (lane < B2) acc = df_add(acc, y);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) jdiag = max(jdiag, __shfl_xor_sync(0xffffffffu, jdiag, o));
    if (lane < B2 && jdiag >= 0) {
      double v = -(f2d(acc.hi) + f2d(acc.lo));
      if (rc || g.constrained[BS * P + k] != 0) {
        const int64_t j = rb + jdiag;
        v = (i == k) ? (double)(g.bptr[j + 1] - g.bptr[j]) : 0.0;
      }
      g.K[rowp + jdiag * BS + k] = v;
    }
  }
}

}  // namespace

void launch_load_vec(int bs, int64_t r0, int64_t r1, const int32_t *fptr, const int32_t *fcontrib,
                     const float2 *Fe2, double *F, cudaStream_t s) {
  if (r1 <= r0) return;
  int dev = 0, n_sm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  int64_t blocks = (r1 - r0 + 255) / 256;
  if (blocks > (int64_t)n_sm * 16) blocks = (int64_t)n_sm * 16;
  if (bs == 1) k_load_vec<1><<<(int)blocks, 256, 0, s>>>(r0, r1, fptr, fcontrib, Fe2, F);
  else if (bs == 3) k_load_vec<3><<<(int)blocks, 256, 0, s>>>(r0, r1, fptr, fcontrib, Fe2, F);
}

void launch_gather_f(const GatherArgs &g, cudaStream_t s) {
  launch_load_vec(g.bs, g.row_begin, g.row_end ? g.row_end : g.n_dofs / g.bs, g.fptr, g.fcontrib, g.Fe2, g.F, s);
}

bool gather_built(int bs) { return bs == 1 || bs == 3; }

void launch_gather(const GatherArgs &g0, bool mixed, cudaStream_t s) {
  GatherArgs g = g0;
  if (g.row_end == 0) g.row_end = g.n_dofs / g.bs;
  int dev = 0, n_sm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t warps = g.row_end - g.row_begin;
  int64_t blocks = (warps + 7) / 8;
  const int64_t cap = (int64_t)n_sm * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (mixed) {
    if (g.bs == 1) k_gather_mixed<1><<<(int)blocks, 256, 0, s>>>(g);
    else if (g.bs == 3) k_gather_mixed<3><<<(int)blocks, 256, 0, s>>>(g);
  } else {  // persistent: every resident warp walks block rows P, P + all warps, ...
    int per_sm = 1;
    if (g.bs == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather<1>, GW * 32, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather<3>, GW * 32, 0);
    const int64_t rows = std::min<int64_t>((warps + GW * RG - 1) / (GW * RG), (int64_t)n_sm * std::max(per_sm, 1));
    if (g.bs == 1) k_gather<1><<<(unsigned)rows, GW * 32, 0, s>>>(g);
    else if (g.bs == 3) k_gather<3><<<(unsigned)rows, GW * 32, 0, s>>>(g);
  }
  launch_load_vec(g.bs, g.row_begin, g.row_end, g.fptr, g.fcontrib, g.Fe2, g.F, s);
}

}  // namespace lmg
