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

#include "assemble.cuh"
#include "df.cuh"
#include "row_load.cuh"

namespace lmg {

namespace {

template <int BS>
__device__ __forceinline__ void row_load(const GatherArgs &g, int64_t P, int lane) {
  row_load_f<BS>(g.fptr, g.fcontrib, g.Fe2, g.F, P, lane);
}

// Contributions of one block slot to one entry, summed in double-float in
// element order; four predicated loads in flight per step.
template <int B2, typename TV>
__device__ __forceinline__ DF slot_sum(const GatherArgs &g, const TV *Kb, int32_t c0, int32_t c1, int rem, int tr,
                                       bool coded) {
  DF s = {0.f, 0.f};
  for (int32_t c = c0; c < c1; c += 4) {
    int32_t x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = (c + u < c1) ? __ldg(g.bcontrib + c + u) : -1;
    TV v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      int64_t idx = 0;
      if (x[u] >= 0) idx = coded ? (int64_t)(x[u] >> 1) * B2 + ((x[u] & 1) ? tr : rem) : (int64_t)x[u] * B2 + rem;
      v[u] = (x[u] >= 0) ? __ldg(Kb + idx) : TV{};
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (x[u] >= 0) {
        if constexpr (sizeof(TV) == 8) s = df_add(s, DF{((const float2 &)v[u]).x, ((const float2 &)v[u]).y});
        else s = df_add1(s, (const float &)v[u]);
      }
  }
  return s;
}

// FP64 drop-in insertion, warp per block row P.  Lane l < (32/B2)*B2 owns entry
// rem = l % B2 of the slots jj = l / B2 + (32/B2) t, so the B2 values of one
// stored element block are read by B2 neighbouring lanes as one chunk.  Every
// slot of the row is summed (a lower slot reads the stored upper element block
// transposed), so each row of K is written contiguously: writing the upper
// values into their transposed slots instead scatters 8-byte stores over other
// rows and measured slower.  Both forms are symmetric and a slot and its
// transpose sum the same entries in the same element order, so K_QP = K_PQ^T bit
// for bit.  Each value is the sum, in element order, of the double-float
// element entries that land on it, rounded once to FP64.
template <int BS>
__global__ void __launch_bounds__(256) k_gather(GatherArgs g) {
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
    for (int jj = js; act && jj < deg; jj += SPL) {
      const int64_t j = rb + jj;
      const int32_t Q = g.bcol[j];
      const int32_t c0 = g.bptr[j], c1 = g.bptr[j + 1];
      const bool diag = Q == (int32_t)P;
      const DF s = diag ? slot_sum<B2>(g, g.Kdiag2, c0, c1, rem, rem, false)
                        : slot_sum<B2>(g, g.Koff2, c0, c1, rem, tr, true);
      g.K[rowp + jj * BS + k] = df_to_double(s);
    }
    row_load<BS>(g, P, lane);
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
    row_load<BS>(g, P, lane);
  }
}

// Load vector only (QoI derivative): warp per block row, F from the element loads.
template <int BS>
__global__ void __launch_bounds__(256) k_gather_f(GatherArgs g) {
  const int lane = threadIdx.x & 31;
  for (int64_t P = g.row_begin + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); P < g.row_end;
       P += ((int64_t)gridDim.x * blockDim.x) >> 5)
    row_load<BS>(g, P, lane);
}

}  // namespace

void launch_gather_f(const GatherArgs &g0, cudaStream_t s) {
  GatherArgs g = g0;
  if (g.row_end == 0) g.row_end = g.n_dofs / g.bs;
  int dev = 0, n_sm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  int64_t blocks = (g.n_dofs / g.bs + 7) / 8;
  if (blocks > (int64_t)n_sm * 16) blocks = (int64_t)n_sm * 16;
  if (blocks < 1) blocks = 1;
  if (g.bs == 1) k_gather_f<1><<<(int)blocks, 256, 0, s>>>(g);
  else if (g.bs == 3) k_gather_f<3><<<(int)blocks, 256, 0, s>>>(g);
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
  } else {
    if (g.bs == 1) k_gather<1><<<(int)blocks, 256, 0, s>>>(g);
    else if (g.bs == 3) k_gather<3><<<(int)blocks, 256, 0, s>>>(g);
  }
}

}  // namespace lmg
