// Global insertion without floating-point atomics.
//
// libMesh adds each element block into the PETSc matrix in element order
// (SparseMatrix::add_matrix -> MatSetValues(ADD_VALUES), src/numerics/petsc_matrix.C:735-755;
// NumericVector::add_vector, src/numerics/petsc_vector.C:174-195), so every CSR
// value is ((0 + c_e1) + c_e2) + ... over the elements touching it, in element
// order.  Here the scatter is inverted into a gather: the element kernels
// write every stored element block into the slot-ordered store, where the
// contributions of each block slot of the upper triangle lie contiguous and
// in element order, and one warp per block row sums the runs of its slots (a
// slot below the diagonal reads its mirror's run transposed).  The result is
// deterministic and the summation order is the reference's.
//
// Lanes own the bs*bs entries of consecutive slots, so the bs*bs values of
// one stored block are read by bs*bs neighbouring lanes (one contiguous
// chunk) and consecutive contributions of a slot are consecutive chunks.
// Sums run in double-float (df.cuh) on the FP32 pipe; GB300's FP64 pipe
// would otherwise bound this memory-streaming kernel.
#include <cuda_runtime.h>

#include <algorithm>

#include "assemble.cuh"
#include "df.cuh"
#include "row_load.cuh"

namespace lmg {

namespace {

template <int BS>
__device__ __forceinline__ void row_load(const GatherArgs &g, int64_t P, int lane) {
  row_load_f<BS>(g.fptr, g.fcontrib, g.Fe2, g.F, P, lane);
}

// Running double-float sum of double-float terms: TwoSum on the high parts,
// the rounding error and the low parts collected in `lo` (normalised only when
// the sum is rounded to FP64), 8 FP32 operations per term.
struct DFAcc {
  float hi, lo;
};

__device__ __forceinline__ void acc_add(DFAcc &a, float2 v) {
  const float s = __fadd_rn(a.hi, v.x);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(v.x, bb));
  a.lo = __fadd_rn(a.lo, __fadd_rn(e, v.y));
  a.hi = s;
}

// FP64 drop-in insertion, warp per block row P (persistent grid).  Lane
// l < (32/B2)*B2 owns entry (i, k) of the slots jj = l / B2 + (32/B2) t: it
// sums that entry over the slot's run in element order (the first term starts
// the sum, four loads in flight), in double-float, and writes
// K[BS P + i][BS Q + k] rounded once to FP64.  Every row of K is written
// contiguously; a slot and its transpose sum the same entries in the same
// order, so K_QP = K_PQ^T bit for bit.
template <int BS>
__global__ void __launch_bounds__(256) k_gather(GatherArgs g) {
  constexpr int B2 = BS * BS, SPL = 32 / B2;
  const int lane = threadIdx.x & 31;
  const int js = lane / B2, rem = lane - js * B2;
  const bool act = lane < SPL * B2;
  const int i = rem / BS, k = rem - i * BS, trn = k * BS + i;
  for (int64_t P = g.row_begin + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); P < g.row_end;
       P += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t rb = g.brow_ptr[P];
    const int deg = (int)(g.brow_ptr[P + 1] - rb);
    const int32_t rowp = act ? g.row_ptr[BS * P + i] : 0;
    for (int jj = js; act && jj < deg; jj += SPL) {
      const int2 r = __ldg(g.srange + rb + jj);
      const int cnt = r.y & 0x7fffffff;
      const float2 *src = g.Kso + (int64_t)r.x * B2 + (r.y < 0 ? trn : rem);
      DFAcc s = {0.f, 0.f};
      if (cnt > 0) {
        const float2 v = __ldg(src);
        s = {v.x, v.y};
      }
      int c = 1;
      for (; c + 3 < cnt; c += 4) {
        const float2 v0 = __ldg(src + (int64_t)c * B2), v1 = __ldg(src + (int64_t)(c + 1) * B2);
        const float2 v2 = __ldg(src + (int64_t)(c + 2) * B2), v3 = __ldg(src + (int64_t)(c + 3) * B2);
        acc_add(s, v0);
        acc_add(s, v1);
        acc_add(s, v2);
        acc_add(s, v3);
      }
      for (; c < cnt; ++c) acc_add(s, __ldg(src + (int64_t)c * B2));
      g.K[rowp + jj * BS + k] = f2d(s.hi) + f2d(s.lo);
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
      // FP32 sum of the FP32 contributions, in element order
      const int2 r = __ldg(g.srange + j);
      const int cnt = r.y & 0x7fffffff;
      const float *src = g.Kso32 + (int64_t)r.x * B2 + (r.y < 0 ? tr : rem);
      float kv = 0.f;
      int c = 0;
      for (; c + 3 < cnt; c += 4) {
        const float v0 = __ldg(src + (int64_t)c * B2), v1 = __ldg(src + (int64_t)(c + 1) * B2);
        const float v2 = __ldg(src + (int64_t)(c + 2) * B2), v3 = __ldg(src + (int64_t)(c + 3) * B2);
        kv = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(kv, v0), v1), v2), v3);
      }
      for (; c < cnt; ++c) kv = __fadd_rn(kv, __ldg(src + (int64_t)c * B2));
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
  } else {  // persistent: every resident warp walks block rows P, P + all warps, ...
    int per_sm = 1;
    if (g.bs == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather<1>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather<3>, 256, 0);
    const int64_t rows = std::min<int64_t>((warps + 7) / 8, (int64_t)n_sm * std::max(per_sm, 1));
    if (g.bs == 1) k_gather<1><<<(unsigned)rows, 256, 0, s>>>(g);
    else if (g.bs == 3) k_gather<3><<<(unsigned)rows, 256, 0, s>>>(g);
  }
}

}  // namespace lmg
