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
// summing, to keep several independent loads in flight.
#include <cuda_runtime.h>

#include "assemble.cuh"

namespace lmg {

namespace {

template <typename TO, int BS>
__global__ void __launch_bounds__(256) k_gather(GatherArgs g, const TO *Koff) {
  constexpr int B2 = BS * BS;
  const int lane = threadIdx.x & 31;
  const int64_t n_brows = g.n_dofs / BS;
  for (int64_t P = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; P < n_brows;
       P += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t rb = g.brow_ptr[P];
    const int deg = (int)(g.brow_ptr[P + 1] - rb);
    const int total = deg * B2;
    int32_t rowp[BS];
#pragma unroll
    for (int i = 0; i < BS; ++i) rowp[i] = g.row_ptr[BS * P + i];
    for (int m = lane; m < total; m += 32) {
      const int jj = m / B2, rem = m - jj * B2;
      const int i = rem / BS, k = rem - i * BS;
      const int64_t j = rb + jj;
      const int32_t c0 = g.bptr[j], c1 = g.bptr[j + 1];
      double s = 0.0;
      if (g.bcol[j] == (int32_t)P) {
        for (int32_t c = c0; c < c1; ++c) s += g.Kdiag[(int64_t)g.bcontrib[c] * B2 + rem];
      } else {
        const int tr = k * BS + i;
        int32_t c = c0;
        for (; c + 4 <= c1; c += 4) {
          int32_t x[4];
          double v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) x[u] = g.bcontrib[c + u];
#pragma unroll
          for (int u = 0; u < 4; ++u) v[u] = (double)Koff[(int64_t)(x[u] >> 1) * B2 + ((x[u] & 1) ? tr : rem)];
#pragma unroll
          for (int u = 0; u < 4; ++u) s += v[u];
        }
        for (; c < c1; ++c) {
          const int32_t x = g.bcontrib[c];
          s += (double)Koff[(int64_t)(x >> 1) * B2 + ((x & 1) ? tr : rem)];
        }
      }
      g.K[rowp[i] + jj * BS + k] = s;
    }
    if (lane < BS) {
      double s = 0.0;
      for (int32_t c = g.fptr[P]; c < g.fptr[P + 1]; ++c) s += g.Fe[(int64_t)g.fcontrib[c] * BS + lane];
      g.F[BS * P + lane] = s;
    }
  }
}

template <typename TO>
void launch_bs(const GatherArgs &g, const TO *Koff, cudaStream_t s, int blocks) {
  switch (g.bs) {
    case 1: k_gather<TO, 1><<<blocks, 256, 0, s>>>(g, Koff); break;
    case 3: k_gather<TO, 3><<<blocks, 256, 0, s>>>(g, Koff); break;
    default: break;
  }
}

}  // namespace

bool gather_built(int bs) { return bs == 1 || bs == 3; }

void launch_gather(const GatherArgs &g, bool mixed, cudaStream_t s) {
  int dev = 0, n_sm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t warps = g.n_dofs / g.bs;
  int64_t blocks = (warps + 7) / 8;
  const int64_t cap = (int64_t)n_sm * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (mixed) launch_bs<float>(g, g.Koff32, s, (int)blocks);
  else launch_bs<double>(g, g.Koff, s, (int)blocks);
}

}  // namespace lmg
