// Global insertion without floating-point atomics.
//
// libMesh adds each element block into the PETSc matrix in element order
// (SparseMatrix::add_matrix -> MatSetValues(ADD_VALUES), src/numerics/petsc_matrix.C:735-755;
// NumericVector::add_vector, src/numerics/petsc_vector.C:174-195), so every CSR
// value is ((0 + c_e1) + c_e2) + ... over the elements touching it, in element
// order.  Here the scatter is inverted into a gather: the plan lists, for every
// block slot of the CSR, the element blocks that land on it in ascending element
// order, and one warp per CSR row sums them.  The result is deterministic and
// the summation order is the reference's.
#include <cuda_runtime.h>

#include "assemble.cuh"

namespace lmg {

namespace {

template <typename KT>
__global__ void __launch_bounds__(256) k_gather(GatherArgs g, const KT *Ke) {
  const int lane = threadIdx.x & 31;
  const int bs = g.bs, bs2 = g.bs * g.bs;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < g.n_dofs;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t P = r / bs;
    const int i = (int)(r - P * bs);
    const int64_t rb = g.brow_ptr[P];
    const int64_t len = (g.brow_ptr[P + 1] - rb) * bs;
    double *out = g.K + g.row_ptr[r];
    for (int64_t m = lane; m < len; m += 32) {
      const int64_t j = rb + m / bs;
      const int k = (int)(m % bs);
      const int32_t c0 = g.bptr[j], c1 = g.bptr[j + 1];
      double s = 0.0;
      for (int32_t c = c0; c < c1; ++c) s += (double)Ke[(int64_t)g.bcontrib[c] * bs2 + i * bs + k];
      out[m] = s;
    }
    if (lane == 0) {
      double s = 0.0;
      for (int32_t c = g.fptr[P]; c < g.fptr[P + 1]; ++c) s += g.Fe[(int64_t)g.fcontrib[c] * bs + i];
      g.F[r] = s;
    }
  }
}

}  // namespace

void launch_gather(const GatherArgs &g, bool mixed, cudaStream_t s) {
  int dev = 0, n_sm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t warps = g.n_dofs;
  int64_t blocks = (warps + 7) / 8;
  const int64_t cap = (int64_t)n_sm * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (mixed)
    k_gather<float><<<(int)blocks, 256, 0, s>>>(g, g.Ke32);
  else
    k_gather<double><<<(int)blocks, 256, 0, s>>>(g, g.Ke);
}

}  // namespace lmg
