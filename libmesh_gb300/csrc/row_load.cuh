// Load vector of one block row: row_load_seq (element order: the mixed
// insertions, the fused row kernel) and row_load_f (a butterfly over the
// warp: the matrix-free residual's per-dof sums).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "df.cuh"

namespace lmg {

// Load vector of block row P: the element entries that land on each of its bs
// dofs, summed in double-float by a fixed butterfly over the warp (lane l takes
// contributions l, l+32, ... in element order), rounded once to FP64.
template <int BS>
__device__ __forceinline__ void row_load_f(const int32_t *fptr, const int32_t *fcontrib, const float2 *Fe2, double *F,
                                           int64_t P, int lane) {
  const int32_t f0 = fptr[P], f1 = fptr[P + 1];
  DF s[BS];
#pragma unroll
  for (int i = 0; i < BS; ++i) s[i] = {0.f, 0.f};
  for (int32_t c = f0 + lane; c < f1; c += 32) {
    const int64_t base = (int64_t)fcontrib[c] * BS;
#pragma unroll
    for (int i = 0; i < BS; ++i) {
      const float2 v = Fe2[base + i];
      s[i] = df_add(s[i], DF{v.x, v.y});
    }
  }
#pragma unroll
  for (int i = 0; i < BS; ++i)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      DF y;
      y.hi = __shfl_xor_sync(0xffffffffu, s[i].hi, o);
      y.lo = __shfl_xor_sync(0xffffffffu, s[i].lo, o);
      s[i] = (lane & o) ? df_add(y, s[i]) : df_add(s[i], y);
    }
  if (lane < BS) {
    DF r = s[0];
#pragma unroll
    for (int i = 1; i < BS; ++i)
      if (lane == i) r = s[i];
    F[BS * P + lane] = df_to_double(r);
  }
}

// Load vector of block row P in element order: lane i < BS sums the element
// entries of dof BS P + i one after the other (the order of
// NumericVector::add_vector over the elements, src/numerics/petsc_vector.C:174-195)
// in double-float, rounded once to FP64.
template <int BS>
__device__ __forceinline__ void row_load_seq(const int32_t *fptr, const int32_t *fcontrib, const float2 *Fe2,
                                             double *F, int64_t P, int lane) {
  if (lane >= BS) return;
  const int32_t f0 = fptr[P], f1 = fptr[P + 1];
  DFAcc s = {0.f, 0.f};
  int32_t c = f0;
  for (; c + 1 < f1; c += 2) {  // two loads in flight
    const float2 v0 = __ldg(Fe2 + (int64_t)__ldg(fcontrib + c) * BS + lane);
    const float2 v1 = __ldg(Fe2 + (int64_t)__ldg(fcontrib + c + 1) * BS + lane);
    acc_add(s, v0);
    acc_add(s, v1);
  }
  if (c < f1) acc_add(s, __ldg(Fe2 + (int64_t)__ldg(fcontrib + c) * BS + lane));
  F[BS * P + lane] = f2d(s.hi) + f2d(s.lo);
}

}  // namespace lmg
