// Per-dof sums of element vectors over one block row by a butterfly over the
// warp: the matrix-free residual's R (the assembled load vector F is summed
// in element order by the insertions' k_load_vec, gather.cu).
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

}  // namespace lmg
