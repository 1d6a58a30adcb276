// Double-float arithmetic: a value is an unevaluated sum hi + lo of two FP32
// numbers (|lo| <= ulp(hi)/2), which carries a 48-bit significand.  GB300 runs
// FP32 at 64x its FP64 rate, so the assembly contractions and sums run here on
// the FP32 pipe while keeping FP64-level accuracy (~2^-46 relative per
// operation).  The algorithms are the classical error-free transformations:
// Knuth's TwoSum, Dekker's FastTwoSum and the FMA-based TwoProduct
// (Ogita, Rump, Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 2005).
// Every step uses the _rn intrinsics so that nothing is contracted or
// reassociated by the compiler.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace lmg {

struct DF {
  float hi, lo;
};

__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ DF fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DF df_add(DF x, DF y) {
  const DF s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ DF df_add1(DF x, float y) {
  const DF s = two_sum(x.hi, y);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, x.lo));
}

// acc + a*b with the product's rounding error and cross terms folded into
// acc.lo; the caller renormalises once at the end of a short dot product.
__device__ __forceinline__ DF df_fma_lazy(DF acc, DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const DF s = two_sum(acc.hi, p);
  return {s.hi, __fadd_rn(acc.lo, __fadd_rn(s.lo, e))};
}

__device__ __forceinline__ DF df_norm(DF x) { return fast_two_sum(x.hi, x.lo); }

// Running double-float sum of double-float terms: TwoSum on the high parts,
// the rounding error and the low parts collected in `lo` (normalised only when
// the sum is rounded to FP64), 7 FP32 operations per term.  From {0, 0} the
// first term is taken exactly.
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

// Exact float -> double by moving the bits (keeps the FP64 pipe free); zero,
// subnormal, inf and NaN take the hardware conversion.  (An integer-only
// version that also normalises subnormals measured slower in the insertion
// kernels: more instructions on every call for a case that does not occur.)
__device__ __forceinline__ double f2d(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu)
    return (u & 0x7fffffffu) == 0u ? __longlong_as_double((long long)(u & 0x80000000u) << 32) : (double)f;
  const uint64_t bits = ((uint64_t)(u & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                        ((uint64_t)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ double df_to_double(DF x) { return f2d(x.hi) + f2d(x.lo); }

// Normalised double-float product (TwoProduct by FMA plus the cross terms).
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ DF df_sub(DF a, DF b) { return df_add(a, DF{-b.hi, -b.lo}); }

// 1 / x: the rounded FP32 reciprocal refined by one Newton step in
// double-float, r + r (1 - x r), about 2^-46 relative for normal x.
__device__ __forceinline__ DF df_recip(DF x) {
  const float r = __frcp_rn(x.hi);
  const DF xr = df_mul(x, DF{r, 0.f});
  const DF e = df_sub(DF{1.f, 0.f}, xr);
  return fast_two_sum(r, __fmul_rn(r, e.hi));
}

__host__ __device__ __forceinline__ DF df_split(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}

}  // namespace lmg
