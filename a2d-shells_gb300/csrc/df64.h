// Double-float ("df64") numbers: an unevaluated sum hi + lo of two FP32
// values (~48-bit significand), computed on the FP32 pipe, which on GB300
// runs ~58x the FP64 rate.  Used by the double-float factorization.
#pragma once
#include <cuda_runtime.h>

namespace a2ds {

struct __align__(8) df64 {
  float hi, lo;
};

// (hi, lo) -= a b: the FP32 product a.hi b.hi with its exact error (FMA),
// cross terms in FP32, Knuth's two-sum for the leading parts, and the
// low-order terms gathered in lo.  The _rn intrinsics keep the compiler from
// fusing the two-sum's operations into FMAs, which would break its exactness.
__device__ __forceinline__ void df_sub_prod(float &hi, float &lo, df64 a, df64 b) {
  const float ph = __fmul_rn(a.hi, b.hi);
  float pe = fmaf(a.hi, b.hi, -ph);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  const float s = __fsub_rn(hi, ph);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(-ph, bb));
  hi = s;
  lo = __fadd_rn(lo, __fsub_rn(err, pe));
}
__device__ __forceinline__ df64 df_norm(float hi, float lo) {
  const float s = __fadd_rn(hi, lo);
  return df64{s, __fsub_rn(lo, __fsub_rn(s, hi))};
}
// FP64 -> df64: the nearest FP32 value and the FP32-rounded remainder.
__device__ __forceinline__ df64 df_split(double v) {
  const float h = __double2float_rn(v);
  return df64{h, __double2float_rn(v - (double)h)};
}

}  // namespace a2ds
