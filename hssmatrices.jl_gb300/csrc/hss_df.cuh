// Double-float arithmetic on the FP32 pipe: a value is an unevaluated pair
// (hi, lo) of floats (hi = fl32(x), lo = fl32(x - hi), ~48 significant bits).
// Products use the exact FMA product error, sums use TwoSum (Knuth); every
// step is a separately rounded FP32 operation (no contraction).
#pragma once
#include <cuda_runtime.h>

namespace hss {

// (sh, sl) += a * x
__device__ __forceinline__ void df_fma(float& sh, float& sl, float2 a, float2 x) {
  const float p = __fmul_rn(a.x, x.x);
  float e = __fmaf_rn(a.x, x.x, -p);
  e = __fmaf_rn(a.x, x.y, e);
  e = __fmaf_rn(a.y, x.x, e);
  const float t = __fadd_rn(sh, p);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// (sh, sl) += (bh, bl)
__device__ __forceinline__ void df_add(float& sh, float& sl, float bh, float bl) {
  const float t = __fadd_rn(sh, bh);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(bh, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, bl));
}

// renormalised pair (|lo| <= ulp(hi) / 2)
__device__ __forceinline__ float2 df_norm(float sh, float sl) {
  const float s = __fadd_rn(sh, sl);
  return make_float2(s, __fsub_rn(sl, __fsub_rn(s, sh)));
}

__device__ __forceinline__ float2 split_d(double x) {
  const float h = __double2float_rn(x);
  const float l = __double2float_rn(x - (double)h);
  return make_float2(h, l);
}

}  // namespace hss
