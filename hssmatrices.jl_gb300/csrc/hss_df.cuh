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

// (hi, lo) floats with hi + lo = x to ~2^-47 relative, from x's bits by
// integer operations (GB300 runs FP64 instructions, conversions included, far
// below its FP32 and integer rates): hi = x truncated to 24 significant bits,
// lo = the remaining 29 bits rounded to 24 (nearest, ties to even).  Doubles
// whose pieces leave float's normal range (|x| < 2^-74 but not zero,
// |x| >= 2^128, inf, nan) take the conversion path, which is kept out of
// line so that its FP64 instructions are not if-converted into every call.
static __device__ __noinline__ float2 split_far(double x) { return split_d(x); }

static __device__ __forceinline__ float2 split_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
  if ((b << 1) == 0ull) return make_float2(__uint_as_float(sgn), 0.f);   // +-0 (masked and padding entries)
  const int e = (int)((b >> 52) & 0x7ffu) - 1023;
  if (e < -74 || e > 127) return split_far(x);
  const float h = __uint_as_float(sgn | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
  const unsigned low = (unsigned)b & 0x1fffffffu;   // value low * 2^(e - 52)
  if (low == 0u) return make_float2(h, 0.f);
  const int lz = __clz(low) - 3;                    // low < 2^29
  const unsigned m = low << lz;                     // bit 28 set: value 1.f * 2^(e - 24 - lz)
  unsigned mant = m >> 5;
  const unsigned rem = m & 31u;
  if (rem > 16u || (rem == 16u && (mant & 1u))) ++mant;
  int el = e - 24 - lz;
  if (mant >> 24) {
    mant >>= 1;
    ++el;
  }
  return make_float2(h, __uint_as_float(sgn | ((unsigned)(el + 127) << 23) | (mant & 0x7fffffu)));
}

}  // namespace hss
