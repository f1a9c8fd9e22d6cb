// Device helpers shared by the kernels: type-exact math (a float argument must
// never be promoted to double: FP64 throughput on GB300 is ~1/64 of FP32) and
// LAPACK's dlarfg/slarfg.
#pragma once
#include <cuda_runtime.h>

namespace hss {

__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dhypot(float a, float b) { return hypotf(a, b); }
__device__ __forceinline__ double dhypot(double a, double b) { return hypot(a, b); }
__device__ __forceinline__ float dcopysign(float a, float b) { return copysignf(a, b); }
__device__ __forceinline__ double dcopysign(double a, double b) { return copysign(a, b); }
__device__ __forceinline__ float dabs(float a) { return fabsf(a); }
__device__ __forceinline__ double dabs(double a) { return fabs(a); }

// Householder generation (LAPACK xLARFG) from alpha and the squared norm of
// the tail: beta = -sign(alpha) * ||(alpha, x)||, tau = (beta - alpha) / beta,
// v = x * scal with scal = 1 / (alpha - beta); tau = 0 (H = I) when x == 0.
template <typename T>
__device__ __forceinline__ void larfg_ss(T alpha, T ss, T& beta, T& tau, T& scal) {
  if (ss == T(0)) {
    tau = T(0);
    beta = alpha;
    scal = T(1);
  } else {
    const T xnorm = dsqrt(ss);
    beta = -dcopysign(dhypot(alpha, xnorm), alpha);
    tau = (beta - alpha) / beta;
    scal = T(1) / (alpha - beta);
  }
}

}  // namespace hss
