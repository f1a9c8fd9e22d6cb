// Truncated column-pivoted QR of many small matrices at once, the kernel of
// orthonormalize_generators! and recompress! on the device (reference
// src/generators.jl:64-114, src/compression.jl:22-30, :148-260).
//
// Each task factors its matrix G (p x q) in place in global memory (the
// coupling matrices of recompress! widen from level to level, so they are not
// staged) with the steps of LAPACK xLAQP2: pivot = first column of largest
// partial norm, xLARFG reflector, partial norms downdated with the recompute
// safeguard.  The rank is the number of leading |R_jj| above
// max(atol, rtol |R_11|) (`_compress_block!`'s rule); the task writes Q's
// first `rank` columns explicitly (p x rank) and R's first `rank` rows with
// the column pivoting undone (rank x q, the R[:, invperm(p)] of the reference).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int QT = 256;

__device__ __forceinline__ void amax_merge(double& v, int& i, double ov, int oi) {
  if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
}

// beta, tau and the scale of the reflector's tail from alpha and the squared
// tail norm (xLARFG; no rescaling of tiny norms: the inputs here are generators
// of moderate size)
__device__ __forceinline__ void larfg_d(double alpha, double ss, double& beta, double& tau, double& scal) {
  if (ss == 0.0) {
    tau = 0.0;
    beta = alpha;
    scal = 1.0;
    return;
  }
  const double nrm = sqrt(fma(alpha, alpha, ss));
  beta = -copysign(nrm, alpha);
  tau = (beta - alpha) / beta;
  scal = 1.0 / (alpha - beta);
}

__global__ void __launch_bounds__(QT) pqr_kernel(const PqrTask* __restrict__ tasks) {
  extern __shared__ __align__(16) unsigned char qsm[];
  const PqrTask t = tasks[blockIdx.x];
  const int p = t.p, q = t.q;
  const int kmax = min(p, q);
  double* vn1 = (double*)qsm;          // q
  double* vn2 = vn1 + q;               // q
  double* taus = vn2 + q;              // kmax
  int* perm = (int*)(taus + kmax);     // q
  __shared__ double red_v[QT / 32 + 2];
  __shared__ int red_i[QT / 32 + 1];
  __shared__ int s_rank;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double* G = t.G;
  const int64_t ld = t.ldg;
  for (int c = tid; c < q; c += QT) {
    double ss = 0.0;
    for (int i = 0; i < p; ++i) ss = fma(G[i + c * ld], G[i + c * ld], ss);
    vn1[c] = sqrt(ss);
    vn2[c] = vn1[c];
    perm[c] = c;
  }
  if (tid == 0) s_rank = 0;
  __syncthreads();
  const double tol3z = 1.0536712127723509e-08;   // sqrt(2^-53)
  double tol = 0.0;
  int rk = 0;
  for (int j = 0; j < kmax; ++j) {
    double bv = -1.0;
    int bi = q;
    for (int c = j + tid; c < q; c += QT) amax_merge(bv, bi, vn1[c], c);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
      amax_merge(bv, bi, __shfl_down_sync(0xffffffffu, bv, off), __shfl_down_sync(0xffffffffu, bi, off));
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      double v = red_v[0];
      int i = red_i[0];
      for (int w = 1; w < QT / 32; ++w) amax_merge(v, i, red_v[w], red_i[w]);
      red_i[QT / 32] = i < q ? i : j;
    }
    __syncthreads();
    const int piv = red_i[QT / 32];
    if (piv != j) {
      for (int i = tid; i < p; i += QT) {
        const double x = G[i + j * ld];
        G[i + j * ld] = G[i + piv * ld];
        G[i + piv * ld] = x;
      }
      __syncthreads();
      if (tid == 0) {
        const int x = perm[j]; perm[j] = perm[piv]; perm[piv] = x;
        vn1[piv] = vn1[j];
        vn2[piv] = vn2[j];
      }
    }
    __syncthreads();
    double* colj = G + j * ld;
    if (warp == 0) {
      double ss = 0.0;
      for (int i = j + 1 + lane; i < p; i += 32) ss = fma(colj[i], colj[i], ss);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, off);
      double beta, tau, scal;
      larfg_d(colj[j], ss, beta, tau, scal);
      __syncwarp();
      if (tau != 0.0)
        for (int i = j + 1 + lane; i < p; i += 32) colj[i] *= scal;
      if (lane == 0) {
        colj[j] = beta;
        red_v[QT / 32] = beta;
        red_v[QT / 32 + 1] = tau;
        taus[j] = tau;
      }
    }
    __syncthreads();
    const double beta = red_v[QT / 32], tau = red_v[QT / 32 + 1];
    if (j == 0) tol = fmax(t.atol, t.rtol * fabs(beta));
    if (!(fabs(beta) > tol)) break;
    rk = j + 1;
    for (int c = j + 1 + tid; c < q; c += QT) {
      double* mc = G + c * ld;
      if (tau != 0.0) {
        double w = mc[j];
        for (int i = j + 1; i < p; ++i) w = fma(colj[i], mc[i], w);
        const double tw = tau * w;
        mc[j] -= tw;
        for (int i = j + 1; i < p; ++i) mc[i] = fma(-tw, colj[i], mc[i]);
      }
      if (vn1[c] != 0.0) {
        double temp = fabs(mc[j]) / vn1[c];
        temp = fmax(1.0 - temp * temp, 0.0);
        const double ratio = vn1[c] / vn2[c];
        if (temp * ratio * ratio <= tol3z) {
          double ss = 0.0;
          for (int i = j + 1; i < p; ++i) ss = fma(mc[i], mc[i], ss);
          vn1[c] = sqrt(ss);
          vn2[c] = vn1[c];
        } else {
          vn1[c] *= sqrt(temp);
        }
      }
    }
    __syncthreads();
  }
  // R with the pivoting undone: R(0:rk, perm[c]) = upper part of column c
  for (int64_t e = tid; e < (int64_t)rk * q; e += QT) {
    const int i = (int)(e % rk), c = (int)(e / rk);
    t.R[i + (int64_t)perm[c] * t.ldr] = i <= c ? G[i + c * ld] : 0.0;
  }
  // Q = H_0 ... H_{rk-1} [I; 0] (xORG2R), column c by thread
  for (int c = tid; c < rk; c += QT) {
    double* qc = t.Q + (int64_t)c * t.ldq;
    for (int i = 0; i < p; ++i) qc[i] = i == c ? 1.0 : 0.0;
    for (int j = min(c, rk - 1); j >= 0; --j) {
      const double tj = taus[j];
      if (tj == 0.0) continue;
      const double* vj = G + j * ld;   // v = (1, G[j+1.., j])
      double w = qc[j];
      for (int i = j + 1; i < p; ++i) w = fma(vj[i], qc[i], w);
      const double tw = tj * w;
      qc[j] -= tw;
      for (int i = j + 1; i < p; ++i) qc[i] = fma(-tw, vj[i], qc[i]);
    }
  }
  if (tid == 0) *t.rank = rk;
}

}  // namespace

size_t pqr_smem(int qmax, int kmax) { return (size_t)qmax * 3 * 8 + (size_t)kmax * 8 + 64; }

void launch_pqr(const PqrTask* tasks, int64_t count, int qmax, int kmax, cudaStream_t st) {
  const size_t smem = pqr_smem(qmax, kmax);
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    cudaFuncSetAttribute(pqr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  for (int64_t b = 0; b < count; b += 65535) {
    const unsigned g = (unsigned)std::min<int64_t>(65535, count - b);
    pqr_kernel<<<g, QT, smem, st>>>(tasks + b);
  }
}

}  // namespace hss
