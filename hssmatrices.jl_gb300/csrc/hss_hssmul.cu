// HSS x HSS product on the device (reference src/matmul.jl:65-117).
//
// The product of two HSS matrices on matching cluster trees is an HSS matrix
// on the same tree whose ranks are the sums of the operands' ranks.  Its
// generators come from three sweeps of small dense products:
//
//   * upsweep (post-order): Z = V_A^T U_B at a leaf, Z = W1_A^T Z1 R1_B +
//     W2_A^T Z2 R2_B at a branch (matmul.jl:86-94);
//   * downsweep (pre-order): F of the children, F1 = B12_A Z2 B21_B +
//     R1_A F W1_B^T, F2 = B21_A Z1 B12_B + R2_A F W2_B^T (:72-73, :104-105);
//   * assembly: D = D_A D_B + U_A F V_B^T, U = [U_A, D_A U_B],
//     V = [D_B^T V_A, V_B] at a leaf (:98-101); the block generators of a
//     branch (:106-111), written straight into the new handle's buffer.
//
// Every step is a list of independent tasks C = a1 op(A1) op(B1) +
// a2 op(A2) op(B2) (or a block copy / zero fill) run by one kernel launch,
// one block per task; the host orders the launches so that every task's
// inputs are complete.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int MT = 256;   // threads per task
constexpr int TI = 32;    // output tile (rows and columns) of the tiled path
constexpr int TK = 16;    // K chunk of the tiled path

__device__ __forceinline__ double opA(const double* A, int lda, int ta, int i, int l) {
  return ta ? A[l + (int64_t)i * lda] : A[i + (int64_t)l * lda];
}
__device__ __forceinline__ double opB(const double* B, int ldb, int tb, int l, int j) {
  return tb ? B[j + (int64_t)l * ldb] : B[l + (int64_t)j * ldb];
}

// One task: its output in 32 x 32 tiles, each term's operands staged in K
// chunks of 16 (thread (r, c) computes rows r, r+16 and columns c, c+16 of a tile).
__global__ void __launch_bounds__(MT) mm_list_kernel(const MmTask* __restrict__ tasks) {
  __shared__ double As[TK][TI + 1];
  __shared__ double Bs[TK][TI + 1];
  const MmTask t = tasks[blockIdx.x];
  const int tid = threadIdx.x;
  if (t.k1 < 0) {   // copy (A1 != null) or zero fill, by cmode
    for (int64_t e = tid; e < (int64_t)t.m * t.n; e += MT) {
      const int i = (int)(e % t.m), j = (int)(e / t.m);
      double* c = t.C + i + (int64_t)j * t.ldc;
      double v = t.cmode == MM_EYE ? (i == j ? 1.0 : 0.0) : (t.A1 ? opA(t.A1, t.lda1, t.ta1, i, j) : 0.0);
      if (t.cmode == MM_TRIL && j > i) v = 0.0;
      if (t.cmode == MM_AXPY) v = t.beta != 0.0 ? fma(t.a1, v, t.beta * *c) : t.a1 * v;
      *c = v;
    }
    return;
  }
  const int tr = tid & 15, tc = tid >> 4;
  for (int i0 = 0; i0 < t.m; i0 += TI)
    for (int j0 = 0; j0 < t.n; j0 += TI) {
      double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
      for (int term = 0; term < 2; ++term) {
        const double* A = term ? t.A2 : t.A1;
        const double* B = term ? t.B2 : t.B1;
        const int K = term ? t.k2 : t.k1;
        if (!A || K <= 0) continue;
        const int lda = term ? t.lda2 : t.lda1, ldb = term ? t.ldb2 : t.ldb1;
        const int ta = term ? t.ta2 : t.ta1, tb = term ? t.tb2 : t.tb1;
        const double a = term ? t.a2 : t.a1;
        double part[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
        for (int l0 = 0; l0 < K; l0 += TK) {
          __syncthreads();
          for (int e = tid; e < TK * TI; e += MT) {
            const int l = e % TK, q = e / TK;
            const bool okl = l0 + l < K;
            As[l][q] = (okl && i0 + q < t.m) ? opA(A, lda, ta, i0 + q, l0 + l) : 0.0;
            Bs[l][q] = (okl && j0 + q < t.n) ? opB(B, ldb, tb, l0 + l, j0 + q) : 0.0;
          }
          __syncthreads();
#pragma unroll
          for (int l = 0; l < TK; ++l) {
            const double a0 = As[l][tr], a1 = As[l][tr + 16];
            const double b0 = Bs[l][tc], b1 = Bs[l][tc + 16];
            part[0][0] = fma(a0, b0, part[0][0]);
            part[0][1] = fma(a0, b1, part[0][1]);
            part[1][0] = fma(a1, b0, part[1][0]);
            part[1][1] = fma(a1, b1, part[1][1]);
          }
        }
#pragma unroll
        for (int x = 0; x < 2; ++x)
#pragma unroll
          for (int y = 0; y < 2; ++y) acc[x][y] = fma(a, part[x][y], acc[x][y]);
      }
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
          const int i = i0 + tr + 16 * x, j = j0 + tc + 16 * y;
          if (i < t.m && j < t.n) {
            double* c = t.C + i + (int64_t)j * t.ldc;
            *c = t.beta != 0.0 ? fma(t.beta, *c, acc[x][y]) : acc[x][y];
          }
        }
    }
}

}  // namespace

void launch_mm_list(const MmTask* tasks, int64_t count, cudaStream_t st) {
  for (int64_t b = 0; b < count; b += 1 << 30) {
    const unsigned g = (unsigned)std::min<int64_t>(1 << 30, count - b);
    mm_list_kernel<<<g, MT, 0, st>>>(tasks + b);
  }
}

}  // namespace hss
