// Row transforms of the HSS-valued division (reference src/ulvdivide.jl).
//
// The division hssA \ hssB eliminates A level by level with the ULV reduction
// (QL of U, LQ of the first rows of D) and applies the same transforms to the
// rows of B's leaf blocks.  A's reductions are those of its FP64 ULV
// factorization (the blocked factor kernel stores the QL reflectors in U's
// storage, L1 / L2 in D's, the LQ reflectors explicitly as columns of Qt, the
// root block's LU with row swaps), so the kernels here read a factored node:
//
//   * DIV_QL  (:30-32, :115-129): X <- Q_ql^T X; the first mk rows solved with
//     L1 (trsm) and written to `top` with the other rows zeroed; the last k
//     rows written to `bot`;
//   * DIV_LQ  (:51, :130-136):    X <- Q_lq^T X (rows of the LQ column space);
//   * DIV_ROOT (:23-26):          X <- D^-1 X with the root block's LU.
//
// One thread block per (task, 32 columns); each column is held by 8 lanes of
// a warp (row l8 + 8 s in register s), so the reflector dot products, the
// row swaps and the triangular solves need warp shuffles only.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int DT = 256;   // threads per block: 32 columns x 8 lanes
constexpr int DC = 32;    // columns per block

__device__ __forceinline__ double sum8(double v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  return v;
}

// the value of row i of this lane group's column (all 8 lanes get it)
template <int RPT>
__device__ __forceinline__ double row_value(const double (&b)[RPT], int i, int lane) {
  double v = 0.0;
#pragma unroll
  for (int s = 0; s < RPT; ++s)
    if (s == (i >> 3)) v = b[s];
  return __shfl_sync(0xffffffffu, v, (lane & ~7) | (i & 7));
}

// b <- H b for the Householder vector v (entries v(row) from `vat`), tau
template <int RPT, typename F>
__device__ __forceinline__ void reflect(double (&b)[RPT], int rows, int l8, double tau, F vat) {
  double d0 = 0.0, d1 = 0.0;
#pragma unroll
  for (int s = 0; s < RPT; ++s) {
    const int row = l8 + 8 * s;
    if (row < rows) {
      const double v = vat(row);
      if (s & 1) d1 = fma(v, b[s], d1);
      else d0 = fma(v, b[s], d0);
    }
  }
  const double w = sum8(d0 + d1) * tau;
#pragma unroll
  for (int s = 0; s < RPT; ++s) {
    const int row = l8 + 8 * s;
    if (row < rows) b[s] = fma(-w, vat(row), b[s]);
  }
}

// forward substitution with the lower triangle of L (ld ldl), nrows rows;
// unit diagonal if UNIT
template <int RPT, bool UNIT>
__device__ __forceinline__ void lower_subst(double (&b)[RPT], const double* L, int ldl, int nrows, int l8, int lane) {
  for (int i = 0; i < nrows; ++i) {
    double x = row_value<RPT>(b, i, lane);
    if (!UNIT) x /= L[i + (int64_t)i * ldl];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int row = l8 + 8 * s;
      if (row == i) b[s] = x;
      else if (row > i && row < nrows) b[s] = fma(-L[row + (int64_t)i * ldl], x, b[s]);
    }
  }
}

// back substitution with the upper triangle of U (ld ldu)
template <int RPT>
__device__ __forceinline__ void upper_subst(double (&b)[RPT], const double* U, int ldu, int nrows, int l8, int lane) {
  for (int i = nrows - 1; i >= 0; --i) {
    const double x = row_value<RPT>(b, i, lane) / U[i + (int64_t)i * ldu];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int row = l8 + 8 * s;
      if (row == i) b[s] = x;
      else if (row < i) b[s] = fma(-U[row + (int64_t)i * ldu], x, b[s]);
    }
  }
}

template <int RPT>
__global__ void __launch_bounds__(DT) div_rows_kernel(const DivTask* __restrict__ tasks) {
  const DivTask t = tasks[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, l8 = tid & 7;
  const int jl = tid >> 3;
  const int j0 = blockIdx.y * DC;
  if (j0 >= t.cols) return;
  const int j = j0 + jl;
  const bool act = j < t.cols;
  const Node& nd = *t.nd;
  const double* fb = t.fb;
  const int rows = t.rows;
  double b[RPT];
#pragma unroll
  for (int s = 0; s < RPT; ++s) {
    const int row = l8 + 8 * s;
    b[s] = (act && row < rows) ? t.src[row + (int64_t)j * t.lds] : 0.0;
  }
  if (t.mode == DIV_ROOT) {
    // the LU's row swaps (sequential), then the unit lower and the upper solve
    const int32_t* piv = (const int32_t*)(fb + nd.fpiv);
    for (int c = 0; c < rows; ++c) {
      const int p = piv[c];
      if (p == c) continue;
      const double vc = row_value<RPT>(b, c, lane), vp = row_value<RPT>(b, p, lane);
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int row = l8 + 8 * s;
        if (row == c) b[s] = vp;
        else if (row == p) b[s] = vc;
      }
    }
    const double* LU = fb + nd.fD;
    lower_subst<RPT, true>(b, LU, nd.m, rows, l8, lane);
    upper_subst<RPT>(b, LU, nd.m, rows, l8, lane);
    if (act)
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int row = l8 + 8 * s;
        if (row < rows) t.top[row + (int64_t)j * t.ldt] = b[s];
      }
    return;
  }
  if (t.mode == DIV_QL) {
    // Q_ql^T: reflectors c = k-1 .. 0 in generation order; v(p) = 1 at p = mk + c,
    // v = U(:, c) above it, 0 below
    const int mk = nd.mk, k = nd.k, m = nd.m;
    const double* Up = fb + nd.fU;
    const double* tq = fb + nd.ftq;
    for (int c = k - 1; c >= 0; --c) {
      const double tau = tq[c];
      if (tau == 0.0) continue;
      const int p = mk + c;
      const double* v = Up + (int64_t)c * m;
      reflect<RPT>(b, rows, l8, tau, [&](int row) { return row < p ? v[row] : (row == p ? 1.0 : 0.0); });
    }
    // zloc = L1 \ X[0:mk]
    lower_subst<RPT, false>(b, fb + nd.fD, m, mk, l8, lane);
    if (act)
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int row = l8 + 8 * s;
        if (row < rows) {
          t.top[row + (int64_t)j * t.ldt] = row < mk ? b[s] : 0.0;
          if (row >= mk) t.bot[(row - mk) + (int64_t)j * t.ldb] = b[s];
        }
      }
    return;
  }
  // DIV_LQ: Q_lq^T, reflectors i = nl-1 .. 0, stored as explicit columns of Qt
  const int n = nd.n, nl = min(nd.mk, n);
  const double* Qt = fb + nd.fQt;
  const double* tl = fb + nd.ftl;
  for (int i = nl - 1; i >= 0; --i) {
    const double tau = tl[i];
    if (tau == 0.0) continue;
    const double* v = Qt + (int64_t)i * n;
    reflect<RPT>(b, rows, l8, tau, [&](int row) { return v[row]; });
  }
  if (act)
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int row = l8 + 8 * s;
      if (row < rows) t.top[row + (int64_t)j * t.ldt] = b[s];
    }
}

}  // namespace

int div_rows_max() { return 64 * 8; }

cudaError_t launch_div_rows(const DivTask* tasks, int64_t count, int maxrows, int maxcols, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  const unsigned gy = (unsigned)std::max(1, (maxcols + DC - 1) / DC);
  for (int64_t b0 = 0; b0 < count; b0 += 1 << 30) {
    const dim3 grid((unsigned)std::min<int64_t>(1 << 30, count - b0), gy);
    if (maxrows <= 64) div_rows_kernel<8><<<grid, DT, 0, st>>>(tasks + b0);
    else if (maxrows <= 128) div_rows_kernel<16><<<grid, DT, 0, st>>>(tasks + b0);
    else if (maxrows <= 256) div_rows_kernel<32><<<grid, DT, 0, st>>>(tasks + b0);
    else div_rows_kernel<64><<<grid, DT, 0, st>>>(tasks + b0);
  }
  return cudaGetLastError();
}

}  // namespace hss
