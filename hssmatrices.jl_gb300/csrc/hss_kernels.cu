// sm_103a kernels of the HSS hot path.
//
// Every kernel processes one task list (the nodes of one tree level, across
// all trees of a forest), one thread block per node.  Generators are FP64;
// the ULV factorization and solve are templated on the working type T
// (double: plain FP64 form; float: FP32 form refined in FP64 by the host).
//
// Householder conventions follow LAPACK as called by the reference:
//   * QL of U (geqlf!, src/ulvfactor.jl:39): reflector c (0-based) has its
//     pivot at row mk+c of column c, vector stored above it; Q^T is applied
//     in generation order c = k-1 .. 0 (ormql! 'L','T', :41-42);
//   * LQ of D[0:mk, :] (gelqf!, :44): reflector i has its pivot at (i,i),
//     vector stored in row i to the right; C Q^T and Q V apply i = 0 .. mk-1
//     (ormlq! 'R','T' :47 and 'L','N' :50); Q^T z applies i = mk-1 .. 0
//     (ormlq! 'L','T', :102).
//   * dlarfg: beta = -sign(alpha) * ||(alpha, x)||, tau = (beta - alpha) / beta,
//     v = x / (alpha - beta); tau = 0 (H = I) when x == 0.
#include <cuda_runtime.h>
#include <cstdint>
#include "hss_device.cuh"
#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

constexpr int NT = 256;   // threads per block for every kernel here
constexpr int NW = NT / 32;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block; every thread gets the result.  `red` holds >= NW values.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* red) {
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  T s = T(0);
#pragma unroll
  for (int i = 0; i < NW; ++i) s += red[i];
  return s;
}

template <typename T>
__device__ __forceinline__ void householder(T alpha, T ss, T& beta, T& tau, T& scal) {
  larfg_ss(alpha, ss, beta, tau, scal);
}

// ---------------------------------------------------------------------------
// HSS x dense product (src/matmul.jl:32-62)
// ---------------------------------------------------------------------------

// C(rows, j) = alpha * A(rows, :) * X(:, j) [+ beta * Y], A is m x n col-major,
// X is n x r (ldx).  Threads: row i, split-K groups over the columns of A.
// `acc_c` adds to the existing C instead of the Y term.
template <int NJ>
__device__ __forceinline__ void rows_times_cols(const double* __restrict__ A, int m, int n,
                                                const double* __restrict__ X, int64_t ldx,
                                                int j0, double* Xs, double* part,
                                                double alpha, double beta,
                                                const double* __restrict__ Y, int64_t ldy,
                                                double* __restrict__ C, int64_t ldc,
                                                bool acc_c, double* colnorm2) {
  constexpr int LT = 256;     // staged rows of X per pass
  const int tid = threadIdx.x;
  for (int r0 = 0; r0 < m; r0 += NT) {
    const int rows = min(NT, m - r0);
    int rp = 1;
    while (rp < rows) rp <<= 1;           // power-of-two row slots
    const int G = NT / rp;                 // split-K groups
    const int i = r0 + (tid % rp);
    const int g = tid / rp;
    const bool act = (tid % rp) < rows && g < G;
    double acc[NJ];
#pragma unroll
    for (int q = 0; q < NJ; ++q) acc[q] = 0.0;
    for (int l0 = 0; l0 < n; l0 += LT) {
      const int nl = min(LT, n - l0);
      __syncthreads();
      for (int e = tid; e < nl * NJ; e += NT) {
        const int l = e % nl, q = e / nl;
        Xs[l * NJ + q] = X[(int64_t)(l0 + l) + (int64_t)(j0 + q) * ldx];
      }
      __syncthreads();
      if (act) {
        const double* a = A + i + (int64_t)l0 * m;
#pragma unroll 4
        for (int l = g; l < nl; l += G) {
          const double d = a[(int64_t)l * m];
#pragma unroll
          for (int q = 0; q < NJ; ++q) acc[q] = fma(d, Xs[l * NJ + q], acc[q]);
        }
      }
    }
    // combine split-K partials
    __syncthreads();
    if (act) {
#pragma unroll
      for (int q = 0; q < NJ; ++q) part[(g * rp + (tid % rp)) * NJ + q] = acc[q];
    }
    __syncthreads();
    if (act && g == 0) {
#pragma unroll
      for (int q = 0; q < NJ; ++q) {
        double s = 0.0;
        for (int gg = 0; gg < G; ++gg) s += part[(gg * rp + (tid % rp)) * NJ + q];
        const int64_t j = j0 + q;
        double* c = C + i + j * ldc;
        double v = alpha * s;
        if (acc_c) v += *c;
        else if (beta != 0.0 && Y != nullptr) v += beta * Y[i + j * ldy];
        *c = v;
        part[(tid % rp) * NJ + q] = v * v;   // reuse slot 0 for the norm
      }
    }
    if (colnorm2 != nullptr) {
      __syncthreads();
      // column sums of squares over this row pass
      for (int q = tid >> 5; q < NJ; q += NW) {
        double s = 0.0;
        for (int ii = (tid & 31); ii < rows; ii += 32) s += part[ii * NJ + q];
        s = warp_sum(s);
        if ((tid & 31) == 0) atomicAdd(colnorm2 + j0 + q, s);
      }
    }
    __syncthreads();
  }
}

__device__ void block_rows_times_cols(const double* A, int m, int n, const double* X, int64_t ldx,
                                      int r, double* Xs, double* part, double alpha, double beta,
                                      const double* Y, int64_t ldy, double* C, int64_t ldc,
                                      bool acc_c, double* colnorm2) {
  int j0 = 0;
  for (; j0 + 8 <= r; j0 += 8)
    rows_times_cols<8>(A, m, n, X, ldx, j0, Xs, part, alpha, beta, Y, ldy, C, ldc, acc_c, colnorm2);
  if (r - j0 >= 4) {
    rows_times_cols<4>(A, m, n, X, ldx, j0, Xs, part, alpha, beta, Y, ldy, C, ldc, acc_c, colnorm2);
    j0 += 4;
  }
  if (r - j0 >= 2) {
    rows_times_cols<2>(A, m, n, X, ldx, j0, Xs, part, alpha, beta, Y, ldy, C, ldc, acc_c, colnorm2);
    j0 += 2;
  }
  if (r - j0 >= 1)
    rows_times_cols<1>(A, m, n, X, ldx, j0, Xs, part, alpha, beta, Y, ldy, C, ldc, acc_c, colnorm2);
}

// Leaves: Z = V^T B_leaf (src/matmul.jl:34) and C = alpha D B_leaf + beta Y (:46).
// One thread block per (leaf, chunk of rc right-hand sides).
__global__ void __launch_bounds__(NT) mv_leaf_kernel(const Task* __restrict__ tasks,
                                                     const Slot* __restrict__ slots, int rc, int nchunk) {
  __shared__ double Xs[256 * 8];
  __shared__ double part[NT * 8];
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * rc;
  const Node& nd = tk.nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  if (j0 >= sl.r) return;
  const int m = nd.gm, n = nd.gn, kv = nd.kv, r = min(rc, sl.r - j0);
  const double* Bl = sl.B + nd.col0 + (int64_t)j0 * sl.ldb;
  if (kv > 0) {
    double* Z = (double*)sl.ws + nd.wz + (int64_t)j0 * sl.ldws;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = warp; o < kv * r; o += NW) {
      const int c = o % kv, j = o / kv;
      const double* v = nd.V + (int64_t)c * n;
      const double* b = Bl + (int64_t)j * sl.ldb;
      double s = 0.0;
      for (int l = lane; l < n; l += 32) s = fma(v[l], b[l], s);
      s = warp_sum(s);
      if (lane == 0) Z[c + (int64_t)j * sl.ldws] = s;
    }
  }
  block_rows_times_cols(nd.D, m, n, Bl, sl.ldb, r, Xs, part, sl.alpha, sl.beta,
                        sl.Y ? sl.Y + nd.row0 + (int64_t)j0 * sl.ldy : nullptr, sl.ldy,
                        sl.C + nd.row0 + (int64_t)j0 * sl.ldc, sl.ldc, false, nullptr);
}

// Generic (unstaged) sweeps for ranks whose staged blocks do not fit in shared memory.
// Upsweep, non-root branch: Z = W1^T Z1 + W2^T Z2 (src/matmul.jl:39).
__global__ void __launch_bounds__(NT) mv_up_kernel(const Task* __restrict__ tasks,
                                                   const Slot* __restrict__ slots) {
  const Task tk = tasks[blockIdx.x];
  const Node& nd = tk.nodes[tk.node];
  const Node& c1 = tk.nodes[nd.left];
  const Node& c2 = tk.nodes[nd.right];
  const Slot& sl = slots[tk.slot];
  const double* ws = (const double*)sl.ws;
  double* Z = (double*)sl.ws + nd.wz;
  const int64_t ld = sl.ldws;
  const int kv = nd.kv, r = sl.r;
  for (int o = threadIdx.x; o < kv * r; o += NT) {
    const int c = o % kv, j = o / kv;
    double s = 0.0;
    const double* z1 = ws + c1.wz + j * ld;
    const double* z2 = ws + c2.wz + j * ld;
    for (int l = 0; l < c1.kv; ++l) s = fma(nd.W1[l + (int64_t)c * c1.kv], z1[l], s);
    for (int l = 0; l < c2.kv; ++l) s = fma(nd.W2[l + (int64_t)c * c2.kv], z2[l], s);
    Z[c + j * ld] = s;
  }
}

// Downsweep, branch: F1 = B12 Z2 + R1 F, F2 = B21 Z1 + R2 F (src/matmul.jl:50-56).
__global__ void __launch_bounds__(NT) mv_down_kernel(const Task* __restrict__ tasks,
                                                     const Slot* __restrict__ slots) {
  const Task tk = tasks[blockIdx.x];
  const Node& nd = tk.nodes[tk.node];
  const Node& c1 = tk.nodes[nd.left];
  const Node& c2 = tk.nodes[nd.right];
  const Slot& sl = slots[tk.slot];
  double* ws = (double*)sl.ws;
  const int64_t ld = sl.ldws;
  const int r = sl.r, ku = nd.root ? 0 : nd.ku;
  const int n1 = c1.ku * r;
  for (int o = threadIdx.x; o < (c1.ku + c2.ku) * r; o += NT) {
    double s = 0.0;
    if (o < n1) {
      const int i = o % c1.ku, j = o / c1.ku;
      const double* z2 = ws + c2.wz + j * ld;
      for (int l = 0; l < c2.kv; ++l) s = fma(nd.B12[i + (int64_t)l * c1.ku], z2[l], s);
      const double* f = ws + nd.wf + j * ld;
      for (int l = 0; l < ku; ++l) s = fma(nd.R1[i + (int64_t)l * c1.ku], f[l], s);
      ws[c1.wf + i + j * ld] = s;
    } else {
      const int o2 = o - n1;
      const int i = o2 % c2.ku, j = o2 / c2.ku;
      const double* z1 = ws + c1.wz + j * ld;
      for (int l = 0; l < c1.kv; ++l) s = fma(nd.B21[i + (int64_t)l * c2.ku], z1[l], s);
      const double* f = ws + nd.wf + j * ld;
      for (int l = 0; l < ku; ++l) s = fma(nd.R2[i + (int64_t)l * c2.ku], f[l], s);
      ws[c2.wf + i + j * ld] = s;
    }
  }
}

// Staged variants of the two translator sweeps: every operand of the node is
// first copied into shared memory with all threads (independent, coalesced
// loads), then the small products run out of shared memory.  Right-hand sides
// are processed in chunks (one thread block per node and chunk).

__device__ __forceinline__ void stage(double* dst, const double* __restrict__ src, int64_t cnt) {
  for (int64_t e = threadIdx.x; e < cnt; e += NT) dst[e] = src[e];
}
// dst(c + l*cols) = src(l + c*rows): a transposed copy (rows x cols source)
__device__ __forceinline__ void stage_t(double* dst, const double* __restrict__ src, int rows, int cols) {
  for (int e = threadIdx.x; e < rows * cols; e += NT) {
    const int l = e % rows, c = e / rows;
    dst[c + l * cols] = src[e];
  }
}
__device__ __forceinline__ void stage_cols(double* dst, const double* __restrict__ src, int rows, int64_t ld,
                                           int ncols) {
  for (int e = threadIdx.x; e < rows * ncols; e += NT) {
    const int i = e % rows, j = e / rows;
    dst[e] = src[i + (int64_t)j * ld];
  }
}

// Upsweep, non-root branch: Z = W1^T Z1 + W2^T Z2 (src/matmul.jl:39).
// One thread block per (node, chunk of rc right-hand sides).
__global__ void __launch_bounds__(NT) mv_up_staged_kernel(const Task* __restrict__ tasks,
                                                          const Slot* __restrict__ slots, int rc, int nchunk) {
  extern __shared__ __align__(16) double sm[];
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * rc;
  const Node& nd = tk.nodes[tk.node];
  const Node& c1 = tk.nodes[nd.left];
  const Node& c2 = tk.nodes[nd.right];
  const Slot& sl = slots[tk.slot];
  if (j0 >= sl.r) return;
  const int nc = min(rc, sl.r - j0);
  const double* ws = (const double*)sl.ws;
  const int64_t ld = sl.ldws;
  const int kv = nd.kv, k1 = c1.kv, k2 = c2.kv;
  double* W1t = sm;                  // kv x k1 (transposed)
  double* W2t = W1t + kv * k1;       // kv x k2
  double* Z1 = W2t + kv * k2;        // k1 x rc
  double* Z2 = Z1 + k1 * rc;         // k2 x rc
  stage_t(W1t, nd.W1, k1, kv);
  stage_t(W2t, nd.W2, k2, kv);
  stage_cols(Z1, ws + c1.wz + (int64_t)j0 * ld, k1, ld, nc);
  stage_cols(Z2, ws + c2.wz + (int64_t)j0 * ld, k2, ld, nc);
  __syncthreads();
  double* Z = (double*)sl.ws + nd.wz + (int64_t)j0 * ld;
  for (int o = threadIdx.x; o < kv * nc; o += NT) {
    const int c = o % kv, j = o / kv;
    double s0 = 0.0, s1 = 0.0;
    for (int l = 0; l < k1; ++l) s0 = fma(W1t[c + l * kv], Z1[l + j * k1], s0);
    for (int l = 0; l < k2; ++l) s1 = fma(W2t[c + l * kv], Z2[l + j * k2], s1);
    Z[c + (int64_t)j * ld] = s0 + s1;
  }
}

// Downsweep, branch: F1 = B12 Z2 + R1 F, F2 = B21 Z1 + R2 F (src/matmul.jl:50-56).
__global__ void __launch_bounds__(NT) mv_down_staged_kernel(const Task* __restrict__ tasks,
                                                            const Slot* __restrict__ slots, int rc, int nchunk) {
  extern __shared__ __align__(16) double sm[];
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * rc;
  const Node& nd = tk.nodes[tk.node];
  const Node& c1 = tk.nodes[nd.left];
  const Node& c2 = tk.nodes[nd.right];
  const Slot& sl = slots[tk.slot];
  if (j0 >= sl.r) return;
  const int nc = min(rc, sl.r - j0);
  double* ws = (double*)sl.ws;
  const int64_t ld = sl.ldws;
  const int ku = nd.root ? 0 : nd.ku, u1 = c1.ku, u2 = c2.ku, v1 = c1.kv, v2 = c2.kv;
  double* B12 = sm;                  // u1 x v2
  double* B21 = B12 + u1 * v2;       // u2 x v1
  double* R1 = B21 + u2 * v1;        // u1 x ku
  double* R2 = R1 + u1 * ku;         // u2 x ku
  double* Z1 = R2 + u2 * ku;         // v1 x rc
  double* Z2 = Z1 + v1 * rc;         // v2 x rc
  double* Fs = Z2 + v2 * rc;         // ku x rc
  stage(B12, nd.B12, (int64_t)u1 * v2);
  stage(B21, nd.B21, (int64_t)u2 * v1);
  if (ku > 0) {
    stage(R1, nd.R1, (int64_t)u1 * ku);
    stage(R2, nd.R2, (int64_t)u2 * ku);
  }
  stage_cols(Z1, ws + c1.wz + (int64_t)j0 * ld, v1, ld, nc);
  stage_cols(Z2, ws + c2.wz + (int64_t)j0 * ld, v2, ld, nc);
  if (ku > 0) stage_cols(Fs, ws + nd.wf + (int64_t)j0 * ld, ku, ld, nc);
  __syncthreads();
  for (int o = threadIdx.x; o < (u1 + u2) * nc; o += NT) {
    double s0 = 0.0, s1 = 0.0;
    if (o < u1 * nc) {
      const int i = o % u1, j = o / u1;
      for (int l = 0; l < v2; ++l) s0 = fma(B12[i + l * u1], Z2[l + j * v2], s0);
      for (int l = 0; l < ku; ++l) s1 = fma(R1[i + l * u1], Fs[l + j * ku], s1);
      ws[c1.wf + i + (int64_t)(j0 + j) * ld] = s0 + s1;
    } else {
      const int o2 = o - u1 * nc;
      const int i = o2 % u2, j = o2 / u2;
      for (int l = 0; l < v1; ++l) s0 = fma(B21[i + l * u2], Z1[l + j * v1], s0);
      for (int l = 0; l < ku; ++l) s1 = fma(R2[i + l * u2], Fs[l + j * ku], s1);
      ws[c2.wf + i + (int64_t)(j0 + j) * ld] = s0 + s1;
    }
  }
}

// Leaves: C += alpha U F (src/matmul.jl:47), and per-column sums of squares.
__global__ void __launch_bounds__(NT) mv_leaf_final_kernel(const Task* __restrict__ tasks,
                                                           const Slot* __restrict__ slots, int rc, int nchunk) {
  __shared__ double Xs[256 * 8];
  __shared__ double part[NT * 8];
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * rc;
  const Node& nd = tk.nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  if (j0 >= sl.r) return;
  const int m = nd.gm, ku = nd.root ? 0 : nd.ku, r = min(rc, sl.r - j0);
  double* Cl = sl.C + nd.row0 + (int64_t)j0 * sl.ldc;
  double* cn = sl.colnorm2 ? sl.colnorm2 + j0 : nullptr;
  if (ku > 0) {
    block_rows_times_cols(nd.U, m, ku, (const double*)sl.ws + nd.wf + (int64_t)j0 * sl.ldws, sl.ldws, r, Xs, part,
                          sl.alpha, 0.0, nullptr, 0, Cl, sl.ldc, true, cn);
  } else if (cn != nullptr) {
    for (int j = threadIdx.x >> 5; j < r; j += NW) {
      double s = 0.0;
      for (int i = threadIdx.x & 31; i < m; i += 32) {
        const double c = Cl[i + (int64_t)j * sl.ldc];
        s = fma(c, c, s);
      }
      s = warp_sum(s);
      if ((threadIdx.x & 31) == 0) atomicAdd(cn + j, s);
    }
  }
}

// ---------------------------------------------------------------------------
// ULV factorization (src/ulvfactor.jl:22-96, factor-only split of
// src/ulvdivide.jl:58-85)
// ---------------------------------------------------------------------------

// QL of U (m x k, k < m) with Q^T applied to D (m x n): geqlf!/ormql! (:39-41).
template <typename T>
__device__ void ql_sweep(T* U, T* D, T* tq, int m, int n, int k, T* red) {
  const int mk = m - k;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  __shared__ T sh[3];
  for (int c = k - 1; c >= 0; --c) {
    const int p = mk + c;
    T* u = U + (int64_t)c * m;
    T ss = T(0);
    for (int i = tid; i < p; i += NT) ss += u[i] * u[i];
    ss = block_sum(ss, red);
    if (tid == 0) {
      T beta, tau, scal;
      householder(u[p], ss, beta, tau, scal);
      sh[0] = beta; sh[1] = tau; sh[2] = scal;
    }
    __syncthreads();
    const T tau = sh[1], scal = sh[2];
    if (tau != T(0))
      for (int i = tid; i < p; i += NT) u[i] *= scal;
    __syncthreads();
    if (tid == 0) { u[p] = sh[0]; tq[c] = tau; }
    if (tau == T(0)) { __syncthreads(); continue; }
    const int ncols = c + n;
    for (int jj = warp; jj < ncols; jj += NW) {
      T* col = (jj < c) ? U + (int64_t)jj * m : D + (int64_t)(jj - c) * m;
      T w = T(0);
      for (int i = lane; i < p; i += 32) w += u[i] * col[i];
      w = warp_sum(w);
      w = (w + col[p]) * tau;
      __syncwarp();
      for (int i = lane; i < p; i += 32) col[i] -= w * u[i];
      if (lane == 0) col[p] -= w;
    }
    __syncthreads();
  }
}

// LQ of D[0:mk, :] with C Q^T applied to D[mk:m, :] and Q V to V (n x kv):
// gelqf!/ormlq! (src/ulvfactor.jl:44-50).
template <typename T>
__device__ void lq_sweep(T* D, T* V, T* tl, int m, int n, int mk, int kv, T* red) {
  const int nl = min(mk, n);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  __shared__ T sh[3];
  for (int i = 0; i < nl; ++i) {
    T ss = T(0);
    for (int l = i + 1 + tid; l < n; l += NT) {
      const T x = D[i + (int64_t)l * m];
      ss += x * x;
    }
    ss = block_sum(ss, red);
    if (tid == 0) {
      T beta, tau, scal;
      householder(D[i + (int64_t)i * m], ss, beta, tau, scal);
      sh[0] = beta; sh[1] = tau; sh[2] = scal;
    }
    __syncthreads();
    const T tau = sh[1], scal = sh[2];
    if (tau != T(0))
      for (int l = i + 1 + tid; l < n; l += NT) D[i + (int64_t)l * m] *= scal;
    __syncthreads();
    if (tid == 0) { D[i + (int64_t)i * m] = sh[0]; tl[i] = tau; }
    if (tau == T(0)) { __syncthreads(); continue; }
    const T* v = D + i;   // v[l*m] for l > i, implicit 1 at l = i
    for (int j = i + 1 + tid; j < m; j += NT) {
      T w = D[j + (int64_t)i * m];
      for (int l = i + 1; l < n; ++l) w += D[j + (int64_t)l * m] * v[(int64_t)l * m];
      w *= tau;
      D[j + (int64_t)i * m] -= w;
      for (int l = i + 1; l < n; ++l) D[j + (int64_t)l * m] -= w * v[(int64_t)l * m];
    }
    for (int c = warp; c < kv; c += NW) {
      T* vc = V + (int64_t)c * n;
      T w = T(0);
      for (int l = i + 1 + lane; l < n; l += 32) w += v[(int64_t)l * m] * vc[l];
      w = warp_sum(w);
      w = (w + vc[i]) * tau;
      __syncwarp();
      if (lane == 0) vc[i] -= w;
      for (int l = i + 1 + lane; l < n; l += 32) vc[l] -= w * v[(int64_t)l * m];
    }
    __syncthreads();
  }
}

// LU with partial pivoting of the root block (the dense `D \ b`, src/ulvfactor.jl:82-83).
template <typename T>
__device__ void lu_factor(T* A, int m, int32_t* piv, int32_t* err) {
  __shared__ T bv[NW];
  __shared__ int bi[NW];
  __shared__ int pivot_row;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int c = 0; c < m; ++c) {
    T best = T(-1);
    int idx = m;
    for (int i = c + tid; i < m; i += NT) {
      const T a = dabs(A[i + (int64_t)c * m]);
      if (a > best) { best = a; idx = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
      if (ob > best || (ob == best && oi < idx)) { best = ob; idx = oi; }
    }
    if (lane == 0) { bv[warp] = best; bi[warp] = idx; }
    __syncthreads();
    if (tid == 0) {
      T b = bv[0];
      int ix = bi[0];
      for (int w = 1; w < NW; ++w)
        if (bv[w] > b || (bv[w] == b && bi[w] < ix)) { b = bv[w]; ix = bi[w]; }
      if (ix >= m) ix = c;
      pivot_row = ix;
      piv[c] = ix;
      if (A[ix + (int64_t)c * m] == T(0) && err != nullptr) atomicExch(err, DEV_SINGULAR);
    }
    __syncthreads();
    const int p = pivot_row;
    if (p != c) {
      for (int j = tid; j < m; j += NT) {
        const T t = A[c + (int64_t)j * m];
        A[c + (int64_t)j * m] = A[p + (int64_t)j * m];
        A[p + (int64_t)j * m] = t;
      }
    }
    __syncthreads();
    const T d = A[c + (int64_t)c * m];
    if (d != T(0))
      for (int i = c + 1 + tid; i < m; i += NT) A[i + (int64_t)c * m] /= d;
    __syncthreads();
    const int rem = m - c - 1;
    for (int o = tid; o < rem * rem; o += NT) {
      const int i = c + 1 + o % rem, j = c + 1 + o / rem;
      A[i + (int64_t)j * m] -= A[i + (int64_t)c * m] * A[c + (int64_t)j * m];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(NT) ulv_factor_kernel(const Task* __restrict__ tasks,
                                                        const Slot* __restrict__ slots) {
  __shared__ T red[NW];
  const Task tk = tasks[blockIdx.x];
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* fb = (T*)sl.fbase;
  const int m = nd.m, n = nd.n, ku = nd.ku, kv = nd.kv;
  T* D = fb + nd.fD;
  T* U = fb + nd.fU;
  T* V = fb + nd.fV;
  const int tid = threadIdx.x;
  if (nd.leaf) {
    // copy D, U, V (src/ulvfactor.jl:63)
    for (int64_t e = tid; e < (int64_t)m * n; e += NT) D[e] = (T)nd.D[e];
    if (!nd.root) {
      for (int64_t e = tid; e < (int64_t)m * ku; e += NT) U[e] = (T)nd.U[e];
      for (int64_t e = tid; e < (int64_t)n * kv; e += NT) V[e] = (T)nd.V[e];
    }
  } else {
    // merge the children's reduced blocks (src/ulvfactor.jl:74-79)
    const Node& c1 = nodes[nd.left];
    const Node& c2 = nodes[nd.right];
    const T* D1 = fb + c1.fD + c1.mk + (int64_t)c1.nk * c1.m;
    const T* D2 = fb + c2.fD + c2.mk + (int64_t)c2.nk * c2.m;
    const T* U1 = fb + c1.fU + c1.mk;
    const T* U2 = fb + c2.fU + c2.mk;
    const T* V1 = fb + c1.fV + c1.nk;
    const T* V2 = fb + c2.fV + c2.nk;
    T* T12 = fb + nd.fT12;
    T* T21 = fb + nd.fT21;
    // T12 = U1 B12 (mr1 x kv2), T21 = U2 B21 (mr2 x kv1); U1, U2 tril when reduced
    for (int o = tid; o < c1.mr * c2.kv; o += NT) {
      const int i = o % c1.mr, j = o / c1.mr;
      const int lmax = c1.lower_u ? min(i + 1, c1.ku) : c1.ku;
      T s = T(0);
      for (int l = 0; l < lmax; ++l) s += U1[i + (int64_t)l * c1.m] * (T)nd.B12[l + (int64_t)j * c1.ku];
      T12[i + (int64_t)j * c1.mr] = s;
    }
    for (int o = tid; o < c2.mr * c1.kv; o += NT) {
      const int i = o % c2.mr, j = o / c2.mr;
      const int lmax = c2.lower_u ? min(i + 1, c2.ku) : c2.ku;
      T s = T(0);
      for (int l = 0; l < lmax; ++l) s += U2[i + (int64_t)l * c2.m] * (T)nd.B21[l + (int64_t)j * c2.ku];
      T21[i + (int64_t)j * c2.mr] = s;
    }
    if (!nd.root) {
      for (int o = tid; o < m * ku; o += NT) {
        const int i = o % m, j = o / m;
        T s = T(0);
        if (i < c1.mr) {
          const int lmax = c1.lower_u ? min(i + 1, c1.ku) : c1.ku;
          for (int l = 0; l < lmax; ++l) s += U1[i + (int64_t)l * c1.m] * (T)nd.R1[l + (int64_t)j * c1.ku];
        } else {
          const int i2 = i - c1.mr;
          const int lmax = c2.lower_u ? min(i2 + 1, c2.ku) : c2.ku;
          for (int l = 0; l < lmax; ++l) s += U2[i2 + (int64_t)l * c2.m] * (T)nd.R2[l + (int64_t)j * c2.ku];
        }
        U[i + (int64_t)j * m] = s;
      }
      for (int o = tid; o < n * kv; o += NT) {
        const int i = o % n, j = o / n;
        T s = T(0);
        if (i < c1.nr) {
          for (int l = 0; l < c1.kv; ++l) s += V1[i + (int64_t)l * c1.n] * (T)nd.W1[l + (int64_t)j * c1.kv];
        } else {
          const int i2 = i - c1.nr;
          for (int l = 0; l < c2.kv; ++l) s += V2[i2 + (int64_t)l * c2.n] * (T)nd.W2[l + (int64_t)j * c2.kv];
        }
        V[i + (int64_t)j * n] = s;
      }
    }
    __syncthreads();
    for (int o = tid; o < m * n; o += NT) {
      const int i = o % m, j = o / m;
      T val;
      if (i < c1.mr) {
        if (j < c1.nr) {
          val = D1[i + (int64_t)j * c1.m];
        } else {
          const int j2 = j - c1.nr;
          T s = T(0);
          for (int l = 0; l < c2.kv; ++l) s += T12[i + (int64_t)l * c1.mr] * V2[j2 + (int64_t)l * c2.n];
          val = s;
        }
      } else {
        const int i2 = i - c1.mr;
        if (j < c1.nr) {
          T s = T(0);
          for (int l = 0; l < c1.kv; ++l) s += T21[i2 + (int64_t)l * c2.mr] * V1[j + (int64_t)l * c1.n];
          val = s;
        } else {
          val = D2[i2 + (int64_t)(j - c1.nr) * c2.m];
        }
      }
      D[i + (int64_t)j * m] = val;
    }
  }
  __syncthreads();
  if (nd.root) {
    lu_factor(D, m, (int32_t*)(fb + nd.fpiv), sl.err);
    return;
  }
  if (nd.mk == 0) return;   // k >= m: nothing to eliminate (src/ulvfactor.jl:32-36)
  ql_sweep(U, D, fb + nd.ftq, m, n, nd.k, red);
  lq_sweep(D, V, fb + nd.ftl, m, n, nd.mk, kv, red);
  __syncthreads();
  T* Qt = fb + nd.fQt;
  for (int e = tid; e < nd.mk * n; e += NT) {
    const int col = e % n, i = e / n;
    Qt[col + (int64_t)i * n] = col < i ? T(0) : (col == i ? T(1) : D[i + (int64_t)col * m]);
  }
}

// ---------------------------------------------------------------------------
// ULV solve: upward (b, u, zloc per node) and downward (Q_lq^T, scatter)
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(NT) ulv_solve_up_kernel(const Task* __restrict__ tasks,
                                                          const Slot* __restrict__ slots) {
  const Task tk = tasks[blockIdx.x];
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* ws = (T*)sl.ws;
  const int64_t ld = sl.ldws;
  const T* fb = (const T*)sl.fbase;
  const int m = nd.m, n = nd.n, kv = nd.kv, r = sl.r;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* b = ws + nd.wb;
  T* u = ws + nd.wu;
  if (nd.leaf) {
    for (int o = tid; o < m * r; o += NT) {
      const int i = o % m, j = o / m;
      const double bv = sl.B[nd.row0 + i + (int64_t)j * sl.ldb];
      b[i + j * ld] = sl.colinv ? (T)(bv * sl.colinv[j]) : (T)bv;
    }
  } else {
    // b = [b1; b2] - [U1 B12 u2; U2 B21 u1] (src/ulvfactor.jl:74)
    const Node& c1 = nodes[nd.left];
    const Node& c2 = nodes[nd.right];
    const T* T12 = fb + nd.fT12;
    const T* T21 = fb + nd.fT21;
    const T* b1 = ws + c1.wb + c1.mk;
    const T* b2 = ws + c2.wb + c2.mk;
    const T* u1 = ws + c1.wu;
    const T* u2 = ws + c2.wu;
    for (int o = tid; o < m * r; o += NT) {
      const int i = o % m, j = o / m;
      T s;
      if (i < c1.mr) {
        s = b1[i + j * ld];
        for (int l = 0; l < c2.kv; ++l) s -= T12[i + (int64_t)l * c1.mr] * u2[l + j * ld];
      } else {
        const int i2 = i - c1.mr;
        s = b2[i2 + j * ld];
        for (int l = 0; l < c1.kv; ++l) s -= T21[i2 + (int64_t)l * c2.mr] * u1[l + j * ld];
      }
      b[i + j * ld] = s;
    }
    if (!nd.root) {
      // u accumulates W1^T u1 + W2^T u2 (src/ulvfactor.jl:89)
      for (int o = tid; o < kv * r; o += NT) {
        const int c = o % kv, j = o / kv;
        T s = T(0);
        for (int l = 0; l < c1.kv; ++l) s += (T)nd.W1[l + (int64_t)c * c1.kv] * u1[l + j * ld];
        for (int l = 0; l < c2.kv; ++l) s += (T)nd.W2[l + (int64_t)c * c2.kv] * u2[l + j * ld];
        u[c + j * ld] = s;
      }
    }
  }
  __syncthreads();
  if (nd.root) {
    // z[cols] = D \ b with the stored LU (src/ulvfactor.jl:83)
    const T* A = fb + nd.fD;
    const int32_t* piv = (const int32_t*)(fb + nd.fpiv);
    T* x = ws + nd.wx;
    for (int j = warp; j < r; j += NW) {
      T* bj = b + j * ld;
      if (lane == 0)
        for (int c = 0; c < m; ++c) {
          const int p = piv[c];
          if (p != c) { const T t = bj[c]; bj[c] = bj[p]; bj[p] = t; }
        }
      __syncwarp();
      for (int c = 0; c < m; ++c) {
        const T xc = bj[c];
        __syncwarp();
        for (int i = c + 1 + lane; i < m; i += 32) bj[i] -= A[i + (int64_t)c * m] * xc;
        __syncwarp();
      }
      for (int c = m - 1; c >= 0; --c) {
        const T xc = bj[c] / A[c + (int64_t)c * m];
        __syncwarp();
        if (lane == 0) bj[c] = xc;
        for (int i = lane; i < c; i += 32) bj[i] -= A[i + (int64_t)c * m] * xc;
        __syncwarp();
      }
      for (int i = lane; i < m; i += 32) x[i + j * ld] = bj[i];
    }
    return;
  }
  if (nd.mk == 0) {
    // nothing eliminated: b passes up unchanged, u = 0 at a leaf (src/ulvfactor.jl:32-36)
    if (nd.leaf)
      for (int o = tid; o < kv * r; o += NT) u[(o % kv) + (o / kv) * ld] = T(0);
    return;
  }
  const int k = nd.k, mk = nd.mk, nk = nd.nk;
  const T* Uf = fb + nd.fU;
  const T* tq = fb + nd.ftq;
  const T* Df = fb + nd.fD;
  const T* Vf = fb + nd.fV;
  for (int j = warp; j < r; j += NW) {
    T* bj = b + j * ld;
    // b <- Q_ql^T b (src/ulvfactor.jl:42)
    for (int c = k - 1; c >= 0; --c) {
      const T tau = tq[c];
      if (tau == T(0)) continue;
      const int p = mk + c;
      const T* v = Uf + (int64_t)c * m;
      T w = T(0);
      for (int i = lane; i < p; i += 32) w += v[i] * bj[i];
      w = warp_sum(w);
      w = (w + bj[p]) * tau;
      __syncwarp();
      for (int i = lane; i < p; i += 32) bj[i] -= w * v[i];
      if (lane == 0) bj[p] -= w;
      __syncwarp();
    }
    // zloc = L1 \ b[0:mk] (trsm, src/ulvfactor.jl:48)
    for (int c = 0; c < mk; ++c) {
      const T xc = bj[c] / Df[c + (int64_t)c * m];
      __syncwarp();
      if (lane == 0) bj[c] = xc;
      for (int i = c + 1 + lane; i < mk; i += 32) bj[i] -= Df[i + (int64_t)c * m] * xc;
      __syncwarp();
    }
  }
  __syncthreads();
  // b_red = b[mk:m] - L2[:, 0:nk] zloc (:49); u += V[0:mk,:]^T zloc (:51); z[cols[0:mk]] = zloc (:65)
  for (int o = tid; o < k * r; o += NT) {
    const int i = o % k, j = o / k;
    T s = b[mk + i + j * ld];
    for (int l = 0; l < nk; ++l) s -= Df[mk + i + (int64_t)l * m] * b[l + j * ld];
    b[mk + i + j * ld] = s;
  }
  for (int o = tid; o < kv * r; o += NT) {
    const int c = o % kv, j = o / kv;
    T s = nd.leaf ? T(0) : u[c + j * ld];
    for (int l = 0; l < nk; ++l) s += Vf[l + (int64_t)c * n] * b[l + j * ld];
    u[c + j * ld] = s;
  }
  T* x = ws + nd.wx;
  for (int o = tid; o < mk * r; o += NT) {
    const int i = o % mk, j = o / mk;
    x[i + j * ld] = b[i + j * ld];
  }
}

template <typename T>
__global__ void __launch_bounds__(NT) ulv_solve_down_kernel(const Task* __restrict__ tasks,
                                                            const Slot* __restrict__ slots) {
  const Task tk = tasks[blockIdx.x];
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* ws = (T*)sl.ws;
  const int64_t ld = sl.ldws;
  const T* fb = (const T*)sl.fbase;
  const int m = nd.m, n = nd.n, r = sl.r;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* x = ws + nd.wx;
  if (!nd.root && nd.mk > 0) {
    // z[cols] = Q_lq^T z[cols] (src/ulvfactor.jl:98-107)
    const T* Df = fb + nd.fD;
    const T* tl = fb + nd.ftl;
    const int nl = min(nd.mk, n);
    for (int j = warp; j < r; j += NW) {
      T* xj = x + j * ld;
      for (int i = nl - 1; i >= 0; --i) {
        const T tau = tl[i];
        if (tau == T(0)) continue;
        T w = T(0);
        for (int l = i + 1 + lane; l < n; l += 32) w += Df[i + (int64_t)l * m] * xj[l];
        w = warp_sum(w);
        w = (w + xj[i]) * tau;
        __syncwarp();
        if (lane == 0) xj[i] -= w;
        for (int l = i + 1 + lane; l < n; l += 32) xj[l] -= w * Df[i + (int64_t)l * m];
        __syncwarp();
      }
    }
    __syncthreads();
  }
  if (nd.leaf) {
    for (int o = tid; o < n * r; o += NT) {
      const int i = o % n, j = o / n;
      const double s = sl.colscale ? sl.colscale[j] : 1.0;
      const double v = s * (double)x[i + j * ld];
      double* out = sl.C + nd.col0 + i + (int64_t)j * sl.ldc;
      if (sl.mode) *out += v;
      else *out = v;
    }
  } else {
    const Node& c1 = nodes[nd.left];
    const Node& c2 = nodes[nd.right];
    for (int o = tid; o < n * r; o += NT) {
      const int i = o % n, j = o / n;
      const T v = x[i + j * ld];
      if (i < c1.nr) ws[c1.wx + c1.nk + i + j * ld] = v;
      else ws[c2.wx + c2.nk + (i - c1.nr) + j * ld] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------

__global__ void colnorm2_kernel(const double* __restrict__ B, int64_t ldb, int64_t n, int64_t r,
                                double* __restrict__ out) {
  const int64_t j = blockIdx.y;
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    const double v = B[i + j * ldb];
    s = fma(v, v, s);
  }
  __shared__ double red[NW];
  s = block_sum(s, red);
  if (threadIdx.x == 0) atomicAdd(out + j, s);
}

__global__ void sqrt_scale_kernel(const double* __restrict__ n2, double* __restrict__ s, int64_t r) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < r; j += (int64_t)gridDim.x * blockDim.x) {
    const double v = n2[j];
    const double sc = v > 0.0 ? sqrt(v) : 1.0;
    s[j] = sc;
    s[r + j] = 1.0 / sc;
  }
}

// Convergence check of the refinement loop on the device (one block): the
// largest relative residual over all columns, ||r_j|| / ||b_j|| (||r_j|| where
// b_j = 0), written to `st`, and the condition of the enclosing while node set
// to 1 when another step follows: not converged, no NaN, fewer than maxit steps
// taken and no device error in any slot.  `next` grows by one per continued
// step, so the loop ends after at most maxit steps.
__global__ void refine_check_kernel(const double* __restrict__ bn2, const double* __restrict__ rn2, int64_t r,
                                    double tol, int32_t maxit, RefineStatus* st, const Slot* __restrict__ slots,
                                    int32_t nslots, cudaGraphConditionalHandle cond) {
  __shared__ double s_max[NT];
  __shared__ int s_nan[NT];
  double m = 0.0;
  int nan = 0;
  for (int64_t j = threadIdx.x; j < r; j += blockDim.x) {
    const double bn = sqrt(bn2[j]), rn = sqrt(rn2[j]);
    const double rel = bn > 0.0 ? rn / bn : rn;
    if (isnan(rel)) nan = 1;
    else m = fmax(m, rel);
  }
  s_max[threadIdx.x] = m;
  s_nan[threadIdx.x] = nan;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s_max[threadIdx.x] = fmax(s_max[threadIdx.x], s_max[threadIdx.x + w]);
      s_nan[threadIdx.x] |= s_nan[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int err = 0;
    for (int32_t i = 0; i < nslots; ++i)
      if (slots[i].err && *(const volatile int32_t*)slots[i].err != DEV_OK) err = 1;
    const double res = s_nan[0] ? __longlong_as_double(0x7ff8000000000000ll) : s_max[0];
    const int it = st->next;
    const int conv = (!s_nan[0] && res <= tol) ? 1 : 0;
    const int more = (!conv && !s_nan[0] && !err && it < maxit) ? 1 : 0;
    st->residual = res;
    st->iterations = it;
    st->converged = conv;
    st->next = it + more;
    cudaGraphSetConditional(cond, (unsigned)more);
  }
}

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------

// Leaf products: one thread block per (leaf, 8 right-hand sides) once r >= 16.
static int leaf_chunk(int rmax) { return rmax >= 16 ? 8 : (rmax > 0 ? rmax : 1); }

void launch_mv_leaf(const Task* t, int64_t nt, const Slot* s, int rmax, cudaStream_t st) {
  const int rc = leaf_chunk(rmax), nchunk = (rmax + rc - 1) / rc;
  if (nt > 0 && nchunk > 0) mv_leaf_kernel<<<(unsigned)(nt * nchunk), NT, 0, st>>>(t, s, rc, nchunk);
}
void launch_mv_leaf_final(const Task* t, int64_t nt, const Slot* s, int rmax, cudaStream_t st) {
  const int rc = leaf_chunk(rmax), nchunk = (rmax + rc - 1) / rc;
  if (nt > 0 && nchunk > 0) mv_leaf_final_kernel<<<(unsigned)(nt * nchunk), NT, 0, st>>>(t, s, rc, nchunk);
}
void launch_mv_up(const Task* t, int64_t nt, const Slot* s, cudaStream_t st) {
  if (nt > 0) mv_up_kernel<<<(unsigned)nt, NT, 0, st>>>(t, s);
}
void launch_mv_down(const Task* t, int64_t nt, const Slot* s, cudaStream_t st) {
  if (nt > 0) mv_down_kernel<<<(unsigned)nt, NT, 0, st>>>(t, s);
}

// Right-hand sides per thread block of the staged translator sweeps: small
// chunks spread the few nodes of the upper levels over more SMs.
constexpr int MV_RC_BLOCK = 8;

size_t mv_up_staged_smem(int kv, int k1max, int k2max) {
  return sizeof(double) * ((size_t)kv * (k1max + k2max) + (size_t)(k1max + k2max) * MV_RC_BLOCK);
}
size_t mv_down_staged_smem(int ku, int u1, int u2, int v1, int v2) {
  return sizeof(double) * ((size_t)u1 * v2 + (size_t)u2 * v1 + (size_t)(u1 + u2) * ku +
                           (size_t)(v1 + v2 + ku) * MV_RC_BLOCK);
}
void launch_mv_up_staged(const Task* t, int64_t nt, const Slot* s, size_t smem, int rmax, cudaStream_t st) {
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(mv_up_staged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    set = true;
  }
  const int nchunk = (rmax + MV_RC_BLOCK - 1) / MV_RC_BLOCK;
  if (nt > 0 && nchunk > 0) mv_up_staged_kernel<<<(unsigned)(nt * nchunk), NT, smem, st>>>(t, s, MV_RC_BLOCK, nchunk);
}
void launch_mv_down_staged(const Task* t, int64_t nt, const Slot* s, size_t smem, int rmax, cudaStream_t st) {
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(mv_down_staged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    set = true;
  }
  const int nchunk = (rmax + MV_RC_BLOCK - 1) / MV_RC_BLOCK;
  if (nt > 0 && nchunk > 0) mv_down_staged_kernel<<<(unsigned)(nt * nchunk), NT, smem, st>>>(t, s, MV_RC_BLOCK, nchunk);
}

template <typename T>
void launch_ulv_factor(const Task* t, int64_t nt, const Slot* s, int, int, cudaStream_t st) {
  if (nt > 0) ulv_factor_kernel<T><<<(unsigned)nt, NT, 0, st>>>(t, s);
}
template <typename T>
void launch_ulv_solve_up(const Task* t, int64_t nt, const Slot* s, cudaStream_t st) {
  if (nt > 0) ulv_solve_up_kernel<T><<<(unsigned)nt, NT, 0, st>>>(t, s);
}
template <typename T>
void launch_ulv_solve_down(const Task* t, int64_t nt, const Slot* s, cudaStream_t st) {
  if (nt > 0) ulv_solve_down_kernel<T><<<(unsigned)nt, NT, 0, st>>>(t, s);
}

template void launch_ulv_factor<double>(const Task*, int64_t, const Slot*, int, int, cudaStream_t);
template void launch_ulv_factor<float>(const Task*, int64_t, const Slot*, int, int, cudaStream_t);
template void launch_ulv_solve_up<double>(const Task*, int64_t, const Slot*, cudaStream_t);
template void launch_ulv_solve_up<float>(const Task*, int64_t, const Slot*, cudaStream_t);
template void launch_ulv_solve_down<double>(const Task*, int64_t, const Slot*, cudaStream_t);
template void launch_ulv_solve_down<float>(const Task*, int64_t, const Slot*, cudaStream_t);

void launch_colnorm2(const double* B, int64_t ldb, int64_t n, int64_t r, double* out, cudaStream_t st) {
  if (n <= 0 || r <= 0) return;
  int64_t bx = (n + NT - 1) / NT;
  if (bx > 64) bx = 64;
  for (int64_t j0 = 0; j0 < r; j0 += 65535) {
    const int64_t rc = r - j0 < 65535 ? r - j0 : 65535;
    colnorm2_kernel<<<dim3((unsigned)bx, (unsigned)rc), NT, 0, st>>>(B + j0 * ldb, ldb, n, rc, out + j0);
  }
}
void launch_sqrt_scale(const double* n2, double* s, int64_t r, cudaStream_t st) {
  if (r <= 0) return;
  sqrt_scale_kernel<<<(unsigned)((r + 255) / 256), 256, 0, st>>>(n2, s, r);
}
void launch_refine_check(const double* bn2, const double* rn2, int64_t r, double tol, int32_t maxit,
                         RefineStatus* status, const Slot* slots, int32_t nslots, cudaGraphConditionalHandle cond,
                         cudaStream_t st) {
  refine_check_kernel<<<1, NT, 0, st>>>(bn2, rn2, r, tol, maxit, status, slots, nslots, cond);
}

}  // namespace hss
