// Randomized compression on the device (reference src/compression.jl:278-444).
//
//  * sample products S = A * Omega, S = A^T * Omega of the dense matrix
//    (:290-291, :326-327, :336-337): FP64 tiles, split over K when the tile
//    grid alone would not fill the GPU (partials reduced in a fixed order);
//    or the same tiles in double-float arithmetic on the FP32 pipe
//    (HSS_OPT_SAMPLE_DF), the mixed-precision form of the sampling;
//  * leaf corrections S_i -= D_i * Omega_i, S_i -= D_i^T * Omega_i (:360-361),
//    D_i addressed in place inside A (hss_blkdiag, :447-475, needs no copy);
//  * the tree pass of `_randcompress!` (:358-430), one launch per tree level,
//    one thread block per (node, side): assembles the node's sample (branch:
//    S1 - B12 * Omega2, S2 - B21 * Omega1 with B gathered from A at the
//    children's selected rows/columns, :394-398), takes its interpolative
//    decomposition (`_interpolate`, :433-444: QR with column pivoting in FP64,
//    rank = #{|R_jj| > min(atol, rtol |R_11|)}, X = R11^{-1} [R11 R12] P^T),
//    writes the generator X^T (U, V or [R1; R2], [W1; W2]), the selected
//    indices J, the reduced sample S[J, :] and the reduced test matrix
//    X * Omega (the V' * Omega, U' * Omega of :384-387).  Ranks stay on the
//    device; the host reads them once, after the root.
//
// The pivoted QR follows LAPACK xLAQP2 (the unblocked kernel of xGEQP3 that
// Julia's qr(A, ColumnNorm()) calls): pivot = first column of largest
// partial norm, Householder reflector by xLARFG, partial norms downdated
// with the Drmac-Bujanovic safeguard (recomputed when the downdate loses
// more than half the digits).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "hss_df.cuh"
#include "hss_device.cuh"
#include "hss_sample.h"

namespace hss {

namespace {

// ---------------------------------------------------------------------------
// dense sample product
// ---------------------------------------------------------------------------

constexpr int GT = 256;   // threads
constexpr int TM = 64;    // output rows per block (2 per lane)
constexpr int TN = 32;    // output columns per block (4 per warp)
constexpr int TK = 16;    // K panel

struct GemmProblem {
  const double* A;
  int64_t lda;
  const double* X;
  int64_t ldx;
  double* Y;
  int64_t ldy;
  int64_t m, k, r;
};

// acc = op(A)(rows row0.., k in [k0, k1)) * X(k0..k1, cols col0..); warps whose
// four columns lie beyond r skip the FMAs (no work on padding columns).
__device__ __forceinline__ void gemm_tile_acc(const GemmProblem& p, int trans, int64_t row0, int64_t col0,
                                              int64_t k0, int64_t k1, double (*As)[TM + 1],
                                              double (*Xs)[TN + 1], double acc[2][4]) {
  const int tid = threadIdx.x;
  const int tr = tid & 31, tc = tid >> 5;
  const bool active = col0 + tc * 4 < p.r;
  for (int64_t kb = k0; kb < k1; kb += TK) {
    for (int e = tid; e < TK * TM; e += GT) {
      int i, kk;
      if (!trans) { i = e % TM; kk = e / TM; }   // consecutive threads walk A's rows
      else { kk = e % TK; i = e / TK; }          // consecutive threads walk A's columns
      const int64_t gi = row0 + i, gk = kb + kk;
      double v = 0.0;
      if (gi < p.m && gk < k1) v = trans ? p.A[gk + gi * p.lda] : p.A[gi + gk * p.lda];
      As[kk][i] = v;
    }
    for (int e = tid; e < TK * TN; e += GT) {
      const int kk = e % TK, j = e / TK;
      const int64_t gk = kb + kk, gj = col0 + j;
      Xs[kk][j] = (gk < k1 && gj < p.r) ? p.X[gk + gj * p.ldx] : 0.0;
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int kk = 0; kk < TK; ++kk) {
        const double a0 = As[kk][tr], a1 = As[kk][tr + 32];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const double x = Xs[kk][tc * 4 + b];
          acc[0][b] = fma(a0, x, acc[0][b]);
          acc[1][b] = fma(a1, x, acc[1][b]);
        }
      }
    }
    __syncthreads();
  }
}

// ksplit == 1: Y = alpha * acc + beta * Y.  ksplit > 1: partial z of the
// K range goes to P + z * m * r (ld m); sample_reduce_kernel finishes.
__global__ void __launch_bounds__(GT) sample_gemm_kernel(GemmProblem p, int trans, double alpha, double beta,
                                                         int64_t kchunk, double* P) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Xs[TK][TN + 1];
  const int64_t row0 = (int64_t)blockIdx.x * TM, col0 = (int64_t)blockIdx.y * TN;
  const int64_t k0 = (int64_t)blockIdx.z * kchunk, k1 = min(p.k, k0 + kchunk);
  double acc[2][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  gemm_tile_acc(p, trans, row0, col0, k0, k1, As, Xs, acc);
  const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const int64_t gi = row0 + tr + 32 * a;
    if (gi >= p.m) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t gj = col0 + tc * 4 + b;
      if (gj >= p.r) continue;
      if (P) {
        P[(int64_t)blockIdx.z * p.m * p.r + gi + gj * p.m] = acc[a][b];
      } else {
        double* y = p.Y + gi + gj * p.ldy;
        *y = beta == 0.0 ? alpha * acc[a][b] : fma(alpha, acc[a][b], beta * *y);
      }
    }
  }
}

__global__ void sample_reduce_kernel(const double* __restrict__ P, int nsplit, int64_t m, int64_t r, double* Y,
                                     int64_t ldy, double alpha, double beta) {
  const int64_t tot = m * r;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int z = 0; z < nsplit; ++z) acc += P[z * tot + e];
    const int64_t i = e % m, j = e / m;
    double* y = Y + i + j * ldy;
    *y = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *y);
  }
}

// ---------------------------------------------------------------------------
// double-float sample product
// ---------------------------------------------------------------------------

// Double-float sample product: A and X split into float pairs as they are
// staged, every product accumulated by df_fma (exact FMA product error,
// TwoSum accumulation): ~2^-47 per operation instead of FP64's 2^-53.
// Partials and the alpha/beta epilogue are FP64 (hi + lo is exact there).
// Row-per-thread tiles for the narrow samples of randcompress (s = kest +
// noversampling, stepsize: 20 columns by default): a block covers DR rows x
// NC columns, each thread one row and all NC columns, so no warp idles when s
// is not a multiple of 32.  K panels of TK as above.  With lrow/lin (leaf
// index of every row / inner index of op(A)), entries whose row and inner
// index lie in the same leaf are skipped: the product of A minus its diagonal
// leaf blocks, whose FP64 part is added separately.
constexpr int DR = 256;

// 8-byte asynchronous copy global -> shared; src_bytes = 0 zero-fills (src
// must still be a valid address).
__device__ __forceinline__ void cp8z(void* s, const void* g, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"((unsigned)__cvta_generic_to_shared(s)),
               "l"(g), "r"(src_bytes)
               : "memory");
}

// Shared memory: two raw FP64 panels of op(A) (TK x DR) and of X (TK x NC),
// the split X panel, the leaf indices of the panel's inner index.
template <int NC>
constexpr size_t dfrows_smem() {
  return (size_t)2 * TK * DR * 8 + (size_t)2 * TK * NC * 8 + (size_t)TK * NC * 8 + (size_t)2 * TK * 4;
}

// The next panel's copies are in flight while the current one is used; A is
// split into its float pair where it is used (each element by one thread),
// X once per panel (every thread uses every element).
template <int NC>
__global__ void __launch_bounds__(GT) dfsample_rows_kernel(GemmProblem p, int trans, double alpha, double beta,
                                                           int64_t kchunk, double* P, const int32_t* lrow,
                                                           const int32_t* lin) {
  extern __shared__ __align__(16) unsigned char dfr_smem[];
  double (*Araw)[TK][DR] = (double (*)[TK][DR])dfr_smem;                      // [2][TK][DR]
  double (*Xraw)[TK][NC] = (double (*)[TK][NC])(dfr_smem + 2 * TK * DR * 8);  // [2][TK][NC]
  float2 (*Xs)[NC] = (float2 (*)[NC])(dfr_smem + 2 * TK * DR * 8 + 2 * TK * NC * 8);
  int32_t (*Ls)[TK] = (int32_t (*)[TK])(dfr_smem + 2 * TK * DR * 8 + 3 * TK * NC * 8);
  const int64_t row0 = (int64_t)blockIdx.x * DR, col0 = (int64_t)blockIdx.y * NC;
  const int64_t k0 = (int64_t)blockIdx.z * kchunk, k1 = min(p.k, k0 + kchunk);
  const int tid = threadIdx.x;
  const int64_t gi = row0 + tid;
  const int32_t myleaf = (lrow && gi < p.m) ? __ldg(lrow + gi) : -1;
  auto issue = [&](int64_t kb, int buf) {
    for (int e = tid; e < TK * DR; e += GT) {
      int i, kk;
      if (!trans) { i = e % DR; kk = e / DR; }   // consecutive threads walk A's rows
      else { kk = e % TK; i = e / TK; }          // consecutive threads walk A's columns
      const int64_t ri = row0 + i, gk = kb + kk;
      const bool ok = ri < p.m && gk < k1;
      const double* src = ok ? (trans ? p.A + gk + ri * p.lda : p.A + ri + gk * p.lda) : p.A;
      cp8z(&Araw[buf][kk][i], src, ok ? 8 : 0);
    }
    for (int e = tid; e < TK * NC; e += GT) {
      const int kk = e % TK, j = e / TK;
      const int64_t gk = kb + kk, gj = col0 + j;
      const bool ok = gk < k1 && gj < p.r;
      cp8z(&Xraw[buf][kk][j], ok ? p.X + gk + gj * p.ldx : p.X, ok ? 8 : 0);
    }
    if (tid < TK) Ls[buf][tid] = (lin && kb + tid < k1) ? __ldg(lin + kb + tid) : -2;
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  float ah[NC], al[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) ah[c] = al[c] = 0.f;
  int buf = 0;
  if (k0 < k1) issue(k0, 0);
  for (int64_t kb = k0; kb < k1; kb += TK, buf ^= 1) {
    if (kb + TK < k1) {
      issue(kb + TK, buf ^ 1);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();   // panel kb is in place; the previous panel's Xs is no longer read
    for (int e = tid; e < TK * NC; e += GT) Xs[e / NC][e % NC] = split_bits(Xraw[buf][e / NC][e % NC]);
    __syncthreads();
#pragma unroll(NC > 24 ? 1 : 2)
    for (int kk = 0; kk < TK; ++kk) {
      const double v = Araw[buf][kk][tid];
      const float2 a = split_bits(myleaf >= 0 && Ls[buf][kk] == myleaf ? 0.0 : v);
#pragma unroll
      for (int c = 0; c < NC; ++c) df_fma(ah[c], al[c], a, Xs[kk][c]);
    }
    __syncthreads();   // every thread is done with buffer buf before it is refilled
  }
  if (gi >= p.m) return;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int64_t gj = col0 + c;
    if (gj >= p.r) continue;
    const double acc = (double)ah[c] + (double)al[c];
    if (P) {
      P[(int64_t)blockIdx.z * p.m * p.r + gi + gj * p.m] = acc;
    } else {
      double* y = p.Y + gi + gj * p.ldy;
      *y = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *y);
    }
  }
}

template <int NC>
void launch_dfrows(dim3 grid, cudaStream_t st, const GemmProblem& p, int trans, double alpha, double beta,
                   int64_t kchunk, double* P, const int32_t* lrow, const int32_t* lin) {
  constexpr size_t smem = dfrows_smem<NC>();
  static bool attr = false;   // set once per instantiation (the size is a compile-time constant)
  if (!attr) {
    cudaFuncSetAttribute(dfsample_rows_kernel<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  dfsample_rows_kernel<NC><<<grid, GT, smem, st>>>(p, trans, alpha, beta, kchunk, P, lrow, lin);
}

// Block-diagonal product: problem z is the rows[z] x cols[z] block of A at
// (row0[z], col0[z]).  trans = 0: Y[row0.., :] = alpha * blk * X[col0.., :] +
// beta * Y[row0.., :]; trans = 1: Y[col0.., :] = alpha * blk^T * X[row0.., :] + beta * Y[col0.., :].
__global__ void __launch_bounds__(GT) blockdiag_gemm_kernel(const double* __restrict__ A, int64_t lda,
                                                            const int64_t* __restrict__ row0,
                                                            const int64_t* __restrict__ rows,
                                                            const int64_t* __restrict__ col0,
                                                            const int64_t* __restrict__ cols, int trans,
                                                            const double* X, int64_t ldx, int64_t r, double* Y,
                                                            int64_t ldy, double alpha, double beta) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Xs[TK][TN + 1];
  const int z = blockIdx.z;
  GemmProblem p;
  p.A = A + row0[z] + col0[z] * lda;
  p.lda = lda;
  if (!trans) {
    p.m = rows[z]; p.k = cols[z];
    p.X = X + col0[z]; p.Y = Y + row0[z];
  } else {
    p.m = cols[z]; p.k = rows[z];
    p.X = X + row0[z]; p.Y = Y + col0[z];
  }
  p.ldx = ldx; p.ldy = ldy; p.r = r;
  const int64_t r0 = (int64_t)blockIdx.x * TM, c0 = (int64_t)blockIdx.y * TN;
  if (r0 >= p.m) return;   // block-uniform: smaller blocks of the level
  double acc[2][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  gemm_tile_acc(p, trans, r0, c0, 0, p.k, As, Xs, acc);
  const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const int64_t gi = r0 + tr + 32 * a;
    if (gi >= p.m) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t gj = c0 + tc * 4 + b;
      if (gj >= p.r) continue;
      double* y = p.Y + gi + gj * p.ldy;
      *y = beta == 0.0 ? alpha * acc[a][b] : fma(alpha, acc[a][b], beta * *y);
    }
  }
}

// ---------------------------------------------------------------------------
// tree pass: interpolative decompositions, one block per (node, side)
// ---------------------------------------------------------------------------

constexpr int IT = 256;   // threads of the ID kernel

__device__ __forceinline__ void argmax_merge(double& v, int& i, double ov, int oi) {
  if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
}

__global__ void __launch_bounds__(IT) rc_id_kernel(RcArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int side = blockIdx.y;
  const int32_t xi = a.list[blockIdx.x];
  const RcNode& x = a.nodes[xi];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int64_t s = a.s;
  const double* A = a.A;
  const int64_t lda = a.lda;

  // children's ranks and selected indices (branches)
  int kc1 = 0, kc2 = 0, kr1 = 0, kr2 = 0;
  const RcNode* c1 = nullptr;
  const RcNode* c2 = nullptr;
  if (!x.leaf) {
    c1 = &a.nodes[x.left];
    c2 = &a.nodes[x.right];
    kc1 = a.rank[2 * x.left]; kr1 = a.rank[2 * x.left + 1];
    kc2 = a.rank[2 * x.right]; kr2 = a.rank[2 * x.right + 1];
    if (side == 0) {
      // B12 = A[Jc1, Jr2] (kc1 x kr2), B21 = A[Jc2, Jr1] (kc2 x kr1)  (:394-395)
      for (int e = tid; e < kc1 * kr2; e += nt) {
        const int q = e % kc1, t = e / kc1;
        x.B12[e] = A[c1->J[0][q] + c2->J[1][t] * lda];
      }
      for (int e = tid; e < kc2 * kr1; e += nt) {
        const int q = e % kc2, t = e / kc2;
        x.B21[e] = A[c2->J[0][q] + c1->J[1][t] * lda];
      }
    }
    if (x.root) return;   // the root keeps only B12, B21 (:400-409)
  } else if (x.root) {
    return;
  }

  // the node's sample S (p x s); row q of S belongs to index Jin(q) and to
  // row q of the test matrix Omega_in
  const int p = x.leaf ? (int)(side == 0 ? x.m : x.n) : (side == 0 ? kc1 + kc2 : kr1 + kr2);
  const int split = x.leaf ? p : (side == 0 ? kc1 : kr1);
  const int64_t lds = x.leaf ? x.lds[side] : p;
  double* S = x.S[side];
  auto jin = [&](int q) -> int64_t {
    if (x.leaf) return (side == 0 ? x.r0 : x.c0) + q;
    return q < split ? c1->J[side][q] : c2->J[side][q - split];
  };
  // side 0 reduces Omega_row (U' * Omega_row), side 1 reduces Omega_col (V' * Omega_col)
  auto omega_in = [&](int q, int64_t l) -> double {
    if (x.leaf) return side == 0 ? a.Orow[x.r0 + q + l * a.ldor] : a.Ocol[x.c0 + q + l * a.ldoc];
    return q < split ? c1->Or[side][q + l * s] : c2->Or[side][(q - split) + l * s];
  };

  const int ldm = (int)(s | 1);
  double* M;
  double* dyn = reinterpret_cast<double*>(smem_raw);
  if (a.m_in_smem) {
    M = dyn;
    dyn += (int64_t)ldm * a.pmax;
  } else {
    M = a.gscratch + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * (int64_t)ldm * a.pmax;
  }
  double* vn1 = dyn;
  double* vn2 = vn1 + a.pmax;
  double* red_v = vn2 + a.pmax;                       // 8 per-warp maxima + beta, tau
  int* perm = reinterpret_cast<int*>(red_v + 16);
  int* red_i = perm + a.pmax;                         // 8 per-warp argmax + pivot

  // ---- assemble S (branches: :397-398) and M = S^T ----
  if (x.leaf) {
    for (int64_t e = tid; e < (int64_t)p * s; e += nt) {
      const int q = (int)(e % p);
      const int64_t l = e / p;
      M[l + (int64_t)q * ldm] = S[q + l * lds];
    }
  } else {
    for (int64_t e = tid; e < (int64_t)p * s; e += nt) {
      const int q = (int)(e % p);
      const int64_t l = e / p;
      double acc = 0.0, v;
      if (side == 0) {
        if (q < kc1) {   // Scol1 - B12 * Omega_col2
          for (int t = 0; t < kr2; ++t) acc = fma(A[c1->J[0][q] + c2->J[1][t] * lda], c2->Or[1][t + l * s], acc);
          v = c1->Sr[0][q + l * s] - acc;
        } else {         // Scol2 - B21 * Omega_col1
          const int qq = q - kc1;
          for (int t = 0; t < kr1; ++t) acc = fma(A[c2->J[0][qq] + c1->J[1][t] * lda], c1->Or[1][t + l * s], acc);
          v = c2->Sr[0][qq + l * s] - acc;
        }
      } else {
        if (q < kr1) {   // Srow1 - B21' * Omega_row2
          for (int t = 0; t < kc2; ++t) acc = fma(A[c2->J[0][t] + c1->J[1][q] * lda], c2->Or[0][t + l * s], acc);
          v = c1->Sr[1][q + l * s] - acc;
        } else {         // Srow2 - B12' * Omega_row1
          const int qq = q - kr1;
          for (int t = 0; t < kc1; ++t) acc = fma(A[c1->J[0][t] + c2->J[1][qq] * lda], c1->Or[0][t + l * s], acc);
          v = c2->Sr[1][qq + l * s] - acc;
        }
      }
      S[q + l * p] = v;
      M[l + (int64_t)q * ldm] = v;
    }
  }
  __syncthreads();

  // ---- QR with column pivoting of M (s x p) ----
  for (int c = tid; c < p; c += nt) {
    double ss = 0.0;
    for (int64_t i = 0; i < s; ++i) ss = fma(M[i + (int64_t)c * ldm], M[i + (int64_t)c * ldm], ss);
    vn1[c] = sqrt(ss);
    vn2[c] = vn1[c];
    perm[c] = c;
  }
  __syncthreads();
  const int kmax = (int)(s < (int64_t)p ? s : (int64_t)p);
  const double tol3z = 1.0536712127723509e-08;   // sqrt(2^-53), LAPACK's sqrt(dlamch('Epsilon'))
  double tol = 0.0;
  int rk = 0;
  const int lane = tid & 31, warp = tid >> 5;
  for (int j = 0; j < kmax; ++j) {
    // pivot: first column of largest partial norm
    double bv = -1.0;
    int bi = p;
    for (int c = j + tid; c < p; c += nt) argmax_merge(bv, bi, vn1[c], c);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
      argmax_merge(bv, bi, __shfl_down_sync(0xffffffffu, bv, off), __shfl_down_sync(0xffffffffu, bi, off));
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      double v = red_v[0];
      int i = red_i[0];
      for (int w = 1; w < nt / 32; ++w) argmax_merge(v, i, red_v[w], red_i[w]);
      red_i[8] = i < p ? i : j;   // NaN norms never compare greater: keep column j
    }
    __syncthreads();
    const int piv = red_i[8];
    if (piv != j) {
      for (int64_t i = tid; i < s; i += nt) {
        const double t = M[i + (int64_t)j * ldm];
        M[i + (int64_t)j * ldm] = M[i + (int64_t)piv * ldm];
        M[i + (int64_t)piv * ldm] = t;
      }
      __syncthreads();   // every thread read vn1[j] during the argmax
      if (tid == 0) {
        const int t = perm[j]; perm[j] = perm[piv]; perm[piv] = t;
        vn1[piv] = vn1[j];
        vn2[piv] = vn2[j];
      }
    }
    __syncthreads();
    // reflector of column j, rows j..s-1 (xLARFG)
    double* colj = M + (int64_t)j * ldm;
    if (warp == 0) {
      double ss = 0.0;
      for (int64_t i = j + 1 + lane; i < s; i += 32) ss = fma(colj[i], colj[i], ss);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, off);
      double beta, tau, scal;
      larfg_ss<double>(colj[j], ss, beta, tau, scal);
      __syncwarp();
      if (tau != 0.0)
        for (int64_t i = j + 1 + lane; i < s; i += 32) colj[i] *= scal;
      if (lane == 0) {
        colj[j] = beta;
        red_v[8] = beta;
        red_v[9] = tau;
      }
    }
    __syncthreads();
    const double beta = red_v[8], tau = red_v[9];
    if (j == 0) tol = fmin(a.atol, a.rtol * fabs(beta));
    if (!(fabs(beta) > tol)) break;
    rk = j + 1;
    // apply H = I - tau v v' to columns j+1.. (v = (1, colj[j+1..])) and downdate norms
    for (int c = j + 1 + tid; c < p; c += nt) {
      double* mc = M + (int64_t)c * ldm;
      if (tau != 0.0) {
        double w = mc[j];
        for (int64_t i = j + 1; i < s; ++i) w = fma(colj[i], mc[i], w);
        const double tw = tau * w;
        mc[j] -= tw;
        for (int64_t i = j + 1; i < s; ++i) mc[i] = fma(-tw, colj[i], mc[i]);
      }
      if (vn1[c] != 0.0) {
        double temp = fabs(mc[j]) / vn1[c];
        temp = fmax(1.0 - temp * temp, 0.0);
        const double ratio = vn1[c] / vn2[c];
        const double temp2 = temp * ratio * ratio;
        if (temp2 <= tol3z) {
          double ss = 0.0;
          for (int64_t i = j + 1; i < s; ++i) ss = fma(mc[i], mc[i], ss);
          vn1[c] = sqrt(ss);
          vn2[c] = vn1[c];
        } else {
          vn1[c] *= sqrt(temp);
        }
      }
    }
    __syncthreads();
  }
  __syncthreads();

  // ---- Y = R11^{-1} R12 in place (column-oriented back substitution) ----
  for (int c = rk + tid; c < p; c += nt) {
    double* mc = M + (int64_t)c * ldm;
    for (int k = rk - 1; k >= 0; --k) {
      const double y = mc[k] / M[k + (int64_t)k * ldm];
      mc[k] = y;
      if (y != 0.0)
        for (int i = 0; i < k; ++i) mc[i] = fma(-y, M[i + (int64_t)k * ldm], mc[i]);
    }
  }
  __syncthreads();

  // ---- outputs ----
  if (tid == 0) a.rank[2 * xi + side] = rk;
  double* G = x.G[side];   // X^T: p x rk, ld p
  for (int c = tid; c < p; c += nt) {
    const int q = perm[c];
    for (int j = 0; j < rk; ++j)
      G[q + (int64_t)j * p] = c < rk ? (j == c ? 1.0 : 0.0) : M[j + (int64_t)c * ldm];
  }
  for (int j = tid; j < rk; j += nt) x.J[side][j] = jin(perm[j]);
  const int64_t lds_out = x.leaf ? lds : p;
  for (int64_t e = tid; e < (int64_t)rk * s; e += nt) {
    const int j = (int)(e % rk);
    const int64_t l = e / rk;
    x.Sr[side][j + l * s] = S[perm[j] + l * lds_out];
    double acc = omega_in(perm[j], l);
    for (int c = rk; c < p; ++c) acc = fma(M[j + (int64_t)c * ldm], omega_in(perm[c], l), acc);
    x.Or[side][j + l * s] = acc;
  }
}

__global__ void copy_blocks_kernel(const CopyTask* __restrict__ t) {
  const CopyTask c = t[blockIdx.x];
  const int64_t tot = c.rows * c.cols;
  for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) {
    const int64_t i = e % c.rows, j = e / c.rows;
    c.dst[e] = c.src[i + j * c.lds];
  }
}

}  // namespace

int sample_ksplit(int64_t m, int64_t k, int64_t r, int sms, bool df) {
  const int64_t tiles = df ? ((m + DR - 1) / DR) * ((r + 31) / 32) : ((m + TM - 1) / TM) * ((r + TN - 1) / TN);
  const int64_t want = 8LL * sms;   // several resident blocks per SM
  int64_t z = (want + tiles - 1) / tiles;
  z = std::min<int64_t>(z, std::max<int64_t>(1, k / (4 * TK)));   // at least 64 K per split
  return (int)std::max<int64_t>(1, std::min<int64_t>(z, 64));
}

int64_t sample_kchunk(int64_t k, int nsplit) {
  int64_t c = (k + nsplit - 1) / nsplit;
  return (c + TK - 1) / TK * TK;
}

void launch_sample_gemm(const double* A, int64_t lda, int64_t m, int64_t k, int trans, const double* X,
                        int64_t ldx, int64_t r, double* Y, int64_t ldy, double alpha, double beta, int nsplit,
                        double* partial, bool df, const int32_t* lrow, const int32_t* lin, cudaStream_t st) {
  if (m <= 0 || r <= 0) return;
  GemmProblem p{A, lda, X, ldx, Y, ldy, m, k, r};
  if (df) {
    // row-per-thread tiles: NC = r rounded up to 4 (at most 32 per column tile)
    const int nc = (int)std::min<int64_t>(32, (r + 3) / 4 * 4);
    const int64_t kchunk = sample_kchunk(std::max<int64_t>(k, 1), nsplit);
    nsplit = (int)((std::max<int64_t>(k, 1) + kchunk - 1) / kchunk);
    const dim3 grid((unsigned)((m + DR - 1) / DR), (unsigned)((r + nc - 1) / nc), (unsigned)nsplit);
    double* P = nsplit > 1 ? partial : nullptr;
    switch (nc) {
      case 4: launch_dfrows<4>(grid, st, p, trans, alpha, beta, kchunk, P, lrow, lin); break;
      case 8: launch_dfrows<8>(grid, st, p, trans, alpha, beta, kchunk, P, lrow, lin); break;
      case 12: launch_dfrows<12>(grid, st, p, trans, alpha, beta, kchunk, P, lrow, lin); break;
      case 16: launch_dfrows<16>(grid, st, p, trans, alpha, beta, kchunk, P, lrow, lin); break;
      case 20: launch_dfrows<20>(grid, st, p, trans, alpha, beta, kchunk, P, lrow, lin); break;
      case 24: launch_dfrows<24>(grid, st, p, trans, alpha, beta, kchunk, P, lrow, lin); break;
      case 28: launch_dfrows<28>(grid, st, p, trans, alpha, beta, kchunk, P, lrow, lin); break;
      default: launch_dfrows<32>(grid, st, p, trans, alpha, beta, kchunk, P, lrow, lin); break;
    }
    if (nsplit > 1) {
      const int64_t tot = m * r;
      const unsigned blocks = (unsigned)std::min<int64_t>((tot + 255) / 256, 4096);
      sample_reduce_kernel<<<blocks, 256, 0, st>>>(partial, nsplit, m, r, Y, ldy, alpha, beta);
    }
    return;
  }
  const int64_t kchunk = sample_kchunk(std::max<int64_t>(k, 1), nsplit);
  nsplit = (int)((std::max<int64_t>(k, 1) + kchunk - 1) / kchunk);
  const dim3 grid((unsigned)((m + TM - 1) / TM), (unsigned)((r + TN - 1) / TN), (unsigned)nsplit);
  sample_gemm_kernel<<<grid, GT, 0, st>>>(p, trans, alpha, beta, kchunk, nsplit > 1 ? partial : nullptr);
  if (nsplit > 1) {
    const int64_t tot = m * r;
    const unsigned blocks = (unsigned)std::min<int64_t>((tot + 255) / 256, 4096);
    sample_reduce_kernel<<<blocks, 256, 0, st>>>(partial, nsplit, m, r, Y, ldy, alpha, beta);
  }
}

void launch_blockdiag_gemm(int32_t count, int64_t max_dim, const double* A, int64_t lda, const int64_t* row0,
                           const int64_t* rows, const int64_t* col0, const int64_t* cols, int trans,
                           const double* X, int64_t ldx, int64_t r, double* Y, int64_t ldy, double alpha,
                           double beta, cudaStream_t st) {
  if (count <= 0 || r <= 0 || max_dim <= 0) return;
  const dim3 grid((unsigned)((max_dim + TM - 1) / TM), (unsigned)((r + TN - 1) / TN), (unsigned)count);
  blockdiag_gemm_kernel<<<grid, GT, 0, st>>>(A, lda, row0, rows, col0, cols, trans, X, ldx, r, Y, ldy, alpha,
                                             beta);
}

size_t rc_id_smem(int64_t s, int64_t pmax, bool m_in_smem) {
  const int64_t ldm = s | 1;
  size_t b = (size_t)(2 * pmax + 16) * sizeof(double) + (size_t)(pmax + 16) * sizeof(int);
  if (m_in_smem) b += (size_t)ldm * pmax * sizeof(double);
  return b;
}

int64_t rc_id_scratch(int64_t s, int64_t pmax) { return (s | 1) * pmax; }

cudaError_t launch_rc_id(const RcArgs& a, int32_t count, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  const size_t smem = rc_id_smem(a.s, a.pmax, a.m_in_smem != 0);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(rc_id_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  rc_id_kernel<<<dim3((unsigned)count, 2), IT, smem, st>>>(a);
  return cudaGetLastError();
}

void launch_copy_blocks(const CopyTask* tasks, int64_t count, cudaStream_t st) {
  if (count <= 0) return;
  copy_blocks_kernel<<<(unsigned)count, 256, 0, st>>>(tasks);
}

}  // namespace hss
