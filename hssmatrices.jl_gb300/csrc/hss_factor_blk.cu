// Blocked ULV reduction of one node per thread block, FP32 or FP64, for nodes
// up to 128 x 128 with ranks up to 64 (every node of the leafsize-128 and
// leafsize-64 workloads).  Restated from src/ulvfactor.jl:22-57 (the leaf
// reduction) and :74-79 (the merge), with the reference's reflector order:
//
//   P0  load the leaf's D and U (FP64 -> T) or assemble the merged block of the
//       children (D, U in shared memory; V = [V1 W1; V2 W2], T12, T21 to global);
//   P1  QL of U (geqlf!, :39) by panels of 32 columns from the last: inside a
//       panel every reflector is generated and applied one at a time (8 lanes per
//       column, one barrier per reflector); the panel's product
//       H(c0)...H(c1-1) = I - Y T Y^T (compact WY, T from the Gram matrix of Y)
//       is then applied to D and to the U columns left of the panel as
//       shared-memory GEMMs (ormql!, :41);
//   P2  LQ of D[0:mk, :] (gelqf!, :44) by panels of 32 rows, each panel applied
//       to the rows below it, C <- C - (C Y^T) T Y (ormlq!, :47), and to V,
//       V <- V - Y^T T^T Y V (ormlq!('L', 'N'), :50).
//
// FP32 nodes of at most 64 x 64 with a single QL and a single LQ panel (the
// merges of rank-32 children) skip the block updates instead: each reflector
// is applied to D (QL) or to D's trailing rows and V (LQ) in the panel loop
// itself, as it is generated; T and the L1 inverses are still stored.
//
// Y is never copied for the QL panels: it is read from the panel's columns of
// U (entries above the pivot, an implicit 1 at the pivot, zeros below); the LQ
// panel is copied reflector-major (rows of D are strided in shared memory).
// Each GEMM streams C in chunks of 64 columns (rows), so that an FP32 leaf
// needs about 110 KB of shared memory and two leaves run on an SM at once
// (FP64: about 220 KB, one per SM).  Global loads (the leaf's generators, the
// children's reduced blocks of a merge) are issued 16 per thread at a time.
//
// Outputs (factor storage, precision T): D (L1, LQ reflectors, L2, reduced D),
// U (QL reflectors + reduced U), V, the two tau vectors, the LQ reflectors
// transposed (Qt, n x mk), per panel the compact-WY T (32 x 32) of the QL and
// LQ reflectors, and the inverses of L1's 32 x 32 diagonal blocks.  The root
// gets an LU with partial pivoting in shared memory (src/ulvfactor.jl:83).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "hss_device.cuh"
#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int NT = 256;             // threads per block
constexpr int NW = NT / 32;
constexpr int BMAX = 128;           // largest m, n
constexpr int BKMAX = 64;           // largest ku, kv
constexpr int BP = 32;              // panel width (reflectors per panel)
constexpr int PL = 8;               // lanes per panel column (QL) or row (LQ)
constexpr int XC = 64;              // columns (QL) or rows (LQ) of C per GEMM chunk
constexpr int XP = XC + 4;          // ld of the GEMM intermediate (>= kv, multiple of 4)
constexpr int GP = BP + 1;          // ld of the Gram matrix and of T
constexpr int SVP = BMAX;           // length of a broadcast reflector
constexpr size_t kBlkSmemCap = 226 * 1024;
static_assert(NT == 8 * BP, "the panel mapping puts 8 lanes on each of 32 columns (rows)");
static_assert(XP >= BKMAX, "X holds Y V (32 x kv) in the V update");

__host__ __device__ constexpr size_t sz4(size_t e) { return (e + 3) & ~size_t(3); }
__host__ __device__ constexpr size_t zmax(size_t a, size_t b) { return a > b ? a : b; }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

// shared-memory layout (elements of T), the same on host and device:
//   D (m x n, ld LDD) | W: U (ld LDU) in the QL phase, the LQ panel (ld YP) in
//   the LQ phase, the L1-inverse scratch at the end | V (n x kv, ld LDV) |
//   X (GEMM intermediate; the Gram matrix and the broadcast reflectors overlay
//   it, they are dead before X is written) | T | taus.
// The merge staging of P0 overlays X and what follows it.
struct BlkLayout {
  int LDD, LDU, YP, LDV;
  size_t oW, oV, oX, oG, oSV, oT, oTau, total;
  // S: the level's node-size bucket (largest m and n rounded up to 32)
  __host__ __device__ BlkLayout(int S, int kumax, int kvmax, size_t extra) {
    LDD = S + 1;                         // odd: conflict-free column walks
    LDU = S + 4;                         // 16-byte aligned column segments
    YP = S + 4;                          // LQ panel, reflector-major
    LDV = S + 1;
    const int ku = kumax > 0 ? kumax : 1, kvv = kvmax > 0 ? kvmax : 1;
    const size_t w = zmax(zmax((size_t)LDU * ku, (size_t)BP * YP), (size_t)4 * BP * GP);
    oW = sz4((size_t)LDD * S);
    oV = oW + sz4(w);
    oX = oV + sz4((size_t)LDV * kvv);
    oG = oX;
    oSV = oX + sz4((size_t)BP * GP);
    oT = oX + (size_t)BP * XP;
    oTau = oT + sz4((size_t)BP * GP);
    const size_t tail = oTau + 2 * BP - oX;
    total = oX + zmax(tail, sz4(extra));
  }
};
__host__ __device__ constexpr int size_bucket(int mmax, int nmax) {
  return (((mmax > nmax ? mmax : nmax) + 31) / 32) * 32;
}
static_assert(BP * GP + 4 + 2 * SVP <= BP * XP, "the Gram matrix and the broadcast reflectors fit in X");

// dst(i, j) = (T) src[i + j * sld] for i < rows <= 128, j < cols (dst ld `ld`):
// each warp takes four columns at a time, so that every lane has 16 loads in flight.
template <typename T, typename S>
__device__ void stage_cols(T* dst, int ld, const S* __restrict__ src, int64_t sld, int rows, int cols) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j0 = warp; j0 < cols; j0 += 4 * NW) {
    S v[16];
#pragma unroll
    for (int h = 0; h < 4; ++h)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = lane + 32 * q, c = j0 + h * NW;
        v[4 * h + q] = (r < rows && c < cols) ? __ldg(src + r + (int64_t)c * sld) : S(0);
      }
#pragma unroll
    for (int h = 0; h < 4; ++h)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = lane + 32 * q, c = j0 + h * NW;
        if (r < rows && c < cols) dst[r + c * ld] = (T)v[4 * h + q];
      }
  }
}

// One copy of a rows x cols block (source ld sld) into shared memory (ld dld);
// tril: entries above the diagonal become zero.
template <typename S>
struct CopyJob {
  const S* src;
  int64_t sld;
  int rows, cols, dld, tril;
  int dst;   // element offset of the destination in shared memory
};

// One warp copies one job: lane = row (32 at a time), 16 columns per round, so
// that every lane has 16 loads in flight.
template <typename T, typename S>
__device__ __forceinline__ void stage_warp(T* sm, const CopyJob<S>& J) {
  const int lane = threadIdx.x & 31;
  for (int r0 = 0; r0 < J.rows; r0 += 32) {
    const int i = r0 + lane;
    for (int j0 = 0; j0 < J.cols; j0 += 16) {
      S v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int j = j0 + q;
        v[q] = (i < J.rows && j < J.cols && !(J.tril && j > i)) ? __ldg(J.src + i + (int64_t)j * J.sld) : S(0);
      }
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int j = j0 + q;
        if (i < J.rows && j < J.cols) sm[J.dst + i + j * J.dld] = (T)v[q];
      }
    }
  }
}

// Y(i, j) = sum_l A[i + l lda] * B[j bj + l bl] for i < rows, j < cols (B or
// B^T by the strides), thread (row i, columns j = jb, jb + NT / RMAX, ...); also
// written to Yg (column-major, ld rows) when it is not null.
template <int RMAX, typename T>
__device__ __forceinline__ void small_mm_r(T* Y, int ldy, T* Yg, const T* A, int lda, const T* B, int bj, int bl,
                                           int rows, int cols, int K) {
  const int i = threadIdx.x % RMAX, jb = threadIdx.x / RMAX;
  if (i >= rows) return;
  for (int j = jb; j < cols; j += NT / RMAX) {
    T s = T(0);
    for (int l = 0; l < K; ++l) s = fma_t(A[i + l * lda], B[j * bj + l * bl], s);
    Y[i + j * ldy] = s;
    if (Yg) Yg[i + j * rows] = s;
  }
}
// the same with the row span matched to `rows` (<= 128), so that every thread works
template <typename T>
__device__ __forceinline__ void small_mm(T* Y, int ldy, T* Yg, const T* A, int lda, const T* B, int bj, int bl,
                                         int rows, int cols, int K) {
  if (rows <= 32) small_mm_r<32>(Y, ldy, Yg, A, lda, B, bj, bl, rows, cols, K);
  else if (rows <= 64) small_mm_r<64>(Y, ldy, Yg, A, lda, B, bj, bl, rows, cols, K);
  else small_mm_r<128>(Y, ldy, Yg, A, lda, B, bj, bl, rows, cols, K);
}

template <typename T>
__device__ __forceinline__ T gsum8(T v, unsigned gm) {   // sum over the 8 lanes of a group
  v += __shfl_xor_sync(gm, v, 4);
  v += __shfl_xor_sync(gm, v, 2);
  v += __shfl_xor_sync(gm, v, 1);
  return v;
}

// xLARFG from alpha and the squared tail norm: the norm as sqrt(alpha^2 + ss)
// (hypot only near overflow or underflow); FP32 with correctly rounded
// reciprocals, FP64 with divisions.
__device__ __forceinline__ void larfg_t(float alpha, float ss, float& beta, float& tau, float& scal) {
  if (ss == 0.f) {
    tau = 0.f;
    beta = alpha;
    scal = 1.f;
    return;
  }
  const float t = fmaf(alpha, alpha, ss);
  const float nrm = t <= 3.0e38f ? sqrtf(t) : hypotf(alpha, sqrtf(ss));
  beta = -copysignf(nrm, alpha);
  tau = (beta - alpha) * __frcp_rn(beta);
  scal = __frcp_rn(alpha - beta);
}
__device__ __forceinline__ void larfg_t(double alpha, double ss, double& beta, double& tau, double& scal) {
  // FP64 runs at 1/64 of the FP32 rate here: the norm as sqrt(alpha^2 + ss)
  // (hypot only outside [1e-290, 1e290]), the two divisions independent
  if (ss == 0.0) {
    tau = 0.0;
    beta = alpha;
    scal = 1.0;
    return;
  }
  const double t = fma(alpha, alpha, ss);
  const double nrm = (t > 1e-290 && t < 1e290) ? sqrt(t) : hypot(alpha, sqrt(ss));
  beta = -copysign(nrm, alpha);
  tau = (beta - alpha) / beta;
  scal = 1.0 / (alpha - beta);
}


// four consecutive elements, 16-byte aligned (FP32) or 32-byte aligned (FP64)
__device__ __forceinline__ void ld4(float (&v)[4], const float* p) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ld4(double (&v)[4], const double* p) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

// acc += a . b over four entries as a chain of fused multiply-adds
template <typename T>
__device__ __forceinline__ void fma4(T& acc, const T (&a)[4], const T (&b)[4]) {
  acc = fma_t(a[0], b[0], acc);
  acc = fma_t(a[1], b[1], acc);
  acc = fma_t(a[2], b[2], acc);
  acc = fma_t(a[3], b[3], acc);
}

// Y of a QL panel read from U: column a of the panel has its pivot at row p;
// rows above hold the reflector, the pivot an implicit 1, rows below zeros.
template <typename T>
__device__ __forceinline__ void ymask4(T (&y)[4], int r, int p) {
#pragma unroll
  for (int q = 0; q < 4; ++q) y[q] = r + q < p ? y[q] : (r + q == p ? T(1) : T(0));
}

// LU with partial pivoting of an m x m block in shared memory (ld).
template <typename T>
__device__ void lu_blk(T* A, int m, int ld, int32_t* piv, int32_t* err, T* bv, int* bi, int* prow) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int c = 0; c < m; ++c) {
    T best = T(-1);
    int idx = m;
    for (int i = c + tid; i < m; i += NT) {
      const T a = dabs(A[i + c * ld]);
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
      *prow = ix;
      piv[c] = ix;
      if (A[ix + c * ld] == T(0) && err != nullptr) atomicExch(err, DEV_SINGULAR);
    }
    __syncthreads();
    const int p = *prow;
    if (p != c)
      for (int j = tid; j < m; j += NT) {
        const T t = A[c + j * ld];
        A[c + j * ld] = A[p + j * ld];
        A[p + j * ld] = t;
      }
    __syncthreads();
    const T d = A[c + c * ld];
    if (d != T(0))
      for (int i = c + 1 + tid; i < m; i += NT) A[i + c * ld] /= d;
    __syncthreads();
    const int rem = m - c - 1;
    for (int e = tid; e < rem * rem; e += NT) {
      const int i = c + 1 + e % rem, j = c + 1 + e / rem;
      A[i + j * ld] -= A[i + c * ld] * A[c + j * ld];
    }
    __syncthreads();
  }
}

// T = S^{-1} (S = diag(1/tau) + strictly upper G) by warp 0, one row of T per
// lane in registers, columns in order (xLARFT's recurrence T(i,i) = tau_i,
// T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i)).  Tm row-major (ld GP, zero
// outside the upper triangle), also written column-major to Tg (32 x 32).
template <typename T>
__device__ void blk_tmat(int nb, const T* G, const T* tau, T* Tm, T* Tg) {
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    T tr[BP];
#pragma unroll
    for (int q = 0; q < BP; ++q) tr[q] = T(0);
#pragma unroll
    for (int i = 0; i < BP; ++i) {
      if (i < nb) {   // warp-uniform
        T s0 = T(0), s1 = T(0);
#pragma unroll
        for (int q = 0; q < i; ++q) {
          if (q & 1) s1 += tr[q] * G[q * GP + i];
          else s0 += tr[q] * G[q * GP + i];
        }
        const T ti = tau[i];
        tr[i] = l < i ? -ti * (s0 + s1) : (l == i ? ti : T(0));
      }
    }
#pragma unroll
    for (int q = 0; q < BP; ++q) {
      Tm[l * GP + q] = tr[q];
      Tg[l + q * BP] = tr[q];
    }
  }
  __syncthreads();
}

// Inverses of the 32 x 32 diagonal blocks of L1 (lower part of D[0:mk, 0:mk],
// ld LDD), block w by warp w: lane b holds column b of the inverse, rows in
// order (forward substitution); written column-major to Lg + 1024 w through
// `scr` (4 x 32 x GP) so that the global stores are coalesced.
template <typename T>
__device__ __forceinline__ void blk_linv(int mk, const T* sD, int LDD, T* scr, T* Lg) {
  const int w = threadIdx.x >> 5, b = threadIdx.x & 31;
  const int i0 = w * BP;
  if (w < 4 && i0 < mk) {
    const int nb = min(BP, mk - i0);
    T xc[BP];
#pragma unroll
    for (int a = 0; a < BP; ++a) xc[a] = T(0);
#pragma unroll
    for (int a = 0; a < BP; ++a) {
      if (a < nb) {   // warp-uniform
        const T* La = sD + (i0 + a) + (int64_t)i0 * LDD;
        T s0 = T(0), s1 = T(0);
#pragma unroll
        for (int q = 0; q < a; ++q) {
          if (q & 1) s1 += La[q * LDD] * xc[q];
          else s0 += La[q * LDD] * xc[q];
        }
        const T d = La[a * LDD];
        const T r = T(1) / d;
        xc[a] = a == b ? r : (a > b ? -(s0 + s1) * r : T(0));
      }
    }
    T* x = scr + w * BP * GP;
#pragma unroll
    for (int a = 0; a < BP; ++a) x[a * GP + b] = xc[a];
    __syncwarp();
    for (int e = b; e < BP * BP; e += 32) Lg[w * 1024 + e] = x[(e % BP) * GP + e / BP];
  }
  __syncthreads();
}

// ---- QL panel updates -------------------------------------------------------

// Strictly upper Gram matrix of a QL panel, G(a, b) = Y(:, a)^T Y(:, b) for
// a < b < nb, Y read from U (column c0 + a, pivot row mk + c0 + a).
template <typename T>
__device__ __forceinline__ void ql_gram(const T* sU, int LDU, int c0, int nb, int mk, T* G) {
  const int a = threadIdx.x & 31, bq = threadIdx.x >> 5;   // G(a, 4 bq .. 4 bq + 3)
  const int pa = mk + c0 + a;
  T acc[4] = {T(0), T(0), T(0), T(0)};
  if (a < nb) {
    const T* ua = sU + (c0 + a) * LDU;
    const int rfree = (mk + c0) & ~3;   // rows above every pivot of the panel: no mask
    for (int r = 0; r <= pa; r += 4) {
      T ya[4];
      ld4(ya, ua + r);
      if (r >= rfree) ymask4(ya, r, pa);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int b = 4 * bq + q;
        if (b < nb) {
          T yb[4];
          ld4(yb, sU + (c0 + b) * LDU + r);
          if (r >= rfree) ymask4(yb, r, mk + c0 + b);
          fma4(acc[q], ya, yb);
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) G[a * GP + 4 * bq + q] = acc[q];
  __syncthreads();
}

// C (m rows, ncols columns, ld ldc) <- C - Y (T (Y^T C)) for the QL panel
// (columns c0 .. c0 + nb - 1 of U), in chunks of XC columns.  Rows from
// mk + c0 + nb on are not touched (Y is zero there).
template <typename T>
__device__ __forceinline__ void ql_apply(T* C, int ldc, int ncols, int m, const T* sU, int LDU, int c0, int nb, int mk,
                         const T* Tm, T* X) {
  const int tid = threadIdx.x, jj = tid & (XC - 1), grp = tid / XC;   // grp: 0..3
  const int rlim = min(m, mk + c0 + nb);
  for (int j0 = 0; j0 < ncols; j0 += XC) {
    const int jn = min(XC, ncols - j0);
    // X = Y^T C: thread (column jj, reflectors 8 grp .. 8 grp + 7)
    if (jj < jn && 8 * grp < nb) {
      const T* cj = C + (int64_t)(j0 + jj) * ldc;
      T acc[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = T(0);
      const int rfree = (mk + c0) & ~3;   // rows above every pivot of the panel: no mask
      for (int r = 0; r < rfree; r += 4) {
        T c4[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) c4[q] = cj[r + q];
#pragma unroll
        for (int q8 = 0; q8 < 8; ++q8) {
          if (8 * grp + q8 < nb) {
            T y[4];
            ld4(y, sU + (c0 + 8 * grp + q8) * LDU + r);
            fma4(acc[q8], y, c4);
          }
        }
      }
      for (int r = rfree; r < rlim; r += 4) {
        T c4[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) c4[q] = r + q < m ? cj[r + q] : T(0);
#pragma unroll
        for (int q8 = 0; q8 < 8; ++q8) {
          const int a = 8 * grp + q8;
          if (a < nb) {
            T y[4];
            ld4(y, sU + (c0 + a) * LDU + r);
            ymask4(y, r, mk + c0 + a);
            fma4(acc[q8], y, c4);
          }
        }
      }
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) X[(8 * grp + q8) * XP + jj] = acc[q8];
    }
    __syncthreads();
    // X = T X (T upper triangular)
    T nx[8];
    if (jj < jn && 8 * grp < nb) {
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) nx[q8] = T(0);
      for (int b = 8 * grp; b < nb; ++b) {
        const T xv = X[b * XP + jj];
#pragma unroll
        for (int q8 = 0; q8 < 8; ++q8) nx[q8] += Tm[(8 * grp + q8) * GP + b] * xv;
      }
    }
    __syncthreads();
    if (jj < jn && 8 * grp < nb) {
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) X[(8 * grp + q8) * XP + jj] = nx[q8];
    }
    __syncthreads();
    // C -= Y X: thread (column jj, rows 8 grp + 32 t .. + 7, t = 0..3)
    if (jj < jn) {
      T* cj = C + (int64_t)(j0 + jj) * ldc;
      T acc[4][8];
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[t][q] = T(0);
      for (int a = 0; a < nb; ++a) {
        const T xv = X[a * XP + jj];
        const int p = mk + c0 + a;
        const T* ua = sU + (c0 + a) * LDU;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int r0 = 8 * grp + 32 * t;
          if (r0 < rlim) {
            T y0[4], y1[4];
            ld4(y0, ua + r0);
            ld4(y1, ua + r0 + 4);
            if (r0 + 8 > mk + c0) {   // rows at or below the panel's first pivot
              ymask4(y0, r0, p);
              ymask4(y1, r0 + 4, p);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              acc[t][q] += y0[q] * xv;
              acc[t][q + 4] += y1[q] * xv;
            }
          }
        }
      }
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int r0 = 8 * grp + 32 * t;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (r0 + q < rlim) cj[r0 + q] -= acc[t][q];
      }
    }
    __syncthreads();
  }
}

// ---- LQ panel updates -------------------------------------------------------

// Strictly upper Gram matrix of an LQ panel held reflector-major in Yc.
template <typename T>
__device__ __forceinline__ void lq_gram(const T* Yc, int YP, int n, int nb, T* G) {
  const int a = threadIdx.x & 31, bq = threadIdx.x >> 5;
  T acc[4] = {T(0), T(0), T(0), T(0)};
  if (a < nb) {
    for (int c = 0; c < n; c += 4) {
      T ya[4];
      ld4(ya, Yc + a * YP + c);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (4 * bq + q < nb) {
          T yb[4];
          ld4(yb, Yc + (4 * bq + q) * YP + c);
          fma4(acc[q], ya, yb);
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) G[a * GP + 4 * bq + q] = acc[q];
  __syncthreads();
}

// Rows r0 .. m-1 of C (n columns, ld ldc) <- C - (C Y^T) T Y, Y = Yc (nb x n,
// reflector-major, zero-padded to a multiple of 4 columns), chunks of XC rows.
template <typename T>
__device__ __forceinline__ void lq_apply_right(T* C, int ldc, int r0, int m, int n, const T* Yc, int YP, int nb, const T* Tm,
                               T* X) {
  const int tid = threadIdx.x, rr = tid & (XC - 1), grp = tid / XC;
  for (int R0 = r0; R0 < m; R0 += XC) {
    const int rn = min(XC, m - R0);
    const int r = R0 + rr;
    // X = C Y^T, stored reflector-major: thread (row rr, reflectors 8 grp ..)
    if (rr < rn && 8 * grp < nb) {
      T acc[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = T(0);
      for (int c = 0; c < n; c += 4) {
        T c4[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) c4[q] = c + q < n ? C[r + (int64_t)(c + q) * ldc] : T(0);
#pragma unroll
        for (int q8 = 0; q8 < 8; ++q8) {
          if (8 * grp + q8 < nb) {
            T y[4];
            ld4(y, Yc + (8 * grp + q8) * YP + c);
            fma4(acc[q8], y, c4);
          }
        }
      }
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) X[(8 * grp + q8) * XP + rr] = acc[q8];
    }
    __syncthreads();
    // X = X T (T upper): X(:, a) = sum_{b <= a} X(:, b) T(b, a)
    T nx[8];
    if (rr < rn && 8 * grp < nb) {
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) nx[q8] = T(0);
      const int hi = min(nb, 8 * grp + 8);
      for (int b = 0; b < hi; ++b) {
        const T xv = X[b * XP + rr];
#pragma unroll
        for (int q8 = 0; q8 < 8; ++q8) nx[q8] += xv * Tm[b * GP + 8 * grp + q8];
      }
    }
    __syncthreads();
    if (rr < rn && 8 * grp < nb) {
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) X[(8 * grp + q8) * XP + rr] = nx[q8];
    }
    __syncthreads();
    // C -= X Y: thread (row rr, columns 8 grp + 32 t .. + 7)
    if (rr < rn) {
      T acc[4][8];
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[t][q] = T(0);
      for (int a = 0; a < nb; ++a) {
        const T xv = X[a * XP + rr];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int c0 = 8 * grp + 32 * t;
          if (c0 < n) {
            T y0[4], y1[4];
            ld4(y0, Yc + a * YP + c0);
            ld4(y1, Yc + a * YP + c0 + 4);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              acc[t][q] += xv * y0[q];
              acc[t][q + 4] += xv * y1[q];
            }
          }
        }
      }
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int c0 = 8 * grp + 32 * t;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (c0 + q < n) C[r + (int64_t)(c0 + q) * ldc] -= acc[t][q];
      }
    }
    __syncthreads();
  }
}

// V (n x kv, ld LDV) <- V - Y^T (T^T (Y V)) for one LQ panel, Y = Yc (nb x n).
template <typename T>
__device__ __forceinline__ void lq_apply_v(T* V, int LDV, int n, int kv, const T* Yc, int YP, int nb, const T* Tm, T* X) {
  const int tid = threadIdx.x, c = tid & 31, ab = tid >> 5;   // ab: reflectors 4 ab .. 4 ab + 3
  // Z = Y V (nb x kv) into X
  for (int cc = c; cc < kv; cc += 32) {
    if (4 * ab >= nb) break;
    const T* vc = V + cc * LDV;
    T acc[4] = {T(0), T(0), T(0), T(0)};
    for (int col = 0; col < n; col += 4) {
      T v4[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v4[q] = col + q < n ? vc[col + q] : T(0);
#pragma unroll
      for (int q4 = 0; q4 < 4; ++q4) {
        if (4 * ab + q4 < nb) {
          T y[4];
          ld4(y, Yc + (4 * ab + q4) * YP + col);
          fma4(acc[q4], y, v4);
        }
      }
    }
#pragma unroll
    for (int q4 = 0; q4 < 4; ++q4) X[(4 * ab + q4) * XP + cc] = acc[q4];
  }
  __syncthreads();
  // Z = T^T Z: Z(a, :) = sum_{b <= a} T(b, a) Z(b, :)
  T nz[2][4];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int cc = c + 32 * h;
#pragma unroll
    for (int q4 = 0; q4 < 4; ++q4) nz[h][q4] = T(0);
    if (cc < kv && 4 * ab < nb) {
      const int hi = min(nb, 4 * ab + 4);
      for (int b = 0; b < hi; ++b) {
        const T zv = X[b * XP + cc];
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) nz[h][q4] += Tm[b * GP + 4 * ab + q4] * zv;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int cc = c + 32 * h;
    if (cc < kv && 4 * ab < nb) {
#pragma unroll
      for (int q4 = 0; q4 < 4; ++q4) X[(4 * ab + q4) * XP + cc] = nz[h][q4];
    }
  }
  __syncthreads();
  // V -= Y^T Z: thread (row col of V, columns 4 j .. 4 j + 3 of V, j = tid >> 7 + 2 i)
  for (int o = tid; o < BMAX * (BKMAX / 4); o += NT) {
    const int col = o & (BMAX - 1), c4 = (o / BMAX) * 4;
    if (col >= n || c4 >= kv) continue;
    T acc[4] = {T(0), T(0), T(0), T(0)};
    for (int a = 0; a < nb; ++a) {
      const T y = Yc[a * YP + col];
      T z[4];
      ld4(z, X + a * XP + c4);
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] += y * z[q];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (c4 + q < kv) V[col + (c4 + q) * LDV] -= acc[q];
  }
  __syncthreads();
}

template <typename T, int S>
__global__ void __launch_bounds__(NT, (sizeof(T) == 4 ? 2 : 1))
    ulv_factor_blk_kernel(const Task* __restrict__ tasks, const Slot* __restrict__ slots, int kumax, int kvmax,
                          int extra) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ T bvals[NW];
  __shared__ int bidx[NW];
  __shared__ int prow;
  const BlkLayout Lo(S, kumax, kvmax, (size_t)extra);
  const Task tk = tasks[blockIdx.x];
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* fb = (T*)sl.fbase;
  const int m = nd.m, n = nd.n, ku = nd.ku, kv = nd.kv;
  constexpr int LDD = S + 1, LDU = S + 4, YP = S + 4, LDV = S + 1;   // as in BlkLayout
  constexpr int PE = S / PL;                                        // panel entries per lane
  T* sm = (T*)smraw;
  T* sD = sm;                 // m x n, ld LDD
  T* sW = sm + Lo.oW;         // U (ld LDU) / LQ panel (ld YP) / L1-inverse scratch
  T* sV = sm + Lo.oV;         // n x kv, ld LDV
  T* X = sm + Lo.oX;          // GEMM intermediate, BP x XP; merge staging overlays X .. tau
  T* G = sm + Lo.oG;
  T* Tm = sm + Lo.oT;
  T* sv = sm + Lo.oSV;        // two broadcast reflectors
  T* stau = sm + Lo.oTau;     // two taus of the panel loop, then the panel's taus
  T* ptau = stau + 2;
  T* gD = fb + nd.fD;
  T* gU = fb + nd.fU;
  T* gV = fb + nd.fV;
  const int tid = threadIdx.x, lane = tid & 31;

  // ---- P0: load or assemble ---------------------------------------------------
  if (nd.leaf) {
    stage_cols(sD, LDD, nd.D, m, m, n);
    if (!nd.root) {
      stage_cols(sW, LDU, nd.U, m, m, ku);
      stage_cols(sV, LDV, nd.V, n, n, kv);
    }
  } else {
    // Merge (src/ulvfactor.jl:74-79): the generator blocks (converted to T) and
    // the children's reduced U, V staged in shared memory, the children's
    // reduced D blocks copied to the diagonal of D, all in one pass of loads.
    const Node& c1 = nodes[nd.left];
    const Node& c2 = nodes[nd.right];
    const int u1 = c1.ku, u2 = c2.ku, v1 = c1.kv, v2 = c2.kv;
    const int mr1 = c1.mr, mr2 = c2.mr, nr1 = c1.nr, nr2 = c2.nr;
    const int kuo = nd.root ? 0 : ku, kvo = nd.root ? 0 : kv;
    const int oB12 = (int)Lo.oX;      // u1 x v2
    const int oB21 = oB12 + u1 * v2;  // u2 x v1
    const int oR1 = oB21 + u2 * v1;   // u1 x ku
    const int oR2 = oR1 + u1 * kuo;   // u2 x ku
    const int oW1 = oR2 + u2 * kuo;   // v1 x kv
    const int oW2 = oW1 + v1 * kvo;   // v2 x kv
    const int oU1 = oW2 + v2 * kvo;   // mr1 x u1 (tril when reduced)
    const int oU2 = oU1 + mr1 * u1;   // mr2 x u2
    const int oV1 = oU2 + mr2 * u2;   // nr1 x v1
    const int oV2 = oV1 + nr1 * v1;   // nr2 x v2
    const int o12 = oV2 + nr2 * v2;   // T12 = U1 B12, mr1 x v2
    const int o21 = o12 + mr1 * v2;   // T21 = U2 B21, mr2 x v1
    {
      // one job per warp: the FP64 generator blocks (converted to T), and the
      // children's reduced blocks (factor storage, already T)
      const int w = tid >> 5;
      CopyJob<double> G64{nullptr, 0, 0, 0, 0, 0, 0};
      switch (w) {
        case 0: G64 = {nd.B12, u1, u1, v2, u1, 0, oB12}; break;
        case 1: G64 = {nd.B21, u2, u2, v1, u2, 0, oB21}; break;
        case 2: G64 = {nd.R1, u1, u1, kuo, u1, 0, oR1}; break;
        case 3: G64 = {nd.R2, u2, u2, kuo, u2, 0, oR2}; break;
        case 4: G64 = {nd.W1, v1, v1, kvo, v1, 0, oW1}; break;
        case 5: G64 = {nd.W2, v2, v2, kvo, v2, 0, oW2}; break;
        default: break;
      }
      if (w < 6) stage_warp(sm, G64);
      CopyJob<T> J{nullptr, 0, 0, 0, 0, 0, 0};
      const int wc = (w + 6) % NW;   // warps 6 and 7 take the first of these, the others follow
      switch (wc) {
        case 0: J = {fb + c1.fU + c1.mk, c1.m, mr1, u1, mr1, c1.lower_u, oU1}; break;
        case 1: J = {fb + c2.fU + c2.mk, c2.m, mr2, u2, mr2, c2.lower_u, oU2}; break;
        case 2: J = {fb + c1.fV + c1.nk, c1.n, nr1, v1, nr1, 0, oV1}; break;
        case 3: J = {fb + c2.fV + c2.nk, c2.n, nr2, v2, nr2, 0, oV2}; break;
        case 4: J = {fb + c1.fD + c1.mk + (int64_t)c1.nk * c1.m, c1.m, mr1, nr1, LDD, 0, 0}; break;
        case 5: J = {fb + c2.fD + c2.mk + (int64_t)c2.nk * c2.m, c2.m, mr2, nr2, LDD, 0, mr1 + nr1 * LDD}; break;
        default: break;
      }
      if (wc < 6) stage_warp(sm, J);
    }
    __syncthreads();
    const T* gB12 = sm + oB12;
    const T* gB21 = sm + oB21;
    const T* gR1 = sm + oR1;
    const T* gR2 = sm + oR2;
    const T* gW1 = sm + oW1;
    const T* gW2 = sm + oW2;
    const T* cU1 = sm + oU1;
    const T* cU2 = sm + oU2;
    const T* cV1 = sm + oV1;
    const T* cV2 = sm + oV2;
    T* sT12 = sm + o12;
    T* sT21 = sm + o21;
    // T12 = U1 B12, T21 = U2 B21 (also kept for the solve); U = [U1 R1; U2 R2],
    // V = [V1 W1; V2 W2] (src/ulvfactor.jl:78-79)
    small_mm(sT12, mr1, fb + nd.fT12, cU1, mr1, gB12, u1, 1, mr1, v2, u1);
    small_mm(sT21, mr2, fb + nd.fT21, cU2, mr2, gB21, u2, 1, mr2, v1, u2);
    if (!nd.root) {
      small_mm(sW, LDU, (T*)nullptr, cU1, mr1, gR1, u1, 1, mr1, ku, u1);
      small_mm(sW + mr1, LDU, (T*)nullptr, cU2, mr2, gR2, u2, 1, mr2, ku, u2);
      small_mm(sV, LDV, (T*)nullptr, cV1, nr1, gW1, v1, 1, nr1, kv, v1);
      small_mm(sV + nr1, LDV, (T*)nullptr, cV2, nr2, gW2, v2, 1, nr2, kv, v2);
    }
    __syncthreads();
    // the off-diagonal blocks U1 B12 V2^T and U2 B21 V1^T (src/ulvfactor.jl:75)
    small_mm(sD + nr1 * LDD, LDD, (T*)nullptr, sT12, mr1, cV2, 1, nr2, mr1, nr2, v2);
    small_mm(sD + mr1, LDD, (T*)nullptr, sT21, mr2, cV1, 1, nr1, mr2, nr1, v1);
  }
  __syncthreads();

  if (nd.root) {
    lu_blk(sD, m, LDD, (int32_t*)(fb + nd.fpiv), sl.err, bvals, bidx, &prow);
    for (int e = tid; e < m * n; e += NT) gD[e] = sD[(e % m) + (e / m) * LDD];
    return;
  }
  if (nd.mk == 0) {
    // nothing to eliminate: the block passes up as it is (src/ulvfactor.jl:32-36)
    for (int e = tid; e < m * n; e += NT) gD[e] = sD[(e % m) + (e / m) * LDD];
    for (int e = tid; e < m * ku; e += NT) gU[e] = sW[(e % m) + (e / m) * LDU];
    for (int e = tid; e < n * kv; e += NT) gV[e] = sV[(e % n) + (e / n) * LDV];
    return;
  }

  const int k = nd.k, mk = nd.mk;
  T* tq = fb + nd.ftq;
  T* tl = fb + nd.ftl;
  const int g = tid >> 3, l8 = tid & 7;            // panel column / row g, lane l8 of its group
  const unsigned gm = 0xFFu << (lane & 24);        // the group's 8 lanes

  if constexpr (S == 64 && sizeof(T) == sizeof(float)) {
    if (k <= BP && ku <= BP && mk <= BP && m - mk <= BP && kv <= BP) {
      // FP32 nodes of at most 64 x 64 with one QL and one LQ panel (the merges
      // of rank-32 children; FP64 keeps the block updates, measured faster on
      // its slower FMA pipe): every reflector is applied, as soon as it is
      // generated, to everything it acts on, each column (row) held in
      // registers by a group of 8 lanes, one barrier per reflector.  QL: the
      // U panel and D's columns (two per group); LQ: the panel rows, D's rows
      // below them and V's columns (one each per group).  This replaces the
      // panels' block updates (shared-memory GEMMs after the panel loops); the
      // panels' T matrices and the L1 block inverses are still formed and
      // stored for the blocked solve, so the factor storage is the same.
      auto refl = [&](T(&x)[PE], const T(&vv)[PE], T tau) {
        T w0 = T(0), w1 = T(0);
#pragma unroll
        for (int t = 0; t < PE; t += 2) {
          w0 = fma_t(vv[t], x[t], w0);
          w1 = fma_t(vv[t + 1], x[t + 1], w1);
        }
        const T w = gsum8(w0 + w1, gm) * tau;
#pragma unroll
        for (int t = 0; t < PE; ++t) x[t] = fma_t(-w, vv[t], x[t]);
      };
      // ---- QL of U (geqlf!, :39), applied to D (ormql!, :41) ----
      {
        T u[PE], dq0[PE], dq1[PE];
#pragma unroll
        for (int t = 0; t < PE; ++t) {
          const int row = l8 + PL * t;
          u[t] = (g < k && row < m) ? sW[row + g * LDU] : T(0);
          dq0[t] = (g < n && row < m) ? sD[row + g * LDD] : T(0);
          dq1[t] = (g + BP < n && row < m) ? sD[row + (g + BP) * LDD] : T(0);
        }
        auto gen = [&](int c, int buf) {   // the 8 lanes of column c
          const int p = mk + c;
          T sq[4] = {T(0), T(0), T(0), T(0)}, mine = T(0);
#pragma unroll
          for (int t = 0; t < PE; ++t) {
            const int row = l8 + PL * t;
            if (row < p) sq[t & 3] = fma_t(u[t], u[t], sq[t & 3]);
            if (row == p) mine = u[t];
          }
          const T ss = gsum8((sq[0] + sq[1]) + (sq[2] + sq[3]), gm);
          const T alpha = __shfl_sync(gm, mine, (lane & 24) | (p & 7));
          T beta, tau, sc;
          larfg_t(alpha, ss, beta, tau, sc);
#pragma unroll
          for (int t = 0; t < PE; ++t) {
            const int row = l8 + PL * t;
            if (row < p && tau != T(0)) u[t] *= sc;
            if (row == p) u[t] = beta;
            sv[buf * SVP + row] = row < p ? u[t] : (row == p ? T(1) : T(0));
          }
          if (l8 == 0) {
            stau[buf] = tau;
            ptau[c] = tau;
            tq[c] = tau;
          }
        };
        if (g == k - 1) gen(k - 1, 0);
        __syncthreads();
        for (int c = k - 1; c >= 0; --c) {
          const int cur = (k - 1 - c) & 1;
          const T tau = stau[cur];
          const T* v = sv + cur * SVP;
          T vv[PE];
#pragma unroll
          for (int t = 0; t < PE; ++t) vv[t] = v[l8 + PL * t];
          if (g < c && tau != T(0)) refl(u, vv, tau);
          if (c > 0 && g == c - 1) gen(c - 1, cur ^ 1);   // the next reflector first: it is on the critical path
          if (tau != T(0)) {
            if (g < n) refl(dq0, vv, tau);
            if (g + BP < n) refl(dq1, vv, tau);
          }
          __syncthreads();
        }
#pragma unroll
        for (int t = 0; t < PE; ++t) {
          const int row = l8 + PL * t;
          if (row < m) {
            if (g < k) sW[row + g * LDU] = u[t];
            if (g < n) sD[row + g * LDD] = dq0[t];
            if (g + BP < n) sD[row + (g + BP) * LDD] = dq1[t];
          }
        }
      }
      __syncthreads();
      ql_gram(sW, LDU, 0, k, mk, G);
      blk_tmat(k, G, ptau, Tm, fb + nd.fTq);
      for (int e = tid; e < m * ku; e += NT) gU[e] = sW[(e % m) + (e / m) * LDU];
      __syncthreads();
      // ---- LQ of D[0:mk, :] (gelqf!, :44), applied to the rows below (:47) and to V (:50) ----
      {
        T d[PE], dt[PE], vc[PE];
#pragma unroll
        for (int t = 0; t < PE; ++t) {
          const int col = l8 + PL * t;
          d[t] = (g < mk && col < n) ? sD[g + col * LDD] : T(0);
          dt[t] = (mk + g < m && col < n) ? sD[(mk + g) + col * LDD] : T(0);
          vc[t] = (g < kv && col < n) ? sV[col + g * LDV] : T(0);
        }
        auto gen = [&](int i, int buf) {   // the 8 lanes of row i
          T sq[4] = {T(0), T(0), T(0), T(0)}, mine = T(0);
#pragma unroll
          for (int t = 0; t < PE; ++t) {
            const int col = l8 + PL * t;
            if (col > i) sq[t & 3] = fma_t(d[t], d[t], sq[t & 3]);
            if (col == i) mine = d[t];
          }
          const T ss = gsum8((sq[0] + sq[1]) + (sq[2] + sq[3]), gm);
          const T alpha = __shfl_sync(gm, mine, (lane & 24) | (i & 7));
          T beta, tau, sc;
          larfg_t(alpha, ss, beta, tau, sc);
#pragma unroll
          for (int t = 0; t < PE; ++t) {
            const int col = l8 + PL * t;
            if (col > i && tau != T(0)) d[t] *= sc;
            if (col == i) d[t] = beta;
            sv[buf * SVP + col] = col < i ? T(0) : (col == i ? T(1) : d[t]);
          }
          if (l8 == 0) {
            stau[buf] = tau;
            ptau[i] = tau;
            tl[i] = tau;
          }
        };
        if (g == 0) gen(0, 0);
        __syncthreads();
        for (int i = 0; i < mk; ++i) {
          const int cur = i & 1;
          const T tau = stau[cur];
          const T* v = sv + cur * SVP;
          T vv[PE];
#pragma unroll
          for (int t = 0; t < PE; ++t) vv[t] = v[l8 + PL * t];
          if (g > i && g < mk && tau != T(0)) refl(d, vv, tau);
          if (i + 1 < mk && g == i + 1) gen(i + 1, cur ^ 1);
          if (tau != T(0)) {
            if (mk + g < m) refl(dt, vv, tau);
            if (g < kv) refl(vc, vv, tau);
          }
          __syncthreads();
        }
        // write back; the reflectors also reflector-major (zero-padded to YP - 4
        // columns) for the Gram matrix, and transposed to global memory
        T* gQt = fb + nd.fQt;
        T* Yc = sW;   // U is in global memory now
#pragma unroll
        for (int t = 0; t < PE; ++t) {
          const int col = l8 + PL * t;
          const T y = col < g ? T(0) : (col == g ? T(1) : d[t]);
          if (col < n) {
            if (g < mk) {
              sD[g + col * LDD] = d[t];
              gQt[col + (int64_t)g * n] = y;
            }
            if (mk + g < m) sD[(mk + g) + col * LDD] = dt[t];
            if (g < kv) sV[col + g * LDV] = vc[t];
          }
          if (g < mk && col < YP - 4) Yc[g * YP + col] = col < n ? y : T(0);
        }
        __syncthreads();
        lq_gram(Yc, YP, n, mk, G);
        blk_tmat(mk, G, ptau, Tm, fb + nd.fTl);
      }
      blk_linv(mk, sD, LDD, sW, fb + nd.fLi);
      for (int e = tid; e < m * n; e += NT) gD[e] = sD[(e % m) + (e / m) * LDD];
      for (int e = tid; e < n * kv; e += NT) gV[e] = sV[(e % n) + (e / n) * LDV];
      return;
    }
  }

  // ---- P1: QL of U, panels of BP columns from the last -------------------------
  for (int c1 = k; c1 > 0; c1 -= BP) {
    const int c0 = max(0, c1 - BP), nb = c1 - c0;
    const int col = c0 + g;
    T u[PE];
#pragma unroll
    for (int t = 0; t < PE; ++t) {
      const int row = l8 + PL * t;
      u[t] = (g < nb && row < m) ? sW[row + col * LDU] : T(0);
    }
    auto gen = [&](int c, int buf) {   // the 8 lanes of column c
      const int p = mk + c;
      T sq[4] = {T(0), T(0), T(0), T(0)}, mine = T(0);
#pragma unroll
      for (int t = 0; t < PE; ++t) {
        const int row = l8 + PL * t;
        if (row < p) sq[t & 3] = fma_t(u[t], u[t], sq[t & 3]);
        if (row == p) mine = u[t];
      }
      const T ss = gsum8((sq[0] + sq[1]) + (sq[2] + sq[3]), gm);
      const T alpha = __shfl_sync(gm, mine, (lane & 24) | (p & 7));
      T beta, tau, sc;
      larfg_t(alpha, ss, beta, tau, sc);
#pragma unroll
      for (int t = 0; t < PE; ++t) {
        const int row = l8 + PL * t;
        if (row < p && tau != T(0)) u[t] *= sc;
        if (row == p) u[t] = beta;
        sv[buf * SVP + row] = row < p ? u[t] : (row == p ? T(1) : T(0));
      }
      if (l8 == 0) {
        stau[buf] = tau;
        ptau[c - c0] = tau;
        tq[c] = tau;
      }
    };
    if (g == nb - 1) gen(c1 - 1, 0);
    __syncthreads();
    for (int c = c1 - 1; c >= c0; --c) {
      const int cur = (c1 - 1 - c) & 1;
      const T tau = stau[cur];
      if (g < c - c0 && tau != T(0)) {
        const T* v = sv + cur * SVP;
        T vv[PE];
#pragma unroll
        for (int t = 0; t < PE; ++t) vv[t] = v[l8 + PL * t];
        T w0 = T(0), w1 = T(0);
#pragma unroll
        for (int t = 0; t < PE; t += 2) {
          w0 = fma_t(vv[t], u[t], w0);
          w1 = fma_t(vv[t + 1], u[t + 1], w1);
        }
        const T w = gsum8(w0 + w1, gm) * tau;
#pragma unroll
        for (int t = 0; t < PE; ++t) u[t] = fma_t(-w, vv[t], u[t]);
      }
      if (c > c0 && g == c - 1 - c0) gen(c - 1, cur ^ 1);
      __syncthreads();
    }
    if (g < nb) {
#pragma unroll
      for (int t = 0; t < PE; ++t) {
        const int row = l8 + PL * t;
        if (row < m) sW[row + col * LDU] = u[t];
      }
    }
    __syncthreads();
    ql_gram(sW, LDU, c0, nb, mk, G);
    blk_tmat(nb, G, ptau, Tm, fb + nd.fTq + (int64_t)((k - c1) / BP) * 1024);
    ql_apply(sD, LDD, n, m, sW, LDU, c0, nb, mk, Tm, X);
    if (c0 > 0) ql_apply(sW, LDU, c0, m, sW, LDU, c0, nb, mk, Tm, X);
  }
  for (int e = tid; e < m * ku; e += NT) gU[e] = sW[(e % m) + (e / m) * LDU];
  __syncthreads();

  // ---- P2: LQ of D[0:mk, :], panels of BP rows ---------------------------------
  T* Yc = sW;   // the panel's reflectors, reflector-major (U is in global memory now)
  T* gQt = fb + nd.fQt;
  for (int i0 = 0; i0 < mk; i0 += BP) {
    const int i1 = min(mk, i0 + BP), nb = i1 - i0;
    const int row = i0 + g;
    T d[PE];
#pragma unroll
    for (int t = 0; t < PE; ++t) {
      const int col = l8 + PL * t;
      d[t] = (g < nb && col < n) ? sD[row + col * LDD] : T(0);
    }
    auto gen = [&](int i, int buf) {   // the 8 lanes of row i
      T sq[4] = {T(0), T(0), T(0), T(0)}, mine = T(0);
#pragma unroll
      for (int t = 0; t < PE; ++t) {
        const int col = l8 + PL * t;
        if (col > i) sq[t & 3] = fma_t(d[t], d[t], sq[t & 3]);
        if (col == i) mine = d[t];
      }
      const T ss = gsum8((sq[0] + sq[1]) + (sq[2] + sq[3]), gm);
      const T alpha = __shfl_sync(gm, mine, (lane & 24) | (i & 7));
      T beta, tau, sc;
      larfg_t(alpha, ss, beta, tau, sc);
#pragma unroll
      for (int t = 0; t < PE; ++t) {
        const int col = l8 + PL * t;
        if (col > i && tau != T(0)) d[t] *= sc;
        if (col == i) d[t] = beta;
        sv[buf * SVP + col] = col < i ? T(0) : (col == i ? T(1) : d[t]);
      }
      if (l8 == 0) {
        stau[buf] = tau;
        ptau[i - i0] = tau;
        tl[i] = tau;
      }
    };
    if (g == 0) gen(i0, 0);
    __syncthreads();
    for (int i = i0; i < i1; ++i) {
      const int cur = (i - i0) & 1;
      const T tau = stau[cur];
      if (g > i - i0 && g < nb && tau != T(0)) {
        const T* v = sv + cur * SVP;
        T vv[PE];
#pragma unroll
        for (int t = 0; t < PE; ++t) vv[t] = v[l8 + PL * t];
        T w0 = T(0), w1 = T(0);
#pragma unroll
        for (int t = 0; t < PE; t += 2) {
          w0 = fma_t(vv[t], d[t], w0);
          w1 = fma_t(vv[t + 1], d[t + 1], w1);
        }
        const T w = gsum8(w0 + w1, gm) * tau;
#pragma unroll
        for (int t = 0; t < PE; ++t) d[t] = fma_t(-w, vv[t], d[t]);
      }
      if (i + 1 < i1 && g == i + 1 - i0) gen(i + 1, cur ^ 1);
      __syncthreads();
    }
    // write back; the panel's reflectors reflector-major (zero-padded to YP - 4
    // columns) and transposed to global memory
    if (g < nb) {
#pragma unroll
      for (int t = 0; t < PE; ++t) {
        const int col = l8 + PL * t;
        const T y = col < row ? T(0) : (col == row ? T(1) : d[t]);
        if (col < n) {
          sD[row + col * LDD] = d[t];
          gQt[col + (int64_t)row * n] = y;
        }
        if (col < YP - 4) Yc[g * YP + col] = col < n ? y : T(0);
      }
    }
    __syncthreads();
    lq_gram(Yc, YP, n, nb, G);
    blk_tmat(nb, G, ptau, Tm, fb + nd.fTl + (int64_t)(i0 / BP) * 1024);
    if (i1 < m) lq_apply_right(sD, LDD, i1, m, n, Yc, YP, nb, Tm, X);
    if (kv > 0) lq_apply_v(sV, LDV, n, kv, Yc, YP, nb, Tm, X);   // V <- Q V (ormlq!('L', 'N'), :50)
  }
  // inverses of L1's diagonal blocks for the solve (the panel buffer is free)
  blk_linv(mk, sD, LDD, sW, fb + nd.fLi);
  for (int e = tid; e < m * n; e += NT) gD[e] = sD[(e % m) + (e / m) * LDD];
  for (int e = tid; e < n * kv; e += NT) gV[e] = sV[(e % n) + (e / n) * LDV];
}

}  // namespace

template <typename T>
size_t factor_blk_smem(int mmax, int nmax, int kumax, int kvmax, size_t extra) {
  return BlkLayout(size_bucket(mmax, nmax), kumax, kvmax, extra).total * sizeof(T);
}

template <typename T>
bool factor_blk_fits(int mmax, int nmax, int kumax, int kvmax, size_t extra) {
  return mmax <= BMAX && nmax <= BMAX && kumax <= BKMAX && kvmax <= BKMAX &&
         factor_blk_smem<T>(mmax, nmax, kumax, kvmax, extra) <= kBlkSmemCap;
}

namespace {
template <typename T, int S>
void launch_blk_sized(const Task* t, int64_t nt, const Slot* s, int kumax, int kvmax, size_t extra, size_t smem,
                      cudaStream_t st) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(ulv_factor_blk_kernel<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBlkSmemCap);
    attr_set = true;
  }
  ulv_factor_blk_kernel<T, S><<<(unsigned)nt, NT, smem, st>>>(t, s, kumax, kvmax, (int)extra);
}
}  // namespace

template <typename T>
void launch_ulv_factor_blk(const Task* t, int64_t nt, const Slot* s, int mmax, int nmax, int kumax, int kvmax,
                           size_t extra, cudaStream_t st) {
  if (nt <= 0) return;
  const size_t smem = factor_blk_smem<T>(mmax, nmax, kumax, kvmax, extra);
  switch (size_bucket(mmax, nmax)) {
    case 32: launch_blk_sized<T, 32>(t, nt, s, kumax, kvmax, extra, smem, st); break;
    case 64: launch_blk_sized<T, 64>(t, nt, s, kumax, kvmax, extra, smem, st); break;
    case 96: launch_blk_sized<T, 96>(t, nt, s, kumax, kvmax, extra, smem, st); break;
    default: launch_blk_sized<T, 128>(t, nt, s, kumax, kvmax, extra, smem, st); break;
  }
}

template bool factor_blk_fits<double>(int, int, int, int, size_t);
template bool factor_blk_fits<float>(int, int, int, int, size_t);
template size_t factor_blk_smem<double>(int, int, int, int, size_t);
template size_t factor_blk_smem<float>(int, int, int, int, size_t);
template void launch_ulv_factor_blk<double>(const Task*, int64_t, const Slot*, int, int, int, int, size_t,
                                            cudaStream_t);
template void launch_ulv_factor_blk<float>(const Task*, int64_t, const Slot*, int, int, int, int, size_t,
                                           cudaStream_t);

}  // namespace hss
