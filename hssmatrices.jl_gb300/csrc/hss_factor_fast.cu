// ULV reduction of one node per thread block, for nodes up to 128 x 128 with
// ranks up to 64 (every node of the leafsize-128 and leafsize-64 workloads).
//
// Same arithmetic and reflector order as ulv_factor_kernel (hss_kernels.cu),
// restated from src/ulvfactor.jl:22-57 and :74-79, but with the working block
// on chip:
//   P0  load the leaf generators (FP64 -> T) or assemble the merged block of
//       the children into shared memory (D: m x n, U: m x ku, ld odd);
//   P1  QL of U with Q^T applied to D (geqlf!/ormql!, :39-41) in shared
//       memory: one thread per column and row quarter, partial dot products
//       combined through shared memory;
//   P2  LQ of D[0:mk, :] with the reflectors applied to the rows below and to
//       V (gelqf!/ormlq!, :44-50) with D held in registers: thread (row j,
//       quarter q) owns D[j, 32q:32q+32]; the reflector row is broadcast
//       through a bank-padded shared vector; V lives in registers as 16-row
//       strips per column.
// The root block gets an LU with partial pivoting in shared memory instead.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include "hss_device.cuh"
#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int FT = 512;           // threads per block
constexpr int FW = FT / 32;
constexpr int FMAX = 128;         // max m, n
constexpr int FKMAX = 64;         // max ku, kv
constexpr int PART_COLS = FMAX + FKMAX;
constexpr size_t kFastSmemCap = 226 * 1024;   // dynamic part; the static part is < 1 KB
constexpr int SVLEN = FMAX + (FMAX / 32) * 4 + 8;   // padded broadcast vector (16-byte multiple)
static_assert(SVLEN % 4 == 0 && PART_COLS % 4 == 0, "broadcast vectors must stay 16-byte aligned");

__host__ __device__ constexpr size_t smem_align4(size_t e) { return (e + 3) & ~size_t(3); }

template <typename T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T bsum(T v, T* red) {
  v = wsum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  T s = T(0);
#pragma unroll
  for (int i = 0; i < FW; ++i) s += red[i];
  return s;
}

template <typename T>
__device__ __forceinline__ void larfg(T alpha, T ss, T& beta, T& tau, T& scal) {
  larfg_ss(alpha, ss, beta, tau, scal);
}

// padded index of the broadcast vector: 36 slots per 32 entries, so that each
// 32-entry quarter starts 16-byte aligned and the four quarters a warp reads
// with 128-bit loads sit in distinct banks
__device__ __forceinline__ int vp(int i) { return i + ((i >> 5) << 2); }

// v[0..31] = buf[36q .. 36q+31] with 128-bit shared loads
template <typename T>
__device__ __forceinline__ void load_quarter(T (&v)[32], const T* buf, int q) {
  const T* b = buf + 36 * q;
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float4 t = reinterpret_cast<const float4*>(b)[k];
      v[4 * k] = t.x; v[4 * k + 1] = t.y; v[4 * k + 2] = t.z; v[4 * k + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const double2 t = reinterpret_cast<const double2*>(b)[k];
      v[2 * k] = t.x; v[2 * k + 1] = t.y;
    }
  }
}

// sum_l a[l] * v[l] over 32 entries with four independent chains
template <typename T>
__device__ __forceinline__ T dot32(const T (&a)[32], const T (&v)[32]) {
  T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
#pragma unroll
  for (int l = 0; l < 32; l += 4) {
    s0 += a[l] * v[l];
    s1 += a[l + 1] * v[l + 1];
    s2 += a[l + 2] * v[l + 2];
    s3 += a[l + 3] * v[l + 3];
  }
  return (s0 + s1) + (s2 + s3);
}

// LU with partial pivoting of an m x m block in shared memory (ld = ld).
template <typename T>
__device__ void lu_smem(T* A, int m, int ld, int32_t* piv, int32_t* err, T* bv, int* bi, int* prow) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int c = 0; c < m; ++c) {
    T best = T(-1);
    int idx = m;
    for (int i = c + tid; i < m; i += FT) {
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
      for (int w = 1; w < FW; ++w)
        if (bv[w] > b || (bv[w] == b && bi[w] < ix)) { b = bv[w]; ix = bi[w]; }
      if (ix >= m) ix = c;
      *prow = ix;
      piv[c] = ix;
      if (A[ix + c * ld] == T(0) && err != nullptr) atomicExch(err, DEV_SINGULAR);
    }
    __syncthreads();
    const int p = *prow;
    if (p != c)
      for (int j = tid; j < m; j += FT) {
        const T t = A[c + j * ld];
        A[c + j * ld] = A[p + j * ld];
        A[p + j * ld] = t;
      }
    __syncthreads();
    const T d = A[c + c * ld];
    if (d != T(0))
      for (int i = c + 1 + tid; i < m; i += FT) A[i + c * ld] /= d;
    __syncthreads();
    const int rem = m - c - 1;
    for (int o = tid; o < rem * rem; o += FT) {
      const int i = c + 1 + o % rem, j = c + 1 + o / rem;
      A[i + j * ld] -= A[i + c * ld] * A[c + j * ld];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Blocked FP32 reduction (P1 + P2 of the FP32 factorization)
//
// The same reflectors, in the same order, as the unblocked path above (up to
// rounding), but each reflector touches only its panel of BP columns (QL) or
// rows (LQ); the rest of the block is updated once per panel with the compact
// WY form of the panel's product, H(a) H(a+1) ... H(b-1) = I - Y T Y^T, as
// shared-memory FP32 GEMMs.  T (forward xLARFT) is formed from its inverse: for
// orthogonal reflectors (tau_j = 2 / y_j^T y_j) T^{-1} = S = diag(1/tau) + the
// strictly upper part of the Gram matrix Y^T Y, so each column of T is one
// independent back substitution (a zero tau gives a zero row, as in T):
//   QL (geqlf!/ormql!, src/ulvfactor.jl:39-42): Q^T C = H(c0) ... H(c1-1) C
//       (generation order c = c1-1 .. c0) = C - Y (T (Y^T C)) for C = D and the
//       U columns left of the panel;
//   LQ (gelqf!/ormlq!, :44-50): C Q^T over rows i0..i1-1 = C H(i0) ... H(i1-1)
//       = C - (C Y^T) T Y for the rows below the panel, and Q V =
//       H(i1-1) ... H(i0) V = V - Y^T (T^T (Y V)).
// Panel threads: a half-warp per column (QL) or row (LQ), 8 entries per thread,
// so every reduction of a reflector step is a 16-lane shuffle; one barrier per
// step (the owner of the next reflector applies the current one first).
// ---------------------------------------------------------------------------

constexpr int BP = 32;                    // panel width
constexpr int YP = 132;                   // ld of the reflector-major copy of Y (>= 128, multiple of 4)
constexpr int KP = 36;                    // ld of the row-major copy of Y (>= BP, multiple of 4)
constexpr int XP = 132;                   // ld of the GEMM intermediate
constexpr int GP = 33;                    // ld of the Gram matrix and T
constexpr size_t kBlkElems = (size_t)BP * YP + (size_t)FMAX * KP + (size_t)BP * XP + 2 * (size_t)BP * GP + 2 * BP;
static_assert((size_t)BP * XP >= 4 * (size_t)BP * GP, "the L1 block inverses use X as scratch");

// xLARFG from alpha and the squared tail norm, FP32 panels: the norm as
// sqrt(alpha^2 + ss) (hypot only when that overflows) and correctly rounded
// reciprocals instead of divisions.
__device__ __forceinline__ void larfg_f32(float alpha, float ss, float& beta, float& tau, float& scal) {
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

__device__ __forceinline__ float hsum(float v, unsigned m) {
  v += __shfl_xor_sync(m, v, 8);
  v += __shfl_xor_sync(m, v, 4);
  v += __shfl_xor_sync(m, v, 2);
  v += __shfl_xor_sync(m, v, 1);
  return v;
}

__device__ __forceinline__ void ld8(float (&v)[8], const float* p) {   // p 16-byte aligned
  const float4 a = reinterpret_cast<const float4*>(p)[0];
  const float4 b = reinterpret_cast<const float4*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void st8(float* p, const float (&v)[8]) {
  reinterpret_cast<float4*>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
  reinterpret_cast<float4*>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
}

// Strictly upper part of the Gram matrix: G(a, b) = sum_{r < len} Yt[r*KP + a] Yt[r*KP + b]
// for a < b < nb.  Ends with a barrier.
__device__ void blk_gram(int nb, int len, const float* Yt, float* G) {
  for (int o = threadIdx.x; o < nb * nb; o += FT) {
    const int b = o % nb, a = o / nb;
    if (a >= b) continue;
    float s0 = 0.f, s1 = 0.f;
    int r = 0;
    for (; r + 1 < len; r += 2) {
      s0 = fmaf(Yt[r * KP + a], Yt[r * KP + b], s0);
      s1 = fmaf(Yt[(r + 1) * KP + a], Yt[(r + 1) * KP + b], s1);
    }
    if (r < len) s0 = fmaf(Yt[r * KP + a], Yt[r * KP + b], s0);
    G[a * GP + b] = s0 + s1;
  }
  __syncthreads();
}

// T = S^{-1} explicitly (S = diag(1/tau) + strictly upper G) by warp 0, one
// row of T per lane in registers, columns in order (the recurrence of xLARFT):
// T(i,i) = tau_i, T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i).  G's column i is
// read as broadcasts; every step is 32 lanes' independent dot products.
// Tm is row-major (ld GP), zero outside the upper triangle; also written to Tg
// (32 x 32, column-major) for the solve.  Ends with a barrier.
__device__ void blk_tmat(int nb, const float* G, const float* tau, float* Tm, float* Tg) {
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    float tr[BP];
#pragma unroll
    for (int q = 0; q < BP; ++q) tr[q] = 0.f;
#pragma unroll
    for (int i = 0; i < BP; ++i) {
      if (i < nb) {   // warp-uniform
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int q = 0; q < i; ++q) {
          if (q & 1) s1 = fmaf(tr[q], G[q * GP + i], s1);
          else s0 = fmaf(tr[q], G[q * GP + i], s0);
        }
        const float ti = tau[i];
        tr[i] = l < i ? -ti * (s0 + s1) : (l == i ? ti : 0.f);
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

// Inverses of the 32 x 32 diagonal blocks of L1 = lower part of D[0:mk, 0:mk]
// (ld LDD), block p by warp p: lane b holds column b of the inverse in
// registers, rows in order (forward substitution, L(a, 0:a) read as
// broadcasts); written column-major to Lg + 1024 p through `scr`
// (4 x 32 x 33 floats) so that the global stores are coalesced.
__device__ void blk_linv(int mk, const float* sD, int LDD, float* scr, float* Lg) {
  const int w = threadIdx.x >> 5, b = threadIdx.x & 31;
  const int i0 = w * BP;
  if (i0 < mk && w < 4) {
    const int nb = min(BP, mk - i0);
    float xc[BP];
#pragma unroll
    for (int a = 0; a < BP; ++a) xc[a] = 0.f;
#pragma unroll
    for (int a = 0; a < BP; ++a) {
      if (a < nb) {   // warp-uniform
        const float* La = sD + (i0 + a) + (int64_t)i0 * LDD;   // L(a, q) = La[q * LDD]
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int q = 0; q < a; ++q) {
          if (q & 1) s1 = fmaf(La[q * LDD], xc[q], s1);
          else s0 = fmaf(La[q * LDD], xc[q], s0);
        }
        const float r = __frcp_rn(La[a * LDD]);
        xc[a] = a == b ? r : (a > b ? -(s0 + s1) * r : 0.f);
      }
    }
    float* x = scr + w * BP * GP;   // row-major a*GP + b
#pragma unroll
    for (int a = 0; a < BP; ++a) x[a * GP + b] = xc[a];
    __syncwarp();
    for (int e = b; e < BP * BP; e += 32) Lg[w * 1024 + e] = x[(e % BP) * GP + e / BP];
  }
  __syncthreads();
}

// C (rows 0..m-1, N columns, ld ldc) <- C - Y (T (Y^T C)), Y = Yc (reflector-major,
// nb x m) / Yt (row-major, m x nb).  Ends with a barrier.
__device__ void blk_apply_left(float* C, int ldc, int m, int N, int nb, const float* Yc, const float* Yt,
                               const float* Tm, float* X) {
  const int tid = threadIdx.x;
  const int j = tid & 127, cb = tid >> 7;   // column, block of 8 reflectors
  // X = Y^T C (nb x N)
  if (j < N && cb * 8 < nb) {
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int r = 0; r < m; ++r) {
      const float c = C[r + j * ldc];
      float y[8];
      ld8(y, Yt + r * KP + cb * 8);
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = fmaf(y[q], c, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (cb * 8 + q < nb) X[(cb * 8 + q) * XP + j] = acc[q];
  }
  __syncthreads();
  // X = T X (T upper)
  float nx[8];
  if (j < N && cb * 8 < nb) {
#pragma unroll
    for (int q = 0; q < 8; ++q) nx[q] = 0.f;
    for (int c2 = cb * 8; c2 < nb; ++c2) {
      const float xv = X[c2 * XP + j];
#pragma unroll
      for (int q = 0; q < 8; ++q) nx[q] = fmaf(Tm[(cb * 8 + q) * GP + c2], xv, nx[q]);
    }
  }
  __syncthreads();
  if (j < N && cb * 8 < nb) {
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (cb * 8 + q < nb) X[(cb * 8 + q) * XP + j] = nx[q];
  }
  __syncthreads();
  // C -= Y X
  if (j < N) {
    for (int r0 = cb * 8; r0 < m; r0 += 32) {
      float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      for (int c = 0; c < nb; ++c) {
        const float xv = X[c * XP + j];
        float y[8];
        ld8(y, Yc + c * YP + r0);
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = fmaf(y[q], xv, acc[q]);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (r0 + q < m) C[r0 + q + j * ldc] -= acc[q];
    }
  }
  __syncthreads();
}

// Rows r0..m-1 of C (n columns, ld ldc) <- C - (C Y^T) T Y with Y = Yc (nb x n,
// reflector-major) / Yt (n x nb).  Ends with a barrier.
__device__ void blk_apply_right(float* C, int ldc, int r0, int m, int n, int nb, const float* Yc, const float* Yt,
                                const float* Tm, float* X) {
  const int tid = threadIdx.x;
  const int r = r0 + (tid & 127), ab = tid >> 7;
  const bool act = r < m && ab * 8 < nb;
  // X = C Y^T ((m - r0) x nb), stored reflector-major
  if (act) {
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int col = 0; col < n; ++col) {
      const float c = C[r + col * ldc];
      float y[8];
      ld8(y, Yt + col * KP + ab * 8);
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = fmaf(c, y[q], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (ab * 8 + q < nb) X[(ab * 8 + q) * XP + (r - r0)] = acc[q];
  }
  __syncthreads();
  // X = X T (T upper)
  float nx[8];
  if (act) {
#pragma unroll
    for (int q = 0; q < 8; ++q) nx[q] = 0.f;
    const int hi = min(nb, ab * 8 + 8);
    for (int a2 = 0; a2 < hi; ++a2) {
      const float xv = X[a2 * XP + (r - r0)];
#pragma unroll
      for (int q = 0; q < 8; ++q) nx[q] = fmaf(xv, Tm[a2 * GP + ab * 8 + q], nx[q]);
    }
  }
  __syncthreads();
  if (act) {
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (ab * 8 + q < nb) X[(ab * 8 + q) * XP + (r - r0)] = nx[q];
  }
  __syncthreads();
  // C -= X Y
  if (r < m) {
    for (int col0 = ab * 8; col0 < n; col0 += 32) {
      float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      for (int a = 0; a < nb; ++a) {
        const float xv = X[a * XP + (r - r0)];
        float y[8];
        ld8(y, Yc + a * YP + col0);
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = fmaf(xv, y[q], acc[q]);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (col0 + q < n) C[r + (col0 + q) * ldc] -= acc[q];
    }
  }
  __syncthreads();
}

// V (n x kv, ld ldv) <- V - Y^T (T^T (Y V)).  Ends with a barrier.
__device__ void blk_apply_v(float* V, int ldv, int n, int kv, int nb, const float* Yc, const float* Yt,
                            const float* Tm, float* X) {
  const int tid = threadIdx.x;
  // Z = Y V (nb x kv): thread (column c, block of 4 reflectors)
  for (int o = tid; o < kv * 8; o += FT) {
    const int c = o % kv, ab = o / kv;
    if (ab * 4 >= nb) continue;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int col = 0; col < n; ++col) {
      const float v = V[col + c * ldv];
      const float4 y = *reinterpret_cast<const float4*>(Yt + col * KP + ab * 4);
      acc[0] = fmaf(y.x, v, acc[0]);
      acc[1] = fmaf(y.y, v, acc[1]);
      acc[2] = fmaf(y.z, v, acc[2]);
      acc[3] = fmaf(y.w, v, acc[3]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (ab * 4 + q < nb) X[(ab * 4 + q) * XP + c] = acc[q];
  }
  __syncthreads();
  // Z = T^T Z
  {
    float nz[4] = {0.f, 0.f, 0.f, 0.f};
    const int c = tid % kv, ab = tid / kv;   // kv * 8 <= 512 threads
    const bool act = tid < kv * 8 && ab * 4 < nb;
    if (act) {
      const int hi = min(nb, ab * 4 + 4);
      for (int a2 = 0; a2 < hi; ++a2) {
        const float zv = X[a2 * XP + c];
#pragma unroll
        for (int q = 0; q < 4; ++q) nz[q] = fmaf(Tm[a2 * GP + ab * 4 + q], zv, nz[q]);
      }
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (ab * 4 + q < nb) X[(ab * 4 + q) * XP + c] = nz[q];
    }
  }
  __syncthreads();
  // V -= Y^T Z: thread (row col, block of 8 columns of V)
  const int col = tid & 127, cb = tid >> 7;
  if (col < n) {
    for (int c0 = cb * 8; c0 < kv; c0 += 32) {
      float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      for (int a = 0; a < nb; ++a) {
        const float y = Yc[a * YP + col];
        float z[8];
        ld8(z, X + a * XP + c0);
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = fmaf(y, z[q], acc[q]);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (c0 + q < kv) V[col + (c0 + q) * ldv] -= acc[q];
    }
  }
  __syncthreads();
}

// P1 + P2 of one node in FP32 (see above).  In: sD (m x n) and sU (m x ku),
// ld LDD, and sV (n x kv, ld LDV) in shared memory.  Out: the same blocks in
// shared memory plus tau vectors and the transposed LQ reflectors in global
// memory (tq, tl, gQt).
__device__ void ulv_reduce_blocked(const Node& nd, float* sD, float* sU, int LDD, float* sV, int LDV, float* sv,
                                   float* stau, float* blk, float* tq, float* tl, float* gQt, float* gTq, float* gTl,
                                   float* gLi) {
  const int m = nd.m, n = nd.n, k = nd.k, mk = nd.mk, kv = nd.kv;
  const int tid = threadIdx.x;
  const unsigned hm = 0xFFFFu << (tid & 16);   // this thread's half-warp
  const int hl = tid & 16;                     // its first lane
  float* Yc = blk;                             // BP x YP
  float* Yt = Yc + BP * YP;                    // FMAX x KP
  float* X = Yt + FMAX * KP;                   // BP x XP
  float* G = X + BP * XP;                      // BP x GP (strictly upper part used)
  float* Tm = G + BP * GP;                     // BP x GP, row-major T of the panel
  float* ptau = Tm + BP * GP;                  // BP taus of the panel

  // ---- P1: QL of U, panels of BP columns from the last -----------------------
  {
    const int cc = tid >> 4, rs = tid & 15, r0 = rs * 8;
    for (int c1 = k; c1 > 0; c1 -= BP) {
      const int c0 = max(0, c1 - BP), nb = c1 - c0;
      const int col = c0 + cc;
      float u[8];
#pragma unroll
      for (int l = 0; l < 8; ++l) u[l] = (cc < nb && r0 + l < m) ? sU[r0 + l + col * LDD] : 0.f;
      auto gen = [&](int c, int buf) {   // the 16 threads of column c
        const int p = mk + c;
        float ss = 0.f, mine = 0.f;
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const int row = r0 + l;
          if (row < p) ss = fmaf(u[l], u[l], ss);
          if (row == p) mine = u[l];
        }
        ss = hsum(ss, hm);
        const float alpha = __shfl_sync(hm, mine, hl + (p >> 3));
        float beta, tau, sc;
        larfg_f32(alpha, ss, beta, tau, sc);
        float v[8];
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const int row = r0 + l;
          if (row < p && tau != 0.f) u[l] *= sc;
          if (row == p) u[l] = beta;
          v[l] = row < p ? u[l] : (row == p ? 1.f : 0.f);
        }
        st8(sv + buf * SVLEN + r0, v);
        if (rs == 0) {
          stau[buf] = tau;
          ptau[c - c0] = tau;
          tq[c] = tau;
        }
      };
      if (cc == nb - 1) gen(c1 - 1, 0);
      __syncthreads();
      for (int c = c1 - 1; c >= c0; --c) {
        const int cur = (c1 - 1 - c) & 1;
        const float tau = stau[cur];
        if (cc < c - c0 && tau != 0.f) {
          float v[8];
          ld8(v, sv + cur * SVLEN + r0);
          float w = 0.f;
#pragma unroll
          for (int l = 0; l < 8; ++l) w = fmaf(v[l], u[l], w);
          w = hsum(w, hm) * tau;
#pragma unroll
          for (int l = 0; l < 8; ++l) u[l] = fmaf(-w, v[l], u[l]);
        }
        if (c > c0 && cc == c - 1 - c0) gen(c - 1, cur ^ 1);
        __syncthreads();
      }
      // write back the panel and its reflectors (Y zero below each pivot)
      if (cc < nb) {
        const int p = mk + col;
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const int row = r0 + l;
          if (row < m) {
            sU[row + col * LDD] = u[l];
            const float y = row < p ? u[l] : (row == p ? 1.f : 0.f);
            Yc[cc * YP + row] = y;
            Yt[row * KP + cc] = y;
          }
        }
      }
      __syncthreads();
      blk_gram(nb, m, Yt, G);
      blk_tmat(nb, G, ptau, Tm, gTq + (int64_t)((k - c1) / BP) * 1024);
      blk_apply_left(sD, LDD, m, n, nb, Yc, Yt, Tm, X);
      if (c0 > 0) blk_apply_left(sU, LDD, m, c0, nb, Yc, Yt, Tm, X);
    }
  }

  // ---- P2: LQ of D[0:mk, :], panels of BP rows ------------------------------
  {
    const int rr = tid >> 4, cs = tid & 15, q0 = cs * 8;
    for (int i0 = 0; i0 < mk; i0 += BP) {
      const int i1 = min(mk, i0 + BP), nb = i1 - i0;
      const int row = i0 + rr;
      float d[8];
#pragma unroll
      for (int l = 0; l < 8; ++l) d[l] = (rr < nb && q0 + l < n) ? sD[row + (q0 + l) * LDD] : 0.f;
      auto gen = [&](int i, int buf) {   // the 16 threads of row i
        float ss = 0.f, mine = 0.f;
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const int col = q0 + l;
          if (col > i) ss = fmaf(d[l], d[l], ss);
          if (col == i) mine = d[l];
        }
        ss = hsum(ss, hm);
        const float alpha = __shfl_sync(hm, mine, hl + (i >> 3));
        float beta, tau, sc;
        larfg_f32(alpha, ss, beta, tau, sc);
        float v[8];
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const int col = q0 + l;
          if (col > i && tau != 0.f) d[l] *= sc;
          if (col == i) d[l] = beta;
          v[l] = col < i ? 0.f : (col == i ? 1.f : d[l]);
        }
        st8(sv + buf * SVLEN + q0, v);
        if (cs == 0) {
          stau[buf] = tau;
          ptau[i - i0] = tau;
          tl[i] = tau;
        }
      };
      if (rr == 0) gen(i0, 0);
      __syncthreads();
      for (int i = i0; i < i1; ++i) {
        const int cur = (i - i0) & 1;
        const float tau = stau[cur];
        if (rr > i - i0 && rr < nb && tau != 0.f) {
          float v[8];
          ld8(v, sv + cur * SVLEN + q0);
          float w = 0.f;
#pragma unroll
          for (int l = 0; l < 8; ++l) w = fmaf(v[l], d[l], w);
          w = hsum(w, hm) * tau;
#pragma unroll
          for (int l = 0; l < 8; ++l) d[l] = fmaf(-w, v[l], d[l]);
        }
        if (i + 1 < i1 && rr == i + 1 - i0) gen(i + 1, cur ^ 1);
        __syncthreads();
      }
      if (rr < nb) {
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const int col = q0 + l;
          if (col < n) {
            sD[row + col * LDD] = d[l];
            const float y = col < row ? 0.f : (col == row ? 1.f : d[l]);
            Yc[rr * YP + col] = y;
            Yt[col * KP + rr] = y;
            gQt[col + (int64_t)row * n] = y;
          }
        }
      }
      __syncthreads();
      blk_gram(nb, n, Yt, G);
      blk_tmat(nb, G, ptau, Tm, gTl + (int64_t)(i0 / BP) * 1024);
      if (i1 < m) blk_apply_right(sD, LDD, i1, m, n, nb, Yc, Yt, Tm, X);
      if (kv > 0) blk_apply_v(sV, LDV, n, kv, nb, Yc, Yt, Tm, X);
    }
  }
  // inverses of L1's diagonal blocks for the solve (X is free now)
  blk_linv(mk, sD, LDD, X, gLi);
}

template <typename T>
__global__ void __launch_bounds__(FT, 1) ulv_factor_fast_kernel(const Task* __restrict__ tasks,
                                                                const Slot* __restrict__ slots,
                                                                int LDD, int nmax, int kumax, int kvmax,
                                                                int extra) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ T red[FW];
  __shared__ T scal3[3];
  __shared__ int bi[FW];
  __shared__ int prow;
  __shared__ T stau[2];
  const Task tk = tasks[blockIdx.x];
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* fb = (T*)sl.fbase;
  const int m = nd.m, n = nd.n, ku = nd.ku, kv = nd.kv;
  // region starts are rounded up to 4 elements: the broadcast vectors are
  // read with 128-bit loads and must be 16-byte aligned
  T* sD = (T*)smraw;                                // m x n, ld LDD
  T* sU = sD + smem_align4((size_t)LDD * nmax);     // m x ku, ld LDD
  T* part = sU + smem_align4((size_t)LDD * (kumax > 0 ? kumax : 1));
  T* sv = part + 4 * PART_COLS;                     // padded broadcast vectors (2)
  T* sx = sv + 2 * SVLEN;                           // merge staging (branches)
  T* gD = fb + nd.fD;
  T* gU = fb + nd.fU;
  T* gV = fb + nd.fV;
  const int tid = threadIdx.x;

  // ---- P0: load or assemble the node's block --------------------------------
  if (nd.leaf) {
    // column j by warp, rows by lane: coalesced, no index division
    const int lane = tid & 31, warp = tid >> 5;
    const double* gD0 = nd.D;
    const double* gU0 = nd.U;
#pragma unroll 2
    for (int j = warp; j < n; j += FW) {
      const double* col = gD0 + (int64_t)j * m;
#pragma unroll 4
      for (int i = lane; i < m; i += 32) sD[i + j * LDD] = (T)__ldg(col + i);
    }
    if (!nd.root)
      for (int j = warp; j < ku; j += FW) {
        const double* col = gU0 + (int64_t)j * m;
#pragma unroll 4
        for (int i = lane; i < m; i += 32) sU[i + j * LDD] = (T)__ldg(col + i);
      }
  } else {
    // Merge (src/ulvfactor.jl:74-79).  Generator blocks are converted to T
    // once and, with the children's reduced U and V, staged in shared memory.
    const Node& c1 = nodes[nd.left];
    const Node& c2 = nodes[nd.right];
    const int u1 = c1.ku, u2 = c2.ku, v1 = c1.kv, v2 = c2.kv;
    const int mr1 = c1.mr, mr2 = c2.mr, nr1 = c1.nr, nr2 = c2.nr;
    const int kuo = nd.root ? 0 : ku, kvo = nd.root ? 0 : kv;
    T* gB12 = sx;                     // u1 x v2
    T* gB21 = gB12 + u1 * v2;         // u2 x v1
    T* gR1 = gB21 + u2 * v1;          // u1 x ku
    T* gR2 = gR1 + u1 * kuo;          // u2 x ku
    T* gW1 = gR2 + u2 * kuo;          // v1 x kv
    T* gW2 = gW1 + v1 * kvo;          // v2 x kv
    T* cU1 = gW2 + v2 * kvo;          // mr1 x u1 (tril applied when reduced)
    T* cU2 = cU1 + mr1 * u1;          // mr2 x u2
    T* cV1 = cU2 + mr2 * u2;          // nr1 x v1
    T* cV2 = cV1 + nr1 * v1;          // nr2 x v2
    T* sT12 = cV2 + nr2 * v2;         // mr1 x v2
    T* sT21 = sT12 + mr1 * v2;        // mr2 x v1
    for (int e = tid; e < u1 * v2; e += FT) gB12[e] = (T)nd.B12[e];
    for (int e = tid; e < u2 * v1; e += FT) gB21[e] = (T)nd.B21[e];
    for (int e = tid; e < u1 * kuo; e += FT) gR1[e] = (T)nd.R1[e];
    for (int e = tid; e < u2 * kuo; e += FT) gR2[e] = (T)nd.R2[e];
    for (int e = tid; e < v1 * kvo; e += FT) gW1[e] = (T)nd.W1[e];
    for (int e = tid; e < v2 * kvo; e += FT) gW2[e] = (T)nd.W2[e];
    {
      const T* U1 = fb + c1.fU + c1.mk;   // ld c1.m
      const T* U2 = fb + c2.fU + c2.mk;
      const T* V1 = fb + c1.fV + c1.nk;   // ld c1.n
      const T* V2 = fb + c2.fV + c2.nk;
      for (int e = tid; e < mr1 * u1; e += FT) {
        const int i = e % mr1, l = e / mr1;
        cU1[e] = (c1.lower_u && l > i) ? T(0) : U1[i + (int64_t)l * c1.m];
      }
      for (int e = tid; e < mr2 * u2; e += FT) {
        const int i = e % mr2, l = e / mr2;
        cU2[e] = (c2.lower_u && l > i) ? T(0) : U2[i + (int64_t)l * c2.m];
      }
      for (int e = tid; e < nr1 * v1; e += FT) cV1[e] = V1[(e % nr1) + (int64_t)(e / nr1) * c1.n];
      for (int e = tid; e < nr2 * v2; e += FT) cV2[e] = V2[(e % nr2) + (int64_t)(e / nr2) * c2.n];
    }
    __syncthreads();
    T* T12 = fb + nd.fT12;
    T* T21 = fb + nd.fT21;
    for (int o = tid; o < mr1 * v2; o += FT) {
      const int i = o % mr1, j = o / mr1;
      T s = T(0);
      for (int l = 0; l < u1; ++l) s += cU1[i + l * mr1] * gB12[l + j * u1];
      sT12[o] = s;
      T12[o] = s;
    }
    for (int o = tid; o < mr2 * v1; o += FT) {
      const int i = o % mr2, j = o / mr2;
      T s = T(0);
      for (int l = 0; l < u2; ++l) s += cU2[i + l * mr2] * gB21[l + j * u2];
      sT21[o] = s;
      T21[o] = s;
    }
    if (!nd.root) {
      for (int o = tid; o < m * ku; o += FT) {
        const int i = o % m, j = o / m;
        T s = T(0);
        if (i < mr1) {
          for (int l = 0; l < u1; ++l) s += cU1[i + l * mr1] * gR1[l + j * u1];
        } else {
          const int i2 = i - mr1;
          for (int l = 0; l < u2; ++l) s += cU2[i2 + l * mr2] * gR2[l + j * u2];
        }
        sU[i + j * LDD] = s;
      }
      for (int o = tid; o < n * kv; o += FT) {
        const int i = o % n, j = o / n;
        T s = T(0);
        if (i < nr1) {
          for (int l = 0; l < v1; ++l) s += cV1[i + l * nr1] * gW1[l + j * v1];
        } else {
          const int i2 = i - nr1;
          for (int l = 0; l < v2; ++l) s += cV2[i2 + l * nr2] * gW2[l + j * v2];
        }
        gV[i + (int64_t)j * n] = s;
      }
    }
    __syncthreads();
    const T* D1 = fb + c1.fD + c1.mk + (int64_t)c1.nk * c1.m;
    const T* D2 = fb + c2.fD + c2.mk + (int64_t)c2.nk * c2.m;
    for (int o = tid; o < m * n; o += FT) {
      const int i = o % m, j = o / m;
      T val;
      if (i < mr1) {
        if (j < nr1) {
          val = D1[i + (int64_t)j * c1.m];
        } else {
          const int j2 = j - nr1;
          T s = T(0);
          for (int l = 0; l < v2; ++l) s += sT12[i + l * mr1] * cV2[j2 + l * nr2];
          val = s;
        }
      } else {
        const int i2 = i - mr1;
        if (j < nr1) {
          T s = T(0);
          for (int l = 0; l < v1; ++l) s += sT21[i2 + l * mr2] * cV1[j + l * nr1];
          val = s;
        } else {
          val = D2[i2 + (int64_t)(j - nr1) * c2.m];
        }
      }
      sD[i + j * LDD] = val;
    }
  }
  __syncthreads();

  if (nd.root) {
    lu_smem(sD, m, LDD, (int32_t*)(fb + nd.fpiv), sl.err, red, bi, &prow);
    for (int e = tid; e < m * n; e += FT) gD[e] = sD[(e % m) + (e / m) * LDD];
    return;
  }
  if (nd.mk == 0) {
    // nothing to eliminate: the block passes up as it is (src/ulvfactor.jl:32-36)
    for (int e = tid; e < m * n; e += FT) gD[e] = sD[(e % m) + (e / m) * LDD];
    for (int e = tid; e < m * ku; e += FT) gU[e] = sU[(e % m) + (e / m) * LDD];
    if (nd.leaf)
      for (int e = tid; e < n * kv; e += FT) gV[e] = (T)nd.V[e];
    return;
  }

  const int k = nd.k, mk = nd.mk;
  T* tq = fb + nd.ftq;
  T* tl = fb + nd.ftl;

  if constexpr (sizeof(T) == 4) {
    // FP32: blocked reduction with the block and V in shared memory; its
    // buffers reuse the merge staging region (dead after the assembly)
    const int LDV = nmax | 1;
    T* sVb = sx;
    T* blk = sVb + smem_align4((size_t)LDV * (kvmax > 0 ? kvmax : 1));
    {
      const int lane = tid & 31, warp = tid >> 5;
      const double* gV0 = nd.V;
      for (int c = warp; c < kv; c += FW)
#pragma unroll 4
        for (int row = lane; row < n; row += 32)
          sVb[row + c * LDV] = nd.leaf ? (T)__ldg(gV0 + row + (int64_t)c * n) : gV[row + (int64_t)c * n];
    }
    __syncthreads();
    ulv_reduce_blocked(nd, sD, sU, LDD, sVb, LDV, sv, stau, blk, tq, tl, fb + nd.fQt, fb + nd.fTq, fb + nd.fTl,
                       fb + nd.fLi);
    for (int e = tid; e < m * n; e += FT) gD[e] = sD[(e % m) + (e / m) * LDD];
    for (int e = tid; e < m * ku; e += FT) gU[e] = sU[(e % m) + (e / m) * LDD];
    for (int e = tid; e < n * kv; e += FT) gV[e] = sVb[(e % n) + (e / n) * LDV];
  } else {

  // ---- P1: QL of U, Q^T applied to D -------------------------------------------
  // Broadcast vectors are double-buffered: while every thread applies reflector
  // c, the owner of the next column (already updated) builds reflector c-1, so
  // each step needs one barrier.
  T* sv0 = sv;
  T* sv1 = sv + SVLEN;
  {
    // FP64: the working block stays in shared memory; one thread per column
    // and row quarter, partial dot products combined through shared memory.
    const int cs = tid & 127, rq = tid >> 7, r0 = rq * 32;
    for (int c = k - 1; c >= 0; --c) {
      const int p = mk + c;
      T* u = sU + c * LDD;
      T ss = (tid < p) ? u[tid] * u[tid] : T(0);
      ss = bsum(ss, red);
      if (tid == 0) {
        T beta, tau, sc;
        larfg(u[p], ss, beta, tau, sc);
        scal3[0] = beta; scal3[1] = tau; scal3[2] = sc;
      }
      __syncthreads();
      const T tau = scal3[1];
      if (tau != T(0) && tid < p) u[tid] *= scal3[2];
      __syncthreads();
      if (tid == 0) { u[p] = scal3[0]; tq[c] = tau; }
      if (tau == T(0)) { __syncthreads(); continue; }
      const int lim = min(32, p + 1 - r0);
      T vr[32];
#pragma unroll
      for (int l = 0; l < 32; ++l) {
        const int i = r0 + l;
        vr[l] = (l < lim) ? (i < p ? u[i] : T(1)) : T(0);
      }
      const int ncols = c + n;
      for (int col = cs; col < ncols; col += 128) {
        const T* cp = col < n ? sD + col * LDD : sU + (col - n) * LDD;
        T sacc = T(0);
#pragma unroll
        for (int l = 0; l < 32; ++l)
          if (l < lim) sacc += vr[l] * cp[r0 + l];
        part[rq * PART_COLS + col] = sacc;
      }
      __syncthreads();
      for (int col = cs; col < ncols; col += 128) {
        T* cp = col < n ? sD + col * LDD : sU + (col - n) * LDD;
        const T w = tau * (part[col] + part[PART_COLS + col] + part[2 * PART_COLS + col] +
                           part[3 * PART_COLS + col]);
#pragma unroll
        for (int l = 0; l < 32; ++l)
          if (l < lim) cp[r0 + l] -= w * vr[l];
      }
      __syncthreads();
    }
    for (int e = tid; e < m * ku; e += FT) gU[e] = sU[(e % m) + (e / m) * LDD];
  }

  // ---- P2: LQ of D[0:mk, :], applied to D[i+1:m, :] and to V (registers) ----
  const int j = tid >> 2, q = tid & 3, c0 = q * 32;
  const unsigned gmask = 0xFu << ((tid & 31) & ~3);     // the 4 lanes of row j
  T d[32];
#pragma unroll
  for (int l = 0; l < 32; ++l) {
    const int col = c0 + l;
    d[l] = (j < m && col < n) ? sD[j + col * LDD] : T(0);
  }
  const int vcol = tid >> 4, vseg = tid & 15;
  T vv[2][8];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int c = vcol + 32 * h;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int row = 8 * vseg + r;
      T x = T(0);
      if (c < kv && row < n) x = nd.leaf ? (T)nd.V[row + (int64_t)c * n] : gV[row + (int64_t)c * n];
      vv[h][r] = x;
    }
  }
  const int nl = min(mk, n);
  auto lq_reflector = [&](int i, T* buf, int slot) {   // called by the 4 owners of row i
    T s4[4] = {T(0), T(0), T(0), T(0)}, mine = T(0);
#pragma unroll
    for (int l = 0; l < 32; ++l) {
      const int col = c0 + l;
      if (col > i) s4[l & 3] += d[l] * d[l];
      if (col == i) mine = d[l];
    }
    T ss = (s4[0] + s4[1]) + (s4[2] + s4[3]);
    ss += __shfl_xor_sync(gmask, ss, 1);
    ss += __shfl_xor_sync(gmask, ss, 2);
    const T alpha = __shfl_sync(gmask, mine, i >> 5, 4);
    T beta, tau, sc;
    larfg(alpha, ss, beta, tau, sc);
#pragma unroll
    for (int l = 0; l < 32; ++l) {
      const int col = c0 + l;
      if (col > i && tau != T(0)) d[l] *= sc;
      if (col == i) d[l] = beta;
      buf[vp(col)] = col < i ? T(0) : (col == i ? T(1) : d[l]);
    }
    if (q == 0) { stau[slot] = tau; tl[i] = tau; }
  };
  if (nl > 0 && j == 0) lq_reflector(0, sv0, 0);
  __syncthreads();
  for (int i = 0; i < nl; ++i) {
    const int cur = i & 1;
    const T* svc = cur ? sv1 : sv0;
    const T tau = stau[cur];
    if (tau != T(0)) {
      if (j > i && j < m) {
        T vq[32];
        load_quarter(vq, svc, q);
        T w = dot32(d, vq);
        w += __shfl_xor_sync(gmask, w, 1);
        w += __shfl_xor_sync(gmask, w, 2);
        w *= tau;
#pragma unroll
        for (int l = 0; l < 32; ++l) d[l] -= w * vq[l];
      }
      {
        // every lane takes part (columns >= kv hold zeros): full-warp shuffles
        T sr[8];
        const T* vb = svc + vp(8 * vseg);   // 8 consecutive entries, 16-byte aligned
        if constexpr (sizeof(T) == 4) {
          const float4 a = reinterpret_cast<const float4*>(vb)[0];
          const float4 b = reinterpret_cast<const float4*>(vb)[1];
          sr[0] = a.x; sr[1] = a.y; sr[2] = a.z; sr[3] = a.w;
          sr[4] = b.x; sr[5] = b.y; sr[6] = b.z; sr[7] = b.w;
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const double2 a = reinterpret_cast<const double2*>(vb)[k];
            sr[2 * k] = a.x; sr[2 * k + 1] = a.y;
          }
        }
        T w0a = T(0), w0b = T(0), w1a = T(0), w1b = T(0);
#pragma unroll
        for (int r = 0; r < 8; r += 2) {
          w0a += sr[r] * vv[0][r];
          w0b += sr[r + 1] * vv[0][r + 1];
          w1a += sr[r] * vv[1][r];
          w1b += sr[r + 1] * vv[1][r + 1];
        }
        T w0 = w0a + w0b, w1 = w1a + w1b;
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
          w0 += __shfl_xor_sync(0xffffffffu, w0, o);
          w1 += __shfl_xor_sync(0xffffffffu, w1, o);
        }
        w0 *= tau;
        w1 *= tau;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          vv[0][r] -= w0 * sr[r];
          vv[1][r] -= w1 * sr[r];
        }
      }
    }
    if (i + 1 < nl && j == i + 1) lq_reflector(i + 1, cur ? sv0 : sv1, cur ^ 1);
    __syncthreads();
  }
  T* gQt = fb + nd.fQt;
#pragma unroll
  for (int l = 0; l < 32; ++l) {
    const int col = c0 + l;
    if (j < m && col < n) gD[j + (int64_t)col * m] = d[l];
    if (j < mk && col < n) gQt[col + (int64_t)j * n] = col < j ? T(0) : (col == j ? T(1) : d[l]);
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int c = vcol + 32 * h;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int row = 8 * vseg + r;
      if (c < kv && row < n) gV[row + (int64_t)c * n] = vv[h][r];
    }
  }
  }
}

}  // namespace

template <typename T>
size_t factor_fast_smem(int mmax, int nmax, int kumax, int kvmax, size_t extra) {
  const int LDD = mmax | 1;
  size_t e = smem_align4((size_t)LDD * nmax) + smem_align4((size_t)LDD * (kumax > 0 ? kumax : 1)) + 4 * PART_COLS +
             2 * SVLEN;
  // the FP32 blocked buffers (V and the panel workspace) overlay the merge staging
  const size_t blk = sizeof(T) == 4 ? smem_align4((size_t)(nmax | 1) * (kvmax > 0 ? kvmax : 1)) + kBlkElems : 0;
  e += std::max(smem_align4(extra), blk);
  return e * sizeof(T);
}

template <typename T>
bool factor_fast_fits(int mmax, int nmax, int kumax, int kvmax, size_t extra) {
  return mmax <= FMAX && nmax <= FMAX && kumax <= FKMAX && kvmax <= FKMAX &&
         factor_fast_smem<T>(mmax, nmax, kumax, kvmax, extra) <= kFastSmemCap;
}

template <typename T>
void launch_ulv_factor_fast(const Task* t, int64_t nt, const Slot* s, int mmax, int nmax, int kumax, int kvmax,
                            size_t extra, cudaStream_t st) {
  if (nt <= 0) return;
  const size_t smem = factor_fast_smem<T>(mmax, nmax, kumax, kvmax, extra);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(ulv_factor_fast_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFastSmemCap);
    attr_set = true;
  }
  ulv_factor_fast_kernel<T><<<(unsigned)nt, FT, smem, st>>>(t, s, mmax | 1, nmax, kumax, kvmax, (int)extra);
}

template bool factor_fast_fits<double>(int, int, int, int, size_t);
template bool factor_fast_fits<float>(int, int, int, int, size_t);
template void launch_ulv_factor_fast<double>(const Task*, int64_t, const Slot*, int, int, int, int, size_t,
                                             cudaStream_t);
template void launch_ulv_factor_fast<float>(const Task*, int64_t, const Slot*, int, int, int, int, size_t,
                                            cudaStream_t);

}  // namespace hss
