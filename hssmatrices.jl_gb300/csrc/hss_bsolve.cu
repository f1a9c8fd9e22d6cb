// Blocked FP32 ULV solve sweeps (reference src/ulvfactor.jl:10-107) over a
// factorization made by the blocked reduction (hss_factor_blk.cu), which
// also stores, per node, the compact-WY T of every panel of 32 QL and LQ
// reflectors and the inverses of L1's 32 x 32 diagonal blocks.
//
// One thread block per (node, chunk of 32 right-hand sides); the chunk lives
// row-major in shared memory (lane = column) and every step is a small GEMM:
//   upward (per node, :22-57, :74, :89)
//     b = rhs rows (leaf) or [b1; b2] - [T12 u2; T21 u1] (branch)
//     b <- Q_ql^T b = (I - Y T Y^T) b per QL panel (generation order)
//     z = L1 \ b[0:mk]: per 32-row block, rhs -= L1(blk, 0:i0) z(0:i0), z(blk) = inv(L1(blk, blk)) rhs
//     b_red = b[mk:m] - L2 z;  u = V[0:mk, :]^T z (+ W1^T u1 + W2^T u2);  x[0:mk] = z
//     root: x = LU \ b (:83)
//   downward (:98-107)
//     x <- Q_lq^T x = P_0 P_1 ... x with P_p = I - Y_p^T T_p Y_p, last panel first
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int BT = 256;   // threads: 8 warps
constexpr int CW = 32;    // right-hand sides per block (lane = column)
constexpr int BL = 33;    // ld of the row-major right-hand-side blocks
constexpr int PB = 32;    // reflectors per panel (the factorization's panel width)
constexpr int KPS = 36;   // ld of the reflector-major staged reflectors

__host__ __device__ constexpr int r4(int x) { return (x + 3) & ~3; }
__host__ __device__ constexpr int imax(int a, int b) { return a > b ? a : b; }

enum { MM_SET = 0, MM_ADD = 1, MM_SUB = 2 };

// C(i, j) (=, +=, -=) sum_{l < K} A(i + l*lda) B(l*BL + j) for i < R, j < CW.
// A column-major, 16-byte aligned, lda % 4 == 0 (rows up to r4(R) are read);
// B, C row-major with ld BL.  Warp w takes rows 4w.. + 32s, lane j column j.
template <int MODE>
__device__ void mm(int R, int K, const float* A, int lda, const float* B, float* C) {
  const int j = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i0 = w * 4; i0 < R; i0 += 32) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    const float* ap = A + i0;
#pragma unroll 4
    for (int l = 0; l < K; ++l) {
      const float4 a = *reinterpret_cast<const float4*>(ap + l * lda);
      const float b = B[l * BL + j];
      a0 = fmaf(a.x, b, a0);
      a1 = fmaf(a.y, b, a1);
      a2 = fmaf(a.z, b, a2);
      a3 = fmaf(a.w, b, a3);
    }
    const float acc[4] = {a0, a1, a2, a3};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = i0 + q;
      if (i < R) {
        float* c = C + i * BL + j;
        *c = MODE == MM_SET ? acc[q] : (MODE == MM_ADD ? *c + acc[q] : *c - acc[q]);
      }
    }
  }
}

// dst(i + l*ldd) = src(i + l*lds), i < rows, l < cols (warp per column).
__device__ void stage_cm(float* dst, int ldd, const float* src, int64_t lds, int rows, int cols) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int l = w; l < cols; l += BT / 32)
    for (int i = lane; i < rows; i += 32) dst[i + l * ldd] = __ldg(src + i + (int64_t)l * lds);
}

// dst(l + i*ldd) = src(i + l*lds): the transpose of a column-major block.
__device__ void stage_tr(float* dst, int ldd, const float* src, int64_t lds, int rows, int cols) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int l = w; l < cols; l += BT / 32)
    for (int i = lane; i < rows; i += 32) dst[l + i * ldd] = __ldg(src + i + (int64_t)l * lds);
}

// Shared-memory layout (floats) of the two kernels, from the level's largest sizes.
struct Lay {
  int sb, su, su1, su2, sX, sX2, sT, sA, sB, total;
};

__host__ __device__ inline Lay layout(int mmax, int nmax, int kmax, int kvmax) {
  const int rows = imax(mmax, nmax);
  const int kk = imax(kmax, 1), kv = imax(kvmax, 1);
  int stage = rows * KPS;
  stage = imax(stage, r4(rows) * PB);
  stage = imax(stage, r4(kk) * rows);
  stage = imax(stage, r4(kv) * rows);
  stage = imax(stage, r4(kk) * kv);
  stage = imax(stage, r4(kv) * kv);
  stage = r4(stage);
  Lay L;
  int o = 0;
  L.sb = o;  o += r4(rows * BL);
  L.su = o;  o += r4(kv * BL);
  L.su1 = o; o += r4(kv * BL);
  L.su2 = o; o += r4(kv * BL);
  L.sX = o;  o += r4(PB * BL);
  L.sX2 = o; o += r4(PB * BL);
  L.sT = o;  o += PB * PB;
  L.sA = o;  o += stage;
  L.sB = o;  o += stage;
  L.total = o;
  return L;
}

// Upward sweep of one node for columns j0 .. j0+31.
__global__ void __launch_bounds__(BT) bsolve_up(const Task* __restrict__ tasks, const Slot* __restrict__ slots,
                                                int nchunk, Lay ly) {
  extern __shared__ __align__(16) float smf[];
  __shared__ Node snd, sc1, sc2;   // node records on chip (no reloads across shared stores)
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * CW;
  const Node* nodes = tk.nodes;
  const Slot& sl = slots[tk.slot];
  const int r = sl.r;
  if (j0 >= r) return;
  if (threadIdx.x == 0) {
    snd = nodes[tk.node];
    if (!snd.leaf) {
      sc1 = nodes[snd.left];
      sc2 = nodes[snd.right];
    }
  }
  __syncthreads();
  const Node& nd = snd;
  float* ws = (float*)sl.ws;
  const int64_t ld = sl.ldws;
  const float* fb = (const float*)sl.fbase;
  const int m = nd.m, k = nd.k, mk = nd.mk, kv = nd.kv, mr = m - mk;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  float* sb = smf + ly.sb;
  float* su = smf + ly.su;
  float* su1 = smf + ly.su1;
  float* su2 = smf + ly.su2;
  float* sX = smf + ly.sX;
  float* sX2 = smf + ly.sX2;
  float* sT = smf + ly.sT;
  float* sA = smf + ly.sA;
  float* sB = smf + ly.sB;
  const int ncol = min(CW, r - j0);

  // ---- b (and the branch part of u)
  if (nd.leaf) {
    const double* B = sl.B + nd.row0;
    for (int q = w; q < CW; q += BT / 32) {
      const int col = j0 + q;
      const double sc = (col < r && sl.colinv) ? sl.colinv[col] : 1.0;
      for (int row = lane; row < m; row += 32)
        sb[row * BL + q] = col < r ? (float)(B[row + (int64_t)col * sl.ldb] * sc) : 0.f;
    }
    if (mk == 0)
      for (int e = tid; e < kv * BL; e += BT) su[e] = 0.f;
  } else {
    const Node& c1 = sc1;
    const Node& c2 = sc2;
    const int kv1 = c1.kv, kv2 = c2.kv, mr1 = c1.mr, mr2 = c2.mr;
    for (int q = w; q < CW; q += BT / 32) {
      const bool cv = q < ncol;
      const int64_t co = (int64_t)(j0 + q) * ld;
      for (int i = lane; i < kv1; i += 32) su1[i * BL + q] = cv ? ws[c1.wu + i + co] : 0.f;
      for (int i = lane; i < kv2; i += 32) su2[i * BL + q] = cv ? ws[c2.wu + i + co] : 0.f;
      for (int i = lane; i < mr1; i += 32) sb[i * BL + q] = cv ? ws[c1.wb + c1.mk + i + co] : 0.f;
      for (int i = lane; i < mr2; i += 32) sb[(mr1 + i) * BL + q] = cv ? ws[c2.wb + c2.mk + i + co] : 0.f;
    }
    stage_cm(sA, r4(mr1), fb + nd.fT12, mr1, mr1, kv2);
    stage_cm(sB, r4(mr2), fb + nd.fT21, mr2, mr2, kv1);
    __syncthreads();
    mm<MM_SUB>(mr1, kv2, sA, r4(mr1), su2, sb);              // b1 -= T12 u2 (:74)
    mm<MM_SUB>(mr2, kv1, sB, r4(mr2), su1, sb + mr1 * BL);   // b2 -= T21 u1
    if (!nd.root) {
      __syncthreads();
      // W1^T, W2^T (FP64 generators) transposed into column-major kv x kv1 / kv x kv2
      const int lk = r4(kv);
      for (int e = tid; e < kv1 * kv; e += BT) sA[(e / kv1) + (e % kv1) * lk] = (float)nd.W1[e];
      for (int e = tid; e < kv2 * kv; e += BT) sB[(e / kv2) + (e % kv2) * lk] = (float)nd.W2[e];
      __syncthreads();
      mm<MM_SET>(kv, kv1, sA, lk, su1, su);   // u = W1^T u1 + W2^T u2 (:89)
      mm<MM_ADD>(kv, kv2, sB, lk, su2, su);
    }
  }
  __syncthreads();

  if (nd.root) {
    // x = LU \ b, column per lane of warp 0 (:83)
    if (w == 0) {
      const float* A = fb + nd.fD;
      const int32_t* piv = (const int32_t*)(fb + nd.fpiv);
      float* b = sb + lane;
      for (int c = 0; c < m; ++c) {
        const int p = piv[c];
        if (p != c) {
          const float t = b[c * BL];
          b[c * BL] = b[p * BL];
          b[p * BL] = t;
        }
      }
      for (int c = 0; c < m; ++c) {
        const float bc = b[c * BL];
        for (int row = c + 1; row < m; ++row) b[row * BL] = fmaf(-A[row + c * m], bc, b[row * BL]);
      }
      for (int c = m - 1; c >= 0; --c) {
        const float bc = b[c * BL] / A[c + c * m];
        b[c * BL] = bc;
        for (int row = 0; row < c; ++row) b[row * BL] = fmaf(-A[row + c * m], bc, b[row * BL]);
      }
    }
    __syncthreads();
    for (int q = w; q < ncol; q += BT / 32)
      for (int row = lane; row < m; row += 32) ws[nd.wx + row + (int64_t)(j0 + q) * ld] = sb[row * BL + q];
    return;
  }

  if (mk > 0) {
    const float* U = fb + nd.fU;   // QL reflectors, m x k
    const float* D = fb + nd.fD;   // L1 (rows 0..mk-1), L2 (rows mk..m-1)
    // b <- Q_ql^T b, panels in generation order (:42)
    for (int c1 = k; c1 > 0; c1 -= PB) {
      const int c0 = max(0, c1 - PB), nb = c1 - c0;
      const int lm = r4(m);
      for (int e = tid; e < m * nb; e += BT) {
        const int row = e % m, c = e / m;
        const int p = mk + c0 + c;
        const float y = row < p ? U[row + (int64_t)(c0 + c) * m] : (row == p ? 1.f : 0.f);
        sA[c + row * KPS] = y;    // Y^T operand
        sB[row + c * lm] = y;     // Y operand
      }
      for (int e = tid; e < PB * PB; e += BT) sT[e] = fb[nd.fTq + (int64_t)((k - c1) / PB) * 1024 + e];
      __syncthreads();
      mm<MM_SET>(nb, m, sA, KPS, sb, sX);   // X = Y^T b
      __syncthreads();
      mm<MM_SET>(nb, nb, sT, PB, sX, sX2);  // X = T X
      __syncthreads();
      mm<MM_SUB>(m, nb, sB, lm, sX2, sb);   // b -= Y X
      __syncthreads();
    }
    // z = L1 \ b[0:mk] (:48), 32-row blocks
    for (int i0 = 0; i0 < mk; i0 += PB) {
      const int nb = min(PB, mk - i0);
      if (i0 > 0) {
        stage_cm(sA, PB, D + i0, m, nb, i0);
        __syncthreads();
        mm<MM_SUB>(nb, i0, sA, PB, sb, sb + i0 * BL);
        __syncthreads();
      }
      for (int e = tid; e < PB * PB; e += BT) sT[e] = fb[nd.fLi + (int64_t)(i0 / PB) * 1024 + e];
      __syncthreads();
      mm<MM_SET>(nb, nb, sT, PB, sb + i0 * BL, sX);
      __syncthreads();
      for (int e = tid; e < nb * BL; e += BT) sb[i0 * BL + e] = sX[e];
      __syncthreads();
    }
    // b_red = b[mk:m] - L2 z (:49);  u (+)= V[0:mk, :]^T z (:51)
    stage_cm(sA, r4(mr), D + mk, m, mr, mk);
    {
      const float* V = fb + nd.fV;
      const int lk = r4(kv);
      for (int e = tid; e < mk * kv; e += BT) {
        const int l = e % mk, c = e / mk;
        sB[c + l * lk] = V[l + (int64_t)c * nd.n];
      }
    }
    __syncthreads();
    mm<MM_SUB>(mr, mk, sA, r4(mr), sb, sb + mk * BL);
    if (nd.leaf) mm<MM_SET>(kv, mk, sB, r4(kv), sb, su);
    else mm<MM_ADD>(kv, mk, sB, r4(kv), sb, su);
    __syncthreads();
  }
  // outputs: b_red, u, x[0:mk] = z
  for (int q = w; q < ncol; q += BT / 32) {
    const int64_t co = (int64_t)(j0 + q) * ld;
    for (int i = lane; i < mr; i += 32) ws[nd.wb + mk + i + co] = sb[(mk + i) * BL + q];
    for (int i = lane; i < kv; i += 32) ws[nd.wu + i + co] = su[i * BL + q];
    for (int i = lane; i < mk; i += 32) ws[nd.wx + i + co] = sb[i * BL + q];
  }
}

// Downward sweep of one node for columns j0 .. j0+31: x <- Q_lq^T x (:102),
// then the un-eliminated tail goes to the children (or the output at a leaf).
__global__ void __launch_bounds__(BT) bsolve_down(const Task* __restrict__ tasks, const Slot* __restrict__ slots,
                                                  int nchunk, Lay ly) {
  extern __shared__ __align__(16) float smf[];
  __shared__ Node snd, sc1, sc2;
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * CW;
  const Node* nodes = tk.nodes;
  const Slot& sl = slots[tk.slot];
  const int r = sl.r;
  if (j0 >= r) return;
  if (threadIdx.x == 0) {
    snd = nodes[tk.node];
    if (!snd.leaf) {
      sc1 = nodes[snd.left];
      sc2 = nodes[snd.right];
    }
  }
  __syncthreads();
  const Node& nd = snd;
  float* ws = (float*)sl.ws;
  const int64_t ld = sl.ldws;
  const float* fb = (const float*)sl.fbase;
  const int n = nd.n, mk = nd.root ? 0 : nd.mk;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  float* sb = smf + ly.sb;
  float* sX = smf + ly.sX;
  float* sX2 = smf + ly.sX2;
  float* sT = smf + ly.sT;
  float* sA = smf + ly.sA;
  float* sB = smf + ly.sB;
  const int ncol = min(CW, r - j0);
  for (int q = w; q < CW; q += BT / 32) {
    const bool cv = q < ncol;
    const int64_t co = (int64_t)(j0 + q) * ld;
    for (int row = lane; row < n; row += 32) sb[row * BL + q] = cv ? ws[nd.wx + row + co] : 0.f;
  }
  if (mk > 0) {
    const float* Qt = fb + nd.fQt;   // n x mk: reflector i in column i
    const int ln = r4(n);
    for (int p = (mk - 1) / PB; p >= 0; --p) {
      const int i0 = p * PB, nb = min(PB, mk - i0);
      __syncthreads();
      stage_tr(sA, KPS, Qt + (int64_t)i0 * n, n, n, nb);   // Y (rows = reflectors)
      stage_cm(sB, ln, Qt + (int64_t)i0 * n, n, n, nb);    // Y^T
      for (int e = tid; e < PB * PB; e += BT) sT[e] = fb[nd.fTl + (int64_t)p * 1024 + e];
      __syncthreads();
      mm<MM_SET>(nb, n, sA, KPS, sb, sX);    // X = Y x
      __syncthreads();
      mm<MM_SET>(nb, nb, sT, PB, sX, sX2);   // X = T X
      __syncthreads();
      mm<MM_SUB>(n, nb, sB, ln, sX2, sb);    // x -= Y^T X
    }
  }
  __syncthreads();
  if (nd.leaf) {
    for (int q = w; q < ncol; q += BT / 32) {
      const int col = j0 + q;
      const double sc = sl.colscale ? sl.colscale[col] : 1.0;
      double* out = sl.C + nd.col0 + (int64_t)col * sl.ldc;
      for (int row = lane; row < n; row += 32) {
        const double v = sc * (double)sb[row * BL + q];
        if (sl.mode) out[row] += v;
        else out[row] = v;
      }
    }
  } else {
    const Node& c1 = sc1;
    const Node& c2 = sc2;
    for (int q = w; q < ncol; q += BT / 32) {
      const int64_t co = (int64_t)(j0 + q) * ld;
      for (int row = lane; row < n; row += 32) {
        const float v = sb[row * BL + q];
        if (row < c1.nr) ws[c1.wx + c1.nk + row + co] = v;
        else ws[c2.wx + c2.nk + (row - c1.nr) + co] = v;
      }
    }
  }
}

constexpr size_t kBsolveSmemCap = 200 * 1024;

}  // namespace

bool bsolve_fits(int mmax, int nmax, int kmax, int kvmax) {
  return mmax <= 128 && nmax <= 128 && kmax <= 64 && kvmax <= 64 &&
         (size_t)layout(mmax, nmax, kmax, kvmax).total * sizeof(float) <= kBsolveSmemCap;
}

void launch_bsolve_up(const Task* t, int64_t nt, const Slot* s, int mmax, int nmax, int kmax, int kvmax, int r,
                      cudaStream_t st) {
  if (nt <= 0 || r <= 0) return;
  const Lay ly = layout(mmax, nmax, kmax, kvmax);
  const size_t smem = (size_t)ly.total * sizeof(float);
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(bsolve_up, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBsolveSmemCap);
    set = true;
  }
  const int nchunk = (r + CW - 1) / CW;
  bsolve_up<<<(unsigned)(nt * nchunk), BT, smem, st>>>(t, s, nchunk, ly);
}

void launch_bsolve_down(const Task* t, int64_t nt, const Slot* s, int mmax, int nmax, int kmax, int kvmax, int r,
                        cudaStream_t st) {
  if (nt <= 0 || r <= 0) return;
  const Lay ly = layout(mmax, nmax, kmax, kvmax);
  const size_t smem = (size_t)ly.total * sizeof(float);
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(bsolve_down, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBsolveSmemCap);
    set = true;
  }
  const int nchunk = (r + CW - 1) / CW;
  bsolve_down<<<(unsigned)(nt * nchunk), BT, smem, st>>>(t, s, nchunk, ly);
}

}  // namespace hss
