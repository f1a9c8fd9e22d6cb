// Entry extraction A[rows, cols] and full(A) on the device (reference
// src/hssmatrix.jl:102-153 getindex / _getidx, :270-305 full / _full!).
//
// The reference restricts the tree to the (sorted) requested rows and
// columns and expands the restricted tree with `full`.  Here the same
// expansion runs level by level over the restricted tree:
//
//   * basis pass (one launch per tree height, one block per node): the
//     expanded bases restricted to the node's requested rows / columns,
//     Ub = U[rows, :] at a leaf and Ub = [Ub1 R1; Ub2 R2] at a branch (Vb the
//     same with V, W1, W2), and at every branch the left factors of its two
//     off-diagonal blocks, T12 = Ub1 B12 and T21 = Ub2 B21;
//   * block pass (one launch): every off-diagonal block
//     out[rows(c1), cols(c2)] = T12 Vb2^T and out[rows(c2), cols(c1)] = T21 Vb1^T
//     in 64 x 64 tiles (a flat tile list over all branches), FP64;
//   * leaf pass (one launch): out[rows(l), cols(l)] = D[rows, cols].
//
// Rows and columns are sorted on the host; every output element is written
// through the inverse permutations, so any order and repeated indices are
// allowed, as in the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int GT = 256;   // threads
constexpr int TT = 64;    // output tile (rows and columns)
constexpr int KC = 16;    // K chunk of the tile product

// out(i, q) = sum_l A(i, l) B(l, q), A (m x K, ld lda), B (K x N, ld ldb),
// out ld ldo: the small products of the basis pass, one output per thread step.
__device__ void small_gemm(const double* A, int64_t lda, const double* B, int64_t ldb, double* out, int64_t ldo,
                           int64_t m, int K, int N) {
  for (int64_t e = threadIdx.x; e < m * N; e += GT) {
    const int64_t i = e % m;
    const int q = (int)(e / m);
    double s = 0.0;
    for (int l = 0; l < K; ++l) s = fma(A[i + l * lda], B[l + (int64_t)q * ldb], s);
    out[i + q * ldo] = s;
  }
}

__global__ void __launch_bounds__(GT) gi_basis_kernel(const Node* __restrict__ nodes, const GiRange* __restrict__ rg,
                                                      const int32_t* __restrict__ list, const int64_t* __restrict__ R,
                                                      const int64_t* __restrict__ C, double* ws) {
  const int xi = list[blockIdx.x];
  const Node& x = nodes[xi];
  const GiRange& g = rg[xi];
  if (x.leaf) {
    // Ub = U[rows - row0, :], Vb = V[cols - col0, :]
    for (int64_t e = threadIdx.x; e < g.rcnt * x.ku; e += GT) {
      const int64_t i = e % g.rcnt, q = e / g.rcnt;
      ws[g.ub + e] = x.U[(R[g.rlo + i] - x.row0) + q * x.gm];
    }
    for (int64_t e = threadIdx.x; e < g.ccnt * x.kv; e += GT) {
      const int64_t j = e % g.ccnt, q = e / g.ccnt;
      ws[g.vb + e] = x.V[(C[g.clo + j] - x.col0) + q * x.gn];
    }
    return;
  }
  const GiRange& g1 = rg[x.left];
  const GiRange& g2 = rg[x.right];
  const Node& c1 = nodes[x.left];
  const Node& c2 = nodes[x.right];
  // T12 = Ub1 B12 (rcnt1 x kv2), T21 = Ub2 B21 (rcnt2 x kv1)  (src/hssmatrix.jl:293-294)
  small_gemm(ws + g1.ub, g1.rcnt, x.B12, c1.ku, ws + g.t12, g1.rcnt, g1.rcnt, c1.ku, c2.kv);
  small_gemm(ws + g2.ub, g2.rcnt, x.B21, c2.ku, ws + g.t21, g2.rcnt, g2.rcnt, c2.ku, c1.kv);
  if (x.root) return;
  // Ub = [Ub1 R1; Ub2 R2], Vb = [Vb1 W1; Vb2 W2]  (:296-299)
  small_gemm(ws + g1.ub, g1.rcnt, x.R1, c1.ku, ws + g.ub, g.rcnt, g1.rcnt, c1.ku, x.ku);
  small_gemm(ws + g2.ub, g2.rcnt, x.R2, c2.ku, ws + g.ub + g1.rcnt, g.rcnt, g2.rcnt, c2.ku, x.ku);
  small_gemm(ws + g1.vb, g1.ccnt, x.W1, c1.kv, ws + g.vb, g.ccnt, g1.ccnt, c1.kv, x.kv);
  small_gemm(ws + g2.vb, g2.ccnt, x.W2, c2.kv, ws + g.vb + g1.ccnt, g.ccnt, g2.ccnt, c2.kv, x.kv);
}

// One 64 x 64 tile of an off-diagonal block: out(r, c) = sum_q T(r, q) Vb(c, q).
// Thread (ty, tx) computes rows ty*4.. and columns tx + 16*b: output writes
// along a tile column are consecutive rows.
__global__ void __launch_bounds__(GT) gi_block_kernel(const GiTile* __restrict__ tiles, const double* __restrict__ ws,
                                                      const int64_t* __restrict__ prow,
                                                      const int64_t* __restrict__ pcol, double* out, int64_t ldo) {
  __shared__ double Ts[KC][TT + 1];
  __shared__ double Vs[KC][TT + 1];
  const GiTile t = tiles[blockIdx.x];
  const int tid = threadIdx.x;
  const int tr = tid & 15, tc = tid >> 4;   // rows tr + 16 a, columns tc + 16 b
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int q0 = 0; q0 < t.k; q0 += KC) {
    for (int e = tid; e < KC * TT; e += GT) {
      const int i = e % TT, q = e / TT;
      const bool okq = q0 + q < t.k;
      Ts[q][i] = (okq && i < t.rows) ? ws[t.T + (t.r0 + i) + (int64_t)(q0 + q) * t.ldt] : 0.0;
      Vs[q][i] = (okq && i < t.cols) ? ws[t.V + (t.c0 + i) + (int64_t)(q0 + q) * t.ldv] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < KC; ++q) {
      double tv[4], vv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) tv[a] = Ts[q][tr + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) vv[b] = Vs[q][tc + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma(tv[a], vv[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int j = tc + 16 * b;
    if (j >= t.cols) continue;
    const int64_t oc = pcol[t.cs + t.c0 + j] * ldo;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int i = tr + 16 * a;
      if (i < t.rows) out[prow[t.rs + t.r0 + i] + oc] = acc[a][b];
    }
  }
}

// Diagonal leaf blocks: out[rows(l), cols(l)] = D[rows - row0, cols - col0].
__global__ void __launch_bounds__(GT) gi_leaf_kernel(const Node* __restrict__ nodes, const GiRange* __restrict__ rg,
                                                     const int32_t* __restrict__ leaves, const int64_t* __restrict__ R,
                                                     const int64_t* __restrict__ C, const int64_t* __restrict__ prow,
                                                     const int64_t* __restrict__ pcol, double* out, int64_t ldo) {
  const int xi = leaves[blockIdx.x];
  const Node& x = nodes[xi];
  const GiRange& g = rg[xi];
  for (int64_t e = threadIdx.x; e < g.rcnt * g.ccnt; e += GT) {
    const int64_t i = e % g.rcnt, j = e / g.rcnt;
    out[prow[g.rlo + i] + pcol[g.clo + j] * ldo] =
        x.D[(R[g.rlo + i] - x.row0) + (C[g.clo + j] - x.col0) * x.gm];
  }
}

}  // namespace

void launch_gi_basis(const Node* nodes, const GiRange* rg, const int32_t* list, int64_t count, const int64_t* R,
                     const int64_t* C, double* ws, cudaStream_t st) {
  for (int64_t b = 0; b < count; b += 65535) {
    const unsigned g = (unsigned)std::min<int64_t>(65535, count - b);
    gi_basis_kernel<<<g, GT, 0, st>>>(nodes, rg, list + b, R, C, ws);
  }
}

void launch_gi_blocks(const GiTile* tiles, int64_t count, const double* ws, const int64_t* prow, const int64_t* pcol,
                      double* out, int64_t ldo, cudaStream_t st) {
  for (int64_t b = 0; b < count; b += 1 << 30) {
    const unsigned g = (unsigned)std::min<int64_t>(1 << 30, count - b);
    gi_block_kernel<<<g, GT, 0, st>>>(tiles + b, ws, prow, pcol, out, ldo);
  }
}

void launch_gi_leaves(const Node* nodes, const GiRange* rg, const int32_t* leaves, int64_t count, const int64_t* R,
                      const int64_t* C, const int64_t* prow, const int64_t* pcol, double* out, int64_t ldo,
                      cudaStream_t st) {
  for (int64_t b = 0; b < count; b += 65535) {
    const unsigned g = (unsigned)std::min<int64_t>(65535, count - b);
    gi_leaf_kernel<<<g, GT, 0, st>>>(nodes, rg, leaves + b, R, C, prow, pcol, out, ldo);
  }
}

int gi_tile_rows() { return TT; }

}  // namespace hss
