// HSS x dense product in double-float arithmetic (the refinement residual).
//
// GB300 runs FP64 at ~1/64 of its FP32 rate, so the FP64 residual r = b - A x
// of the mixed-precision solve is formed on the FP32 pipe instead: every
// generator entry and every right-hand-side entry is an unevaluated pair
// (hi, lo) of floats (hi = fl32(x), lo = fl32(x - hi), 48 significant bits),
// products use the exact FMA product error and sums use TwoSum, giving
// ~1e-14 relative accuracy -- enough for a 1e-10 residual target.
//
// Same sweeps as the FP64 product (src/matmul.jl:32-62):
//   split   X (FP64) -> Xs (float2)
//   leaf    P = D X (kept as pairs), Z = V^T X
//   up      Z = W1^T Z1 + W2^T Z2
//   down    F1 = B12 Z2 + R1 F,  F2 = B21 Z1 + R2 F
//   final   C = alpha (P + U F) + beta Y  (rounded to FP64 once), column norms
#include <cuda_runtime.h>
#include <cstdint>
#include "hss_df.cuh"
#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int DT = 256;
constexpr int DRC = 8;    // right-hand sides per thread block

__device__ __forceinline__ const float2* dfp(const Slot& sl, const double* p) {
  return sl.gdf + (p - sl.gbase);
}

__global__ void df_split_kernel(const double* __restrict__ src, float2* __restrict__ dst, int64_t cnt) {
  for (int64_t e = blockIdx.x * (int64_t)DT + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * DT)
    dst[e] = split_d(src[e]);
}

// Xs (ld n) = split(X (ld ldx)) for an n x r block.
__global__ void df_split_cols_kernel(const double* __restrict__ X, int64_t ldx, int64_t n, int64_t r,
                                     float2* __restrict__ Xs) {
  const int64_t tot = n * r;
  for (int64_t e = blockIdx.x * (int64_t)DT + threadIdx.x; e < tot; e += (int64_t)gridDim.x * DT) {
    const int64_t i = e % n, j = e / n;
    Xs[e] = split_bits(X[i + j * ldx]);
  }
}

// Leaves: P = D X (to the pair buffer), Z = V^T X (pairs).  Thread block per
// (leaf, chunk of DRC columns); thread t owns row t % 128 (+128 steps) and
// columns (t / 128) * 4 .. +3 of the chunk.
__global__ void __launch_bounds__(DT) dfmv_leaf_kernel(const Task* __restrict__ tasks,
                                                       const Slot* __restrict__ slots, int nchunk) {
  __shared__ float2 Xsh[256 * DRC];
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * DRC;
  const Node& nd = tk.nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  if (j0 >= sl.r) return;
  const int m = nd.gm, n = nd.gn, kv = nd.kv, nc = min(DRC, sl.r - j0);
  const float2* X = sl.xs + nd.col0 + (int64_t)j0 * sl.ldx2;
  const float2* D = dfp(sl, nd.D);
  const int tid = threadIdx.x;
  float2* P = sl.tmp + nd.row0 + (int64_t)j0 * sl.ldt2;
  for (int l0 = 0; l0 < n; l0 += 256) {
    const int nl = min(256, n - l0);
    __syncthreads();
    for (int e = tid; e < nl * DRC; e += DT) {
      const int l = e % nl, q = e / nl;
      Xsh[l * DRC + q] = q < nc ? X[l0 + l + (int64_t)q * sl.ldx2] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    // D X: rows in steps of 128, each thread 4 columns
    for (int i = tid & 127; i < m; i += 128) {
      const int q0 = (tid >> 7) * 4;
      float h[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
      if (l0 > 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (q0 + q < nc) { h[q] = P[i + (int64_t)(q0 + q) * sl.ldt2].x; lo[q] = P[i + (int64_t)(q0 + q) * sl.ldt2].y; }
      }
      const float2* a = D + i + (int64_t)l0 * m;
#pragma unroll 4
      for (int l = 0; l < nl; ++l) {
        const float2 d = a[(int64_t)l * m];
#pragma unroll
        for (int q = 0; q < 4; ++q) df_fma(h[q], lo[q], d, Xsh[l * DRC + q0 + q]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q0 + q < nc) P[i + (int64_t)(q0 + q) * sl.ldt2] = df_norm(h[q], lo[q]);
    }
    // Z = V^T X: one warp per (column c of V, rhs q)
    if (kv > 0) {
      const float2* V = dfp(sl, nd.V);
      float2* Z = sl.ws2 + nd.wz + (int64_t)j0 * sl.ldws;
      const int lane = tid & 31, warp = tid >> 5;
      for (int o = warp; o < kv * nc; o += DT / 32) {
        const int c = o % kv, q = o / kv;
        float h = 0.f, lo = 0.f;
        for (int l = lane; l < nl; l += 32) df_fma(h, lo, V[l0 + l + (int64_t)c * n], Xsh[l * DRC + q]);
        // reduce pairs over the warp
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const float oh = __shfl_xor_sync(0xffffffffu, h, off);
          const float ol = __shfl_xor_sync(0xffffffffu, lo, off);
          df_add(h, lo, oh, ol);
        }
        if (lane == 0) {
          if (l0 > 0) { const float2 z = Z[c + (int64_t)q * sl.ldws]; df_add(h, lo, z.x, z.y); }
          Z[c + (int64_t)q * sl.ldws] = df_norm(h, lo);
        }
      }
    }
  }
}

// Upsweep (non-root branch): Z = W1^T Z1 + W2^T Z2, pairs.
__global__ void __launch_bounds__(DT) dfmv_up_kernel(const Task* __restrict__ tasks,
                                                     const Slot* __restrict__ slots, int nchunk) {
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * DRC;
  const Node& nd = tk.nodes[tk.node];
  const Node& c1 = tk.nodes[nd.left];
  const Node& c2 = tk.nodes[nd.right];
  const Slot& sl = slots[tk.slot];
  if (j0 >= sl.r) return;
  const int nc = min(DRC, sl.r - j0), kv = nd.kv;
  const int64_t ld = sl.ldws;
  const float2* W1 = dfp(sl, nd.W1);
  const float2* W2 = dfp(sl, nd.W2);
  for (int o = threadIdx.x; o < kv * nc; o += DT) {
    const int c = o % kv, q = o / kv;
    const float2* z1 = sl.ws2 + c1.wz + (int64_t)(j0 + q) * ld;
    const float2* z2 = sl.ws2 + c2.wz + (int64_t)(j0 + q) * ld;
    float h = 0.f, lo = 0.f;
    for (int l = 0; l < c1.kv; ++l) df_fma(h, lo, W1[l + (int64_t)c * c1.kv], z1[l]);
    for (int l = 0; l < c2.kv; ++l) df_fma(h, lo, W2[l + (int64_t)c * c2.kv], z2[l]);
    sl.ws2[nd.wz + c + (int64_t)(j0 + q) * ld] = df_norm(h, lo);
  }
}

// Downsweep (branch): F1 = B12 Z2 + R1 F, F2 = B21 Z1 + R2 F, pairs.
__global__ void __launch_bounds__(DT) dfmv_down_kernel(const Task* __restrict__ tasks,
                                                       const Slot* __restrict__ slots, int nchunk) {
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * DRC;
  const Node& nd = tk.nodes[tk.node];
  const Node& c1 = tk.nodes[nd.left];
  const Node& c2 = tk.nodes[nd.right];
  const Slot& sl = slots[tk.slot];
  if (j0 >= sl.r) return;
  const int nc = min(DRC, sl.r - j0), ku = nd.root ? 0 : nd.ku;
  const int64_t ld = sl.ldws;
  const float2* B12 = dfp(sl, nd.B12);
  const float2* B21 = dfp(sl, nd.B21);
  const float2* R1 = ku ? dfp(sl, nd.R1) : nullptr;
  const float2* R2 = ku ? dfp(sl, nd.R2) : nullptr;
  const int n1 = c1.ku * nc;
  for (int o = threadIdx.x; o < (c1.ku + c2.ku) * nc; o += DT) {
    float h = 0.f, lo = 0.f;
    if (o < n1) {
      const int i = o % c1.ku, q = o / c1.ku;
      const float2* z2 = sl.ws2 + c2.wz + (int64_t)(j0 + q) * ld;
      const float2* f = sl.ws2 + nd.wf + (int64_t)(j0 + q) * ld;
      for (int l = 0; l < c2.kv; ++l) df_fma(h, lo, B12[i + (int64_t)l * c1.ku], z2[l]);
      for (int l = 0; l < ku; ++l) df_fma(h, lo, R1[i + (int64_t)l * c1.ku], f[l]);
      sl.ws2[c1.wf + i + (int64_t)(j0 + q) * ld] = df_norm(h, lo);
    } else {
      const int o2 = o - n1;
      const int i = o2 % c2.ku, q = o2 / c2.ku;
      const float2* z1 = sl.ws2 + c1.wz + (int64_t)(j0 + q) * ld;
      const float2* f = sl.ws2 + nd.wf + (int64_t)(j0 + q) * ld;
      for (int l = 0; l < c1.kv; ++l) df_fma(h, lo, B21[i + (int64_t)l * c2.ku], z1[l]);
      for (int l = 0; l < ku; ++l) df_fma(h, lo, R2[i + (int64_t)l * c2.ku], f[l]);
      sl.ws2[c2.wf + i + (int64_t)(j0 + q) * ld] = df_norm(h, lo);
    }
  }
}

// Leaves: C = alpha (P + U F) + beta Y in FP64, with per-column sums of squares.
__global__ void __launch_bounds__(DT) dfmv_final_kernel(const Task* __restrict__ tasks,
                                                        const Slot* __restrict__ slots, int nchunk) {
  __shared__ float2 Fsh[64 * DRC];
  __shared__ double red[DT / 32][DRC];
  const Task tk = tasks[blockIdx.x / nchunk];
  const int j0 = (blockIdx.x % nchunk) * DRC;
  const Node& nd = tk.nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  if (j0 >= sl.r) return;
  const int m = nd.gm, ku = nd.root ? 0 : nd.ku, nc = min(DRC, sl.r - j0);
  const int tid = threadIdx.x;
  const float2* U = ku ? dfp(sl, nd.U) : nullptr;
  const float2* F = sl.ws2 + nd.wf + (int64_t)j0 * sl.ldws;
  const bool fsh = ku <= 64;
  if (fsh)
    for (int e = tid; e < ku * DRC; e += DT) {
      const int l = e % ku, q = e / ku;
      Fsh[l * DRC + q] = q < nc ? F[l + (int64_t)q * sl.ldws] : make_float2(0.f, 0.f);
    }
  __syncthreads();
  double sq[DRC];
#pragma unroll
  for (int q = 0; q < DRC; ++q) sq[q] = 0.0;
  const float2* P = sl.tmp + nd.row0 + (int64_t)j0 * sl.ldt2;
  for (int i = tid; i < m; i += DT) {
    float h[DRC], lo[DRC];
#pragma unroll
    for (int q = 0; q < DRC; ++q) {
      const float2 p = q < nc ? P[i + (int64_t)q * sl.ldt2] : make_float2(0.f, 0.f);
      h[q] = p.x;
      lo[q] = p.y;
    }
    for (int l = 0; l < ku; ++l) {
      const float2 u = U[i + (int64_t)l * m];
#pragma unroll
      for (int q = 0; q < DRC; ++q)
        df_fma(h[q], lo[q], u, fsh ? Fsh[l * DRC + q] : (q < nc ? F[l + (int64_t)q * sl.ldws] : make_float2(0.f, 0.f)));
    }
#pragma unroll
    for (int q = 0; q < DRC; ++q) {
      if (q >= nc) continue;
      const int64_t j = j0 + q;
      double v = sl.alpha * ((double)h[q] + (double)lo[q]);
      if (sl.beta != 0.0 && sl.Y != nullptr) v += sl.beta * sl.Y[nd.row0 + i + j * sl.ldy];
      sl.C[nd.row0 + i + j * sl.ldc] = v;
      sq[q] = fma(v, v, sq[q]);
    }
  }
  if (sl.colnorm2 != nullptr) {
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int q = 0; q < DRC; ++q) {
      double v = sq[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (tid < nc) {
      double v = 0.0;
      for (int w = 0; w < DT / 32; ++w) v += red[w][tid];
      atomicAdd(sl.colnorm2 + j0 + tid, v);
    }
  }
}

}  // namespace

void launch_df_split(const double* src, float2* dst, int64_t cnt, cudaStream_t st) {
  if (cnt <= 0) return;
  int64_t blocks = (cnt + DT - 1) / DT;
  if (blocks > 152 * 16) blocks = 152 * 16;
  df_split_kernel<<<(unsigned)blocks, DT, 0, st>>>(src, dst, cnt);
}

void launch_df_split_cols(const double* X, int64_t ldx, int64_t n, int64_t r, float2* Xs, cudaStream_t st) {
  if (n <= 0 || r <= 0) return;
  int64_t blocks = (n * r + DT - 1) / DT;
  if (blocks > 152 * 16) blocks = 152 * 16;
  df_split_cols_kernel<<<(unsigned)blocks, DT, 0, st>>>(X, ldx, n, r, Xs);
}

static int nchunks(int rmax) { return (rmax + DRC - 1) / DRC; }

void launch_dfmv_leaf(const Task* t, int64_t nt, const Slot* s, int rmax, cudaStream_t st) {
  if (nt > 0 && rmax > 0) dfmv_leaf_kernel<<<(unsigned)(nt * nchunks(rmax)), DT, 0, st>>>(t, s, nchunks(rmax));
}
void launch_dfmv_up(const Task* t, int64_t nt, const Slot* s, int rmax, cudaStream_t st) {
  if (nt > 0 && rmax > 0) dfmv_up_kernel<<<(unsigned)(nt * nchunks(rmax)), DT, 0, st>>>(t, s, nchunks(rmax));
}
void launch_dfmv_down(const Task* t, int64_t nt, const Slot* s, int rmax, cudaStream_t st) {
  if (nt > 0 && rmax > 0) dfmv_down_kernel<<<(unsigned)(nt * nchunks(rmax)), DT, 0, st>>>(t, s, nchunks(rmax));
}
void launch_dfmv_final(const Task* t, int64_t nt, const Slot* s, int rmax, cudaStream_t st) {
  if (nt > 0 && rmax > 0) dfmv_final_kernel<<<(unsigned)(nt * nchunks(rmax)), DT, 0, st>>>(t, s, nchunks(rmax));
}

}  // namespace hss
