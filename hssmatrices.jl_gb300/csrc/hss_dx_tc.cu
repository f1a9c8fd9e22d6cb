// The leaf products Y_i = D_i X_i of the refinement residual (reference
// src/matmul.jl:46, the D*B of `_matmatdown!`) at FP64-level accuracy on the
// 5th-generation tensor cores (tcgen05, bf16 inputs, FP32 accumulation in
// tensor memory), written as double-float pairs for the persistent product.
//
// Splitting (the error-free splitting of Ozaki, Ogita, Oishi and Rump, 2012):
// every row r of D_i is written in 49-bit fixed point relative to its largest
// exponent, D(r, k) = F(r, k) 2^(E_r - 49), and F in 7 slices of 7 bits,
// F = sum_p a_p 2^(7 (6 - p)), |a_p| <= 127; every column c of X_i likewise
// with G_c and slices b_q.  The slices are exact in bf16, and a slice product
// summed over K <= 128 is an integer below 128 * 127^2 < 2^21, so that the
// seven products of one anti-diagonal d = p + q (at most 7 of them) add up
// exactly in FP32 (< 2^24).  Accumulator d of tensor memory holds
// S_d = sum_{p+q=d} A_p B_q; anti-diagonals d > 6 (weight 2^-49 and below) are
// dropped.  Then
//     D X (r, c) = 2^(E_r + G_c - 14) sum_{d=0..6} 2^(-7 d) S_d(r, c),
// summed from d = 6 down in double-float arithmetic (TwoSum) and scaled by the
// power of two: about 48 significant bits, as the rest of the residual.
//
// One block of 256 threads per (leaf, chunk of 32 right-hand sides), leaves
// up to 128 x 128.  K is processed in two halves of 64: for each half the
// threads write the 7 slices of D (128 x 64 bf16 each) and of X (32 x 64) to
// shared memory in the no-swizzle K-major layout of 8 x 8 core matrices, and
// one thread issues the 28 slice products (4 MMAs of K = 16 each, M = 128,
// N = 32) into the 7 accumulators; a commit to an mbarrier tells the block
// that the half's operands are consumed.  Four warps read the accumulators
// back (tcgen05.ld, one row per thread) and write the pairs.  Waits are
// bounded: a wait that runs out records DEV_TIMEOUT, waits (bounded) for the
// tensor core once more and frees tensor memory before returning.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int XT = 256;        // threads
constexpr int NS = 7;          // slices per operand
constexpr int XN = 32;         // right-hand sides per block (MMA N)
constexpr int XM = 128;        // rows per block (MMA M)
constexpr int XKH = 64;        // K per half
constexpr uint32_t kTmemCols = 256;                   // 7 accumulators x 32 columns
constexpr int A_SLICE = XM * XKH * 2;                 // bytes: 16 KB
constexpr int B_SLICE = XN * XKH * 2;                 // bytes: 4 KB
constexpr int SMEM_BYTES = NS * (A_SLICE + B_SLICE);  // 140 KB
constexpr uint32_t kWaitLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, byte offset between core
// matrices along K (leading) and along M/N (stride), descriptor version 1, no
// swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, N = 32, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(XN >> 3) << 17) | ((uint32_t)(XM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(kIdesc), "r"(accumulate));
}

// Bounded wait for the mbarrier phase `parity`; false when it ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    asm volatile(
        "{\n.reg .pred q;\nmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\nselp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity));
    if (done) return true;
  }
  return false;
}

// The seven 7-bit slices of a 49-bit fixed-point value, from the bits of x
// relative to the largest biased exponent emax of its row (column), as bf16
// (exact: |slice| <= 127), packed two per 32-bit word is left to the caller.
__device__ __forceinline__ void slices7(unsigned long long bits, int emax, float (&s)[NS]) {
  const int eb = (int)((bits >> 52) & 0x7FF);
  unsigned long long F = 0ull;
  if (eb != 0) {   // zeros and subnormals: 0 (far below 2^-49 of any normal row maximum)
    const int sh = emax - eb + 4;   // >= 4: F < 2^49
    const unsigned long long mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    F = sh < 64 ? (mant >> sh) : 0ull;
  }
  const bool neg = (bits >> 63) != 0;
#pragma unroll
  for (int p = 0; p < NS; ++p) {
    const int a = (int)((F >> (7 * (NS - 1 - p))) & 127ull);
    s[p] = (float)(neg ? -a : a);
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

__global__ void __launch_bounds__(XT, 1) dx_tc_kernel(const Task* __restrict__ leaves, int nchunk,
                                                      const Slot* __restrict__ slots) {
  extern __shared__ __align__(1024) unsigned char xsm[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int s_emax[2][XM];   // per row of D: largest biased exponent, per half of the columns
  __shared__ int s_gmax[XN];      // per column of X
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  const Task tk = leaves[blockIdx.x / nchunk];
  const int ch = blockIdx.x % nchunk;
  const Slot& sl = slots[tk.slot];
  const Node& nd = tk.nodes[tk.node];
  const int j0 = ch * XN;
  if (nd.root || j0 >= sl.r) return;   // uniform over the block
  const int m = nd.gm, n = nd.gn, nc = min(XN, sl.r - j0);
  const double* D = nd.D;                                            // m x n, ld m
  const double* X = sl.B + nd.col0 + (int64_t)j0 * sl.ldb;           // n x nc, ld ldb
  unsigned char* Abuf = xsm;                                         // NS slices of A
  unsigned char* Bbuf = xsm + NS * A_SLICE;                          // NS slices of B

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_fail = 0;
  }
  // largest exponent of every row of D (thread: row r, every other column) ...
  {
    const int r = tid & (XM - 1), h = tid >> 7;
    int emax = 0;
    if (r < m)
      for (int c = h; c < n; c += 2) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(__ldg(D + r + (int64_t)c * m));
        emax = max(emax, (int)((b >> 52) & 0x7FF));
      }
    s_emax[h][r] = emax;
  }
  // ... and of every column of X (8 threads per column)
  {
    const int c = tid >> 3, t8 = tid & 7;
    int g = 0;
    if (c < nc)
      for (int k = t8; k < n; k += 8) {
        const unsigned long long b =
            (unsigned long long)__double_as_longlong(__ldg(X + k + (int64_t)c * sl.ldb));
        g = max(g, (int)((b >> 52) & 0x7FF));
      }
    g = max(g, __shfl_xor_sync(0xffffffffu, g, 4));
    g = max(g, __shfl_xor_sync(0xffffffffu, g, 2));
    g = max(g, __shfl_xor_sync(0xffffffffu, g, 1));
    if (t8 == 0) s_gmax[c] = g;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;

  const int nhalf = n > XKH ? 2 : 1;
  bool ok = true;
  for (int h = 0; h < nhalf; ++h) {
    // A slices: thread (row r, core-matrix column groups kg = cg, cg + 2, ...):
    // eight consecutive columns per group, one 16-byte store per slice
    {
      const int r = tid & (XM - 1), cg = tid >> 7;
      const int emax = max(s_emax[0][r], s_emax[1][r]);
      for (int kg = cg; kg < XKH / 8; kg += 2) {
        float sv[8][NS];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int c = XKH * h + 8 * kg + e;
          unsigned long long b = 0ull;
          if (r < m && c < n) b = (unsigned long long)__double_as_longlong(__ldg(D + r + (int64_t)c * m));
          slices7(b, emax, sv[e]);
        }
        const int off = (r >> 3) * 1024 + kg * 128 + (r & 7) * 16;
#pragma unroll
        for (int p = 0; p < NS; ++p) {
          uint4 w;
          w.x = pack_bf16(sv[0][p], sv[1][p]);
          w.y = pack_bf16(sv[2][p], sv[3][p]);
          w.z = pack_bf16(sv[4][p], sv[5][p]);
          w.w = pack_bf16(sv[6][p], sv[7][p]);
          *reinterpret_cast<uint4*>(Abuf + p * A_SLICE + off) = w;
        }
      }
    }
    // B slices: thread (column c of X, core-matrix row group kg of K)
    {
      const int c = tid & (XN - 1), kg = tid >> 5;   // kg: 0..7
      const int gmax = s_gmax[c];
      float sv[8][NS];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int k = XKH * h + 8 * kg + e;
        unsigned long long b = 0ull;
        if (c < nc && k < n) b = (unsigned long long)__double_as_longlong(__ldg(X + k + (int64_t)c * sl.ldb));
        slices7(b, gmax, sv[e]);
      }
      const int off = (c >> 3) * 1024 + kg * 128 + (c & 7) * 16;
#pragma unroll
      for (int p = 0; p < NS; ++p) {
        uint4 w;
        w.x = pack_bf16(sv[0][p], sv[1][p]);
        w.y = pack_bf16(sv[2][p], sv[3][p]);
        w.z = pack_bf16(sv[4][p], sv[5][p]);
        w.w = pack_bf16(sv[6][p], sv[7][p]);
        *reinterpret_cast<uint4*>(Bbuf + p * B_SLICE + off) = w;
      }
    }
    // the generic-proxy stores become visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = smem_u32(Abuf), b0 = smem_u32(Bbuf);
      for (int d = 0; d < NS; ++d)
        for (int p = 0; p <= d; ++p) {
          const int q = d - p;
#pragma unroll
          for (int kk = 0; kk < XKH / 16; ++kk) {
            const uint64_t ad = sdesc(a0 + p * A_SLICE + kk * 256, 128, 1024);
            const uint64_t bd = sdesc(b0 + q * B_SLICE + kk * 256, 128, 1024);
            mma_bf16(tmem + (uint32_t)(XN * d), ad, bd, (h > 0 || p > 0 || kk > 0) ? 1u : 0u);
          }
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&s_bar)));
    }
    if (!mbar_wait(&s_bar, (uint32_t)h)) {
      s_fail = 1;
      ok = false;
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (s_fail) break;
  }
  ok = ok && !s_fail;

  // read the accumulators back: warp w (< 4) has rows 32 w .. 32 w + 31
  if (ok && warp < 4) {
    const int r = tid;
    float hi[XN], lo[XN];
    for (int d = NS - 1; d >= 0; --d) {
      uint32_t v[XN];
      const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(XN * d);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
          "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
            "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
            "=r"(v[30]), "=r"(v[31])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int c = 0; c < XN; ++c) {
        const float sd = __uint_as_float(v[c]);   // an exact integer
        if (d == NS - 1) {
          hi[c] = sd;
          lo[c] = 0.f;
        } else {   // (hi, lo) <- S_d + 2^-7 (hi, lo), exact scaling, TwoSum
          float s, e;
          two_sum(sd, __fmul_rn(hi[c], 0.0078125f), s, e);
          const float l = __fadd_rn(e, __fmul_rn(lo[c], 0.0078125f));
          hi[c] = __fadd_rn(s, l);
          lo[c] = __fsub_rn(l, __fsub_rn(hi[c], s));
        }
      }
    }
    if (r < m) {
      const int er = max(s_emax[0][r], s_emax[1][r]);
      float2* T = (float2*)sl.tmp + nd.row0 + r + (int64_t)j0 * sl.ldt2;
#pragma unroll
      for (int c = 0; c < XN; ++c) {
        if (c < nc) {
          // 2^(E_r + G_c - 14) with E = biased exponent - 1023 + 1
          const int ex = (er - 1022) + (s_gmax[c] - 1022) - 14;
          T[(int64_t)c * sl.ldt2] = make_float2(ldexpf(hi[c], ex), ldexpf(lo[c], ex));
        }
      }
    }
  }
  if (!ok && tid == 0) {
    if (sl.err) atomicCAS((int*)sl.err, DEV_OK, DEV_TIMEOUT);
    // the tensor core may still be working on this block's operands
    mbar_wait(&s_bar, (uint32_t)(nhalf - 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

bool dx_tc_fits(int mleaf, int nleaf) { return mleaf <= XM && nleaf <= 2 * XKH; }

cudaError_t launch_dx_tc(const Task* leaves, int64_t nleaves, const Slot* slots, int rmax, cudaStream_t st) {
  if (nleaves <= 0 || rmax <= 0) return cudaSuccess;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(dx_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int nchunk = (rmax + XN - 1) / XN;
  dx_tc_kernel<<<(unsigned)(nleaves * nchunk), XT, SMEM_BYTES, st>>>(leaves, nchunk, slots);
  return cudaGetLastError();
}

}  // namespace hss
