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
// The slices of D depend only on the generators: dx_prep_kernel writes them
// once per plan (with each row's exponent) to global memory, already in the
// shared-memory layout of the MMA operands (no-swizzle K-major 8 x 8 core
// matrices), by quarters of K = 32.  A residual call then runs one block of
// 256 threads per (leaf, chunk of 32 right-hand sides), leaves up to
// 128 x 128: per quarter of K, one thread starts bulk asynchronous copies
// (cp.async.bulk, the TMA engine) of the 7 slices of D into shared memory
// while the threads slice X (32 x 32) next to them, and one thread issues the
// 28 slice products (2 MMAs of K = 16 each, M = 128, N = 32) into the 7
// accumulators; mbarriers track the copies (transaction bytes) and the MMAs
// (commit).  A block holds 70 KB of operands, so two blocks share an SM and
// overlap each other's copies.  Four warps read the accumulators back
// (tcgen05.ld, one row per thread) and write the pairs.  Waits are bounded: a
// wait that runs out records DEV_TIMEOUT, waits (bounded) for the tensor core
// once more and frees tensor memory before returning.
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
constexpr int XKQ = 32;        // K per quarter
constexpr int NQ = 4;          // quarters (K <= 128)
constexpr uint32_t kTmemCols = 256;                   // 7 accumulators x 32 columns
constexpr int AQ = XM * XKQ * 2;                      // bytes of one slice of D per quarter: 8 KB
constexpr int BQ = XN * XKQ * 2;                      // of X: 2 KB
constexpr int OPER_BYTES = NS * (AQ + BQ);            // 70 KB
constexpr int SMEM_BYTES = 100 * 1024;                // requested: at most two blocks per SM (tensor memory)
constexpr uint32_t kWaitLimit = 1u << 24;
static_assert(OPER_BYTES <= SMEM_BYTES, "operands fit the requested shared memory");

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

// Largest biased exponent of row r of D over its n columns (0: the row is zero).
__device__ __forceinline__ int row_emax(const double* D, int m, int n, int r, int c0, int cstep) {
  int emax = 0;
  if (r < m) {
    int c = c0;
    for (; c + 7 * cstep < n; c += 8 * cstep) {   // eight loads in flight
      unsigned long long b[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) b[u] = (unsigned long long)__double_as_longlong(__ldg(D + r + (int64_t)(c + u * cstep) * m));
#pragma unroll
      for (int u = 0; u < 8; ++u) emax = max(emax, (int)((b[u] >> 52) & 0x7FF));
    }
    for (; c < n; c += cstep)
      emax = max(emax, (int)(((unsigned long long)__double_as_longlong(__ldg(D + r + (int64_t)c * m)) >> 52) & 0x7FF));
  }
  return emax;
}

// Eight consecutive K entries of one row (column) into the seven slices, one
// 16-byte store per slice at dst + p * stride.
template <class Ld>
__device__ __forceinline__ void slice_row8(unsigned char* dst, int stride, int emax, Ld ld) {
  float sv[8][NS];
#pragma unroll
  for (int e = 0; e < 8; ++e) slices7(ld(e), emax, sv[e]);
#pragma unroll
  for (int p = 0; p < NS; ++p) {
    uint4 w;
    w.x = pack_bf16(sv[0][p], sv[1][p]);
    w.y = pack_bf16(sv[2][p], sv[3][p]);
    w.z = pack_bf16(sv[4][p], sv[5][p]);
    w.w = pack_bf16(sv[6][p], sv[7][p]);
    *reinterpret_cast<uint4*>(dst + p * stride) = w;
  }
}

// Once per plan: the slices of every non-root leaf's D and its row exponents.
// Leaf region (at nd.fdx): quarter q, slice p at (q NS + p) AQ bytes, the
// 128 row exponents (int) after the nq quarters.
__global__ void __launch_bounds__(XT) dx_prep_kernel(const Task* __restrict__ leaves, unsigned char* __restrict__ base) {
  __shared__ int s_emax[2][XM];
  const Task tk = leaves[blockIdx.x];
  const Node& nd = tk.nodes[tk.node];
  if (nd.root || nd.fdx < 0) return;
  const int m = nd.gm, n = nd.gn, tid = threadIdx.x;
  const double* D = nd.D;
  unsigned char* reg = base + nd.fdx;
  const int nq = (n + XKQ - 1) / XKQ;
  {
    const int r = tid & (XM - 1), h = tid >> 7;
    s_emax[h][r] = row_emax(D, m, n, r, h, 2);
  }
  __syncthreads();
  const int r = tid & (XM - 1), kgh = tid >> 7;
  const int emax = max(s_emax[0][r], s_emax[1][r]);
  if (kgh == 0) reinterpret_cast<int*>(reg + (size_t)nq * NS * AQ)[r] = emax;
  for (int q = 0; q < nq; ++q)
    for (int kg = kgh; kg < XKQ / 8; kg += 2) {
      const int off = (r >> 3) * 512 + kg * 128 + (r & 7) * 16;
      slice_row8(reg + (size_t)q * NS * AQ + off, AQ, emax, [&](int e) {
        const int c = XKQ * q + 8 * kg + e;
        return (r < m && c < n) ? (unsigned long long)__double_as_longlong(__ldg(D + r + (int64_t)c * m)) : 0ull;
      });
    }
}

__global__ void __launch_bounds__(XT, 2) dx_tc_kernel(const Task* __restrict__ leaves, int nchunk,
                                                      const Slot* __restrict__ slots) {
  extern __shared__ __align__(1024) unsigned char xsm[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar[2];   // [0]: copies of D's slices, [1]: MMAs
  __shared__ int s_gmax[XN];                   // per column of X
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  const Task tk = leaves[blockIdx.x / nchunk];
  const int ch = blockIdx.x % nchunk;
  const Slot& sl = slots[tk.slot];
  const Node& nd = tk.nodes[tk.node];
  const int j0 = ch * XN;
  if (nd.root || nd.fdx < 0 || j0 >= sl.r) return;   // uniform over the block
  const int m = nd.gm, n = nd.gn, nc = min(XN, sl.r - j0), nq = (n + XKQ - 1) / XKQ;
  const double* X = sl.B + nd.col0 + (int64_t)j0 * sl.ldb;           // n x nc, ld ldb
  const unsigned char* reg = sl.dxs + nd.fdx;                        // prepared slices of D
  unsigned char* Abuf = xsm;                                         // NS slices of D, one quarter
  unsigned char* Bbuf = xsm + NS * AQ;                               // NS slices of X, one quarter

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_fail = 0;
  }
  // largest exponent of every column of X (8 threads per column)
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

  bool ok = true;
  int qfail = 0;
  for (int q = 0; q < nq; ++q) {
    qfail = q;
    // the quarter's slices of D: bulk copies, completion counted in bytes
    if (tid == 0) {
      const uint32_t bar = smem_u32(&s_bar[0]);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"((uint32_t)(NS * AQ)));
      for (int p = 0; p < NS; ++p)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(Abuf + p * AQ)),
                     "l"(reg + (size_t)(q * NS + p) * AQ), "r"((uint32_t)AQ), "r"(bar)
                     : "memory");
    }
    // the quarter's slices of X: thread (column c, core-matrix row group kg)
    if (tid < XN * (XKQ / 8)) {
      const int c = tid & (XN - 1), kg = tid >> 5;
      const int gmax = s_gmax[c];
      slice_row8(Bbuf + (c >> 3) * 512 + kg * 128 + (c & 7) * 16, BQ, gmax, [&](int e) {
        const int k = XKQ * q + 8 * kg + e;
        return (c < nc && k < n) ? (unsigned long long)__double_as_longlong(__ldg(X + k + (int64_t)c * sl.ldb))
                                 : 0ull;
      });
    }
    asm volatile("fence.proxy.async.shared::cta;");   // generic-proxy stores -> tensor core
    __syncthreads();
    if (!mbar_wait(&s_bar[0], (uint32_t)(q & 1))) s_fail = 1;
    __syncthreads();
    if (s_fail) {
      ok = false;
      break;
    }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = smem_u32(Abuf), b0 = smem_u32(Bbuf);
      for (int d = 0; d < NS; ++d)
        for (int p = 0; p <= d; ++p) {
          const int qq = d - p;
#pragma unroll
          for (int kk = 0; kk < XKQ / 16; ++kk) {
            const uint64_t ad = sdesc(a0 + p * AQ + kk * 256, 128, 512);
            const uint64_t bd = sdesc(b0 + qq * BQ + kk * 256, 128, 512);
            mma_bf16(tmem + (uint32_t)(XN * d), ad, bd, (q > 0 || p > 0 || kk > 0) ? 1u : 0u);
          }
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&s_bar[1])));
    }
    if (!mbar_wait(&s_bar[1], (uint32_t)(q & 1))) s_fail = 1;
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (s_fail) {
      ok = false;
      break;
    }
  }

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
      const int er = reinterpret_cast<const int*>(reg + (size_t)nq * NS * AQ)[r];
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
    // a copy or the tensor core may still be working on this block's buffers
    mbar_wait(&s_bar[0], (uint32_t)(qfail & 1));
    mbar_wait(&s_bar[1], (uint32_t)(qfail & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

bool dx_tc_fits(int mleaf, int nleaf) { return mleaf <= XM && nleaf <= NQ * XKQ; }

int64_t dx_leaf_bytes(int n) {
  return (int64_t)((n + XKQ - 1) / XKQ) * NS * AQ + XM * (int64_t)sizeof(int);
}

cudaError_t launch_dx_prep(const Task* leaves, int64_t nleaves, unsigned char* base, cudaStream_t st) {
  if (nleaves <= 0) return cudaSuccess;
  dx_prep_kernel<<<(unsigned)nleaves, XT, 0, st>>>(leaves, base);
  return cudaGetLastError();
}

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
