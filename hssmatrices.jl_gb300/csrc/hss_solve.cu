// ULV solve kernels with the right-hand sides held in registers.
//
// One thread block per tree node; a group of TPC consecutive lanes owns one
// right-hand-side column, lane gl holding rows gl, gl+TPC, gl+2*TPC, ... (up
// to MR rows).  Reflector applications are group dot products (shuffle
// reductions inside the group) followed by register updates; the triangular
// solves broadcast each solved entry from its owner lane.  No block-wide
// barrier sits inside the sequential sweeps.
//
// Upward pass per node (reference src/ulvfactor.jl:22-57, :74, :89):
//   b = rhs rows (leaf) or [b1; b2] - [T12 u2; T21 u1] (branch)
//   b <- Q_ql^T b;  zloc = L1 \ b[0:mk];  b_red = b[mk:m] - L2 zloc;
//   u = V[0:mk,:]^T zloc (+ W1^T u1 + W2^T u2);  x[0:mk] = zloc;
//   root: x = LU \ b (src/ulvfactor.jl:83).
// Downward pass per node (src/ulvfactor.jl:98-107): x <- Q_lq^T x, then the
// un-eliminated tail goes to the children (or the output at a leaf).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int ST = 256;
constexpr int LDS = 257;   // odd leading dimension of the shared staging block

// Asynchronous element copy global -> shared (cp.async, 4 or 8 bytes): the
// staging copies of a block are all in flight at once; cpa_wait() waits for
// this thread's copies, a barrier then publishes everyone's.  The sources
// (factor blocks, the previous level's workspace) do not change during the
// launch.
template <typename T>
__device__ __forceinline__ void cpa(T* s, const T* g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  if constexpr (sizeof(T) == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(g) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int TPC, typename T>
__device__ __forceinline__ T gsum(T v) {
#pragma unroll
  for (int o = TPC / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, TPC);
  return v;
}

// Forward substitution L x = b in registers (L lower, ld ldl, size nr).
template <typename T, int TPC, int RPT, bool UNIT>
__device__ __forceinline__ void lower_solve(T (&b)[RPT], const T* __restrict__ L, int ldl, int nr, int gl) {
#pragma unroll
  for (int s = 0; s < RPT; ++s) {
    if (s * TPC >= nr) break;
    for (int o = 0; o < TPC; ++o) {
      const int c = s * TPC + o;
      if (c >= nr) break;
      const T bc = __shfl_sync(0xffffffffu, b[s], o, TPC);
      const T xc = UNIT ? bc : bc / L[c + (int64_t)c * ldl];
      if (gl == o) b[s] = xc;
#pragma unroll
      for (int s2 = s; s2 < RPT; ++s2) {
        const int row = gl + s2 * TPC;
        if (row > c && row < nr) b[s2] -= L[row + (int64_t)c * ldl] * xc;
      }
    }
  }
}

// Backward substitution U x = b (U upper, non-unit).
template <typename T, int TPC, int RPT>
__device__ __forceinline__ void upper_solve(T (&b)[RPT], const T* __restrict__ A, int lda, int nr, int gl) {
#pragma unroll
  for (int s = RPT - 1; s >= 0; --s) {
    if (s * TPC >= nr) continue;
    for (int o = TPC - 1; o >= 0; --o) {
      const int c = s * TPC + o;
      if (c >= nr) continue;
      const T bc = __shfl_sync(0xffffffffu, b[s], o, TPC);
      const T xc = bc / A[c + (int64_t)c * lda];
      if (gl == o) b[s] = xc;
#pragma unroll
      for (int s2 = 0; s2 <= s; ++s2) {
        const int row = gl + s2 * TPC;
        if (row < c) b[s2] -= A[row + (int64_t)c * lda] * xc;
      }
    }
  }
}

// Elements of shared memory the upward kernel stages for one node (beyond the
// LDS x CPB right-hand-side block); the host sizes launches with the level's
// largest value.
__host__ __device__ inline int64_t solve_up_stage_elems(int m, int k, int mk, int nk, int kv, bool leaf, bool root,
                                                       int mr1, int mr2, int kv1, int kv2, int cpb) {
  int64_t e = 0;
  if (root) e += (int64_t)m * m;
  else if (mk > 0) e += (int64_t)m * k + (int64_t)mk * mk + (int64_t)k * nk + (int64_t)nk * kv;
  if (!leaf) {
    e += (int64_t)mr1 * kv2 + (int64_t)mr2 * kv1 + (int64_t)(kv1 + kv2) * cpb;
    if (!root) e += (int64_t)(kv1 + kv2) * kv;
  }
  return e;
}

template <typename T, int TPC, int MR>
__global__ void __launch_bounds__(ST) ulv_solve_up_reg(const Task* __restrict__ tasks,
                                                       const Slot* __restrict__ slots, int64_t stage_cap,
                                                       int nchunk) {
  constexpr int RPT = MR / TPC;
  constexpr int CPB = ST / TPC;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sb = (T*)smraw;          // LDS x CPB right-hand sides
  T* sx = sb + LDS * CPB;     // staged operands
  const Task tk = tasks[blockIdx.x / nchunk];
  const int jchunk = (blockIdx.x % nchunk) * CPB;   // this block's columns: jchunk .. jchunk+CPB-1
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* ws = (T*)sl.ws;
  const int64_t ld = sl.ldws;
  const T* fb = (const T*)sl.fbase;
  const int m = nd.m, n = nd.n, kv = nd.kv, r = sl.r;
  if (jchunk >= r) return;
  const int tid = threadIdx.x, g = tid / TPC, gl = tid % TPC;
  const int k = nd.k, mk = nd.mk, nk = nd.nk;
  T* u = ws + nd.wu;
  const Node* c1 = nd.leaf ? nullptr : &nodes[nd.left];
  const Node* c2 = nd.leaf ? nullptr : &nodes[nd.right];
  const int mr1 = c1 ? c1->mr : 0, mr2 = c2 ? c2->mr : 0, kv1 = c1 ? c1->kv : 0, kv2 = c2 ? c2->kv : 0;
  const bool staged = solve_up_stage_elems(m, k, mk, nk, kv, nd.leaf, nd.root, mr1, mr2, kv1, kv2, CPB) <= stage_cap;

  // Every factor / generator block an inner loop reads is copied on chip once
  // (bulk, coalesced), unless the level's blocks do not fit: then they are
  // read from global memory in place.  Leading dimensions follow the copy.
  const T* Up = fb + nd.fU;  int ldU = m;       // QL reflectors m x k
  const T* Lp = fb + nd.fD;  int ldL = m;       // L1 (mk x mk) or the root LU (m x m)
  const T* L2p = fb + nd.fD + mk;  int ldL2 = m;      // L2[:, 0:nk], k x nk
  const T* Vap = fb + nd.fV; int ldVa = n;      // V[0:nk, :], nk x kv
  const T* T12p = nd.leaf ? nullptr : fb + nd.fT12;   // mr1 x kv2
  const T* T21p = nd.leaf ? nullptr : fb + nd.fT21;   // mr2 x kv1
  T* sW1 = nullptr;  T* sW2 = nullptr;  T* su1 = nullptr;  T* su2 = nullptr;
  if (staged) {
    T* p = sx;
    if (nd.root) {
      for (int e = tid; e < m * m; e += ST) cpa(p + e, Lp + e);
      Lp = p; ldL = m; p += m * m;
    } else if (mk > 0) {
      T* q = p;
      for (int e = tid; e < m * k; e += ST) cpa(q + e, Up + e);
      Up = q; ldU = m; q += m * k;
      for (int e = tid; e < mk * mk; e += ST) cpa(q + e, Lp + (e % mk) + (int64_t)(e / mk) * m);
      Lp = q; ldL = mk; q += mk * mk;
      for (int e = tid; e < k * nk; e += ST) cpa(q + e, L2p + (e % k) + (int64_t)(e / k) * m);
      L2p = q; ldL2 = k; q += k * nk;
      // V[0:nk, :] transposed (element (l, c) at c + l*kv): consecutive threads read consecutive c
      for (int e = tid; e < nk * kv; e += ST) cpa(q + (e / nk) + (e % nk) * kv, Vap + (e % nk) + (int64_t)(e / nk) * n);
      Vap = q; ldVa = -1; q += nk * kv;
      p = q;
    }
    if (!nd.leaf) {
      for (int e = tid; e < mr1 * kv2; e += ST) cpa(p + e, T12p + e);
      T12p = p; p += mr1 * kv2;
      for (int e = tid; e < mr2 * kv1; e += ST) cpa(p + e, T21p + e);
      T21p = p; p += mr2 * kv1;
      if (!nd.root) {
        sW1 = p; p += kv1 * kv;
        sW2 = p; p += kv2 * kv;
        // W1, W2 transposed (element (l, c) at c + l*kv)
        // (converted from the FP64 generators: register loads, four in flight per thread)
        auto stage_w = [&](T* dst, const double* src, int kc) {
          for (int e0 = tid; e0 < kc * kv; e0 += 4 * ST) {
            double w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = e0 + q * ST < kc * kv ? __ldg(src + e0 + q * ST) : 0.0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int e = e0 + q * ST;
              if (e < kc * kv) dst[(e / kc) + (e % kc) * kv] = (T)w[q];
            }
          }
        };
        stage_w(sW1, nd.W1, kv1);
        stage_w(sW2, nd.W2, kv2);
      }
      su1 = p; p += kv1 * CPB;
      su2 = p; p += kv2 * CPB;
    }
  }
  for (int j0 = jchunk; j0 < jchunk + CPB && j0 < r; j0 += CPB) {
    const int ncol = min(CPB, r - j0);
    // ---- gather b for this chunk of columns into shared memory
    if (nd.leaf) {
      for (int e = tid; e < m * CPB; e += ST) {
        const int row = e % m, gg = e / m, j = j0 + gg;
        T val = T(0);
        if (j < r) {
          const double bv = sl.B[nd.row0 + row + (int64_t)j * sl.ldb];
          val = sl.colinv ? (T)(bv * sl.colinv[j]) : (T)bv;
        }
        sb[row + gg * LDS] = val;
      }
    } else {
      // children's u for this chunk (kv1 x ncol, kv2 x ncol), then
      // b = [b1; b2] - [T12 u2; T21 u1] (src/ulvfactor.jl:74)
      const T* u1g = ws + c1->wu + (int64_t)j0 * ld;
      const T* u2g = ws + c2->wu + (int64_t)j0 * ld;
      const T* u1p = u1g;  int64_t ldu1 = ld;
      const T* u2p = u2g;  int64_t ldu2 = ld;
      if (staged) {
        for (int e = tid; e < kv1 * ncol; e += ST) cpa(su1 + e, u1g + (e % kv1) + (int64_t)(e / kv1) * ld);
        for (int e = tid; e < kv2 * ncol; e += ST) cpa(su2 + e, u2g + (e % kv2) + (int64_t)(e / kv2) * ld);
        u1p = su1; ldu1 = kv1;
        u2p = su2; ldu2 = kv2;
        cpa_wait();
        __syncthreads();
      }
      for (int e = tid; e < m * CPB; e += ST) {
        const int row = e % m, gg = e / m;
        T val = T(0);
        if (gg < ncol) {
          const int64_t j = j0 + gg;
          T acc0 = T(0), acc1 = T(0);
          if (row < mr1) {
            val = ws[c1->wb + c1->mk + row + j * ld];
            const T* uu = u2p + (int64_t)gg * ldu2;
            int l = 0;
            for (; l + 1 < kv2; l += 2) {
              acc0 += T12p[row + l * mr1] * uu[l];
              acc1 += T12p[row + (l + 1) * mr1] * uu[l + 1];
            }
            if (l < kv2) acc0 += T12p[row + l * mr1] * uu[l];
          } else {
            const int i2 = row - mr1;
            val = ws[c2->wb + c2->mk + i2 + j * ld];
            const T* uu = u1p + (int64_t)gg * ldu1;
            int l = 0;
            for (; l + 1 < kv1; l += 2) {
              acc0 += T21p[i2 + l * mr2] * uu[l];
              acc1 += T21p[i2 + (l + 1) * mr2] * uu[l + 1];
            }
            if (l < kv1) acc0 += T21p[i2 + l * mr2] * uu[l];
          }
          val -= acc0 + acc1;
        }
        sb[row + gg * LDS] = val;
      }
      if (!nd.root) {
        // u accumulates W1^T u1 + W2^T u2 (src/ulvfactor.jl:89)
        for (int e = tid; e < kv * ncol; e += ST) {
          const int c = e % kv, gg = e / kv;
          const T* a1 = u1p + (int64_t)gg * ldu1;
          const T* a2 = u2p + (int64_t)gg * ldu2;
          T s = T(0);
          if (staged) {
            T s1 = T(0);
            for (int l = 0; l < kv1; ++l) s += sW1[c + l * kv] * a1[l];
            for (int l = 0; l < kv2; ++l) s1 += sW2[c + l * kv] * a2[l];
            s += s1;
          } else {
            for (int l = 0; l < kv1; ++l) s += (T)nd.W1[l + (int64_t)c * kv1] * a1[l];
            for (int l = 0; l < kv2; ++l) s += (T)nd.W2[l + (int64_t)c * kv2] * a2[l];
          }
          u[c + (int64_t)(j0 + gg) * ld] = s;
        }
      }
    }
    cpa_wait();   // leaves: the staged factor blocks
    __syncthreads();
    const int j = j0 + g;
    if (nd.root) {
      const T* A = Lp;
      const int32_t* piv = (const int32_t*)(fb + nd.fpiv);
      if (gl == 0) {
        T* col = sb + g * LDS;
        for (int c = 0; c < m; ++c) {
          const int p = piv[c];
          if (p != c) { const T t = col[c]; col[c] = col[p]; col[p] = t; }
        }
      }
      __syncwarp();
      T b[RPT];
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int row = gl + s * TPC;
        b[s] = row < m ? sb[row + g * LDS] : T(0);
      }
      lower_solve<T, TPC, RPT, true>(b, A, ldL, m, gl);
      upper_solve<T, TPC, RPT>(b, A, ldL, m, gl);
      if (j < r) {
        T* x = ws + nd.wx + (int64_t)j * ld;
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
          const int row = gl + s * TPC;
          if (row < m) x[row] = b[s];
        }
      }
      __syncthreads();
      continue;
    }
    if (mk > 0) {
      const T* tq = fb + nd.ftq;
      T b[RPT];
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int row = gl + s * TPC;
        b[s] = row < m ? sb[row + g * LDS] : T(0);
      }
      // b <- Q_ql^T b (src/ulvfactor.jl:42), reflectors in generation order
      for (int c = k - 1; c >= 0; --c) {
        const T tau = tq[c];
        if (tau == T(0)) continue;
        const int p = mk + c;
        const T* v = Up + (int64_t)c * ldU;
        T d0 = T(0), d1 = T(0);
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
          const int row = gl + s * TPC;
          const T vr = row < p ? v[row] : (row == p ? T(1) : T(0));
          if (s & 1) d1 += vr * b[s];
          else d0 += vr * b[s];
        }
        const T dot = gsum<TPC>(d0 + d1) * tau;
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
          const int row = gl + s * TPC;
          const T vr = row < p ? v[row] : (row == p ? T(1) : T(0));
          b[s] -= dot * vr;
        }
      }
      // zloc = L1 \ b[0:mk] (trsm, src/ulvfactor.jl:48)
      lower_solve<T, TPC, RPT, false>(b, Lp, ldL, mk, gl);
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int row = gl + s * TPC;
        if (row < m) sb[row + g * LDS] = b[s];
      }
    }
    __syncthreads();
    // ---- outputs: b_red (:49), u (:51, :89), x[0:mk] = zloc (:65)
    for (int e = tid; e < (m - mk) * ncol; e += ST) {
      const int i = e % (m - mk), gg = e / (m - mk);
      const T* bb = sb + gg * LDS;
      T s0 = bb[mk + i], s1 = T(0);
      int l = 0;
      for (; l + 1 < nk; l += 2) {
        s0 -= L2p[i + l * ldL2] * bb[l];
        s1 -= L2p[i + (l + 1) * ldL2] * bb[l + 1];
      }
      if (l < nk) s0 -= L2p[i + l * ldL2] * bb[l];
      ws[nd.wb + mk + i + (int64_t)(j0 + gg) * ld] = s0 + s1;
    }
    for (int e = tid; e < kv * ncol; e += ST) {
      const int c = e % kv, gg = e / kv;
      const T* bb = sb + gg * LDS;
      T s0 = nd.leaf ? T(0) : u[c + (int64_t)(j0 + gg) * ld], s1 = T(0);
      if (ldVa < 0) {   // staged transposed
        int l = 0;
        for (; l + 1 < nk; l += 2) {
          s0 += Vap[c + l * kv] * bb[l];
          s1 += Vap[c + (l + 1) * kv] * bb[l + 1];
        }
        if (l < nk) s0 += Vap[c + l * kv] * bb[l];
      } else {
        for (int l = 0; l < nk; ++l) s0 += Vap[l + c * ldVa] * bb[l];
      }
      u[c + (int64_t)(j0 + gg) * ld] = s0 + s1;
    }
    for (int e = tid; e < mk * ncol; e += ST) {
      const int i = e % mk, gg = e / mk;
      ws[nd.wx + i + (int64_t)(j0 + gg) * ld] = sb[i + gg * LDS];
    }
    __syncthreads();
  }
}

template <typename T, int TPC, int MR>
__global__ void __launch_bounds__(ST) ulv_solve_down_reg(const Task* __restrict__ tasks,
                                                         const Slot* __restrict__ slots, int stage_cap,
                                                         int nchunk) {
  constexpr int RPT = MR / TPC;
  constexpr int CPB = ST / TPC;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sQ = (T*)smraw;
  const Task tk = tasks[blockIdx.x / nchunk];
  const int jchunk = (blockIdx.x % nchunk) * CPB;
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* ws = (T*)sl.ws;
  const int64_t ld = sl.ldws;
  const T* fb = (const T*)sl.fbase;
  const int n = nd.n, r = sl.r;
  if (jchunk >= r) return;
  const int tid = threadIdx.x, g = tid / TPC, gl = tid % TPC;
  const T* x = ws + nd.wx;
  const T* Qt = fb + nd.fQt;
  if (!nd.root && nd.mk > 0 && n * nd.mk <= stage_cap) {
    for (int e = tid; e < n * nd.mk; e += ST) cpa(sQ + e, Qt + e);
    Qt = sQ;
    cpa_wait();
    __syncthreads();
  }
  for (int j0 = jchunk; j0 < jchunk + CPB && j0 < r; j0 += CPB) {
    const int j = j0 + g;
    const bool act = j < r;
    T b[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int row = gl + s * TPC;
      b[s] = (act && row < n) ? x[row + (int64_t)j * ld] : T(0);
    }
    if (!nd.root && nd.mk > 0) {
      // z[cols] = Q_lq^T z[cols]: reflectors i = mk-1 .. 0 (src/ulvfactor.jl:102)
      const T* tl = fb + nd.ftl;
      const int nl = min(nd.mk, n);
      for (int i = nl - 1; i >= 0; --i) {
        const T tau = tl[i];
        if (tau == T(0)) continue;
        const T* v = Qt + (int64_t)i * n;
        T d0 = T(0), d1 = T(0);
#pragma unroll
        for (int s = 0; s < RPT; s += 2) {
          const int row = gl + s * TPC;
          if (row < n) d0 += v[row] * b[s];
          if (s + 1 < RPT && row + TPC < n) d1 += v[row + TPC] * b[s + 1];
        }
        const T w = gsum<TPC>(d0 + d1) * tau;
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
          const int row = gl + s * TPC;
          if (row >= i && row < n) b[s] -= w * v[row];
        }
      }
    }
    if (!act) continue;
    if (nd.leaf) {
      const double sc = sl.colscale ? sl.colscale[j] : 1.0;
      double* out = sl.C + nd.col0 + (int64_t)j * sl.ldc;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int row = gl + s * TPC;
        if (row < n) {
          const double v = sc * (double)b[s];
          if (sl.mode) out[row] += v;
          else out[row] = v;
        }
      }
    } else {
      const Node& c1 = nodes[nd.left];
      const Node& c2 = nodes[nd.right];
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int row = gl + s * TPC;
        if (row < n) {
          if (row < c1.nr) ws[c1.wx + c1.nk + row + (int64_t)j * ld] = b[s];
          else ws[c2.wx + c2.nk + (row - c1.nr) + (int64_t)j * ld] = b[s];
        }
      }
    }
  }
}

constexpr size_t kSolveSmemCap = 200 * 1024;

template <typename T, int TPC, int MR>
void up_launch(const Task* t, int64_t nt, const Slot* s, size_t want, int rmax, cudaStream_t st) {
  const size_t base = (size_t)LDS * (ST / TPC) * sizeof(T);
  size_t smem = base + want * sizeof(T);
  if (smem > kSolveSmemCap) smem = base;   // operands stay in global memory
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(ulv_solve_up_reg<T, TPC, MR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSolveSmemCap);
    set = true;
  }
  const int nchunk = (rmax + ST / TPC - 1) / (ST / TPC);
  ulv_solve_up_reg<T, TPC, MR><<<(unsigned)(nt * nchunk), ST, smem, st>>>(t, s, (int64_t)((smem - base) / sizeof(T)),
                                                                          nchunk);
}

template <typename T, int TPC, int MR>
void down_launch(const Task* t, int64_t nt, const Slot* s, size_t want, int rmax, cudaStream_t st) {
  size_t smem = want * sizeof(T);
  if (smem > kSolveSmemCap) smem = 0;
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(ulv_solve_down_reg<T, TPC, MR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSolveSmemCap);
    set = true;
  }
  const int nchunk = (rmax + ST / TPC - 1) / (ST / TPC);
  ulv_solve_down_reg<T, TPC, MR><<<(unsigned)(nt * nchunk), ST, smem, st>>>(t, s, (int)(smem / sizeof(T)), nchunk);
}

}  // namespace

bool solve_reg_fits(int mmax, int nmax) { return mmax <= 256 && nmax <= 256; }

int64_t solve_up_stage_need(int m, int k, int mk, int nk, int kv, bool leaf, bool root, int mr1, int mr2, int kv1,
                            int kv2) {
  return solve_up_stage_elems(m, k, mk, nk, kv, leaf, root, mr1, mr2, kv1, kv2, ST / 32);
}

// One warp per right-hand-side column, 8 columns per thread block; the grid
// covers (node, column chunk) pairs so that few-node levels still fill SMs.
template <typename T>
void launch_ulv_solve_up_reg(const Task* t, int64_t nt, const Slot* s, int mmax, int64_t stage, int r,
                             cudaStream_t st) {
  if (nt <= 0 || r <= 0) return;
  const size_t want = (size_t)stage;
  if (mmax <= 64) up_launch<T, 32, 64>(t, nt, s, want, r, st);
  else if (mmax <= 128) up_launch<T, 32, 128>(t, nt, s, want, r, st);
  else up_launch<T, 32, 256>(t, nt, s, want, r, st);
}

template <typename T>
void launch_ulv_solve_down_reg(const Task* t, int64_t nt, const Slot* s, int nmax, int mkmax, int r,
                               cudaStream_t st) {
  if (nt <= 0 || r <= 0) return;
  const size_t want = (size_t)nmax * mkmax;
  if (nmax <= 64) down_launch<T, 32, 64>(t, nt, s, want, r, st);
  else if (nmax <= 128) down_launch<T, 32, 128>(t, nt, s, want, r, st);
  else down_launch<T, 32, 256>(t, nt, s, want, r, st);
}

template void launch_ulv_solve_up_reg<double>(const Task*, int64_t, const Slot*, int, int64_t, int, cudaStream_t);
template void launch_ulv_solve_up_reg<float>(const Task*, int64_t, const Slot*, int, int64_t, int, cudaStream_t);
template void launch_ulv_solve_down_reg<double>(const Task*, int64_t, const Slot*, int, int, int, cudaStream_t);
template void launch_ulv_solve_down_reg<float>(const Task*, int64_t, const Slot*, int, int, int, cudaStream_t);

}  // namespace hss
