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

template <typename T, int TPC, int MR>
__global__ void __launch_bounds__(ST) ulv_solve_up_reg(const Task* __restrict__ tasks,
                                                       const Slot* __restrict__ slots, int stage_cap) {
  constexpr int RPT = MR / TPC;
  constexpr int CPB = ST / TPC;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sb = (T*)smraw;   // LDS x CPB
  T* sfac = sb + LDS * CPB;   // staged factor blocks (stage_cap elements)
  const Task tk = tasks[blockIdx.x];
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* ws = (T*)sl.ws;
  const int64_t ld = sl.ldws;
  const T* fb = (const T*)sl.fbase;
  const int m = nd.m, kv = nd.kv, r = sl.r;
  const int tid = threadIdx.x, g = tid / TPC, gl = tid % TPC;
  const int k = nd.k, mk = nd.mk, nk = nd.nk;
  T* u = ws + nd.wu;
  // Factor blocks read inside the sequential sweeps are copied on chip once:
  // the QL reflectors (m x k) and L1 (mk x mk), or the root LU (m x m).
  const T* Up = fb + nd.fU;     // ld m
  const T* Lp = fb + nd.fD;     // ld m
  int ldL = m;
  if (nd.root) {
    if (m * m <= stage_cap) {
      for (int e = tid; e < m * m; e += ST) sfac[e] = Lp[e];
      Lp = sfac;
    }
  } else if (mk > 0 && m * k + mk * mk <= stage_cap) {
    T* sU = sfac;
    T* sL = sfac + m * k;
    for (int e = tid; e < m * k; e += ST) sU[e] = Up[e];
    for (int e = tid; e < mk * mk; e += ST) sL[e] = Lp[(e % mk) + (int64_t)(e / mk) * m];
    Up = sU;
    Lp = sL;
    ldL = mk;
  }
  for (int j0 = 0; j0 < r; j0 += CPB) {
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
      const Node& c1 = nodes[nd.left];
      const Node& c2 = nodes[nd.right];
      const T* T12 = fb + nd.fT12;
      const T* T21 = fb + nd.fT21;
      for (int e = tid; e < m * CPB; e += ST) {
        const int row = e % m, gg = e / m, j = j0 + gg;
        T val = T(0);
        if (j < r) {
          if (row < c1.mr) {
            val = ws[c1.wb + c1.mk + row + (int64_t)j * ld];
            const T* u2 = ws + c2.wu + (int64_t)j * ld;
            for (int l = 0; l < c2.kv; ++l) val -= T12[row + (int64_t)l * c1.mr] * u2[l];
          } else {
            const int i2 = row - c1.mr;
            val = ws[c2.wb + c2.mk + i2 + (int64_t)j * ld];
            const T* u1 = ws + c1.wu + (int64_t)j * ld;
            for (int l = 0; l < c1.kv; ++l) val -= T21[i2 + (int64_t)l * c2.mr] * u1[l];
          }
        }
        sb[row + gg * LDS] = val;
      }
      if (!nd.root) {
        for (int e = tid; e < kv * CPB; e += ST) {
          const int c = e % kv, j = j0 + e / kv;
          if (j >= r) continue;
          const T* u1 = ws + c1.wu + (int64_t)j * ld;
          const T* u2 = ws + c2.wu + (int64_t)j * ld;
          T s = T(0);
          for (int l = 0; l < c1.kv; ++l) s += (T)nd.W1[l + (int64_t)c * c1.kv] * u1[l];
          for (int l = 0; l < c2.kv; ++l) s += (T)nd.W2[l + (int64_t)c * c2.kv] * u2[l];
          u[c + (int64_t)j * ld] = s;
        }
      }
    }
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
      lower_solve<T, TPC, RPT, true>(b, A, m, m, gl);
      upper_solve<T, TPC, RPT>(b, A, m, m, gl);
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
      const T* Uf = Up;
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
        const T* v = Uf + (int64_t)c * m;
        T dot = T(0);
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
          const int row = gl + s * TPC;
          const T vr = row < p ? v[row] : (row == p ? T(1) : T(0));
          dot += vr * b[s];
        }
        dot = gsum<TPC>(dot) * tau;
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
    const T* Df = fb + nd.fD;
    const T* Vf = fb + nd.fV;
    for (int e = tid; e < (m - mk) * CPB; e += ST) {
      const int i = e % (m - mk), gg = e / (m - mk), jj = j0 + gg;
      if (jj >= r) continue;
      const T* bb = sb + gg * LDS;
      T s = bb[mk + i];
      for (int l = 0; l < nk; ++l) s -= Df[mk + i + (int64_t)l * m] * bb[l];
      ws[nd.wb + mk + i + (int64_t)jj * ld] = s;
    }
    for (int e = tid; e < kv * CPB; e += ST) {
      const int c = e % kv, gg = e / kv, jj = j0 + gg;
      if (jj >= r) continue;
      const T* bb = sb + gg * LDS;
      T s = nd.leaf ? T(0) : u[c + (int64_t)jj * ld];
      for (int l = 0; l < nk; ++l) s += Vf[l + (int64_t)c * nd.n] * bb[l];
      u[c + (int64_t)jj * ld] = s;
    }
    for (int e = tid; e < mk * CPB; e += ST) {
      const int i = e % mk, gg = e / mk, jj = j0 + gg;
      if (jj < r) ws[nd.wx + i + (int64_t)jj * ld] = sb[i + gg * LDS];
    }
    __syncthreads();
  }
}

template <typename T, int TPC, int MR>
__global__ void __launch_bounds__(ST) ulv_solve_down_reg(const Task* __restrict__ tasks,
                                                         const Slot* __restrict__ slots, int stage_cap) {
  constexpr int RPT = MR / TPC;
  constexpr int CPB = ST / TPC;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sQ = (T*)smraw;
  const Task tk = tasks[blockIdx.x];
  const Node* nodes = tk.nodes;
  const Node& nd = nodes[tk.node];
  const Slot& sl = slots[tk.slot];
  T* ws = (T*)sl.ws;
  const int64_t ld = sl.ldws;
  const T* fb = (const T*)sl.fbase;
  const int n = nd.n, r = sl.r;
  const int tid = threadIdx.x, g = tid / TPC, gl = tid % TPC;
  const T* x = ws + nd.wx;
  const T* Qt = fb + nd.fQt;
  if (!nd.root && nd.mk > 0 && n * nd.mk <= stage_cap) {
    for (int e = tid; e < n * nd.mk; e += ST) sQ[e] = Qt[e];
    Qt = sQ;
    __syncthreads();
  }
  for (int j0 = 0; j0 < r; j0 += CPB) {
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
void up_launch(const Task* t, int64_t nt, const Slot* s, size_t want, cudaStream_t st) {
  const size_t base = (size_t)LDS * (ST / TPC) * sizeof(T);
  size_t smem = base + want * sizeof(T);
  if (smem > kSolveSmemCap) smem = base;   // factor blocks stay in global memory
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(ulv_solve_up_reg<T, TPC, MR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSolveSmemCap);
    set = true;
  }
  ulv_solve_up_reg<T, TPC, MR><<<(unsigned)nt, ST, smem, st>>>(t, s, (int)((smem - base) / sizeof(T)));
}

template <typename T, int TPC, int MR>
void down_launch(const Task* t, int64_t nt, const Slot* s, size_t want, cudaStream_t st) {
  size_t smem = want * sizeof(T);
  if (smem > kSolveSmemCap) smem = 0;
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(ulv_solve_down_reg<T, TPC, MR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSolveSmemCap);
    set = true;
  }
  ulv_solve_down_reg<T, TPC, MR><<<(unsigned)nt, ST, smem, st>>>(t, s, (int)(smem / sizeof(T)));
}

}  // namespace

bool solve_reg_fits(int mmax, int nmax) { return mmax <= 256 && nmax <= 256; }

template <typename T>
void launch_ulv_solve_up_reg(const Task* t, int64_t nt, const Slot* s, int mmax, int kmax, int mkmax, int r,
                             cudaStream_t st) {
  if (nt <= 0) return;
  const bool wide = r > 8;
  // staged elements: reflectors + L1, or the root's LU (whichever is larger)
  const size_t want = std::max((size_t)mmax * kmax + (size_t)mkmax * mkmax, (size_t)mmax * mmax);
  if (mmax <= 64) wide ? up_launch<T, 8, 64>(t, nt, s, want, st) : up_launch<T, 32, 64>(t, nt, s, want, st);
  else if (mmax <= 128) wide ? up_launch<T, 8, 128>(t, nt, s, want, st) : up_launch<T, 32, 128>(t, nt, s, want, st);
  else wide ? up_launch<T, 8, 256>(t, nt, s, want, st) : up_launch<T, 32, 256>(t, nt, s, want, st);
}

template <typename T>
void launch_ulv_solve_down_reg(const Task* t, int64_t nt, const Slot* s, int nmax, int mkmax, int r,
                               cudaStream_t st) {
  if (nt <= 0) return;
  const bool wide = r > 8;
  const size_t want = (size_t)nmax * mkmax;
  if (nmax <= 64) wide ? down_launch<T, 8, 64>(t, nt, s, want, st) : down_launch<T, 32, 64>(t, nt, s, want, st);
  else if (nmax <= 128) wide ? down_launch<T, 8, 128>(t, nt, s, want, st) : down_launch<T, 32, 128>(t, nt, s, want, st);
  else wide ? down_launch<T, 8, 256>(t, nt, s, want, st) : down_launch<T, 32, 256>(t, nt, s, want, st);
}

template void launch_ulv_solve_up_reg<double>(const Task*, int64_t, const Slot*, int, int, int, int, cudaStream_t);
template void launch_ulv_solve_up_reg<float>(const Task*, int64_t, const Slot*, int, int, int, int, cudaStream_t);
template void launch_ulv_solve_down_reg<double>(const Task*, int64_t, const Slot*, int, int, int, cudaStream_t);
template void launch_ulv_solve_down_reg<float>(const Task*, int64_t, const Slot*, int, int, int, cudaStream_t);

}  // namespace hss
