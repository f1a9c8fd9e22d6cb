// Persistent HSS x dense product: the whole product C = alpha A B + beta Y of
// a forest in one cooperative launch (reference src/matmul.jl:18-62).
//
// The level-by-level product needs 2 + (levels up) + (levels down) dependent
// launches, and the upper levels hold a few KB of work each, so their cost is
// launch and load latency.  Here every block of the grid is resident
// (cooperative launch) and the tree's dependencies are resolved on the device:
//
//   1. upsweep by climbing: for each (leaf, column chunk) pair a block forms
//      Z = V^T B (matmul.jl:34) and arrives at the parent's counter of that chunk.  The second
//      child to arrive computes the parent, Z = W1^T Z1 + W2^T Z2 (:39), together
//      with the B-terms of the parent's children, G1 = B12 Z2 and G2 = B21 Z1
//      (:51, :55), then climbs on.  No block waits.  The block that completes a
//      root starts the downsweep of that tree (F of the root's children = G).
//   2. the leaf products D B (:46) are bulk units; upsweep and bulk units are
//      taken, upsweep first, from one global counter whenever no tree task is ready;
//   3. downsweep tasks go through a ready queue: the task of an internal node p,
//      enqueued once F_p is final, forms F_c = G_c + R_c F_p (:50-56) for both
//      children and enqueues them; the final task of a leaf (C += U F, :47) is
//      enqueued by whichever of its prerequisites (F of the leaf, every bulk
//      unit of the leaf) completes last.
// A block claims a queue entry by taking a ticket (one atomicAdd, never
// retried) whenever produced entries are unclaimed, and then polls only its
// own entry's tag; between bulk units it looks for unclaimed entries first, so
// the tree's dependency chain runs underneath the bandwidth-bound bulk work.
// Once the bulk units are gone every block takes a ticket or leaves.  Waits
// are bounded: a block whose entry does not appear within the poll limit
// records DEV_TIMEOUT and exits.  The last block to finish resets the launch
// counters, and the per-node counters reset themselves, so consecutive
// launches need no clearing.  Small products (upsweep, translators, downsweep)
// are split over all warps of the block, because GB300's FP64 units issue a
// warp instruction only every 64 cycles per SM sub-partition.
//
// Two arithmetics share the code: FP64 (the product of hss_matmul) and
// double-float pairs on the FP32 pipe (the refinement residual, with the
// generators pre-split into pairs and B split on the fly).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "hss_df.cuh"
#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int PT = 256;                      // threads per block
constexpr int RC = 8;                        // widest column chunk
constexpr int kSyncChunks = 64;              // column chunks per node in the counter array
constexpr int LCH = 64;                      // rows of V staged per pass (leaf upsweep)
constexpr uint32_t kIdleLimit = 1u << 22;    // polls of an idle block before it gives up
constexpr int PART_ELEMS = PT * 4;           // split-K partials (8-byte accumulators)

// launch counters, one 128-byte line each, then one epoch tag per queue entry
enum { ST_HEAD = 0, ST_TAIL = 32, ST_BULK = 64, ST_DONE = 96, ST_WORDS = 128 };

struct PmvArgs {
  const Task* leaves;
  const Slot* slots;
  uint32_t* state;       // launch counters and queue tags
  int2* qtask;           // queue entries: (slot, node)
  const char* pf;        // translator generators, prefetched into L2 at the start
  int64_t pf_bytes;
  int32_t nleaves, ntasks, nchunk, nbulk;
  int32_t cw;            // columns per chunk (<= RC)
  int32_t mcap;          // shared elements available for the staged translators
  uint32_t epoch;
};

// ---- arithmetic policies ----------------------------------------------------

struct PF64 {
  using E = double;
  struct Acc { double s; };
  __device__ static __forceinline__ Acc zero() { return Acc{0.0}; }
  __device__ static __forceinline__ void fma(Acc& a, E g, E x) { a.s = ::fma(g, x, a.s); }
  __device__ static __forceinline__ void acc(Acc& a, const Acc& b) { a.s += b.s; }
  __device__ static __forceinline__ void addE(Acc& a, E x) { a.s += x; }
  __device__ static __forceinline__ E fin(const Acc& a) { return a.s; }
  __device__ static __forceinline__ double dbl(const Acc& a) { return a.s; }
  __device__ static __forceinline__ const E* gen(const Slot&, const double* p) { return p; }
  __device__ static __forceinline__ E* ws(const Slot& s) { return (E*)s.ws; }
  __device__ static __forceinline__ E xin(double x) { return x; }
};

struct PDF {
  using E = float2;
  struct Acc { float h, l; };
  __device__ static __forceinline__ Acc zero() { return Acc{0.f, 0.f}; }
  __device__ static __forceinline__ void fma(Acc& a, E g, E x) { df_fma(a.h, a.l, g, x); }
  __device__ static __forceinline__ void acc(Acc& a, const Acc& b) { df_add(a.h, a.l, b.h, b.l); }
  __device__ static __forceinline__ void addE(Acc& a, E x) { df_add(a.h, a.l, x.x, x.y); }
  __device__ static __forceinline__ E fin(const Acc& a) { return df_norm(a.h, a.l); }
  __device__ static __forceinline__ double dbl(const Acc& a) { return (double)a.h + (double)a.l; }
  __device__ static __forceinline__ const E* gen(const Slot& s, const double* p) { return s.gdf + (p - s.gbase); }
  __device__ static __forceinline__ E* ws(const Slot& s) { return s.ws2; }
  __device__ static __forceinline__ E xin(double x) { return split_d(x); }
};

// ---- device-side scheduling -------------------------------------------------

__device__ __forceinline__ uint32_t ld_vol(const uint32_t* p) { return *(const volatile uint32_t*)p; }

__device__ __forceinline__ void set_err(const Slot& sl, int code) {
  if (sl.err) atomicCAS((int*)sl.err, DEV_OK, code);
}

// counter of (node, chunk)
__device__ __forceinline__ int32_t* counter(const Slot& sl, int node, int ch) {
  return sl.sync + (int64_t)node * kSyncChunks + ch;
}

// Appends task (slot, node, chunk) to the ready queue (one thread; the caller
// fenced its data).
__device__ void push(const PmvArgs& a, int slot, int node, int ch, const Slot& sl) {
  const uint32_t idx = atomicAdd(&a.state[ST_TAIL], 1u);
  if (idx >= (uint32_t)a.ntasks) {   // more tasks than the host counted: the tree tables disagree
    set_err(sl, DEV_BAD);
    return;
  }
  a.qtask[idx] = make_int2(slot, node * kSyncChunks + ch);
  __threadfence();
  atomicExch(&a.state[ST_WORDS + idx], a.epoch);
}

// One of the two prerequisites of a leaf chunk's final task is done (F of the
// leaf, or the leaf's bulk unit); the second one enqueues the task.
__device__ void leaf_event(const PmvArgs& a, int slot, const Slot& sl, int leaf, int ch) {
  int32_t* c = counter(sl, leaf, ch);
  if (atomicAdd(c, 1) == 1) {
    atomicExch(c, 0);
    push(a, slot, leaf, ch, sl);
  }
}

// Releases the children of node p, whose F of chunk ch is now final.
__device__ void release_children(const PmvArgs& a, int slot, const Slot& sl, const Node* nodes, const Node& p,
                                 int ch) {
  const int cs[2] = {p.left, p.right};
  for (int i = 0; i < 2; ++i) {
    if (nodes[cs[i]].leaf) leaf_event(a, slot, sl, cs[i], ch);
    else push(a, slot, cs[i], ch, sl);
  }
}

// ---- per-node work (one column chunk: columns j0 .. j0 + nc - 1) -------------

// Split-K layout of a small product over the block: op output slots (a power
// of two >= min(nout, PT)) x G = PT / op groups of terms.
__device__ __forceinline__ int out_slots(int nout) {
  int op = 1;
  while (op < nout && op < PT) op <<= 1;
  return op;
}

// out(o) = sum_{l < K} term(o, l) for o < nout with every thread taking part;
// epi(o, sum) consumes each result.  `part` holds PT accumulators.
template <class P, class Term, class Epi>
__device__ void sdot(int nout, int K, typename P::Acc* part, Term term, Epi epi) {
  using Acc = typename P::Acc;
  const int op = out_slots(nout), G = PT / op;
  const int slot = threadIdx.x % op, g = threadIdx.x / op;
  for (int o0 = 0; o0 < nout; o0 += op) {
    const int o = o0 + slot;
    Acc acc = P::zero();
    if (o < nout) {
#pragma unroll 4
      for (int l = g; l < K; l += G) term(o, l, acc);
    }
    if (G > 1) {
      __syncthreads();
      part[threadIdx.x] = acc;
      __syncthreads();
      if (g == 0 && o < nout)
        for (int gg = 1; gg < G; ++gg) P::acc(acc, part[gg * op + slot]);
    }
    if (g == 0 && o < nout) epi(o, acc);
  }
}

// Z = V^T B for one leaf (matmul.jl:34).  B is staged, V in passes of LCH rows
// (ld LCH + 1); thread (output slot, group) keeps its partial sums over the passes.
template <class P>
__device__ void leaf_up(const Slot& sl, const Node& nd, int j0, int nc, typename P::Acc* part,
                        typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  const int n = nd.gn, kv = nd.kv;
  if (kv == 0 || nc <= 0) return;
  const E* V = P::gen(sl, nd.V);
  E* ws = P::ws(sl);
  E* Xs = sm;                       // n x RC
  E* Vs = sm + n * RC;              // LCH x kv, ld LCH + 1
  const int nout = kv * nc, op = out_slots(nout), G = PT / op;
  const int slot = threadIdx.x % op, g = threadIdx.x / op;
  const double* X = sl.B + nd.col0 + (int64_t)j0 * sl.ldb;
  for (int e = threadIdx.x; e < n * nc; e += PT) {
    const int l = e % n, q = e / n;
    Xs[l + q * n] = P::xin(__ldg(X + l + (int64_t)q * sl.ldb));
  }
  Acc acc[2] = {P::zero(), P::zero()};   // nout <= 512 = 2 PT
  for (int l0 = 0; l0 < n; l0 += LCH) {
    const int nl = min(LCH, n - l0);
    __syncthreads();
    for (int e = threadIdx.x; e < nl * kv; e += PT) {
      const int l = e % nl, c = e / nl;
      Vs[l + c * (LCH + 1)] = __ldg(V + l0 + l + (int64_t)c * n);
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int o = s * op + slot;
      if (o < nout) {
        const int c = o % kv, q = o / kv;
        const E* v = Vs + c * (LCH + 1);
        const E* x = Xs + l0 + q * n;
#pragma unroll 4
        for (int l = g; l < nl; l += G) P::fma(acc[s], v[l], x[l]);
      }
    }
  }
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int o = s * op + slot;
    if (G > 1) {
      __syncthreads();
      part[threadIdx.x] = acc[s];
      __syncthreads();
      if (g == 0 && o < nout)
        for (int gg = 1; gg < G; ++gg) P::acc(acc[s], part[gg * op + slot]);
    }
    if (g == 0 && o < nout) ws[nd.wz + (o % kv) + (int64_t)(j0 + o / kv) * sl.ldws] = P::fin(acc[s]);
  }
}

// Climb step at branch p once both children's Z are final: Z_p = W1^T Z1 + W2^T Z2
// (matmul.jl:39; not for a root) and the B-terms G1 = B12 Z2, G2 = B21 Z1
// (:51, :55) into the children's F slots.
template <class P>
__device__ void climb_node(const PmvArgs& a, const Slot& sl, const Node* nodes, const Node& p, int j0, int nc,
                           typename P::Acc* part, typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  if (nc <= 0) return;
  const Node& c1 = nodes[p.left];
  const Node& c2 = nodes[p.right];
  const int v1 = c1.kv, v2 = c2.kv, u1 = c1.ku, u2 = c2.ku, kv = p.root ? 0 : p.kv;
  E* ws = P::ws(sl);
  const int64_t ld = sl.ldws;
  const int ldw = kv | 1;
  E* Z1 = sm;
  E* Z2 = Z1 + v1 * RC;
  E* M = Z2 + v2 * RC;
  const int needW = kv > 0 ? ldw * (v1 + v2) : 0, needB = u1 * v2 + u2 * v1;
  const bool together = needW + needB <= a.mcap;
  E* W1t = M;
  E* W2t = M + ldw * v1;
  E* B12 = together ? M + needW : M;
  E* B21 = B12 + u1 * v2;
  const E* gB12 = P::gen(sl, p.B12);
  const E* gB21 = P::gen(sl, p.B21);
  for (int e = threadIdx.x; e < v1 * nc; e += PT) Z1[e] = __ldcg(ws + c1.wz + (e % v1) + (int64_t)(j0 + e / v1) * ld);
  for (int e = threadIdx.x; e < v2 * nc; e += PT) Z2[e] = __ldcg(ws + c2.wz + (e % v2) + (int64_t)(j0 + e / v2) * ld);
  if (kv > 0) {
    const E* gW1 = P::gen(sl, p.W1);
    const E* gW2 = P::gen(sl, p.W2);
    for (int e = threadIdx.x; e < v1 * kv; e += PT) W1t[(e / v1) + (e % v1) * ldw] = __ldg(gW1 + e);
    for (int e = threadIdx.x; e < v2 * kv; e += PT) W2t[(e / v2) + (e % v2) * ldw] = __ldg(gW2 + e);
  }
  auto stageB = [&]() {
    for (int e = threadIdx.x; e < u1 * v2; e += PT) B12[e] = __ldg(gB12 + e);
    for (int e = threadIdx.x; e < u2 * v1; e += PT) B21[e] = __ldg(gB21 + e);
  };
  if (together) stageB();
  __syncthreads();
  if (kv > 0)
    sdot<P>(kv * nc, v1 + v2, part,
            [&](int o, int l, Acc& s) {
              const int c = o % kv, q = o / kv;
              if (l < v1) P::fma(s, W1t[c + l * ldw], Z1[l + q * v1]);
              else P::fma(s, W2t[c + (l - v1) * ldw], Z2[(l - v1) + q * v2]);
            },
            [&](int o, const Acc& s) { ws[p.wz + (o % kv) + (int64_t)(j0 + o / kv) * ld] = P::fin(s); });
  if (!together) {
    __syncthreads();
    stageB();
    __syncthreads();
  }
  sdot<P>((u1 + u2) * nc, max(v1, v2), part,
          [&](int o, int l, Acc& s) {
            if (o < u1 * nc) {
              const int i = o % u1, q = o / u1;
              if (l < v2) P::fma(s, B12[i + l * u1], Z2[l + q * v2]);
            } else {
              const int o2 = o - u1 * nc;
              const int i = o2 % u2, q = o2 / u2;
              if (l < v1) P::fma(s, B21[i + l * u2], Z1[l + q * v1]);
            }
          },
          [&](int o, const Acc& s) {
            if (o < u1 * nc) ws[c1.wf + (o % u1) + (int64_t)(j0 + o / u1) * ld] = P::fin(s);
            else ws[c2.wf + ((o - u1 * nc) % u2) + (int64_t)(j0 + (o - u1 * nc) / u2) * ld] = P::fin(s);
          });
}

// Arrival of a finished node (chunk ch) at its parent; the second child to arrive climbs.
template <class P>
__device__ void climb_from(const PmvArgs& a, int slot, const Slot& sl, const Node* nodes, int node, int ch,
                           typename P::Acc* part, typename P::E* sm) {
  __shared__ int s_go;
  const int j0 = ch * a.cw, nc = min(a.cw, sl.r - j0);
  for (;;) {
    const Node& x = nodes[node];
    if (x.root) return;
    __threadfence();   // every thread publishes its writes of x's Z / B-terms
    __syncthreads();
    if (threadIdx.x == 0) {
      int32_t* c = counter(sl, x.parent, ch);
      const int old = atomicAdd(c, 1);
      s_go = old == 1;
      if (old == 1) atomicExch(c, 0);
    }
    __syncthreads();
    if (!s_go) return;
    __threadfence();
    const Node& p = nodes[x.parent];
    climb_node<P>(a, sl, nodes, p, j0, nc, part, sm);
    if (p.root) {
      // F of the root's children is their B-term (the root has no F)
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) release_children(a, slot, sl, nodes, p, ch);
      return;
    }
    node = x.parent;
  }
}

// Downsweep task of a non-root branch p (F_p final):
// F_c = G_c + R_c F_p for both children (matmul.jl:50-56), in place over G_c.
template <class P>
__device__ void down_node(const Slot& sl, const Node* nodes, const Node& p, int j0, int nc, typename P::Acc* part,
                          typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  if (nc <= 0) return;
  const Node& c1 = nodes[p.left];
  const Node& c2 = nodes[p.right];
  const int u1 = c1.ku, u2 = c2.ku, kp = p.ku;
  E* ws = P::ws(sl);
  const int64_t ld = sl.ldws;
  E* Fp = sm;                 // kp x RC
  E* R1 = Fp + kp * RC;       // u1 x kp
  E* R2 = R1 + u1 * kp;       // u2 x kp
  const E* gR1 = P::gen(sl, p.R1);
  const E* gR2 = P::gen(sl, p.R2);
  for (int e = threadIdx.x; e < kp * nc; e += PT) Fp[e] = __ldcg(ws + p.wf + (e % kp) + (int64_t)(j0 + e / kp) * ld);
  for (int e = threadIdx.x; e < u1 * kp; e += PT) R1[e] = __ldg(gR1 + e);
  for (int e = threadIdx.x; e < u2 * kp; e += PT) R2[e] = __ldg(gR2 + e);
  __syncthreads();
  sdot<P>((u1 + u2) * nc, kp, part,
          [&](int o, int l, Acc& s) {
            if (o < u1 * nc) P::fma(s, R1[(o % u1) + l * u1], Fp[l + (o / u1) * kp]);
            else P::fma(s, R2[((o - u1 * nc) % u2) + l * u2], Fp[l + ((o - u1 * nc) / u2) * kp]);
          },
          [&](int o, const Acc& s) {
            const bool first = o < u1 * nc;
            const int o2 = first ? o : o - u1 * nc;
            const int uc = first ? u1 : u2;
            E* f = ws + (first ? c1.wf : c2.wf) + (o2 % uc) + (int64_t)(j0 + o2 / uc) * ld;
            Acc t = s;
            P::addE(t, __ldcg(f));
            *f = P::fin(t);
          });
}

// out(i, q) = sum_l A(i + l*lda) Xs(l + q*ldx) for i < m, q < NQ, l < K, A from
// global memory (read-only), Xs staged; `epi(i, q, acc)` consumes each result and
// returns the FP64 value written (for the column sums of squares when cn != 0).
// Threads: row slot ii of rp (a power of two >= rows of the pass), split-K group g.
template <class P, int NQ, class Epi>
__device__ void rows_cols(const typename P::E* __restrict__ A, int m, int K, int64_t lda,
                          const typename P::E* Xs, int ldx, typename P::Acc* part, double* cn, Epi epi) {
  using Acc = typename P::Acc;
  const int tid = threadIdx.x;
  double sq[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) sq[q] = 0.0;
  for (int r0 = 0; r0 < m; r0 += PT) {
    const int rows = min(PT, m - r0);
    int rp = 1;
    while (rp < rows) rp <<= 1;
    const int G = PT / rp;
    const int ii = tid % rp, g = tid / rp;
    const int i = r0 + ii;
    const bool act = ii < rows;
    Acc acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = P::zero();
    if (act) {
      const typename P::E* a = A + i;
#pragma unroll 8
      for (int l = g; l < K; l += G) {
        const typename P::E d = __ldg(a + (int64_t)l * lda);
#pragma unroll
        for (int q = 0; q < NQ; ++q) P::fma(acc[q], d, Xs[l + q * ldx]);
      }
    }
    if (G > 1) {
      __syncthreads();
#pragma unroll
      for (int q = 0; q < NQ; ++q) part[(g * rp + ii) * NQ + q] = acc[q];
      __syncthreads();
      if (g == 0 && act) {
        for (int gg = 1; gg < G; ++gg)
#pragma unroll
          for (int q = 0; q < NQ; ++q) P::acc(acc[q], part[(gg * rp + ii) * NQ + q]);
      }
    }
    if (g == 0 && act) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const double v = epi(i, q, acc[q]);
        sq[q] = fma(v, v, sq[q]);
      }
    }
  }
  if (cn != nullptr) {
    const int lane = tid & 31;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double v = sq[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0 && v != 0.0) atomicAdd(cn + q, v);
    }
  }
}

// Runs rows_cols over nc <= RC columns in groups of 4, 2, 1; `epi(i, q, acc)`
// receives the absolute column q within the pass.
template <class P, class Epi>
__device__ void rows_cols_n(const typename P::E* A, int m, int K, int64_t lda, const typename P::E* Xs, int ldx,
                            int nc, typename P::Acc* part, double* cn, Epi epi) {
  int q0 = 0;
  auto run = [&](auto nq) {
    constexpr int NQ = decltype(nq)::value;
    rows_cols<P, NQ>(A, m, K, lda, Xs + q0 * ldx, ldx, part, cn ? cn + q0 : nullptr,
                     [&](int i, int q, const typename P::Acc& s) { return epi(i, q0 + q, s); });
    q0 += NQ;
  };
  while (nc - q0 >= 4) run(std::integral_constant<int, 4>());
  if (nc - q0 >= 2) run(std::integral_constant<int, 2>());
  if (nc - q0 >= 1) run(std::integral_constant<int, 1>());
}

// Bulk unit: the leaf product D B for one column chunk (matmul.jl:46).  FP64:
// C = alpha D B + beta Y; pairs: D B kept in the pair buffer for the final task.
// A single-leaf tree (the leaf is the root) finishes here, column norms included.
template <class P>
__device__ void bulk_unit(const PmvArgs& a, int u, typename P::Acc* part, typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  const int t = u / a.nchunk, ch = u % a.nchunk;
  const Task tk = a.leaves[t];
  const Slot& sl = a.slots[tk.slot];
  const Node& nd = tk.nodes[tk.node];
  const int j0 = ch * a.cw;
  if (j0 < sl.r) {
    const int nc = min(a.cw, sl.r - j0), m = nd.gm, n = nd.gn;
    E* Xs = sm;
    __syncthreads();
    const double* X = sl.B + nd.col0 + (int64_t)j0 * sl.ldb;
    for (int e = threadIdx.x; e < n * nc; e += PT) {
      const int l = e % n, q = e / n;
      Xs[l + q * n] = P::xin(__ldg(X + l + (int64_t)q * sl.ldb));
    }
    __syncthreads();
    const E* D = P::gen(sl, nd.D);
    double* C = sl.C + nd.row0 + (int64_t)j0 * sl.ldc;
    const double* Y = sl.Y ? sl.Y + nd.row0 + (int64_t)j0 * sl.ldy : nullptr;
    const bool yterm = sl.beta != 0.0 && Y != nullptr;
    double* cn = (nd.root && sl.colnorm2) ? sl.colnorm2 + j0 : nullptr;
    constexpr bool pairs = !std::is_same<E, double>::value;
    if (pairs && !nd.root) {
      E* T = (E*)sl.tmp + nd.row0 + (int64_t)j0 * sl.ldt2;
      rows_cols_n<P>(D, m, n, m, Xs, n, nc, part, nullptr, [&](int i, int q, const Acc& s) {
        T[i + (int64_t)q * sl.ldt2] = P::fin(s);
        return 0.0;
      });
    } else {
      rows_cols_n<P>(D, m, n, m, Xs, n, nc, part, cn, [&](int i, int q, const Acc& s) {
        double v = sl.alpha * P::dbl(s);
        if (yterm) v += sl.beta * __ldcg(Y + i + (int64_t)q * sl.ldy);
        C[i + (int64_t)q * sl.ldc] = v;
        return v;
      });
    }
  }
  if (!nd.root) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) leaf_event(a, tk.slot, sl, tk.node, ch);
  }
}

// Final task of a non-root leaf chunk (F final, bulk done): C += alpha U F
// (matmul.jl:47), or for pairs C = alpha (D B + U F) + beta Y, with the column
// sums of squares.
template <class P>
__device__ void final_leaf(const Slot& sl, const Node& nd, int j0, int nc, typename P::Acc* part,
                           typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  constexpr bool pairs = !std::is_same<E, double>::value;
  if (nc <= 0) return;
  const int m = nd.gm, ku = nd.ku;
  E* ws = P::ws(sl);
  E* Fs = sm;                              // ku x RC
  const E* U = P::gen(sl, nd.U);
  __syncthreads();
  for (int e = threadIdx.x; e < ku * nc; e += PT) Fs[e] = __ldcg(ws + nd.wf + (e % ku) + (int64_t)(j0 + e / ku) * sl.ldws);
  __syncthreads();
  double* C = sl.C + nd.row0 + (int64_t)j0 * sl.ldc;
  double* cn = sl.colnorm2 ? sl.colnorm2 + j0 : nullptr;
  if (pairs) {
    const E* T = (const E*)sl.tmp + nd.row0 + (int64_t)j0 * sl.ldt2;
    const double* Y = sl.Y ? sl.Y + nd.row0 + (int64_t)j0 * sl.ldy : nullptr;
    const bool yterm = sl.beta != 0.0 && Y != nullptr;
    rows_cols_n<P>(U, m, ku, m, Fs, ku, nc, part, cn, [&](int i, int q, const Acc& s) {
      Acc t = s;
      P::addE(t, __ldcg(T + i + (int64_t)q * sl.ldt2));
      double v = sl.alpha * P::dbl(t);
      if (yterm) v += sl.beta * __ldcg(Y + i + (int64_t)q * sl.ldy);
      C[i + (int64_t)q * sl.ldc] = v;
      return v;
    });
  } else {
    rows_cols_n<P>(U, m, ku, m, Fs, ku, nc, part, cn, [&](int i, int q, const Acc& s) {
      const double v = __ldcg(C + i + (int64_t)q * sl.ldc) + sl.alpha * P::dbl(s);
      C[i + (int64_t)q * sl.ldc] = v;
      return v;
    });
  }
}

template <class P>
__global__ void __launch_bounds__(PT, 4) pmv_kernel(PmvArgs a) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  extern __shared__ __align__(16) unsigned char pmv_smem[];
  Acc* part = (Acc*)pmv_smem;                    // PART_ELEMS split-K partials
  E* sm = (E*)pmv_smem + PART_ELEMS;             // per-phase staging
  __shared__ int s_cmd, s_x, s_y;

  // the translators are read by the tree chain: have them in L2 before it starts
  for (int64_t off = ((int64_t)blockIdx.x * PT + threadIdx.x) * 128; off < a.pf_bytes;
       off += (int64_t)gridDim.x * PT * 128)
    asm volatile("prefetch.global.L2::evict_last [%0];" ::"l"(a.pf + off));

  // Work units of one counter: the nbulk (leaf, chunk) upsweep units first (they
  // start the tree chain), then the nbulk bulk units; claimed queue entries first.
  const uint32_t nwork = 2u * (uint32_t)a.nbulk;
  uint32_t idle = 0;
  int ticket = -1;   // queue entry this block has claimed (thread 0)
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      int cmd = 0;
      if (ticket < 0) {
        const uint32_t hd = ld_vol(&a.state[ST_HEAD]);
        if (hd < ld_vol(&a.state[ST_TAIL])) {          // produced, unclaimed entries
          const uint32_t t = atomicAdd(&a.state[ST_HEAD], 1u);
          if (t < (uint32_t)a.ntasks) ticket = (int)t;
        }
        if (ticket < 0) {
          if (ld_vol(&a.state[ST_BULK]) < nwork) {
            const uint32_t u = atomicAdd(&a.state[ST_BULK], 1u);
            if (u < nwork) {
              s_x = (int)u;
              cmd = 2;
            }
          }
          if (cmd == 0) {                                // no bulk left: claim or leave
            const uint32_t t = hd < (uint32_t)a.ntasks ? atomicAdd(&a.state[ST_HEAD], 1u) : (uint32_t)a.ntasks;
            if (t < (uint32_t)a.ntasks) ticket = (int)t;
            else cmd = 3;
          }
        }
      }
      if (ticket >= 0 && ld_vol(&a.state[ST_WORDS + ticket]) == a.epoch) {
        __threadfence();
        const int2 q = __ldcg(&a.qtask[ticket]);
        s_x = q.x;
        s_y = q.y;
        cmd = 1;
        ticket = -1;
      }
      if (cmd == 0) {
        if (++idle > kIdleLimit) {
          set_err(a.slots[0], DEV_TIMEOUT);
          cmd = 3;
        } else {
          __nanosleep(32);
        }
      } else {
        idle = 0;
      }
      s_cmd = cmd;
    }
    __syncthreads();
    const int cmd = s_cmd;
    if (cmd == 3) break;
    if (cmd == 1) {
      const int slot = s_x, node = s_y / kSyncChunks, ch = s_y % kSyncChunks;
      const Slot& sl = a.slots[slot];
      const Node* nodes = sl.nodes;
      const Node& x = nodes[node];
      const int j0 = ch * a.cw, nc = min(a.cw, sl.r - j0);
      if (x.leaf) {
        final_leaf<P>(sl, x, j0, nc, part, sm);
      } else {
        down_node<P>(sl, nodes, x, j0, nc, part, sm);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) release_children(a, slot, sl, nodes, x, ch);
      }
    } else if (cmd == 2) {
      const int u = s_x;
      if (u < a.nbulk) {
        // upsweep unit (leaf, chunk): Z = V^T B, then climb
        const int ch = u % a.nchunk;
        const Task tk = a.leaves[u / a.nchunk];
        const Slot& sl = a.slots[tk.slot];
        const Node& nd = tk.nodes[tk.node];
        if (!nd.root) {
          const int j0 = ch * a.cw;
          leaf_up<P>(sl, nd, j0, min(a.cw, sl.r - j0), part, sm);
          climb_from<P>(a, tk.slot, sl, tk.nodes, tk.node, ch, part, sm);
        }
      } else {
        bulk_unit<P>(a, u - a.nbulk, part, sm);
      }
    }
  }

  // the last block out resets the launch counters
  if (threadIdx.x == 0) {
    __threadfence();
    const uint32_t d = atomicAdd(&a.state[ST_DONE], 1u);
    if (d == gridDim.x - 1) {
      a.state[ST_HEAD] = 0;
      a.state[ST_TAIL] = 0;
      a.state[ST_BULK] = 0;
      __threadfence();
      a.state[ST_DONE] = 0;
    }
  }
}

template <class P>
struct Occ {
  size_t smem = 0;
  int blocks = 0;
};

template <class P>
int resident_blocks(size_t smem, int device) {
  static Occ<P> cache[8];
  if (device < 0 || device >= 8) device = 0;
  Occ<P>& c = cache[device];
  if (c.smem == smem && c.blocks > 0) return c.blocks;
  if (smem > 48 * 1024) cudaFuncSetAttribute(pmv_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pmv_kernel<P>, PT, smem) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  c.smem = smem;
  c.blocks = per_sm * sms;
  return c.blocks;
}

}  // namespace

// Shared memory (elements of 8 bytes) the persistent product needs for leaves
// of at most nleaf columns, ranks of at most kmax; mcap receives the part
// available for staged translators.
size_t pmv_smem_elems(int nleaf, int kmax, int* mcap) {
  const size_t k = kmax > 0 ? kmax : 1;
  const size_t up = (size_t)nleaf * RC + (size_t)(LCH + 1) * k;
  const size_t bulk = (size_t)nleaf * RC;
  const size_t fin = k * RC;
  const size_t down = k * RC + 2 * k * k;
  const size_t zst = 2 * k * RC;
  const size_t two = std::max((k | 1) * 2 * k, 2 * k * k);
  const size_t all = (k | 1) * 2 * k + 2 * k * k;
  const size_t need = std::max(std::max(up, bulk), std::max(fin, down));
  // stage all four translators at once when the whole buffer stays within 48 KB
  const size_t with_all = PART_ELEMS + std::max(need, zst + all);
  const size_t total = with_all * 8 <= 48 * 1024 ? with_all : PART_ELEMS + std::max(need, zst + two);
  if (mcap) *mcap = (int)(total - PART_ELEMS - zst);
  return total;
}

bool pmv_fits(int nleaf, int mleaf, int kmax) {
  return nleaf <= 512 && mleaf <= 1 << 20 && kmax <= 64 && pmv_smem_elems(nleaf, kmax, nullptr) * 8 <= 160 * 1024;
}

int pmv_chunks(bool pairs, int rmax) {
  const int cw = pairs ? RC : 4;
  const int nc = std::max(1, (rmax + cw - 1) / cw);
  return nc <= kSyncChunks ? nc : 0;
}
int64_t pmv_state_words(int64_t entries) { return ST_WORDS + entries; }
int pmv_sync_chunks() { return kSyncChunks; }

cudaError_t launch_pmv(bool pairs, const Task* leaves, int64_t nleaves, const Slot* slots, int64_t ntasks, int rmax,
                       int nleaf, int kmax, uint32_t* state, int2* qtask, uint32_t epoch, const void* prefetch,
                       int64_t prefetch_bytes, int device, cudaStream_t st) {
  if (nleaves <= 0) return cudaSuccess;
  int mcap = 0;
  const size_t smem = pmv_smem_elems(nleaf, kmax, &mcap) * 8;
  PmvArgs a;
  a.leaves = leaves;
  a.slots = slots;
  a.state = state;
  a.qtask = qtask;
  a.nleaves = (int32_t)nleaves;
  a.cw = pairs ? RC : 4;   // FP64: narrower chunks spread the slow FP64 work over more SMs
  a.nchunk = pmv_chunks(pairs, rmax);
  if (a.nchunk == 0) return cudaErrorInvalidValue;
  a.nbulk = (int32_t)(nleaves * a.nchunk);
  a.ntasks = (int32_t)(ntasks * a.nchunk);
  a.mcap = mcap;
  a.epoch = epoch;
  a.pf = (const char*)prefetch;
  a.pf_bytes = prefetch ? prefetch_bytes : 0;
  void* args[] = {&a};
  const int cap = pairs ? resident_blocks<PDF>(smem, device) : resident_blocks<PF64>(smem, device);
  if (cap <= 0) return cudaErrorLaunchOutOfResources;
  // every block must be resident; more blocks than work units would only poll
  const unsigned grid = (unsigned)std::min<int64_t>(cap, std::max<int64_t>(1, 2 * (int64_t)a.nbulk));
  return pairs ? cudaLaunchCooperativeKernel((void*)pmv_kernel<PDF>, grid, PT, args, smem, st)
               : cudaLaunchCooperativeKernel((void*)pmv_kernel<PF64>, grid, PT, args, smem, st);
}

}  // namespace hss
