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
//      child to arrive computes the parent, Z = W1^T Z1 + W2^T Z2 (:39), and
//      climbs on; no block waits.  The B-terms of a branch's children, G1 = B12 Z2
//      and G2 = B21 Z1 (:51, :55), are a separate queue task, off the climb's
//      critical path.  The block that reaches a root forms the root's B-terms
//      and starts the downsweep of that tree (F of the root's children = G).
//   2. the leaf products D B (:46) are bulk units; upsweep and bulk units are
//      taken, upsweep first, from one global counter whenever no tree task is ready;
//   3. downsweep tasks go through a ready queue: the task of an internal node p,
//      enqueued once F_p is final and the B-terms of p's children are done, forms
//      F_c = G_c + R_c F_p (:50-56) for both children; the final task of a leaf
//      (C += U F, :47) is enqueued once F of the leaf is final and the leaf's bulk
//      unit is done.  Each pair of prerequisites meets on a per-node counter.
// A block claims a queue entry by taking a ticket (one atomicAdd, never
// retried) whenever produced entries are unclaimed, and then polls only its
// own entry's tag; between bulk units it looks for unclaimed entries first, so
// the tree's dependency chain runs underneath the bandwidth-bound bulk work.
// Once the bulk units are gone every block takes a ticket or leaves.  Waits
// are bounded: a block whose entry does not appear within the poll limit
// records DEV_TIMEOUT and exits.  The last block to finish resets the launch
// counters; the per-node counters are even between launches (each launch adds
// an even number), so consecutive launches need no clearing.  Small products (upsweep, translators, downsweep)
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
constexpr uint32_t kIdleLimit = 1u << 22;    // default polls of an idle block before it gives up
uint32_t g_idle_limit = kIdleLimit;          // host copy, passed to every launch (hss_set_option)
constexpr int PART_ELEMS = PT * 4;           // split-K partials (8-byte accumulators)

// launch counters, one 128-byte line each (the flat product uses the same
// words for its own counters and four more lines)
enum { ST_HEAD = 0, ST_TAIL = 32, ST_BULK = 64, ST_DONE = 96, ST_WORDS = 224 };
enum { FL_A = 0, FL_B = 32, FL_C = 64, FL_DONE = 96, FL_AFIN = 128, FL_D = 160, FL_BFIN = 192 };

// A queue entry is one 64-bit word, so that a consumer reads the task and its
// tag in one load: epoch (21 bits) | kind (1) | slot (16) | node (20) | column
// chunk (6).  Kinds: the node's downsweep task (a leaf's final task), or the
// B-terms of the node's children.
constexpr int QE_EPOCH = 43, QE_KIND = 42, QE_SLOT = 26, QE_NODE = 6;
enum { TK_DOWN = 0, TK_BTERM = 1 };

struct PmvArgs {
  const Task* leaves;
  const Slot* slots;
  uint32_t* state;       // launch counters
  unsigned long long* qent;   // queue entries
  const char* pf;        // translator generators, prefetched into L2 at the start
  int64_t pf_bytes;
  int32_t nleaves, ntasks, nchunk, nbulk;
  int32_t cw;            // columns per chunk (<= RC)
  uint32_t epoch;
  uint32_t idle_limit;   // polls of an idle block before DEV_TIMEOUT
  int32_t dx_ready;      // pairs: the non-root leaves' D B is already in the pair buffer (tensor cores)
  int32_t leaf_ext;      // pairs: Z = V^T B is in the workspace and the final products follow the launch
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
  __device__ static __forceinline__ E xin(double x) { return split_bits(x); }
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

__device__ __forceinline__ unsigned long long qentry(uint32_t epoch, int kind, int slot, int node, int ch) {
  return ((unsigned long long)epoch << QE_EPOCH) | ((unsigned long long)kind << QE_KIND) |
         ((unsigned long long)slot << QE_SLOT) | ((unsigned long long)node << QE_NODE) | (unsigned long long)ch;
}

// Appends np <= 2 tasks (kind[i], slot, node[i], chunk) to the ready queue: one
// thread, after a barrier of the block and a fence that published the tasks' data.
__device__ void push(const PmvArgs& a, int slot, const int* node, const int* kind, int np, int ch, const Slot& sl) {
  if (np == 0) return;
  const uint32_t idx = atomicAdd(&a.state[ST_TAIL], (uint32_t)np);
  for (int i = 0; i < np; ++i) {
    if (idx + i >= (uint32_t)a.ntasks) {   // more tasks than the host counted: the tree tables disagree
      set_err(sl, DEV_BAD);
      return;
    }
    *(volatile unsigned long long*)&a.qent[idx + i] = qentry(a.epoch, kind[i], slot, node[i], ch);
  }
}

// Every non-root node's downsweep task (a leaf: its final task) has two
// prerequisites: its F is final, and either the B-terms of its children
// (branch) or its bulk unit (leaf) are done.  The second of the two events on
// the node's counter enqueues the task.  Counters are never reset: a launch
// adds an even number to each (a branch: two arrivals, then two events; a
// leaf: two events), so the second event of a pair is the one that reads an
// odd value.
__device__ void node_event(const PmvArgs& a, int slot, const Slot& sl, int node, int ch) {
  int32_t* c = counter(sl, node, ch);
  if (atomicAdd(c, 1) & 1) {
    // the first event's writes, observed through the counter, are published
    // with the entry (fence between observing and enqueueing)
    __threadfence();
    const int k = TK_DOWN;
    push(a, slot, &node, &k, 1, ch, sl);
  }
}

// F of both children of p (chunk ch) is final (thread 0, after the block's
// barrier and a fence): both counter updates are in flight together and the
// queue slots are taken with one atomic.
__device__ void release_children(const PmvArgs& a, int slot, const Slot& sl, const Node& p, int ch) {
  const int cs[2] = {p.left, p.right};
  int old[2];
  for (int i = 0; i < 2; ++i) old[i] = atomicAdd(counter(sl, cs[i], ch), 1);
  int go[2], kd[2] = {TK_DOWN, TK_DOWN}, np = 0;
  for (int i = 0; i < 2; ++i)
    if (old[i] & 1) go[np++] = cs[i];
  if (np == 0) return;
  __threadfence();   // as in node_event: the other events' writes go out with the entries
  push(a, slot, go, kd, np, ch, sl);
}

// ---- staging into shared memory ---------------------------------------------

// Asynchronous 8-byte copies global -> shared (cp.async), all of a phase in
// flight at once.  Only for data that no block writes during the launch (the
// generators): the copies go through L1.
__device__ __forceinline__ void cp8(void* s, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(s)), "l"(g)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// rows x cols column-major block (global ld ldg) into shared memory (ld lds):
// warps take columns, lanes rows.
template <class E>
__device__ __forceinline__ void stage_gen(E* s, int lds, const E* g, int64_t ldg, int rows, int cols) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c = w; c < cols; c += PT / 32)
    for (int l = lane; l < rows; l += 32) cp8(s + l + c * lds, g + l + (int64_t)c * ldg);
}

// The same for workspace blocks written by other blocks of this launch: loads
// that bypass L1 (an SM may hold a stale line of a neighbouring block).
template <class E>
__device__ __forceinline__ void stage_ws(E* s, int lds, const E* g, int64_t ldg, int rows, int cols) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c = w; c < cols; c += PT / 32)
    for (int l = lane; l < rows; l += 32) s[l + c * lds] = __ldcg(g + l + (int64_t)c * ldg);
}

// ---- per-node work (one column chunk: columns j0 .. j0 + nc - 1) -------------

// Split-K layout of a small product over the block: op output slots (a power
// of two >= min(nout, PT)) x G = PT / op groups of terms.
__device__ __forceinline__ int out_slots(int nout) {
  int op = 1;
  while (op < nout && op < PT) op <<= 1;
  return op;
}

// The terms of one output of a small product: at most two strided segments,
// sum_{l < k1} a1[l sa1] b1[l sb1] + sum_{l < k2} a2[l sa2] b2[l sb2].  The
// call sites form the segment pointers once per output, so the inner loops
// hold no index arithmetic.
template <class E>
struct Terms {
  const E* a1;
  const E* b1;
  int sa1, sb1, k1;
  const E* a2;
  const E* b2;
  int sa2, sb2, k2;
};

template <class E>
__device__ __forceinline__ Terms<E> terms1(const E* a, int sa, const E* b, int sb, int k) {
  return Terms<E>{a, b, sa, sb, k, nullptr, nullptr, 0, 0, 0};
}

// acc[0..3] += the segment's terms l = g, g + G, ...: four independent chains
template <class P>
__device__ __forceinline__ void seg_acc(typename P::Acc (&acc)[4], const typename P::E* a, int sa,
                                        const typename P::E* b, int sb, int k, int g, int G) {
  int l = g;
  for (; l + 3 * G < k; l += 4 * G) {
    P::fma(acc[0], a[l * sa], b[l * sb]);
    P::fma(acc[1], a[(l + G) * sa], b[(l + G) * sb]);
    P::fma(acc[2], a[(l + 2 * G) * sa], b[(l + 2 * G) * sb]);
    P::fma(acc[3], a[(l + 3 * G) * sa], b[(l + 3 * G) * sb]);
  }
  for (; l < k; l += G) P::fma(acc[0], a[l * sa], b[l * sb]);
}

// out(o) = the sum of terms(o) for o < nout with every thread taking part (at
// most gmax groups of terms per output); epi(o, sum) consumes each result.
// `part` holds PT accumulators.
template <class P, class Setup, class Epi>
__device__ void sdot(int nout, typename P::Acc* part, Setup terms, Epi epi, int gmax = PT) {
  using Acc = typename P::Acc;
  const int op = max(out_slots(nout), PT / gmax), G = PT / op;
  const int slot = threadIdx.x % op, g = threadIdx.x / op;
  for (int o0 = 0; o0 < nout; o0 += op) {
    const int o = o0 + slot;
    Acc acc = P::zero();
    if (o < nout) {
      const Terms<typename P::E> t = terms(o);
      Acc a4[4] = {P::zero(), P::zero(), P::zero(), P::zero()};
      if (t.k1 > 0) seg_acc<P>(a4, t.a1, t.sa1, t.b1, t.sb1, t.k1, g, G);
      if (t.k2 > 0) seg_acc<P>(a4, t.a2, t.sa2, t.b2, t.sb2, t.k2, g, G);
      P::acc(a4[0], a4[1]);
      P::acc(a4[2], a4[3]);
      P::acc(a4[0], a4[2]);
      acc = a4[0];
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
// (ld LCH + 1) through two buffers, the next pass's copies in flight while one
// is used; thread (output slot, group) keeps its partial sums over the passes.
// zsm (nullable, at least kv x nc elements, may overlay the V buffers) also
// receives Z (ld kv).
template <class P>
__device__ void leaf_up(const Slot& sl, const Node& nd, int j0, int nc, typename P::Acc* part,
                        typename P::E* sm, typename P::E* zsm = nullptr) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  const int n = nd.gn, kv = nd.kv;
  if (kv == 0 || nc <= 0) return;
  const E* V = P::gen(sl, nd.V);
  E* ws = P::ws(sl);
  E* Xs = sm;                                      // n x RC
  E* Vb[2] = {sm + n * RC, sm + n * RC + (LCH + 1) * kv};   // LCH x kv each, ld LCH + 1
  const int npass = (n + LCH - 1) / LCH;
  auto issue = [&](int ps) {
    const int l0 = ps * LCH;
    stage_gen(Vb[ps & 1], LCH + 1, V + l0, n, min(LCH, n - l0), kv);
    cp_commit();
  };
  issue(0);
  if (npass > 1) issue(1);
  const int nout = kv * nc, op = out_slots(nout), G = PT / op;
  const int slot = threadIdx.x % op, g = threadIdx.x / op;
  const double* X = sl.B + nd.col0 + (int64_t)j0 * sl.ldb;
  {
    // four loads of a lane in flight before their conversions
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = w; q < nc; q += PT / 32)
      for (int l0 = 0; l0 < n; l0 += 128) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = l0 + lane + 32 * u;
          v[u] = l < n ? __ldg(X + l + (int64_t)q * sl.ldb) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = l0 + lane + 32 * u;
          if (l < n) Xs[l + q * n] = P::xin(v[u]);
        }
      }
  }
  // nout <= 512 = 2 PT outputs per thread slot; four accumulator chains each
  Acc acc4[2][4];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc4[s][c] = P::zero();
  for (int ps = 0; ps < npass; ++ps) {
    const int l0 = ps * LCH, nl = min(LCH, n - l0);
    const E* Vs = Vb[ps & 1];
    if (ps + 1 < npass) cp_wait<1>();
    else cp_wait<0>();
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int o = s * op + slot;
      if (o < nout) {
        const int c = o % kv, q = o / kv;
        seg_acc<P>(acc4[s], Vs + c * (LCH + 1), 1, Xs + l0 + q * n, 1, nl, g, G);
      }
    }
    if (ps + 2 < npass) {
      __syncthreads();   // every thread is done with this buffer
      issue(ps + 2);
    }
  }
  if (zsm != nullptr) __syncthreads();   // every thread is done with the V buffers
  Acc acc[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    P::acc(acc4[s][0], acc4[s][1]);
    P::acc(acc4[s][2], acc4[s][3]);
    P::acc(acc4[s][0], acc4[s][2]);
    acc[s] = acc4[s][0];
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
    if (g == 0 && o < nout) {
      const E z = P::fin(acc[s]);
      ws[nd.wz + (o % kv) + (int64_t)(j0 + o / kv) * sl.ldws] = z;
      if (zsm != nullptr) zsm[o] = z;
    }
  }
}

// Climb step at a non-root branch p once both children's Z are final:
// Z_p = W1^T Z1 + W2^T Z2 (matmul.jl:39).  The children's sizes and offsets come
// from p's descriptor (here a copy in shared memory).
template <class P>
__device__ void z_node(const Slot& sl, const Node& p, int j0, int nc, typename P::Acc* part, typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  const int v1 = p.ckv[0], v2 = p.ckv[1], kv = p.kv;
  if (nc <= 0 || kv == 0) return;
  E* ws = P::ws(sl);
  const int64_t ld = sl.ldws;
  // W1, W2 column-major with odd leading dimensions (lanes take columns in the product)
  const int ld1 = v1 | 1, ld2 = v2 | 1;
  E* Z1 = sm;
  E* Z2 = Z1 + v1 * RC;
  E* W1s = Z2 + v2 * RC;
  E* W2s = W1s + ld1 * kv;
  stage_gen(W1s, ld1, P::gen(sl, p.W1), v1, v1, kv);
  stage_gen(W2s, ld2, P::gen(sl, p.W2), v2, v2, kv);
  cp_commit();
  stage_ws(Z1, v1, ws + p.cwz[0] + (int64_t)j0 * ld, ld, v1, nc);
  stage_ws(Z2, v2, ws + p.cwz[1] + (int64_t)j0 * ld, ld, v2, nc);
  cp_wait<0>();
  __syncthreads();
  sdot<P>(kv * nc, part,
          [&](int o) {
            const int c = o % kv, q = o / kv;
            return Terms<E>{W1s + c * ld1, Z1 + q * v1, 1, 1, v1, W2s + c * ld2, Z2 + q * v2, 1, 1, v2};
          },
          [&](int o, const Acc& s) { ws[p.wz + (o % kv) + (int64_t)(j0 + o / kv) * ld] = P::fin(s); });
}

// B-terms of branch p's children, G1 = B12 Z2 and G2 = B21 Z1 (matmul.jl:51,
// :55), into the children's F slots.  Off the upsweep's critical path: a queue
// task (the root's inline, its children's downsweep waits for them).
template <class P>
__device__ void bterm_node(const Slot& sl, const Node& p, int j0, int nc, typename P::Acc* part,
                           typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  if (nc <= 0) return;
  const int v1 = p.ckv[0], v2 = p.ckv[1], u1 = p.cku[0], u2 = p.cku[1];
  E* ws = P::ws(sl);
  const int64_t ld = sl.ldws;
  E* Z1 = sm;
  E* Z2 = Z1 + v1 * RC;
  E* B12 = Z2 + v2 * RC;
  E* B21 = B12 + u1 * v2;
  stage_gen(B12, u1, P::gen(sl, p.B12), u1, u1, v2);
  stage_gen(B21, u2, P::gen(sl, p.B21), u2, u2, v1);
  cp_commit();
  stage_ws(Z1, v1, ws + p.cwz[0] + (int64_t)j0 * ld, ld, v1, nc);
  stage_ws(Z2, v2, ws + p.cwz[1] + (int64_t)j0 * ld, ld, v2, nc);
  cp_wait<0>();
  __syncthreads();
  sdot<P>((u1 + u2) * nc, part,
          [&](int o) {
            if (o < u1 * nc) return terms1<E>(B12 + o % u1, u1, Z2 + (o / u1) * v2, 1, v2);
            const int o2 = o - u1 * nc;
            return terms1<E>(B21 + o2 % u2, u2, Z1 + (o2 / u2) * v1, 1, v1);
          },
          [&](int o, const Acc& s) {
            if (o < u1 * nc) ws[p.cwf[0] + (o % u1) + (int64_t)(j0 + o / u1) * ld] = P::fin(s);
            else ws[p.cwf[1] + ((o - u1 * nc) % u2) + (int64_t)(j0 + (o - u1 * nc) / u2) * ld] = P::fin(s);
          });
}

// Arrival of a finished node x (its Z of chunk ch written by this block) at its
// parent; the second child to arrive climbs.  While thread 0 fences and
// arrives, warp 1 enqueues the B-term task of x (a branch) and warp 2 copies
// the parent's descriptor into shared memory, so the next step reads no
// descriptor from global memory.  At the root the block forms the root's
// B-terms, which are F of the root's children, and releases them.
template <class P>
__device__ void climb_from(const PmvArgs& a, int slot, const Slot& sl, const Node* nodes, int node, int ch,
                           typename P::Acc* part, typename P::E* sm) {
  __shared__ int s_go;
  __shared__ Node s_node;
  const int j0 = ch * a.cw, nc = min(a.cw, sl.r - j0);
  const Node* x = &nodes[node];
  for (;;) {
    const int xpar = x->parent;
    const bool xroot = x->root != 0, xbranch = !x->leaf;
    __syncthreads();   // x's Z is written; nobody reads s_node any more
    if (xroot) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
      __threadfence();   // publishes the block's writes (cumulative over the barrier)
      const int old = atomicAdd(counter(sl, xpar, ch), 1);
      s_go = old & 1;
      if (old & 1) __threadfence();   // acquire: the sibling's Z is read after the barrier below
    } else if (threadIdx.x == 32 && xbranch) {
      __threadfence();
      const int k = TK_BTERM;
      push(a, slot, &node, &k, 1, ch, sl);
    } else if (w == 2) {
      const unsigned long long* src = (const unsigned long long*)&nodes[xpar];
      unsigned long long* dst = (unsigned long long*)&s_node;
      for (int i = lane; i < (int)(sizeof(Node) / 8); i += 32) dst[i] = src[i];
    }
    __syncthreads();
    if (!s_go) return;
    const Node& p = s_node;
    node = xpar;
    if (p.root) {
      bterm_node<P>(sl, p, j0, nc, part, sm);
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        release_children(a, slot, sl, p, ch);
      }
      return;
    }
    z_node<P>(sl, p, j0, nc, part, sm);
    x = &s_node;
  }
}

// Downsweep task of a non-root branch p (F_p final, its children's B-terms G_c
// done): F_c = G_c + R_c F_p for both children (matmul.jl:50-56), in place over G_c.
template <class P>
__device__ void down_node(const Slot& sl, const Node& p, int j0, int nc, typename P::Acc* part, typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  if (nc <= 0) return;
  const int u1 = p.cku[0], u2 = p.cku[1], kp = p.ku;
  const int64_t f1 = p.cwf[0], f2 = p.cwf[1];
  E* ws = P::ws(sl);
  const int64_t ld = sl.ldws;
  E* Fp = sm;                 // kp x RC
  E* R1 = Fp + kp * RC;       // u1 x kp
  E* R2 = R1 + u1 * kp;       // u2 x kp
  E* G1 = R2 + u2 * kp;       // u1 x RC: the children's B-terms
  E* G2 = G1 + u1 * RC;       // u2 x RC
  stage_gen(R1, u1, P::gen(sl, p.R1), u1, u1, kp);
  stage_gen(R2, u2, P::gen(sl, p.R2), u2, u2, kp);
  cp_commit();
  stage_ws(Fp, kp, ws + p.wf + (int64_t)j0 * ld, ld, kp, nc);
  stage_ws(G1, u1, ws + f1 + (int64_t)j0 * ld, ld, u1, nc);
  stage_ws(G2, u2, ws + f2 + (int64_t)j0 * ld, ld, u2, nc);
  cp_wait<0>();
  __syncthreads();
  sdot<P>((u1 + u2) * nc, part,
          [&](int o) {
            if (o < u1 * nc) return terms1<E>(R1 + o % u1, u1, Fp + (o / u1) * kp, 1, kp);
            const int o2 = o - u1 * nc;
            return terms1<E>(R2 + o2 % u2, u2, Fp + (o2 / u2) * kp, 1, kp);
          },
          [&](int o, const Acc& s) {
            const bool first = o < u1 * nc;
            const int o2 = first ? o : o - u1 * nc;
            const int uc = first ? u1 : u2;
            Acc t = s;
            P::addE(t, (first ? G1 : G2)[o2]);   // G[i + q uc] with i = o2 % uc, q = o2 / uc
            ws[(first ? f1 : f2) + (o2 % uc) + (int64_t)(j0 + o2 / uc) * ld] = P::fin(t);
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
  if (ch == 0 && !nd.root && nd.ku > 0) {
    // U is read by the leaf's final tasks at the end of the downsweep: into L2 now
    const char* ub = (const char*)P::gen(sl, nd.U);
    const int64_t bytes = (int64_t)nd.gm * nd.ku * (int64_t)sizeof(E);
    for (int64_t off = (int64_t)threadIdx.x * 128; off < bytes; off += PT * 128)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(ub + off));
  }
  constexpr bool pairs_e = !std::is_same<E, double>::value;
  if (j0 < sl.r && !(pairs_e && a.dx_ready && !nd.root)) {
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
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      node_event(a, tk.slot, sl, tk.node, ch);
    }
  }
}

// Final task of a non-root leaf chunk (F final, bulk done): C += alpha U F
// (matmul.jl:47), or for pairs C = alpha (D B + U F) + beta Y, with the column
// sums of squares.  Thread (row ii, group g) takes the columns of group g
// whole (no split over K, no cross-thread sums), FQ at a time, and loads
// its epilogue operands (D B, Y, or C) before the product, so that their
// latency overlaps the loop over U's columns.
template <class P>
__device__ void final_leaf(const Slot& sl, const Node& nd, int j0, int nc, typename P::Acc* part,
                           typename P::E* sm) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  constexpr bool pairs = !std::is_same<E, double>::value;
  constexpr int FQ = 2;   // columns per pass (registers: the launch allows 64 per thread)
  (void)part;
  if (nc <= 0) return;
  const int m = nd.gm, ku = nd.ku;
  E* ws = P::ws(sl);
  E* Fs = sm;                              // ku x RC
  const E* U = P::gen(sl, nd.U);
  __syncthreads();
  stage_ws(Fs, ku, ws + nd.wf + (int64_t)j0 * sl.ldws, sl.ldws, ku, nc);
  __syncthreads();
  double* C = sl.C + nd.row0 + (int64_t)j0 * sl.ldc;
  double* cn = sl.colnorm2 ? sl.colnorm2 + j0 : nullptr;
  const E* T = pairs ? (const E*)sl.tmp + nd.row0 + (int64_t)j0 * sl.ldt2 : nullptr;
  const double* Y = sl.Y ? sl.Y + nd.row0 + (int64_t)j0 * sl.ldy : nullptr;
  const bool yterm = pairs && sl.beta != 0.0 && Y != nullptr;
  const int tid = threadIdx.x;
  for (int r0 = 0; r0 < m; r0 += PT) {
    const int rows = min(PT, m - r0);
    int rp = 1;
    while (rp < rows) rp <<= 1;
    const int G = PT / rp, ii = tid % rp, g = tid / rp;
    const int i = r0 + ii;
    const int cpg = (nc + G - 1) / G, q0 = g * cpg, q1 = min(nc, q0 + cpg);
    for (int qb = q0; qb < q1; qb += FQ) {
      const int nq = min(FQ, q1 - qb);
      const bool act = ii < rows;
      // epilogue operands first
      E tv[FQ];
      double yv[FQ];
#pragma unroll
      for (int q = 0; q < FQ; ++q) {
        tv[q] = E{};
        yv[q] = 0.0;
        if (act && q < nq) {
          if (pairs) {
            tv[q] = __ldcg(T + i + (int64_t)(qb + q) * sl.ldt2);
            if (yterm) yv[q] = __ldcg(Y + i + (int64_t)(qb + q) * sl.ldy);
          } else {
            yv[q] = __ldcg(C + i + (int64_t)(qb + q) * sl.ldc);
          }
        }
      }
      Acc acc[FQ];
#pragma unroll
      for (int q = 0; q < FQ; ++q) acc[q] = P::zero();
      if (act) {
        const E* a = U + i;
#pragma unroll 8
        for (int l = 0; l < ku; ++l) {
          const E d = __ldg(a + (int64_t)l * m);
#pragma unroll
          for (int q = 0; q < FQ; ++q)
            if (q < nq) P::fma(acc[q], d, Fs[l + (qb + q) * ku]);
        }
      }
#pragma unroll
      for (int q = 0; q < FQ; ++q) {
        double v = 0.0;
        if (act && q < nq) {
          if (pairs) {
            Acc t = acc[q];
            P::addE(t, tv[q]);
            v = sl.alpha * P::dbl(t);
            if (yterm) v += sl.beta * yv[q];
          } else {
            v = yv[q] + sl.alpha * P::dbl(acc[q]);
          }
          C[i + (int64_t)(qb + q) * sl.ldc] = v;
        }
        if (cn != nullptr) {
          // a warp lies within one group when rp >= 32: warp sums, one atomic per column
          double v2 = v * v;
          if (rp >= 32) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v2 += __shfl_xor_sync(0xffffffffu, v2, o);
            if ((tid & 31) == 0 && q < nq && v2 != 0.0) atomicAdd(cn + qb + q, v2);
          } else if (q < nq && v2 != 0.0) {
            atomicAdd(cn + qb + q, v2);
          }
        }
      }
    }
  }
}

template <class P>
__global__ void __launch_bounds__(PT, 4) pmv_kernel(PmvArgs a) {
  using E = typename P::E;
  using Acc = typename P::Acc;
  extern __shared__ __align__(16) unsigned char pmv_smem[];
  constexpr bool pairs_k = !std::is_same<E, double>::value;
  Acc* part = (Acc*)pmv_smem;                    // PART_ELEMS split-K partials
  E* sm = (E*)pmv_smem + PART_ELEMS;             // per-phase staging
  __shared__ int s_cmd, s_x, s_y, s_k;

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
      if (ticket >= 0) {
        const unsigned long long w = *(const volatile unsigned long long*)&a.qent[ticket];
        if ((uint32_t)(w >> QE_EPOCH) == a.epoch) {
          __threadfence();   // acquire: the task's inputs are read after the barrier below
          s_x = (int)((w >> QE_SLOT) & 0xffffu);
          s_y = (int)(w & ((1u << QE_SLOT) - 1));   // node * kSyncChunks + chunk
          s_k = (int)((w >> QE_KIND) & 1u);
          cmd = 1;
          ticket = -1;
        }
      }
      if (cmd == 0) {
        if (++idle > a.idle_limit) {
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
      if (s_k == TK_BTERM) {
        bterm_node<P>(sl, x, j0, nc, part, sm);
        __syncthreads();
        if (threadIdx.x == 0) {
          __threadfence();
          node_event(a, slot, sl, node, ch);
        }
      } else if (x.leaf) {
        // with the leaf products outside the launch (leaf_ext), the final
        // products C = alpha (D B + U F) + beta Y follow it (leaf_uf_kernel)
        if (!(pairs_k && a.leaf_ext)) final_leaf<P>(sl, x, j0, nc, part, sm);
      } else {
        down_node<P>(sl, x, j0, nc, part, sm);
        __syncthreads();
        if (threadIdx.x == 0) {
          __threadfence();
          release_children(a, slot, sl, x, ch);
        }
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
          // leaf_ext: Z = V^T B is already in the workspace (leaf_vtx_kernel)
          if (!(pairs_k && a.leaf_ext)) leaf_up<P>(sl, nd, j0, min(a.cw, sl.r - j0), part, sm);
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

// ---- leaf products of the double-float residual outside the persistent launch ----
//
// With the leaf blocks D X on the tensor cores (dx_tc_kernel), the other two
// leaf products of the residual are streamed over all leaves at the width of
// 32 columns, before and after the tree part: Z = V^T X into the workspace
// (matmul.jl:34) and C = alpha (D X + U F) + beta Y with the column sums of
// squares (:46-47).  Each block stages its leaf's generator block and column
// block once in shared memory; a thread keeps two outputs of one row (V^T X)
// or four of one row (U F) with their own accumulator chains.

constexpr int XW = 32;   // columns per block of the leaf kernels
constexpr int LB = 16;   // global loads in flight per thread while a block stages its operands

__device__ void leaf_vtx_unit(const Task tk, const Slot* __restrict__ slots, int cb) {
  extern __shared__ __align__(16) unsigned char ext_smem[];
  using P = PDF;
  using Acc = P::Acc;
  const Slot& sl = slots[tk.slot];
  const Node& nd = tk.nodes[tk.node];
  const int j0 = cb * XW;
  if (nd.root || nd.kv == 0 || j0 >= sl.r) return;
  const int n = nd.gn, kv = nd.kv, nc = min(XW, sl.r - j0);
  const int ld = n | 1;             // odd: a warp's rows c (or columns q) fall in distinct bank pairs
  float2* Vs = (float2*)ext_smem;   // n x kv, ld ld
  float2* Xs = Vs + ld * kv;        // n x nc, ld ld
  // staging: LB loads in flight per thread before the shared-memory stores
  const float2* V = P::gen(sl, nd.V);
  for (int e0 = threadIdx.x; e0 < n * kv; e0 += LB * PT) {
    float2 v[LB];
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int e = e0 + u * PT;
      v[u] = e < n * kv ? __ldg(V + e) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int e = e0 + u * PT;
      if (e < n * kv) Vs[e % n + (e / n) * ld] = v[u];
    }
  }
  const double* X = sl.B + nd.col0 + (int64_t)j0 * sl.ldb;
  for (int e0 = threadIdx.x; e0 < n * nc; e0 += LB * PT) {
    double v[LB];
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int e = e0 + u * PT;
      v[u] = e < n * nc ? __ldg(X + e % n + (int64_t)(e / n) * sl.ldb) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int e = e0 + u * PT;
      if (e < n * nc) Xs[e % n + (e / n) * ld] = split_bits(v[u]);
    }
  }
  __syncthreads();
  float2* ws = sl.ws2;
  // 2 x 2 tiles: rows c, c + hc of Z, columns q, q + hq
  const int hc = (kv + 1) / 2, hq = (nc + 1) / 2;
  for (int it = threadIdx.x; it < hc * hq; it += PT) {
    const int c = it % hc, q = it / hc;
    const int c2 = c + hc < kv ? c + hc : c, q2 = q + hq < nc ? q + hq : q;
    const float2* va = Vs + c * ld;
    const float2* vb = Vs + c2 * ld;
    const float2* xa = Xs + q * ld;
    const float2* xb = Xs + q2 * ld;
    Acc s00 = P::zero(), s01 = P::zero(), s10 = P::zero(), s11 = P::zero();
#pragma unroll 2
    for (int l = 0; l < n; ++l) {
      const float2 a0 = va[l], a1 = vb[l], b0 = xa[l], b1 = xb[l];
      P::fma(s00, a0, b0);
      P::fma(s01, a0, b1);
      P::fma(s10, a1, b0);
      P::fma(s11, a1, b1);
    }
    ws[nd.wz + c + (int64_t)(j0 + q) * sl.ldws] = P::fin(s00);
    if (q2 != q) ws[nd.wz + c + (int64_t)(j0 + q2) * sl.ldws] = P::fin(s01);
    if (c2 != c) ws[nd.wz + c2 + (int64_t)(j0 + q) * sl.ldws] = P::fin(s10);
    if (c2 != c && q2 != q) ws[nd.wz + c2 + (int64_t)(j0 + q2) * sl.ldws] = P::fin(s11);
  }
}

__device__ void leaf_uf_unit(const Task tk, const Slot* __restrict__ slots, int cb) {
  extern __shared__ __align__(16) unsigned char ext_smem[];
  using P = PDF;
  using Acc = P::Acc;
  const Slot& sl = slots[tk.slot];
  const Node& nd = tk.nodes[tk.node];
  const int j0 = cb * XW;
  if (nd.root || j0 >= sl.r) return;
  const int m = nd.gm, ku = nd.ku, nc = min(XW, sl.r - j0);
  float2* Us = (float2*)ext_smem;   // m x ku, ld m
  float2* Fs = Us + m * ku;         // ku x nc, ld ku
  if (ku > 0) {
    const float2* U = P::gen(sl, nd.U);
    for (int e0 = threadIdx.x; e0 < m * ku; e0 += LB * PT) {
      float2 v[LB];
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int e = e0 + u * PT;
        v[u] = e < m * ku ? __ldg(U + e) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int e = e0 + u * PT;
        if (e < m * ku) Us[e] = v[u];
      }
    }
    const float2* F = sl.ws2 + nd.wf + (int64_t)j0 * sl.ldws;
    for (int e0 = threadIdx.x; e0 < ku * nc; e0 += LB * PT) {
      float2 v[LB];
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int e = e0 + u * PT;
        v[u] = e < ku * nc ? __ldcg(F + e % ku + (int64_t)(e / ku) * sl.ldws) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int e = e0 + u * PT;
        if (e < ku * nc) Fs[e] = v[u];
      }
    }
  }
  __syncthreads();
  const float2* T = (const float2*)sl.tmp + nd.row0 + (int64_t)j0 * sl.ldt2;
  const double* Y = sl.Y ? sl.Y + nd.row0 + (int64_t)j0 * sl.ldy : nullptr;
  const bool yterm = sl.beta != 0.0 && Y != nullptr;
  double* C = sl.C + nd.row0 + (int64_t)j0 * sl.ldc;
  double* cn = sl.colnorm2 ? sl.colnorm2 + j0 : nullptr;
  const int tid = threadIdx.x, lane = tid & 31;
  // a warp takes 32 consecutive rows and, per pass, 4 columns (each thread
  // 2 rows 32 apart x 4 columns: 8 accumulator chains); warps cycle through
  // (row block, column block) pairs
  const int nrb = (m + 63) / 64, ncb = (nc + 3) / 4;
  for (int job = tid >> 5; job < nrb * ncb; job += PT / 32) {
    const int rb = job % nrb, cb = job / nrb;
    const int i0 = rb * 64 + lane, i1 = i0 + 32;
    const int qb = cb * 4, nq = min(4, nc - qb);
    const bool a0 = i0 < m, a1 = i1 < m;
    Acc acc0[4] = {P::zero(), P::zero(), P::zero(), P::zero()};
    Acc acc1[4] = {P::zero(), P::zero(), P::zero(), P::zero()};
    const float2* f = Fs + qb * ku;
#pragma unroll 2
    for (int l = 0; l < ku; ++l) {
      const float2 u0 = a0 ? Us[i0 + l * m] : make_float2(0.f, 0.f);
      const float2 u1 = a1 ? Us[i1 + l * m] : make_float2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float2 fq = q < nq ? f[l + q * ku] : make_float2(0.f, 0.f);
        P::fma(acc0[q], u0, fq);
        P::fma(acc1[q], u1, fq);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      double v2 = 0.0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = h ? i1 : i0;
        if ((h ? a1 : a0) && q < nq) {
          Acc t = h ? acc1[q] : acc0[q];
          P::addE(t, __ldcg(T + i + (int64_t)(qb + q) * sl.ldt2));
          double v = sl.alpha * P::dbl(t);
          if (yterm) v += sl.beta * __ldcg(Y + i + (int64_t)(qb + q) * sl.ldy);
          C[i + (int64_t)(qb + q) * sl.ldc] = v;
          v2 = fma(v, v, v2);
        }
      }
      if (cn != nullptr) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v2 += __shfl_xor_sync(0xffffffffu, v2, o);
        if (lane == 0 && q < nq && v2 != 0.0) atomicAdd(cn + qb + q, v2);
      }
    }
  }
}

// Units (leaf, block of XW columns) taken in turn by a grid of resident blocks,
// so that the last wave is not a partial one.  The final products fit four
// blocks per SM (64 registers, 40 KB of shared memory at k = 32), so 512
// leaves take one round instead of two.
template <bool FINAL>
__global__ void __launch_bounds__(PT, (FINAL ? 4 : 2)) leaf_ext_kernel(const Task* __restrict__ leaves, const Slot* __restrict__ slots,
                                                      int nunits, int ncb) {
  for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
    const Task tk = leaves[u / ncb];
    if (FINAL) leaf_uf_unit(tk, slots, u % ncb);
    else leaf_vtx_unit(tk, slots, u % ncb);
    __syncthreads();   // the shared buffers are reused by the next unit
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

// ---- flat product (FP64, few right-hand sides) ------------------------------
//
// The queued product above hands every tree node from block to block, so its
// time is the tree's chain of hand-offs (two per level).  With few columns the
// small products are cheap next to that chain, and the flat product trades
// them for it: every leaf carries its own chain of translator products, and
// the launch has three phases, each starting once every unit of the one
// before it has finished (a count of finished units, not a grid barrier).
//
//   A. per leaf, Z = V^T B (matmul.jl:34), the B-term that Z feeds
//      (G_sibling = B Z, :51/:55), and the leaf's contributions to its
//      ancestors' Z, W_a^T ... W_x^T Z (the terms of :39 unrolled);
//   B. per non-root branch p, Z_p = the sum of its leaves' contributions (in
//      leaf order, so the result does not depend on the schedule), then the
//      B-term it feeds;
//   C. per leaf, F along the root-to-leaf path, F_c = G_c + R_c F_p (:50-56,
//      F of the root's children = G), then C += alpha U F (:47).
//
// The leaf products C = alpha D B + beta Y (:46), per leaf and row piece, have
// no tree dependency: they are filler work, taken from their own counter by
// any block that waits for the next phase or finds its phase's list empty,
// and by a phase-C unit whose leaf still has pieces outstanding (a per-leaf
// counter of finished pieces orders the two writes of C).  The translators above a leaf
// are multiplied once per leaf below them instead of once, which costs FP64
// issue slots but no extra HBM traffic (they stay in L2).

constexpr int kFlatCw = 4;      // columns per chunk

struct FlatArgs {
  const Task* leaves;      // leaf list (a subtree's leaves are contiguous)
  const Task* branches;    // non-root branches by height, lowest first
  const FlatLink* links;   // by node index
  const int32_t* paths;    // leaf t's ancestor at depth d: paths[t * dep + d]
  const Slot* slots;
  uint32_t* state;
  double* ctb;             // contributions: ((depth * nleaves + leaf) * nchunk + chunk) * kw + (c + q kv)
  uint32_t* dcnt;          // finished leaf-product pieces per (leaf, chunk); zero between launches
  int32_t nleaves, nbranch, nchunk, npiece, dep, kmax, kw;
  int32_t rows;            // rows of a leaf's D per leaf-product unit
  uint32_t idle_limit;     // polls of a waiting block before DEV_TIMEOUT
};

using FA = PF64::Acc;

// A finished unit of phase A or B: its writes published, then counted.
__device__ void flat_finish(uint32_t* ctr) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctr, 1u);
  }
}

// Next unit of a phase, or -1 (uniform over the block).
__device__ int flat_claim(uint32_t* ctr, int n, int* s_u) {
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t u = (uint32_t)n;
    if (ld_vol(ctr) < (uint32_t)n) u = atomicAdd(ctr, 1u);
    *s_u = u < (uint32_t)n ? (int)u : -1;
  }
  __syncthreads();
  return *s_u;
}

// Copies the links of leaf t's path (depths 1 .. D) into shared memory.
__device__ void flat_path(const FlatArgs& a, int t, int D, FlatLink* lk) {
  constexpr int W = (int)(sizeof(FlatLink) / 8);
  for (int e = threadIdx.x; e < D * W; e += PT) {
    const int d = 1 + e / W, w = e % W;
    const int node = __ldg(a.paths + (int64_t)t * a.dep + d);
    ((unsigned long long*)&lk[d])[w] = __ldg((const unsigned long long*)&a.links[node] + w);
  }
  __syncthreads();
}

// The B-term that Z_x feeds (zs: kv x nc, ld kv), into the sibling's F slot.
__device__ void flat_bterm(const Slot& sl, const FlatLink& lk, const double* zs, int j0, int nc, FA* part) {
  const int ks = lk.sku, kv = lk.kv;
  const double* B = lk.B;
  double* ws = (double*)sl.ws;
  const int64_t ld = sl.ldws, off = lk.swf;
  sdot<PF64>(ks * nc, part,
             [&](int o) { return terms1<double>(B + o % ks, ks, zs + (o / ks) * kv, 1, kv); },
             [&](int o, const FA& s) { ws[off + (o % ks) + (int64_t)(j0 + o / ks) * ld] = s.s; }, 4);
}

// Phase A, upsweep unit of leaf t: Z, the B-term it feeds, and the chain of
// contributions t_{d-1} = W_d^T t_d up to depth 1, W staged one step ahead.
__device__ void flat_up(const FlatArgs& a, int t, int ch, FA* part, double* sm, FlatLink* lk) {
  const Task tk = a.leaves[t];
  const Slot& sl = a.slots[tk.slot];
  const Node& x = tk.nodes[tk.node];
  const int j0 = ch * kFlatCw, nc = min(kFlatCw, sl.r - j0);
  if (x.root || nc <= 0) return;
  const int D = x.depth;
  flat_path(a, t, D, lk);
  const int km = a.kmax, kk = km * kFlatCw;
  double* cur = sm + x.gn * RC;   // over leaf_up's V buffers
  double* nxt = cur + kk;
  double* const Wb = nxt + kk;   // two buffers of (km | 1) x km
  const int wstride = (km | 1) * km;
  leaf_up<PF64>(sl, x, j0, nc, part, sm, cur);
  auto stage_w = [&](int d, int b) {
    const FlatLink& L = lk[d];
    stage_gen(Wb + b * wstride, L.kv | 1, L.W, L.kv, L.kv, L.kpv);
    cp_commit();
  };
  __syncthreads();
  if (D >= 2) stage_w(D, 0);
  flat_bterm(sl, lk[D], cur, j0, nc, part);
  int buf = 0;
  for (int d = D; d >= 2; --d) {
    if (d > 2) {
      stage_w(d - 1, buf ^ 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const FlatLink& L = lk[d];
    const int ky = L.kv, kq = L.kpv, ldw = ky | 1;
    const double* Ws = Wb + buf * wstride;
    double* dst = a.ctb + ((int64_t)((d - 1) * a.nleaves + t) * a.nchunk + ch) * a.kw;
    sdot<PF64>(kq * nc, part,
               [&](int o) { return terms1<double>(Ws + (o % kq) * ldw, 1, cur + (o / kq) * ky, 1, ky); },
               [&](int o, const FA& s) {
                 nxt[o] = s.s;
                 dst[o] = s.s;
               },
               4);
    __syncthreads();
    double* tmp = cur;
    cur = nxt;
    nxt = tmp;
    buf ^= 1;
  }
}

// Leaf-product unit: rows pc * a.rows .. of C = alpha D B + beta Y
// (a single-leaf tree: the whole product, column norms included).
__device__ void flat_dpiece(const FlatArgs& a, int t, int pc, int ch, FA* part, double* Xs) {
  const Task tk = a.leaves[t];
  const Slot& sl = a.slots[tk.slot];
  const Node& nd = tk.nodes[tk.node];
  const int j0 = ch * kFlatCw, m = nd.gm, n = nd.gn, r0 = pc * a.rows;
  if (j0 >= sl.r || r0 >= m) return;
  const int nc = min(kFlatCw, sl.r - j0), mr = min(a.rows, m - r0);
  __syncthreads();
  const double* X = sl.B + nd.col0 + (int64_t)j0 * sl.ldb;
  for (int e = threadIdx.x; e < n * nc; e += PT) {
    const int l = e % n, q = e / n;
    Xs[l + q * n] = __ldg(X + l + (int64_t)q * sl.ldb);
  }
  __syncthreads();
  double* C = sl.C + nd.row0 + r0 + (int64_t)j0 * sl.ldc;
  const double* Y = sl.Y ? sl.Y + nd.row0 + r0 + (int64_t)j0 * sl.ldy : nullptr;
  const bool yterm = sl.beta != 0.0 && Y != nullptr;
  double* cn = (nd.root && sl.colnorm2) ? sl.colnorm2 + j0 : nullptr;
  rows_cols_n<PF64>(nd.D + r0, mr, n, m, Xs, n, nc, part, cn, [&](int i, int q, const FA& s) {
    double v = sl.alpha * s.s;
    if (yterm) v += sl.beta * __ldcg(Y + i + (int64_t)q * sl.ldy);
    C[i + (int64_t)q * sl.ldc] = v;
    return v;
  });
}

// Leaf-product unit u (leaf, piece, chunk), then its (leaf, chunk) counter.
__device__ void flat_dunit(const FlatArgs& a, int u, FA* part, double* sm) {
  const int per = a.npiece * a.nchunk, t = u / per, ch = u % a.nchunk;
  flat_dpiece(a, t, (u % per) / a.nchunk, ch, part, sm);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(&a.dcnt[t * a.nchunk + ch], 1u);
  }
}

// Runs leaf-product units until `done` holds (thread 0 evaluates it; the
// caller's acquire follows) or, with done = nullptr, until none are left.
// The wait for `done` is bounded: DEV_TIMEOUT, then the block goes on.
template <class Done>
__device__ void flat_fill(const FlatArgs& a, Done done, bool drain, FA* part, double* sm, int* s_u) {
  const int nd = a.nleaves * a.npiece * a.nchunk;
  uint32_t polls = 0;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      int cmd = -1;   // -2: finished, >= 0: a unit, -1: nothing to do yet
      if (!drain && done()) {
        cmd = -2;
      } else if (ld_vol(&a.state[FL_D]) < (uint32_t)nd) {
        const uint32_t u = atomicAdd(&a.state[FL_D], 1u);
        if (u < (uint32_t)nd) cmd = (int)u;
      }
      if (cmd == -1) {
        if (drain) {
          cmd = -2;
        } else if (++polls > a.idle_limit) {
          set_err(a.slots[0], DEV_TIMEOUT);
          cmd = -2;
        } else {
          __nanosleep(64);
        }
      }
      *s_u = cmd;
    }
    __syncthreads();
    const int cmd = *s_u;
    if (cmd == -2) break;
    if (cmd >= 0) flat_dunit(a, cmd, part, sm);
  }
  if (threadIdx.x == 0) __threadfence();   // acquire
  __syncthreads();
}

// Phase B unit: Z of branch bi from its leaves' contributions, then its B-term.
__device__ void flat_z(const FlatArgs& a, int bi, int ch, FA* part, double* sm) {
  const Task tk = a.branches[bi];
  const Slot& sl = a.slots[tk.slot];
  const FlatLink lk = a.links[tk.node];
  const int j0 = ch * kFlatCw, nc = min(kFlatCw, sl.r - j0);
  if (nc <= 0) return;
  double* zs = sm;
  // the leaves' contributions are consecutive blocks of kw (ld nchunk kw); the
  // block sums them with eight loads in flight per thread
  const int64_t lstride = (int64_t)a.nchunk * a.kw;
  const double* src = a.ctb + ((int64_t)(lk.depth * a.nleaves + lk.lf0) * a.nchunk + ch) * a.kw;
  const int nout = lk.kv * nc, op = out_slots(nout), G = PT / op;
  const int slot = threadIdx.x % op, g = threadIdx.x / op;
  for (int o0 = 0; o0 < nout; o0 += op) {
    const int o = o0 + slot;
    double acc = 0.0;
    if (o < nout) {
      for (int l0 = g; l0 < lk.lfn; l0 += 8 * G) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int l = l0 + u * G;
          v[u] = l < lk.lfn ? __ldcg(src + (int64_t)l * lstride + o) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) acc += v[u];
      }
    }
    if (G > 1) {
      __syncthreads();
      part[threadIdx.x].s = acc;
      __syncthreads();
      if (g == 0 && o < nout)
        for (int gg = 1; gg < G; ++gg) acc += part[gg * op + slot].s;
    }
    if (g == 0 && o < nout) zs[o] = acc;
  }
  __syncthreads();
  flat_bterm(sl, lk, zs, j0, nc, part);
}

// Phase C unit of leaf t: the G of every node on its path in one round of
// loads, F down the path with R staged one step ahead, then C += alpha U F.
__device__ void flat_down(const FlatArgs& a, int t, int ch, FA* part, double* sm, FlatLink* lk, int* s_u) {
  const Task tk = a.leaves[t];
  const Slot& sl = a.slots[tk.slot];
  const Node& x = tk.nodes[tk.node];
  const int j0 = ch * kFlatCw, nc = min(kFlatCw, sl.r - j0);
  if (x.root || nc <= 0) return;
  const int D = x.depth;
  flat_path(a, t, D, lk);
  const int km = a.kmax, kk = km * kFlatCw;   // every F / G block below has ld km
  double* Gs = sm;                            // depth d at Gs + d kk (d = 1 .. D)
  double* const Fb = Gs + (D + 1) * kk;   // two F buffers (kk each)
  double* const Rb = Gs + (D + 3) * kk;   // two R buffers (km x km each)
  auto stage_r = [&](int d, int b) {
    const FlatLink& L = lk[d];
    stage_gen(Rb + b * km * km, L.ku, L.R, L.ku, L.ku, L.kpu);
    cp_commit();
  };
  if (D >= 2) stage_r(2, 0);
  const double* ws = (const double*)sl.ws;
  const int64_t ld = sl.ldws;
  for (int e0 = threadIdx.x; e0 < D * kk; e0 += 4 * PT) {
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * PT;
      v[u] = 0.0;
      if (e < D * kk) {
        const FlatLink& L = lk[1 + e / kk];
        const int i = (e % kk) % km, q = (e % kk) / km;
        if (i < L.ku && q < nc) v[u] = __ldcg(ws + L.wf + i + (int64_t)(j0 + q) * ld);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (e0 + u * PT < D * kk) Gs[kk + e0 + u * PT] = v[u];
  }
  __syncthreads();
  const double* f = Gs + kk;   // F at depth 1 = G
  int buf = 0;
  for (int d = 2; d <= D; ++d) {
    if (d < D) {
      stage_r(d + 1, buf ^ 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const FlatLink& L = lk[d];
    const int kc = L.ku, kp = L.kpu;
    const double* Rs = Rb + buf * km * km;
    const double* G = Gs + d * kk;
    double* out = Fb + buf * kk;
    sdot<PF64>(kc * nc, part,
               [&](int o) { return terms1<double>(Rs + o % kc, kc, f + (o / kc) * km, 1, kp); },
               [&](int o, const FA& s) {
                 const int i = o % kc, q = o / kc;
                 out[i + q * km] = s.s + G[i + q * km];
               },
               4);
    __syncthreads();
    f = out;
    buf ^= 1;
  }
  // C holds alpha D B + beta Y once the leaf's pieces are done; help with them
  const uint32_t* cnt = a.dcnt + t * a.nchunk + ch;
  flat_fill(a, [&] { return ld_vol(cnt) >= (uint32_t)a.npiece; }, false, part, Rb, s_u);   // R buffers are free
  double* C = sl.C + x.row0 + (int64_t)j0 * sl.ldc;
  double* cn = sl.colnorm2 ? sl.colnorm2 + j0 : nullptr;
  rows_cols_n<PF64>(x.U, x.gm, x.ku, x.gm, f, km, nc, part, cn, [&](int i, int q, const FA& s) {
    const double v = __ldcg(C + i + (int64_t)q * sl.ldc) + sl.alpha * s.s;
    C[i + (int64_t)q * sl.ldc] = v;
    return v;
  });
}

__global__ void __launch_bounds__(PT, 4) pmv_flat_kernel(FlatArgs a) {
  extern __shared__ __align__(16) unsigned char pmv_smem[];
  FA* part = (FA*)pmv_smem;
  double* sm = (double*)pmv_smem + PART_ELEMS;
  __shared__ FlatLink s_lk[kFlatDep];
  __shared__ int s_u;
  const int nup = a.nleaves * a.nchunk, nb = a.nbranch * a.nchunk;
  for (;;) {   // A
    const int u = flat_claim(&a.state[FL_A], nup, &s_u);
    if (u < 0) break;
    flat_up(a, u / a.nchunk, u % a.nchunk, part, sm, s_lk);
    flat_finish(&a.state[FL_AFIN]);
  }
  // B starts once every A unit is done (not every block: blocks busy with a
  // leaf product join late)
  flat_fill(a, [&] { return ld_vol(&a.state[FL_AFIN]) >= (uint32_t)nup; }, false, part, sm, &s_u);
  for (;;) {   // B: branches, highest first (the longest sums)
    const int u = flat_claim(&a.state[FL_B], nb, &s_u);
    if (u < 0) break;
    flat_z(a, a.nbranch - 1 - u / a.nchunk, u % a.nchunk, part, sm);
    flat_finish(&a.state[FL_BFIN]);
  }
  flat_fill(a, [&] { return ld_vol(&a.state[FL_BFIN]) >= (uint32_t)nb; }, false, part, sm, &s_u);
  for (;;) {   // C
    const int u = flat_claim(&a.state[FL_C], nup, &s_u);
    if (u < 0) break;
    flat_down(a, u / a.nchunk, u % a.nchunk, part, sm, s_lk, &s_u);
  }
  flat_fill(a, [] { return true; }, true, part, sm, &s_u);   // the leaf products left
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_u = atomicAdd(&a.state[FL_DONE], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_u) {   // the last block out resets the counters
    for (int i = threadIdx.x; i < a.nleaves * a.nchunk; i += PT) a.dcnt[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
      a.state[FL_A] = 0;
      a.state[FL_B] = 0;
      a.state[FL_C] = 0;
      a.state[FL_D] = 0;
      a.state[FL_AFIN] = 0;
      a.state[FL_BFIN] = 0;
      __threadfence();
      a.state[FL_DONE] = 0;
    }
  }
}

int flat_resident_blocks(size_t smem, int device) {
  static Occ<PF64> cache[8];
  if (device < 0 || device >= 8) device = 0;
  Occ<PF64>& c = cache[device];
  if (c.smem == smem && c.blocks > 0) return c.blocks;
  if (smem > 48 * 1024) cudaFuncSetAttribute(pmv_flat_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pmv_flat_kernel, PT, smem) != cudaSuccess) return 0;
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
  const size_t up = (size_t)nleaf * RC + 2 * (size_t)(LCH + 1) * k;   // X + two V buffers
  const size_t bulk = (size_t)nleaf * RC;
  const size_t fin = k * RC;
  const size_t down = 3 * k * RC + 2 * k * k;                         // F_p, R1, R2, G1, G2
  const size_t climb = 2 * k * RC + 2 * (k | 1) * k;                  // Z1, Z2, W1, W2
  const size_t bterm = 2 * k * RC + 2 * k * k;                        // Z1, Z2, B12, B21
  const size_t total = PART_ELEMS + std::max(std::max(std::max(up, bulk), std::max(fin, down)), std::max(climb, bterm));
  if (mcap) *mcap = (int)(total - PART_ELEMS);
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
int64_t pmv_queue_entries(int64_t ntasks, int64_t ninner, int chunks) { return (ntasks + ninner) * chunks; }
int64_t pmv_state_words() { return ST_WORDS; }
uint32_t pmv_epoch_limit() { return (1u << (64 - QE_EPOCH)) - 1; }
bool pmv_queue_fits(int64_t nodes, int64_t slots) {
  return nodes <= (int64_t(1) << (QE_SLOT - QE_NODE)) && slots <= (int64_t(1) << (QE_EPOCH - QE_SLOT));
}
int pmv_sync_chunks() { return kSyncChunks; }
void pmv_set_poll_limit(uint32_t polls) { g_idle_limit = polls == 0 ? kIdleLimit : polls; }
uint32_t pmv_poll_limit() { return g_idle_limit; }

cudaError_t launch_pmv(bool pairs, const Task* leaves, int64_t nleaves, const Slot* slots, int64_t ntasks,
                       int64_t ninner, int rmax,
                       int nleaf, int kmax, uint32_t* state, unsigned long long* qent, uint32_t epoch,
                       const void* prefetch,
                       int64_t prefetch_bytes, int device, cudaStream_t st, bool dx_ready, bool leaf_ext) {
  if (nleaves <= 0) return cudaSuccess;
  const size_t smem = pmv_smem_elems(nleaf, kmax, nullptr) * 8;
  PmvArgs a;
  a.leaves = leaves;
  a.slots = slots;
  a.state = state;
  a.qent = qent;
  a.nleaves = (int32_t)nleaves;
  a.cw = pairs ? RC : 4;   // FP64: narrower chunks spread the slow FP64 work over more SMs
  a.nchunk = pmv_chunks(pairs, rmax);
  if (a.nchunk == 0) return cudaErrorInvalidValue;
  a.nbulk = (int32_t)(nleaves * a.nchunk);
  a.ntasks = (int32_t)pmv_queue_entries(ntasks, ninner, a.nchunk);
  a.epoch = epoch;
  a.pf = (const char*)prefetch;
  a.pf_bytes = prefetch ? prefetch_bytes : 0;
  a.idle_limit = g_idle_limit;
  a.dx_ready = (pairs && dx_ready) ? 1 : 0;
  a.leaf_ext = (pairs && leaf_ext) ? 1 : 0;
  void* args[] = {&a};
  const int cap = pairs ? resident_blocks<PDF>(smem, device) : resident_blocks<PF64>(smem, device);
  if (cap <= 0) return cudaErrorLaunchOutOfResources;
  // every block must be resident; more blocks than work units would only poll
  const unsigned grid = (unsigned)std::min<int64_t>(cap, std::max<int64_t>(1, 2 * (int64_t)a.nbulk));
  return pairs ? cudaLaunchCooperativeKernel((void*)pmv_kernel<PDF>, grid, PT, args, smem, st)
               : cudaLaunchCooperativeKernel((void*)pmv_kernel<PF64>, grid, PT, args, smem, st);
}


size_t pmv_flat_smem_elems(int nleaf, int kmax, int dep) {
  const size_t k = kmax > 0 ? kmax : 1, kk = k * kFlatCw;
  const size_t up = std::max((size_t)nleaf * RC + 2 * (size_t)(LCH + 1) * k,   // leaf_up
                             (size_t)nleaf * RC + 2 * kk + 2 * (k | 1) * k);   // the W chain
  const size_t down = (size_t)(dep + 2) * kk + std::max(2 * k * k, (size_t)nleaf * RC);   // G's, F, R buffers
                                                                                      // (or a leaf product)
  return PART_ELEMS + std::max(std::max(up, down), std::max((size_t)nleaf * RC, kk));
}

bool pmv_flat_fits(int nleaf, int kmax, int dep, int rmax) {
  return rmax >= 1 && rmax <= kFlatCw && dep >= 2 && dep <= kFlatDep && nleaf <= 512 && kmax <= 64 &&
         pmv_flat_smem_elems(nleaf, kmax, dep) * 8 <= 160 * 1024;
}

int64_t pmv_flat_chunks(int rmax) { return (std::max(rmax, 1) + kFlatCw - 1) / kFlatCw; }

int64_t pmv_flat_ctb_elems(int64_t nleaves, int dep, int kmax, int rmax) {
  const int64_t nchunk = (std::max(rmax, 1) + kFlatCw - 1) / kFlatCw;
  return std::max<int64_t>(1, nleaves * dep * nchunk * (int64_t)std::max(kmax, 1) * kFlatCw);
}

cudaError_t launch_pmv_flat(const Task* leaves, int64_t nleaves, const Task* branches, int64_t nbranch,
                            const FlatLink* links, const int32_t* paths, int dep, const Slot* slots, int rmax,
                            int nleaf, int mleaf, int kmax, uint32_t* state, double* ctb, uint32_t* dcnt,
                            int device, cudaStream_t st) {
  if (nleaves <= 0) return cudaSuccess;
  if (!pmv_flat_fits(nleaf, kmax, dep, rmax)) return cudaErrorInvalidValue;
  const size_t smem = pmv_flat_smem_elems(nleaf, kmax, dep) * 8;
  FlatArgs a;
  a.leaves = leaves;
  a.branches = branches;
  a.links = links;
  a.paths = paths;
  a.slots = slots;
  a.state = state;
  a.ctb = ctb;
  a.dcnt = dcnt;
  a.nleaves = (int32_t)nleaves;
  a.nbranch = (int32_t)nbranch;
  a.nchunk = (rmax + kFlatCw - 1) / kFlatCw;
  // pieces of 64 rows for one or two columns (fewer, longer units: 6 % faster
  // at r = 1 on n = 65536), 32 rows for three or four (better balance)
  a.rows = rmax <= 2 ? 64 : 32;
  a.npiece = (std::max(mleaf, 1) + a.rows - 1) / a.rows;
  a.dep = dep;
  a.kmax = std::max(kmax, 1);
  a.kw = a.kmax * kFlatCw;
  a.idle_limit = g_idle_limit;
  const int cap = flat_resident_blocks(smem, device);
  if (cap <= 0) return cudaErrorLaunchOutOfResources;
  const int64_t units = nleaves * a.nchunk * (1 + a.npiece);
  const unsigned grid = (unsigned)std::min<int64_t>(cap, std::max<int64_t>(1, units));
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((void*)pmv_flat_kernel, grid, PT, args, smem, st);
}

size_t leaf_ext_smem(int nleaf, int mleaf, int kmax) {
  const size_t up = ((size_t)(nleaf | 1) * kmax + (size_t)(nleaf | 1) * XW) * sizeof(float2);
  const size_t fin = ((size_t)mleaf * kmax + (size_t)kmax * XW) * sizeof(float2);
  return std::max(up, fin);
}

bool leaf_ext_fits(int nleaf, int mleaf, int kmax) { return leaf_ext_smem(nleaf, mleaf, kmax) <= 160 * 1024; }

cudaError_t launch_leaf_ext(bool final_part, const Task* leaves, int64_t nleaves, const Slot* slots, int rmax, int nleaf,
                            int mleaf, int kmax, cudaStream_t st) {
  if (nleaves <= 0 || rmax <= 0) return cudaSuccess;
  const size_t smem = leaf_ext_smem(nleaf, mleaf, kmax);
  void (*k)(const Task*, const Slot*, int, int) = final_part ? leaf_ext_kernel<true> : leaf_ext_kernel<false>;
  // resident blocks per SM for this shared-memory size (cached per kernel)
  static size_t c_smem[2] = {0, 0};
  static int c_blocks[2] = {0, 0};
  const int w = final_part ? 1 : 0;
  if (c_smem[w] != smem || c_blocks[w] <= 0) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(smem, 1));
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0, dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, PT, smem)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    c_smem[w] = smem;
    c_blocks[w] = std::max(1, per_sm * sms);
  }
  const int ncb = (rmax + XW - 1) / XW;
  const int64_t units = nleaves * (int64_t)ncb;
  if (units > (int64_t)INT32_MAX) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)std::min<int64_t>(units, c_blocks[w]);
  k<<<grid, PT, smem, st>>>(leaves, slots, (int)units, ncb);
  return cudaGetLastError();
}

}  // namespace hss
