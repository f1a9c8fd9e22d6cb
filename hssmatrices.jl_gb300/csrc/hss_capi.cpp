// Host side of the C ABI declared in include/hssgpu.h: plan construction
// (validation, level lists, workspace and factor-storage layout), buffer
// management, launch sequencing and the FP64 iterative refinement loop.
#include "hssgpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <functional>
#include <limits>
#include <cstring>
#include <string>
#include <vector>

#include "hss_host.h"
#include "hss_internal.h"
#include "hss_launch.h"
#include "hss_sample.h"

using namespace hss;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? HSS_ERR_OOM : HSS_ERR_CUDA;
}

#define CUDA_TRY(x)                                   \
  do {                                                \
    cudaError_t e_ = (x);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x);  \
  } while (0)

// Slot table on the device, re-uploaded only when its contents change, and
// the launch state of the persistent product run with it.
// A launch sequence captured as a CUDA graph, replayed while its key (the
// task lists, slot table, sizes and kernel choices that shaped it) is unchanged.
struct GraphCache {
  uint64_t key = 0, seen = 0;     // seen: key of the last uncaptured run
  cudaGraphExec_t exec = nullptr;
  int64_t launches = 0;           // kernel launches inside the graph
  bool flag = false;              // a result of the captured run (factor: every level fast)
  GraphCache() = default;
  GraphCache(const GraphCache&) = delete;
  GraphCache& operator=(const GraphCache&) = delete;
  ~GraphCache() { reset(); }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    key = 0;
  }
};

struct SlotTable {
  DBuf<Slot> dev;
  std::vector<Slot> last;
  GraphCache graph;
  // a second stream and two events, for launches of a product that may overlap
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaError_t ensure_side() {
    cudaError_t e = cudaSuccess;
    if (!side) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e == cudaSuccess && !ev_fork) e = cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess && !ev_join) e = cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming);
    return e;
  }
  SlotTable() = default;
  SlotTable(const SlotTable&) = delete;
  SlotTable& operator=(const SlotTable&) = delete;
  ~SlotTable() {
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
  }
  DBuf<uint32_t> pstate;             // launch counters: zero between launches
  DBuf<unsigned long long> pq;       // queue entries, tagged with the epoch of their launch
  uint32_t epoch = 0;                // tag of the last persistent launch on pq
  DBuf<double> ctb;                  // the flat product's leaf contributions
  DBuf<uint32_t> dcnt;               // its per-(leaf, chunk) counters: zero between launches
  cudaError_t ensure_flat(int64_t ctb_elems, int64_t counters, cudaStream_t st) {
    cudaError_t e = ctb.ensure((size_t)ctb_elems);
    if (e != cudaSuccess || (dcnt.p && dcnt.cap >= (size_t)counters)) return e;
    e = dcnt.ensure((size_t)counters);
    if (e == cudaSuccess) e = cudaMemsetAsync(dcnt.p, 0, dcnt.cap * sizeof(uint32_t), st);
    return e;
  }
  cudaError_t ensure_pmv(int64_t entries, cudaStream_t st) {
    const size_t words = (size_t)pmv_state_words(), ents = (size_t)std::max<int64_t>(entries, 1);
    if (pstate.p && pstate.cap >= words && pq.p && pq.cap >= ents && epoch < pmv_epoch_limit()) return cudaSuccess;
    pstate.release();
    pq.release();
    cudaError_t e = pstate.ensure(words);
    if (e == cudaSuccess) e = cudaMemsetAsync(pstate.p, 0, pstate.cap * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = pq.ensure(ents);
    if (e == cudaSuccess) e = cudaMemsetAsync(pq.p, 0, pq.cap * sizeof(unsigned long long), st);
    epoch = 0;
    return e;
  }
  cudaError_t upload(const std::vector<Slot>& s, cudaStream_t st) {
    if (s.size() == last.size() && dev.p &&
        std::memcmp(s.data(), last.data(), s.size() * sizeof(Slot)) == 0)
      return cudaSuccess;
    cudaError_t e = dev.ensure(s.size());
    if (e != cudaSuccess) return e;
    // pageable source: the copy is staged before the call returns
    e = cudaMemcpyAsync(dev.p, s.data(), s.size() * sizeof(Slot), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) last = s;
    return e;
  }
};

struct Seg {
  int64_t off = 0, cnt = 0;
  int mmax = 0, nmax = 0, kumax = 0, kvmax = 0;   // largest node of the list
  int c1u = 0, c2u = 0, c1v = 0, c2v = 0;          // largest children's ranks (branches)
  int kmax = 0, mkmax = 0;                         // largest ULV k and m - k
  int c1mr = 0, c2mr = 0, c1nr = 0, c2nr = 0;      // largest children's reduced sizes
  int64_t sv_stage = 0;                            // largest upward-solve staging need
};

inline int64_t align16(int64_t x) { return (x + 15) & ~int64_t(15); }

// Launch accounting and optional CUDA-event bracketing of one kernel kind.
// Kernel launches of the process (host calls may come from several threads).
// Launches issued while a thread captures a graph are counted into that
// thread's capture counter and added each time the graph is replayed.
std::atomic<int64_t> g_launches{0};
thread_local int64_t* t_capture = nullptr;
// Set while this thread records the refinement loop into a graph: launches
// whose per-launch host state (the persistent product's queue epoch) would be
// frozen by the recording reset that state on the device instead.
thread_local bool t_graph_capture = false;
inline void add_launches(int64_t n) {
  if (t_capture) *t_capture += n;
  else g_launches += n;
}
// Forces the global-memory factor kernel for every level (parity tests of the two kernels).
bool g_generic_factor = false;
// Forces the native FP64 product for the refinement residual.
bool g_residual_fp64 = false;
// Forces the level-by-level product kernels instead of the persistent one.
bool g_level_product = false;
// Lets FP64 products of few columns run the flat form of the persistent product.
bool g_flat_product = true;
bool g_tensor_dx = true;   // HSS_OPT_TENSOR_RESIDUAL
// Replays factor and solve launch sequences as CUDA graphs (non-default streams).
bool g_graphs = false;
// Autotuner: forces every solve level to the register (0) or the blocked (1)
// kernel where the blocked one is eligible; -1 leaves the choice to the factor.
int g_pick_force = -1;
struct TraceState {
  int kind = -1;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
} g_trace;

cudaEvent_t trace_event() {
  if (g_trace.used == g_trace.pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    g_trace.pool.push_back(e);
  }
  return g_trace.pool[g_trace.used++];
}

// Runs `launch` (which issues one kernel when cnt > 0) and brackets it with
// events when its kind is being traced.
template <typename F>
void traced(int kind, int64_t cnt, cudaStream_t st, F&& launch) {
  if (cnt <= 0) return;
  const bool on = g_trace.kind == kind;
  if (on) {
    cudaEvent_t a = trace_event();
    if (a) cudaEventRecord(a, st);
  }
  launch();
  add_launches(1);
  if (on) {
    cudaEvent_t b = trace_event();
    if (b) cudaEventRecord(b, st);
  }
}

}  // namespace

struct hss_plan_s {
  uint64_t serial = 0;                  // unique per plan for the life of the process (cache key)
  int device = 0;
  int32_t ntrees = 0;
  std::vector<Node> nodes;              // host copy, device pointers inside
  std::vector<int32_t> tree_root;
  std::vector<int64_t> tree_m, tree_n;
  double* d_gen = nullptr;
  Node* d_nodes = nullptr;
  Task* d_tasks = nullptr;
  std::vector<Seg> by_h, by_d, mv_up, mv_dn;
  Seg leaves;
  int64_t ws_mv = 0, ws_sv = 0;         // workspace rows
  int64_t fac_elems = 0;                // factor storage elements
  int max_m = 0, max_n = 0;
  int32_t* d_err = nullptr;
  DBuf<double> mv_ws;
  SlotTable mv_slots;
  DBuf<double> hB, hC;                  // staging for the _host product
  hss_factor_s* fused[2] = {nullptr, nullptr};   // storage reused by hss_ulvfactsolve_host
  int64_t gen_len = 0;                  // elements of d_gen
  float2* d_gen_df = nullptr;           // generators as (hi, lo) float pairs, made on first use
  unsigned char* d_dx = nullptr;        // slices of the leaf blocks D for the tensor-core residual (first use)
  int64_t dx_bytes = 0;
  int32_t* d_sync = nullptr;            // per-node arrival counters of the persistent product
  int pmv_nleaf = 0, pmv_mleaf = 0, pmv_kmax = 0;   // largest leaf columns / rows, largest rank
  int64_t pmv_ninner = 0;                           // branches that are not roots
  int64_t tr_lo = 0, tr_hi = 0;         // element range of d_gen holding every translator (B, R, W)
  // flat product tables (flat_dep = 0: it does not apply): per-node links,
  // per-leaf ancestor paths (flat_dep entries each), the non-root branches
  FlatLink* d_links = nullptr;
  int32_t* d_paths = nullptr;
  int32_t flat_dep = 0;
  Seg branches;
  std::vector<Task> h_tasks;            // host copy of the task lists (merged batches)
  std::vector<int64_t> h_table;         // node table of a single-tree plan (hss_export)
  int64_t h_npacked = 0;                // its packed generator length
  hss_plan_s* tplan = nullptr;          // the adjoint's plan (hss_matmul_t), made on first use
  std::string ulv_why;                  // why the ULV reduction cannot factor this plan (empty: it can)
  cudaStream_t host_st = nullptr;       // stream of the host-buffer solves (made on first use)
  cudaEvent_t host_ev = nullptr;
  cudaStream_t copy_st = nullptr;       // their right-hand sides' copy, beside the factorization
  cudaEvent_t copy_ev = nullptr;
  ~hss_plan_s();
};

// Per-call buffers of a (batched) solve with refinement.
struct SolveBufs {
  DBuf<double> R, bn2, rn2, scale;
  HBuf<double> h_bn2, h_rn2;
  DBuf<float2> xs, tmp;
  SlotTable sv0, sv1, mv;
  // the refinement loop recorded as one CUDA graph: the first pass, the first
  // residual and its check, then a while node around (correction, residual,
  // check); the check kernel sets the node's condition
  DBuf<double> status;                  // RefineStatus
  HBuf<double> h_status;
  GraphCache loop;
  int64_t loop_body_launches = 0;       // kernel launches of one pass of the while body
  uint64_t loop_failed = 0;             // key whose recording failed (the host loop runs it)
};

struct hss_factor_s {
  hss_plan_s* plan = nullptr;
  int prec = HSS_PREC_FP64;
  bool blocked = false;                 // FP32 factors of the blocked reduction on every level
  // autotuned kernel per tree level (hss_autotune): 1 blocked solve, 0 register
  // solve, -1 (or empty) the built-in rule; residual product 1 persistent, 0 per level
  std::vector<int8_t> tune_up, tune_down;
  int tune_pmv = -1;
  void* d_fac = nullptr;
  size_t fac_bytes = 0;
  DBuf<char> sv_ws;                     // solve workspace (this factor's plan layout)
  DBuf<float2> ws2;                     // double-float product workspace
  SlotTable fac_slots;
  SolveBufs bufs;
  DBuf<double> hB, hX;                  // staging for the _host solve
  // the pipelined factorization + first solve (hss_ulvfactsolve): a stream for
  // the upward solve, one for the factorization, and events [fork, solve join,
  // factorization join, prelude done, level 0, level 1, ...]
  cudaStream_t pipe_st = nullptr;
  cudaStream_t fac_st = nullptr;        // the factorization's stream there (highest priority)
  std::vector<cudaEvent_t> pipe_ev;
  GraphCache pipe_graph;
  ~hss_factor_s() {
    pipe_graph.reset();
    for (cudaEvent_t e : pipe_ev) cudaEventDestroy(e);
    if (pipe_st) cudaStreamDestroy(pipe_st);
    if (fac_st) cudaStreamDestroy(fac_st);
    if (d_fac) cudaFree(d_fac);
  }
};

hss_plan_s::~hss_plan_s() {
  if (host_ev) cudaEventDestroy(host_ev);
  if (host_st) cudaStreamDestroy(host_st);
  if (copy_ev) cudaEventDestroy(copy_ev);
  if (copy_st) cudaStreamDestroy(copy_st);
  delete tplan;
  delete fused[0];
  delete fused[1];
  if (d_gen_df) cudaFree(d_gen_df);
  if (d_dx) cudaFree(d_dx);
  if (d_gen) cudaFree(d_gen);
  if (d_nodes) cudaFree(d_nodes);
  if (d_tasks) cudaFree(d_tasks);
  if (d_err) cudaFree(d_err);
  if (d_sync) cudaFree(d_sync);
  if (d_links) cudaFree(d_links);
  if (d_paths) cudaFree(d_paths);
}


namespace {

// ---------------------------------------------------------------------------
// plan construction
// ---------------------------------------------------------------------------

struct TreeIn {
  int64_t nnodes;
  const int64_t* table;
  const double* packed;
  int64_t npacked;
};

// Generator pointers are recorded as offsets into the forest's packed buffer
// during validation and turned into device pointers after the upload.
struct GenOffsets {
  int64_t D = -1, U = -1, V = -1, B12 = -1, B21 = -1, R1 = -1, R2 = -1, W1 = -1, W2 = -1;
};

// Host-only phase: validates every tree (the dimension checks of `checkdims`,
// src/hssmatrix.jl:308-322, plus the ULV size rules of src/ulvfactor.jl:27-28),
// numbers nodes, computes depths, heights, leaf offsets, ULV reduce sizes,
// workspace and factor-storage layout, and the level task lists.
int layout_plan(hss_plan_s* P, const std::vector<TreeIn>& trees, std::vector<GenOffsets>& go,
                std::vector<Task>& tasks, std::vector<int64_t>& gbases) {
  P->ntrees = (int32_t)trees.size();
  int64_t total_nodes = 0, total_gen = 0;
  for (auto& t : trees) {
    if (t.nnodes <= 0 || t.table == nullptr) return fail(HSS_ERR_INVALID, "empty node table");
    if (t.npacked < 0) return fail(HSS_ERR_INVALID, "negative packed length");
    total_nodes += t.nnodes;
    gbases.push_back(total_gen);
    total_gen += align16(t.npacked);
  }
  gbases.push_back(total_gen);
  if (total_nodes > (int64_t)INT32_MAX) return fail(HSS_ERR_BAD_DIMS, "too many nodes");
  P->nodes.assign(total_nodes, Node{});
  go.assign(total_nodes, GenOffsets{});
  int64_t nbase = 0;
  int max_h = 0, max_d = 0;
  int64_t ws_mv = 0, ws_sv = 0, fac = 0;
  for (size_t ti = 0; ti < trees.size(); ++ti) {
    const TreeIn& t = trees[ti];
    const int64_t nn = t.nnodes;
    const int64_t gbase = gbases[ti];
    auto F = [&](int64_t i, int f) { return t.table[i * HSS_NODE_FIELDS + f]; };
    auto gchk = [&](int64_t off, int64_t len, const char* what, int64_t* out) -> int {
      if (len == 0) { *out = -1; return HSS_OK; }
      if (off < 0 || off + len > t.npacked)
        return fail(HSS_ERR_BAD_DIMS, std::string("generator block out of range: ") + what);
      *out = gbase + off;
      return HSS_OK;
    };
    // topology
    std::vector<int32_t> parent(nn, -1);
    for (int64_t i = 0; i < nn; ++i) {
      const int64_t l = F(i, 0), r = F(i, 1);
      if ((l < 0) != (r < 0)) return fail(HSS_ERR_BAD_DIMS, "node with only one child");
      for (int64_t c : {l, r}) {
        if (c < 0) continue;
        if (c >= nn || c == 0) return fail(HSS_ERR_BAD_DIMS, "child index out of range");
        if (parent[c] != -1) return fail(HSS_ERR_BAD_DIMS, "node with two parents");
        parent[c] = (int32_t)i;
      }
    }
    for (int64_t i = 1; i < nn; ++i)
      if (parent[i] < 0) return fail(HSS_ERR_BAD_DIMS, "unreachable node");
    // pre-order traversal (left first) from the root
    std::vector<int32_t> pre;
    pre.reserve(nn);
    {
      std::vector<int32_t> stack{0};
      while (!stack.empty() && (int64_t)pre.size() <= nn) {
        int32_t x = stack.back();
        stack.pop_back();
        pre.push_back(x);
        if (F(x, 0) >= 0) {
          stack.push_back((int32_t)F(x, 1));
          stack.push_back((int32_t)F(x, 0));
        }
      }
    }
    if ((int64_t)pre.size() != nn) return fail(HSS_ERR_BAD_DIMS, "node table is not a tree");
    Node* N = P->nodes.data() + nbase;
    GenOffsets* O = go.data() + nbase;
    for (int64_t i = 0; i < nn; ++i) {
      Node& x = N[i];
      x.left = F(i, 0) >= 0 ? (int32_t)(nbase + F(i, 0)) : -1;
      x.right = F(i, 1) >= 0 ? (int32_t)(nbase + F(i, 1)) : -1;
      x.parent = parent[i] >= 0 ? (int32_t)(nbase + parent[i]) : -1;
      x.leaf = F(i, 0) < 0;
      x.root = i == 0;
      x.tree = (int32_t)ti;
    }
    for (int32_t i : pre) {
      N[i].depth = i == 0 ? 0 : N[parent[i]].depth + 1;
      max_d = std::max(max_d, N[i].depth);
    }
    int64_t row = 0, col = 0;
    for (int32_t i : pre) {   // leaf offsets in pre-order
      if (N[i].leaf) {
        N[i].row0 = row;
        N[i].col0 = col;
        row += F(i, 2);
        col += F(i, 3);
      }
    }
    // post-order: sizes, generator blocks, ULV reduce sizes
    for (auto it = pre.rbegin(); it != pre.rend(); ++it) {
      const int32_t i = *it;
      Node& x = N[i];
      GenOffsets& o = O[i];
      const bool root = i == 0;
      x.ku = root ? 0 : (int32_t)F(i, 4);
      x.kv = root ? 0 : (int32_t)F(i, 5);
      if (F(i, 4) < 0 || F(i, 5) < 0 || F(i, 4) > (1 << 20) || F(i, 5) > (1 << 20))
        return fail(HSS_ERR_BAD_DIMS, "generator rank out of range");
      int rc;
      if (x.leaf) {
        const int64_t m = F(i, 2), n = F(i, 3);
        if (m <= 0 || n <= 0 || m > (1 << 20) || n > (1 << 20))
          return fail(HSS_ERR_BAD_DIMS, "leaf block size out of range");
        x.gm = (int32_t)m;
        x.gn = (int32_t)n;
        x.height = 0;
        x.m = x.gm;
        x.n = x.gn;
        if ((rc = gchk(F(i, 6), m * n, "D", &o.D))) return rc;
        if ((rc = gchk(F(i, 7), m * x.ku, "U", &o.U))) return rc;
        if ((rc = gchk(F(i, 8), n * x.kv, "V", &o.V))) return rc;
      } else {
        const Node& c1 = N[F(i, 0)];
        const Node& c2 = N[F(i, 1)];
        if ((int64_t)c1.gm + c2.gm > (1LL << 31) - 1 || (int64_t)c1.gn + c2.gn > (1LL << 31) - 1)
          return fail(HSS_ERR_BAD_DIMS, "matrix too large");
        x.gm = c1.gm + c2.gm;
        x.gn = c1.gn + c2.gn;
        x.row0 = c1.row0;
        x.col0 = c1.col0;
        x.height = std::max(c1.height, c2.height) + 1;
        if ((rc = gchk(F(i, 9), (int64_t)c1.ku * c2.kv, "B12", &o.B12))) return rc;
        if ((rc = gchk(F(i, 10), (int64_t)c2.ku * c1.kv, "B21", &o.B21))) return rc;
        if ((rc = gchk(F(i, 11), (int64_t)c1.ku * x.ku, "R1", &o.R1))) return rc;
        if ((rc = gchk(F(i, 12), (int64_t)c2.ku * x.ku, "R2", &o.R2))) return rc;
        if ((rc = gchk(F(i, 13), (int64_t)c1.kv * x.kv, "W1", &o.W1))) return rc;
        if ((rc = gchk(F(i, 14), (int64_t)c2.kv * x.kv, "W2", &o.W2))) return rc;
        x.m = c1.mr + c2.mr;   // merged block (src/ulvfactor.jl:75)
        x.n = c1.nr + c2.nr;
      }
      max_h = std::max(max_h, x.height);
      // a plan that the ULV reduction cannot factor (rectangular, or a block
      // with m - k > n) is still a valid operand of the products; its
      // factorization is refused when asked for
      if (root) {
        if (x.m != x.n && P->ulv_why.empty()) P->ulv_why = "root block of the ULV reduction is not square";
        x.k = x.m; x.mk = 0; x.nk = 0; x.mr = x.m; x.nr = x.n; x.lower_u = 0;
      } else {
        x.k = std::min(x.ku, x.m);               // src/ulvfactor.jl:27
        x.mk = x.m - x.k;
        x.nk = std::min(x.mk, x.n);              // :28
        if (x.mk > x.n && P->ulv_why.empty())
          P->ulv_why = "m - k > n in the ULV reduction (trsm needs a square L1)";
        x.mr = x.m - x.mk;
        x.nr = x.n - x.nk;
        x.lower_u = x.mk > 0;
      }
      P->max_m = std::max(P->max_m, x.m);
      P->max_n = std::max(P->max_n, x.n);
    }
    {
      // Block shapes follow from the ranks, so a rank that disagrees with the
      // stored blocks shows up as overlapping blocks: require them disjoint.
      std::vector<std::pair<int64_t, int64_t>> blocks;
      for (int64_t i = 0; i < nn; ++i) {
        const Node& x = N[i];
        const GenOffsets& o = O[i];
        auto add = [&](int64_t off, int64_t len) {
          if (off >= 0 && len > 0) blocks.emplace_back(off, len);
        };
        if (x.leaf) {
          add(o.D, (int64_t)x.gm * x.gn);
          add(o.U, (int64_t)x.gm * x.ku);
          add(o.V, (int64_t)x.gn * x.kv);
        } else {
          const Node& c1 = N[x.left - nbase];
          const Node& c2 = N[x.right - nbase];
          add(o.B12, (int64_t)c1.ku * c2.kv);
          add(o.B21, (int64_t)c2.ku * c1.kv);
          add(o.R1, (int64_t)c1.ku * x.ku);
          add(o.R2, (int64_t)c2.ku * x.ku);
          add(o.W1, (int64_t)c1.kv * x.kv);
          add(o.W2, (int64_t)c2.kv * x.kv);
        }
      }
      std::sort(blocks.begin(), blocks.end());
      for (size_t b = 1; b < blocks.size(); ++b)
        if (blocks[b - 1].first + blocks[b - 1].second > blocks[b].first)
          return fail(HSS_ERR_BAD_DIMS, "generator blocks overlap: ranks disagree with the stored blocks");
    }
    P->tree_root.push_back((int32_t)nbase);
    P->tree_m.push_back(N[0].gm);
    P->tree_n.push_back(N[0].gn);
    // workspace rows and factor storage (elements)
    for (int32_t i : pre) {
      Node& x = N[i];
      x.wz = ws_mv; ws_mv += x.kv;
      x.wf = ws_mv; ws_mv += x.ku;
      x.wb = ws_sv; ws_sv += x.m;
      x.wu = ws_sv; ws_sv += x.kv;
      x.wx = ws_sv; ws_sv += x.n;
      x.fD = fac; fac += align16((int64_t)x.m * x.n);
      x.fU = fac; fac += align16((int64_t)x.m * x.ku);
      x.fV = fac; fac += align16((int64_t)x.n * x.kv);
      x.ftq = fac; fac += align16(x.root ? 0 : x.k);
      x.ftl = fac; fac += align16(x.mk);
      x.fQt = fac; fac += align16((int64_t)x.n * x.mk);
      if (!x.leaf) {
        const Node& c1 = N[F(i, 0)];
        const Node& c2 = N[F(i, 1)];
        x.fT12 = fac; fac += align16((int64_t)c1.mr * c2.kv);
        x.fT21 = fac; fac += align16((int64_t)c2.mr * c1.kv);
      }
      if (x.root) { x.fpiv = fac; fac += align16(x.m); }
      x.fdx = -1;
      if (x.leaf && !x.root && dx_tc_fits(x.m, x.n)) {
        x.fdx = P->dx_bytes;
        P->dx_bytes += (dx_leaf_bytes(x.n) + 255) & ~int64_t(255);
      }
      if (!x.root && x.mk > 0) {
        x.fTq = fac; fac += align16((int64_t)((x.k + 31) / 32) * 1024);
        x.fTl = fac; fac += align16((int64_t)((x.mk + 31) / 32) * 1024);
        x.fLi = fac; fac += align16((int64_t)((x.mk + 31) / 32) * 1024);
      }
    }
    for (int32_t i : pre) {
      Node& x = N[i];
      if (x.leaf) continue;
      for (int c = 0; c < 2; ++c) {
        const Node& y = N[F(i, c)];
        x.cku[c] = y.ku;
        x.ckv[c] = y.kv;
        x.cleaf[c] = y.leaf;
        x.cwz[c] = y.wz;
        x.cwf[c] = y.wf;
      }
    }
    nbase += nn;
  }
  P->ws_mv = std::max<int64_t>(ws_mv, 1);
  P->ws_sv = std::max<int64_t>(ws_sv, 1);
  P->fac_elems = std::max<int64_t>(fac, 1);
  // task lists
  auto add_seg = [&](std::vector<Seg>& v, auto pred, int nlev, bool by_height) {
    v.assign(nlev + 1, Seg{});
    for (int lv = 0; lv <= nlev; ++lv) {
      v[lv].off = (int64_t)tasks.size();
      for (int64_t i = 0; i < total_nodes; ++i) {
        const Node& x = P->nodes[i];
        if ((by_height ? x.height : x.depth) == lv && pred(x)) {
          tasks.push_back(Task{nullptr, (int32_t)i, x.tree});
          v[lv].mmax = std::max(v[lv].mmax, x.m);
          v[lv].nmax = std::max(v[lv].nmax, x.n);
          v[lv].kumax = std::max(v[lv].kumax, x.ku);
          v[lv].kvmax = std::max(v[lv].kvmax, x.kv);
          v[lv].kmax = std::max(v[lv].kmax, x.root ? 0 : x.k);
          v[lv].mkmax = std::max(v[lv].mkmax, x.mk);
          {
            const Node* a = x.leaf ? nullptr : &P->nodes[x.left];
            const Node* b = x.leaf ? nullptr : &P->nodes[x.right];
            v[lv].sv_stage = std::max(v[lv].sv_stage,
                                      solve_up_stage_need(x.m, x.k, x.mk, x.nk, x.kv, x.leaf, x.root, a ? a->mr : 0,
                                                          b ? b->mr : 0, a ? a->kv : 0, b ? b->kv : 0));
          }
          if (!x.leaf) {
            const Node& c1 = P->nodes[x.left];
            const Node& c2 = P->nodes[x.right];
            v[lv].c1u = std::max(v[lv].c1u, c1.ku);
            v[lv].c2u = std::max(v[lv].c2u, c2.ku);
            v[lv].c1v = std::max(v[lv].c1v, c1.kv);
            v[lv].c2v = std::max(v[lv].c2v, c2.kv);
            v[lv].c1mr = std::max(v[lv].c1mr, c1.mr);
            v[lv].c2mr = std::max(v[lv].c2mr, c2.mr);
            v[lv].c1nr = std::max(v[lv].c1nr, c1.nr);
            v[lv].c2nr = std::max(v[lv].c2nr, c2.nr);
          }
        }
      }
      v[lv].cnt = (int64_t)tasks.size() - v[lv].off;
    }
  };
  add_seg(P->by_h, [](const Node&) { return true; }, max_h, true);
  add_seg(P->by_d, [](const Node&) { return true; }, max_d, false);
  add_seg(P->mv_up, [](const Node& x) { return !x.leaf && !x.root; }, max_h, true);
  add_seg(P->mv_dn, [](const Node& x) { return !x.leaf; }, max_d, false);
  P->leaves.off = (int64_t)tasks.size();
  for (int64_t i = 0; i < total_nodes; ++i)
    if (P->nodes[i].leaf) tasks.push_back(Task{nullptr, (int32_t)i, P->nodes[i].tree});
  P->leaves.cnt = (int64_t)tasks.size() - P->leaves.off;
  return HSS_OK;
}

// Serial numbers of plans: a freed plan's address can be reused by a new one,
// so caches keyed on plans use these instead of pointers.
std::atomic<uint64_t> g_plan_serial{0};

// Tables of the flat product: the edge of every non-root node to its parent,
// and every leaf's ancestors by depth.  It applies when each subtree's leaves
// are contiguous in the leaf list (pre-order node numbering gives that) and
// the trees are not deeper than kFlatDep - 1.
int build_flat_tables(hss_plan_s* P, const std::vector<Task>& tasks) {
  const std::vector<Node>& N = P->nodes;
  const int64_t nn = (int64_t)N.size();
  std::vector<int32_t> lo(nn, INT32_MAX), hi(nn, -1), cnt(nn, 0);
  int maxd = 0;
  for (int64_t t = 0; t < P->leaves.cnt; ++t) {
    const int32_t i = tasks[P->leaves.off + t].node;
    maxd = std::max(maxd, N[i].depth);
    for (int32_t y = i; y >= 0; y = N[y].parent) {
      lo[y] = std::min<int32_t>(lo[y], (int32_t)t);
      hi[y] = std::max<int32_t>(hi[y], (int32_t)t);
      ++cnt[y];
    }
  }
  for (int64_t i = 0; i < nn; ++i)
    if (cnt[i] > 0 && hi[i] - lo[i] + 1 != cnt[i]) return HSS_OK;
  const int dep = maxd + 1;
  if (dep < 2 || dep > kFlatDep) return HSS_OK;
  std::vector<FlatLink> links(nn);
  std::memset(links.data(), 0, links.size() * sizeof(FlatLink));
  for (int64_t i = 0; i < nn; ++i) {
    const Node& x = N[i];
    if (x.root) continue;
    const Node& p = N[x.parent];
    const bool left = p.left == (int32_t)i;
    const Node& sib = N[left ? p.right : p.left];
    FlatLink& L = links[i];
    L.W = left ? p.W1 : p.W2;
    L.R = left ? p.R1 : p.R2;
    L.B = left ? p.B21 : p.B12;
    L.wf = x.wf;
    L.swf = sib.wf;
    L.ku = x.ku;
    L.kv = x.kv;
    L.kpu = p.ku;
    L.kpv = p.kv;
    L.sku = sib.ku;
    L.depth = x.depth;
    L.lf0 = lo[i];
    L.lfn = cnt[i];
  }
  std::vector<int32_t> paths((size_t)std::max<int64_t>(P->leaves.cnt, 1) * dep, 0);
  for (int64_t t = 0; t < P->leaves.cnt; ++t)
    for (int32_t y = tasks[P->leaves.off + t].node; !N[y].root; y = N[y].parent) paths[t * dep + N[y].depth] = y;
  CUDA_TRY(dev_alloc((void**)&P->d_links, std::max<size_t>(links.size(), 1) * sizeof(FlatLink)));
  CUDA_TRY(cudaMemcpy(P->d_links, links.data(), links.size() * sizeof(FlatLink), cudaMemcpyHostToDevice));
  CUDA_TRY(dev_alloc((void**)&P->d_paths, paths.size() * sizeof(int32_t)));
  CUDA_TRY(cudaMemcpy(P->d_paths, paths.data(), paths.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  P->branches.off = P->mv_up.empty() ? 0 : P->mv_up.front().off;
  P->branches.cnt = 0;
  for (const Seg& g : P->mv_up) P->branches.cnt += g.cnt;
  P->flat_dep = dep;
  return HSS_OK;
}

// device_fill: the generator buffer is left for the caller to write on the device.
int build_plan(hss_plan_s* P, const std::vector<TreeIn>& trees, bool device_fill = false) {
  P->serial = ++g_plan_serial;
  for (auto& t : trees)
    if (t.npacked > 0 && t.packed == nullptr && !device_fill) return fail(HSS_ERR_INVALID, "null packed buffer");
  std::vector<GenOffsets> go;
  std::vector<Task> tasks;
  std::vector<int64_t> gbases;
  int rc = layout_plan(P, trees, go, tasks, gbases);
  if (rc) return rc;
  // device phase
  CUDA_TRY(cudaGetDevice(&P->device));
  const int64_t total_gen = gbases.back();
  P->gen_len = total_gen;
  CUDA_TRY(dev_alloc((void**)&P->d_gen, std::max<int64_t>(total_gen, 1) * sizeof(double)));
  CUDA_TRY(dev_alloc((void**)&P->d_err, sizeof(int32_t)));
  CUDA_TRY(cudaMemset(P->d_err, 0, sizeof(int32_t)));
  const size_t nsync = std::max<size_t>(P->nodes.size(), 1) * pmv_sync_chunks();
  CUDA_TRY(dev_alloc((void**)&P->d_sync, nsync * sizeof(int32_t)));
  CUDA_TRY(cudaMemset(P->d_sync, 0, nsync * sizeof(int32_t)));
  for (const Node& x : P->nodes) {
    if (x.leaf) {
      P->pmv_nleaf = std::max(P->pmv_nleaf, x.gn);
      P->pmv_mleaf = std::max(P->pmv_mleaf, x.gm);
    }
    P->pmv_kmax = std::max(P->pmv_kmax, std::max(x.ku, x.kv));
    if (!x.leaf && !x.root) ++P->pmv_ninner;
  }
  for (size_t ti = 0; ti < trees.size(); ++ti)
    if (trees[ti].npacked > 0 && !device_fill)
      CUDA_TRY(cudaMemcpy(P->d_gen + gbases[ti], trees[ti].packed, trees[ti].npacked * sizeof(double),
                          cudaMemcpyHostToDevice));
  if (trees.size() == 1)
  {
    P->h_table.assign(trees[0].table, trees[0].table + trees[0].nnodes * HSS_NODE_FIELDS);
    P->h_npacked = trees[0].npacked;
  }
  {
    // translator range (prefetched into L2 by the persistent product); kept only
    // when it is not much larger than the translators themselves
    int64_t lo = INT64_MAX, hi = 0, tot = 0;
    for (size_t i = 0; i < P->nodes.size(); ++i) {
      const Node& x = P->nodes[i];
      if (x.leaf) continue;
      const Node& c1 = P->nodes[x.left];
      const Node& c2 = P->nodes[x.right];
      const GenOffsets& o = go[i];
      const int64_t offs[6] = {o.B12, o.B21, o.R1, o.R2, o.W1, o.W2};
      const int64_t lens[6] = {(int64_t)c1.ku * c2.kv, (int64_t)c2.ku * c1.kv, (int64_t)c1.ku * x.ku,
                               (int64_t)c2.ku * x.ku, (int64_t)c1.kv * x.kv, (int64_t)c2.kv * x.kv};
      for (int j = 0; j < 6; ++j)
        if (offs[j] >= 0 && lens[j] > 0) {
          lo = std::min(lo, offs[j]);
          hi = std::max(hi, offs[j] + lens[j]);
          tot += lens[j];
        }
    }
    if (tot > 0 && hi - lo <= 2 * tot) {
      P->tr_lo = lo;
      P->tr_hi = hi;
    }
  }
  auto gp = [&](int64_t off) -> const double* { return off < 0 ? nullptr : P->d_gen + off; };
  for (size_t i = 0; i < P->nodes.size(); ++i) {
    Node& x = P->nodes[i];
    const GenOffsets& o = go[i];
    x.D = gp(o.D); x.U = gp(o.U); x.V = gp(o.V);
    x.B12 = gp(o.B12); x.B21 = gp(o.B21);
    x.R1 = gp(o.R1); x.R2 = gp(o.R2); x.W1 = gp(o.W1); x.W2 = gp(o.W2);
  }
  const int64_t total_nodes = (int64_t)P->nodes.size();
  CUDA_TRY(dev_alloc((void**)&P->d_nodes, total_nodes * sizeof(Node)));
  CUDA_TRY(cudaMemcpy(P->d_nodes, P->nodes.data(), total_nodes * sizeof(Node), cudaMemcpyHostToDevice));
  for (auto& t : tasks) t.nodes = P->d_nodes;
  P->h_tasks = tasks;
  CUDA_TRY(dev_alloc((void**)&P->d_tasks, std::max<size_t>(tasks.size(), 1) * sizeof(Task)));
  CUDA_TRY(cudaMemcpy(P->d_tasks, tasks.data(), tasks.size() * sizeof(Task), cudaMemcpyHostToDevice));
  return build_flat_tables(P, tasks);
}

// ---------------------------------------------------------------------------
// launch sequences
// ---------------------------------------------------------------------------

// The task lists one launch sequence walks: a plan's own (slot = tree of the
// forest) or lists merged over several single-tree plans (slot = item).
struct Levels {
  const Task* d_tasks = nullptr;
  const std::vector<Seg>* by_h = nullptr;
  const std::vector<Seg>* by_d = nullptr;
  const std::vector<Seg>* mv_up = nullptr;
  const std::vector<Seg>* mv_dn = nullptr;
  Seg leaves;
  // persistent product: largest leaf columns / rows, largest rank, non-root nodes
  int nleaf = 0, mleaf = 0, kmax = 0;
  int64_t ntasks = 0;
  int64_t nodes_max = 0, nslots = 0;   // largest node array of a slot's plan; slots
  int64_t ninner = 0;                  // non-root branches
  int device = 0;
  // flat product tables (flat_dep = 0: not available)
  const FlatLink* links = nullptr;
  const int32_t* paths = nullptr;
  int flat_dep = 0;
  Seg branches;
  // translators to prefetch into L2 (FP64 and pair copies; null: none)
  const double* pf64 = nullptr;
  const float2* pfdf = nullptr;
  int64_t pf_elems = 0;
};

Levels plan_levels(const hss_plan_s* P) {
  Levels L;
  L.d_tasks = P->d_tasks;
  L.by_h = &P->by_h;
  L.by_d = &P->by_d;
  L.mv_up = &P->mv_up;
  L.mv_dn = &P->mv_dn;
  L.leaves = P->leaves;
  L.nleaf = P->pmv_nleaf;
  L.mleaf = P->pmv_mleaf;
  L.kmax = P->pmv_kmax;
  L.ntasks = (int64_t)P->nodes.size() - P->ntrees;
  L.nodes_max = (int64_t)P->nodes.size();
  L.nslots = P->ntrees;
  L.ninner = P->pmv_ninner;
  L.device = P->device;
  L.links = P->d_links;
  L.paths = P->d_paths;
  L.flat_dep = P->flat_dep;
  L.branches = P->branches;
  if (P->tr_hi > P->tr_lo) {
    L.pf64 = P->d_gen + P->tr_lo;
    L.pfdf = P->d_gen_df ? P->d_gen_df + P->tr_lo : nullptr;
    L.pf_elems = P->tr_hi - P->tr_lo;
  }
  return L;
}

// The persistent product runs when a launch state is given, it is not
// switched off, and the forest's leaves and ranks fit its shared memory.
bool use_pmv(const Levels& L, const SlotTable* pm, bool pairs, int rmax) {
  return pm != nullptr && !g_level_product && L.leaves.cnt > 0 && pmv_fits(L.nleaf, L.mleaf, L.kmax) &&
         pmv_chunks(pairs, rmax) > 0 && pmv_queue_fits(L.nodes_max, L.nslots);
}

// The flat product takes FP64 products of few columns on plans that have its tables.
bool use_flat(const Levels& L, bool pairs, int rmax) {
  return !pairs && g_flat_product && L.flat_dep > 0 && pmv_flat_fits(L.nleaf, L.kmax, L.flat_dep, rmax);
}

// dx: the slots carry prepared slices of their leaf blocks (pairs only): the
// leaf products D X run on the tensor cores before the persistent product.
int run_pmv(const Levels& L, const Slot* slots, int rmax, bool pairs, SlotTable& pm, cudaStream_t st,
            bool dx_slices = false) {
  if (use_flat(L, pairs, rmax)) {
    CUDA_TRY(pm.ensure_pmv(1, st));
    CUDA_TRY(pm.ensure_flat(pmv_flat_ctb_elems(L.leaves.cnt, L.flat_dep, L.kmax, rmax),
                            L.leaves.cnt * pmv_flat_chunks(rmax), st));
    cudaError_t e = cudaSuccess;
    traced(HSS_TRACE_MV_LEAF, L.leaves.cnt, st, [&] {
      e = launch_pmv_flat(L.d_tasks + L.leaves.off, L.leaves.cnt, L.d_tasks + L.branches.off, L.branches.cnt,
                          L.links, L.paths, L.flat_dep, slots, rmax, L.nleaf, L.mleaf, L.kmax, pm.pstate.p,
                          pm.ctb.p, pm.dcnt.p, L.device, st);
    });
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(e, "flat product launch");
    }
    return HSS_OK;
  }
  const int64_t qents = pmv_queue_entries(L.ntasks, L.ninner, pmv_chunks(pairs, rmax));
  CUDA_TRY(pm.ensure_pmv(qents, st));
  ++pm.epoch;
  // a recorded launch replays with this epoch: its queue entries are cleared first
  if (t_graph_capture) CUDA_TRY(cudaMemsetAsync(pm.pq.p, 0, (size_t)qents * sizeof(unsigned long long), st));
  cudaError_t e = cudaSuccess;
  // double-float residual: the leaf products D X on the tensor cores first,
  // and the leaf products Z = V^T X and C = alpha (D X + U F) + beta Y as
  // streams over all leaves around the persistent launch, which keeps the tree
  // part.  D X and Z = V^T X (both read X, write different buffers) run
  // concurrently on two streams, joined before the persistent launch.
  const bool dx = pairs && dx_slices && dx_tc_fits(L.mleaf, L.nleaf);
  const bool ext = dx && leaf_ext_fits(L.nleaf, L.mleaf, L.kmax);
  cudaStream_t sv = st;   // stream of the V^T X launch
  if (ext) {
    CUDA_TRY(pm.ensure_side());
    CUDA_TRY(cudaEventRecord(pm.ev_fork, st));
    CUDA_TRY(cudaStreamWaitEvent(pm.side, pm.ev_fork, 0));
    sv = pm.side;
    traced(HSS_TRACE_MV_UP, L.leaves.cnt, sv, [&] {
      e = launch_leaf_ext(false, L.d_tasks + L.leaves.off, L.leaves.cnt, slots, rmax, L.nleaf, L.mleaf, L.kmax, sv);
    });
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(e, "leaf upsweep launch");
    }
  }
  if (dx) {
    traced(HSS_TRACE_MV_DX, L.leaves.cnt, st, [&] { e = launch_dx_tc(L.d_tasks + L.leaves.off, L.leaves.cnt,
                                                                     slots, rmax, st); });
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(e, "tensor-core leaf product launch");
    }
  }
  if (ext) {
    CUDA_TRY(cudaEventRecord(pm.ev_join, sv));
    CUDA_TRY(cudaStreamWaitEvent(st, pm.ev_join, 0));
  }
  traced(HSS_TRACE_MV_LEAF, L.leaves.cnt, st, [&] {
    const void* pf = pairs ? (const void*)L.pfdf : (const void*)L.pf64;
    e = launch_pmv(pairs, L.d_tasks + L.leaves.off, L.leaves.cnt, slots, L.ntasks, L.ninner, rmax, L.nleaf, L.kmax,
                   pm.pstate.p,
                   pm.pq.p, pm.epoch, pf, pf ? L.pf_elems * 8 : 0, L.device, st, dx, ext);
  });
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_fail(e, "persistent product launch");
  }
  if (ext) {
    traced(HSS_TRACE_MV_FINAL, L.leaves.cnt, st, [&] {
      e = launch_leaf_ext(true, L.d_tasks + L.leaves.off, L.leaves.cnt, slots, rmax, L.nleaf, L.mleaf, L.kmax, st);
    });
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(e, "leaf final launch");
    }
  }
  return HSS_OK;
}

// The launch state run_pmv needs, allocated ahead (nothing is allocated while
// the launches are recorded into a graph).
cudaError_t pmv_prepare(const Levels& L, bool pairs, int rmax, SlotTable& pm, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (use_flat(L, pairs, rmax)) {
    e = pm.ensure_pmv(1, st);
    if (e == cudaSuccess)
      e = pm.ensure_flat(pmv_flat_ctb_elems(L.leaves.cnt, L.flat_dep, L.kmax, rmax),
                         L.leaves.cnt * pmv_flat_chunks(rmax), st);
  } else {
    e = pm.ensure_pmv(pmv_queue_entries(L.ntasks, L.ninner, pmv_chunks(pairs, rmax)), st);
  }
  if (e == cudaSuccess) e = pm.ensure_side();
  return e;
}

int run_matvec(const Levels& L, const Slot* slots, int rmax, cudaStream_t st, SlotTable* pm = nullptr) {
  if (use_pmv(L, pm, false, rmax)) return run_pmv(L, slots, rmax, false, *pm, st);
  const Task* T = L.d_tasks;
  constexpr size_t kStagedCap = 200 * 1024;
  traced(HSS_TRACE_MV_LEAF, L.leaves.cnt, st,
         [&] { launch_mv_leaf(T + L.leaves.off, L.leaves.cnt, slots, rmax, st); });
  for (size_t h = 1; h < L.mv_up->size(); ++h) {
    const Seg& g = (*L.mv_up)[h];
    traced(HSS_TRACE_MV_UP, g.cnt, st, [&] {
      const size_t sm = mv_up_staged_smem(g.kvmax, g.c1v, g.c2v);
      if (sm <= kStagedCap) launch_mv_up_staged(T + g.off, g.cnt, slots, sm, rmax, st);
      else launch_mv_up(T + g.off, g.cnt, slots, st);
    });
  }
  for (size_t d = 0; d < L.mv_dn->size(); ++d) {
    const Seg& g = (*L.mv_dn)[d];
    traced(HSS_TRACE_MV_DOWN, g.cnt, st, [&] {
      const size_t sm = mv_down_staged_smem(g.kumax, g.c1u, g.c2u, g.c1v, g.c2v);
      if (sm <= kStagedCap) launch_mv_down_staged(T + g.off, g.cnt, slots, sm, rmax, st);
      else launch_mv_down(T + g.off, g.cnt, slots, st);
    });
  }
  traced(HSS_TRACE_MV_FINAL, L.leaves.cnt, st,
         [&] { launch_mv_leaf_final(T + L.leaves.off, L.leaves.cnt, slots, rmax, st); });
  return HSS_OK;
}
int run_matvec(hss_plan_s* P, const Slot* slots, int rmax, cudaStream_t st, SlotTable* pm = nullptr) {
  return run_matvec(plan_levels(P), slots, rmax, st, pm);
}

int run_matvec_df(const Levels& L, const Slot* slots, int rmax, cudaStream_t st, SlotTable* pm = nullptr,
                  bool dx_slices = false) {
  if (use_pmv(L, pm, true, rmax)) return run_pmv(L, slots, rmax, true, *pm, st, dx_slices);
  const Task* T = L.d_tasks;
  traced(HSS_TRACE_MV_LEAF, L.leaves.cnt, st,
         [&] { launch_dfmv_leaf(T + L.leaves.off, L.leaves.cnt, slots, rmax, st); });
  for (size_t h = 1; h < L.mv_up->size(); ++h)
    traced(HSS_TRACE_MV_UP, (*L.mv_up)[h].cnt, st,
           [&] { launch_dfmv_up(T + (*L.mv_up)[h].off, (*L.mv_up)[h].cnt, slots, rmax, st); });
  for (size_t d = 0; d < L.mv_dn->size(); ++d)
    traced(HSS_TRACE_MV_DOWN, (*L.mv_dn)[d].cnt, st,
           [&] { launch_dfmv_down(T + (*L.mv_dn)[d].off, (*L.mv_dn)[d].cnt, slots, rmax, st); });
  traced(HSS_TRACE_MV_FINAL, L.leaves.cnt, st,
         [&] { launch_dfmv_final(T + L.leaves.off, L.leaves.cnt, slots, rmax, st); });
  return HSS_OK;
}

// The tensor-core residual's slices of every leaf block D, made once per plan
// (the generators do not change); false when the plan has no such leaves or
// the buffer cannot be allocated (the residual then runs without them).
bool ensure_dx(hss_plan_s* P, cudaStream_t st) {
  if (P->d_dx) return true;
  if (P->dx_bytes <= 0 || P->leaves.cnt <= 0) return false;
  if (dev_alloc((void**)&P->d_dx, (size_t)P->dx_bytes) != cudaSuccess) {
    P->d_dx = nullptr;
    cudaGetLastError();
    return false;
  }
  if (launch_dx_prep(P->d_tasks + P->leaves.off, P->leaves.cnt, P->d_dx, st) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(P->d_dx);
    P->d_dx = nullptr;
    return false;
  }
  add_launches(1);
  return true;
}

int ensure_df(hss_plan_s* P, cudaStream_t st) {
  if (P->d_gen_df) return HSS_OK;
  CUDA_TRY(dev_alloc((void**)&P->d_gen_df, std::max<int64_t>(P->gen_len, 1) * sizeof(float2)));
  launch_df_split(P->d_gen, P->d_gen_df, P->gen_len, st);
  add_launches(1);
  CUDA_TRY(cudaGetLastError());
  return HSS_OK;
}

// Returns true when every level ran the on-chip kernel (for FP32 the blocked
// reduction, whose factors also carry the panel T matrices and L1 block inverses).
// merge staging of a factor level: converted generators, children's reduced U/V, T12/T21
inline size_t factor_extra(const Seg& g) {
  return (size_t)g.c1u * g.c2v + (size_t)g.c2u * g.c1v + (size_t)(g.c1u + g.c2u) * g.kumax +
         (size_t)(g.c1v + g.c2v) * g.kvmax + (size_t)g.c1mr * g.c1u + (size_t)g.c2mr * g.c2u +
         (size_t)g.c1nr * g.c1v + (size_t)g.c2nr * g.c2v + (size_t)g.c1mr * g.c2v + (size_t)g.c2mr * g.c1v;
}

template <typename T>
bool factor_level_fast(const Seg& g) {
  return !g_generic_factor && factor_blk_fits<T>(g.mmax, g.nmax, g.kumax, g.kvmax, factor_extra(g));
}

// One factor level (h = tree height); true when it ran the on-chip kernel.
template <typename T>
bool run_factor_level(const Levels& L, size_t h, const Slot* slots, cudaStream_t st) {
  const Seg& g = (*L.by_h)[h];
  const bool fast = factor_level_fast<T>(g);
  traced(h == 0 ? HSS_TRACE_FACTOR_LEAF : HSS_TRACE_FACTOR_MERGE, g.cnt, st, [&] {
    if (fast)
      launch_ulv_factor_blk<T>(L.d_tasks + g.off, g.cnt, slots, g.mmax, g.nmax, g.kumax, g.kvmax, factor_extra(g), st);
    else
      launch_ulv_factor<T>(L.d_tasks + g.off, g.cnt, slots, g.mmax, g.nmax, st);
  });
  return fast;
}

template <typename T>
bool run_factor(const Levels& L, const Slot* slots, cudaStream_t st) {
  bool all_fast = true;
  for (size_t h = 0; h < L.by_h->size(); ++h) all_fast = run_factor_level<T>(L, h, slots, st) && all_fast;
  return all_fast;
}

// Largest rank a level's blocked solve stages (its own and its children's).
inline int seg_kmax(const Seg& g) { return std::max({g.kmax, g.kumax, g.c1mr, g.c2mr, 1}); }
inline int seg_kvmax(const Seg& g) { return std::max({g.kvmax, g.c1v, g.c2v, 1}); }

// The blocked solve (GEMM steps, one block per 32 right-hand sides) wins on
// levels of large nodes; the register kernels (one warp per right-hand side)
// win on levels of small nodes (64 x 64 merges, the root).
inline bool use_bsolve(bool blocked, const Seg& g) {
  return blocked && std::max(g.mmax, g.nmax) > 64 && bsolve_fits(g.mmax, g.nmax, seg_kmax(g), seg_kvmax(g));
}

// Kernel of one solve level: the autotuner's forced choice, else the factor's
// tuned choice (tuned[level] of the plan's own lists), else the rule above.
inline bool pick_bsolve(bool blocked, const Seg& g, const std::vector<int8_t>* tuned, size_t level) {
  const bool eligible = blocked && bsolve_fits(g.mmax, g.nmax, seg_kmax(g), seg_kvmax(g));
  if (!eligible) return false;
  if (g_pick_force >= 0) return g_pick_force == 1;
  if (tuned && level < tuned->size() && (*tuned)[level] >= 0) return (*tuned)[level] == 1;
  return use_bsolve(blocked, g);
}

// blocked: the factors come from the blocked FP32 reduction (T = float only);
// tf: the factor whose tuned choices apply (the plan's own task lists), or null.
template <typename T>
void run_solve_up_level(const Levels& L, size_t h, const Slot* slots, int rmax, cudaStream_t st, bool blocked,
                        const std::vector<int8_t>* tup) {
  const Seg& g = (*L.by_h)[h];
  traced(HSS_TRACE_SOLVE_UP, g.cnt, st, [&] {
    if (pick_bsolve(blocked, g, tup, h))
      launch_bsolve_up(L.d_tasks + g.off, g.cnt, slots, g.mmax, g.nmax, seg_kmax(g), seg_kvmax(g), rmax, st);
    else if (!g_generic_factor && solve_reg_fits(g.mmax, g.nmax))
      launch_ulv_solve_up_reg<T>(L.d_tasks + g.off, g.cnt, slots, g.mmax, g.sv_stage, rmax, st);
    else
      launch_ulv_solve_up<T>(L.d_tasks + g.off, g.cnt, slots, st);
  });
}

template <typename T>
void run_solve_down(const Levels& L, const Slot* slots, int rmax, cudaStream_t st, bool blocked,
                    const std::vector<int8_t>* tdn);

template <typename T>
void run_solve(const Levels& L, const Slot* slots, int rmax, cudaStream_t st, bool blocked = false,
               const hss_factor_s* tf = nullptr) {
  const std::vector<int8_t>* tup = tf ? &tf->tune_up : nullptr;
  const std::vector<int8_t>* tdn = tf ? &tf->tune_down : nullptr;
  for (size_t h = 0; h < L.by_h->size(); ++h) run_solve_up_level<T>(L, h, slots, rmax, st, blocked, tup);
  run_solve_down<T>(L, slots, rmax, st, blocked, tdn);
}

template <typename T>
void run_solve_down(const Levels& L, const Slot* slots, int rmax, cudaStream_t st, bool blocked,
                    const std::vector<int8_t>* tdn) {
  for (size_t d = 0; d < L.by_d->size(); ++d) {
    const Seg& g = (*L.by_d)[d];
    traced(HSS_TRACE_SOLVE_DOWN, g.cnt, st, [&] {
      if (pick_bsolve(blocked, g, tdn, d))
        launch_bsolve_down(L.d_tasks + g.off, g.cnt, slots, g.mmax, g.nmax, seg_kmax(g), seg_kvmax(g), rmax, st);
      else if (!g_generic_factor && solve_reg_fits(g.mmax, g.nmax))
        launch_ulv_solve_down_reg<T>(L.d_tasks + g.off, g.cnt, slots, g.nmax, g.mkmax, rmax, st);
      else
        launch_ulv_solve_down<T>(L.d_tasks + g.off, g.cnt, slots, st);
    });
  }
}

// Task lists merged over several single-tree plans, uploaded per call.
struct MergedLevels {
  std::vector<Seg> by_h, by_d, mv_up, mv_dn;
  Seg leaves;
  std::vector<Task> h;
  DBuf<Task> d;
  int nleaf = 0, mleaf = 0, kmax = 0, device = 0;
  int64_t ntasks = 0, nodes_max = 0, nslots = 0, ninner = 0;
  Levels view() const {
    Levels L;
    L.d_tasks = d.p;
    L.by_h = &by_h;
    L.by_d = &by_d;
    L.mv_up = &mv_up;
    L.mv_dn = &mv_dn;
    L.leaves = leaves;
    L.nleaf = nleaf;
    L.mleaf = mleaf;
    L.kmax = kmax;
    L.ntasks = ntasks;
    L.nodes_max = nodes_max;
    L.nslots = nslots;
    L.ninner = ninner;
    L.device = device;
    return L;
  }
};

Seg merge_seg_dims(Seg a, const Seg& b) {
  a.mmax = std::max(a.mmax, b.mmax); a.nmax = std::max(a.nmax, b.nmax);
  a.kumax = std::max(a.kumax, b.kumax); a.kvmax = std::max(a.kvmax, b.kvmax);
  a.c1u = std::max(a.c1u, b.c1u); a.c2u = std::max(a.c2u, b.c2u);
  a.c1v = std::max(a.c1v, b.c1v); a.c2v = std::max(a.c2v, b.c2v);
  a.kmax = std::max(a.kmax, b.kmax); a.mkmax = std::max(a.mkmax, b.mkmax);
  a.c1mr = std::max(a.c1mr, b.c1mr); a.c2mr = std::max(a.c2mr, b.c2mr);
  a.c1nr = std::max(a.c1nr, b.c1nr); a.c2nr = std::max(a.c2nr, b.c2nr);
  a.sv_stage = std::max(a.sv_stage, b.sv_stage);
  return a;
}

int merge_levels(const std::vector<hss_plan_s*>& plans, MergedLevels& M, cudaStream_t st) {
  M.h.clear();
  auto merge = [&](std::vector<Seg>& out, std::vector<Seg> hss_plan_s::*field) {
    size_t nlev = 0;
    for (auto* P : plans) nlev = std::max(nlev, (P->*field).size());
    out.assign(nlev, Seg{});
    for (size_t lv = 0; lv < nlev; ++lv) {
      Seg g;
      g.off = (int64_t)M.h.size();
      for (size_t i = 0; i < plans.size(); ++i) {
        const hss_plan_s* P = plans[i];
        if (lv >= (P->*field).size()) continue;
        const Seg& s = (P->*field)[lv];
        for (int64_t t = 0; t < s.cnt; ++t) {
          Task x = P->h_tasks[s.off + t];
          x.slot = (int32_t)i;
          M.h.push_back(x);
        }
        g = merge_seg_dims(g, s);
      }
      g.cnt = (int64_t)M.h.size() - g.off;
      out[lv] = g;
    }
  };
  merge(M.by_h, &hss_plan_s::by_h);
  merge(M.by_d, &hss_plan_s::by_d);
  merge(M.mv_up, &hss_plan_s::mv_up);
  merge(M.mv_dn, &hss_plan_s::mv_dn);
  M.leaves = Seg{};
  M.leaves.off = (int64_t)M.h.size();
  for (size_t i = 0; i < plans.size(); ++i) {
    const hss_plan_s* P = plans[i];
    for (int64_t t = 0; t < P->leaves.cnt; ++t) {
      Task x = P->h_tasks[P->leaves.off + t];
      x.slot = (int32_t)i;
      M.h.push_back(x);
    }
  }
  M.leaves.cnt = (int64_t)M.h.size() - M.leaves.off;
  M.nleaf = M.mleaf = M.kmax = 0;
  M.ntasks = 0;
  M.nodes_max = 0;
  M.ninner = 0;
  for (auto* P : plans) {
    M.nleaf = std::max(M.nleaf, P->pmv_nleaf);
    M.mleaf = std::max(M.mleaf, P->pmv_mleaf);
    M.kmax = std::max(M.kmax, P->pmv_kmax);
    M.ntasks += (int64_t)P->nodes.size() - P->ntrees;
    M.nodes_max = std::max<int64_t>(M.nodes_max, (int64_t)P->nodes.size());
    M.ninner += P->pmv_ninner;
  }
  M.nslots = (int64_t)plans.size();
  M.device = plans.empty() ? 0 : plans[0]->device;
  CUDA_TRY(M.d.ensure(std::max<size_t>(M.h.size(), 1)));
  // pageable source: staged before the call returns; stream order protects
  // the previous batch's reads of the same buffer
  CUDA_TRY(cudaMemcpyAsync(M.d.p, M.h.data(), M.h.size() * sizeof(Task), cudaMemcpyHostToDevice, st));
  return HSS_OK;
}

struct Cols {   // per-tree product / solve operands
  const double* B;
  int64_t ldb;
  int64_t r;
  double* C;
  int64_t ldc;
};

int check_cols(hss_plan_s* P, const std::vector<Cols>& io, bool solve) {
  for (int32_t t = 0; t < P->ntrees; ++t) {
    const Cols& c = io[t];
    if (c.r < 0) return fail(HSS_ERR_BAD_DIMS, "negative number of right-hand sides");
    if (c.r == 0) continue;
    if (c.B == nullptr || c.C == nullptr) return fail(HSS_ERR_INVALID, "null operand");
    const int64_t rows_in = solve ? P->tree_m[t] : P->tree_n[t];
    const int64_t rows_out = solve ? P->tree_n[t] : P->tree_m[t];
    if (c.ldb < rows_in)
      return fail(HSS_ERR_BAD_DIMS, "First dimension of B does not match second dimension of A");
    if (c.ldc < rows_out) return fail(HSS_ERR_BAD_DIMS, "Dimensions of C don't match up with A and B.");
    if (c.r > (1 << 24)) return fail(HSS_ERR_BAD_DIMS, "too many right-hand sides");
  }
  return HSS_OK;
}

int matmul_impl(hss_plan_s* P, const std::vector<Cols>& io, double alpha, double beta,
                cudaStream_t st, const double* const* Y, double* colnorm2, const int64_t* cn_off,
                SlotTable& table) {
  int64_t rmax = 0;
  for (auto& c : io) rmax = std::max(rmax, c.r);
  if (rmax == 0) return HSS_OK;
  CUDA_TRY(P->mv_ws.ensure((size_t)P->ws_mv * rmax));
  std::vector<Slot> s(P->ntrees);
  for (int32_t t = 0; t < P->ntrees; ++t) {
    Slot& x = s[t];
    std::memset(&x, 0, sizeof(Slot));
    x.B = io[t].B; x.ldb = io[t].ldb;
    x.C = io[t].C; x.ldc = io[t].ldc;
    x.Y = Y ? Y[t] : io[t].C;
    x.ldy = Y ? io[t].ldb : io[t].ldc;
    x.alpha = alpha; x.beta = beta;
    x.ws = P->mv_ws.p; x.ldws = P->ws_mv;
    x.r = (int32_t)io[t].r;
    x.colnorm2 = colnorm2 ? colnorm2 + cn_off[t] : nullptr;
    x.err = P->d_err;
    x.nodes = P->d_nodes;
    x.sync = P->d_sync;
  }
  CUDA_TRY(table.upload(s, st));
  int rc = run_matvec(P, table.dev.p, (int)rmax, st, &table);
  if (rc) return rc;
  CUDA_TRY(cudaGetLastError());
  return HSS_OK;
}

inline uint64_t fnv(uint64_t h, uint64_t v) {
  for (int i = 0; i < 8; ++i) {
    h ^= (v >> (8 * i)) & 0xffu;
    h *= 1099511628211ull;
  }
  return h;
}

// Key of a launch sequence over task lists L with the device slot table `slots`.
uint64_t levels_key(const Levels& L, const void* slots, int64_t extra) {
  uint64_t h = 1469598103934665603ull;
  h = fnv(h, (uint64_t)(uintptr_t)L.d_tasks);
  h = fnv(h, (uint64_t)(uintptr_t)slots);
  h = fnv(h, (uint64_t)extra);
  for (const std::vector<Seg>* v : {L.by_h, L.by_d})
    for (const Seg& g : *v) {
      const int64_t f[] = {g.off, g.cnt, g.mmax, g.nmax, g.kumax, g.kvmax, g.c1u, g.c2u, g.c1v, g.c2v,
                           g.kmax, g.mkmax, g.c1mr, g.c2mr, g.c1nr, g.c2nr, g.sv_stage};
      for (int64_t x : f) h = fnv(h, (uint64_t)x);
    }
  return h;
}

// Runs `launch` (which issues kernels on st and returns a flag) directly or,
// with graphs enabled on a non-default stream, as a replayed CUDA graph: the
// second run with an unchanged key is captured and every later one replays it.
template <typename F>
int graphed(GraphCache& gc, uint64_t key, cudaStream_t st, bool& flag, F&& launch, unsigned inst_flags = 0) {
  const bool can = g_graphs && st != nullptr && g_trace.kind < 0 && g_pick_force < 0;
  if (!can || (gc.key != key && gc.seen != key)) {
    if (can) gc.seen = key;
    flag = launch();
    return HSS_OK;
  }
  if (gc.key != key) {
    gc.reset();
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int64_t captured = 0;
    t_capture = &captured;
    const bool fl = launch();
    t_capture = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    const cudaError_t ie = cudaGraphInstantiate(&gc.exec, g, inst_flags);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      gc.exec = nullptr;
      return cuda_fail(ie, "cudaGraphInstantiate");
    }
    gc.key = key;
    gc.launches = captured;
    gc.flag = fl;
  }
  CUDA_TRY(cudaGraphLaunch(gc.exec, st));
  add_launches(gc.launches);
  flag = gc.flag;
  return HSS_OK;
}

// One factorization of a launch sequence: slot i of the sequence.
template <typename T>
int factor_items(const std::vector<hss_factor_s*>& fs, const Levels& L, SlotTable& table, cudaStream_t st) {
  std::vector<Slot> s(fs.size());
  for (size_t i = 0; i < fs.size(); ++i) {
    Slot& x = s[i];
    std::memset(&x, 0, sizeof(Slot));
    x.fbase = fs[i]->d_fac;
    x.err = fs[i]->plan->d_err;
  }
  CUDA_TRY(table.upload(s, st));
  bool fast = false;
  const uint64_t key = levels_key(L, table.dev.p, (int64_t)sizeof(T) + (g_generic_factor ? 16 : 0));
  int rc = graphed(table.graph, key, st, fast, [&] { return run_factor<T>(L, table.dev.p, st); });
  if (rc) return rc;
  for (auto* f : fs) f->blocked = fast && sizeof(T) == sizeof(float);
  CUDA_TRY(cudaGetLastError());
  return HSS_OK;
}

template <typename T>
int factor_impl(hss_factor_s* f, cudaStream_t st) {
  hss_plan_s* P = f->plan;
  std::vector<hss_factor_s*> fs(P->ntrees, f);   // every tree of a forest shares the storage
  return factor_items<T>(fs, plan_levels(P), f->fac_slots, st);
}

// One solve operand set: tree `tree` of item.f's plan, slot i of the sequence.
struct Item {
  hss_factor_s* f;
  int32_t tree;
  Cols io;
};

// A solve pass made ready to launch: its slot table uploaded and the key of
// its launch sequence.
struct PassPrep {
  uint64_t key = 0;
  int64_t rmax = 0;
  bool blocked = false;
};

template <typename T>
int solve_prep(const std::vector<Item>& items, const Levels& L, const double* scale, const int64_t* off,
               int64_t rtot, int mode, bool residual_input, const int64_t* roff, double* R, SlotTable& table,
               cudaStream_t st, const hss_factor_s* tf, PassPrep& pp) {
  int64_t rmax = 0;
  for (auto& it : items) rmax = std::max(rmax, it.io.r);
  pp.rmax = rmax;
  if (rmax == 0) return HSS_OK;
  std::vector<Slot> s(items.size());
  for (size_t i = 0; i < items.size(); ++i) {
    const Item& it = items[i];
    hss_plan_s* P = it.f->plan;
    CUDA_TRY(it.f->sv_ws.ensure((size_t)P->ws_sv * rmax * sizeof(T)));
    Slot& x = s[i];
    std::memset(&x, 0, sizeof(Slot));
    if (residual_input) {
      x.B = R + roff[i]; x.ldb = P->tree_m[it.tree];
    } else {
      x.B = it.io.B; x.ldb = it.io.ldb;
    }
    x.C = it.io.C; x.ldc = it.io.ldc;
    x.ws = it.f->sv_ws.p; x.ldws = P->ws_sv;
    x.fbase = it.f->d_fac;
    x.colscale = scale ? scale + off[i] : nullptr;
    x.colinv = scale ? scale + rtot + off[i] : nullptr;
    x.r = (int32_t)it.io.r;
    x.mode = mode;
    x.err = P->d_err;
  }
  CUDA_TRY(table.upload(s, st));
  bool blocked = true;
  for (auto& it : items) blocked = blocked && it.f->blocked;
  pp.blocked = blocked;
  uint64_t key = levels_key(L, table.dev.p, rmax * 64 + (blocked ? 1 : 0) + (sizeof(T) == 4 ? 2 : 0));
  if (tf)
    for (const std::vector<int8_t>* v : {&tf->tune_up, &tf->tune_down})
      for (int8_t c : *v) key = fnv(key, (uint64_t)(c + 2));
  pp.key = key;
  return HSS_OK;
}

template <typename T>
void solve_issue(const Levels& L, const SlotTable& table, const PassPrep& pp, cudaStream_t st,
                 const hss_factor_s* tf) {
  if (pp.rmax > 0) run_solve<T>(L, table.dev.p, (int)pp.rmax, st, pp.blocked, tf);
}

template <typename T>
int solve_pass(const std::vector<Item>& items, const Levels& L, const double* scale, const int64_t* off,
               int64_t rtot, int mode, bool residual_input, const int64_t* roff, double* R, SlotTable& table,
               cudaStream_t st, const hss_factor_s* tf = nullptr) {
  PassPrep pp;
  int rc = solve_prep<T>(items, L, scale, off, rtot, mode, residual_input, roff, R, table, st, tf, pp);
  if (rc || pp.rmax == 0) return rc;
  bool unused = false;
  rc = graphed(table.graph, pp.key, st, unused, [&] {
    solve_issue<T>(L, table, pp, st, tf);
    return true;
  });
  if (rc) return rc;
  CUDA_TRY(cudaGetLastError());
  return HSS_OK;
}

// The factorization of f's plan and the first solve pass of `items` (all on
// f's plan) in one launch sequence: level h is factored on a stream of the
// highest priority, then the upward solve of level h runs on a second stream
// once that level is done (an event per level), so the upward solve runs one
// level behind the factorization instead of after it; the downward solve
// follows both on st.  Replayed as one CUDA graph (fork and join through
// events, node priorities kept) where graphs apply.
template <typename T>
int factsolve_prep(hss_factor_s* f, const std::vector<Item>& items, const Levels& L, const double* scale,
                   const int64_t* off, int64_t rtot, SlotTable& table, cudaStream_t st, PassPrep& pp) {
  hss_plan_s* P = f->plan;
  int64_t rmax = 0;
  for (auto& it : items) rmax = std::max(rmax, it.io.r);
  pp.rmax = rmax;
  std::vector<Slot> fsl(P->ntrees);
  for (Slot& x : fsl) {
    std::memset(&x, 0, sizeof(Slot));
    x.fbase = f->d_fac;
    x.err = P->d_err;
  }
  CUDA_TRY(f->fac_slots.upload(fsl, st));
  std::vector<Slot> s(items.size());
  for (size_t i = 0; i < items.size(); ++i) {
    const Item& it = items[i];
    CUDA_TRY(it.f->sv_ws.ensure((size_t)P->ws_sv * std::max<int64_t>(rmax, 1) * sizeof(T)));
    Slot& x = s[i];
    std::memset(&x, 0, sizeof(Slot));
    x.B = it.io.B; x.ldb = it.io.ldb;
    x.C = it.io.C; x.ldc = it.io.ldc;
    x.ws = it.f->sv_ws.p; x.ldws = P->ws_sv;
    x.fbase = f->d_fac;
    x.colscale = scale ? scale + off[i] : nullptr;
    x.colinv = scale ? scale + rtot + off[i] : nullptr;
    x.r = (int32_t)it.io.r;
    x.mode = 0;
    x.err = P->d_err;
  }
  CUDA_TRY(table.upload(s, st));
  bool all_fast = true;
  for (size_t h = 0; h < L.by_h->size(); ++h) all_fast = factor_level_fast<T>((*L.by_h)[h]) && all_fast;
  pp.blocked = all_fast && sizeof(T) == sizeof(float);
  if (!f->pipe_st) CUDA_TRY(cudaStreamCreateWithFlags(&f->pipe_st, cudaStreamNonBlocking));
  if (!f->fac_st) {
    int least = 0, greatest = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CUDA_TRY(cudaStreamCreateWithPriority(&f->fac_st, cudaStreamNonBlocking, greatest));
  }
  while (f->pipe_ev.size() < 4 + L.by_h->size()) {
    cudaEvent_t e = nullptr;
    CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    f->pipe_ev.push_back(e);
  }
  uint64_t key = fnv(levels_key(L, f->fac_slots.dev.p, (int64_t)sizeof(T) + (g_generic_factor ? 16 : 0)),
                     levels_key(L, table.dev.p, rmax * 64 + (pp.blocked ? 1 : 0) + (sizeof(T) == 4 ? 2 : 0)));
  for (const std::vector<int8_t>* v : {&f->tune_up, &f->tune_down})
    for (int8_t c : *v) key = fnv(key, (uint64_t)(c + 2));
  pp.key = key;
  // the solves that follow (and the correction passes of a refinement) read
  // this factorization's kind
  f->blocked = pp.blocked;
  return HSS_OK;
}

template <typename T>
cudaError_t factsolve_issue(hss_factor_s* f, const Levels& L, const SlotTable& table, const PassPrep& pp,
                            cudaStream_t st, const std::function<int()>* pre = nullptr) {
  cudaError_t ev_err = cudaSuccess;
  auto chk = [&](cudaError_t e) { if (e != cudaSuccess && ev_err == cudaSuccess) ev_err = e; };
  // the factorization on the highest-priority stream, so that the merges (a
  // chain of small launches) are scheduled ahead of the upward solve's blocks;
  // `pre` (launches on st that the solve needs and the factorization does not,
  // such as waiting for the right-hand sides' copy) runs beside it
  cudaStream_t s2 = f->pipe_st, sf = f->fac_st;
  chk(cudaEventRecord(f->pipe_ev[0], st));
  chk(cudaStreamWaitEvent(sf, f->pipe_ev[0], 0));
  if (pre) {
    if ((*pre)() != HSS_OK && ev_err == cudaSuccess) ev_err = cudaErrorLaunchFailure;
    chk(cudaEventRecord(f->pipe_ev[3], st));
    chk(cudaStreamWaitEvent(s2, f->pipe_ev[3], 0));
  } else {
    chk(cudaStreamWaitEvent(s2, f->pipe_ev[0], 0));
  }
  for (size_t h = 0; h < L.by_h->size(); ++h) {
    run_factor_level<T>(L, h, f->fac_slots.dev.p, sf);
    chk(cudaEventRecord(f->pipe_ev[4 + h], sf));
    chk(cudaStreamWaitEvent(s2, f->pipe_ev[4 + h], 0));
    run_solve_up_level<T>(L, h, table.dev.p, (int)pp.rmax, s2, pp.blocked, &f->tune_up);
  }
  chk(cudaEventRecord(f->pipe_ev[2], sf));
  chk(cudaEventRecord(f->pipe_ev[1], s2));
  chk(cudaStreamWaitEvent(st, f->pipe_ev[2], 0));
  chk(cudaStreamWaitEvent(st, f->pipe_ev[1], 0));
  run_solve_down<T>(L, table.dev.p, (int)pp.rmax, st, pp.blocked, &f->tune_down);
  return ev_err;
}

template <typename T>
int factsolve_pass(hss_factor_s* f, const std::vector<Item>& items, const Levels& L, const double* scale,
                   const int64_t* off, int64_t rtot, SlotTable& table, cudaStream_t st) {
  PassPrep pp;
  int rc = factsolve_prep<T>(f, items, L, scale, off, rtot, table, st, pp);
  if (rc) return rc;
  bool unused = false;
  cudaError_t ev_err = cudaSuccess;
  rc = graphed(
      f->pipe_graph, pp.key, st, unused,
      [&] {
        ev_err = factsolve_issue<T>(f, L, table, pp, st);
        return true;
      },
      cudaGraphInstantiateFlagUseNodePriority);
  if (rc) return rc;
  if (ev_err != cudaSuccess) return cuda_fail(ev_err, "pipelined factorization events");
  CUDA_TRY(cudaGetLastError());
  return HSS_OK;
}

int read_dev_err(hss_plan_s* P, cudaStream_t st) {
  int32_t e = 0;
  CUDA_TRY(cudaMemcpyAsync(&e, P->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (e == DEV_SINGULAR) {
    cudaMemsetAsync(P->d_err, 0, sizeof(int32_t), st);
    return fail(HSS_ERR_SINGULAR, "root block of the ULV factorization is singular");
  }
  if (e == DEV_TIMEOUT || e == DEV_BAD) {
    // a persistent launch gave up: its per-node counters may be left non-zero
    cudaMemsetAsync(P->d_sync, 0, std::max<size_t>(P->nodes.size(), 1) * pmv_sync_chunks() * sizeof(int32_t), st);
    cudaMemsetAsync(P->d_err, 0, sizeof(int32_t), st);
    cudaStreamSynchronize(st);
    return e == DEV_TIMEOUT ? fail(HSS_ERR_TIMEOUT, "persistent product: no ready work within the poll limit")
                            : fail(HSS_ERR_CUDA, "persistent product: more downsweep tasks than tree nodes");
  }
  return HSS_OK;
}

// Records the refinement loop into a graph: `first` issues the launches up
// to and including the first convergence check, `body` one refinement step
// ending with a check; both get the while node's condition handle.  Returns
// false (nothing recorded, the stream out of capture, errors cleared) when the
// runtime refuses any part of it.
template <typename F0, typename F1>
bool record_loop(GraphCache& gc, uint64_t key, int64_t& body_launches, cudaStream_t st, F0&& first, F1&& body) {
  cudaGraph_t G = nullptr;
  if (cudaGraphCreate(&G, 0) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaGraphConditionalHandle cond = 0;
  int64_t n0 = 0, n1 = 0;
  bool ok = cudaGraphConditionalHandleCreate(&cond, G, 0, cudaGraphCondAssignDefault) == cudaSuccess &&
            cudaStreamBeginCaptureToGraph(st, G, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                cudaSuccess;
  std::vector<cudaGraphNode_t> tail;
  if (ok) {
    t_capture = &n0;
    t_graph_capture = true;
    const int rc = first(cond);
    t_capture = nullptr;
    t_graph_capture = false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd) == cudaSuccess &&
        cs == cudaStreamCaptureStatusActive && deps)
      tail.assign(deps, deps + nd);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    ok = rc == HSS_OK && e == cudaSuccess && g == G && !tail.empty();
  }
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};   // the rest zero
  if (ok) {
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    ok = cudaGraphAddNode(&node, G, tail.data(), nullptr, tail.size(), &cp) == cudaSuccess &&
         cp.conditional.phGraph_out != nullptr;
  }
  if (ok) {
    cudaGraph_t bg = cp.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(st, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      t_capture = &n1;
      t_graph_capture = true;
      const int rc = body(cond);
      t_capture = nullptr;
      t_graph_capture = false;
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(st, &g);
      ok = rc == HSS_OK && e == cudaSuccess;
    }
  }
  cudaGraphExec_t ex = nullptr;
  // kernel nodes keep the priority of the stream they were recorded from (the
  // factorization's high-priority stream)
  if (ok && cudaGraphInstantiate(&ex, G, cudaGraphInstantiateFlagUseNodePriority) != cudaSuccess) {
    ex = nullptr;
    ok = false;
  }
  cudaGraphDestroy(G);
  cudaGetLastError();
  if (!ok) return false;
  gc.reset();
  gc.exec = ex;
  gc.key = key;
  gc.launches = n0;
  body_launches = n1;
  return true;
}

// Largest maxit run by the recorded loop (larger ones run the host loop).
constexpr int32_t kLoopMaxIt = 64;

// Solve every item, then refine (FP32 factors, or FP64 with tol > 0) until the
// largest relative residual over all columns of all items is <= tol.
// With graphs enabled on a non-default stream the whole loop is one replayed
// graph: the convergence check runs on the device and sets the condition of a
// while node, and the host reads the loop's status once at the end.
// ready: an event the launches that read the right-hand sides wait for (their
// copy on another stream), or null.
int solve_items(const std::vector<Item>& items, const Levels& L, SolveBufs& B, double tol, int32_t maxit,
                hss_solve_stats* stats, cudaStream_t st, const hss_factor_s* tf = nullptr,
                hss_factor_s* fuse = nullptr, cudaEvent_t ready = nullptr) {
  if (items.empty()) return HSS_OK;
  const int prec = items[0].f->prec;
  for (auto& it : items)
    if (it.f->prec != prec) return fail(HSS_ERR_INVALID, "a batched solve needs factorizations of one precision");
  const bool fp32 = prec == HSS_PREC_FP32;
  // tol < 0: a single solve in the factor's precision, no residual
  const bool refine = tol >= 0.0 && (fp32 || tol > 0.0);
  if (stats) { stats->iterations = 0; stats->converged = refine ? 0 : 1; stats->residual = -1.0; }
  const size_t ni = items.size();
  std::vector<int64_t> off(ni + 1, 0), roff(ni + 1, 0), xoff(ni + 1, 0);
  for (size_t i = 0; i < ni; ++i) {
    hss_plan_s* P = items[i].f->plan;
    off[i + 1] = off[i] + items[i].io.r;
    roff[i + 1] = roff[i] + items[i].io.r * P->tree_m[items[i].tree];
    xoff[i + 1] = xoff[i] + items[i].io.r * P->tree_n[items[i].tree];
  }
  const int64_t rtot = off[ni];
  if (rtot == 0) {
    if (stats) stats->converged = 1;
    if (fuse)
      return fuse->prec == HSS_PREC_FP32 ? factor_impl<float>(fuse, st) : factor_impl<double>(fuse, st);
    return HSS_OK;
  }
  int64_t rmax = 0;
  for (auto& it : items) rmax = std::max(rmax, it.io.r);
  auto first_pass = [&](const double* scale) {
    return fuse ? (fp32 ? factsolve_pass<float>(fuse, items, L, scale, off.data(), rtot, B.sv0, st)
                        : factsolve_pass<double>(fuse, items, L, scale, off.data(), rtot, B.sv0, st))
                : (fp32 ? solve_pass<float>(items, L, scale, off.data(), rtot, 0, false, nullptr, nullptr, B.sv0,
                                            st, tf)
                        : solve_pass<double>(items, L, scale, off.data(), rtot, 0, false, nullptr, nullptr, B.sv0,
                                             st, tf));
  };
  if (!refine) {
    if (ready) CUDA_TRY(cudaStreamWaitEvent(st, ready, 0));
    return first_pass(nullptr);
  }
  CUDA_TRY(B.bn2.ensure(rtot));
  CUDA_TRY(B.rn2.ensure(rtot));
  CUDA_TRY(B.scale.ensure(2 * rtot));
  CUDA_TRY(B.R.ensure(std::max<int64_t>(roff[ni], 1)));
  CUDA_TRY(B.h_bn2.ensure(rtot));
  CUDA_TRY(B.h_rn2.ensure(rtot));
  const double* scale = fp32 ? B.scale.p : nullptr;
  // ||b_j||^2 of every column (and the FP32 column scaling from it)
  auto issue_norms = [&]() -> int {
    CUDA_TRY(cudaMemsetAsync(B.bn2.p, 0, rtot * sizeof(double), st));
    for (size_t i = 0; i < ni; ++i) {
      const Item& it = items[i];
      launch_colnorm2(it.io.B, it.io.ldb, it.f->plan->tree_m[it.tree], it.io.r, B.bn2.p + off[i], st);
      add_launches(1);
    }
    if (fp32) {
      launch_sqrt_scale(B.bn2.p, B.scale.p, rtot, st);
      add_launches(1);
    }
    return HSS_OK;
  };
  // refinement: R = b - A x (double-float product for FP32 factors unless
  // the FP64 product is forced), x += A_f^{-1} R
  bool dfres = fp32 && !g_residual_fp64;
  for (auto& it : items) dfres = dfres && it.f->plan->d_gen_df != nullptr;
  if (dfres) {
    CUDA_TRY(B.xs.ensure(std::max<int64_t>(xoff[ni], 1)));
    CUDA_TRY(B.tmp.ensure(std::max<int64_t>(roff[ni], 1)));
  }
  std::vector<Slot> ms(ni);
  bool dx_slices = dfres && g_tensor_dx;   // every item's plan has its leaf slices prepared
  for (size_t i = 0; i < ni; ++i) {
    const Item& it = items[i];
    hss_plan_s* P = it.f->plan;
    Slot& x = ms[i];
    std::memset(&x, 0, sizeof(Slot));
    x.B = it.io.C; x.ldb = it.io.ldc;                  // current solution
    x.C = B.R.p + roff[i]; x.ldc = P->tree_m[it.tree]; // residual
    x.Y = it.io.B; x.ldy = it.io.ldb;                  // right-hand side
    x.alpha = -1.0; x.beta = 1.0;
    x.r = (int32_t)it.io.r;
    x.colnorm2 = B.rn2.p + off[i];
    x.err = P->d_err;
    x.nodes = P->d_nodes;
    x.sync = P->d_sync;
    if (dfres) {
      CUDA_TRY(it.f->ws2.ensure((size_t)P->ws_mv * rmax));
      x.xs = B.xs.p + xoff[i];
      x.ldx2 = P->tree_n[it.tree];
      x.tmp = B.tmp.p + roff[i];
      x.ldt2 = P->tree_m[it.tree];
      x.ws2 = it.f->ws2.p;
      x.ldws = P->ws_mv;
      x.gdf = P->d_gen_df;
      x.gbase = P->d_gen;
      x.dxs = (g_tensor_dx && ensure_dx(P, st)) ? P->d_dx : nullptr;
      dx_slices = dx_slices && x.dxs != nullptr;
    } else {
      CUDA_TRY(P->mv_ws.ensure((size_t)P->ws_mv * rmax));
      x.ws = P->mv_ws.p;
      x.ldws = P->ws_mv;
    }
  }
  // the tuned residual product of this factor, else the persistent one where it fits
  SlotTable* pm = (tf && tf->tune_pmv == 0) ? nullptr : &B.mv;
  const bool persistent = use_pmv(L, pm, dfres, (int)rmax);
  // R = b - A x and ||R_j||^2 into rn2
  auto issue_residual = [&]() -> int {
    CUDA_TRY(cudaMemsetAsync(B.rn2.p, 0, rtot * sizeof(double), st));
    if (dfres && !persistent)   // the persistent product splits B itself
      for (size_t i = 0; i < ni; ++i) {
        const Item& it = items[i];
        launch_df_split_cols(it.io.C, it.io.ldc, it.f->plan->tree_n[it.tree], it.io.r, B.xs.p + xoff[i], st);
        add_launches(1);
      }
    return dfres ? run_matvec_df(L, B.mv.dev.p, (int)rmax, st, pm, dx_slices)
                 : run_matvec(L, B.mv.dev.p, (int)rmax, st, pm);
  };
  const bool loop_on_device = g_graphs && st != nullptr && g_trace.kind < 0 && g_pick_force < 0 &&
                              maxit >= 0 && maxit <= kLoopMaxIt && ni <= (size_t)INT32_MAX;
  if (loop_on_device) {
    // everything the recorded launches read from the host is made ready here
    PassPrep p0, p1;
    int rc = fuse ? (fp32 ? factsolve_prep<float>(fuse, items, L, scale, off.data(), rtot, B.sv0, st, p0)
                          : factsolve_prep<double>(fuse, items, L, scale, off.data(), rtot, B.sv0, st, p0))
                  : (fp32 ? solve_prep<float>(items, L, scale, off.data(), rtot, 0, false, nullptr, nullptr, B.sv0,
                                              st, tf, p0)
                          : solve_prep<double>(items, L, scale, off.data(), rtot, 0, false, nullptr, nullptr,
                                               B.sv0, st, tf, p0));
    if (rc) return rc;
    rc = fp32 ? solve_prep<float>(items, L, B.scale.p, off.data(), rtot, 1, true, roff.data(), B.R.p, B.sv1, st,
                                  tf, p1)
              : solve_prep<double>(items, L, B.scale.p, off.data(), rtot, 1, true, roff.data(), B.R.p, B.sv1, st,
                                   tf, p1);
    if (rc) return rc;
    CUDA_TRY(B.mv.upload(ms, st));
    if (persistent) CUDA_TRY(pmv_prepare(L, dfres, (int)rmax, *pm, st));
    CUDA_TRY(B.status.ensure(4));
    CUDA_TRY(B.h_status.ensure(4));
    // every address and choice the recorded launches hold
    uint64_t key = fnv(fnv(p0.key, p1.key), levels_key(L, B.mv.dev.p, rmax));
    for (const Item& it : items)
      for (uint64_t v : {(uint64_t)(uintptr_t)it.f, (uint64_t)it.tree, (uint64_t)(uintptr_t)it.io.B,
                         (uint64_t)it.io.ldb, (uint64_t)(uintptr_t)it.io.C, (uint64_t)it.io.ldc, (uint64_t)it.io.r})
        key = fnv(key, v);
    double tolv = tol;
    uint64_t tolbits = 0;
    std::memcpy(&tolbits, &tolv, sizeof(tolbits));
    for (uint64_t v : {(uint64_t)(uintptr_t)fuse, (uint64_t)(uintptr_t)ready, tolbits, (uint64_t)maxit,
                       (uint64_t)fp32, (uint64_t)dfres,
                       (uint64_t)persistent, (uint64_t)dx_slices, (uint64_t)(uintptr_t)pm,
                       (uint64_t)g_generic_factor, (uint64_t)g_flat_product, (uint64_t)pmv_poll_limit(),
                       (uint64_t)(uintptr_t)B.mv.pq.p, (uint64_t)(uintptr_t)B.mv.pstate.p,
                       (uint64_t)(uintptr_t)B.mv.ctb.p, (uint64_t)(uintptr_t)B.mv.dcnt.p,
                       (uint64_t)(uintptr_t)B.bn2.p, (uint64_t)(uintptr_t)B.rn2.p, (uint64_t)(uintptr_t)B.scale.p,
                       (uint64_t)(uintptr_t)B.R.p, (uint64_t)(uintptr_t)B.xs.p, (uint64_t)(uintptr_t)B.tmp.p,
                       (uint64_t)(uintptr_t)B.status.p})
      key = fnv(key, v);
    GraphCache& gc = B.loop;
    RefineStatus* dst = (RefineStatus*)B.status.p;
    auto issue_check = [&](cudaGraphConditionalHandle cond) {
      launch_refine_check(B.bn2.p, B.rn2.p, rtot, tol, maxit, dst, B.mv.dev.p, (int32_t)ni, cond, st);
      add_launches(1);
    };
    bool have = gc.key == key;
    if (!have && gc.seen == key && B.loop_failed != key) {
      have = record_loop(
          gc, key, B.loop_body_launches, st,
          [&](cudaGraphConditionalHandle cond) -> int {
            // the right-hand sides' copy (an external event of the graph), their
            // norms and the status reset: beside the factorization when fused
            const std::function<int()> pre = [&]() -> int {
              if (ready) CUDA_TRY(cudaStreamWaitEvent(st, ready, cudaEventWaitExternal));
              const int e = issue_norms();
              if (e) return e;
              CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(RefineStatus), st));
              return HSS_OK;
            };
            int e = HSS_OK;
            if (fuse) {
              CUDA_TRY(fp32 ? factsolve_issue<float>(fuse, L, B.sv0, p0, st, &pre)
                            : factsolve_issue<double>(fuse, L, B.sv0, p0, st, &pre));
            } else {
              if ((e = pre())) return e;
              if (fp32) solve_issue<float>(L, B.sv0, p0, st, tf);
              else solve_issue<double>(L, B.sv0, p0, st, tf);
            }
            if ((e = issue_residual())) return e;
            issue_check(cond);
            return HSS_OK;
          },
          [&](cudaGraphConditionalHandle cond) -> int {
            launch_sqrt_scale(B.rn2.p, B.scale.p, rtot, st);
            add_launches(1);
            if (fp32) solve_issue<float>(L, B.sv1, p1, st, tf);
            else solve_issue<double>(L, B.sv1, p1, st, tf);
            const int e = issue_residual();
            if (e) return e;
            issue_check(cond);
            return HSS_OK;
          });
      if (!have) {
        B.loop_failed = key;
        g_err.clear();
      }
    }
    if (have) {
      CUDA_TRY(cudaGraphLaunch(gc.exec, st));
      CUDA_TRY(cudaMemcpyAsync(B.h_status.p, dst, sizeof(RefineStatus), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
      RefineStatus rs;
      std::memcpy(&rs, B.h_status.p, sizeof(rs));
      add_launches(gc.launches + B.loop_body_launches * (int64_t)rs.iterations);
      for (auto& it : items) {
        rc = read_dev_err(it.f->plan, st);
        if (rc) return rc;
      }
      if (stats) {
        stats->iterations = rs.iterations;
        stats->residual = rs.residual;
        stats->converged = rs.converged;
      }
      if (rs.converged) return HSS_OK;
      return fail(HSS_ERR_NO_CONVERGENCE, "iterative refinement did not reach the tolerance (residual " +
                                              std::to_string(rs.residual) + ")");
    }
    gc.seen = key;   // recorded on the next call with this key
  }
  // the loop on the host: one read of the residual norms per step
  if (ready) CUDA_TRY(cudaStreamWaitEvent(st, ready, 0));
  int rc = issue_norms();
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(B.h_bn2.p, B.bn2.p, rtot * sizeof(double), cudaMemcpyDeviceToHost, st));
  if ((rc = first_pass(scale))) return rc;
  double res = 0.0;
  for (int32_t iter = 0;; ++iter) {
    CUDA_TRY(B.mv.upload(ms, st));
    rc = issue_residual();
    if (rc) return rc;
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(B.h_rn2.p, B.rn2.p, rtot * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    res = 0.0;
    bool nan = false;
    for (int64_t j = 0; j < rtot; ++j) {
      const double bn = std::sqrt(B.h_bn2.p[j]);
      const double rn = std::sqrt(B.h_rn2.p[j]);
      const double rel = bn > 0.0 ? rn / bn : rn;
      if (std::isnan(rel)) nan = true;
      else if (rel > res) res = rel;
    }
    if (nan) res = std::numeric_limits<double>::quiet_NaN();
    if (stats) { stats->iterations = iter; stats->residual = res; }
    if (res <= tol) {
      if (stats) stats->converged = 1;
      for (auto& it : items) {
        rc = read_dev_err(it.f->plan, st);
        if (rc) return rc;
      }
      return HSS_OK;
    }
    if (iter >= maxit || nan) break;
    launch_sqrt_scale(B.rn2.p, B.scale.p, rtot, st);
    add_launches(1);
    rc = fp32 ? solve_pass<float>(items, L, B.scale.p, off.data(), rtot, 1, true, roff.data(), B.R.p, B.sv1, st, tf)
              : solve_pass<double>(items, L, B.scale.p, off.data(), rtot, 1, true, roff.data(), B.R.p, B.sv1, st, tf);
    if (rc) return rc;
  }
  for (auto& it : items) {
    rc = read_dev_err(it.f->plan, st);
    if (rc) return rc;
  }
  return fail(HSS_ERR_NO_CONVERGENCE, "iterative refinement did not reach the tolerance (residual " +
                                          std::to_string(res) + ")");
}

int solve_impl(hss_factor_s* f, const std::vector<Cols>& io, double tol, int32_t maxit,
               hss_solve_stats* stats, cudaStream_t st, bool refactor = false, cudaEvent_t ready = nullptr) {
  hss_plan_s* P = f->plan;
  int rc = check_cols(P, io, true);
  if (rc) return rc;
  std::vector<Item> items;
  for (int32_t t = 0; t < P->ntrees; ++t) items.push_back(Item{f, t, io[t]});
  return solve_items(items, plan_levels(P), f->bufs, tol, maxit, stats, st, f, refactor ? f : nullptr, ready);
}

// Per-launch times (ms) of the traced kind since hss_trace_begin, in launch order.
std::vector<double> trace_pairs() {
  std::vector<double> t;
  for (size_t i = 0; i + 1 < g_trace.used; i += 2) {
    float ms = 0.f;
    if (cudaEventSynchronize(g_trace.pool[i + 1]) != cudaSuccess ||
        cudaEventElapsedTime(&ms, g_trace.pool[i], g_trace.pool[i + 1]) != cudaSuccess)
      ms = 0.f;
    t.push_back(ms);
  }
  g_trace.kind = -1;
  g_trace.used = 0;
  return t;
}

// The autotuner (hss_autotune): times the kernel variants of every solve level
// and the two residual products on scratch right-hand sides (r columns of
// zeros: the kernels' time does not depend on the values) and keeps the
// faster per level in the factor.
int autotune_impl(hss_factor_s* f, int64_t r, cudaStream_t st) {
  hss_plan_s* P = f->plan;
  const Levels L = plan_levels(P);
  int64_t mtot = 0, ntot = 0;
  for (int32_t t = 0; t < P->ntrees; ++t) {
    mtot += P->tree_m[t];
    ntot += P->tree_n[t];
  }
  DBuf<double> Bs, Xs;
  CUDA_TRY(Bs.ensure((size_t)mtot * r));
  CUDA_TRY(Xs.ensure((size_t)ntot * r));
  CUDA_TRY(cudaMemsetAsync(Bs.p, 0, (size_t)mtot * r * sizeof(double), st));
  std::vector<Item> items;
  int64_t mo = 0, no = 0;
  for (int32_t t = 0; t < P->ntrees; ++t) {
    items.push_back(Item{f, t, Cols{Bs.p + mo, P->tree_m[t], r, Xs.p + no, P->tree_n[t]}});
    mo += P->tree_m[t] * r;
    no += P->tree_n[t] * r;
  }
  f->tune_up.clear();
  f->tune_down.clear();
  f->tune_pmv = -1;
  constexpr int kReps = 3;
  int rc = HSS_OK;
  auto per_level = [&](int kind, int force, const std::vector<Seg>& segs, std::vector<double>& out) -> int {
    g_pick_force = force;
    int e = solve_items(items, L, f->bufs, -1.0, 0, nullptr, st, f);   // warm-up
    if (!e) {
      hss_trace_begin(kind);
      for (int i = 0; i < kReps && !e; ++i) e = solve_items(items, L, f->bufs, -1.0, 0, nullptr, st, f);
      const std::vector<double> t = trace_pairs();
      out.assign(segs.size(), 0.0);
      size_t li = 0;
      for (int i = 0; i < kReps; ++i)
        for (size_t lv = 0; lv < segs.size(); ++lv)
          if (segs[lv].cnt > 0 && li < t.size()) out[lv] += t[li++];
    }
    g_pick_force = -1;
    return e;
  };
  if (f->prec == HSS_PREC_FP32 && f->blocked) {
    std::vector<double> up0, up1, dn0, dn1;
    if ((rc = per_level(HSS_TRACE_SOLVE_UP, 0, P->by_h, up0))) return rc;
    if ((rc = per_level(HSS_TRACE_SOLVE_UP, 1, P->by_h, up1))) return rc;
    if ((rc = per_level(HSS_TRACE_SOLVE_DOWN, 0, P->by_d, dn0))) return rc;
    if ((rc = per_level(HSS_TRACE_SOLVE_DOWN, 1, P->by_d, dn1))) return rc;
    f->tune_up.resize(P->by_h.size());
    f->tune_down.resize(P->by_d.size());
    for (size_t h = 0; h < P->by_h.size(); ++h) f->tune_up[h] = up1[h] < up0[h] ? 1 : 0;
    for (size_t d = 0; d < P->by_d.size(); ++d) f->tune_down[d] = dn1[d] < dn0[d] ? 1 : 0;
  }
  // residual product: one refinement step (solve, residual, correction,
  // residual) with each product; only the product differs between the two
  if (f->prec == HSS_PREC_FP32) {
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    double best[2] = {0.0, 0.0};
    for (int v = 1; v >= 0; --v) {
      f->tune_pmv = v;
      solve_items(items, L, f->bufs, 0.0, 1, nullptr, st, f);   // warm-up (ends without convergence)
      cudaEventRecord(a, st);
      for (int i = 0; i < kReps; ++i) solve_items(items, L, f->bufs, 0.0, 1, nullptr, st, f);
      cudaEventRecord(b, st);
      float ms = 0.f;
      cudaEventSynchronize(b);
      cudaEventElapsedTime(&ms, a, b);
      best[v] = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    f->tune_pmv = best[1] <= best[0] ? 1 : 0;
    g_err.clear();
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  CUDA_TRY(cudaGetLastError());
  return HSS_OK;
}

int copy_in(DBuf<double>& d, const double* h, int64_t rows, int64_t ld, int64_t r, cudaStream_t st) {
  CUDA_TRY(d.ensure((size_t)std::max<int64_t>(rows * r, 1)));
  if (rows * r > 0)
    CUDA_TRY(cudaMemcpy2DAsync(d.p, rows * sizeof(double), h, ld * sizeof(double), rows * sizeof(double),
                               r, cudaMemcpyHostToDevice, st));
  return HSS_OK;
}

int copy_out(double* h, int64_t ld, const double* d, int64_t rows, int64_t r, cudaStream_t st) {
  if (rows * r > 0)
    CUDA_TRY(cudaMemcpy2DAsync(h, ld * sizeof(double), d, rows * sizeof(double), rows * sizeof(double), r,
                               cudaMemcpyDeviceToHost, st));
  return HSS_OK;
}

}  // namespace

// A reusable executor for batches over several independently created plans
// (the serving form): merged task lists and per-call buffers.
struct hss_batcher_s {
  MergedLevels M;
  std::vector<uint64_t> last;      // serial numbers of the plans of the merged lists
  SolveBufs bufs;
  SlotTable fac_slots;
};

namespace {

int batcher_levels(hss_batcher_s* b, const std::vector<hss_plan_s*>& plans, cudaStream_t st) {
  std::vector<uint64_t> ids(plans.size());
  for (size_t i = 0; i < plans.size(); ++i) ids[i] = plans[i]->serial;
  if (ids == b->last && b->M.d.p) return HSS_OK;
  b->last.clear();
  int rc = merge_levels(plans, b->M, st);
  if (rc) return rc;
  b->last = ids;
  return HSS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

namespace hss {

int set_error(int code, const std::string& msg) { return fail(code, msg); }
int set_cuda_error(cudaError_t e, const char* what) { return cuda_fail(e, what); }
void count_launches(int64_t n) { add_launches(n); }

// Armed allocation failure (HSS_OPT_FAIL_ALLOC): 0 = none, k > 0 = the k-th
// allocation from now fails.
std::atomic<int64_t> g_fail_alloc{0};

cudaError_t dev_alloc(void** p, size_t bytes) {
  int64_t k = g_fail_alloc.load();
  while (k > 0) {
    if (g_fail_alloc.compare_exchange_weak(k, k - 1)) {
      if (k == 1) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
      }
      break;
    }
  }
  return cudaMalloc(p, bytes);
}

cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t st) {
  int64_t k = g_fail_alloc.load();
  while (k > 0) {
    if (g_fail_alloc.compare_exchange_weak(k, k - 1)) {
      if (k == 1) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
      }
      break;
    }
  }
  // the device's default pool keeps up to 4 GB of freed blocks for reuse
  // (a setting of this process's pool, not of the device)
  static bool pool_set[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && !pool_set[dev]) {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = uint64_t(4) << 30;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    pool_set[dev] = true;
  }
  return cudaMallocAsync(p, bytes, st);
}

int plan_create_device(int64_t nnodes, const int64_t* table, int64_t npacked, hss_plan_s** out, double** d_gen) {
  *out = nullptr;
  *d_gen = nullptr;
  auto* P = new hss_plan_s();
  int rc = build_plan(P, {TreeIn{nnodes, table, nullptr, npacked}}, true);
  if (rc) { delete P; return rc; }
  *out = P;
  *d_gen = P->d_gen;
  return HSS_OK;
}

void plan_destroy(hss_plan_s* p) { delete p; }

const std::vector<Node>& plan_nodes(const hss_plan_s* p) { return p->nodes; }
const Node* plan_device_nodes(const hss_plan_s* p) { return p->d_nodes; }
int plan_device(const hss_plan_s* p) { return p->device; }
int32_t plan_ntrees(const hss_plan_s* p) { return p->ntrees; }
int64_t plan_rows(const hss_plan_s* p) { return p->tree_m[0]; }
int64_t plan_cols(const hss_plan_s* p) { return p->tree_n[0]; }
const void* factor_storage(const hss_factor_s* f) { return f->d_fac; }
size_t factor_storage_bytes(const hss_factor_s* f) { return f->fac_bytes; }
const double* plan_gen(const hss_plan_s* p, int64_t* len) {
  *len = p->gen_len;
  return p->d_gen;
}

}  // namespace hss

extern "C" {

const char* hss_last_error(void) { return g_err.c_str(); }
int32_t hss_version(void) { return 1; }

int hss_create(int64_t nnodes, const int64_t* nodes, const double* packed, int64_t npacked,
               hss_handle* out) {
  if (!out) return fail(HSS_ERR_INVALID, "null output handle");
  *out = nullptr;
  auto* P = new hss_plan_s();
  int rc = build_plan(P, {TreeIn{nnodes, nodes, packed, npacked}});
  if (rc) { delete P; return rc; }
  *out = P;
  return HSS_OK;
}

int hss_create_batch(int32_t count, const int64_t* nnodes, const int64_t* const* nodes,
                     const double* const* packed, const int64_t* npacked, hss_handle* out) {
  if (!out || count <= 0 || !nnodes || !nodes || !packed || !npacked)
    return fail(HSS_ERR_INVALID, "bad batch arguments");
  *out = nullptr;
  std::vector<TreeIn> trees;
  for (int32_t i = 0; i < count; ++i) trees.push_back(TreeIn{nnodes[i], nodes[i], packed[i], npacked[i]});
  auto* P = new hss_plan_s();
  int rc = build_plan(P, trees);
  if (rc) { delete P; return rc; }
  *out = P;
  return HSS_OK;
}

int hss_inspect(int64_t nnodes, const int64_t* nodes, int64_t npacked, int64_t* info) {
  hss_plan_s P;
  std::vector<GenOffsets> go;
  std::vector<Task> tasks;
  std::vector<int64_t> gbases;
  int rc = layout_plan(&P, {TreeIn{nnodes, nodes, nullptr, npacked}}, go, tasks, gbases);
  if (rc) return rc;
  if (info)
    for (int64_t i = 0; i < nnodes; ++i) {
      const Node& x = P.nodes[i];
      const int64_t v[HSS_INFO_FIELDS] = {x.depth, x.height, x.row0, x.col0, x.m, x.n, x.ku,
                                          x.kv, x.k, x.mk, x.nk, x.leaf, x.tree};
      std::memcpy(info + i * HSS_INFO_FIELDS, v, sizeof(v));
    }
  return HSS_OK;
}

int hss_destroy(hss_handle h) {
  delete h;
  return HSS_OK;
}

int hss_export_size(hss_handle h, int64_t* nnodes, int64_t* npacked) {
  if (!h || h->ntrees != 1 || h->h_table.empty()) return fail(HSS_ERR_INVALID, "export needs a single-tree handle");
  if (nnodes) *nnodes = (int64_t)h->h_table.size() / HSS_NODE_FIELDS;
  if (npacked) *npacked = h->h_npacked;
  return HSS_OK;
}

int hss_export(hss_handle h, int64_t* nodes, double* packed) {
  if (!h || h->ntrees != 1 || h->h_table.empty()) return fail(HSS_ERR_INVALID, "export needs a single-tree handle");
  CUDA_TRY(cudaSetDevice(h->device));
  if (nodes) std::memcpy(nodes, h->h_table.data(), h->h_table.size() * sizeof(int64_t));
  if (packed && h->h_npacked > 0)
    CUDA_TRY(cudaMemcpy(packed, h->d_gen, h->h_npacked * sizeof(double), cudaMemcpyDeviceToHost));
  return HSS_OK;
}

int hss_size(hss_handle h, int32_t tree, int64_t* m, int64_t* n) {
  if (!h || tree < 0 || tree >= h->ntrees) return fail(HSS_ERR_INVALID, "bad handle or tree");
  if (m) *m = h->tree_m[tree];
  if (n) *n = h->tree_n[tree];
  return HSS_OK;
}

int hss_ntrees(hss_handle h, int32_t* count) {
  if (!h || !count) return fail(HSS_ERR_INVALID, "bad handle");
  *count = h->ntrees;
  return HSS_OK;
}

int hss_node_info(hss_handle h, int64_t node, int64_t* f) {
  if (!h || !f || node < 0 || node >= (int64_t)h->nodes.size()) return fail(HSS_ERR_INVALID, "bad node");
  const Node& x = h->nodes[node];
  const int64_t v[HSS_INFO_FIELDS] = {x.depth, x.height, x.row0, x.col0, x.m, x.n, x.ku,
                                      x.kv, x.k, x.mk, x.nk, x.leaf, x.tree};
  std::memcpy(f, v, sizeof(v));
  return HSS_OK;
}

int hss_ulv_cols(hss_handle h, int64_t node, int64_t* cols, int64_t cap, int64_t* len) {
  if (!h || !len || node < 0 || node >= (int64_t)h->nodes.size()) return fail(HSS_ERR_INVALID, "bad node");
  // cols of a leaf: its column range; of a branch: the un-eliminated tails of
  // its children (src/ulvfactor.jl:62,76)
  std::vector<int64_t> out;
  std::vector<int64_t> tmp;
  struct Rec {
    const std::vector<Node>& N;
    void run(int32_t i, std::vector<int64_t>& o) const {
      const Node& x = N[i];
      if (x.leaf) {
        for (int64_t c = 0; c < x.n; ++c) o.push_back(x.col0 + c);
        return;
      }
      std::vector<int64_t> a, b;
      run(x.left, a);
      run(x.right, b);
      const Node& c1 = N[x.left];
      const Node& c2 = N[x.right];
      o.insert(o.end(), a.begin() + c1.nk, a.end());
      o.insert(o.end(), b.begin() + c2.nk, b.end());
    }
  } rec{h->nodes};
  rec.run((int32_t)node, out);
  *len = (int64_t)out.size();
  if (cols) std::memcpy(cols, out.data(), std::min<int64_t>(cap, *len) * sizeof(int64_t));
  return HSS_OK;
}

int hss_matmul(hss_handle h, const double* dB, int64_t ldb, int64_t r, double* dC, int64_t ldc,
               double alpha, double beta, void* stream) {
  if (!h) return fail(HSS_ERR_INVALID, "null handle");
  if (h->ntrees != 1) return fail(HSS_ERR_INVALID, "use hss_matmul_batch for a forest");
  std::vector<Cols> io{Cols{dB, ldb, r, dC, ldc}};
  int rc = check_cols(h, io, false);
  if (rc) return rc;
  return matmul_impl(h, io, alpha, beta, (cudaStream_t)stream, nullptr, nullptr, nullptr, h->mv_slots);
}

int hss_matmul_t(hss_handle h, const double* dB, int64_t ldb, int64_t r, double* dC, int64_t ldc, double alpha,
                 double beta, void* stream) {
  if (!h) return fail(HSS_ERR_INVALID, "null handle");
  if (h->ntrees != 1) return fail(HSS_ERR_INVALID, "the product with the adjoint takes a single matrix");
  if (!h->tplan) {
    CUDA_TRY(cudaSetDevice(h->device));
    int rc = plan_transpose(h, &h->tplan, (cudaStream_t)stream);
    if (rc) return rc;
  }
  return hss_matmul(h->tplan, dB, ldb, r, dC, ldc, alpha, beta, stream);
}

int hss_matmul_noalloc(hss_handle h, const double* dB, int64_t ldb, int64_t r, double* dC, int64_t ldc,
                       double alpha, double beta, void* stream) {
  if (!h) return fail(HSS_ERR_INVALID, "null handle");
  if (h->ntrees != 1) return fail(HSS_ERR_INVALID, "the allocation-free product takes a single matrix");
  std::vector<Cols> io{Cols{dB, ldb, r, dC, ldc}};
  int rc = check_cols(h, io, false);
  if (rc) return rc;
  if (r == 0) return HSS_OK;
  if ((int64_t)h->ws_mv * r > noalloc_ws_capacity())
    return fail(HSS_ERR_BAD_DIMS, "allocation-free product: workspace of " + std::to_string(h->ws_mv) + " rows x " +
                                      std::to_string(r) + " right-hand sides exceeds the fixed scratch of " +
                                      std::to_string(noalloc_ws_capacity()) + " doubles");
  // the plan's node tables live on its device: run there, with that device's scratch
  CUDA_TRY(cudaSetDevice(h->device));
  double* ws = nullptr;
  Slot* dslot = nullptr;
  std::string err;
  rc = noalloc_scratch(h->device, &ws, &dslot, &err);
  if (rc) return fail(rc, err);
  Slot x;
  std::memset(&x, 0, sizeof(Slot));
  x.B = dB; x.ldb = ldb;
  x.C = dC; x.ldc = ldc;
  x.Y = dC; x.ldy = ldc;
  x.alpha = alpha; x.beta = beta;
  x.ws = ws; x.ldws = h->ws_mv;
  x.r = (int32_t)r;
  x.err = h->d_err;
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(noalloc_write_slot(dslot, x, st));
  add_launches(1);
  // level kernels: the persistent product's state would be allocated
  if ((rc = run_matvec(h, dslot, (int)r, st))) return rc;
  CUDA_TRY(cudaGetLastError());
  return HSS_OK;
}

int hss_matmul_batch(hss_handle h, const double* const* dB, const int64_t* ldb, const int64_t* r,
                     double* const* dC, const int64_t* ldc, double alpha, double beta, void* stream) {
  if (!h || !dB || !ldb || !r || !dC || !ldc) return fail(HSS_ERR_INVALID, "bad batch arguments");
  std::vector<Cols> io(h->ntrees);
  for (int32_t t = 0; t < h->ntrees; ++t) io[t] = Cols{dB[t], ldb[t], r[t], dC[t], ldc[t]};
  int rc = check_cols(h, io, false);
  if (rc) return rc;
  return matmul_impl(h, io, alpha, beta, (cudaStream_t)stream, nullptr, nullptr, nullptr, h->mv_slots);
}

int hss_matmul_host(hss_handle h, const double* B, int64_t ldb, int64_t r, double* C, int64_t ldc,
                    double alpha, double beta) {
  if (!h) return fail(HSS_ERR_INVALID, "null handle");
  if (h->ntrees != 1) return fail(HSS_ERR_INVALID, "host product takes a single matrix");
  if (r == 0) return HSS_OK;
  const int64_t m = h->tree_m[0], n = h->tree_n[0];
  std::vector<Cols> io{Cols{B, ldb, r, C, ldc}};
  int rc = check_cols(h, io, false);
  if (rc) return rc;
  cudaStream_t st = 0;
  if ((rc = copy_in(h->hB, B, n, ldb, r, st))) return rc;
  CUDA_TRY(h->hC.ensure((size_t)m * r));
  if (beta != 0.0 && (rc = copy_in(h->hC, C, m, ldc, r, st))) return rc;
  std::vector<Cols> dio{Cols{h->hB.p, n, r, h->hC.p, m}};
  if ((rc = matmul_impl(h, dio, alpha, beta, st, nullptr, nullptr, nullptr, h->mv_slots))) return rc;
  if ((rc = copy_out(C, ldc, h->hC.p, m, r, st))) return rc;
  CUDA_TRY(cudaStreamSynchronize(st));
  return read_dev_err(h, st);   // a persistent product that gave up (HSS_ERR_TIMEOUT)
}

int hss_ulvfactor(hss_handle h, int32_t precision, hss_factor* out, void* stream) {
  if (!h || !out) return fail(HSS_ERR_INVALID, "null handle");
  if (precision != HSS_PREC_FP64 && precision != HSS_PREC_FP32)
    return fail(HSS_ERR_INVALID, "precision must be HSS_PREC_FP64 or HSS_PREC_FP32");
  *out = nullptr;
  if (!h->ulv_why.empty()) return fail(HSS_ERR_BAD_DIMS, h->ulv_why);
  auto* f = new hss_factor_s();
  f->plan = h;
  f->prec = precision;
  const size_t es = precision == HSS_PREC_FP32 ? sizeof(float) : sizeof(double);
  f->fac_bytes = (size_t)h->fac_elems * es;
  cudaError_t e = dev_alloc(&f->d_fac, f->fac_bytes);
  if (e != cudaSuccess) {
    delete f;
    return cuda_fail(e, "device allocation (factor)");
  }
  int rc = precision == HSS_PREC_FP32 ? ensure_df(h, (cudaStream_t)stream) : HSS_OK;
  if (!rc)
    rc = precision == HSS_PREC_FP32 ? factor_impl<float>(f, (cudaStream_t)stream)
                                    : factor_impl<double>(f, (cudaStream_t)stream);
  if (rc) { delete f; return rc; }
  *out = f;
  return HSS_OK;
}

int hss_factor_destroy(hss_factor f) {
  delete f;
  return HSS_OK;
}

int hss_ulvrefactor(hss_factor f, void* stream) {
  if (!f) return fail(HSS_ERR_INVALID, "null factor");
  return f->prec == HSS_PREC_FP32 ? factor_impl<float>(f, (cudaStream_t)stream)
                                  : factor_impl<double>(f, (cudaStream_t)stream);
}

int hss_trace_begin(int32_t kind) {
  if (kind < -1 || kind >= HSS_TRACE_KINDS) return fail(HSS_ERR_INVALID, "unknown trace kind");
  g_trace.kind = kind;
  g_trace.used = 0;
  return HSS_OK;
}

int hss_trace_end(double* total_ms, int64_t* launches) {
  double tot = 0.0;
  int64_t n = 0;
  for (size_t i = 0; i + 1 < g_trace.used; i += 2) {
    float ms = 0.f;
    CUDA_TRY(cudaEventSynchronize(g_trace.pool[i + 1]));
    CUDA_TRY(cudaEventElapsedTime(&ms, g_trace.pool[i], g_trace.pool[i + 1]));
    tot += ms;
    ++n;
  }
  g_trace.kind = -1;
  g_trace.used = 0;
  if (total_ms) *total_ms = tot;
  if (launches) *launches = n;
  return HSS_OK;
}

int hss_trace_times(double* ms, int64_t cap, int64_t* launches) {
  int64_t n = 0;
  for (size_t i = 0; i + 1 < g_trace.used; i += 2) {
    float t = 0.f;
    CUDA_TRY(cudaEventSynchronize(g_trace.pool[i + 1]));
    CUDA_TRY(cudaEventElapsedTime(&t, g_trace.pool[i], g_trace.pool[i + 1]));
    if (ms && n < cap) ms[n] = t;
    ++n;
  }
  g_trace.kind = -1;
  g_trace.used = 0;
  if (launches) *launches = n;
  return HSS_OK;
}

int64_t hss_launch_counter(void) { return g_launches.load(); }

int hss_set_option(int32_t option, int64_t value) {
  if (option == HSS_OPT_GENERIC_FACTOR) {
    g_generic_factor = value != 0;
    return HSS_OK;
  }
  if (option == HSS_OPT_RESIDUAL_FP64) {
    g_residual_fp64 = value != 0;
    return HSS_OK;
  }
  if (option == HSS_OPT_LEVEL_PRODUCT) {
    g_level_product = value != 0;
    return HSS_OK;
  }
  if (option == HSS_OPT_GRAPHS) {
    g_graphs = value != 0;
    return HSS_OK;
  }
  if (option == HSS_OPT_SAMPLE_DF) {
    g_sample_df = value != 0;
    return HSS_OK;
  }
  if (option == HSS_OPT_FLAT_PRODUCT) {
    g_flat_product = value != 0;
    return HSS_OK;
  }
  if (option == HSS_OPT_TENSOR_RESIDUAL) {
    g_tensor_dx = value != 0;
    return HSS_OK;
  }
  if (option == HSS_OPT_FAIL_ALLOC) {
    if (value < 0) return fail(HSS_ERR_INVALID, "allocation-failure countdown must be >= 0");
    g_fail_alloc.store(value);
    return HSS_OK;
  }
  if (option == HSS_OPT_POLL_LIMIT) {
    if (value < 0 || value > 0xffffffffll) return fail(HSS_ERR_INVALID, "poll limit must be in [0, 2^32)");
    pmv_set_poll_limit((uint32_t)value);
    return HSS_OK;
  }
  return fail(HSS_ERR_INVALID, "unknown option");
}

int hss_autotune(hss_factor f, int64_t r, void* stream) {
  if (!f) return fail(HSS_ERR_INVALID, "null factor");
  if (r <= 0 || r > (1 << 16)) return fail(HSS_ERR_BAD_DIMS, "autotune needs 1 <= r <= 65536 right-hand sides");
  return autotune_impl(f, r, (cudaStream_t)stream);
}

int hss_autotune_info(hss_factor f, int32_t* nup, int8_t* up, int32_t* ndown, int8_t* down, int32_t* pmv) {
  if (!f) return fail(HSS_ERR_INVALID, "null factor");
  if (nup) *nup = (int32_t)f->tune_up.size();
  if (ndown) *ndown = (int32_t)f->tune_down.size();
  if (up) std::memcpy(up, f->tune_up.data(), f->tune_up.size());
  if (down) std::memcpy(down, f->tune_down.data(), f->tune_down.size());
  if (pmv) *pmv = f->tune_pmv;
  return HSS_OK;
}

int hss_factor_bytes(hss_factor f, int64_t* bytes) {
  if (!f || !bytes) return fail(HSS_ERR_INVALID, "null factor");
  *bytes = (int64_t)f->fac_bytes;
  return HSS_OK;
}

int hss_device_bytes(hss_handle h, hss_factor f, int64_t* bytes) {
  if (!bytes || (!h && !f)) return fail(HSS_ERR_INVALID, "null handle and factor");
  auto slots = [](const SlotTable& s) {
    return (int64_t)(s.dev.cap * sizeof(Slot) + s.pstate.cap * 4 + s.pq.cap * 8 + s.ctb.cap * 8 + s.dcnt.cap * 4);
  };
  int64_t b = 0;
  if (h) {
    const int64_t nn = (int64_t)h->nodes.size();
    b += h->gen_len * 8;
    if (h->d_gen_df) b += h->gen_len * 8;
    if (h->d_dx) b += h->dx_bytes;
    // node descriptors, task lists, flat-product links, paths and counters
    b += nn * (int64_t)(sizeof(Node) + 4 * sizeof(Task) + sizeof(FlatLink) + 4 * (h->flat_dep + 1));
    b += (int64_t)(h->mv_ws.cap + h->hB.cap + h->hC.cap) * 8 + slots(h->mv_slots);
  }
  if (f) {
    b += (int64_t)f->fac_bytes + (int64_t)f->sv_ws.cap + (int64_t)f->ws2.cap * 8 + slots(f->fac_slots);
    const SolveBufs& q = f->bufs;
    b += (int64_t)(q.R.cap + q.bn2.cap + q.rn2.cap + q.scale.cap + q.xs.cap + q.tmp.cap) * 8;
    b += slots(q.sv0) + slots(q.sv1) + slots(q.mv) + (int64_t)(f->hB.cap + f->hX.cap) * 8;
  }
  *bytes = b;
  return HSS_OK;
}

int hss_ulvsolve(hss_factor f, const double* dB, int64_t ldb, int64_t r, double* dX, int64_t ldx,
                 double tol, int32_t maxit, hss_solve_stats* stats, void* stream) {
  if (!f) return fail(HSS_ERR_INVALID, "null factor");
  if (f->plan->ntrees != 1) return fail(HSS_ERR_INVALID, "use hss_ulvsolve_batch for a forest");
  return solve_impl(f, {Cols{dB, ldb, r, dX, ldx}}, tol, maxit, stats, (cudaStream_t)stream);
}

int hss_ulvfactsolve(hss_factor f, const double* dB, int64_t ldb, int64_t r, double* dX, int64_t ldx, double tol,
                     int32_t maxit, hss_solve_stats* stats, void* stream) {
  if (!f) return fail(HSS_ERR_INVALID, "null factor");
  if (f->plan->ntrees != 1) return fail(HSS_ERR_INVALID, "the fused factorization and solve take a single matrix");
  CUDA_TRY(cudaSetDevice(f->plan->device));
  return solve_impl(f, {Cols{dB, ldb, r, dX, ldx}}, tol, maxit, stats, (cudaStream_t)stream, true);
}

int hss_ulvsolve_batch(hss_factor f, const double* const* dB, const int64_t* ldb, const int64_t* r,
                       double* const* dX, const int64_t* ldx, double tol, int32_t maxit,
                       hss_solve_stats* stats, void* stream) {
  if (!f || !dB || !ldb || !r || !dX || !ldx) return fail(HSS_ERR_INVALID, "bad batch arguments");
  std::vector<Cols> io(f->plan->ntrees);
  for (int32_t t = 0; t < f->plan->ntrees; ++t) io[t] = Cols{dB[t], ldb[t], r[t], dX[t], ldx[t]};
  return solve_impl(f, io, tol, maxit, stats, (cudaStream_t)stream);
}

// The stream of the host-buffer solves: the plan's own non-blocking stream,
// ordered after the work already queued on the legacy default stream, so that
// their launch sequences (and refinement loop) replay as graphs like those of
// the device entry points on a user stream.  The calls return after their
// results are on the host.
int host_stream(hss_plan_s* P, cudaStream_t* out) {
  if (!P->host_st) CUDA_TRY(cudaStreamCreateWithFlags(&P->host_st, cudaStreamNonBlocking));
  if (!P->host_ev) CUDA_TRY(cudaEventCreateWithFlags(&P->host_ev, cudaEventDisableTiming));
  CUDA_TRY(cudaEventRecord(P->host_ev, 0));
  CUDA_TRY(cudaStreamWaitEvent(P->host_st, P->host_ev, 0));
  *out = P->host_st;
  return HSS_OK;
}

int hss_ulvsolve_host(hss_factor f, const double* B, int64_t ldb, int64_t r, double* X, int64_t ldx,
                      double tol, int32_t maxit, hss_solve_stats* stats) {
  if (!f) return fail(HSS_ERR_INVALID, "null factor");
  hss_plan_s* P = f->plan;
  if (P->ntrees != 1) return fail(HSS_ERR_INVALID, "host solve takes a single matrix");
  const int64_t m = P->tree_m[0], n = P->tree_n[0];
  std::vector<Cols> io{Cols{B, ldb, r, X, ldx}};
  int rc = check_cols(P, io, true);
  if (rc) return rc;
  if (r == 0) return HSS_OK;
  cudaStream_t st = 0;
  if ((rc = host_stream(P, &st))) return rc;
  if ((rc = copy_in(f->hB, B, m, ldb, r, st))) return rc;
  CUDA_TRY(f->hX.ensure((size_t)n * r));
  rc = solve_impl(f, {Cols{f->hB.p, m, r, f->hX.p, n}}, tol, maxit, stats, st);
  if (rc && rc != HSS_ERR_NO_CONVERGENCE) return rc;
  int rc2 = copy_out(X, ldx, f->hX.p, n, r, st);
  if (rc2) return rc2;
  CUDA_TRY(cudaStreamSynchronize(st));
  if (!rc) rc = read_dev_err(P, st);
  return rc;
}

int hss_ulvfactsolve_host(hss_handle h, int32_t precision, const double* B, int64_t ldb, int64_t r,
                          double* X, int64_t ldx, double tol, int32_t maxit, hss_solve_stats* stats) {
  if (!h) return fail(HSS_ERR_INVALID, "null handle");
  if (precision != HSS_PREC_FP64 && precision != HSS_PREC_FP32)
    return fail(HSS_ERR_INVALID, "precision must be HSS_PREC_FP64 or HSS_PREC_FP32");
  // the factorization is recomputed on every call; only its storage is reused
  int rc;
  hss_factor& f = h->fused[precision];
  if (f == nullptr) {
    rc = hss_ulvfactor(h, precision, &f, nullptr);
    if (rc) return rc;
    return hss_ulvsolve_host(f, B, ldb, r, X, ldx, tol, maxit, stats);
  }
  // later calls: the factorization pipelined with the first solve pass
  const int64_t m = h->tree_m[0], n = h->tree_n[0];
  std::vector<Cols> io{Cols{B, ldb, r, X, ldx}};
  if ((rc = check_cols(h, io, true))) return rc;
  cudaStream_t st = 0;
  if ((rc = host_stream(h, &st))) return rc;
  // the right-hand sides are copied on a second stream while the
  // factorization (which does not read them) starts
  if (!h->copy_st) CUDA_TRY(cudaStreamCreateWithFlags(&h->copy_st, cudaStreamNonBlocking));
  if (!h->copy_ev) CUDA_TRY(cudaEventCreateWithFlags(&h->copy_ev, cudaEventDisableTiming));
  CUDA_TRY(cudaStreamWaitEvent(h->copy_st, h->host_ev, 0));   // after the legacy default stream's work
  if ((rc = copy_in(f->hB, B, m, ldb, r, h->copy_st))) return rc;
  CUDA_TRY(cudaEventRecord(h->copy_ev, h->copy_st));
  CUDA_TRY(f->hX.ensure((size_t)n * std::max<int64_t>(r, 1)));
  rc = solve_impl(f, {Cols{f->hB.p, m, r, f->hX.p, n}}, tol, maxit, stats, st, true, h->copy_ev);
  if (rc && rc != HSS_ERR_NO_CONVERGENCE) return rc;
  if (r > 0) {
    int rc2 = copy_out(X, ldx, f->hX.p, n, r, st);
    if (rc2) return rc2;
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  if (!rc) rc = read_dev_err(h, st);
  return rc;
}

int hss_batcher_create(hss_batcher* out) {
  if (!out) return fail(HSS_ERR_INVALID, "null output");
  *out = new hss_batcher_s();
  return HSS_OK;
}

int hss_batcher_destroy(hss_batcher b) {
  delete b;
  return HSS_OK;
}

int hss_batcher_factor(hss_batcher b, int32_t count, const hss_handle* hs, int32_t precision, hss_factor* out,
                       void* stream) {
  if (!b || !hs || !out || count <= 0) return fail(HSS_ERR_INVALID, "bad batch arguments");
  if (precision != HSS_PREC_FP64 && precision != HSS_PREC_FP32)
    return fail(HSS_ERR_INVALID, "precision must be HSS_PREC_FP64 or HSS_PREC_FP32");
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<hss_plan_s*> plans(count);
  std::vector<hss_factor_s*> fs(count, nullptr);
  for (int32_t i = 0; i < count; ++i) {
    out[i] = nullptr;
    if (!hs[i] || hs[i]->ntrees != 1) return fail(HSS_ERR_INVALID, "batched factorization takes single-tree plans");
    if (!hs[i]->ulv_why.empty()) return fail(HSS_ERR_BAD_DIMS, hs[i]->ulv_why);
    plans[i] = hs[i];
  }
  int rc = HSS_OK;
  const size_t es = precision == HSS_PREC_FP32 ? sizeof(float) : sizeof(double);
  for (int32_t i = 0; i < count && !rc; ++i) {
    auto* f = new hss_factor_s();
    f->plan = plans[i];
    f->prec = precision;
    f->fac_bytes = (size_t)plans[i]->fac_elems * es;
    cudaError_t e = dev_alloc(&f->d_fac, f->fac_bytes);
    if (e != cudaSuccess) { delete f; rc = cuda_fail(e, "device allocation (factor)"); break; }
    fs[i] = f;
    if (precision == HSS_PREC_FP32) rc = ensure_df(plans[i], st);
  }
  if (!rc) rc = batcher_levels(b, plans, st);
  if (!rc)
    rc = precision == HSS_PREC_FP32 ? factor_items<float>(fs, b->M.view(), b->fac_slots, st)
                                    : factor_items<double>(fs, b->M.view(), b->fac_slots, st);
  if (rc) {
    for (auto* f : fs) delete f;
    return rc;
  }
  for (int32_t i = 0; i < count; ++i) out[i] = fs[i];
  return HSS_OK;
}

int hss_batcher_solve(hss_batcher b, int32_t count, const hss_factor* fs, const double* const* dB,
                      const int64_t* ldb, const int64_t* r, double* const* dX, const int64_t* ldx, double tol,
                      int32_t maxit, hss_solve_stats* stats, void* stream) {
  if (!b || !fs || !dB || !ldb || !r || !dX || !ldx || count <= 0) return fail(HSS_ERR_INVALID, "bad batch arguments");
  std::vector<hss_plan_s*> plans(count);
  std::vector<Item> items(count);
  for (int32_t i = 0; i < count; ++i) {
    if (!fs[i] || fs[i]->plan->ntrees != 1) return fail(HSS_ERR_INVALID, "batched solve takes single-tree factors");
    for (int32_t j = 0; j < i; ++j)
      if (fs[j] == fs[i])
        return fail(HSS_ERR_INVALID, "a factorization appears twice in one batch: join its right-hand sides");
    plans[i] = fs[i]->plan;
    items[i] = Item{fs[i], 0, Cols{dB[i], ldb[i], r[i], dX[i], ldx[i]}};
    int rc = check_cols(plans[i], {items[i].io}, true);
    if (rc) return rc;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc = batcher_levels(b, plans, st);
  if (rc) return rc;
  return solve_items(items, b->M.view(), b->bufs, tol, maxit, stats, st);
}

}  // extern "C"
