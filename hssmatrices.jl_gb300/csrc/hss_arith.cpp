// Host side of the HSS arithmetic on the device (C ABI, include/hssgpu.h):
// entry extraction getindex / full (reference src/hssmatrix.jl:102-153,
// 270-305), the HSS x HSS product (src/matmul.jl:65-117) and
// orthonormalize_generators! / recompress! (src/generators.jl:64-114,
// src/compression.jl:148-260).  Each builds task lists for the kernels of
// hss_getindex.cu, hss_hssmul.cu and hss_recompress.cu, level by level, and
// returns its result in a caller buffer or a new handle.
#include "hssgpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdint>
#include <utility>
#include <vector>

#include "hss_host.h"
#include "hss_internal.h"
#include "hss_launch.h"
#include "hss_stages.h"

using namespace hss;

#define CUDA_TRY(x)                                    \
  do {                                                 \
    cudaError_t e_ = (x);                              \
    if (e_ != cudaSuccess) return set_cuda_error(e_, #x); \
  } while (0)

extern "C" {

// ---- getindex / full (src/hssmatrix.jl:102-153, 270-305) ---------------------

int hss_getindex(hss_handle h, const int64_t* rows, int64_t nr, const int64_t* cols, int64_t nc, double* dOut,
                 int64_t ldo, void* stream) {
  if (!h) return set_error(HSS_ERR_INVALID, "null handle");
  if (plan_ntrees(h) != 1) return set_error(HSS_ERR_INVALID, "getindex takes a single-tree handle");
  if (nr < 0 || nc < 0 || ldo < std::max<int64_t>(1, nr)) return set_error(HSS_ERR_BAD_DIMS, "bad sizes");
  if (nr == 0 || nc == 0) return HSS_OK;
  if (!rows || !cols || !dOut) return set_error(HSS_ERR_INVALID, "null pointer");
  const int64_t m = plan_rows(h), n = plan_cols(h);
  for (int64_t i = 0; i < nr; ++i)
    if (rows[i] < 0 || rows[i] >= m) return set_error(HSS_ERR_BAD_DIMS, "row index out of range");
  for (int64_t j = 0; j < nc; ++j)
    if (cols[j] < 0 || cols[j] >= n) return set_error(HSS_ERR_BAD_DIMS, "column index out of range");
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaSetDevice(plan_device(h)));
  // sorted indices and their output positions (the sortperm of :110)
  auto sorted = [](const int64_t* v, int64_t len, std::vector<int64_t>& val, std::vector<int64_t>& pos) {
    pos.resize(len);
    for (int64_t i = 0; i < len; ++i) pos[i] = i;
    std::stable_sort(pos.begin(), pos.end(), [&](int64_t a, int64_t b) { return v[a] < v[b]; });
    val.resize(len);
    for (int64_t i = 0; i < len; ++i) val[i] = v[pos[i]];
  };
  std::vector<int64_t> R, pr, C, pc;
  sorted(rows, nr, R, pr);
  sorted(cols, nc, C, pc);
  // the restricted tree (_getidx, :117-128): each node's part of the lists
  const int64_t nn = (int64_t)plan_nodes(h).size();
  std::vector<GiRange> rg(nn);
  int64_t ws = 0;
  for (int64_t i = 0; i < nn; ++i) {
    const Node& x = plan_nodes(h)[i];
    GiRange& g = rg[i];
    g.rlo = std::lower_bound(R.begin(), R.end(), x.row0) - R.begin();
    g.rcnt = (std::lower_bound(R.begin(), R.end(), x.row0 + x.gm) - R.begin()) - g.rlo;
    g.clo = std::lower_bound(C.begin(), C.end(), x.col0) - C.begin();
    g.ccnt = (std::lower_bound(C.begin(), C.end(), x.col0 + x.gn) - C.begin()) - g.clo;
  }
  for (int64_t i = 0; i < nn; ++i) {
    const Node& x = plan_nodes(h)[i];
    GiRange& g = rg[i];
    g.ub = ws; ws += x.root ? 0 : g.rcnt * x.ku;
    g.vb = ws; ws += x.root ? 0 : g.ccnt * x.kv;
    g.t12 = g.t21 = ws;
    if (!x.leaf) {
      const Node& c1 = plan_nodes(h)[x.left];
      const Node& c2 = plan_nodes(h)[x.right];
      g.t12 = ws; ws += rg[x.left].rcnt * c2.kv;
      g.t21 = ws; ws += rg[x.right].rcnt * c1.kv;
    }
  }
  // node lists by height (children before parents), leaves, tiles of every off-diagonal block
  int max_h = 0;
  for (const Node& x : plan_nodes(h)) max_h = std::max(max_h, (int)x.height);
  std::vector<int32_t> lists, leaves;
  std::vector<int64_t> loff;
  for (int hh = 0; hh <= max_h; ++hh) {
    loff.push_back((int64_t)lists.size());
    for (int64_t i = 0; i < nn; ++i)
      if (plan_nodes(h)[i].height == hh) lists.push_back((int32_t)i);
  }
  loff.push_back((int64_t)lists.size());
  for (int64_t i = 0; i < nn; ++i)
    if (plan_nodes(h)[i].leaf) leaves.push_back((int32_t)i);
  std::vector<GiTile> tiles;
  const int TTR = gi_tile_rows();
  auto add_block = [&](int64_t T, int64_t ldt, int64_t V, int64_t ldv, int64_t rs, int64_t nrows, int64_t cs,
                       int64_t ncols, int k) {
    for (int64_t r0 = 0; r0 < nrows; r0 += TTR)
      for (int64_t c0 = 0; c0 < ncols; c0 += TTR) {
        GiTile t{};
        t.T = T; t.V = V; t.ldt = std::max<int64_t>(ldt, 1); t.ldv = std::max<int64_t>(ldv, 1);
        t.rs = rs; t.cs = cs;
        t.r0 = (int32_t)r0; t.c0 = (int32_t)c0;
        t.rows = (int32_t)std::min<int64_t>(TTR, nrows - r0);
        t.cols = (int32_t)std::min<int64_t>(TTR, ncols - c0);
        t.k = k;
        tiles.push_back(t);
      }
  };
  for (int64_t i = 0; i < nn; ++i) {
    const Node& x = plan_nodes(h)[i];
    if (x.leaf) continue;
    const GiRange &g = rg[i], &g1 = rg[x.left], &g2 = rg[x.right];
    const Node &c1 = plan_nodes(h)[x.left], &c2 = plan_nodes(h)[x.right];
    if (g1.rcnt > (int64_t)INT32_MAX || g2.rcnt > (int64_t)INT32_MAX) return set_error(HSS_ERR_BAD_DIMS, "too many indices");
    add_block(g.t12, g1.rcnt, g2.vb, g2.ccnt, g1.rlo, g1.rcnt, g2.clo, g2.ccnt, c2.kv);   // A12 block
    add_block(g.t21, g2.rcnt, g1.vb, g1.ccnt, g2.rlo, g2.rcnt, g1.clo, g1.ccnt, c1.kv);   // A21 block
  }
  // device copies (stream-ordered scratch)
  int64_t *dR = nullptr, *dC = nullptr, *dpr = nullptr, *dpc = nullptr;
  GiRange* drg = nullptr;
  GiTile* dtl = nullptr;
  int32_t *dlists = nullptr, *dleaves = nullptr;
  double* dws = nullptr;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](auto** p, size_t count) {
    if (e == cudaSuccess) e = cudaMallocAsync((void**)p, std::max<size_t>(count, 1) * sizeof(**p), st);
  };
  auto put = [&](auto* d, const auto& v) {
    if (e == cudaSuccess && !v.empty())
      e = cudaMemcpyAsync(d, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice, st);
  };
  alloc(&dR, nr); alloc(&dC, nc); alloc(&dpr, nr); alloc(&dpc, nc);
  alloc(&drg, nn); alloc(&dtl, tiles.size()); alloc(&dlists, lists.size()); alloc(&dleaves, leaves.size());
  alloc(&dws, (size_t)ws);
  put(dR, R); put(dC, C); put(dpr, pr); put(dpc, pc); put(drg, rg); put(dtl, tiles); put(dlists, lists);
  put(dleaves, leaves);
  if (e == cudaSuccess) {
    for (int hh = 0; hh <= max_h; ++hh) {
      const int64_t cnt = loff[hh + 1] - loff[hh];
      if (cnt > 0) {
        launch_gi_basis(plan_device_nodes(h), drg, dlists + loff[hh], cnt, dR, dC, dws, st);
        count_launches(1);
      }
    }
    if (!tiles.empty()) {
      launch_gi_blocks(dtl, (int64_t)tiles.size(), dws, dpr, dpc, dOut, ldo, st);
      count_launches(1);
    }
    launch_gi_leaves(plan_device_nodes(h), drg, dleaves, (int64_t)leaves.size(), dR, dC, dpr, dpc, dOut, ldo, st);
    count_launches(1);
    e = cudaGetLastError();
  }
  // pageable sources: the copies were staged before the calls returned
  for (void* p : {(void*)dR, (void*)dC, (void*)dpr, (void*)dpc, (void*)drg, (void*)dtl, (void*)dlists,
                  (void*)dleaves, (void*)dws})
    if (p) cudaFreeAsync(p, st);
  if (e != cudaSuccess) return set_cuda_error(e, "getindex");
  return HSS_OK;
}

// ---- HSS x HSS product (src/matmul.jl:65-117) --------------------------------

int hss_hssmul(hss_handle hA, hss_handle hB, hss_handle* out, void* stream) {
  if (!hA || !hB || !out) return set_error(HSS_ERR_INVALID, "null handle");
  *out = nullptr;
  if (plan_ntrees(hA) != 1 || plan_ntrees(hB) != 1) return set_error(HSS_ERR_INVALID, "hssmul takes single-tree handles");
  const std::vector<Node>& NA = plan_nodes(hA);
  const std::vector<Node>& NB = plan_nodes(hB);
  const int64_t nn = (int64_t)NA.size();
  bool match = (int64_t)NB.size() == nn;
  for (int64_t i = 0; match && i < nn; ++i)
    match = NA[i].leaf == NB[i].leaf && NA[i].left == NB[i].left && NA[i].right == NB[i].right &&
            NA[i].gn == NB[i].gm;
  if (!match) return set_error(HSS_ERR_BAD_DIMS, "Clusters don't seem to match");
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaSetDevice(plan_device(hA)));
  // the product's node table: the same tree, ranks adding up
  std::vector<int32_t> kuC(nn), kvC(nn);
  for (int64_t i = 0; i < nn; ++i) {
    kuC[i] = NA[i].ku + NB[i].ku;
    kvC[i] = NA[i].kv + NB[i].kv;
  }
  std::vector<int64_t> table(nn * HSS_NODE_FIELDS, -1);
  int64_t npk = 0;
  auto blk = [&](int64_t rows, int64_t cols) -> int64_t {
    if (rows * cols == 0) return -1;
    const int64_t o = npk;
    npk += rows * cols;
    return o;
  };
  for (int64_t i = 0; i < nn; ++i) {
    const Node& a = NA[i];
    const Node& b = NB[i];
    int64_t* f = &table[i * HSS_NODE_FIELDS];
    f[0] = a.leaf ? -1 : a.left;
    f[1] = a.leaf ? -1 : a.right;
    f[2] = a.leaf ? a.gm : 0;
    f[3] = a.leaf ? b.gn : 0;
    f[4] = kuC[i];
    f[5] = kvC[i];
    f[15] = 0;
    if (a.leaf) {
      f[6] = blk(a.gm, b.gn);
      f[7] = blk(a.gm, kuC[i]);
      f[8] = blk(b.gn, kvC[i]);
    } else {
      f[9] = blk(kuC[a.left], kvC[a.right]);
      f[10] = blk(kuC[a.right], kvC[a.left]);
      f[11] = blk(kuC[a.left], kuC[i]);
      f[12] = blk(kuC[a.right], kuC[i]);
      f[13] = blk(kvC[a.left], kvC[i]);
      f[14] = blk(kvC[a.right], kvC[i]);
    }
  }
  hss_plan_s* PC = nullptr;
  double* dgen = nullptr;
  int rc = plan_create_device(nn, table.data(), npk, &PC, &dgen);
  if (rc) return rc;
  const std::vector<Node>& NC = plan_nodes(PC);
  // workspace: Z, F per non-root node; T1, T2, G1, G2, H1, H2 per branch; H per leaf
  struct Ws { int64_t Z = -1, F = -1, T1 = -1, T2 = -1, G1 = -1, G2 = -1, H1 = -1, H2 = -1, H = -1; };
  std::vector<Ws> w(nn);
  int64_t wtot = 0;
  auto wal = [&](int64_t rows, int64_t cols) { const int64_t o = wtot; wtot += std::max<int64_t>(rows * cols, 0); return o; };
  for (int64_t i = 0; i < nn; ++i) {
    const Node& a = NA[i];
    const Node& b = NB[i];
    if (!a.root) {
      w[i].Z = wal(a.kv, b.ku);
      w[i].F = wal(a.ku, b.kv);
    }
    if (a.leaf) {
      if (!a.root) w[i].H = wal(a.ku, b.gn);
    } else {
      const Node &a1 = NA[a.left], &a2 = NA[a.right], &b1 = NB[b.left], &b2 = NB[b.right];
      w[i].T1 = wal(a1.kv, b.ku);
      w[i].T2 = wal(a2.kv, b.ku);
      w[i].G1 = wal(a2.kv, b1.kv);
      w[i].G2 = wal(a1.kv, b2.kv);
      w[i].H1 = wal(a.ku, b1.kv);
      w[i].H2 = wal(a.ku, b2.kv);
    }
  }
  double* ws = nullptr;
  MmTask* dtasks = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&ws, std::max<int64_t>(wtot, 1) * sizeof(double), st);
  if (e != cudaSuccess) {
    plan_destroy(PC);
    return set_cuda_error(e, "hssmul workspace");
  }
  auto W = [&](int64_t o) { return ws + o; };
  // task builders: C (m x n) = a1 op(A1) op(B1) [+ op(A2) op(B2)]; copies; zero fills
  std::vector<std::vector<MmTask>> stages;
  auto stage = [&]() { stages.emplace_back(); };
  auto ld1 = [](int64_t v) { return (int32_t)std::max<int64_t>(v, 1); };
  auto mm = [&](double* C, int64_t ldc, int64_t m, int64_t n, const double* A1, int64_t lda1, int ta1, const double* B1,
                int64_t ldb1, int tb1, int64_t k1, const double* A2 = nullptr, int64_t lda2 = 1, int ta2 = 0,
                const double* B2 = nullptr, int64_t ldb2 = 1, int tb2 = 0, int64_t k2 = 0) {
    if (m * n == 0) return;
    MmTask t{};
    t.A1 = k1 > 0 ? A1 : nullptr; t.B1 = B1; t.A2 = k2 > 0 ? A2 : nullptr; t.B2 = B2; t.C = C;
    t.lda1 = ld1(lda1); t.ldb1 = ld1(ldb1); t.lda2 = ld1(lda2); t.ldb2 = ld1(ldb2); t.ldc = ld1(ldc);
    t.m = (int32_t)m; t.n = (int32_t)n; t.k1 = (int32_t)std::max<int64_t>(k1, 0); t.k2 = (int32_t)std::max<int64_t>(k2, 0);
    t.ta1 = ta1; t.tb1 = tb1; t.ta2 = ta2; t.tb2 = tb2;
    t.a1 = 1.0; t.a2 = 1.0; t.beta = 0.0;
    stages.back().push_back(t);
  };
  auto cp = [&](double* C, int64_t ldc, int64_t m, int64_t n, const double* A, int64_t lda) {
    if (m * n == 0) return;
    MmTask t{};
    t.A1 = A; t.C = C; t.lda1 = ld1(lda); t.ldc = ld1(ldc); t.m = (int32_t)m; t.n = (int32_t)n; t.k1 = -1;
    stages.back().push_back(t);
  };
  int max_h = 0, max_d = 0;
  for (const Node& a : NA) { max_h = std::max(max_h, (int)a.height); max_d = std::max(max_d, (int)a.depth); }
  // upsweep (matmul.jl:86-94): Z = V_A^T U_B; Z = W1_A^T (Z1 R1_B) + W2_A^T (Z2 R2_B)
  for (int h = 0; h <= max_h; ++h) {
    stage();
    for (int64_t i = 0; i < nn; ++i) {
      const Node& a = NA[i];
      const Node& b = NB[i];
      if (a.height != h || a.leaf || a.root) continue;
      const Node &a1 = NA[a.left], &a2 = NA[a.right], &b1 = NB[b.left], &b2 = NB[b.right];
      mm(W(w[i].T1), a1.kv, a1.kv, b.ku, W(w[a.left].Z), a1.kv, 0, b.R1, b1.ku, 0, b1.ku);
      mm(W(w[i].T2), a2.kv, a2.kv, b.ku, W(w[a.right].Z), a2.kv, 0, b.R2, b2.ku, 0, b2.ku);
    }
    stage();
    for (int64_t i = 0; i < nn; ++i) {
      const Node& a = NA[i];
      const Node& b = NB[i];
      if (a.height != h || a.root) continue;
      if (a.leaf) {
        mm(W(w[i].Z), a.kv, a.kv, b.ku, a.V, a.gn, 1, b.U, b.gm, 0, a.gn);
      } else {
        const Node &a1 = NA[a.left], &a2 = NA[a.right];
        mm(W(w[i].Z), a.kv, a.kv, b.ku, a.W1, a1.kv, 1, W(w[i].T1), a1.kv, 0, a1.kv, a.W2, a2.kv, 1, W(w[i].T2),
           a2.kv, 0, a2.kv);
      }
    }
  }
  // downsweep (:72-73, :104-105): F1 = B12_A (Z2 B21_B) + R1_A (F W1_B^T), F2 = B21_A (Z1 B12_B) + R2_A (F W2_B^T)
  for (int d = 0; d <= max_d; ++d) {
    stage();
    for (int64_t i = 0; i < nn; ++i) {
      const Node& a = NA[i];
      const Node& b = NB[i];
      if (a.depth != d || a.leaf) continue;
      const Node &a1 = NA[a.left], &a2 = NA[a.right], &b1 = NB[b.left], &b2 = NB[b.right];
      mm(W(w[i].G1), a2.kv, a2.kv, b1.kv, W(w[a.right].Z), a2.kv, 0, b.B21, b2.ku, 0, b2.ku);
      mm(W(w[i].G2), a1.kv, a1.kv, b2.kv, W(w[a.left].Z), a1.kv, 0, b.B12, b1.ku, 0, b1.ku);
      if (!a.root) {
        mm(W(w[i].H1), a.ku, a.ku, b1.kv, W(w[i].F), a.ku, 0, b.W1, b1.kv, 1, b.kv);
        mm(W(w[i].H2), a.ku, a.ku, b2.kv, W(w[i].F), a.ku, 0, b.W2, b2.kv, 1, b.kv);
      }
    }
    stage();
    for (int64_t i = 0; i < nn; ++i) {
      const Node& a = NA[i];
      const Node& b = NB[i];
      if (a.depth != d || a.leaf) continue;
      const Node &a1 = NA[a.left], &a2 = NA[a.right], &b1 = NB[b.left], &b2 = NB[b.right];
      const int64_t kp = a.root ? 0 : a.ku;
      mm(W(w[a.left].F), a1.ku, a1.ku, b1.kv, a.B12, a1.ku, 0, W(w[i].G1), a2.kv, 0, a2.kv, a.R1, a1.ku, 0,
         W(w[i].H1), a.ku, 0, kp);
      mm(W(w[a.right].F), a2.ku, a2.ku, b2.kv, a.B21, a2.ku, 0, W(w[i].G2), a1.kv, 0, a1.kv, a.R2, a2.ku, 0,
         W(w[i].H2), a.ku, 0, kp);
    }
  }
  // assembly (:98-101, :106-111)
  stage();
  for (int64_t i = 0; i < nn; ++i) {
    const Node& a = NA[i];
    const Node& b = NB[i];
    if (a.leaf && !a.root) mm(W(w[i].H), a.ku, a.ku, b.gn, W(w[i].F), a.ku, 0, b.V, b.gn, 1, b.kv);
  }
  stage();
  for (int64_t i = 0; i < nn; ++i) {
    const Node& a = NA[i];
    const Node& b = NB[i];
    const Node& c = NC[i];
    if (a.leaf) {
      const int64_t m = a.gm, n = b.gn, p = a.gn;
      const int64_t ku = a.root ? 0 : a.ku;
      mm((double*)c.D, m, m, n, a.D, m, 0, b.D, p, 0, p, a.U, m, 0, W(w[i].H), std::max<int64_t>(a.ku, 1), 0, ku);
      if (!a.root) {
        cp((double*)c.U, m, m, a.ku, a.U, m);
        mm((double*)c.U + m * a.ku, m, m, b.ku, a.D, m, 0, b.U, p, 0, p);
        mm((double*)c.V, n, n, a.kv, b.D, p, 1, a.V, p, 0, p);
        cp((double*)c.V + n * a.kv, n, n, b.kv, b.V, n);
      }
      continue;
    }
    const Node &a1 = NA[a.left], &a2 = NA[a.right], &b1 = NB[b.left], &b2 = NB[b.right];
    const int64_t kp = a.root ? 0 : a.ku;
    const int64_t u1 = kuC[a.left], u2 = kuC[a.right], v1 = kvC[a.left], v2 = kvC[a.right];
    // B12 = [B12_A, R1_A F W2_B^T; 0, B12_B], B21 likewise
    double* B12 = (double*)c.B12;
    cp(B12, u1, a1.ku, a2.kv, a.B12, a1.ku);
    mm(B12 + u1 * a2.kv, u1, a1.ku, b2.kv, a.R1, a1.ku, 0, W(w[i].H2), a.ku, 0, kp);
    cp(B12 + a1.ku, u1, b1.ku, a2.kv, nullptr, 1);
    cp(B12 + a1.ku + u1 * a2.kv, u1, b1.ku, b2.kv, b.B12, b1.ku);
    double* B21 = (double*)c.B21;
    cp(B21, u2, a2.ku, a1.kv, a.B21, a2.ku);
    mm(B21 + u2 * a1.kv, u2, a2.ku, b1.kv, a.R2, a2.ku, 0, W(w[i].H1), a.ku, 0, kp);
    cp(B21 + a2.ku, u2, b2.ku, a1.kv, nullptr, 1);
    cp(B21 + a2.ku + u2 * a1.kv, u2, b2.ku, b1.kv, b.B21, b2.ku);
    if (a.root) continue;
    // R1 = [R1_A, B12_A Z2 R2_B; 0, R1_B], R2 = [R2_A, B21_A Z1 R1_B; 0, R2_B]
    double* R1 = (double*)c.R1;
    cp(R1, u1, a1.ku, a.ku, a.R1, a1.ku);
    mm(R1 + u1 * a.ku, u1, a1.ku, b.ku, a.B12, a1.ku, 0, W(w[i].T2), a2.kv, 0, a2.kv);
    cp(R1 + a1.ku, u1, b1.ku, a.ku, nullptr, 1);
    cp(R1 + a1.ku + u1 * a.ku, u1, b1.ku, b.ku, b.R1, b1.ku);
    double* R2 = (double*)c.R2;
    cp(R2, u2, a2.ku, a.ku, a.R2, a2.ku);
    mm(R2 + u2 * a.ku, u2, a2.ku, b.ku, a.B21, a2.ku, 0, W(w[i].T1), a1.kv, 0, a1.kv);
    cp(R2 + a2.ku, u2, b2.ku, a.ku, nullptr, 1);
    cp(R2 + a2.ku + u2 * a.ku, u2, b2.ku, b.ku, b.R2, b2.ku);
    // W1 = [W1_A, 0; (Z2 B21_B)^T W2_A, W1_B], W2 = [W2_A, 0; (Z1 B12_B)^T W1_A, W2_B]
    double* W1 = (double*)c.W1;
    cp(W1, v1, a1.kv, a.kv, a.W1, a1.kv);
    cp(W1 + v1 * a.kv, v1, a1.kv, b.kv, nullptr, 1);
    mm(W1 + a1.kv, v1, b1.kv, a.kv, W(w[i].G1), a2.kv, 1, a.W2, a2.kv, 0, a2.kv);
    cp(W1 + a1.kv + v1 * a.kv, v1, b1.kv, b.kv, b.W1, b1.kv);
    double* W2 = (double*)c.W2;
    cp(W2, v2, a2.kv, a.kv, a.W2, a2.kv);
    cp(W2 + v2 * a.kv, v2, a2.kv, b.kv, nullptr, 1);
    mm(W2 + a2.kv, v2, b2.kv, a.kv, W(w[i].G2), a1.kv, 1, a.W1, a1.kv, 0, a1.kv);
    cp(W2 + a2.kv + v2 * a.kv, v2, b2.kv, b.kv, b.W2, b2.kv);
  }
  // one upload, one launch per non-empty stage
  std::vector<MmTask> all;
  std::vector<std::pair<int64_t, int64_t>> ranges;
  for (auto& sg : stages) {
    if (sg.empty()) continue;
    split_mm_columns(sg);   // wide assembly blocks at the upper levels
    ranges.emplace_back((int64_t)all.size(), (int64_t)sg.size());
    all.insert(all.end(), sg.begin(), sg.end());
  }
  if (!all.empty()) {
    e = cudaMallocAsync((void**)&dtasks, all.size() * sizeof(MmTask), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dtasks, all.data(), all.size() * sizeof(MmTask), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      for (auto& r : ranges) launch_mm_list(dtasks + r.first, r.second, st);
      count_launches((int64_t)ranges.size());
      e = cudaGetLastError();
    }
    // the pageable task copy was staged before cudaMemcpyAsync returned
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (dtasks) cudaFreeAsync(dtasks, st);
  cudaFreeAsync(ws, st);
  if (e != cudaSuccess) {
    plan_destroy(PC);
    return set_cuda_error(e, "hssmul");
  }
  *out = PC;
  return HSS_OK;
}

// ---- orthonormalize_generators! / recompress! (src/generators.jl:64-114,
// src/compression.jl:148-260) ----------------------------------------------------

}  // extern "C"

namespace hss {

// orthonormalize_generators! and, unless ortho_only, the truncation of
// recompress!; the result is a new single-tree handle.
int recompress_impl(hss_plan_s* h, double atol, double rtol, bool ortho_only, hss_plan_s** out, cudaStream_t st) {
  const std::vector<Node>& N = plan_nodes(h);
  const int64_t nn = (int64_t)N.size();
  Arena ar;
  ar.on_stream(st);
  Stages S{st, ar, {}, {}};
  struct G { Blk D, U, V, B12, B21, R1, R2, W1, W2, RU, RV; };
  std::vector<G> g(nn);
  // the handle's generators, read in place (never written)
  for (int64_t i = 0; i < nn; ++i) {
    const Node& x = N[i];
    auto gb = [](const double* p, int64_t r, int64_t c) { Blk b; b.p = (double*)p; b.rows = r; b.cols = c; b.ld = std::max<int64_t>(r, 1); return b; };
    if (x.leaf) {
      g[i].D = gb(x.D, x.gm, x.gn);
      g[i].U = gb(x.U, x.gm, x.ku);
      g[i].V = gb(x.V, x.gn, x.kv);
    } else {
      const Node &c1 = N[x.left], &c2 = N[x.right];
      g[i].B12 = gb(x.B12, c1.ku, c2.kv);
      g[i].B21 = gb(x.B21, c2.ku, c1.kv);
      g[i].R1 = gb(x.R1, c1.ku, x.ku);
      g[i].R2 = gb(x.R2, c2.ku, x.ku);
      g[i].W1 = gb(x.W1, c1.kv, x.kv);
      g[i].W2 = gb(x.W2, c2.kv, x.kv);
    }
  }
  const double rtol0 = 5 * 2.220446049250313e-16;   // pqrfact's default relative tolerance (assumed 5 eps)
  cudaError_t e = cudaSuccess;
  std::vector<int32_t> rk;
  int max_h = 0, max_d = 0;
  for (const Node& x : N) { max_h = std::max(max_h, (int)x.height); max_d = std::max(max_d, (int)x.depth); }
  // ---- orthonormalize (bottom-up) ----
  for (int hh = 0; hh <= max_h && e == cudaSuccess; ++hh) {
    // branches: the children's R factors into B, R, W (generators.jl:106-112)
    std::vector<std::array<Blk, 2>> tmp(nn);
    for (int64_t i = 0; i < nn; ++i) {
      const Node& x = N[i];
      if (x.height != hh || x.leaf) continue;
      G& a = g[i];
      const G &c1 = g[x.left], &c2 = g[x.right];
      tmp[i][0] = ar.blk(c1.RU.rows, a.B12.cols);
      tmp[i][1] = ar.blk(c2.RU.rows, a.B21.cols);
      S.gemm(tmp[i][0], c1.RU, 0, a.B12, 0);
      S.gemm(tmp[i][1], c2.RU, 0, a.B21, 0);
      Blk R1 = ar.blk(c1.RU.rows, a.R1.cols), R2 = ar.blk(c2.RU.rows, a.R2.cols);
      Blk W1 = ar.blk(c1.RV.rows, a.W1.cols), W2 = ar.blk(c2.RV.rows, a.W2.cols);
      S.gemm(R1, c1.RU, 0, a.R1, 0); S.gemm(R2, c2.RU, 0, a.R2, 0);
      S.gemm(W1, c1.RV, 0, a.W1, 0); S.gemm(W2, c2.RV, 0, a.W2, 0);
      a.R1 = R1; a.R2 = R2; a.W1 = W1; a.W2 = W2;
    }
    if ((e = S.run_mm()) != cudaSuccess) break;
    for (int64_t i = 0; i < nn; ++i) {
      const Node& x = N[i];
      if (x.height != hh || x.leaf) continue;
      G& a = g[i];
      const G &c1 = g[x.left], &c2 = g[x.right];
      Blk B12 = ar.blk(tmp[i][0].rows, c2.RV.rows), B21 = ar.blk(tmp[i][1].rows, c1.RV.rows);
      S.gemm(B12, tmp[i][0], 0, c2.RV, 1);
      S.gemm(B21, tmp[i][1], 0, c1.RV, 1);
      a.B12 = B12; a.B21 = B21;
    }
    if ((e = S.run_mm()) != cudaSuccess) break;
    // non-root nodes: QR of U (leaf) or [R1; R2] (branch), V / [W1; W2] likewise (:66-103)
    std::vector<int64_t> who;
    std::vector<std::array<Blk, 4>> qrs;   // QU, RU, QV, RV
    for (int64_t i = 0; i < nn; ++i) {
      const Node& x = N[i];
      if (x.height != hh || x.root) continue;
      G& a = g[i];
      Blk GU, GV;
      if (x.leaf) {
        GU = ar.blk(a.U.rows, a.U.cols); S.copy(GU, a.U);
        GV = ar.blk(a.V.rows, a.V.cols); S.copy(GV, a.V);
      } else {
        GU = ar.blk(a.R1.rows + a.R2.rows, a.R1.cols);
        Blk top = GU; top.rows = a.R1.rows; S.copy(top, a.R1);
        Blk bot = GU; bot.p = GU.at(a.R1.rows, 0); bot.rows = a.R2.rows; S.copy(bot, a.R2);
        GV = ar.blk(a.W1.rows + a.W2.rows, a.W1.cols);
        Blk vt = GV; vt.rows = a.W1.rows; S.copy(vt, a.W1);
        Blk vb = GV; vb.p = GV.at(a.W1.rows, 0); vb.rows = a.W2.rows; S.copy(vb, a.W2);
      }
      auto U = S.pqr(GU, 0.0, rtol0);
      auto V = S.pqr(GV, 0.0, rtol0);
      who.push_back(i);
      qrs.push_back({U.first, U.second, V.first, V.second});
    }
    if ((e = S.run_mm()) != cudaSuccess) break;
    // pqr tasks were queued in (U, V) pairs per node; empty blocks queue nothing
    std::vector<int32_t> rks;
    {
      // ranks in queue order: rebuild the per-node mapping from the block sizes
      if ((e = S.run_qr(rks)) != cudaSuccess) break;
    }
    size_t qi = 0;
    for (size_t w = 0; w < who.size(); ++w) {
      const int64_t i = who[w];
      const Node& x = N[i];
      G& a = g[i];
      auto take = [&](const Blk& Q, const Blk& R, int64_t rows) {
        int32_t r = 0;
        if (rows * R.cols > 0) r = rks[qi++];
        Blk q = Q; q.cols = r;
        Blk rr = R; rr.rows = r;
        return std::make_pair(q, rr);
      };
      auto U = take(qrs[w][0], qrs[w][1], qrs[w][0].rows);
      auto V = take(qrs[w][2], qrs[w][3], qrs[w][2].rows);
      a.RU = U.second;
      a.RV = V.second;
      if (x.leaf) {
        a.U = U.first;
        a.V = V.first;
      } else {
        Blk r1 = U.first; r1.rows = a.R1.rows;
        Blk r2 = U.first; r2.p = U.first.at(a.R1.rows, 0); r2.rows = a.R2.rows;
        Blk w1 = V.first; w1.rows = a.W1.rows;
        Blk w2 = V.first; w2.p = V.first.at(a.W1.rows, 0); w2.rows = a.W2.rows;
        a.R1 = r1; a.R2 = r2; a.W1 = w1; a.W2 = w2;
      }
    }
  }
  if (e == cudaSuccess && ar.err != cudaSuccess) e = ar.err;
  // ---- truncation (top-down, compression.jl:157-260) ----
  struct RC { Blk Brow, Bcol; bool has = false; };
  std::vector<RC> rc(nn);
  for (int d = 0; d <= max_d && e == cudaSuccess && !ortho_only; ++d) {
    // the stacked couplings of every branch at depth d
    struct Q4 { Blk B1, B2, B3, B4; std::pair<Blk, Blk> f1, f2, f3, f4; int64_t rm1, rn2, rm2, rn1; };
    std::vector<int64_t> who;
    std::vector<Q4> q4;
    for (int64_t i = 0; i < nn; ++i) {
      const Node& x = N[i];
      if (x.depth != d || x.leaf) continue;
      G& a = g[i];
      Q4 t;
      t.rm1 = a.B12.rows; t.rn2 = a.B12.cols; t.rm2 = a.B21.rows; t.rn1 = a.B21.cols;
      const int64_t cb = x.root ? 0 : rc[i].Brow.cols, cc = x.root ? 0 : rc[i].Bcol.cols;
      // Brow1 = [B12, R1 Brow], Bcol2 = [B12', W2 Bcol], Brow2 = [B21, R2 Brow], Bcol1 = [B21', W1 Bcol]
      t.B1 = ar.blk(a.B12.rows, a.B12.cols + cb);
      t.B2 = ar.blk(a.B12.cols, a.B12.rows + cc);
      t.B3 = ar.blk(a.B21.rows, a.B21.cols + cb);
      t.B4 = ar.blk(a.B21.cols, a.B21.rows + cc);
      Blk l1 = t.B1; l1.cols = a.B12.cols; S.copy(l1, a.B12);
      Blk l2 = t.B2; l2.cols = a.B12.rows; S.copy(l2, a.B12, 1);
      Blk l3 = t.B3; l3.cols = a.B21.cols; S.copy(l3, a.B21);
      Blk l4 = t.B4; l4.cols = a.B21.rows; S.copy(l4, a.B21, 1);
      if (!x.root) {
        Blk r1 = t.B1; r1.p = t.B1.at(0, a.B12.cols); r1.cols = cb; S.gemm(r1, a.R1, 0, rc[i].Brow, 0);
        Blk r2 = t.B2; r2.p = t.B2.at(0, a.B12.rows); r2.cols = cc; S.gemm(r2, a.W2, 0, rc[i].Bcol, 0);
        Blk r3 = t.B3; r3.p = t.B3.at(0, a.B21.cols); r3.cols = cb; S.gemm(r3, a.R2, 0, rc[i].Brow, 0);
        Blk r4 = t.B4; r4.p = t.B4.at(0, a.B21.rows); r4.cols = cc; S.gemm(r4, a.W1, 0, rc[i].Bcol, 0);
      }
      who.push_back(i);
      q4.push_back(t);
    }
    if ((e = S.run_mm()) != cudaSuccess) break;
    for (auto& t : q4) {
      t.f1 = S.pqr(t.B1, atol, rtol);
      t.f2 = S.pqr(t.B2, atol, rtol);
      t.f3 = S.pqr(t.B3, atol, rtol);
      t.f4 = S.pqr(t.B4, atol, rtol);
    }
    std::vector<int32_t> rks;
    if ((e = S.run_qr(rks)) != cudaSuccess) break;
    size_t qi = 0;
    auto rank_of = [&](const Blk& M) { return M.rows * M.cols > 0 ? rks[qi++] : 0; };
    // new couplings and translators, pushes into the children
    std::vector<std::array<Blk, 8>> keep(who.size());   // P1 S2 Q2 T1 P2 S1 Q1 T2 (truncated)
    for (size_t w = 0; w < who.size(); ++w) {
      Q4& t = q4[w];
      const int32_t r1 = rank_of(t.B1), r2 = rank_of(t.B2), r3 = rank_of(t.B3), r4 = rank_of(t.B4);
      Blk P1 = t.f1.first, S2 = t.f1.second, Q2 = t.f2.first, T1 = t.f2.second;
      Blk P2 = t.f3.first, S1 = t.f3.second, Q1 = t.f4.first, T2 = t.f4.second;
      P1.cols = r1; S2.rows = r1; Q2.cols = r2; T1.rows = r2;
      P2.cols = r3; S1.rows = r3; Q1.cols = r4; T2.rows = r4;
      keep[w] = {P1, S2, Q2, T1, P2, S1, Q1, T2};
    }
    std::vector<std::array<Blk, 2>> newB(who.size());
    for (size_t w = 0; w < who.size(); ++w) {
      const int64_t i = who[w];
      const Node& x = N[i];
      G& a = g[i];
      Q4& t = q4[w];
      auto& k = keep[w];
      // B12 = S2[:, 0:rn2] Q2, B21 = S1[:, 0:rn1] Q1
      Blk S2l = k[1]; S2l.cols = t.rn2;
      Blk S1l = k[5]; S1l.cols = t.rn1;
      Blk B12 = ar.blk(k[1].rows, k[2].cols), B21 = ar.blk(k[5].rows, k[6].cols);
      S.gemm(B12, S2l, 0, k[2], 0);
      S.gemm(B21, S1l, 0, k[6], 0);
      newB[w] = {B12, B21};
      if (x.root) {
        a.R1.rows = k[0].cols; a.W2.rows = k[2].cols; a.R2.rows = k[4].cols; a.W1.rows = k[6].cols;
      } else {
        // R1 = P1' R1, W2 = Q2' W2, R2 = P2' R2, W1 = Q1' W1
        Blk R1 = ar.blk(k[0].cols, a.R1.cols), W2 = ar.blk(k[2].cols, a.W2.cols);
        Blk R2 = ar.blk(k[4].cols, a.R2.cols), W1 = ar.blk(k[6].cols, a.W1.cols);
        S.gemm(R1, k[0], 1, a.R1, 0); S.gemm(W2, k[2], 1, a.W2, 0);
        S.gemm(R2, k[4], 1, a.R2, 0); S.gemm(W1, k[6], 1, a.W1, 0);
        a.R1 = R1; a.W2 = W2; a.R2 = R2; a.W1 = W1;
      }
      // the children's bases: U / R1, R2 times P, V / W1, W2 times Q (:176-195)
      auto push = [&](int64_t c, const Blk& P, const Blk& Q) {
        G& y = g[c];
        if (N[c].leaf) {
          Blk U = ar.blk(y.U.rows, P.cols), V = ar.blk(y.V.rows, Q.cols);
          S.gemm(U, y.U, 0, P, 0); S.gemm(V, y.V, 0, Q, 0);
          y.U = U; y.V = V;
        } else {
          Blk R1 = ar.blk(y.R1.rows, P.cols), R2 = ar.blk(y.R2.rows, P.cols);
          Blk W1 = ar.blk(y.W1.rows, Q.cols), W2 = ar.blk(y.W2.rows, Q.cols);
          S.gemm(R1, y.R1, 0, P, 0); S.gemm(R2, y.R2, 0, P, 0);
          S.gemm(W1, y.W1, 0, Q, 0); S.gemm(W2, y.W2, 0, Q, 0);
          y.R1 = R1; y.R2 = R2; y.W1 = W1; y.W2 = W2;
        }
      };
      push(x.left, k[0], k[6]);
      push(x.right, k[4], k[2]);
    }
    if ((e = S.run_mm()) != cudaSuccess) break;
    // the children's Brow / Bcol (:170-173, :248-257)
    for (size_t w = 0; w < who.size(); ++w) {
      const int64_t i = who[w];
      const Node& x = N[i];
      G& a = g[i];
      Q4& t = q4[w];
      auto& k = keep[w];
      a.B12 = newB[w][0];
      a.B21 = newB[w][1];
      auto hcat = [&](const Blk& L, int tl, const Blk& Rt, int64_t c0) {
        // [op(L), Rt[:, c0:]]
        const int64_t lr = tl ? L.cols : L.rows, lc = tl ? L.rows : L.cols;
        const int64_t rcn = std::max<int64_t>(Rt.cols - c0, 0);
        Blk out = ar.blk(lr, lc + rcn);
        Blk left = out; left.cols = lc; S.copy(left, L, tl);
        if (rcn > 0) {
          Blk right = out; right.p = out.at(0, lc); right.cols = rcn;
          Blk src = Rt; src.p = Rt.at(0, c0); src.cols = rcn;
          S.copy(right, src);
        }
        return out;
      };
      if (!N[x.left].leaf) {
        rc[x.left].Brow = x.root ? hcat(a.B12, 0, Blk{}, 0) : hcat(a.B12, 0, k[1], t.rn2);
        rc[x.left].Bcol = x.root ? hcat(a.B21, 1, Blk{}, 0) : hcat(a.B21, 1, k[7], t.rm2);
      }
      if (!N[x.right].leaf) {
        rc[x.right].Brow = x.root ? hcat(a.B21, 0, Blk{}, 0) : hcat(a.B21, 0, k[5], t.rn1);
        rc[x.right].Bcol = x.root ? hcat(a.B12, 1, Blk{}, 0) : hcat(a.B12, 1, k[3], t.rm1);
      }
    }
    if ((e = S.run_mm()) != cudaSuccess) break;
  }
  if (e == cudaSuccess && ar.err != cudaSuccess) e = ar.err;
  if (e != cudaSuccess) return set_cuda_error(e, "recompress");
  // ---- the result as a new handle ----
  std::vector<int64_t> table(nn * HSS_NODE_FIELDS, -1);
  int64_t npk = 0;
  auto off = [&](const Blk& b) -> int64_t {
    if (b.rows * b.cols == 0) return -1;
    const int64_t o = npk;
    npk += b.rows * b.cols;
    return o;
  };
  for (int64_t i = 0; i < nn; ++i) {
    const Node& x = N[i];
    const G& a = g[i];
    int64_t* f = &table[i * HSS_NODE_FIELDS];
    f[0] = x.leaf ? -1 : x.left;
    f[1] = x.leaf ? -1 : x.right;
    f[2] = x.leaf ? x.gm : 0;
    f[3] = x.leaf ? x.gn : 0;
    f[15] = 0;
    if (x.leaf) {
      f[4] = x.root ? 0 : a.U.cols;
      f[5] = x.root ? 0 : a.V.cols;
      f[6] = off(a.D); f[7] = off(a.U); f[8] = off(a.V);
    } else {
      f[4] = x.root ? 0 : a.R1.cols;
      f[5] = x.root ? 0 : a.W1.cols;
      f[9] = off(a.B12); f[10] = off(a.B21);
      if (!x.root) { f[11] = off(a.R1); f[12] = off(a.R2); f[13] = off(a.W1); f[14] = off(a.W2); }
    }
  }
  hss_plan_s* PC = nullptr;
  double* dgen = nullptr;
  int rcode = plan_create_device(nn, table.data(), npk, &PC, &dgen);
  if (rcode) return rcode;
  for (int64_t i = 0; i < nn; ++i) {
    const Node& x = N[i];
    const G& a = g[i];
    const int64_t* f = &table[i * HSS_NODE_FIELDS];
    auto put = [&](int64_t o, const Blk& b) {
      if (o < 0) return;
      Blk dst; dst.p = dgen + o; dst.rows = b.rows; dst.cols = b.cols; dst.ld = std::max<int64_t>(b.rows, 1);
      S.copy(dst, b);
    };
    if (x.leaf) { put(f[6], a.D); put(f[7], a.U); put(f[8], a.V); }
    else {
      put(f[9], a.B12); put(f[10], a.B21);
      if (!x.root) { put(f[11], a.R1); put(f[12], a.R2); put(f[13], a.W1); put(f[14], a.W2); }
    }
  }
  e = S.run_mm();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    plan_destroy(PC);
    return set_cuda_error(e, "recompress");
  }
  *out = PC;
  return HSS_OK;
}

}  // namespace hss

extern "C" {

int hss_recompress(hss_handle h, double atol, double rtol, hss_handle* out, void* stream) {
  if (!h || !out) return set_error(HSS_ERR_INVALID, "null handle");
  *out = nullptr;
  if (plan_ntrees(h) != 1) return set_error(HSS_ERR_INVALID, "recompress takes a single-tree handle");
  if (!(atol >= 0.0) || !(rtol >= 0.0)) return set_error(HSS_ERR_INVALID, "tolerances must be >= 0");
  CUDA_TRY(cudaSetDevice(plan_device(h)));
  return recompress_impl(h, atol, rtol, false, out, (cudaStream_t)stream);
}

int hss_orthonormalize(hss_handle h, hss_handle* out, void* stream) {
  if (!h || !out) return set_error(HSS_ERR_INVALID, "null handle");
  *out = nullptr;
  if (plan_ntrees(h) != 1) return set_error(HSS_ERR_INVALID, "orthonormalize takes a single-tree handle");
  CUDA_TRY(cudaSetDevice(plan_device(h)));
  return recompress_impl(h, 0.0, 0.0, true, out, (cudaStream_t)stream);
}

int hss_full(hss_handle h, double* dOut, int64_t ldo, void* stream) {
  if (!h) return set_error(HSS_ERR_INVALID, "null handle");
  if (plan_ntrees(h) != 1) return set_error(HSS_ERR_INVALID, "full takes a single-tree handle");
  const int64_t m = plan_rows(h), n = plan_cols(h);
  std::vector<int64_t> rows(m), cols(n);
  for (int64_t i = 0; i < m; ++i) rows[i] = i;
  for (int64_t j = 0; j < n; ++j) cols[j] = j;
  return hss_getindex(h, rows.data(), m, cols.data(), n, dOut, ldo, stream);
}

}  // extern "C"
