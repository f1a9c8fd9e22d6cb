// Host side of randomized compression (include/hssgpu.h, hss_rc_*): cluster
// tree validation, per-capacity slot layout, the launch sequence of
// `_randcompress!` (reference src/compression.jl:358-430) -- leaf corrections,
// one interpolative-decomposition launch per tree level, the root couplings --
// and the packing of the generators into a new HSS handle on the device.
#include "hssgpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "hss_host.h"
#include "hss_launch.h"
#include "hss_sample.h"

using namespace hss;

bool hss::g_sample_df = false;

namespace {

#define RC_TRY(x)                                             \
  do {                                                        \
    cudaError_t e_ = (x);                                     \
    if (e_ != cudaSuccess) return set_cuda_error(e_, #x);     \
  } while (0)

constexpr int CL_FIELDS = 6;   // left, right, rlo, rhi, clo, chi

int sm_count(int device) {
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0) n = 132;
  return n;
}

}  // namespace

struct hss_rc_s {
  int device = 0;
  int64_t m = 0, n = 0;
  int64_t nnodes = 0;
  std::vector<int64_t> cl;                    // cluster table (nnodes x 6)
  std::vector<int32_t> pre;                   // pre-order
  std::vector<int32_t> depth, height;
  std::vector<std::vector<int32_t>> levels;   // non-root nodes by height
  std::vector<int32_t> leaves;                // pre-order
  int64_t leaf_pmax = 0, leaf_mmax = 0, leaf_nmax = 0;
  // per capacity s
  int64_t cap = -1;
  std::vector<RcNode> nodes;
  DBuf<double> ws;
  DBuf<int64_t> jws;
  DBuf<int32_t> rank;
  DBuf<RcNode> d_nodes;
  DBuf<int32_t> d_lists;
  std::vector<int64_t> list_off;              // offsets of each level's list (levels, then root)
  DBuf<int64_t> d_leafdims;                   // row0, rows, col0, cols of the leaves
  DBuf<int32_t> d_leafof;                     // leaf index of every row (m), then of every column (n)
  DBuf<double> scorr;                         // corrected samples: m x s then n x s
  DBuf<double> gscratch;
  DBuf<CopyTask> d_tasks;
  std::vector<int32_t> h_rank;

  int64_t F(int64_t i, int f) const { return cl[i * CL_FIELDS + f]; }
  int layout(int64_t s);
};

int hss_rc_s::layout(int64_t s) {
  if (s == cap) return HSS_OK;
  // doubles: Sr, Or (2 each, s x s), G (leaf m x s / n x s; branch 2s x s each), B12, B21 (s x s), S (branch 2s x s each)
  int64_t dbl = 0, ints = 0;
  std::vector<int64_t> off(nnodes * 12, 0);
  for (int64_t i = 0; i < nnodes; ++i) {
    const bool leaf = F(i, 0) < 0;
    const int64_t mi = F(i, 3) - F(i, 2), ni = F(i, 5) - F(i, 4);
    int64_t* o = &off[i * 12];
    for (int k = 0; k < 4; ++k) { o[k] = dbl; dbl += s * s; }                  // Sr0 Sr1 Or0 Or1
    o[4] = dbl; dbl += (leaf ? mi : 2 * s) * s;                               // G0
    o[5] = dbl; dbl += (leaf ? ni : 2 * s) * s;                               // G1
    o[6] = dbl; dbl += leaf ? 0 : s * s;                                      // B12
    o[7] = dbl; dbl += leaf ? 0 : s * s;                                      // B21
    o[8] = dbl; dbl += leaf ? 0 : 2 * s * s;                                  // S0
    o[9] = dbl; dbl += leaf ? 0 : 2 * s * s;                                  // S1
    o[10] = ints; ints += s;                                                  // J0
    o[11] = ints; ints += s;                                                  // J1
  }
  RC_TRY(ws.ensure(std::max<int64_t>(dbl, 1)));
  RC_TRY(jws.ensure(std::max<int64_t>(ints, 1)));
  RC_TRY(scorr.ensure(std::max<int64_t>((m + n) * s, 1)));
  nodes.assign(nnodes, RcNode{});
  for (int64_t i = 0; i < nnodes; ++i) {
    RcNode& x = nodes[i];
    const int64_t* o = &off[i * 12];
    x.left = (int32_t)F(i, 0);
    x.right = (int32_t)F(i, 1);
    x.leaf = F(i, 0) < 0;
    x.root = i == 0;
    x.r0 = F(i, 2); x.m = F(i, 3) - F(i, 2);
    x.c0 = F(i, 4); x.n = F(i, 5) - F(i, 4);
    x.Sr[0] = ws.p + o[0]; x.Sr[1] = ws.p + o[1];
    x.Or[0] = ws.p + o[2]; x.Or[1] = ws.p + o[3];
    x.G[0] = ws.p + o[4]; x.G[1] = ws.p + o[5];
    x.B12 = ws.p + o[6]; x.B21 = ws.p + o[7];
    x.J[0] = jws.p + o[10]; x.J[1] = jws.p + o[11];
    if (x.leaf) {
      x.S[0] = scorr.p + x.r0; x.lds[0] = m;
      x.S[1] = scorr.p + m * s + x.c0; x.lds[1] = n;
    } else {
      x.S[0] = ws.p + o[8]; x.S[1] = ws.p + o[9];
      x.lds[0] = x.lds[1] = 0;
    }
  }
  RC_TRY(d_nodes.ensure(nnodes));
  RC_TRY(cudaMemcpy(d_nodes.p, nodes.data(), nnodes * sizeof(RcNode), cudaMemcpyHostToDevice));
  cap = s;
  return HSS_OK;
}

extern "C" {

int hss_rc_create(int64_t nnodes, const int64_t* clusters, hss_rc* out) {
  if (!out) return set_error(HSS_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (nnodes <= 0 || !clusters) return set_error(HSS_ERR_INVALID, "empty cluster table");
  if (nnodes > (int64_t)INT32_MAX) return set_error(HSS_ERR_BAD_DIMS, "too many nodes");
  auto* R = new hss_rc_s();
  R->nnodes = nnodes;
  R->cl.assign(clusters, clusters + nnodes * CL_FIELDS);
  auto bad = [&](const char* msg) {
    delete R;
    return set_error(HSS_ERR_BAD_DIMS, msg);
  };
  // topology: every non-root node has one parent, both children or none
  std::vector<int32_t> parent(nnodes, -1);
  for (int64_t i = 0; i < nnodes; ++i) {
    const int64_t l = R->F(i, 0), r = R->F(i, 1);
    if ((l < 0) != (r < 0)) return bad("cluster with only one child");
    for (int64_t c : {l, r}) {
      if (c < 0) continue;
      if (c >= nnodes || c == 0) return bad("child index out of range");
      if (parent[c] != -1) return bad("cluster with two parents");
      parent[c] = (int32_t)i;
    }
  }
  {
    std::vector<int32_t> stack{0};
    while (!stack.empty() && (int64_t)R->pre.size() <= nnodes) {
      const int32_t x = stack.back();
      stack.pop_back();
      R->pre.push_back(x);
      if (R->F(x, 0) >= 0) {
        stack.push_back((int32_t)R->F(x, 1));
        stack.push_back((int32_t)R->F(x, 0));
      }
    }
  }
  if ((int64_t)R->pre.size() != nnodes) return bad("cluster table is not a tree");
  // ranges: the root starts at 0, children split the parent's ranges in order
  // (`compatible`, src/clustertree.jl), leaves are not empty
  if (R->F(0, 2) != 0 || R->F(0, 4) != 0) return bad("root cluster does not start at 0");
  R->m = R->F(0, 3);
  R->n = R->F(0, 5);
  if (R->m <= 0 || R->n <= 0) return bad("empty matrix");
  for (int64_t i = 0; i < nnodes; ++i) {
    const int64_t rlo = R->F(i, 2), rhi = R->F(i, 3), clo = R->F(i, 4), chi = R->F(i, 5);
    if (rlo < 0 || rhi > R->m || clo < 0 || chi > R->n || rhi <= rlo || chi <= clo)
      return bad("cluster range out of bounds or empty");
    const int64_t l = R->F(i, 0), r = R->F(i, 1);
    if (l >= 0) {
      if (R->F(l, 2) != rlo || R->F(l, 3) != R->F(r, 2) || R->F(r, 3) != rhi || R->F(l, 4) != clo ||
          R->F(l, 5) != R->F(r, 4) || R->F(r, 5) != chi)
        return bad("row and column clusters are not compatible");
    }
  }
  R->depth.assign(nnodes, 0);
  R->height.assign(nnodes, 0);
  for (int32_t i : R->pre)
    if (i != 0) R->depth[i] = R->depth[parent[i]] + 1;
  int max_h = 0;
  for (auto it = R->pre.rbegin(); it != R->pre.rend(); ++it) {
    const int32_t i = *it;
    if (R->F(i, 0) >= 0) R->height[i] = std::max(R->height[R->F(i, 0)], R->height[R->F(i, 1)]) + 1;
    max_h = std::max(max_h, R->height[i]);
  }
  R->levels.assign(max_h + 1, {});
  for (int32_t i : R->pre)
    if (i != 0) R->levels[R->height[i]].push_back(i);
  for (int32_t i : R->pre)
    if (R->F(i, 0) < 0) {
      R->leaves.push_back(i);
      R->leaf_mmax = std::max(R->leaf_mmax, R->F(i, 3) - R->F(i, 2));
      R->leaf_nmax = std::max(R->leaf_nmax, R->F(i, 5) - R->F(i, 4));
    }
  R->leaf_pmax = std::max(R->leaf_mmax, R->leaf_nmax);
  int rc;
  auto cfail = [&](cudaError_t e, const char* what) {
    delete R;
    return set_cuda_error(e, what);
  };
  cudaError_t e = cudaGetDevice(&R->device);
  if (e != cudaSuccess) return cfail(e, "cudaGetDevice");
  // level lists (non-root levels by height, then the root) and leaf dimensions
  std::vector<int32_t> lists;
  for (auto& lv : R->levels) {
    R->list_off.push_back((int64_t)lists.size());
    lists.insert(lists.end(), lv.begin(), lv.end());
  }
  R->list_off.push_back((int64_t)lists.size());
  lists.push_back(0);
  if ((e = R->d_lists.ensure(lists.size())) != cudaSuccess) return cfail(e, "cudaMalloc");
  if ((e = cudaMemcpy(R->d_lists.p, lists.data(), lists.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return cfail(e, "cudaMemcpy");
  const int64_t nl = (int64_t)R->leaves.size();
  std::vector<int64_t> dims(4 * nl);
  for (int64_t k = 0; k < nl; ++k) {
    const int32_t i = R->leaves[k];
    dims[k] = R->F(i, 2);
    dims[nl + k] = R->F(i, 3) - R->F(i, 2);
    dims[2 * nl + k] = R->F(i, 4);
    dims[3 * nl + k] = R->F(i, 5) - R->F(i, 4);
  }
  if ((e = R->d_leafdims.ensure(dims.size())) != cudaSuccess) return cfail(e, "cudaMalloc");
  if ((e = cudaMemcpy(R->d_leafdims.p, dims.data(), dims.size() * sizeof(int64_t), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return cfail(e, "cudaMemcpy");
  std::vector<int32_t> leafof(R->m + R->n, 0);
  for (int64_t k = 0; k < nl; ++k) {
    const int32_t i = R->leaves[k];
    for (int64_t q = R->F(i, 2); q < R->F(i, 3); ++q) leafof[q] = (int32_t)k;
    for (int64_t q = R->F(i, 4); q < R->F(i, 5); ++q) leafof[R->m + q] = (int32_t)k;
  }
  if ((e = R->d_leafof.ensure(leafof.size())) != cudaSuccess) return cfail(e, "cudaMalloc");
  if ((e = cudaMemcpy(R->d_leafof.p, leafof.data(), leafof.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return cfail(e, "cudaMemcpy");
  (void)rc;
  *out = R;
  return HSS_OK;
}

int hss_rc_destroy(hss_rc rc) {
  delete rc;
  return HSS_OK;
}

int hss_rc_size(hss_rc rc, int64_t* m, int64_t* n) {
  if (!rc) return set_error(HSS_ERR_INVALID, "null handle");
  if (m) *m = rc->m;
  if (n) *n = rc->n;
  return HSS_OK;
}

int hss_sample(const double* dA, int64_t lda, int64_t m, int64_t n, int32_t trans, const double* dX, int64_t ldx,
               int64_t r, double* dY, int64_t ldy, double alpha, double beta, void* stream) {
  if (m < 0 || n < 0 || r < 0 || (trans != 0 && trans != 1)) return set_error(HSS_ERR_BAD_DIMS, "bad sizes");
  const int64_t rows = trans ? n : m, inner = trans ? m : n;
  if (lda < std::max<int64_t>(1, m) || ldx < std::max<int64_t>(1, inner) || ldy < std::max<int64_t>(1, rows))
    return set_error(HSS_ERR_BAD_DIMS, "leading dimension too small");
  if (rows == 0 || r == 0) return HSS_OK;
  if (!dA || !dX || !dY) return set_error(HSS_ERR_INVALID, "null pointer");
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0;
  RC_TRY(cudaGetDevice(&dev));
  const int nsplit = sample_ksplit(rows, inner, r, sm_count(dev), g_sample_df);
  // split-K partial sums: stream-ordered scratch, so calls on different streams do not share it
  double* partial = nullptr;
  if (nsplit > 1) RC_TRY(cudaMallocAsync((void**)&partial, (size_t)nsplit * rows * r * sizeof(double), st));
  launch_sample_gemm(dA, lda, rows, inner, trans, dX, ldx, r, dY, ldy, alpha, beta, nsplit, partial, g_sample_df,
                     nullptr, nullptr, st);
  count_launches(nsplit > 1 ? 2 : 1);
  cudaError_t e = cudaGetLastError();
  if (partial) {
    cudaError_t f = cudaFreeAsync(partial, st);
    if (e == cudaSuccess) e = f;
  }
  if (e != cudaSuccess) return set_cuda_error(e, "sample product");
  return HSS_OK;
}

int hss_rc_sample(hss_rc R, const double* dA, int64_t lda, int32_t trans, const double* dX, int64_t ldx, int64_t r,
                  double* dY, int64_t ldy, void* stream) {
  if (!R) return set_error(HSS_ERR_INVALID, "null handle");
  if (!g_sample_df) return hss_sample(dA, lda, R->m, R->n, trans, dX, ldx, r, dY, ldy, 1.0, 0.0, stream);
  const int64_t m = R->m, n = R->n;
  if (r < 0 || (trans != 0 && trans != 1)) return set_error(HSS_ERR_BAD_DIMS, "bad sizes");
  const int64_t rows = trans ? n : m, inner = trans ? m : n;
  if (lda < m || ldx < inner || ldy < rows) return set_error(HSS_ERR_BAD_DIMS, "leading dimension too small");
  if (r == 0) return HSS_OK;
  if (!dA || !dX || !dY) return set_error(HSS_ERR_INVALID, "null pointer");
  cudaStream_t st = (cudaStream_t)stream;
  RC_TRY(cudaSetDevice(R->device));
  const int32_t* lr = R->d_leafof.p;        // rows of A
  const int32_t* lc = R->d_leafof.p + m;    // columns of A
  const int nsplit = sample_ksplit(rows, inner, r, sm_count(R->device), true);
  double* partial = nullptr;
  if (nsplit > 1) RC_TRY(cudaMallocAsync((void**)&partial, (size_t)nsplit * rows * r * sizeof(double), st));
  // off-diagonal part in double-float, then + D * X of the leaves in FP64
  launch_sample_gemm(dA, lda, rows, inner, trans, dX, ldx, r, dY, ldy, 1.0, 0.0, nsplit, partial, true,
                     trans ? lc : lr, trans ? lr : lc, st);
  count_launches(nsplit > 1 ? 2 : 1);
  const int64_t nl = (int64_t)R->leaves.size();
  const int64_t* dims = R->d_leafdims.p;
  for (int64_t b = 0; b < nl; b += 65535) {
    const int32_t cnt = (int32_t)std::min<int64_t>(65535, nl - b);
    launch_blockdiag_gemm(cnt, trans ? R->leaf_nmax : R->leaf_mmax, dA, lda, dims + b, dims + nl + b,
                          dims + 2 * nl + b, dims + 3 * nl + b, trans, dX, ldx, r, dY, ldy, 1.0, 1.0, st);
    count_launches(1);
  }
  cudaError_t e = cudaGetLastError();
  if (partial) {
    cudaError_t f = cudaFreeAsync(partial, st);
    if (e == cudaSuccess) e = f;
  }
  if (e != cudaSuccess) return set_cuda_error(e, "sample product");
  return HSS_OK;
}

int hss_sumsq(const double* dB, int64_t ldb, int64_t m, int64_t r, double* out, void* stream) {
  if (!out) return set_error(HSS_ERR_INVALID, "null output");
  *out = 0.0;
  if (m < 0 || r < 0 || ldb < std::max<int64_t>(1, m)) return set_error(HSS_ERR_BAD_DIMS, "bad sizes");
  if (m == 0 || r == 0) return HSS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  static thread_local DBuf<double> d;
  static thread_local std::vector<double> h;
  RC_TRY(d.ensure(r));
  RC_TRY(cudaMemsetAsync(d.p, 0, r * sizeof(double), st));
  launch_colnorm2(dB, ldb, m, r, d.p, st);
  count_launches(1);
  h.resize(r);
  RC_TRY(cudaMemcpyAsync(h.data(), d.p, r * sizeof(double), cudaMemcpyDeviceToHost, st));
  RC_TRY(cudaStreamSynchronize(st));
  double acc = 0.0;
  for (double v : h) acc += v;
  *out = acc;
  return HSS_OK;
}

int hss_rc_compress(hss_rc R, const double* dA, int64_t lda, const double* dScol, int64_t ldscol,
                    const double* dSrow, int64_t ldsrow, const double* dOcol, int64_t ldocol, const double* dOrow,
                    int64_t ldorow, int64_t s, double atol, double rtol, hss_handle* out, void* stream) {
  if (!R || !out) return set_error(HSS_ERR_INVALID, "null handle");
  *out = nullptr;
  const int64_t m = R->m, n = R->n;
  if (s < 0 || s > (1 << 16)) return set_error(HSS_ERR_BAD_DIMS, "sample count out of range");
  if (lda < m || ldscol < m || ldsrow < n || ldocol < n || ldorow < m)
    return set_error(HSS_ERR_BAD_DIMS, "leading dimension too small");
  if (!(atol >= 0.0) || !(rtol >= 0.0)) return set_error(HSS_ERR_INVALID, "tolerances must be >= 0");
  if (!dA || (s > 0 && (!dScol || !dSrow || !dOcol || !dOrow))) return set_error(HSS_ERR_INVALID, "null pointer");
  cudaStream_t st = (cudaStream_t)stream;
  RC_TRY(cudaSetDevice(R->device));
  const bool root_leaf = R->F(0, 0) < 0;
  if (!root_leaf && s > 0) {
    int rc = R->layout(s);
    if (rc) return rc;
    const int64_t nl = (int64_t)R->leaves.size();
    RC_TRY(R->rank.ensure(2 * R->nnodes));
    RC_TRY(cudaMemsetAsync(R->rank.p, 0, 2 * R->nnodes * sizeof(int32_t), st));
    // corrected leaf samples: Scol - D * Omega_col, Srow - D^T * Omega_row (:360-361)
    double* Sc = R->scorr.p;
    double* Sr = R->scorr.p + m * s;
    RC_TRY(cudaMemcpy2DAsync(Sc, m * sizeof(double), dScol, ldscol * sizeof(double), m * sizeof(double), s,
                             cudaMemcpyDeviceToDevice, st));
    RC_TRY(cudaMemcpy2DAsync(Sr, n * sizeof(double), dSrow, ldsrow * sizeof(double), n * sizeof(double), s,
                             cudaMemcpyDeviceToDevice, st));
    const int64_t* dims = R->d_leafdims.p;
    for (int64_t b = 0; b < nl; b += 65535) {
      const int32_t cnt = (int32_t)std::min<int64_t>(65535, nl - b);
      launch_blockdiag_gemm(cnt, R->leaf_mmax, dA, lda, dims + b, dims + nl + b, dims + 2 * nl + b,
                            dims + 3 * nl + b, 0, dOcol, ldocol, s, Sc, m, -1.0, 1.0, st);
      launch_blockdiag_gemm(cnt, R->leaf_nmax, dA, lda, dims + b, dims + nl + b, dims + 2 * nl + b,
                            dims + 3 * nl + b, 1, dOrow, ldorow, s, Sr, n, -1.0, 1.0, st);
      count_launches(2);
    }
    RC_TRY(cudaGetLastError());
    // one ID launch per level, then the root's couplings
    RcArgs a{};
    a.nodes = R->d_nodes.p;
    a.rank = R->rank.p;
    a.A = dA;
    a.lda = lda;
    a.Ocol = dOcol;
    a.ldoc = ldocol;
    a.Orow = dOrow;
    a.ldor = ldorow;
    a.s = s;
    a.atol = atol;
    a.rtol = rtol;
    constexpr size_t kSmemCap = 200 * 1024;
    for (size_t h = 0; h <= R->levels.size(); ++h) {
      const bool rootl = h == R->levels.size();
      const int64_t cnt = rootl ? 1 : (int64_t)R->levels[h].size();
      if (cnt == 0) continue;
      a.list = R->d_lists.p + R->list_off[h];
      a.pmax = rootl ? 1 : (h == 0 ? R->leaf_pmax : 2 * s);
      a.m_in_smem = rc_id_smem(s, a.pmax, true) <= kSmemCap;
      a.gscratch = nullptr;
      if (!a.m_in_smem) {
        RC_TRY(R->gscratch.ensure(2 * cnt * rc_id_scratch(s, a.pmax)));
        a.gscratch = R->gscratch.p;
      }
      RC_TRY(launch_rc_id(a, (int32_t)cnt, st));
      count_launches(1);
    }
    R->h_rank.resize(2 * R->nnodes);
    RC_TRY(cudaMemcpyAsync(R->h_rank.data(), R->rank.p, 2 * R->nnodes * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           st));
    RC_TRY(cudaStreamSynchronize(st));
  } else {
    R->h_rank.assign(2 * R->nnodes, 0);
    if (!root_leaf) {
      int rc = R->layout(std::max<int64_t>(s, 1));
      if (rc) return rc;
    }
  }
  // node table (pre-order numbering of the cluster table) and packed layout:
  // leaf D blocks, leaf U, leaf V, then branch blocks depth by depth
  const int64_t nn = R->nnodes;
  auto kc = [&](int64_t i) -> int64_t { return i == 0 ? 0 : R->h_rank[2 * i]; };
  auto kr = [&](int64_t i) -> int64_t { return i == 0 ? 0 : R->h_rank[2 * i + 1]; };
  std::vector<int64_t> table(nn * HSS_NODE_FIELDS, -1);
  std::vector<CopyTask> tasks;
  int64_t off = 0;
  auto put = [&](int64_t i, int field, const double* src, int64_t lds, int64_t rows, int64_t cols) {
    if (rows * cols == 0) return;
    table[i * HSS_NODE_FIELDS + field] = off;
    tasks.push_back(CopyTask{src, lds, nullptr, rows, cols});
    tasks.back().dst = reinterpret_cast<double*>(off);   // rebased after the plan exists
    off += rows * cols;
  };
  for (int64_t i = 0; i < nn; ++i) {
    int64_t* t = &table[i * HSS_NODE_FIELDS];
    t[0] = R->F(i, 0);
    t[1] = R->F(i, 1);
    const bool leaf = t[0] < 0;
    t[2] = leaf ? R->F(i, 3) - R->F(i, 2) : 0;
    t[3] = leaf ? R->F(i, 5) - R->F(i, 4) : 0;
    t[4] = kc(i);
    t[5] = kr(i);
    t[15] = 0;
  }
  for (int32_t i : R->leaves)
    put(i, 6, dA + R->F(i, 2) + R->F(i, 4) * lda, lda, R->F(i, 3) - R->F(i, 2), R->F(i, 5) - R->F(i, 4));
  if (!root_leaf) {
    for (int32_t i : R->leaves) put(i, 7, R->nodes[i].G[0], R->nodes[i].m, R->nodes[i].m, kc(i));
    for (int32_t i : R->leaves) put(i, 8, R->nodes[i].G[1], R->nodes[i].n, R->nodes[i].n, kr(i));
    int max_d = 0;
    for (int32_t i : R->pre) max_d = std::max(max_d, R->depth[i]);
    for (int d = 0; d <= max_d; ++d)
      for (int32_t i : R->pre) {
        if (R->depth[i] != d || R->F(i, 0) < 0) continue;
        const RcNode& x = R->nodes[i];
        const int64_t c1 = R->F(i, 0), c2 = R->F(i, 1);
        put(i, 9, x.B12, kc(c1), kc(c1), kr(c2));
        put(i, 10, x.B21, kc(c2), kc(c2), kr(c1));
        if (i != 0) {
          const int64_t pc = kc(c1) + kc(c2), pr = kr(c1) + kr(c2);
          put(i, 11, x.G[0], pc, kc(c1), kc(i));
          put(i, 12, x.G[0] + kc(c1), pc, kc(c2), kc(i));
          put(i, 13, x.G[1], pr, kr(c1), kr(i));
          put(i, 14, x.G[1] + kr(c1), pr, kr(c2), kr(i));
        }
      }
  }
  hss_plan_s* P = nullptr;
  double* d_gen = nullptr;
  int rc = plan_create_device(nn, table.data(), off, &P, &d_gen);
  if (rc) return rc;
  for (auto& t : tasks) t.dst = d_gen + reinterpret_cast<int64_t>(t.dst);
  cudaError_t e = R->d_tasks.ensure(std::max<size_t>(tasks.size(), 1));
  if (e == cudaSuccess && !tasks.empty())
    e = cudaMemcpyAsync(R->d_tasks.p, tasks.data(), tasks.size() * sizeof(CopyTask), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    launch_copy_blocks(R->d_tasks.p, (int64_t)tasks.size(), st);
    count_launches(tasks.empty() ? 0 : 1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    plan_destroy(P);
    return set_cuda_error(e, "packing compressed generators");
  }
  *out = P;
  return HSS_OK;
}

int hss_rc_ranks(hss_rc R, int32_t* ranks) {
  if (!R || !ranks) return set_error(HSS_ERR_INVALID, "null argument");
  for (size_t i = 0; i < R->h_rank.size(); ++i) ranks[i] = R->h_rank[i];
  return HSS_OK;
}

}  // extern "C"
