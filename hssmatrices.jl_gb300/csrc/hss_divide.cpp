// HSS-valued division on the device: hssA \ hssB and hssB / hssA (reference
// src/ulvdivide.jl:13-252, src/hssmatrix.jl:235-237), and the adjoint of a
// handle (src/hssmatrix.jl:165-171), all as new handles.
//
// The division follows the reference's recursion level by level.  Level l
// works on the tree T_l of the nodes that are still leaves or branches after
// l prune_leaves! steps: a node of A's tree is a leaf of T_l when its height
// is <= l, and it belongs to T_l when its parent's height is > l.  The
// reductions of A's leaves at level l (_ulvfactor_leaves!, :88-112) are those
// of A's FP64 ULV factorization at the nodes of height l (the factorization
// merges children exactly as prune_leaves! + _extract_ccols do, :42-44), so A
// is factored once and every level reads its factored nodes:
//
//   forward, l = 0, 1, ... (:28-47), B_0 = hssB:
//     QB = the last k rows of Q_ql^T B's leaves, Y0 = L1 \ their first mk
//     rows (other rows zero)                        (hss_divide.cu, DIV_QL)
//     QB <- recompress!(QB - L_l * Y0), L_l the reduced A (leaves L2, tril U,
//     Q V; A's translators above), through hss_hssmul and recompress_impl
//     B_{l+1} = prune_leaves!(QB)
//   the root (:23-26): Y = D_root^-1 B with the root block's LU (DIV_ROOT)
//   backward (:50-52): Y_l = recompress!(Q_lq^T unpackadd(Y0_l, Y_{l+1}))
//
// Every block operation is a task of the small-product kernel (copies,
// transposes, identity and zero blocks, scaled adds, products), run stage by
// stage; memory per level is O(n k) (the dense blocks of a level's leaves
// hold k rows, or leafsize rows at level 0, by the columns of B).
#include "hssgpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <memory>
#include <vector>

#include "hss_host.h"
#include "hss_internal.h"
#include "hss_launch.h"
#include "hss_stages.h"

using namespace hss;

namespace {

struct PlanDel {
  void operator()(hss_plan_s* p) const {
    if (p) plan_destroy(p);
  }
};
using PlanPtr = std::unique_ptr<hss_plan_s, PlanDel>;

// the generators of one node, as views into a plan's buffer
struct Gen {
  Blk D, U, V, B12, B21, R1, R2, W1, W2;
};

Blk view(const double* p, int64_t rows, int64_t cols, int64_t ld) {
  Blk b;
  b.p = (double*)p;
  b.rows = rows;
  b.cols = cols;
  b.ld = std::max<int64_t>(ld, 1);
  return b;
}

Blk sub(const Blk& b, int64_t r0, int64_t c0, int64_t rows, int64_t cols) {
  Blk x = b;
  x.p = b.p ? b.at(r0, c0) : nullptr;
  x.rows = rows;
  x.cols = cols;
  return x;
}

std::vector<Gen> plan_views(const hss_plan_s* P) {
  const std::vector<Node>& N = plan_nodes(P);
  std::vector<Gen> g(N.size());
  for (size_t i = 0; i < N.size(); ++i) {
    const Node& x = N[i];
    if (x.leaf) {
      g[i].D = view(x.D, x.gm, x.gn, x.gm);
      g[i].U = view(x.U, x.gm, x.ku, x.gm);
      g[i].V = view(x.V, x.gn, x.kv, x.gn);
    } else {
      const Node &c1 = N[x.left], &c2 = N[x.right];
      g[i].B12 = view(x.B12, c1.ku, c2.kv, c1.ku);
      g[i].B21 = view(x.B21, c2.ku, c1.kv, c2.ku);
      g[i].R1 = view(x.R1, c1.ku, x.ku, c1.ku);
      g[i].R2 = view(x.R2, c2.ku, x.ku, c2.ku);
      g[i].W1 = view(x.W1, c1.kv, x.kv, c1.kv);
      g[i].W2 = view(x.W2, c2.kv, x.kv, c2.kv);
    }
  }
  return g;
}

// The shape of a single-tree plan: children (-1 at leaves), leaf sizes and
// ranks (0 at the root).
struct Shape {
  std::vector<int32_t> left, right;
  std::vector<int64_t> m, n;
  std::vector<int64_t> ku, kv;
  explicit Shape(size_t nn) : left(nn, -1), right(nn, -1), m(nn, 0), n(nn, 0), ku(nn, 0), kv(nn, 0) {}
  size_t size() const { return left.size(); }
};

// a new plan of this shape with an uninitialised generator buffer
void reg_plan(Ranges* rg, const hss_plan_s* P) {
  if (!rg || !P) return;
  int64_t len = 0;
  const double* p = plan_gen(P, &len);
  rg->add(p, (size_t)len * sizeof(double));
}

int make_plan(const Shape& S, PlanPtr& out, std::vector<Gen>& g, Ranges* rg = nullptr) {
  const int64_t nn = (int64_t)S.size();
  std::vector<int64_t> table(nn * HSS_NODE_FIELDS, -1);
  int64_t npk = 0;
  auto blk = [&](int64_t r, int64_t c) -> int64_t {
    if (r * c <= 0) return -1;
    const int64_t o = npk;
    npk += r * c;
    return o;
  };
  for (int64_t i = 0; i < nn; ++i) {
    int64_t* f = &table[i * HSS_NODE_FIELDS];
    const bool leaf = S.left[i] < 0;
    f[0] = S.left[i];
    f[1] = S.right[i];
    f[2] = leaf ? S.m[i] : 0;
    f[3] = leaf ? S.n[i] : 0;
    f[4] = i == 0 ? 0 : S.ku[i];
    f[5] = i == 0 ? 0 : S.kv[i];
    f[15] = 0;
    if (leaf) {
      f[6] = blk(S.m[i], S.n[i]);
      f[7] = blk(S.m[i], f[4]);
      f[8] = blk(S.n[i], f[5]);
    } else {
      const int32_t a = S.left[i], b = S.right[i];
      f[9] = blk(S.ku[a], S.kv[b]);
      f[10] = blk(S.ku[b], S.kv[a]);
      f[11] = blk(S.ku[a], f[4]);
      f[12] = blk(S.ku[b], f[4]);
      f[13] = blk(S.kv[a], f[5]);
      f[14] = blk(S.kv[b], f[5]);
    }
  }
  hss_plan_s* P = nullptr;
  double* dgen = nullptr;
  int rc = plan_create_device(nn, table.data(), npk, &P, &dgen);
  if (rc) return rc;
  out.reset(P);
  reg_plan(rg, P);
  g = plan_views(P);
  return HSS_OK;
}

// the shape of an existing plan
Shape shape_of(const hss_plan_s* P) {
  const std::vector<Node>& N = plan_nodes(P);
  Shape S(N.size());
  for (size_t i = 0; i < N.size(); ++i) {
    const Node& x = N[i];
    if (!x.leaf) {
      S.left[i] = x.left;
      S.right[i] = x.right;
    } else {
      S.m[i] = x.gm;
      S.n[i] = x.gn;
    }
    S.ku[i] = x.root ? 0 : x.ku;
    S.kv[i] = x.root ? 0 : x.kv;
  }
  return S;
}

// DivTask list, uploaded and launched in one go
struct DivList {
  std::vector<DivTask> t;
  int maxrows = 0, maxcols = 0;
  Ranges* rg = nullptr;
  // bot_rows: rows written to bot (DIV_QL: rows - mk)
  void add(const Node* nd, const double* fb, int mode, const Blk& src, const Blk& top, const Blk* bot, int64_t rows,
           int64_t bot_rows = 0) {
    if (src.cols <= 0 || rows <= 0) return;
    if (rg) {
      if (rows > div_rows_max() || top.cols != src.cols || src.rows != rows || top.rows != rows) rg->bad = true;
      rg->check(src.p, src.ld, rows, src.cols);
      rg->check(top.p, top.ld, rows, src.cols);
      if (bot) {
        if (bot->cols != src.cols || bot->rows != bot_rows) rg->bad = true;
        rg->check(bot->p, bot->ld, bot_rows, src.cols);
      }
    }
    DivTask d{};
    d.nd = nd;
    d.fb = fb;
    d.src = src.p;
    d.lds = src.ld;
    d.top = top.p;
    d.ldt = top.ld;
    d.bot = bot ? bot->p : nullptr;
    d.ldb = bot ? bot->ld : 1;
    d.rows = (int32_t)rows;
    d.cols = (int32_t)src.cols;
    d.mode = mode;
    t.push_back(d);
    maxrows = std::max<int>(maxrows, (int)rows);
    maxcols = std::max<int>(maxcols, (int)src.cols);
  }
  cudaError_t run(Arena& ar, cudaStream_t st) {
    if (t.empty()) return cudaSuccess;
    if (rg && rg->bad) return cudaErrorInvalidValue;
    auto* d = (DivTask*)ar.raw(t.size() * sizeof(DivTask));
    if (!d) return ar.err;
    cudaError_t e = cudaMemcpyAsync(d, t.data(), t.size() * sizeof(DivTask), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_div_rows(d, (int64_t)t.size(), maxrows, maxcols, st);
    count_launches(1);
    t.clear();
    maxrows = maxcols = 0;
    return e;
  }
};

int run_stages(Stages& S, Arena& ar) {
  if (S.rg && S.rg->bad) {
    S.mm.clear();
    return set_error(HSS_ERR_INVALID, "division: internal block outside its buffer (not launched)");
  }
  cudaError_t e = S.run_mm();
  if (e == cudaSuccess && ar.err != cudaSuccess) e = ar.err;
  return e == cudaSuccess ? HSS_OK : set_cuda_error(e, "division");
}

// The adjoint (src/hssmatrix.jl:165-171): D^T with U and V exchanged, B12 and
// B21 exchanged and transposed, R and W exchanged; same node numbering.
int transpose_impl(const hss_plan_s* h, PlanPtr& out, cudaStream_t st) {
  Shape S = shape_of(h);
  for (size_t i = 0; i < S.size(); ++i) {
    std::swap(S.m[i], S.n[i]);
    std::swap(S.ku[i], S.kv[i]);
  }
  Ranges rg;
  reg_plan(&rg, h);
  std::vector<Gen> g;
  int rc = make_plan(S, out, g, &rg);
  if (rc) return rc;
  const std::vector<Gen> a = plan_views(h);
  const std::vector<Node>& N = plan_nodes(h);
  Arena ar;
  ar.on_stream(st);
  ar.rg = &rg;
  Stages T{st, ar, {}, {}};
  T.rg = &rg;
  for (size_t i = 0; i < N.size(); ++i) {
    if (N[i].leaf) {
      T.copy(g[i].D, a[i].D, 1);
      T.copy(g[i].U, a[i].V);
      T.copy(g[i].V, a[i].U);
    } else {
      T.copy(g[i].B12, a[i].B21, 1);
      T.copy(g[i].B21, a[i].B12, 1);
      T.copy(g[i].R1, a[i].W1);
      T.copy(g[i].R2, a[i].W2);
      T.copy(g[i].W1, a[i].R1);
      T.copy(g[i].W2, a[i].R2);
    }
  }
  rc = run_stages(T, ar);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? HSS_OK : set_cuda_error(e, "transpose");
}

// One level's tree T_l: its members (A's node ids, increasing) and A's id ->
// position (-1 if absent).
struct Level {
  std::vector<int32_t> mem;
  std::vector<int32_t> pos;
  std::vector<char> leaf;   // per position
};

Level make_level(const std::vector<Node>& NA, const std::vector<int32_t>& parent, int l) {
  Level L;
  L.pos.assign(NA.size(), -1);
  for (size_t i = 0; i < NA.size(); ++i)
    if (parent[i] < 0 || NA[parent[i]].height > l) {
      L.pos[i] = (int32_t)L.mem.size();
      L.mem.push_back((int32_t)i);
      L.leaf.push_back(NA[i].height <= l ? 1 : 0);
    }
  return L;
}

// the tree part of a level's shape (children positions)
void link(Shape& S, const Level& L, const std::vector<Node>& NA) {
  for (size_t t = 0; t < L.mem.size(); ++t) {
    if (L.leaf[t]) continue;
    const Node& x = NA[L.mem[t]];
    S.left[t] = L.pos[x.left];
    S.right[t] = L.pos[x.right];
  }
}

int ldiv_impl(hss_plan_s* hA, hss_plan_s* hB, double atol, double rtol, PlanPtr& result, cudaStream_t st) {
  const std::vector<Node>& NA = plan_nodes(hA);
  const std::vector<Node>& NB0 = plan_nodes(hB);
  const int64_t nn = (int64_t)NA.size();
  bool match = (int64_t)NB0.size() == nn;
  for (int64_t i = 0; match && i < nn; ++i)
    match = NA[i].leaf == NB0[i].leaf && NA[i].left == NB0[i].left && NA[i].right == NB0[i].right &&
            NA[i].gn == NB0[i].gm;
  if (!match) return set_error(HSS_ERR_BAD_DIMS, "the clusters of hssA and hssB are not compatible");
  for (int64_t i = 0; i < nn; ++i) {
    if (NA[i].leaf && NA[i].gm != NA[i].gn)
      return set_error(HSS_ERR_BAD_DIMS, "hssA must be square with square leaves");
    if (NA[i].m > div_rows_max())
      return set_error(HSS_ERR_INVALID, "division: blocks of more than 512 rows are not supported");
  }
  hss_factor F = nullptr;
  int rc = hss_ulvfactor(hA, HSS_PREC_FP64, &F, st);
  if (rc) return rc;
  struct FacDel {
    hss_factor f;
    ~FacDel() { hss_factor_destroy(f); }
  } fguard{F};
  const double* fb = (const double*)factor_storage(F);
  const Node* dn = plan_device_nodes(hA);
  Ranges rg;   // every buffer the division's task lists may touch
  reg_plan(&rg, hA);
  reg_plan(&rg, hB);
  rg.add(fb, factor_storage_bytes(F));
  std::vector<int32_t> parent(nn, -1);
  for (int64_t i = 0; i < nn; ++i)
    if (!NA[i].leaf) parent[NA[i].left] = parent[NA[i].right] = (int32_t)i;
  for (int64_t i = 0; i < nn; ++i)
    if (!NA[i].root && NA[i].mr != NA[i].nr)
      return set_error(HSS_ERR_BAD_DIMS, "hssA's reduced blocks are not square (ranks above the block sizes)");
  const int H = NA[0].height;
  const std::vector<Gen> gA = plan_views(hA);

  std::vector<Level> lev;
  std::vector<PlanPtr> Y0(H + 1);
  PlanPtr Bown;              // B_l for l > 0
  hss_plan_s* Bcur = hB;
  int top = H;               // the level whose solution starts the backward pass
  PlanPtr Ytop;
  for (int l = 0; l <= H; ++l) {
    lev.push_back(make_level(NA, parent, l));
    const Level& L = lev.back();
    const int64_t tn = (int64_t)L.mem.size();
    const std::vector<Node>& NB = plan_nodes(Bcur);
    const std::vector<Gen> gB = plan_views(Bcur);
    // rows of B_l's leaves: a node's block as it enters its reduction, or the
    // k rows it kept after it
    for (int64_t t = 0; t < tn; ++t) {
      if (!L.leaf[t]) continue;
      const Node& x = NA[L.mem[t]];
      const int64_t want = x.height == l ? x.m : x.mr;
      if (NB[t].gm != want) return set_error(HSS_ERR_BAD_DIMS, "division: unexpected block rows");
    }
    Arena ar;
    ar.on_stream(st);
    ar.rg = &rg;
    Stages S{st, ar, {}, {}};
    S.rg = &rg;
    DivList dv;
    dv.rg = &rg;
    if (l == H) {
      // the root (:23-26): Y = D^-1 B, U and V of B (none at the root)
      Shape SY = shape_of(Bcur);
      std::vector<Gen> gy;
      if ((rc = make_plan(SY, Ytop, gy, &rg))) return rc;
      dv.add(dn + 0, fb, DIV_ROOT, gB[0].D, gy[0].D, nullptr, NA[0].m);
      cudaError_t e = dv.run(ar, st);
      if (e != cudaSuccess) return set_cuda_error(e, "division root solve");
      break;
    }
    // ---- QB, Y0 and the reduced A on T_l ----
    Shape SQ(tn), SY(tn), SL(tn);
    link(SQ, L, NA);
    link(SY, L, NA);
    link(SL, L, NA);
    for (int64_t t = 0; t < tn; ++t) {
      const Node& x = NA[L.mem[t]];
      SQ.ku[t] = SY.ku[t] = NB[t].root ? 0 : NB[t].ku;
      SQ.kv[t] = SY.kv[t] = NB[t].root ? 0 : NB[t].kv;
      SL.ku[t] = x.root ? 0 : x.ku;
      SL.kv[t] = x.root ? 0 : x.kv;
      if (L.leaf[t]) {
        SQ.m[t] = x.mr;
        SY.m[t] = NB[t].gm;
        SQ.n[t] = SY.n[t] = NB[t].gn;
        SL.m[t] = x.mr;
        SL.n[t] = x.height == l ? x.n : x.nr;
      }
    }
    PlanPtr QB, YL, LA;
    std::vector<Gen> gq, gy, gl;
    if ((rc = make_plan(SQ, QB, gq, &rg)) || (rc = make_plan(SY, YL, gy, &rg)) || (rc = make_plan(SL, LA, gl, &rg)))
      return rc;
    for (int64_t t = 0; t < tn; ++t) {
      const int32_t a = L.mem[t];
      const Node& x = NA[a];
      if (!L.leaf[t]) {
        for (auto* dst : {&gq, &gy}) {
          Gen& d = (*dst)[t];
          S.copy(d.B12, gB[t].B12); S.copy(d.B21, gB[t].B21);
          S.copy(d.R1, gB[t].R1); S.copy(d.R2, gB[t].R2);
          S.copy(d.W1, gB[t].W1); S.copy(d.W2, gB[t].W2);
        }
        S.copy(gl[t].B12, gA[a].B12); S.copy(gl[t].B21, gA[a].B21);
        S.copy(gl[t].R1, gA[a].R1); S.copy(gl[t].R2, gA[a].R2);
        S.copy(gl[t].W1, gA[a].W1); S.copy(gl[t].W2, gA[a].W2);
        continue;
      }
      const bool fresh = x.height == l;
      S.copy(gq[t].V, gB[t].V);
      S.copy(gy[t].V, gB[t].V);
      if (fresh && x.mk > 0) {
        // U-transforms, row split and L-transforms (:30-32, :115-129)
        dv.add(dn + a, fb, DIV_QL, gB[t].D, gy[t].D, &gq[t].D, x.m, x.m - x.mk);
        dv.add(dn + a, fb, DIV_QL, gB[t].U, gy[t].U, &gq[t].U, x.m, x.m - x.mk);
      } else {
        S.copy(gq[t].D, gB[t].D);
        S.copy(gq[t].U, gB[t].U);
        S.zero(gy[t].D);
        S.zero(gy[t].U);
      }
      // the reduced leaf of A: L2 (or the remainder kept since), tril U, Q V
      const int64_t c0 = fresh ? 0 : x.nk;
      S.copy(gl[t].D, view(fb + x.fD + x.mk + c0 * x.m, x.mr, SL.n[t], x.m));
      const Blk Ur = view(fb + x.fU + x.mk, x.mr, x.ku, x.m);
      if (x.lower_u) S.tril(gl[t].U, Ur);
      else S.copy(gl[t].U, Ur);
      S.copy(gl[t].V, view(fb + x.fV + c0, SL.n[t], x.kv, x.n));
    }
    if ((rc = run_stages(S, ar))) return rc;
    cudaError_t e = dv.run(ar, st);
    if (e != cudaSuccess) return set_cuda_error(e, "division row transforms");
    const std::vector<Node>& NQ = plan_nodes(QB.get());
    if (NQ[0].gm == 0) {
      // every row eliminated (:35): the solution is Y0 after the V-transforms
      top = l;
      Ytop = std::move(YL);
      break;
    }
    // ---- QB - L * Y0, recompressed and pruned (:38-40) ----
    hss_handle Pp = nullptr;
    if ((rc = hss_hssmul(LA.get(), YL.get(), &Pp, st))) return rc;
    PlanPtr P(Pp);
    reg_plan(&rg, Pp);
    LA.reset();
    const std::vector<Node>& NP = plan_nodes(P.get());
    const std::vector<Gen> gp = plan_views(P.get());
    Shape SS(tn);
    link(SS, L, NA);
    for (int64_t t = 0; t < tn; ++t) {
      SS.ku[t] = t == 0 ? 0 : SQ.ku[t] + NP[t].ku;
      SS.kv[t] = t == 0 ? 0 : SQ.kv[t] + NP[t].kv;
      SS.m[t] = SQ.m[t];
      SS.n[t] = SQ.n[t];
    }
    PlanPtr Sd;
    std::vector<Gen> gs;
    if ((rc = make_plan(SS, Sd, gs, &rg))) return rc;
    // stage 1: every block that is not fully written zeroed, first terms copied
    for (int64_t t = 0; t < tn; ++t) {
      if (L.leaf[t]) {
        S.copy(gs[t].D, gq[t].D);
        S.copy(sub(gs[t].U, 0, 0, SS.m[t], SQ.ku[t]), gq[t].U);
        S.copy(sub(gs[t].U, 0, SQ.ku[t], SS.m[t], NP[t].ku), gp[t].U);
        S.copy(sub(gs[t].V, 0, 0, SS.n[t], SQ.kv[t]), gq[t].V);
        S.copy(sub(gs[t].V, 0, SQ.kv[t], SS.n[t], NP[t].kv), gp[t].V);
      } else {
        for (Blk* b : {&gs[t].B12, &gs[t].B21, &gs[t].R1, &gs[t].R2, &gs[t].W1, &gs[t].W2}) S.zero(*b);
      }
    }
    if ((rc = run_stages(S, ar))) return rc;
    // stage 2: D -= D_P; block-diagonal couplings and translators (:225)
    for (int64_t t = 0; t < tn; ++t) {
      if (L.leaf[t]) {
        S.axpy(gs[t].D, gp[t].D, -1.0, 1.0);
        continue;
      }
      const int32_t a = SS.left[t], b = SS.right[t];
      S.copy(sub(gs[t].B12, 0, 0, SQ.ku[a], SQ.kv[b]), gq[t].B12);
      S.axpy(sub(gs[t].B12, SQ.ku[a], SQ.kv[b], NP[a].ku, NP[b].kv), gp[t].B12, -1.0, 0.0);
      S.copy(sub(gs[t].B21, 0, 0, SQ.ku[b], SQ.kv[a]), gq[t].B21);
      S.axpy(sub(gs[t].B21, SQ.ku[b], SQ.kv[a], NP[b].ku, NP[a].kv), gp[t].B21, -1.0, 0.0);
      if (t == 0) continue;
      S.copy(sub(gs[t].R1, 0, 0, SQ.ku[a], SQ.ku[t]), gq[t].R1);
      S.copy(sub(gs[t].R1, SQ.ku[a], SQ.ku[t], NP[a].ku, NP[t].ku), gp[t].R1);
      S.copy(sub(gs[t].R2, 0, 0, SQ.ku[b], SQ.ku[t]), gq[t].R2);
      S.copy(sub(gs[t].R2, SQ.ku[b], SQ.ku[t], NP[b].ku, NP[t].ku), gp[t].R2);
      S.copy(sub(gs[t].W1, 0, 0, SQ.kv[a], SQ.kv[t]), gq[t].W1);
      S.copy(sub(gs[t].W1, SQ.kv[a], SQ.kv[t], NP[a].kv, NP[t].kv), gp[t].W1);
      S.copy(sub(gs[t].W2, 0, 0, SQ.kv[b], SQ.kv[t]), gq[t].W2);
      S.copy(sub(gs[t].W2, SQ.kv[b], SQ.kv[t], NP[b].kv, NP[t].kv), gp[t].W2);
    }
    if ((rc = run_stages(S, ar))) return rc;
    P.reset();
    QB.reset();
    hss_plan_s* Qr = nullptr;
    if ((rc = recompress_impl(Sd.get(), atol, rtol, false, &Qr, st))) return rc;
    PlanPtr QC(Qr);
    reg_plan(&rg, Qr);
    Sd.reset();
    // ---- prune_leaves! onto T_{l+1} ----
    const Level L1 = make_level(NA, parent, l + 1);
    const int64_t tn1 = (int64_t)L1.mem.size();
    const std::vector<Node>& NC = plan_nodes(QC.get());
    const std::vector<Gen> gc = plan_views(QC.get());
    Shape SN(tn1);
    link(SN, L1, NA);
    for (int64_t u = 0; u < tn1; ++u) {
      const int32_t a = L1.mem[u];
      const int32_t t = L.pos[a];
      SN.ku[u] = u == 0 ? 0 : NC[t].ku;
      SN.kv[u] = u == 0 ? 0 : NC[t].kv;
      if (!L1.leaf[u]) continue;
      if (L.leaf[t]) {
        SN.m[u] = NC[t].gm;
        SN.n[u] = NC[t].gn;
      } else {
        const Node &c1 = NC[NC[t].left], &c2 = NC[NC[t].right];
        SN.m[u] = c1.gm + c2.gm;
        SN.n[u] = c1.gn + c2.gn;
      }
    }
    PlanPtr Bn;
    std::vector<Gen> gn;
    if ((rc = make_plan(SN, Bn, gn, &rg))) return rc;
    struct Mid { Blk X12, X21; };
    std::vector<Mid> mid(tn1);
    for (int64_t u = 0; u < tn1; ++u) {
      const int32_t t = L.pos[L1.mem[u]];
      if (!L1.leaf[u]) {
        S.copy(gn[u].B12, gc[t].B12); S.copy(gn[u].B21, gc[t].B21);
        S.copy(gn[u].R1, gc[t].R1); S.copy(gn[u].R2, gc[t].R2);
        S.copy(gn[u].W1, gc[t].W1); S.copy(gn[u].W2, gc[t].W2);
      } else if (L.leaf[t]) {
        S.copy(gn[u].D, gc[t].D); S.copy(gn[u].U, gc[t].U); S.copy(gn[u].V, gc[t].V);
      } else {
        // _hssleaf (src/hssmatrix.jl:339-348): [D1 U1 B12 V2'; U2 B21 V1' D2],
        // [U1 R1; U2 R2], [V1 W1; V2 W2]
        const int32_t c1 = NC[t].left, c2 = NC[t].right;
        const int64_t m1 = NC[c1].gm, n1 = NC[c1].gn, m2 = NC[c2].gm, n2 = NC[c2].gn;
        S.copy(sub(gn[u].D, 0, 0, m1, n1), gc[c1].D);
        S.copy(sub(gn[u].D, m1, n1, m2, n2), gc[c2].D);
        mid[u].X12 = ar.blk(gc[t].B12.rows, n2);
        mid[u].X21 = ar.blk(gc[t].B21.rows, n1);
        S.gemm(mid[u].X12, gc[t].B12, 0, gc[c2].V, 1);
        S.gemm(mid[u].X21, gc[t].B21, 0, gc[c1].V, 1);
        if (u != 0) {
          S.gemm(sub(gn[u].U, 0, 0, m1, SN.ku[u]), gc[c1].U, 0, gc[t].R1, 0);
          S.gemm(sub(gn[u].U, m1, 0, m2, SN.ku[u]), gc[c2].U, 0, gc[t].R2, 0);
          S.gemm(sub(gn[u].V, 0, 0, n1, SN.kv[u]), gc[c1].V, 0, gc[t].W1, 0);
          S.gemm(sub(gn[u].V, n1, 0, n2, SN.kv[u]), gc[c2].V, 0, gc[t].W2, 0);
        }
      }
    }
    if ((rc = run_stages(S, ar))) return rc;
    for (int64_t u = 0; u < tn1; ++u) {
      const int32_t t = L.pos[L1.mem[u]];
      if (!L1.leaf[u] || L.leaf[t]) continue;
      const int32_t c1 = NC[t].left, c2 = NC[t].right;
      const int64_t m1 = NC[c1].gm, n1 = NC[c1].gn, m2 = NC[c2].gm, n2 = NC[c2].gn;
      S.gemm(sub(gn[u].D, 0, n1, m1, n2), gc[c1].U, 0, mid[u].X12, 0);
      S.gemm(sub(gn[u].D, m1, 0, m2, n1), gc[c2].U, 0, mid[u].X21, 0);
    }
    if ((rc = run_stages(S, ar))) return rc;
    e = cudaStreamSynchronize(st);   // the arena's blocks are freed on return
    if (e != cudaSuccess) return set_cuda_error(e, "division prune");
    Y0[l] = std::move(YL);
    Bown = std::move(Bn);
    Bcur = Bown.get();
  }

  // ---- backward: unpack, V-transforms, recompress (:50-52) ----
  PlanPtr Y1 = std::move(Ytop);
  if (top < H) {
    // the early exit: V-transforms of Y0 at level `top`, no recompression
    Arena ar;
    ar.on_stream(st);
    ar.rg = &rg;
    DivList dv;
    dv.rg = &rg;
    const Level& L = lev[top];
    const std::vector<Gen> gy = plan_views(Y1.get());
    for (size_t t = 0; t < L.mem.size(); ++t) {
      const Node& x = NA[L.mem[t]];
      if (!L.leaf[t] || x.height != top || x.mk == 0) continue;
      dv.add(dn + L.mem[t], fb, DIV_LQ, gy[t].D, gy[t].D, nullptr, x.n);
      dv.add(dn + L.mem[t], fb, DIV_LQ, gy[t].U, gy[t].U, nullptr, x.n);
    }
    cudaError_t e = dv.run(ar, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_cuda_error(e, "division");
  }
  for (int l = top - 1; l >= 0; --l) {
    const Level& L = lev[l];
    const Level& L1 = lev[l + 1];
    const int64_t tn = (int64_t)L.mem.size();
    const std::vector<Node>& N0 = plan_nodes(Y0[l].get());
    const std::vector<Node>& N1 = plan_nodes(Y1.get());
    const std::vector<Gen> g0 = plan_views(Y0[l].get());
    const std::vector<Gen> g1 = plan_views(Y1.get());
    auto ku0 = [&](int64_t t) -> int64_t { return N0[t].root ? 0 : N0[t].ku; };
    auto kv0 = [&](int64_t t) -> int64_t { return N0[t].root ? 0 : N0[t].kv; };
    auto ku1 = [&](int64_t u) -> int64_t { return N1[u].root ? 0 : N1[u].ku; };
    auto kv1 = [&](int64_t u) -> int64_t { return N1[u].root ? 0 : N1[u].kv; };
    Shape SZ(tn);
    link(SZ, L, NA);
    for (int64_t t = 0; t < tn; ++t) {
      SZ.m[t] = N0[t].leaf ? N0[t].gm : 0;
      SZ.n[t] = N0[t].leaf ? N0[t].gn : 0;
      const int32_t a = L.mem[t];
      const int32_t u = L1.pos[a];
      if (u >= 0) {
        // a node of both trees: ranks add up (:185-191, :225-231)
        SZ.ku[t] = t == 0 ? 0 : ku0(t) + ku1(u);
        SZ.kv[t] = t == 0 ? 0 : kv0(t) + kv1(u);
      }
      if (!L.leaf[t] && L1.leaf[u]) {
        // a node pruned at l + 1 and its two leaves (:199-215)
        const int64_t r = ku1(u), w = kv1(u);
        const int32_t c1 = SZ.left[t], c2 = SZ.right[t];
        const int64_t q1 = NA[L.mem[c1]].mr, q2 = NA[L.mem[c2]].mr;
        if (N1[u].gm != q1 + q2 || N1[u].gn != N0[c1].gn + N0[c2].gn)
          return set_error(HSS_ERR_BAD_DIMS, "division: unexpected block of the reduced solution");
        SZ.ku[c1] = ku0(c1) + r + q1;
        SZ.kv[c1] = kv0(c1) + w + q2;
        SZ.ku[c2] = ku0(c2) + r + q2;
        SZ.kv[c2] = kv0(c2) + w + q1;
      }
    }
    PlanPtr Z;
    std::vector<Gen> gz;
    if ((rc = make_plan(SZ, Z, gz, &rg))) return rc;
    Arena ar;
    ar.on_stream(st);
    ar.rg = &rg;
    Stages S{st, ar, {}, {}};
    S.rg = &rg;
    // stage 1: zeros (blocks with identity or sparse parts) and the leaves' D
    for (int64_t t = 0; t < tn; ++t) {
      if (L.leaf[t]) {
        S.copy(gz[t].D, g0[t].D);
        S.zero(gz[t].U);
      } else {
        for (Blk* b : {&gz[t].B12, &gz[t].B21, &gz[t].R1, &gz[t].R2, &gz[t].W1, &gz[t].W2}) S.zero(*b);
      }
    }
    if ((rc = run_stages(S, ar))) return rc;
    // stage 2
    for (int64_t t = 0; t < tn; ++t) {
      const int32_t a = L.mem[t];
      const int32_t u = L1.pos[a];
      if (L.leaf[t]) {
        S.copy(sub(gz[t].U, 0, 0, SZ.m[t], ku0(t)), g0[t].U);
        S.copy(sub(gz[t].V, 0, 0, SZ.n[t], kv0(t)), g0[t].V);
        if (u < 0) continue;   // a leaf under a node pruned at l + 1 (below)
        // a leaf of both trees (:225-231): D's last k rows += D1, U = [U0 [0; U1]], V = [V0 V1]
        const int64_t k = N1[u].gm, m = SZ.m[t];
        if (k > m || N1[u].gn != SZ.n[t])
          return set_error(HSS_ERR_BAD_DIMS, "division: unexpected block of the reduced solution");
        S.axpy(sub(gz[t].D, m - k, 0, k, SZ.n[t]), g1[u].D, 1.0, 1.0);
        S.copy(sub(gz[t].U, m - k, ku0(t), k, ku1(u)), g1[u].U);
        S.copy(sub(gz[t].V, 0, kv0(t), SZ.n[t], kv1(u)), g1[u].V);
        continue;
      }
      const int32_t c1 = SZ.left[t], c2 = SZ.right[t];
      if (!L1.leaf[u]) {
        // a branch of both trees: block-diagonal generators (:185-191)
        const int32_t d1 = L1.pos[L.mem[c1]], d2 = L1.pos[L.mem[c2]];
        S.copy(sub(gz[t].B12, 0, 0, ku0(c1), kv0(c2)), g0[t].B12);
        S.copy(sub(gz[t].B12, ku0(c1), kv0(c2), ku1(d1), kv1(d2)), g1[u].B12);
        S.copy(sub(gz[t].B21, 0, 0, ku0(c2), kv0(c1)), g0[t].B21);
        S.copy(sub(gz[t].B21, ku0(c2), kv0(c1), ku1(d2), kv1(d1)), g1[u].B21);
        if (t == 0) continue;
        S.copy(sub(gz[t].R1, 0, 0, ku0(c1), ku0(t)), g0[t].R1);
        S.copy(sub(gz[t].R1, ku0(c1), ku0(t), ku1(d1), ku1(u)), g1[u].R1);
        S.copy(sub(gz[t].R2, 0, 0, ku0(c2), ku0(t)), g0[t].R2);
        S.copy(sub(gz[t].R2, ku0(c2), ku0(t), ku1(d2), ku1(u)), g1[u].R2);
        S.copy(sub(gz[t].W1, 0, 0, kv0(c1), kv0(t)), g0[t].W1);
        S.copy(sub(gz[t].W1, kv0(c1), kv0(t), kv1(d1), kv1(u)), g1[u].W1);
        S.copy(sub(gz[t].W2, 0, 0, kv0(c2), kv0(t)), g0[t].W2);
        S.copy(sub(gz[t].W2, kv0(c2), kv0(t), kv1(d2), kv1(u)), g1[u].W2);
        continue;
      }
      // a node pruned at l + 1 (:199-215): Y1's leaf u unpacked into the leaves c1, c2
      const int64_t r = ku1(u), w = kv1(u);
      const int64_t q1 = NA[L.mem[c1]].mr, q2 = NA[L.mem[c2]].mr;
      const int64_t m1 = SZ.m[c1], n1 = SZ.n[c1], m2 = SZ.m[c2], n2 = SZ.n[c2];
      S.copy(sub(gz[t].B12, 0, 0, ku0(c1), kv0(c2)), g0[t].B12);
      S.eye(sub(gz[t].B12, ku0(c1) + r, kv0(c2) + w, q1, q1));
      S.copy(sub(gz[t].B21, 0, 0, ku0(c2), kv0(c1)), g0[t].B21);
      S.eye(sub(gz[t].B21, ku0(c2) + r, kv0(c1) + w, q2, q2));
      if (t != 0) {
        S.copy(sub(gz[t].R1, 0, 0, ku0(c1), ku0(t)), g0[t].R1);
        S.eye(sub(gz[t].R1, ku0(c1), ku0(t), r, r));
        S.copy(sub(gz[t].R2, 0, 0, ku0(c2), ku0(t)), g0[t].R2);
        S.eye(sub(gz[t].R2, ku0(c2), ku0(t), r, r));
        S.copy(sub(gz[t].W1, 0, 0, kv0(c1), kv0(t)), g0[t].W1);
        S.eye(sub(gz[t].W1, kv0(c1), kv0(t), w, w));
        S.copy(sub(gz[t].W2, 0, 0, kv0(c2), kv0(t)), g0[t].W2);
        S.eye(sub(gz[t].W2, kv0(c2), kv0(t), w, w));
      }
      const Blk& D1 = g1[u].D;
      // leaf c1 (:214, :236-252): its last q1 rows += D1[0:q1, 0:n1];
      // U = [U0, [0; U1[0:q1]], [0; I]]; V = [V0, V1[0:n1], D1[q1:, 0:n1]^T]
      S.axpy(sub(gz[c1].D, m1 - q1, 0, q1, n1), sub(D1, 0, 0, q1, n1), 1.0, 1.0);
      S.copy(sub(gz[c1].U, m1 - q1, ku0(c1), q1, r), sub(g1[u].U, 0, 0, q1, r));
      S.eye(sub(gz[c1].U, m1 - q1, ku0(c1) + r, q1, q1));
      S.copy(sub(gz[c1].V, 0, kv0(c1), n1, w), sub(g1[u].V, 0, 0, n1, w));
      S.copy(sub(gz[c1].V, 0, kv0(c1) + w, n1, q2), sub(D1, q1, 0, q2, n1), 1);
      // leaf c2 (:215)
      S.axpy(sub(gz[c2].D, m2 - q2, 0, q2, n2), sub(D1, q1, n1, q2, n2), 1.0, 1.0);
      S.copy(sub(gz[c2].U, m2 - q2, ku0(c2), q2, r), sub(g1[u].U, q1, 0, q2, r));
      S.eye(sub(gz[c2].U, m2 - q2, ku0(c2) + r, q2, q2));
      S.copy(sub(gz[c2].V, 0, kv0(c2), n2, w), sub(g1[u].V, n1, 0, n2, w));
      S.copy(sub(gz[c2].V, 0, kv0(c2) + w, n2, q1), sub(D1, 0, n1, q1, n2), 1);
    }
    if ((rc = run_stages(S, ar))) return rc;
    // V-transforms of the leaves reduced at this level (:51, :130-136)
    DivList dv;
    dv.rg = &rg;
    for (int64_t t = 0; t < tn; ++t) {
      const Node& x = NA[L.mem[t]];
      if (!L.leaf[t] || x.height != l || x.mk == 0) continue;
      dv.add(dn + L.mem[t], fb, DIV_LQ, gz[t].D, gz[t].D, nullptr, x.n);
      dv.add(dn + L.mem[t], fb, DIV_LQ, gz[t].U, gz[t].U, nullptr, x.n);
    }
    cudaError_t e = dv.run(ar, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_cuda_error(e, "division unpack");
    Y0[l].reset();
    Y1.reset();
    hss_plan_s* Yr = nullptr;
    if ((rc = recompress_impl(Z.get(), atol, rtol, false, &Yr, st))) return rc;
    reg_plan(&rg, Yr);
    Y1.reset(Yr);
  }
  result = std::move(Y1);
  return HSS_OK;
}

}  // namespace

int hss::plan_transpose(const hss_plan_s* h, hss_plan_s** out, cudaStream_t st) {
  PlanPtr T;
  int rc = transpose_impl(h, T, st);
  if (rc) return rc;
  *out = T.release();
  return HSS_OK;
}

extern "C" {

int hss_transpose(hss_handle h, hss_handle* out, void* stream) {
  if (!h || !out) return set_error(HSS_ERR_INVALID, "null handle");
  *out = nullptr;
  if (plan_ntrees(h) != 1) return set_error(HSS_ERR_INVALID, "transpose takes a single-tree handle");
  cudaError_t e = cudaSetDevice(plan_device(h));
  if (e != cudaSuccess) return set_cuda_error(e, "cudaSetDevice");
  PlanPtr T;
  int rc = transpose_impl(h, T, (cudaStream_t)stream);
  if (rc) return rc;
  *out = T.release();
  return HSS_OK;
}

int hss_ldiv(hss_handle hA, hss_handle hB, double atol, double rtol, hss_handle* out, void* stream) {
  if (!hA || !hB || !out) return set_error(HSS_ERR_INVALID, "null handle");
  *out = nullptr;
  if (plan_ntrees(hA) != 1 || plan_ntrees(hB) != 1) return set_error(HSS_ERR_INVALID, "ldiv takes single-tree handles");
  if (!(atol >= 0.0) || !(rtol >= 0.0)) return set_error(HSS_ERR_INVALID, "tolerances must be >= 0");
  if (plan_device(hA) != plan_device(hB)) return set_error(HSS_ERR_INVALID, "handles on different devices");
  cudaError_t e = cudaSetDevice(plan_device(hA));
  if (e != cudaSuccess) return set_cuda_error(e, "cudaSetDevice");
  PlanPtr X;
  int rc = ldiv_impl(hA, hB, atol, rtol, X, (cudaStream_t)stream);
  if (rc) return rc;
  *out = X.release();
  return HSS_OK;
}

int hss_rdiv(hss_handle hB, hss_handle hA, double atol, double rtol, hss_handle* out, void* stream) {
  if (!hA || !hB || !out) return set_error(HSS_ERR_INVALID, "null handle");
  *out = nullptr;
  if (plan_ntrees(hA) != 1 || plan_ntrees(hB) != 1) return set_error(HSS_ERR_INVALID, "rdiv takes single-tree handles");
  if (!(atol >= 0.0) || !(rtol >= 0.0)) return set_error(HSS_ERR_INVALID, "tolerances must be >= 0");
  if (plan_device(hA) != plan_device(hB)) return set_error(HSS_ERR_INVALID, "handles on different devices");
  cudaError_t e = cudaSetDevice(plan_device(hA));
  if (e != cudaSuccess) return set_cuda_error(e, "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  // rdiv!(hssB, hssA) = adjoint(_ldiv!(adjoint(hssA), adjoint(hssB))) (src/ulvdivide.jl:15-17)
  PlanPtr At, Bt, Xt, X;
  int rc = transpose_impl(hA, At, st);
  if (!rc) rc = transpose_impl(hB, Bt, st);
  if (!rc) rc = ldiv_impl(At.get(), Bt.get(), atol, rtol, Xt, st);
  if (!rc) rc = transpose_impl(Xt.get(), X, st);
  if (rc) return rc;
  *out = X.release();
  return HSS_OK;
}

}  // extern "C"
