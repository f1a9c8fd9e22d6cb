// Internal data layout shared by the host plan code and the sm_103a kernels.
//
// A plan is a forest of HSS generator trees held on one GPU:
//   * all generators of all trees live in one FP64 buffer (the packed layout
//     the caller uploads, column-major blocks);
//   * a device array of `Node` descriptors (one per tree node) carries sizes,
//     generator pointers and workspace / factor-storage offsets;
//   * task lists group nodes by height (post-order sweeps: product upsweep,
//     ULV factor, ULV solve upward) and by depth (pre-order sweeps: product
//     downsweep, ULV solve downward).  One kernel launch processes one list,
//     one thread block per node, across every tree of the forest.
// Per-call data (right-hand sides, outputs, workspace, factor storage) is in
// a small `Slot` table indexed by Task::slot, so tasks of different plans can
// be mixed in one launch.
#pragma once
#include <cstdint>
#include <vector_types.h>

namespace hss {

struct Node {
  int32_t left, right, parent, leaf;   // indices into the same node array; -1 if none
  int32_t root, depth, height, tree;
  // ULV reduce-problem sizes (src/ulvfactor.jl:22-57): leaf m x n = D; a branch
  // holds the merged block of its children's reduced parts (src/ulvfactor.jl:74-79).
  int32_t m, n, ku, kv;                // ku/kv = gensize (src/hssmatrix.jl:254-262)
  int32_t k, mk, nk, mr;               // k=min(ku,m), mk=m-k, nk=min(mk,n), mr=m-mk
  int32_t nr, gm, gn, lower_u;         // nr=n-nk; gm x gn = rows x cols of the subtree
                                       // lower_u: 1 if the reduced U is tril (QL done)
  int64_t row0, col0;                  // first row / column of the subtree
  const double *D, *U, *V;             // leaf generators (ld = m, m, n)
  const double *B12, *B21, *R1, *R2, *W1, *W2;   // branch generators
  // workspace row offsets: product Z (kv rows), F (ku rows);
  // solve b (m rows), u (kv rows), x (n rows)
  int64_t wz, wf, wb, wu, wx;
  // factor storage element offsets: D (m x n; root: LU), U (m x ku),
  // V (n x kv), tau_ql (k), tau_lq (mk), T12 (mr1 x kv2), T21 (mr2 x kv1), pivots (root),
  // Qt (n x mk): the LQ reflectors as columns (explicit 1 on the diagonal, 0 above)
  int64_t fD, fU, fV, ftq, ftl, fT12, fT21, fpiv, fQt;
  // blocked FP32 solve: per panel of 32 reflectors the compact-WY T (32 x 32,
  // column-major) of the QL (fTq, ceil(k/32) panels) and LQ (fTl, ceil(mk/32))
  // reflectors, and the inverses of L1's 32 x 32 diagonal blocks (fLi)
  int64_t fTq, fTl, fLi;
  // tensor-core residual: byte offset of this leaf's prepared slices of D in
  // the plan's slice buffer (-1: none)
  int64_t fdx;
  // the children's ranks, leaf flags and product workspace offsets (left, right),
  // so that a product task reads one descriptor
  int32_t cku[2], ckv[2], cleaf[2];
  int64_t cwz[2], cwf[2];
};
static_assert(sizeof(Node) % 8 == 0, "Node is copied as 8-byte words");

// The edge from a non-root node x to its parent p, as the flat product reads
// it (one chain of small products per leaf): the translators of p that act on
// x, the F slots of x and of its sibling, the ranks involved and x's leaves.
struct FlatLink {
  const double* W;      // W1 or W2 of p (kv x kpv, ld kv): Z_p += W^T Z_x
  const double* R;      // R1 or R2 of p (ku x kpu, ld ku): F_x = G_x + R F_p
  const double* B;      // B21 (x left) or B12 (x right) of p (sku x kv, ld sku): G_sibling = B Z_x
  int64_t wf, swf;      // product workspace rows of F_x and of F_sibling
  int32_t ku, kv, kpu, kpv, sku, depth;
  int32_t lf0, lfn;     // x's leaves: positions lf0 .. lf0 + lfn - 1 of the leaf list
};
static_assert(sizeof(FlatLink) % 8 == 0, "FlatLink is copied as 8-byte words");

struct Task {
  const Node* nodes;   // node array the index refers to
  int32_t node;
  int32_t slot;
};

struct Slot {
  const double* B;  int64_t ldb;      // product input / solve right-hand side
  double* C;        int64_t ldc;      // product output / solve output
  const double* Y;  int64_t ldy;      // product beta-term input (may alias C)
  double alpha, beta;
  void* ws;         int64_t ldws;     // workspace (double for products, T for solves)
  void* fbase;                        // factor storage (T)
  const double* colscale;             // solve: rhs column j is divided by colscale[j] ...
  const double* colinv;               // ... i.e. multiplied by colinv[j] = 1 / colscale[j]
  double* colnorm2;                   // product: += sum_i C(i,j)^2 per column (nullable)
  int32_t r, mode;                    // solve: mode 0 x = s*d, 1 x += s*d
  int32_t* err;                       // device status word (nullable)
  // double-float product: X split into (hi, lo) pairs, the D X partial
  // products, pair workspace (same row offsets as ws), and the generators
  // as pairs (gdf[e] pairs gbase[e]).
  const float2* xs;  int64_t ldx2;
  float2* tmp;       int64_t ldt2;
  float2* ws2;
  const float2* gdf;
  const double* gbase;
  // persistent product (hss_pmv.cu): the node array of this slot's plan and
  // its per-node event counters (even between launches)
  const Node* nodes;
  int32_t* sync;
  // tensor-core residual: the plan's prepared slices of the leaf blocks D
  const unsigned char* dxs;
};

// Entry extraction (hss_getindex.cu): per node, the node's part of the sorted
// requested rows [rlo, rlo + rcnt) and columns [clo, clo + ccnt), and the
// workspace offsets of its restricted bases Ub (rcnt x ku), Vb (ccnt x kv) and,
// at a branch, of T12 = Ub1 B12 (rcnt1 x kv2) and T21 = Ub2 B21 (rcnt2 x kv1).
struct GiRange {
  int64_t rlo, rcnt, clo, ccnt;
  int64_t ub, vb, t12, t21;
};

// One 64 x 64 output tile of an off-diagonal block: out rows
// [rs + r0, rs + r0 + rows) of the sorted row list, columns [cs + c0, ...),
// value sum_q ws[T + (r0 + i) + q ldt] ws[V + (c0 + j) + q ldv], q < k.
struct GiTile {
  int64_t T, V, ldt, ldv;
  int64_t rs, cs;
  int32_t r0, c0, rows, cols, k, pad;
};

// One task of the HSS x HSS product (hss_hssmul.cu):
// C (m x n, ld ldc) = a1 op(A1) op(B1) + a2 op(A2) op(B2) + beta C, op = transpose
// when ta / tb is set; K = k1 (k2) columns of op(A); A2 may be null.  k1 = -1:
// a block copy by cmode: MM_COPY C = op(A1) (A1 null: zeros), MM_AXPY
// C = a1 op(A1) + beta C, MM_TRIL C = the lower triangle of op(A1) (zeros above
// the diagonal), MM_EYE C = the identity.
enum { MM_COPY = 0, MM_AXPY = 1, MM_TRIL = 2, MM_EYE = 3 };
struct MmTask {
  const double *A1, *B1, *A2, *B2;
  double* C;
  int32_t lda1, ldb1, lda2, ldb2, ldc;
  int32_t m, n, k1, k2;
  int32_t ta1, tb1, ta2, tb2;
  int32_t cmode;
  double a1, a2, beta;
};

// One block of rows transformed with a factored node of an FP64 ULV
// factorization (hss_divide.cu): columns [0, cols) of src (rows x cols, ld
// lds).  DIV_QL: Q_ql^T, then the first mk rows solved with L1 and written to
// top (rows x cols, the other rows zero), the last rows - mk rows written to
// bot.  DIV_LQ: Q_lq^T, written to top.  DIV_ROOT: the root block's LU solve,
// written to top.  top may alias src.
enum { DIV_QL = 0, DIV_LQ = 1, DIV_ROOT = 2 };
struct DivTask {
  const Node* nd;       // the factored node (device descriptor)
  const double* fb;     // the factorization's storage
  const double* src;
  double* top;
  double* bot;
  int64_t lds, ldt, ldb;
  int32_t rows, cols, mode, pad;
};

// One truncated column-pivoted QR (hss_recompress.cu): G (p x q, ld ldg) is
// factored in place; the rank (leading |R_jj| > max(atol, rtol |R_11|)) goes to
// *rank, Q's first rank columns to Q (ld ldq), R's first rank rows with the
// pivoting undone to R (ld ldr).
struct PqrTask {
  double* G;
  int64_t ldg;
  int32_t p, q;
  double* Q;
  int64_t ldq;
  double* R;
  int64_t ldr;
  double atol, rtol;
  int32_t* rank;
};

// device status codes written into Slot::err
enum { DEV_OK = 0, DEV_SINGULAR = 1, DEV_BAD = 2, DEV_TIMEOUT = 3 };

// State of the refinement loop run on the device (hss_ulvsolve with a
// tolerance): written by the convergence check after every residual.
struct RefineStatus {
  double residual;      // largest relative residual over all columns (NaN if any is NaN)
  int32_t iterations;   // refinement steps before this residual
  int32_t converged;    // residual <= tol
  int32_t next;         // steps taken so far: the loop continues while next grows
  int32_t pad;
};

}  // namespace hss
