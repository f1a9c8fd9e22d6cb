// Host-side building blocks of the device HSS arithmetic (hss_arith.cpp,
// hss_divide.cpp): column-major device blocks, a chunked device arena for
// intermediate blocks, and task lists of small dense products, copies and
// pivoted QRs run stage by stage on one stream.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <utility>
#include <vector>

#include "hss_host.h"
#include "hss_internal.h"
#include "hss_launch.h"

struct hss_plan_s;

namespace hss {

// A column-major block on the device: data, leading dimension, shape.
struct Blk {
  double* p = nullptr;
  int64_t ld = 1, rows = 0, cols = 0;
  double* at(int64_t i, int64_t j) const { return p + i + j * ld; }
};

// Device address ranges the blocks of a task list must lie in.  Checked on
// the host as the tasks are queued: a block outside every range (a shape bug)
// marks the list bad, and the list is then not launched.
struct Ranges {
  std::vector<std::pair<const char*, const char*>> r;
  bool bad = false;
  void add(const void* p, size_t bytes) {
    if (p && bytes) r.emplace_back((const char*)p, (const char*)p + bytes);
  }
  bool inside(const double* p, int64_t ld, int64_t rows, int64_t cols) const {
    if (rows <= 0 || cols <= 0) return true;
    if (!p || ld < rows) return false;
    const char* lo = (const char*)p;
    const char* hi = (const char*)(p + (rows - 1) + (cols - 1) * ld + 1);
    for (const auto& x : r)
      if (lo >= x.first && hi <= x.second) return true;
    return false;
  }
  void check(const double* p, int64_t ld, int64_t rows, int64_t cols) {
    if (!inside(p, ld, rows, cols)) bad = true;
  }
};

// Device memory for the intermediate blocks: chunks of at least 64 MB (16 MB
// from the stream-ordered pool), freed together.
struct Arena {
  Ranges* rg = nullptr;   // chunks are registered here when set
  bool async = false;     // chunks from the pool, ordered on `ast`
  cudaStream_t ast = nullptr;
  void on_stream(cudaStream_t s) {
    async = true;
    ast = s;
  }
  std::vector<void*> chunks;
  char* cur = nullptr;
  size_t left = 0;
  cudaError_t err = cudaSuccess;
  void* raw(size_t bytes) {
    bytes = (std::max<size_t>(bytes, 16) + 255) & ~size_t(255);
    if (bytes > left) {
      const size_t sz = std::max<size_t>(bytes, size_t(async ? 16 : 64) << 20);
      void* q = nullptr;
      const cudaError_t e = async ? dev_alloc_async(&q, sz, ast) : dev_alloc(&q, sz);
      if (e != cudaSuccess) { err = e; return nullptr; }
      chunks.push_back(q);
      if (rg) rg->add(q, sz);
      cur = (char*)q;
      left = sz;
    }
    void* r = cur;
    cur += bytes;
    left -= bytes;
    return r;
  }
  Blk blk(int64_t rows, int64_t cols) {
    Blk b;
    b.rows = rows;
    b.cols = cols;
    b.ld = std::max<int64_t>(rows, 1);
    b.p = (double*)raw((size_t)b.ld * std::max<int64_t>(cols, 1) * sizeof(double));
    return b;
  }
  ~Arena() {
    for (void* q : chunks) {
      if (async) cudaFreeAsync(q, ast);
      else cudaFree(q);
    }
  }
};

// Task lists run stage by stage on one stream.
struct Stages {
  cudaStream_t st;
  Arena& ar;
  std::vector<MmTask> mm;
  std::vector<PqrTask> qr;
  int qmax = 1, kmax = 1;
  Ranges* rg = nullptr;   // when set, every queued block is checked against it
  void chk(const Blk& b, int64_t rows, int64_t cols) {
    if (rg) rg->check(b.p, b.ld, rows, cols);
  }
  // Output columns per task: larger products and copies are split into
  // column slices, so that one big block spreads over many thread blocks.
  static constexpr int64_t kSlice = 256;
  // the columns [j0, j0 + nc) of op(X) as a block of X
  static Blk cols_of(const Blk& X, int tx, int64_t j0, int64_t nc) {
    Blk b = X;
    if (tx) { b.p = X.p ? X.at(j0, 0) : nullptr; b.rows = nc; }
    else { b.p = X.p ? X.at(0, j0) : nullptr; b.cols = nc; }
    return b;
  }
  // rows [i0, i0 + nr) of op(X) as a block of X
  static Blk rows_of(const Blk& X, int tx, int64_t i0, int64_t nr) {
    Blk b = X;
    if (tx) { b.p = X.p ? X.at(0, i0) : nullptr; b.cols = nr; }
    else { b.p = X.p ? X.at(i0, 0) : nullptr; b.rows = nr; }
    return b;
  }
  static constexpr int64_t kRowSlice = 512;
  // C = A1 op B1 (+ A2 op B2): shapes from the blocks, ta / tb transpose
  void gemm(const Blk& C, const Blk& A1, int ta1, const Blk& B1, int tb1, const Blk* A2 = nullptr, int ta2 = 0,
            const Blk* B2 = nullptr, int tb2 = 0) {
    if (C.rows * C.cols == 0) return;
    if (C.rows > kRowSlice) {
      for (int64_t i0 = 0; i0 < C.rows; i0 += kRowSlice) {
        const int64_t nr = std::min(kRowSlice, C.rows - i0);
        Blk Ci = C; Ci.p = C.at(i0, 0); Ci.rows = nr;
        const Blk A1i = rows_of(A1, ta1, i0, nr);
        Blk A2i;
        if (A2) A2i = rows_of(*A2, ta2, i0, nr);
        gemm(Ci, A1i, ta1, B1, tb1, A2 ? &A2i : nullptr, ta2, B2, tb2);
      }
      return;
    }
    if (C.cols > kSlice) {
      for (int64_t j0 = 0; j0 < C.cols; j0 += kSlice) {
        const int64_t nc = std::min(kSlice, C.cols - j0);
        Blk Cj = C; Cj.p = C.at(0, j0); Cj.cols = nc;
        const Blk B1j = cols_of(B1, tb1, j0, nc);
        Blk B2j;
        if (A2) B2j = cols_of(*B2, tb2, j0, nc);
        gemm(Cj, A1, ta1, B1j, tb1, A2, ta2, A2 ? &B2j : nullptr, tb2);
      }
      return;
    }
    MmTask t{};
    const int64_t k1 = ta1 ? A1.rows : A1.cols;
    if (rg) {
      chk(C, C.rows, C.cols);
      if (k1 > 0) {
        chk(A1, A1.rows, A1.cols);
        chk(B1, B1.rows, B1.cols);
        if ((ta1 ? A1.cols : A1.rows) != C.rows || (tb1 ? B1.rows : B1.cols) != C.cols ||
            (tb1 ? B1.cols : B1.rows) != k1)
          rg->bad = true;
      }
      if (A2 && (ta2 ? A2->rows : A2->cols) > 0) {
        chk(*A2, A2->rows, A2->cols);
        chk(*B2, B2->rows, B2->cols);
      }
    }
    t.A1 = k1 > 0 ? A1.p : nullptr; t.B1 = B1.p; t.lda1 = (int32_t)A1.ld; t.ldb1 = (int32_t)B1.ld;
    t.ta1 = ta1; t.tb1 = tb1; t.k1 = (int32_t)k1; t.a1 = 1.0;
    if (A2) {
      const int64_t k2 = ta2 ? A2->rows : A2->cols;
      t.A2 = k2 > 0 ? A2->p : nullptr; t.B2 = B2->p; t.lda2 = (int32_t)A2->ld; t.ldb2 = (int32_t)B2->ld;
      t.ta2 = ta2; t.tb2 = tb2; t.k2 = (int32_t)k2; t.a2 = 1.0;
    } else {
      t.lda2 = t.ldb2 = 1;
    }
    t.C = C.p; t.ldc = (int32_t)C.ld; t.m = (int32_t)C.rows; t.n = (int32_t)C.cols;
    mm.push_back(t);
  }
  // a copy-family task (cmode, see MmTask); COPY and AXPY are split in column slices
  void copy_task(const Blk& C, const Blk& A, int ta, int cmode, double a, double beta) {
    if (C.rows * C.cols == 0) return;
    if ((cmode == MM_COPY || cmode == MM_AXPY) && C.rows > kRowSlice && C.rows * C.cols > kSlice * 64) {
      for (int64_t i0 = 0; i0 < C.rows; i0 += kRowSlice) {
        const int64_t nr = std::min(kRowSlice, C.rows - i0);
        Blk Ci = C; Ci.p = C.at(i0, 0); Ci.rows = nr;
        copy_task(Ci, rows_of(A, ta, i0, nr), ta, cmode, a, beta);
      }
      return;
    }
    if ((cmode == MM_COPY || cmode == MM_AXPY) && C.cols > kSlice && C.rows * C.cols > kSlice * 64) {
      for (int64_t j0 = 0; j0 < C.cols; j0 += kSlice) {
        const int64_t nc = std::min(kSlice, C.cols - j0);
        Blk Cj = C; Cj.p = C.at(0, j0); Cj.cols = nc;
        copy_task(Cj, cols_of(A, ta, j0, nc), ta, cmode, a, beta);
      }
      return;
    }
    if (rg) {
      chk(C, C.rows, C.cols);
      if (A.p) chk(A, ta ? C.cols : C.rows, ta ? C.rows : C.cols);
    }
    MmTask t{};
    t.A1 = A.p; t.lda1 = (int32_t)std::max<int64_t>(A.ld, 1); t.ta1 = ta; t.k1 = -1; t.ldb1 = t.lda2 = t.ldb2 = 1;
    t.C = C.p; t.ldc = (int32_t)C.ld; t.m = (int32_t)C.rows; t.n = (int32_t)C.cols;
    t.cmode = cmode; t.a1 = a; t.beta = beta;
    mm.push_back(t);
  }
  // C = A (or A^T)
  void copy(const Blk& C, const Blk& A, int ta = 0) { copy_task(C, A, ta, MM_COPY, 0.0, 0.0); }
  // C = a op(A) + beta C
  void axpy(const Blk& C, const Blk& A, double a, double beta, int ta = 0) { copy_task(C, A, ta, MM_AXPY, a, beta); }
  // C = the lower triangle of A (zeros above the diagonal)
  void tril(const Blk& C, const Blk& A) { copy_task(C, A, 0, MM_TRIL, 0.0, 0.0); }
  // C = I
  void eye(const Blk& C) { copy_task(C, Blk{}, 0, MM_EYE, 0.0, 0.0); }
  void zero(const Blk& C) { copy_task(C, Blk{}, 0, MM_COPY, 0.0, 0.0); }
  cudaError_t run_mm() {
    if (mm.empty()) return cudaSuccess;
    auto* d = (MmTask*)ar.raw(mm.size() * sizeof(MmTask));
    if (!d) return ar.err;
    cudaError_t e = cudaMemcpyAsync(d, mm.data(), mm.size() * sizeof(MmTask), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) launch_mm_list(d, (int64_t)mm.size(), st);
    count_launches(1);
    mm.clear();
    return e == cudaSuccess ? cudaGetLastError() : e;
  }
  // pivoted QRs of the listed blocks (factored in place); returns their ranks
  // one launch of pivoted QRs; with `rk`, the ranks are read back (synchronises st)
  cudaError_t launch_qr_list(std::vector<PqrTask>& list, std::vector<int32_t>* rk) {
    if (rk) rk->assign(list.size(), 0);
    if (list.empty()) return cudaSuccess;
    int qm = 1, km = 1;
    for (const PqrTask& t : list) {
      qm = std::max(qm, (int)t.q);
      km = std::max(km, (int)std::min(t.p, t.q));
    }
    auto* dr = (int32_t*)ar.raw(list.size() * sizeof(int32_t));
    auto* d = (PqrTask*)ar.raw(list.size() * sizeof(PqrTask));
    if (!d || !dr) return ar.err;
    for (size_t i = 0; i < list.size(); ++i) list[i].rank = dr + i;
    cudaError_t e = cudaMemcpyAsync(d, list.data(), list.size() * sizeof(PqrTask), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) launch_pqr(d, (int64_t)list.size(), qm, km, st);
    count_launches(1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (rk) {
      if (e == cudaSuccess) e = cudaMemcpyAsync(rk->data(), dr, list.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    } else if (e == cudaSuccess) {
      // the host copy of the task list must outlive the asynchronous upload
      e = cudaStreamSynchronize(st);
    }
    return e;
  }
  static bool tall_block(int64_t p, int64_t q) { return p >= 1024 && p >= 4 * q; }
  // Runs the queued QRs.  A tall block (p >= 1024 rows, p >= 4 q) is factored
  // as a tall-skinny QR: its row chunks (4 q rows, at least 256) by
  // unpivoted-rank QRs in parallel, their R factors stacked, and the stack
  // reduced the same way while it is tall; the last stack is factored with the
  // task's own tolerances (the column pivoting and the rank decision of the
  // block: the stacked R's keep its singular values), and Q is assembled back
  // down the levels, Q_l = diag(Q_chunk) Q_{l+1}, by products.  A block-per-task
  // QR of a tall block runs at one SM's FP64 rate; this spreads it over the grid.
  cudaError_t run_qr(std::vector<int32_t>& ranks) {
    ranks.assign(qr.size(), 0);
    if (qr.empty()) return cudaSuccess;
    struct Lev { Blk G, Qc, Rst; int64_t ch, nch; };   // one reduction level of a tall task
    struct Tall { size_t idx; std::vector<Lev> lev; Blk Qf; };
    std::vector<Tall> tall;
    std::vector<PqrTask> s1;
    std::vector<int64_t> s1_owner;
    for (size_t i = 0; i < qr.size(); ++i) {
      const PqrTask& t = qr[i];
      if (tall_block(t.p, t.q)) {
        Tall tl;
        tl.idx = i;
        Blk G;
        G.p = t.G; G.ld = t.ldg; G.rows = t.p; G.cols = t.q;
        while (tall_block(G.rows, G.cols)) {
          Lev L;
          L.G = G;
          L.ch = std::max<int64_t>(256, 4 * G.cols);
          L.nch = (G.rows + L.ch - 1) / L.ch;
          L.Qc = ar.blk(G.rows, G.cols);
          L.Rst = ar.blk(L.nch * G.cols, G.cols);
          if (!L.Qc.p || !L.Rst.p) return ar.err;
          zero(L.Qc);    // columns of chunks of lower rank stay zero
          zero(L.Rst);   // and so do the matching rows of their R
          tl.lev.push_back(L);
          G = L.Rst;
        }
        tall.push_back(tl);
      } else {
        s1.push_back(t);
        s1_owner.push_back((int64_t)i);
      }
    }
    cudaError_t e = run_mm();
    if (e != cudaSuccess) return e;
    // the small tasks, with every tall task's first level
    std::vector<int32_t> rk;
    auto chunk_tasks = [&](const Lev& L, std::vector<PqrTask>& out) {
      for (int64_t c = 0; c < L.nch; ++c) {
        PqrTask u{};
        u.G = L.G.p + c * L.ch;
        u.ldg = L.G.ld;
        u.p = (int32_t)std::min<int64_t>(L.ch, L.G.rows - c * L.ch);
        u.q = (int32_t)L.G.cols;
        u.Q = L.Qc.p + c * L.ch;
        u.ldq = L.Qc.ld;
        u.R = L.Rst.p + c * L.G.cols;
        u.ldr = L.Rst.ld;
        u.atol = 0.0;
        u.rtol = 0.0;
        out.push_back(u);
      }
    };
    for (const Tall& tl : tall) chunk_tasks(tl.lev[0], s1);
    if ((e = launch_qr_list(s1, s1_owner.empty() ? nullptr : &rk)) != cudaSuccess) return e;
    for (size_t j = 0; j < s1_owner.size(); ++j) ranks[(size_t)s1_owner[j]] = rk[j];
    if (tall.empty()) {
      qr.clear();
      qmax = kmax = 1;
      return cudaSuccess;
    }
    // the further reduction levels, all tall tasks together
    size_t maxlev = 0;
    for (const Tall& tl : tall) maxlev = std::max(maxlev, tl.lev.size());
    for (size_t l = 1; l < maxlev; ++l) {
      std::vector<PqrTask> sl;
      for (const Tall& tl : tall)
        if (l < tl.lev.size()) chunk_tasks(tl.lev[l], sl);
      if ((e = launch_qr_list(sl, nullptr)) != cudaSuccess) return e;
    }
    // the last stacks, with the tasks' tolerances
    std::vector<PqrTask> s2;
    for (Tall& tl : tall) {
      const PqrTask& t = qr[tl.idx];
      const Blk& last = tl.lev.back().Rst;
      tl.Qf = ar.blk(last.rows, last.cols);
      if (!tl.Qf.p) return ar.err;
      PqrTask u{};
      u.G = last.p;
      u.ldg = last.ld;
      u.p = (int32_t)last.rows;
      u.q = (int32_t)last.cols;
      u.Q = tl.Qf.p;
      u.ldq = tl.Qf.ld;
      u.R = t.R;
      u.ldr = t.ldr;
      u.atol = t.atol;
      u.rtol = t.rtol;
      s2.push_back(u);
    }
    if ((e = launch_qr_list(s2, &rk)) != cudaSuccess) return e;
    // Q back down the levels: Q_l = diag(chunk Q of level l) Q_{l+1} (r columns)
    for (size_t j = 0; j < tall.size(); ++j) ranks[tall[j].idx] = rk[j];
    for (size_t l = maxlev; l-- > 0;) {
      for (size_t j = 0; j < tall.size(); ++j) {
        Tall& tl = tall[j];
        if (l >= tl.lev.size()) continue;
        const PqrTask& t = qr[tl.idx];
        const int32_t r = rk[j];
        const Lev& L = tl.lev[l];
        const Blk Qn = tl.Qf;   // Q of the level above (rows = L.nch * q), r columns used
        Blk Out;
        if (l == 0) {
          Out.p = t.Q; Out.ld = t.ldq;
        } else {
          Out = ar.blk(L.G.rows, L.G.cols);
          if (!Out.p) return ar.err;
        }
        Out.rows = L.G.rows;
        Out.cols = r;
        for (int64_t c = 0; c < L.nch; ++c) {
          const int64_t rows = std::min<int64_t>(L.ch, L.G.rows - c * L.ch);
          Blk Cq = Out;
          Cq.p = Out.p + c * L.ch;
          Cq.rows = rows;
          Blk A = L.Qc;
          A.p = L.Qc.p + c * L.ch;
          A.rows = rows;
          A.cols = L.G.cols;
          Blk Bq = Qn;
          Bq.p = Qn.p + c * L.G.cols;
          Bq.rows = L.G.cols;
          Bq.cols = r;
          gemm(Cq, A, 0, Bq, 0);
        }
        tl.Qf = Out;
      }
      if ((e = run_mm()) != cudaSuccess) return e;
    }
    qr.clear();
    qmax = kmax = 1;
    return cudaSuccess;
  }
  // queue the QR of a copy of G: returns (Q, R) blocks sized for the full rank
  std::pair<Blk, Blk> pqr(const Blk& G, double atol, double rtol) {
    const int64_t km = std::min(G.rows, G.cols);
    Blk Q = ar.blk(G.rows, km), R = ar.blk(km, G.cols);
    PqrTask t{};
    t.G = G.p; t.ldg = G.ld; t.p = (int32_t)G.rows; t.q = (int32_t)G.cols;
    t.Q = Q.p; t.ldq = Q.ld; t.R = R.p; t.ldr = R.ld; t.atol = atol; t.rtol = rtol;
    if (G.rows * G.cols > 0) {
      qr.push_back(t);
      qmax = std::max<int>(qmax, (int)G.cols);
      kmax = std::max<int>(kmax, (int)km);
    }
    return {Q, R};
  }
};


// Splits products and plain copies wider than `slice` columns into column
// slices (one task each), so that a wide block spreads over many thread blocks.
inline void split_mm_columns(std::vector<MmTask>& v, int64_t slice = Stages::kSlice) {
  std::vector<MmTask> out;
  out.reserve(v.size());
  for (const MmTask& t : v) {
    const bool sliceable = t.n > slice && (t.k1 >= 0 || t.cmode == MM_COPY || t.cmode == MM_AXPY);
    if (!sliceable) {
      out.push_back(t);
      continue;
    }
    for (int64_t j0 = 0; j0 < t.n; j0 += slice) {
      MmTask u = t;
      u.n = (int32_t)std::min<int64_t>(slice, t.n - j0);
      u.C = t.C + j0 * (int64_t)t.ldc;
      if (t.k1 >= 0) {
        if (t.B1) u.B1 = t.tb1 ? t.B1 + j0 : t.B1 + j0 * (int64_t)t.ldb1;
        if (t.B2) u.B2 = t.tb2 ? t.B2 + j0 : t.B2 + j0 * (int64_t)t.ldb2;
      } else if (t.A1) {
        u.A1 = t.ta1 ? t.A1 + j0 : t.A1 + j0 * (int64_t)t.lda1;
      }
      out.push_back(u);
    }
  }
  v.swap(out);
}

// orthonormalize_generators! and (unless ortho_only) recompress! of a
// single-tree handle into a new handle with the same node numbering.
int recompress_impl(hss_plan_s* h, double atol, double rtol, bool ortho_only, hss_plan_s** out, cudaStream_t st);

}  // namespace hss
