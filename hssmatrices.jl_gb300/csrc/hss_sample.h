// Device structures and launchers of the randomized-compression pass
// (hss_sample.cu), used by hss_compress.cpp.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace hss {

// One node of the cluster-tree pair.  Side 0 is the column sample (A * Omega:
// row basis U, selected rows), side 1 the row sample (A^T * Omega: column
// basis V, selected columns).  Slot pointers are fixed per capacity s.
struct RcNode {
  int32_t left, right, leaf, root;
  int64_t r0, m, c0, n;     // row range [r0, r0+m), column range [c0, c0+n)
  double* S[2];             // assembled sample (p x s); leaves: inside the corrected sample copies
  int64_t lds[2];           // leaves: leading dimension of S (branches use p)
  double* Sr[2];            // reduced sample S[J, :] (rank x s, ld s)
  double* Or[2];            // reduced test matrix X * Omega_in (rank x s, ld s)
  int64_t* J[2];            // selected global row (side 0) / column (side 1) indices
  double* G[2];             // generator X^T (p x rank, ld p): U, V or [R1; R2], [W1; W2]
  double* B12;              // A[Jc(left), Jr(right)] (kc1 x kr2, ld kc1)
  double* B21;              // A[Jc(right), Jr(left)] (kc2 x kr1, ld kc2)
};

struct RcArgs {
  const RcNode* nodes;
  const int32_t* list;      // node indices of this launch (one tree level)
  int32_t* rank;            // 2 per node: column-side and row-side rank
  const double* A;
  int64_t lda;
  const double* Ocol;       // n x s
  int64_t ldoc;
  const double* Orow;       // m x s
  int64_t ldor;
  int64_t s;
  double atol, rtol;
  int64_t pmax;             // largest sample height p of the launch
  int32_t m_in_smem;        // 1: the QR works in shared memory; 0: in gscratch
  double* gscratch;         // (s | 1) * pmax doubles per block when m_in_smem == 0
};

// Block copy for packing generators: dst (rows x cols, ld rows) = src (ld lds).
struct CopyTask {
  const double* src;
  int64_t lds;
  double* dst;
  int64_t rows, cols;
};

// Number of K splits of an m x r sample product over k for `sms` SMs (df:
// the double-float kernel's tiles).
int sample_ksplit(int64_t m, int64_t k, int64_t r, int sms, bool df);
// Y = alpha * op(A) * X + beta * Y with op(A) (m x k); trans = 1 reads A as
// k x m.  With nsplit > 1, `partial` holds nsplit * m * r doubles.  df: the
// products in double-float arithmetic on the FP32 pipe (~2^-47 per operation;
// entries of A and X within float's exponent range); with lrow (m leaf
// indices of op(A)'s rows) and lin (k, of its inner index) the entries of the
// diagonal leaf blocks are left out (df only).
void launch_sample_gemm(const double* A, int64_t lda, int64_t m, int64_t k, int trans, const double* X,
                        int64_t ldx, int64_t r, double* Y, int64_t ldy, double alpha, double beta, int nsplit,
                        double* partial, bool df, const int32_t* lrow, const int32_t* lin, cudaStream_t st);
// HSS_OPT_SAMPLE_DF: hss_sample computes in double-float (default: FP64).
extern bool g_sample_df;
// Diagonal-block products of the leaves (see hss_sample.cu).
void launch_blockdiag_gemm(int32_t count, int64_t max_dim, const double* A, int64_t lda, const int64_t* row0,
                           const int64_t* rows, const int64_t* col0, const int64_t* cols, int trans,
                           const double* X, int64_t ldx, int64_t r, double* Y, int64_t ldy, double alpha,
                           double beta, cudaStream_t st);
size_t rc_id_smem(int64_t s, int64_t pmax, bool m_in_smem);
int64_t rc_id_scratch(int64_t s, int64_t pmax);
cudaError_t launch_rc_id(const RcArgs& a, int32_t count, cudaStream_t st);
void launch_copy_blocks(const CopyTask* tasks, int64_t count, cudaStream_t st);

}  // namespace hss
