// Kernel launch wrappers (implemented in hss_kernels.cu, used by hss_capi.cpp).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "hss_internal.h"

namespace hss {

// HSS x dense product (reference src/matmul.jl:18-62), one launch per list.
void launch_mv_leaf(const Task* t, int64_t ntasks, const Slot* s, int rmax, cudaStream_t st);
void launch_mv_up(const Task* t, int64_t ntasks, const Slot* s, cudaStream_t st);
void launch_mv_down(const Task* t, int64_t ntasks, const Slot* s, cudaStream_t st);
void launch_mv_leaf_final(const Task* t, int64_t ntasks, const Slot* s, int rmax, cudaStream_t st);
// Shared-memory staged translator sweeps; smem from the *_smem helpers with the
// level's largest ranks (children's and the node's own).
size_t mv_up_staged_smem(int kv, int k1max, int k2max);
size_t mv_down_staged_smem(int ku, int u1, int u2, int v1, int v2);
void launch_mv_up_staged(const Task* t, int64_t ntasks, const Slot* s, size_t smem, int rmax, cudaStream_t st);
void launch_mv_down_staged(const Task* t, int64_t ntasks, const Slot* s, size_t smem, int rmax, cudaStream_t st);

// Double-float (FP32 pair) product for the refinement residual (hss_matvec_df.cu).
void launch_df_split(const double* src, float2* dst, int64_t cnt, cudaStream_t st);
void launch_df_split_cols(const double* X, int64_t ldx, int64_t n, int64_t r, float2* Xs, cudaStream_t st);
void launch_dfmv_leaf(const Task* t, int64_t ntasks, const Slot* s, int rmax, cudaStream_t st);
void launch_dfmv_up(const Task* t, int64_t ntasks, const Slot* s, int rmax, cudaStream_t st);
void launch_dfmv_down(const Task* t, int64_t ntasks, const Slot* s, int rmax, cudaStream_t st);
void launch_dfmv_final(const Task* t, int64_t ntasks, const Slot* s, int rmax, cudaStream_t st);

// Persistent product (hss_pmv.cu): the whole product of a forest in one
// cooperative launch, FP64 (pairs = false) or double-float (pairs = true).
// Shared-memory elements for leaves of <= nleaf columns and ranks <= kmax;
// *mcap gets the part available for staged translators.
size_t pmv_smem_elems(int nleaf, int kmax, int* mcap);
bool pmv_fits(int nleaf, int mleaf, int kmax);
// Column chunks of a product with rmax right-hand sides (0: too many for the
// persistent product).  Tasks are (node, chunk) pairs: a launch over ntasks
// non-root nodes, ninner of them branches, has (ntasks + ninner) * chunks
// queue entries (downsweep / final tasks and B-term tasks).
int pmv_chunks(bool pairs, int rmax);
int64_t pmv_queue_entries(int64_t ntasks, int64_t ninner, int chunks);
// 32-bit words of launch state (the caller zeroes them once; the kernel leaves
// them zero).  Queue entries are separate 64-bit words, zeroed when allocated;
// each carries the epoch of the launch that wrote it, so epochs must grow from
// 1 and stay <= pmv_epoch_limit() (then: zero the entries and start again).
int64_t pmv_state_words();
uint32_t pmv_epoch_limit();
// Queue entries hold node indices below 2^20 and slot indices below 2^16.
bool pmv_queue_fits(int64_t nodes, int64_t slots);
// Per-node counters: a plan holds nodes * pmv_sync_chunks() of them, zeroed.
int pmv_sync_chunks();
// Polls of an idle or waiting block of the persistent products before it
// records DEV_TIMEOUT and gives up (0: the default, 2^22); taken by later launches.
void pmv_set_poll_limit(uint32_t polls);
uint32_t pmv_poll_limit();
// ntasks = non-root nodes of all trees, ninner = non-root branches; the slots' nodes/sync must be set and
// every sync counter even (zeroed at allocation); epoch must differ from every earlier launch on state.
// [prefetch, prefetch + prefetch_bytes) (nullable) is brought into L2 first.
cudaError_t launch_pmv(bool pairs, const Task* leaves, int64_t nleaves, const Slot* slots, int64_t ntasks,
                       int64_t ninner, int rmax,
                       int nleaf, int kmax, uint32_t* state, unsigned long long* qent, uint32_t epoch,
                       const void* prefetch, int64_t prefetch_bytes, int device, cudaStream_t st,
                       bool dx_ready = false, bool leaf_ext = false);
// The other leaf products of the double-float residual, outside the persistent
// launch (hss_pmv.cu): final_part = false: Z = V^T X of every non-root leaf
// into the pair workspace (before the launch); true: C = alpha (D X + U F) +
// beta Y with the column sums of squares (after it).  With dx_ready the
// persistent launch skips both.
bool leaf_ext_fits(int nleaf, int mleaf, int kmax);
cudaError_t launch_leaf_ext(bool final_part, const Task* leaves, int64_t nleaves, const Slot* slots, int rmax, int nleaf,
                            int mleaf, int kmax, cudaStream_t st);
// Tensor-core leaf products of the double-float residual (hss_dx_tc.cu): for
// every non-root leaf task and chunk of 32 columns, D X at ~48-bit accuracy
// into the slot's pair buffer (sl.tmp), X = the slot's B; leaves up to 128 x 128.
// A persistent pair product launched after it with dx_ready skips those products.
bool dx_tc_fits(int mleaf, int nleaf);
// Bytes of one leaf's prepared slices (n columns), and the once-per-plan
// preparation over the plan's leaf tasks (regions at each leaf's fdx in base).
int64_t dx_leaf_bytes(int n);
cudaError_t launch_dx_prep(const Task* leaves, int64_t nleaves, unsigned char* base, cudaStream_t st);
cudaError_t launch_dx_tc(const Task* leaves, int64_t nleaves, const Slot* slots, int rmax, cudaStream_t st);

// Flat persistent product (hss_pmv.cu), FP64 with few right-hand sides: every
// leaf carries its own chain of small products up to the root and back, so
// the launch has two grid barriers instead of the tree's dependency chain.
// links: one per node of the plan (roots unused); paths: for leaf position t
// of `leaves`, paths[t * dep + d] is its ancestor at depth d (1 <= d <= its
// depth), dep > every leaf depth; branches: the non-root branches.  ctb holds
// pmv_flat_ctb_elems doubles of contributions; dcnt one counter per (leaf,
// chunk), zero before the first launch (the kernel leaves them zero).  The
// state words are those of launch_pmv (zero between launches).
constexpr int kFlatDep = 32;
size_t pmv_flat_smem_elems(int nleaf, int kmax, int dep);
bool pmv_flat_fits(int nleaf, int kmax, int dep, int rmax);
int64_t pmv_flat_ctb_elems(int64_t nleaves, int dep, int kmax, int rmax);
int64_t pmv_flat_chunks(int rmax);
cudaError_t launch_pmv_flat(const Task* leaves, int64_t nleaves, const Task* branches, int64_t nbranch,
                            const FlatLink* links, const int32_t* paths, int dep, const Slot* slots, int rmax,
                            int nleaf, int mleaf, int kmax, uint32_t* state, double* ctb, uint32_t* dcnt,
                            int device, cudaStream_t st);

// Entry extraction (hss_getindex.cu): basis pass for one list of nodes (one
// tree height), the off-diagonal tiles, the diagonal leaf blocks.  R / C are
// the sorted requested rows / columns, prow / pcol their output positions.
void launch_gi_basis(const Node* nodes, const GiRange* rg, const int32_t* list, int64_t count, const int64_t* R,
                     const int64_t* C, double* ws, cudaStream_t st);
void launch_gi_blocks(const GiTile* tiles, int64_t count, const double* ws, const int64_t* prow, const int64_t* pcol,
                      double* out, int64_t ldo, cudaStream_t st);
void launch_gi_leaves(const Node* nodes, const GiRange* rg, const int32_t* leaves, int64_t count, const int64_t* R,
                      const int64_t* C, const int64_t* prow, const int64_t* pcol, double* out, int64_t ldo,
                      cudaStream_t st);
int gi_tile_rows();

// HSS x HSS product (hss_hssmul.cu): one launch runs a list of independent
// small-product / copy tasks, one block per task.
void launch_mm_list(const MmTask* tasks, int64_t count, cudaStream_t st);

// Truncated pivoted QRs (hss_recompress.cu), one block per task; qmax / kmax
// bound the tasks' q and min(p, q).
void launch_pqr(const PqrTask* tasks, int64_t count, int qmax, int kmax, cudaStream_t st);

// ULV factor / solve (reference src/ulvfactor.jl:22-107), T = double or float.
template <typename T>
void launch_ulv_factor(const Task* t, int64_t ntasks, const Slot* s, int max_m, int max_n,
                       cudaStream_t st);
// Blocked on-chip factor kernel (hss_factor_blk.cu), FP32 (two blocks per SM)
// or FP64; `extra` = merge staging elements.
template <typename T>
bool factor_blk_fits(int mmax, int nmax, int kumax, int kvmax, size_t extra);
template <typename T>
size_t factor_blk_smem(int mmax, int nmax, int kumax, int kvmax, size_t extra);
template <typename T>
void launch_ulv_factor_blk(const Task* t, int64_t ntasks, const Slot* s, int mmax, int nmax, int kumax, int kvmax,
                           size_t extra, cudaStream_t st);
// Blocked FP32 solve sweeps (hss_bsolve.cu) over factors of the blocked FP32
// reduction: sizes are the level's largest node and children's ranks.
bool bsolve_fits(int mmax, int nmax, int kmax, int kvmax);
void launch_bsolve_up(const Task* t, int64_t ntasks, const Slot* s, int mmax, int nmax, int kmax, int kvmax, int r,
                      cudaStream_t st);
void launch_bsolve_down(const Task* t, int64_t ntasks, const Slot* s, int mmax, int nmax, int kmax, int kvmax, int r,
                        cudaStream_t st);
// Register-resident solve sweeps for nodes with m, n <= 256 (hss_solve.cu).
bool solve_reg_fits(int mmax, int nmax);
template <typename T>
void launch_ulv_solve_up_reg(const Task* t, int64_t ntasks, const Slot* s, int mmax, int64_t stage, int r,
                             cudaStream_t st);
// Shared-memory elements the upward solve stages for one node.
int64_t solve_up_stage_need(int m, int k, int mk, int nk, int kv, bool leaf, bool root, int mr1, int mr2, int kv1,
                            int kv2);
template <typename T>
void launch_ulv_solve_down_reg(const Task* t, int64_t ntasks, const Slot* s, int nmax, int mkmax, int r,
                               cudaStream_t st);
template <typename T>
void launch_ulv_solve_up(const Task* t, int64_t ntasks, const Slot* s, cudaStream_t st);
template <typename T>
void launch_ulv_solve_down(const Task* t, int64_t ntasks, const Slot* s, cudaStream_t st);

// out[j] += sum_i B(i,j)^2 for i < n, j < r (out must be zeroed by the caller).
void launch_colnorm2(const double* B, int64_t ldb, int64_t n, int64_t r, double* out,
                     cudaStream_t st);
// s[j] = sqrt(n2[j]) (1 where n2[j] == 0) and s[r + j] = 1 / s[j]; s holds 2r values.
void launch_sqrt_scale(const double* n2, double* s, int64_t r, cudaStream_t st);
// The refinement loop's convergence check (one block; sets `cond`, the condition
// of the CUDA graph while node that repeats the refinement step).
void launch_refine_check(const double* bn2, const double* rn2, int64_t r, double tol, int32_t maxit,
                         RefineStatus* status, const Slot* slots, int32_t nslots, cudaGraphConditionalHandle cond,
                         cudaStream_t st);

// Fixed scratch of the allocation-free product (hss_noalloc.cu): device
// addresses of the file-scope arrays on `device`, resolved once per device.
int noalloc_scratch(int device, double** ws, Slot** slot, std::string* err);
int64_t noalloc_ws_capacity();
// Writes `x` into the device slot `dslot` on `st` with a one-thread kernel
// that takes the slot by value (no host staging buffer, no allocation).
cudaError_t noalloc_write_slot(Slot* dslot, const Slot& x, cudaStream_t st);

// Row transforms of the HSS-valued division (hss_divide.cu): one launch over
// the tasks, every task's columns in chunks of 32; rows <= div_rows_max().
int div_rows_max();
cudaError_t launch_div_rows(const DivTask* tasks, int64_t count, int maxrows, int maxcols, cudaStream_t st);

}  // namespace hss
