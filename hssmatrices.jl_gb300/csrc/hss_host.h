// Host-side helpers shared by the C-ABI translation units (hss_capi.cpp,
// hss_compress.cpp): device/pinned buffers, error reporting, and plan
// construction for generators that are written on the device.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

struct hss_plan_s;
struct hss_factor_s;

namespace hss {

// Every device allocation of the library goes through here: cudaMalloc, or,
// while a failure is armed (hss_set_option(HSS_OPT_FAIL_ALLOC, k)), the k-th
// call from then on returns cudaErrorMemoryAllocation without reaching the driver.
cudaError_t dev_alloc(void** p, size_t bytes);
// The same from the device's stream-ordered pool on st (freed with cudaFreeAsync).
cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t st);

// Grow-only device buffer.
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t cap = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  cudaError_t ensure(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    release();
    size_t want = std::max<size_t>(n, 1);
    cudaError_t e = dev_alloc((void**)&p, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    else p = nullptr;
    return e;
  }
};

// Pinned host buffer.
template <typename T>
struct HBuf {
  T* p = nullptr;
  size_t cap = 0;
  HBuf() = default;
  HBuf(const HBuf&) = delete;
  HBuf& operator=(const HBuf&) = delete;
  ~HBuf() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t ensure(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMallocHost((void**)&p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) cap = std::max<size_t>(n, 1);
    return e;
  }
};

// Thread-local error message of hss_last_error(); both return `code`.
int set_error(int code, const std::string& msg);
int set_cuda_error(cudaError_t e, const char* what);
// Adds to the kernel-launch counter of hss_launch_counter().
void count_launches(int64_t n);
// Builds the plan of one tree (node table as for hss_create) with an
// uninitialised generator buffer of npacked doubles that the caller fills on
// the device; *d_gen receives its address.
int plan_create_device(int64_t nnodes, const int64_t* table, int64_t npacked, hss_plan_s** out, double** d_gen);
void plan_destroy(hss_plan_s* p);
// A plan's host copy of its node descriptors (device pointers inside), the
// device copy, and its device, tree count and the first tree's size.
struct Node;
const std::vector<Node>& plan_nodes(const hss_plan_s* p);
const Node* plan_device_nodes(const hss_plan_s* p);
int plan_device(const hss_plan_s* p);
int32_t plan_ntrees(const hss_plan_s* p);
int64_t plan_rows(const hss_plan_s* p);
int64_t plan_cols(const hss_plan_s* p);
// The adjoint of a single-tree plan as a new plan (same node numbering);
// synchronises st.
int plan_transpose(const hss_plan_s* h, hss_plan_s** out, cudaStream_t st);
// A factorization's device storage (elements of its precision) and its size in bytes.
const void* factor_storage(const hss_factor_s* f);
size_t factor_storage_bytes(const hss_factor_s* f);
// A plan's generator buffer and its length (doubles).
const double* plan_gen(const hss_plan_s* p, int64_t* len);

}  // namespace hss
