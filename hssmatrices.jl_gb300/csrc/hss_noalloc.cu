// An HSS x dense product entry point that allocates no memory.
//
// Callers that must not allocate device memory during a call -- code running
// inside a host callback or a driver-managed memory pool, hard real-time
// loops that pre-allocate everything up front, or runtimes that forbid
// cudaMalloc after start-up -- cannot use hss_matmul, whose workspace for
// the upsweep/downsweep vectors (Z, F) and whose slot table grow on demand.
// hss_matmul_noalloc runs the same kernels with that scratch in file-scope
// __device__ arrays of fixed size instead.
//
// Limits and behaviour:
//   * the workspace holds at most kNoAllocWsDoubles doubles (workspace rows
//     of the tree times the number of right-hand sides); larger calls are
//     rejected with HSS_ERR_BAD_DIMS before anything is launched;
//   * the arrays exist once per device for the life of the process and are
//     shared by every call: two calls whose work overlaps on the GPU (e.g. on
//     different streams) race on them; calls on one stream are ordered;
//   * nothing in the scratch needs clearing: every workspace entry is written
//     before it is read within a call;
//   * the argument slot is written on the caller's stream by a one-thread
//     kernel that takes it by value, so nothing is staged in host memory;
//   * the first call on a device looks up the arrays' device addresses
//     (cudaGetSymbolAddress); make that first call before capturing a stream.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "hssgpu.h"
#include "hss_internal.h"
#include "hss_launch.h"

namespace hss {

namespace {

constexpr int64_t kNoAllocWsDoubles = 1 << 20;   // 8 MiB of workspace
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_noalloc_ws[kNoAllocWsDoubles];
__device__ __align__(256) Slot g_noalloc_slot[1];

struct DevScratch {
  bool ready = false;
  double* ws = nullptr;
  Slot* slot = nullptr;
};
DevScratch g_scratch[kMaxDevices];
std::mutex g_scratch_mu;

}  // namespace

// Per-device set-up: the host-side names of the __device__ arrays are not
// device addresses, so they are resolved once per device with the device current.
int noalloc_scratch(int device, double** ws, Slot** slot, std::string* err) {
  if (device < 0 || device >= kMaxDevices) {
    *err = "device index out of range for the allocation-free product";
    return HSS_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  DevScratch& d = g_scratch[device];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_ws);
    if (e != cudaSuccess) {
      *err = std::string("cudaGetSymbolAddress(workspace): ") + cudaGetErrorString(e);
      return HSS_ERR_CUDA;
    }
    d.ws = (double*)p;
    e = cudaGetSymbolAddress(&p, g_noalloc_slot);
    if (e != cudaSuccess) {
      *err = std::string("cudaGetSymbolAddress(slot): ") + cudaGetErrorString(e);
      return HSS_ERR_CUDA;
    }
    d.slot = (Slot*)p;
    d.ready = true;
  }
  *ws = d.ws;
  *slot = d.slot;
  return HSS_OK;
}

int64_t noalloc_ws_capacity() { return kNoAllocWsDoubles; }

namespace {
// The argument slot travels as a kernel parameter, which the launch copies;
// the host object may go out of scope as soon as the launch returns.
__global__ void noalloc_slot_kernel(Slot* dst, Slot x) { *dst = x; }
}  // namespace

cudaError_t noalloc_write_slot(Slot* dslot, const Slot& x, cudaStream_t st) {
  noalloc_slot_kernel<<<1, 1, 0, st>>>(dslot, x);
  return cudaGetLastError();
}

}  // namespace hss
