// rk4_static.cu -- classical RK4 step whose work vectors live in a fixed,
// file-scope device array, for callers that cannot allocate device memory.
//
// Who cannot allocate: host code that advances the solution from inside a
// region where cudaMalloc is not allowed or not wanted -- a stream being
// captured into a CUDA graph in global capture mode (cudaMalloc is illegal
// there), a real-time time loop that must not stall on the allocator, or a
// plugin embedded in a host application whose device memory is owned and
// budgeted by the host application.  Such callers can still pass the state
// vector they already own; dgc_rk4_step_static needs nothing else.
//
// The scratch array is sized for three work vectors of at most
// kStaticVectorBytes each and is held by every GPU that loads this library
// until the process exits.  Calls share it: two calls whose GPU work
// overlaps (different streams, or different handles on the same device at
// the same time) race on it.  The RK4 stage kernels write every work entry
// they later read, so the array needs no clearing between calls.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "dgc_gb300.h"
#include "dgc_internal.hpp"

namespace {

constexpr size_t kStaticVectorBytes = size_t(2) << 20;  // 2 MiB per work vector
constexpr size_t kStaticBytes = 3 * kStaticVectorBytes;  // 6 MiB in total

static __device__ __align__(256) unsigned char g_rk4_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

}  // namespace

extern "C" int dgc_rk4_step_static(dgc_handle h, void* q, double t, double dt, void* stream) {
  if (!h || !q) return dgc::set_error(DGC_ERR_ARG, "null argument");
  const size_t bytes = (size_t)h->K * h->Nf * h->NpP * (h->prec == DGC_F64 ? 8 : 4);
  if (bytes > kStaticVectorBytes)
    return dgc::set_error(DGC_ERR_ARG,
                          "state vector exceeds the 2 MiB per-vector limit of dgc_rk4_step_static; "
                          "use dgc_rk4_step with caller-provided work vectors");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return dgc::set_error(DGC_ERR_CUDA, "dgc_rk4_step_static: no usable current device");
  // the array is looked up per device; a handle's kernels run on its own device
  if (dev != h->device)
    return dgc::set_error(DGC_ERR_ARG, "dgc_rk4_step_static: the handle's device is not the current device");
  void* base = nullptr;
  {
    // one-time set-up per device, with that device current: the host-side name
    // of a __device__ array is not a device address, so look the address up
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_rk4_scratch);
      if (e != cudaSuccess || !p) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "cudaGetSymbolAddress for the RK4 scratch array failed: %s",
                      cudaGetErrorString(e));
        return dgc::set_error(DGC_ERR_CUDA, msg);
      }
      g_scratch_ptr[dev] = p;
    }
    base = g_scratch_ptr[dev];
  }
  unsigned char* b = static_cast<unsigned char*>(base);
  void* work[3] = {b, b + kStaticVectorBytes, b + 2 * kStaticVectorBytes};
  return dgc_rk4_step(h, q, t, dt, work, stream);
}
