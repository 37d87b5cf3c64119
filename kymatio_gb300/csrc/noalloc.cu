// Allocation-free variant of the 2-D forward (kym_s2d_forward_noalloc).
//
// Some callers cannot allocate device memory: code that runs inside a
// fixed memory pool or under an allocator they do not own (a real-time
// pipeline that reserved its memory up front, a plugin of a host that forbids
// allocation after start-up, a process that must not touch the CUDA
// allocator while another library holds it).  This entry point takes only
// the input, output and filters from the caller; its workspace -- the plan's
// task/twiddle tables and the per-chunk input and parent spectra -- lives in
// the file-scope device array below, which every GPU that loads the library
// holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/kymatio_gb300.h"
#include "cascade.cuh"
#include "errors.h"

struct kym_s2d_plan;

namespace kym {
struct CascadePlan;
CascadePlan* plan_of(const kym_s2d_plan* p);
int run_plan_in_scratch(CascadePlan* P, const float* x, float* out, int batch, const float* const* filters,
                        int nfilters, void* scratch, size_t scratch_bytes, cudaStream_t stream);
}  // namespace kym

namespace {

// 32 MiB per device (KYM_NOALLOC_SCRATCH_BYTES in the header).
constexpr size_t kScratchBytes = KYM_NOALLOC_SCRATCH_BYTES;
__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is taken
// with cudaGetSymbolAddress once per device, with that device current.
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    kym::set_error_message("forward_noalloc", cudaGetErrorString(e));
    return KYM_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    kym::set_error_message("forward_noalloc", "device ordinal out of range");
    return KYM_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      kym::set_error_message("forward_noalloc: cudaGetSymbolAddress", cudaGetErrorString(e));
      return KYM_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return KYM_OK;
}

}  // namespace

extern "C" int kym_s2d_forward_noalloc(const kym_s2d_plan* plan, const float* x, float* out, int batch,
                                       const float* const* filters, int n_filters, void* stream) {
  if (!plan) {
    kym::set_error_message("forward_noalloc", "null plan");
    return KYM_ERR_INVALID;
  }
  void* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  return kym::run_plan_in_scratch(kym::plan_of(plan), x, out, batch, filters, n_filters, scratch, kScratchBytes,
                                  static_cast<cudaStream_t>(stream));
}
