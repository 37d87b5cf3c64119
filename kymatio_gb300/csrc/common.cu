// Library-wide C ABI helpers: version string and the last CUDA error text.
#include <cuda_runtime.h>

#include "../../include/kymatio_gb300.h"

extern "C" const char* kym_version(void) { return "0.1.0"; }

extern "C" const char* kym_last_error(void) {
  // peek, not get: the sticky state of the context is left as it is
  return cudaGetErrorString(cudaPeekAtLastError());
}
