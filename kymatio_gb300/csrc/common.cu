// Library-wide C ABI helpers: version string and the last error text.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "../../include/kymatio_gb300.h"
#include "errors.h"

namespace kym {
static thread_local std::string g_last_error;

void set_error_message(const char* where, const char* what) {
  g_last_error = std::string(where) + ": " + what;
}
void clear_error_message() { g_last_error.clear(); }
}  // namespace kym

extern "C" const char* kym_version(void) { return "0.1.0"; }

extern "C" const char* kym_last_error(void) {
  if (!kym::g_last_error.empty()) return kym::g_last_error.c_str();
  // peek, not get: the sticky state of the context is left as it is
  return cudaGetErrorString(cudaPeekAtLastError());
}
