// Registry of the compile-time specialised cascade variants.
#include <mutex>
#include <vector>

#include "ct_cascade.cuh"

namespace kym {

static std::vector<CtEntry>& ct_table() {
  static std::vector<CtEntry> t;
  return t;
}
static std::mutex& ct_mutex() {
  static std::mutex m;
  return m;
}

void ct_register(const CtEntry& e) {
  std::lock_guard<std::mutex> lock(ct_mutex());
  ct_table().push_back(e);
}

const CtEntry* ct_find(int mr, int mc, int sr, int sc, int c, bool oned, int kf) {
  std::lock_guard<std::mutex> lock(ct_mutex());
  const CtEntry* generic = nullptr;
  for (const CtEntry& e : ct_table()) {
    if (e.mr != mr || e.mc != mc || e.sr != sr || e.sc != sc || e.c != c || e.oned != oned) continue;
    if (e.kf == kf) return &e;
    if (e.kf < 0) generic = &e;
  }
  return generic;
}

}  // namespace kym
