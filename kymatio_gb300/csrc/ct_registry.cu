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

const CtEntry* ct_find(int mr, int mc, int sr, int sc, int c, bool oned) {
  std::lock_guard<std::mutex> lock(ct_mutex());
  for (const CtEntry& e : ct_table())
    if (e.mr == mr && e.mc == mc && e.sr == sr && e.sc == sc && e.c == c && e.oned == oned) return &e;
  return nullptr;
}

}  // namespace kym
