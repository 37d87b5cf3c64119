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

// ---- line-split variants (lines.cuh) ----------------------------------------
#include "lines.cuh"

namespace kym {

namespace {
struct LinesEntry {
  int mr, mc, sr, sc, kf;
  LinesLauncher fn;
};
std::vector<LinesEntry>& lines_table() {
  static std::vector<LinesEntry> t;
  return t;
}
}  // namespace

void lines_register(int mr, int mc, int sr, int sc, int kf, LinesLauncher fn) {
  std::lock_guard<std::mutex> lock(ct_mutex());
  lines_table().push_back(LinesEntry{mr, mc, sr, sc, kf, fn});
}

LinesLauncher lines_find(int mr, int mc, int sr, int sc, int kf) {
  std::lock_guard<std::mutex> lock(ct_mutex());
  LinesLauncher generic = nullptr;
  for (const LinesEntry& e : lines_table()) {
    if (e.mr != mr || e.mc != mc || e.sr != sr || e.sc != sc) continue;
    if (e.kf == kf) return e.fn;
    if (e.kf < 0) generic = e.fn;
  }
  return generic;
}

}  // namespace kym
