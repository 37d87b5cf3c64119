// Registry of the tensor-core cascade variants.
#include <mutex>
#include <vector>

#include "tc_cascade.cuh"

namespace kym {
namespace {
struct TcEntry {
  int mr, mc, nr, nc, kf;
  size_t smem;
  TcLauncher fn;
};
std::vector<TcEntry>& table() {
  static std::vector<TcEntry> t;
  return t;
}
std::mutex& mu() {
  static std::mutex m;
  return m;
}
}  // namespace

void tc_register(int mr, int mc, int nr, int nc, int kf, size_t smem, TcLauncher fn) {
  std::lock_guard<std::mutex> lock(mu());
  table().push_back(TcEntry{mr, mc, nr, nc, kf, smem, fn});
}

bool tc_find(int mr, int mc, int nr, int nc, int kf, size_t* smem, TcLauncher* fn) {
  std::lock_guard<std::mutex> lock(mu());
  for (const TcEntry& e : table())
    if (e.mr == mr && e.mc == mc && e.nr == nr && e.nc == nc && e.kf == kf) {
      *smem = e.smem;
      *fn = e.fn;
      return true;
    }
  return false;
}

}  // namespace kym
