// Registry of the tensor-core cascade variants.
#include <mutex>
#include <vector>

#include "tcdft.cuh"

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

namespace kym {
namespace {
struct TcEntryList {
  std::vector<TcEntry> v;
  std::mutex mu;
};
TcEntryList& dft_table() {
  static TcEntryList t;
  return t;
}
}  // namespace

void tcdft_register(int mr, int mc, int nr, int nc, int kf, size_t smem, TcLauncher fn) {
  TcEntryList& t = dft_table();
  std::lock_guard<std::mutex> lock(t.mu);
  t.v.push_back(TcEntry{mr, mc, nr, nc, kf, smem, fn});
}

bool tcdft_find(int mr, int mc, int nr, int nc, int kf, size_t* smem, TcLauncher* fn) {
  TcEntryList& t = dft_table();
  std::lock_guard<std::mutex> lock(t.mu);
  for (const TcEntry& e : t.v)
    if (e.mr == mr && e.mc == mc && e.nr == nr && e.nc == nc && e.kf == kf) {
      *smem = e.smem;
      *fn = e.fn;
      return true;
    }
  return false;
}

}  // namespace kym
