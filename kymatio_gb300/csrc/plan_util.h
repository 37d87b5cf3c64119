// Host helpers for the transform plans: radix schedules, FP64-built twiddle
// tables, device limits.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <vector>

#include "fft_engine.cuh"

namespace kym {

// Largest dynamic shared memory a CTA may opt into (227 KB on sm_100/103).
inline size_t max_dynamic_smem() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess && v > 0)
    return (size_t)v;
  cudaGetLastError();
  return 232448;
}

// Most butterflies per thread a stage of radix R may hold (fft_pass
// dispatch): at most 32 complex values in registers.
inline int max_items(int R) {
  switch (R) {
    case 2: return 16;
    case 4: return 8;
    case 8: return 4;
    case 16: return 2;
    default: return 1;
  }
}

// Radix schedule for length n: 16s, then 8/4/2, then odd primes ascending.
// Returns false when a stage would need more butterflies per thread than the
// engine supports for the CTA size, or a prime factor above 127.
inline bool make_fft_plan(int n, FftPlan* p, int nthreads) {
  p->n = n;
  p->nstages = 0;
  p->tw = nullptr;
  if (n < 1) return false;
  int m = n;
  std::vector<int> rs;
  while (m % 16 == 0) { rs.push_back(16); m /= 16; }
  for (int r : {8, 4, 2})
    while (m % r == 0) { rs.push_back(r); m /= r; }
  for (int f = 3; m > 1; f += 2) {
    while (m % f == 0) {
      if (f > 127) return false;
      rs.push_back(f);
      m /= f;
    }
  }
  if ((int)rs.size() > kMaxStages) return false;
  for (size_t i = 0; i < rs.size(); ++i) {
    const int R = rs[i];
    if ((n / R + nthreads - 1) / nthreads > max_items(R)) return false;
    p->radix[i] = R;
  }
  p->nstages = (int)rs.size();
  return true;
}

// exp(-2 pi i k / n) for every length a plan uses, computed in FP64 and
// rounded once to fp32.  Host copy built at plan creation, device copy
// uploaded on first use per device.
class TwiddleBank {
 public:
  void add(int n) {
    if (n < 1 || off_.count(n)) return;
    off_[n] = host_.size();
    for (int k = 0; k < n; ++k) {
      const double a = -2.0 * M_PI * (double)k / (double)n;
      host_.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
    }
  }
  size_t offset(int n) const {
    auto it = off_.find(n);
    return it == off_.end() ? 0 : it->second;
  }
  const std::vector<float2>& host() const { return host_; }

 private:
  std::map<int, size_t> off_;
  std::vector<float2> host_;
};

}  // namespace kym
