// Backward helpers: the reflect-pad adjoint kernel and the registry of the
// compile-time specialised backward variants.
#include <mutex>
#include <vector>

#include "bwd.cuh"

namespace kym {

// Padded coordinate t = p - pad reflects onto i when t = +-i (mod 2(n-1)).
__device__ __forceinline__ float reflect_sum_1d(int i, int n, int pad, int np, const float* row, int stride) {
  if (n == 1) {
    float s = 0.f;
    for (int p = 0; p < np; ++p) s += row[(size_t)p * stride];
    return s;
  }
  const int period = 2 * (n - 1);
  const int lo = -pad, hi = np - pad;  // t in [lo, hi)
  float s = 0.f;
  // t = i + k*period
  int k0 = (lo - i) >= 0 ? (lo - i + period - 1) / period : -((i - lo) / period);
  for (int t = i + k0 * period; t < hi; t += period)
    if (t >= lo) s += row[(size_t)(t + pad) * stride];
  if (i != 0 && i != n - 1) {
    // t = -i + k*period
    int k1 = (lo + i) >= 0 ? (lo + i + period - 1) / period : -((-i - lo) / period);
    for (int t = -i + k1 * period; t < hi; t += period)
      if (t >= lo) s += row[(size_t)(t + pad) * stride];
  }
  return s;
}

__global__ void reflect_pad_adjoint_kernel(const float* __restrict__ gpad, long long gpad_stride, int Mp, int Np,
                                           float* __restrict__ gx, int M, int N, int pad_t, int pad_l, int nimg,
                                           int img0) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)nimg * M * N) return;
  const int img = (int)(e / ((long long)M * N));
  const int rem = (int)(e % ((long long)M * N));
  const int i = rem / N, j = rem % N;
  const float* g = gpad + (size_t)img * gpad_stride;
  // separable: sum over the row preimages of (sum over the column preimages)
  float acc = 0.f;
  if (M == 1 && Mp == 1) {
    acc = reflect_sum_1d(j, N, pad_l, Np, g, 1);
  } else {
    const int period = 2 * (M - 1);
    const int lo = -pad_t, hi = Mp - pad_t;
    auto add_row = [&](int t) { acc += reflect_sum_1d(j, N, pad_l, Np, g + (size_t)(t + pad_t) * Np, 1); };
    if (M == 1) {
      for (int t = lo; t < hi; ++t) add_row(t);
    } else {
      int k0 = (lo - i) >= 0 ? (lo - i + period - 1) / period : -((i - lo) / period);
      for (int t = i + k0 * period; t < hi; t += period)
        if (t >= lo) add_row(t);
      if (i != 0 && i != M - 1) {
        int k1 = (lo + i) >= 0 ? (lo + i + period - 1) / period : -((-i - lo) / period);
        for (int t = -i + k1 * period; t < hi; t += period)
          if (t >= lo) add_row(t);
      }
    }
  }
  gx[(size_t)(img0 + img) * M * N + rem] = acc;
}

__global__ void bwd_gather_kernel(const BwdTask* __restrict__ tasks, const GatherItem* __restrict__ gather,
                                  FilterTable F, int mr, int mc, float2* __restrict__ gy, long long gy_stride,
                                  const float2* __restrict__ gyc, long long gyc_stride) {
  const BwdTask t = tasks[blockIdx.y];
  if (t.gather_count == 0) return;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= mr * mc) return;
  const int u = e / mc, v = e - (e / mc) * mc;
  const size_t img = blockIdx.z;
  const float2* yc = gyc + img * gyc_stride;
  float2 acc = make_float2(0.f, 0.f);
  for (int c = 0; c < t.gather_count; ++c) {
    const GatherItem gi = gather[t.gather_first + c];
    const float w = __ldg(F.f[gi.psi] + e) / (float)(gi.kr * gi.kc);
    const float2 y = __ldg(yc + gi.gy_off + (size_t)(u % gi.mr) * gi.mc + (v % gi.mc));
    acc.x = fmaf(y.x, w, acc.x);
    acc.y = fmaf(y.y, w, acc.y);
  }
  gy[img * gy_stride + t.gy_off + e] = acc;
}

namespace {
struct BwdEntry {
  int mr, mc, sr, sc, c;
  bool oned;
  size_t smem;
  BwdCtLauncher fn;
};
std::vector<BwdEntry>& table() {
  static std::vector<BwdEntry> t;
  return t;
}
std::mutex& mu() {
  static std::mutex m;
  return m;
}
}  // namespace

void bwd_ct_register(int mr, int mc, int sr, int sc, int c, bool oned, size_t smem, BwdCtLauncher fn) {
  std::lock_guard<std::mutex> lock(mu());
  table().push_back(BwdEntry{mr, mc, sr, sc, c, oned, smem, fn});
}

bool bwd_ct_find(int mr, int mc, int sr, int sc, int c, bool oned, size_t* smem, BwdCtLauncher* fn) {
  std::lock_guard<std::mutex> lock(mu());
  for (const BwdEntry& e : table())
    if (e.mr == mr && e.mc == mc && e.sr == sr && e.sc == sc && e.c == c && e.oned == oned) {
      *smem = e.smem;
      *fn = e.fn;
      return true;
    }
  return false;
}

}  // namespace kym
