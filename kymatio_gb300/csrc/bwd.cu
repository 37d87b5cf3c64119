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

// One block per (strip of kGatherRows rows x tile of blockDim columns, task,
// image); one thread per column.  The task's gather list is staged in shared memory
// kGatherMax items at a time; per child the column residue is one division
// and the row residue advances incrementally.
constexpr int kGatherRows = 8;
constexpr int kGatherMax = 64;

__global__ void bwd_gather_kernel(const BwdTask* __restrict__ tasks, const GatherItem* __restrict__ gather,
                                  FilterTable F, int mr, int mc, float2* __restrict__ gy, long long gy_stride,
                                  const float2* __restrict__ gyc, long long gyc_stride) {
  __shared__ GatherItem items[kGatherMax];
  const BwdTask t = tasks[blockIdx.y];
  if (t.gather_count == 0) return;
  const size_t img = blockIdx.z;
  const float2* yc = gyc + img * gyc_stride;
  float2* out = gy + img * gy_stride + t.gy_off;
  // blockIdx.x = strip * column tiles + tile (long 1-D rows span several tiles)
  const int ctiles = (mc + blockDim.x - 1) / blockDim.x;
  const int u0 = (blockIdx.x / ctiles) * kGatherRows;
  const int u1 = min(u0 + kGatherRows, mr);
  const int v = (blockIdx.x % ctiles) * blockDim.x + threadIdx.x;
  float2 acc[kGatherRows];
#pragma unroll
  for (int r = 0; r < kGatherRows; ++r) acc[r] = make_float2(0.f, 0.f);
  for (int c0 = 0; c0 < t.gather_count; c0 += kGatherMax) {
    const int nc = min(t.gather_count - c0, kGatherMax);
    __syncthreads();
    for (int i = threadIdx.x; i < nc; i += blockDim.x) items[i] = gather[t.gather_first + c0 + i];
    __syncthreads();
    if (v >= mc) continue;
    for (int c = 0; c < nc; ++c) {
      const GatherItem gi = items[c];
      const float* psi = F.f[gi.psi];
      const float w = 1.f / (float)(gi.kr * gi.kc);
      const float2* ycol = yc + gi.gy_off + (v % gi.mc);
      int um = u0 % gi.mr;
#pragma unroll
      for (int r = 0; r < kGatherRows; ++r) {
        if (u0 + r < u1) {
          const float f = __ldg(psi + (size_t)(u0 + r) * mc + v) * w;
          const float2 y = __ldg(ycol + (size_t)um * gi.mc);
          acc[r].x = fmaf(y.x, f, acc[r].x);
          acc[r].y = fmaf(y.y, f, acc[r].y);
        }
        if (++um == gi.mr) um = 0;
      }
    }
  }
  if (v < mc)
#pragma unroll
    for (int r = 0; r < kGatherRows; ++r)
      if (u0 + r < u1) out[(size_t)(u0 + r) * mc + v] = acc[r];
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
