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
// image); one thread per column.  The kernel is bound by load latency, so the
// loads of kGatherUnroll children are issued before their products are
// summed.  The column residues v mod (mc / 2^q) and the strip's row residues
// are tabulated once per block (a child costs a table lookup instead of two
// divisions), and the task's gather list is staged in shared memory
// kGatherMax items at a time.
constexpr int kGatherMax = 64;

__global__ void __launch_bounds__(kGatherThreads) bwd_gather_kernel(const BwdTask* __restrict__ tasks, const GatherItem* __restrict__ gather,
                                  FilterTable F, int mr, int mc, float2* __restrict__ gy, long long gy_stride,
                                  const float2* __restrict__ gyc, long long gyc_stride, int nimg) {
  constexpr int R = kGatherRows, CU = kGatherUnroll;
  __shared__ GatherItem items[kGatherMax];
  __shared__ int vres[kGatherLogs][kGatherThreads];
  __shared__ int ures[kGatherLogs];
  const BwdTask t = tasks[blockIdx.y];
  if (t.gather_count == 0 || (int)blockIdx.z >= nimg) return;
  const float2* yc = gyc + (size_t)blockIdx.z * gyc_stride;
  // blockIdx.x = strip * column tiles + tile (long 1-D rows span several tiles)
  const int ctiles = (mc + blockDim.x - 1) / blockDim.x;
  const int u0 = (blockIdx.x / ctiles) * R;
  const int nr = min(R, mr - u0);
  const int v = (blockIdx.x % ctiles) * blockDim.x + threadIdx.x;
#pragma unroll 1
  for (int q = 0; q < kGatherLogs; ++q) {
    const int m = mc >> q;
    vres[q][threadIdx.x] = m > 0 ? v % m : 0;
  }
  if (threadIdx.x < kGatherLogs) {
    const int m = mr >> threadIdx.x;
    ures[threadIdx.x] = m > 0 ? u0 % m : 0;
  }
  float2 acc[R];
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = make_float2(0.f, 0.f);
  for (int c0 = 0; c0 < t.gather_count; c0 += kGatherMax) {
    const int nc = min(t.gather_count - c0, kGatherMax);
    __syncthreads();
    for (int i = threadIdx.x; i < nc; i += blockDim.x) items[i] = gather[t.gather_first + c0 + i];
    __syncthreads();
    if (v >= mc) continue;
    for (int c = 0; c < nc; c += CU) {
      float f[CU][R];
      float2 y[CU][R];
#pragma unroll
      for (int k = 0; k < CU; ++k) {
        const bool live = c + k < nc;  // uniform over the block
        const GatherItem& gi = items[live ? c + k : c];
        const float* psi = F.f[gi.psi] + (size_t)u0 * mc + v;
        const float2* ycol = yc + gi.gy_off + vres[gi.lkc][threadIdx.x];
        int um = ures[gi.lkr];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const bool ok = live && r < nr;
          f[k][r] = ok ? __ldg(psi + (size_t)r * mc) * gi.w : 0.f;
          y[k][r] = ok ? __ldg(ycol + (size_t)um * gi.mc) : make_float2(0.f, 0.f);
          if (++um == gi.mr) um = 0;
        }
      }
#pragma unroll
      for (int k = 0; k < CU; ++k)
#pragma unroll
        for (int r = 0; r < R; ++r) {
          acc[r].x = fmaf(y[k][r].x, f[k][r], acc[r].x);
          acc[r].y = fmaf(y[k][r].y, f[k][r], acc[r].y);
        }
    }
  }
  if (v < mc) {
    float2* out = gy + (size_t)blockIdx.z * gy_stride + t.gy_off;
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (r < nr) out[(size_t)(u0 + r) * mc + v] = acc[r];
  }
}

template <int NP>
__global__ void __launch_bounds__(kGatherThreads)
    bwd_gather_set_kernel(const BwdTask* __restrict__ tasks, const GatherItem* __restrict__ gather, FilterTable F,
                          int mr, int mc, float2* __restrict__ gy, long long gy_stride,
                          const float2* __restrict__ gyc, long long gyc_stride, int nimg) {
  constexpr int R = kGatherSetRows;
  __shared__ GatherItem items[kGatherMax];
  __shared__ int vres[kGatherLogs][kGatherThreads];
  __shared__ int ures[kGatherLogs];
  const int first = blockIdx.y * NP;  // the set's first task carries the gather list
  const BwdTask t = tasks[first];
  if (t.gather_count == 0 || (int)blockIdx.z >= nimg) return;
  const float2* yc = gyc + (size_t)blockIdx.z * gyc_stride;
  const int ctiles = (mc + blockDim.x - 1) / blockDim.x;
  const int u0 = (blockIdx.x / ctiles) * R;
  const int nr = min(R, mr - u0);
  const int v = (blockIdx.x % ctiles) * blockDim.x + threadIdx.x;
#pragma unroll 1
  for (int q = 0; q < kGatherLogs; ++q) {
    const int m = mc >> q;
    vres[q][threadIdx.x] = m > 0 ? v % m : 0;
  }
  if (threadIdx.x < kGatherLogs) {
    const int m = mr >> threadIdx.x;
    ures[threadIdx.x] = m > 0 ? u0 % m : 0;
  }
  float2 acc[NP][R];
#pragma unroll
  for (int p = 0; p < NP; ++p)
#pragma unroll
    for (int r = 0; r < R; ++r) acc[p][r] = make_float2(0.f, 0.f);
  for (int c0 = 0; c0 < t.gather_count; c0 += kGatherMax) {
    const int nc = min(t.gather_count - c0, kGatherMax);
    __syncthreads();
    for (int i = threadIdx.x; i < nc; i += blockDim.x) items[i] = gather[t.gather_first + c0 + i];
    __syncthreads();
    if (v >= mc) continue;
    for (int c = 0; c < nc; ++c) {
      const GatherItem& gi = items[c];
      const float* psi = F.f[gi.psi] + (size_t)u0 * mc + v;
      const float2* ycol = yc + gi.gy_off + vres[gi.lkc][threadIdx.x];
      int um = ures[gi.lkr];
      float f[R];
      size_t yo[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        f[r] = r < nr ? __ldg(psi + (size_t)r * mc) * gi.w : 0.f;
        yo[r] = (size_t)um * gi.mc;
        if (++um == gi.mr) um = 0;
      }
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const float2* yp = ycol + (size_t)p * gi.gy_pstride;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const float2 y = r < nr ? __ldg(yp + yo[r]) : make_float2(0.f, 0.f);
          acc[p][r].x = fmaf(y.x, f[r], acc[p][r].x);
          acc[p][r].y = fmaf(y.y, f[r], acc[p][r].y);
        }
      }
    }
  }
  if (v < mc) {
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      float2* out = gy + (size_t)blockIdx.z * gy_stride + tasks[first + p].gy_off;
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (r < nr) out[(size_t)(u0 + r) * mc + v] = acc[p][r];
    }
  }
}

cudaError_t launch_gather_set(int np, dim3 grid, int threads, cudaStream_t stream, const BwdTask* tasks,
                              const GatherItem* gather, const FilterTable& F, int mr, int mc, float2* gy,
                              long long gy_stride, const float2* gyc, long long gyc_stride, int nimg) {
  auto kern = np == 8 ? bwd_gather_set_kernel<8> : np == 4 ? bwd_gather_set_kernel<4> : bwd_gather_set_kernel<2>;
  kern<<<grid, threads, 0, stream>>>(tasks, gather, F, mr, mc, gy, gy_stride, gyc, gyc_stride, nimg);
  return cudaGetLastError();
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
