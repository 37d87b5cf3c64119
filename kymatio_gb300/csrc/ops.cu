// Op-level kernels behind the reference's backend operator surface
// (kymatio/scattering2d/backend/torch_backend.py:19-180,
// kymatio/scattering1d/backend/torch_backend.py:18-141,
// kymatio/backend/torch_backend.py:5-219): batched 2-D/1-D FFTs of any
// size the engine plans, complex x real/complex products, periodisation and
// its adjoint, modulus and its adjoint, reflect padding and its adjoint.
// Complex data is interleaved (re, im), the reference's trailing dim of 2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/kymatio_gb300.h"
#include "bwd.cuh"
#include "errors.h"
#include "fft_engine.cuh"
#include "plan_util.h"

namespace kym {

// ---------------------------------------------------------------------------
// batched 2-D FFT: one CTA (or a cluster of C CTAs split by rows) per image
// ---------------------------------------------------------------------------
struct OpFftLaunch {
  FftPlan prow, pcol;  // along a row (length N), along a column (length M)
  int M, N, ld, rows_local, cluster;
  int in_real, out_real, inverse;
  float scale;
  const float* in;
  float* out;
  bool oned;
};

template <bool CL, bool ONED>
__global__ void __launch_bounds__(kThreads, 1) op_fft2_kernel(const __grid_constant__ OpFftLaunch L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  float2** rowp = reinterpret_cast<float2**>(A + (size_t)L.rows_local * L.ld);
  const int C = CL ? L.cluster : 1;
  int rank = 0;
  if constexpr (CL) {
    cg::cluster_group cl = cg::this_cluster();
    rank = static_cast<int>(cl.block_rank());
    for (int g = threadIdx.x; g < L.M; g += blockDim.x) {
      const int owner = g / L.rows_local;
      rowp[g] = cl.map_shared_rank(A, owner) + (size_t)(g - owner * L.rows_local) * L.ld;
    }
  }
  const size_t img = blockIdx.x / C;
  const int row0 = rank * L.rows_local;
  const int nloc = L.rows_local * L.N;
  auto at = [&](int u, int v) -> float2* {
    if constexpr (ONED) return A + (v + (v >> 4));
    else return A + (size_t)u * L.ld + v;
  };
  const size_t base = img * (size_t)L.M * L.N + (size_t)row0 * L.N;
  for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
    float2 v;
    if (L.in_real) v = make_float2(__ldg(L.in + base + e), 0.f);
    else v = __ldg(reinterpret_cast<const float2*>(L.in) + base + e);
    *at(e / L.N, e % L.N) = v;
  }
  __syncthreads();
  Slab w;
  w.local = A;
  w.rowp = rowp;
  w.rows = L.M;
  w.cols = L.N;
  w.ld = L.ld;
  w.rows_local = L.rows_local;
  w.row0 = row0;
  w.nct = C;
  w.rank = rank;
  const bool inv = L.inverse != 0;
  fft_pass<true, ONED, false>(w, L.rows_local, 0, L.prow, inv, Barrier{false});
  if constexpr (!ONED) {
    const int cpc = L.N / C;
    if constexpr (CL) cg::this_cluster().sync();
    fft_pass<false, false, CL>(w, cpc, rank * cpc, L.pcol, inv, Barrier{CL});
  }
  for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
    const float2 v = *at(e / L.N, e % L.N);
    if (L.out_real) L.out[base + e] = v.x * L.scale;
    else reinterpret_cast<float2*>(L.out)[base + e] = make_float2(v.x * L.scale, v.y * L.scale);
  }
}

// Many short 1-D lines per CTA: lines are the local rows of an odd-pitch
// array (pitch L.ld), transformed by the row pass of the 2-D engine.  The
// one-CTA-per-line kernel above leaves most of a CTA idle on lines of a
// few dozen points (the frequency axis of joint time-frequency scattering
// transforms tens of thousands of them per call).
__global__ void __launch_bounds__(kThreads) op_fft_lines_kernel(const __grid_constant__ OpFftLaunch L,
                                                                long long nlines, int lpc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  const long long l0 = (long long)blockIdx.x * lpc;
  const int nl = (int)min((long long)lpc, nlines - l0);
  const int N = L.N, ld = L.ld;
  const size_t base = (size_t)l0 * N;
  for (int e = threadIdx.x; e < nl * N; e += blockDim.x) {
    float2 v;
    if (L.in_real) v = make_float2(__ldg(L.in + base + e), 0.f);
    else v = __ldg(reinterpret_cast<const float2*>(L.in) + base + e);
    A[(e / N) * ld + e % N] = v;
  }
  __syncthreads();
  Slab w;
  w.local = A;
  w.rowp = nullptr;
  w.rows = nl;
  w.cols = N;
  w.ld = ld;
  w.rows_local = nl;
  w.row0 = 0;
  w.nct = 1;
  w.rank = 0;
  fft_pass<true, false, false>(w, nl, 0, L.prow, L.inverse != 0, Barrier{false});
  for (int e = threadIdx.x; e < nl * N; e += blockDim.x) {
    const float2 v = A[(e / N) * ld + e % N];
    if (L.out_real) L.out[base + e] = v.x * L.scale;
    else reinterpret_cast<float2*>(L.out)[base + e] = make_float2(v.x * L.scale, v.y * L.scale);
  }
}

// 1-D lines of at most this many points go through op_fft_lines_kernel
constexpr int kShortLine = 2048;
constexpr size_t kLinesSmem = 48 * 1024;  // shared memory per CTA of the short-line kernel

namespace {

struct OpPlan {
  FftPlan prow, pcol;
  int ld, rows_local, cluster;
  size_t smem;
  bool oned;
  std::map<int, float2*> tw_dev;  // per device: twiddles of N then M
  TwiddleBank tw;
};

std::mutex g_op_mu;
std::map<std::pair<int, int>, OpPlan*> g_op_plans;

OpPlan* op_plan(int M, int N, int* rc) {
  std::lock_guard<std::mutex> lock(g_op_mu);
  auto key = std::make_pair(M, N);
  auto it = g_op_plans.find(key);
  OpPlan* P = nullptr;
  if (it != g_op_plans.end()) {
    P = it->second;
  } else {
    P = new OpPlan();
    P->oned = (M == 1);
    if (!make_fft_plan(N, &P->prow, kThreads) || !make_fft_plan(M, &P->pcol, kThreads)) {
      delete P;
      *rc = KYM_ERR_UNSUPPORTED;
      set_error_message("fft", "size has a prime factor above 127 or lines too long for one CTA");
      return nullptr;
    }
    P->tw.add(N);
    P->tw.add(M);
    const size_t maxs = max_dynamic_smem();
    if (P->oned) {
      P->ld = N + (N >> 4) + 1;
      P->cluster = 1;
      P->rows_local = 1;
      P->smem = (size_t)P->ld * sizeof(float2);
      if (P->smem > maxs) P->smem = 0;
    } else {
      P->ld = (N % 2 == 0) ? N + 1 : N;
      P->smem = 0;
      for (int c : {1, 2, 4, 8}) {
        if (M % c || N % c) continue;
        size_t s = (size_t)(M / c) * P->ld * sizeof(float2) + (c > 1 ? (size_t)M * sizeof(void*) : 0);
        if (s <= maxs) {
          P->cluster = c;
          P->rows_local = M / c;
          P->smem = s;
          break;
        }
      }
    }
    if (!P->smem) {
      delete P;
      *rc = KYM_ERR_UNSUPPORTED;
      set_error_message("fft", "transform does not fit the shared memory of a cluster of 8 CTAs");
      return nullptr;
    }
    g_op_plans[key] = P;
  }
  int d = 0;
  cudaGetDevice(&d);
  if (!P->tw_dev.count(d)) {
    float2* p = nullptr;
    const auto& h = P->tw.host();
    if (cudaMalloc(&p, h.size() * sizeof(float2)) != cudaSuccess ||
        cudaMemcpy(p, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess) {
      *rc = KYM_ERR_CUDA;
      set_error_message("fft", "twiddle table upload failed");
      return nullptr;
    }
    P->tw_dev[d] = p;
  }
  return P;
}

template <bool CL, bool ONED>
cudaError_t launch_op_fft(const OpPlan* P, const OpFftLaunch& L, int batch, cudaStream_t stream) {
  auto kern = op_fft2_kernel<CL, ONED>;
  static SmemOptin optin;
  if (cudaError_t e = optin.ensure(kern, (int)max_dynamic_smem()); e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(batch * P->cluster, 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = P->smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  cfg.attrs = attr;
  if (CL) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = P->cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kern, L);
}

// ---------------------------------------------------------------------------
// elementwise kernels
// ---------------------------------------------------------------------------
__global__ void cdgmm_kernel(const float2* __restrict__ A, const float* __restrict__ B, float2* __restrict__ C,
                             long long batch, long long n, int b_complex) {
  const long long total = batch * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % n;
    const float2 a = A[e];
    if (b_complex) {
      const float2 b = reinterpret_cast<const float2*>(B)[i];
      C[e] = make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    } else {
      const float b = B[i];
      C[e] = make_float2(a.x * b, a.y * b);
    }
  }
}

__global__ void modulus_kernel(const float2* __restrict__ x, float* __restrict__ y, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float2 z = x[e];
    y[e] = sqrtf(z.x * z.x + z.y * z.y);
  }
}

// ModulusStable.backward (kymatio/backend/torch_backend.py:85-96): x g / |x|, 0 where |x| == 0
__global__ void modulus_backward_kernel(const float2* __restrict__ x, const float* __restrict__ g,
                                        float2* __restrict__ gx, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float2 z = x[e];
    const float m = sqrtf(z.x * z.x + z.y * z.y);
    gx[e] = m == 0.f ? make_float2(0.f, 0.f) : make_float2(z.x * g[e] / m, z.y * g[e] / m);
  }
}

// out[b, u, v] = mean over (a, c) < (k, k) of x[b, u + a M/k, v + c N/k] (2-D);
// M = 1 gives the 1-D periodisation.
__global__ void subsample_kernel(const float2* __restrict__ x, float2* __restrict__ y, int batch, int M, int N,
                                 int kr, int kc) {
  const int m = M / kr, n = N / kc;
  const long long total = (long long)batch * m * n;
  const float s = 1.f / (float)(kr * kc);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / ((long long)m * n);
    const int r = (int)(e % ((long long)m * n));
    const int u = r / n, v = r % n;
    float2 acc = make_float2(0.f, 0.f);
    for (int a = 0; a < kr; ++a)
      for (int c = 0; c < kc; ++c) {
        const float2 z = x[(b * M + u + a * m) * (long long)N + v + c * n];
        acc.x += z.x;
        acc.y += z.y;
      }
    y[e] = make_float2(acc.x * s, acc.y * s);
  }
}

// adjoint of the periodisation: gx[b, u, v] = g[b, u mod m, v mod n] / (kr kc)
__global__ void subsample_adjoint_kernel(const float2* __restrict__ g, float2* __restrict__ gx, int batch, int M,
                                         int N, int kr, int kc) {
  const int m = M / kr, n = N / kc;
  const long long total = (long long)batch * M * N;
  const float s = 1.f / (float)(kr * kc);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / ((long long)M * N);
    const int r = (int)(e % ((long long)M * N));
    const int u = r / N, v = r % N;
    const float2 z = g[(b * m + u % m) * (long long)n + v % n];
    gx[e] = make_float2(z.x * s, z.y * s);
  }
}

__device__ __forceinline__ int op_reflect(int i, int n) {
  if (n == 1) return 0;
  const int period = 2 * (n - 1);
  i %= period;
  if (i < 0) i += period;
  return i < n ? i : period - i;
}

__global__ void reflect_pad_kernel(const float* __restrict__ x, float* __restrict__ y, int batch, int M, int N, int top,
                                   int left, int Mp, int Np) {
  const long long total = (long long)batch * Mp * Np;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / ((long long)Mp * Np);
    const int r = (int)(e % ((long long)Mp * Np));
    const int i = op_reflect(r / Np - top, M), j = op_reflect(r % Np - left, N);
    y[e] = x[(b * M + i) * (long long)N + j];
  }
}

int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)); }

int finish(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error_message(what, cudaGetErrorString(e));
    return KYM_ERR_CUDA;
  }
  return KYM_OK;
}

}  // namespace
}  // namespace kym

using namespace kym;

extern "C" int kym_op_fft2(const float* in, float* out, int batch, int M, int N, int in_real, int out_real,
                           int inverse, float scale, void* stream) {
  if (!in || !out || batch < 0 || M < 1 || N < 1) {
    set_error_message("fft", "bad arguments");
    return KYM_ERR_INVALID;
  }
  if (batch == 0) return KYM_OK;
  int rc = KYM_OK;
  OpPlan* P = op_plan(M, N, &rc);
  if (!P) return rc;
  int d = 0;
  cudaGetDevice(&d);
  OpFftLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.prow = P->prow;
  L.pcol = P->pcol;
  L.prow.tw = P->tw_dev[d] + P->tw.offset(N);
  L.pcol.tw = P->tw_dev[d] + P->tw.offset(M);
  L.M = M;
  L.N = N;
  L.ld = P->ld;
  L.rows_local = P->rows_local;
  L.cluster = P->cluster;
  L.in_real = in_real;
  L.out_real = out_real;
  L.inverse = inverse;
  L.scale = scale;
  L.in = in;
  L.out = out;
  L.oned = P->oned;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (P->oned && N <= kShortLine) {
    // many lines per CTA, odd pitch
    OpFftLaunch Ls = L;
    Ls.ld = (N % 2 == 0) ? N + 1 : N;
    const int lpc = (int)std::max<size_t>(1, kLinesSmem / ((size_t)Ls.ld * sizeof(float2)));
    const long long nblk = ((long long)batch + lpc - 1) / lpc;
    const size_t smem = (size_t)std::min<long long>(lpc, batch) * Ls.ld * sizeof(float2);
    op_fft_lines_kernel<<<(unsigned)nblk, kThreads, smem, s>>>(Ls, (long long)batch, lpc);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error_message("fft", cudaGetErrorString(e));
      return KYM_ERR_CUDA;
    }
    return KYM_OK;
  }
  for (int b0 = 0; b0 < batch; b0 += 1 << 20) {
    OpFftLaunch Lb = L;
    const size_t off = (size_t)b0 * M * N * (in_real ? 1 : 2);
    const size_t ooff = (size_t)b0 * M * N * (out_real ? 1 : 2);
    Lb.in = in + off;
    Lb.out = out + ooff;
    const int nb = std::min(batch - b0, 1 << 20);
    if (P->oned) e = launch_op_fft<false, true>(P, Lb, nb, s);
    else if (P->cluster > 1) e = launch_op_fft<true, false>(P, Lb, nb, s);
    else e = launch_op_fft<false, false>(P, Lb, nb, s);
    if (e != cudaSuccess) {
      set_error_message("fft", cudaGetErrorString(e));
      return KYM_ERR_CUDA;
    }
  }
  return KYM_OK;
}

extern "C" int kym_op_cdgmm(const float* A, const float* B, float* C, long long batch, long long n, int b_complex,
                            void* stream) {
  if (!A || !B || !C || batch < 0 || n < 0) return KYM_ERR_INVALID;
  if (batch * n == 0) return KYM_OK;
  cdgmm_kernel<<<grid_for(batch * n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(A), B, reinterpret_cast<float2*>(C), batch, n, b_complex);
  return finish("cdgmm");
}

extern "C" int kym_op_modulus(const float* x, float* y, long long n, void* stream) {
  if (!x || !y || n < 0) return KYM_ERR_INVALID;
  if (n == 0) return KYM_OK;
  modulus_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(reinterpret_cast<const float2*>(x), y,
                                                                           n);
  return finish("modulus");
}

extern "C" int kym_op_modulus_backward(const float* x, const float* g, float* gx, long long n, void* stream) {
  if (!x || !g || !gx || n < 0) return KYM_ERR_INVALID;
  if (n == 0) return KYM_OK;
  modulus_backward_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(x), g, reinterpret_cast<float2*>(gx), n);
  return finish("modulus_backward");
}

extern "C" int kym_op_subsample(const float* x, float* y, int batch, int M, int N, int kr, int kc, void* stream) {
  if (!x || !y || batch < 0 || M < 1 || N < 1 || kr < 1 || kc < 1 || M % kr || N % kc) return KYM_ERR_INVALID;
  if (batch == 0) return KYM_OK;
  const long long total = (long long)batch * (M / kr) * (N / kc);
  subsample_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(x), reinterpret_cast<float2*>(y), batch, M, N, kr, kc);
  return finish("subsample_fourier");
}

extern "C" int kym_op_subsample_adjoint(const float* g, float* gx, int batch, int M, int N, int kr, int kc,
                                        void* stream) {
  if (!g || !gx || batch < 0 || M < 1 || N < 1 || kr < 1 || kc < 1 || M % kr || N % kc) return KYM_ERR_INVALID;
  if (batch == 0) return KYM_OK;
  const long long total = (long long)batch * M * N;
  subsample_adjoint_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(g), reinterpret_cast<float2*>(gx), batch, M, N, kr, kc);
  return finish("subsample_fourier_adjoint");
}

extern "C" int kym_op_reflect_pad(const float* x, float* y, int batch, int M, int N, int top, int bottom, int left,
                                  int right, void* stream) {
  if (!x || !y || batch < 0 || M < 1 || N < 1 || top < 0 || bottom < 0 || left < 0 || right < 0) return KYM_ERR_INVALID;
  if (batch == 0) return KYM_OK;
  const int Mp = M + top + bottom, Np = N + left + right;
  const long long total = (long long)batch * Mp * Np;
  reflect_pad_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, y, batch, M, N, top, left, Mp,
                                                                                    Np);
  return finish("reflect_pad");
}

extern "C" int kym_op_reflect_pad_adjoint(const float* g, float* gx, int batch, int M, int N, int top, int bottom,
                                          int left, int right, void* stream) {
  if (!g || !gx || batch < 0 || M < 1 || N < 1 || top < 0 || bottom < 0 || left < 0 || right < 0)
    return KYM_ERR_INVALID;
  if (batch == 0) return KYM_OK;
  const int Mp = M + top + bottom, Np = N + left + right;
  const int total = batch * M * N;
  reflect_pad_adjoint_kernel<<<(total + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      g, (long long)Mp * Np, Mp, Np, gx, M, N, top, left, batch, 0);
  return finish("reflect_pad_adjoint");
}
