// Device build of the 2-D filter bank (kymatio/scattering2d/filter_bank.py:
// 5-175): the Morlet wavelets psi(j, theta) and the Gaussian low-pass phi,
// each the sum of 5 x 5 periodic images of a slanted, rotated Gabor in space,
// moved to Fourier (real part kept), then cropped to coarser resolutions by
// the masked alias sums of periodize_filter_fft.  The reference builds them
// on the host in complex64 with a Python loop per filter; here every step
// runs in FP64 on the GPU and the result is rounded once to float32, so the
// filters agree with the reference's to float32 rounding (not bit for bit:
// the reference accumulates in complex64).
//
// Steps (one launch each, all filters at once):
//   gabor:  g(x, y) and its envelope e (xi = 0) per filter, FP64 complex
//   sums:   sum(g), sum(e) per filter (the Morlet's zero-mean correction
//           w = g - sum(g) / sum(e) * e, gabor_2d / morlet_2d :94-175)
//   rows:   R = DFT along y of w, FP64 complex
//   cols:   Re(DFT along x of R) = the Fourier-domain filter (real part)
//   crop:   masked alias sums per level (:56-91), rounded to float32, in the
//           order of the reference's tensor{n} buffers
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/kymatio_gb300.h"
#include "errors.h"

namespace kym {
namespace {

struct FbFilter {
  double cxx, cxy, cyy;  // quadratic form of the Gaussian envelope
  double kx, ky;         // xi cos(theta), xi sin(theta)
  double norm;           // 1 / (2 * 3.1415 * sigma^2 / slant), the reference's constant
  int morlet;            // 1: psi (zero-mean correction), 0: phi (plain Gabor)
  int nlev;              // levels kept
  long long out_off;     // float offset of level 0 in the output
};

struct FbSums {
  double gr, gi, er, ei;  // sum(g), sum(e)
};

constexpr int kFbThreads = 256;

// g and e for every pixel of every filter: sum over the 5 x 5 periodic images
__global__ void fb_gabor_kernel(const FbFilter* __restrict__ fl, int M, int N, double2* __restrict__ g,
                                double2* __restrict__ e) {
  const int f = blockIdx.y;
  const FbFilter F = fl[f];
  const long long MN = (long long)M * N;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < MN; p += (long long)gridDim.x * blockDim.x) {
    const int x0 = (int)(p / N), y0 = (int)(p % N);
    double gr = 0.0, gi = 0.0, er = 0.0;
    for (int ex = -2; ex <= 2; ++ex) {
      const double x = (double)(x0 + ex * M);
      for (int ey = -2; ey <= 2; ++ey) {
        const double y = (double)(y0 + ey * N);
        const double a = exp(-(F.cxx * (x * x) + F.cxy * (x * y) + F.cyy * (y * y)));
        double s, c;
        sincos(x * F.kx + y * F.ky, &s, &c);
        gr += a * c;
        gi += a * s;
        er += a;
      }
    }
    g[f * MN + p] = make_double2(gr * F.norm, gi * F.norm);
    e[f * MN + p] = make_double2(er * F.norm, 0.0);
  }
}

// per-filter sums of g and e (one block per filter, fixed order: deterministic)
__global__ void fb_sums_kernel(const double2* __restrict__ g, const double2* __restrict__ e, int M, int N,
                               FbSums* __restrict__ sums) {
  const int f = blockIdx.x;
  const long long MN = (long long)M * N;
  double gr = 0.0, gi = 0.0, er = 0.0, ei = 0.0;
  for (long long p = threadIdx.x; p < MN; p += blockDim.x) {
    const double2 a = g[f * MN + p], b = e[f * MN + p];
    gr += a.x;
    gi += a.y;
    er += b.x;
    ei += b.y;
  }
  __shared__ double red[4][kFbThreads];
  red[0][threadIdx.x] = gr;
  red[1][threadIdx.x] = gi;
  red[2][threadIdx.x] = er;
  red[3][threadIdx.x] = ei;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[f] = FbSums{red[0][0], red[1][0], red[2][0], red[3][0]};
}

// R[x][k] = sum_y w[x][y] exp(-2 pi i k y / N), with w = g - K e (Morlet) or g
__global__ void fb_rows_kernel(const FbFilter* __restrict__ fl, const double2* __restrict__ g,
                               const double2* __restrict__ e, const FbSums* __restrict__ sums,
                               const double2* __restrict__ twn, int M, int N, double2* __restrict__ R) {
  const int f = blockIdx.y;
  const long long MN = (long long)M * N;
  double Kr = 0.0, Ki = 0.0;
  if (fl[f].morlet) {  // K = sum(g) / sum(e)
    const FbSums s = sums[f];
    const double d = s.er * s.er + s.ei * s.ei;
    Kr = (s.gr * s.er + s.gi * s.ei) / d;
    Ki = (s.gi * s.er - s.gr * s.ei) / d;
  }
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < MN; p += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(p / N), k = (int)(p % N);
    const double2* gr = g + f * MN + (long long)x * N;
    const double2* er = e + f * MN + (long long)x * N;
    double ar = 0.0, ai = 0.0;
    for (int y = 0; y < N; ++y) {
      const double2 a = gr[y], b = er[y];
      const double wr = a.x - (Kr * b.x - Ki * b.y), wi = a.y - (Kr * b.y + Ki * b.x);
      const double2 t = twn[(int)(((long long)k * y) % N)];  // exp(-2 pi i k y / N)
      ar += wr * t.x - wi * t.y;
      ai += wr * t.y + wi * t.x;
    }
    R[f * MN + p] = make_double2(ar, ai);
  }
}

// H[k1][k2] = Re sum_x R[x][k2] exp(-2 pi i k1 x / M)
__global__ void fb_cols_kernel(const double2* __restrict__ R, const double2* __restrict__ twm, int M, int N,
                               double* __restrict__ H) {
  const int f = blockIdx.y;
  const long long MN = (long long)M * N;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < MN; p += (long long)gridDim.x * blockDim.x) {
    const int k1 = (int)(p / N), k2 = (int)(p % N);
    double acc = 0.0;
    for (int x = 0; x < M; ++x) {
      const double2 r = R[f * MN + (long long)x * N + k2];
      const double2 t = twm[(int)(((long long)k1 * x) % M)];
      acc += r.x * t.x - r.y * t.y;
    }
    H[f * MN + p] = acc;
  }
}

// level `lev` of filter f: masked alias sum over 2^lev x 2^lev blocks, in the
// reference's block order, rounded to float32
__global__ void fb_crop_kernel(const FbFilter* __restrict__ fl, const double* __restrict__ H, int M, int N,
                               int lev, float* __restrict__ out) {
  const int f = blockIdx.y;
  const FbFilter F = fl[f];
  if (lev >= F.nlev) return;
  const long long MN = (long long)M * N;
  const int k = 1 << lev, mr = M / k, nr = N / k;
  // rows [sx, sx + lx) and columns [sy, sy + ly) are zeroed before the sum
  const int sx = (int)(M * ldexp(1.0, -lev - 1)), lx = (int)(M * (1.0 - ldexp(1.0, -lev)));
  const int sy = (int)(N * ldexp(1.0, -lev - 1)), ly = (int)(N * (1.0 - ldexp(1.0, -lev)));
  long long off = F.out_off;
  for (int l = 0; l < lev; ++l) off += (long long)(M >> l) * (N >> l);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < mr * nr; p += gridDim.x * blockDim.x) {
    const int u = p / nr, v = p % nr;
    double acc = 0.0;
    for (int i = 0; i < k; ++i) {
      const int x = u + i * mr;
      if (x >= sx && x < sx + lx) continue;
      for (int j = 0; j < k; ++j) {
        const int y = v + j * nr;
        if (y >= sy && y < sy + ly) continue;
        acc += H[f * MN + (long long)x * N + y];
      }
    }
    out[off + p] = (float)acc;
  }
}

// Filters in the order of the reference's buffers: phi first, then psi by
// (j, theta); output offsets follow the same order, levels consecutive.
std::vector<FbFilter> make_filters(int M, int N, int J, int L, long long* total) {
  std::vector<FbFilter> fs;
  long long off = 0;
  auto add = [&](double sigma, double theta, double xi, double slant, int morlet, int nlev) {
    // the reference rounds the rotation to float32 (np.float32 R, Rinv)
    const double c = (double)(float)std::cos(theta), s = (double)(float)std::sin(theta);
    // curv = R diag(1, slant^2) R^-1 / (2 sigma^2), R = [[c, -s], [s, c]], R^-1 = [[c, s], [-s, c]]
    const double d = slant * slant;
    const double m00 = c * c + s * s * d, m01 = c * s - s * c * d, m10 = s * c - c * s * d, m11 = s * s + c * c * d;
    const double den = 2.0 * sigma * sigma;
    FbFilter F;
    F.cxx = m00 / den;
    F.cxy = (m01 + m10) / den;
    F.cyy = m11 / den;
    F.kx = xi * std::cos(theta);
    F.ky = xi * std::sin(theta);
    F.norm = 1.0 / (2.0 * 3.1415 * sigma * sigma / slant);
    F.morlet = morlet;
    F.nlev = nlev;
    F.out_off = off;
    for (int l = 0; l < nlev; ++l) off += (long long)(M >> l) * (N >> l);
    fs.push_back(F);
  };
  add(0.8 * std::ldexp(1.0, J - 1), 0.0, 0.0, 1.0, 0, J);
  const int t0 = (int)(L - L / 2.0 - 1);
  for (int j = 0; j < J; ++j)
    for (int t = 0; t < L; ++t)
      add(0.8 * std::ldexp(1.0, j), (t0 - t) * M_PI / L, 3.0 / 4.0 * M_PI / std::ldexp(1.0, j), 4.0 / L, 1,
          std::min(j + 1, std::max(J - 1, 1)));
  *total = off;
  return fs;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace
}  // namespace kym

extern "C" size_t kym_s2d_filter_bank_workspace_bytes(int M_padded, int N_padded, int J, int L) {
  if (M_padded < 1 || N_padded < 1 || J < 1 || L < 1) return 0;
  const size_t nf = 1 + (size_t)J * L, MN = (size_t)M_padded * N_padded;
  return kym::align256(nf * sizeof(kym::FbFilter)) + kym::align256(nf * sizeof(kym::FbSums)) +
         kym::align256(((size_t)M_padded + N_padded) * sizeof(double2)) + 3 * kym::align256(nf * MN * sizeof(double2));
}

extern "C" long long kym_s2d_filter_bank_floats(int M_padded, int N_padded, int J, int L) {
  if (M_padded < 1 || N_padded < 1 || J < 1 || L < 1) return -1;
  long long total = 0;
  kym::make_filters(M_padded, N_padded, J, L, &total);
  return total;
}

extern "C" int kym_s2d_filter_bank(int M_padded, int N_padded, int J, int L, float* out, long long out_floats,
                                   void* workspace, size_t workspace_bytes, void* stream_) {
  using namespace kym;
  if (M_padded < 1 || N_padded < 1 || J < 1 || L < 1 || (M_padded >> (J - 1)) < 1 || (N_padded >> (J - 1)) < 1 ||
      M_padded % (1 << (J - 1)) || N_padded % (1 << (J - 1)) || !out) {
    set_error_message("filter_bank", "needs padded sizes divisible by 2^(J-1), J >= 1, L >= 1 and an output");
    return KYM_ERR_INVALID;
  }
  long long total = 0;
  const std::vector<FbFilter> fs = make_filters(M_padded, N_padded, J, L, &total);
  if (out_floats < total) {
    set_error_message("filter_bank", "output smaller than kym_s2d_filter_bank_floats");
    return KYM_ERR_INVALID;
  }
  const size_t need = kym_s2d_filter_bank_workspace_bytes(M_padded, N_padded, J, L);
  if (!workspace || workspace_bytes < need) {
    set_error_message("filter_bank", "workspace missing or smaller than kym_s2d_filter_bank_workspace_bytes");
    return KYM_ERR_WORKSPACE;
  }
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const int nf = (int)fs.size();
  const size_t MN = (size_t)M_padded * N_padded;
  unsigned char* w = static_cast<unsigned char*>(workspace);
  FbFilter* dfl = reinterpret_cast<FbFilter*>(w);
  w += align256(nf * sizeof(FbFilter));
  FbSums* sums = reinterpret_cast<FbSums*>(w);
  w += align256(nf * sizeof(FbSums));
  double2* twm = reinterpret_cast<double2*>(w);
  double2* twn = twm + M_padded;
  w += align256(((size_t)M_padded + N_padded) * sizeof(double2));
  double2* g = reinterpret_cast<double2*>(w);
  w += align256(nf * MN * sizeof(double2));
  double2* e = reinterpret_cast<double2*>(w);
  w += align256(nf * MN * sizeof(double2));
  double2* R = reinterpret_cast<double2*>(w);
  double* H = reinterpret_cast<double*>(g);  // g is dead once the row DFT has read it
  // twiddles exp(-2 pi i k / n), FP64
  std::vector<double2> tw(M_padded + N_padded);
  for (int k = 0; k < M_padded; ++k)
    tw[k] = make_double2(std::cos(-2.0 * M_PI * k / M_padded), std::sin(-2.0 * M_PI * k / M_padded));
  for (int k = 0; k < N_padded; ++k)
    tw[M_padded + k] = make_double2(std::cos(-2.0 * M_PI * k / N_padded), std::sin(-2.0 * M_PI * k / N_padded));
  // synchronous copies: the host tables are freed when this call returns
  cudaError_t err = cudaMemcpy(dfl, fs.data(), nf * sizeof(FbFilter), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(twm, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    set_error_message("filter_bank", cudaGetErrorString(err));
    return KYM_ERR_CUDA;
  }
  const int bx = (int)std::min<size_t>((MN + kFbThreads - 1) / kFbThreads, 1024);
  fb_gabor_kernel<<<dim3(bx, nf), kFbThreads, 0, stream>>>(dfl, M_padded, N_padded, g, e);
  fb_sums_kernel<<<nf, kFbThreads, 0, stream>>>(g, e, M_padded, N_padded, sums);
  fb_rows_kernel<<<dim3(bx, nf), kFbThreads, 0, stream>>>(dfl, g, e, sums, twn, M_padded, N_padded, R);
  fb_cols_kernel<<<dim3(bx, nf), kFbThreads, 0, stream>>>(R, twm, M_padded, N_padded, H);
  for (int lev = 0; lev < J; ++lev)
    fb_crop_kernel<<<dim3(bx, nf), kFbThreads, 0, stream>>>(dfl, H, M_padded, N_padded, lev, out);
  err = cudaGetLastError();
  if (err != cudaSuccess) {
    set_error_message("filter_bank", cudaGetErrorString(err));
    return KYM_ERR_CUDA;
  }
  return KYM_OK;
}
