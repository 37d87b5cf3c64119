// Fused scattering cascade: one CTA (or one thread-block cluster) runs one
// scattering path of one image end to end in shared memory.
//
// A task reads a source (the real input image with reflect padding, or a
// spectrum in global memory), forms   A = fold_{kr x kc}(src * psi)
// (the cdgmm of kymatio/backend/torch_backend.py:147-219 fused with the
// periodisation of kymatio/scattering2d/backend/torch_backend.py:92-129),
// optionally runs  A <- FFT2(|IFFT2(A)|)  (kymatio/scattering2d/core/
// scattering2d.py:37-39), optionally stores A as the parent spectrum of the
// next order, and finishes with the low-pass branch
//   S = unpad(Re IFFT2(fold_{ksr x ksc}(A * phi)))
// (scattering2d.py:42-46) written straight into its output channel.  The 1-D
// cascade (kymatio/scattering1d/core/scattering1d.py:40-107) is the same
// program on a single row.
#pragma once
#include <atomic>

#include "fft_engine.cuh"

namespace kym {

// Opt a kernel into a large dynamic shared-memory size on the current device.
// The attribute is per device, so each call site keeps one of these (static,
// per kernel instantiation) and sets it once per device ordinal below 64;
// other ordinals set it on every launch.  Concurrent first calls from several
// host threads may both set it, which is harmless.
struct SmemOptin {
  std::atomic<unsigned long long> done{0};
  template <class K>
  cudaError_t ensure(K kern, int bytes) {
    int d = 0;
    cudaError_t e = cudaGetDevice(&d);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = (d >= 0 && d < 64) ? (1ull << d) : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_release);
    return e;
  }
};

constexpr int kMaxFilters = 1024;

struct FilterTable {
  const float* f[kMaxFilters];
};

struct Task {
  long long src_off;  // complex-element offset of the source spectrum within one image's block
  long long dst_off;  // offset of the stored spectrum, -1 if none
  int psi;            // filter index multiplied before the fold, -1 if none
  int phi;            // low-pass filter index
  int out_ch;         // output channel
  int y_off;          // this path's modulus input y within one image's saved block, -1 if none
};

struct CascadeLaunch {
  int mr, mc, kr, kc;     // work size and load-fold factors (source is kr*mr x kc*mc)
  int ld;                 // shared-memory pitch of the work array (complex elements)
  int sr, sc, ldb;        // low-pass output size and its pitch
  int modulus;            // 1: IFFT2, modulus, FFT2
  int src_image;          // 1: source is the real input image
  int cluster;            // CTAs per task
  int rows_local;         // mr / cluster
  FftPlan prow, pcol, psrow, pscol;
  float load_scale, s_scale;
  int out_r0, out_c0, out_nr, out_nc, out_channels;
  // image source (reflect padding folded into the load)
  const float* x;
  int img_M, img_N, pad_t, pad_l;
  long long x_stride;
  // spectra
  const float2* src;
  long long src_stride;
  float2* dst;
  long long dst_stride;
  float* out;
  long long out_stride;
  const Task* tasks;
  int ntasks;
  int img0;     // first image of this chunk (for x/out offsets)
  int skip_s;   // 1: stop after storing the spectrum (backward recomputation)
  const float2* tw_rl;  // exp(-2 pi i k / (mr / cluster)): local column length of a cluster split
  float2* ysave;        // non-null: store y = IFFT2(...) before the modulus (saved for the backward)
  long long ysave_stride;
  long long bsum_off;   // line-split modulus groups: folded low-pass blocks at dst + img * dst_stride + bsum_off
  unsigned char* opnd;  // DFT-GEMM form: per-path operand slots of the launch (image-major, then task)
  int lines_stage;      // line-split groups: 0 every pass, 1 the line passes only, 2 the low-pass kernel only
};

}  // namespace kym
