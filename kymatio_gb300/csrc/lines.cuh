// Line-split form of a large cascade task: sizes whose work array does not
// fit one CTA's shared memory (272x272 and 288x288 complex64, 592-664 KB).
//
// Instead of one CTA cluster per task that keeps the whole array in shared
// memory, the 2-D transforms run as independent line passes over the task's
// spectrum slot in global memory (the parent-spectrum slot of the task, so
// it costs no extra workspace; a chunk of slots stays in L2).  Every pass is
// a grid of small CTAs (16 lines each), several per SM, with no cluster
// barrier or DSMEM access:
//   rows:    load the source rows (reflect-padded image, or the fold of
//            src * psi / k^2), row FFT (inverse on the modulus path) -> slot
//   columns: modulus path: column IFFT, y saved if asked, |.|, column FFT;
//            input stage: column FFT -> slot
//   rows2:   modulus path: row FFT -> slot (the final spectrum); its row
//            blocks are residue classes of the low-pass fold, so it also
//            leaves B = fold_ks(slot * phi) / ks^2 next to the slots
//   lowpass: one CTA per task and image: B (from rows2, or folded from the
//            slot for the input stage), small IFFT2, real part of the unpad
//            window -> output channel.
// The operations and their order per element are those of ct_cascade_kernel
// (kymatio/scattering2d/core/scattering2d.py:1-88 restated as one task).
#pragma once
#include "ct_cascade.cuh"

namespace kym {

constexpr int kLinesPerCta = 16;
constexpr int kLinesThreads = 256;
constexpr int kLinesMinBlocks = 3;  // CTAs per SM the register budget is sized for

template <int MR, int MC>
struct LinesGeom {
  static constexpr int RB = kLinesPerCta;       // rows per CTA (row passes)
  static constexpr int CB = kLinesPerCta;       // columns per CTA (column pass)
  static constexpr int LDR = MC + 1;            // odd pitch of a row block
  static constexpr int LDC = CB + 1;            // odd pitch of a column block
  static constexpr size_t row_smem = (size_t)RB * LDR * sizeof(float2);
  static constexpr size_t col_smem = (size_t)MR * LDC * sizeof(float2);
  static_assert(MR % RB == 0 && MC % CB == 0, "line blocks");
};

// ---- rows: source rows -> row FFT -> slot ------------------------------------
// KF: 0 image source, k > 0 square fold k x k of src * psi, -1 runtime fold.
template <int MR, int MC, int NT, int KF>
__global__ void __launch_bounds__(NT, kLinesMinBlocks)
    lines_rows_in_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F) {
  using G = LinesGeom<MR, MC>;
  constexpr int RB = G::RB, LDR = G::LDR;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  const Task t = L.tasks[blockIdx.y];
  const int img = blockIdx.z;
  const int r0 = blockIdx.x * RB;
  constexpr int NEL = RB * MC;
  if (KF == 0 || (KF < 0 && L.src_image)) {
    const float* x = L.x + (size_t)(L.img0 + img) * L.x_stride;
    for (int e = threadIdx.x; e < NEL; e += NT) {
      const int u = e / MC, v = e % MC;
      const int iy = ct_reflect(r0 + u - L.pad_t, L.img_M);
      const int ix = ct_reflect(v - L.pad_l, L.img_N);
      A[u * LDR + v] = make_float2(__ldg(x + (size_t)iy * L.img_N + ix) * L.load_scale, 0.f);
    }
  } else if constexpr (KF > 0) {
    static_assert(MC % 2 == 0, "paired columns");
    constexpr int SCOLS = KF * MC;
    const float4* src4 = reinterpret_cast<const float4*>(L.src + (size_t)img * L.src_stride + t.src_off);
    const float2* psi2 = reinterpret_cast<const float2*>(F.f[t.psi]);
    const float sc = L.load_scale;
    for (int e = threadIdx.x; e < NEL / 2; e += NT) {
      const int u = (2 * e) / MC, v = (2 * e) % MC;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int a = 0; a < KF; ++a) {
#pragma unroll
        for (int b = 0; b < KF; ++b) {
          const size_t half = ((size_t)(r0 + u + a * MR) * SCOLS + v + b * MC) >> 1;
          const float4 s4 = __ldg(src4 + half);
          const float2 f2 = __ldg(psi2 + half);
          acc.x = fmaf(s4.x, f2.x, acc.x);
          acc.y = fmaf(s4.y, f2.x, acc.y);
          acc.z = fmaf(s4.z, f2.y, acc.z);
          acc.w = fmaf(s4.w, f2.y, acc.w);
        }
      }
      A[u * LDR + v] = make_float2(acc.x * sc, acc.y * sc);
      A[u * LDR + v + 1] = make_float2(acc.z * sc, acc.w * sc);
    }
  } else {
    const float2* src = L.src + (size_t)img * L.src_stride + t.src_off;
    const float* psi = F.f[t.psi];
    const int scols = L.kc * MC;
    for (int e = threadIdx.x; e < NEL; e += NT) {
      const int u = e / MC, v = e % MC;
      float2 acc = make_float2(0.f, 0.f);
      for (int a = 0; a < L.kr; ++a) {
        const size_t rb = (size_t)(r0 + u + a * MR) * scols + v;
        for (int b = 0; b < L.kc; ++b) {
          const size_t idx = rb + (size_t)b * MC;
          const float2 s = __ldg(src + idx);
          const float f = __ldg(psi + idx);
          acc.x = fmaf(s.x, f, acc.x);
          acc.y = fmaf(s.y, f, acc.y);
        }
      }
      A[u * LDR + v] = cscale(acc, L.load_scale);
    }
  }
  __syncthreads();
  ct::fft_lines<MC, RB, NT>(ct::RowLines<LDR, false>{A}, 0, L.prow.tw, L.modulus != 0);
  float2* slot = L.dst + (size_t)img * L.dst_stride + t.dst_off + (size_t)r0 * MC;
  for (int e = threadIdx.x; e < NEL; e += NT) slot[e] = A[(e / MC) * LDR + e % MC];
}

// ---- columns: column transforms (and the modulus) in place in the slot -------
template <int MR, int MC, int NT>
__global__ void __launch_bounds__(NT, kLinesMinBlocks)
    lines_cols_kernel(const __grid_constant__ CascadeLaunch L) {
  using G = LinesGeom<MR, MC>;
  constexpr int CB = G::CB, LDC = G::LDC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  const Task t = L.tasks[blockIdx.y];
  const int img = blockIdx.z;
  const int c0 = blockIdx.x * CB;
  constexpr int NEL = MR * CB;
  float2* slot = L.dst + (size_t)img * L.dst_stride + t.dst_off + c0;
  for (int e = threadIdx.x; e < NEL; e += NT) {
    const int r = e / CB, j = e % CB;
    A[r * LDC + j] = slot[(size_t)r * MC + j];
  }
  __syncthreads();
  const ct::ColLines<LDC> cols{A};
  if (L.modulus) {
    ct::fft_lines<MR, CB, NT>(cols, 0, L.pcol.tw, true);
    float2* ys = (L.ysave && t.y_off >= 0) ? L.ysave + (size_t)img * L.ysave_stride + t.y_off + c0 : nullptr;
    for (int e = threadIdx.x; e < NEL; e += NT) {
      const int r = e / CB, j = e % CB;
      const float2 z = A[r * LDC + j];
      if (ys) ys[(size_t)r * MC + j] = z;  // saved for the backward
      A[r * LDC + j] = make_float2(sqrtf(fmaf(z.x, z.x, z.y * z.y)), 0.f);
    }
    __syncthreads();
  }
  ct::fft_lines<MR, CB, NT>(cols, 0, L.pcol.tw, false);
  for (int e = threadIdx.x; e < NEL; e += NT) {
    const int r = e / CB, j = e % CB;
    slot[(size_t)r * MC + j] = A[r * LDC + j];
  }
}

// ---- rows2: forward row FFT in place (modulus path), low-pass fold ------------
// Block b holds the rows p + SR a for p in [b PB, b PB + PB) and a < KSR
// (a residue class of the low-pass fold), so it also forms the complete
// folded rows p of B = fold_ks(slot * phi) / ks^2 and leaves them at
// dst + img * dst_stride + bsum_off + task * SR * SC.
template <int MR, int MC, int SR, int SC, int NT>
__global__ void __launch_bounds__(NT, kLinesMinBlocks)
    lines_rows_fwd_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F) {
  using G = LinesGeom<MR, MC>;
  constexpr int RB = G::RB, LDR = G::LDR;
  constexpr int KSR = MR / SR, KSC = MC / SC, PB = RB / KSR;
  static_assert(RB % KSR == 0 && SR % PB == 0, "row blocks are residue classes of the fold");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  const int task = blockIdx.y;
  const Task t = L.tasks[task];
  const int img = blockIdx.z;
  const int p0 = blockIdx.x * PB;
  constexpr int NEL = RB * MC;
  // local row u = pp * KSR + a holds global row p0 + pp + SR * a
  auto grow = [&](int u) { return p0 + u / KSR + SR * (u % KSR); };
  float2* slot = L.dst + (size_t)img * L.dst_stride + t.dst_off;
  for (int e = threadIdx.x; e < NEL; e += NT) {
    const int u = e / MC, v = e % MC;
    A[u * LDR + v] = slot[(size_t)grow(u) * MC + v];
  }
  __syncthreads();
  ct::fft_lines<MC, RB, NT>(ct::RowLines<LDR, false>{A}, 0, L.prow.tw, false);
  for (int e = threadIdx.x; e < NEL; e += NT) {
    const int u = e / MC, v = e % MC;
    slot[(size_t)grow(u) * MC + v] = A[u * LDR + v];
  }
  if (L.skip_s) return;
  const float* phi = F.f[t.phi];
  float2* bsum = L.dst + (size_t)img * L.dst_stride + L.bsum_off + (size_t)task * SR * SC;
  for (int e = threadIdx.x; e < PB * SC; e += NT) {
    const int pp = e / SC, q = e % SC;
    const int p = p0 + pp;
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int a = 0; a < KSR; ++a) {
      const float2* row = A + (pp * KSR + a) * LDR;
      const float* frow = phi + (size_t)(p + SR * a) * MC;
#pragma unroll
      for (int b = 0; b < KSC; ++b) {
        const float2 z = row[q + SC * b];
        const float f = __ldg(frow + q + SC * b);
        acc.x = fmaf(z.x, f, acc.x);
        acc.y = fmaf(z.y, f, acc.y);
      }
    }
    bsum[p * SC + q] = cscale(acc, L.s_scale);
  }
}

// ---- lowpass: B (folded by rows2, or folded here from the slot), small
// IFFT2, real part of the unpad window -> output channel -----------------------
template <int MR, int MC, int SR, int SC, int NT>
__global__ void __launch_bounds__(NT)
    lines_lowpass_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F) {
  constexpr int LDB = SC % 2 == 0 ? SC + 1 : SC;
  constexpr int KSR = MR / SR, KSC = MC / SC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* B = reinterpret_cast<float2*>(smem_raw);
  const int task = blockIdx.x;
  const Task t = L.tasks[task];
  const int img = blockIdx.y;
  if (L.modulus) {
    const float2* bsum = L.dst + (size_t)img * L.dst_stride + L.bsum_off + (size_t)task * SR * SC;
    for (int e = threadIdx.x; e < SR * SC; e += NT) B[(e / SC) * LDB + e % SC] = __ldg(bsum + e);
  } else {
    const float2* slot = L.dst + (size_t)img * L.dst_stride + t.dst_off;
    const float* phi = F.f[t.phi];
    for (int e = threadIdx.x; e < SR * SC; e += NT) {
      const int p = e / SC, q = e % SC;
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll
      for (int a = 0; a < KSR; ++a) {
#pragma unroll
        for (int b = 0; b < KSC; ++b) {
          const size_t idx = (size_t)(p + a * SR) * MC + q + b * SC;
          const float2 z = __ldg(slot + idx);
          const float f = __ldg(phi + idx);
          acc.x = fmaf(z.x, f, acc.x);
          acc.y = fmaf(z.y, f, acc.y);
        }
      }
      B[p * LDB + q] = cscale(acc, L.s_scale);
    }
  }
  __syncthreads();
  ct::fft_lines<SC, SR, NT>(ct::RowLines<LDB, false>{B}, 0, L.psrow.tw, true);
  ct::fft_lines<SR, SC, NT>(ct::ColLines<LDB>{B}, 0, L.pscol.tw, true);
  float* out = L.out + (size_t)(L.img0 + img) * L.out_stride + (size_t)t.out_ch * L.out_nr * L.out_nc;
  for (int e = threadIdx.x; e < L.out_nr * L.out_nc; e += NT) {
    const int p = e / L.out_nc + L.out_r0, q = e % L.out_nc + L.out_c0;
    out[e] = B[p * LDB + q].x;
  }
}

using LinesLauncher = cudaError_t (*)(const CascadeLaunch&, const FilterTable&, int nimg, cudaStream_t);

// Runs the passes of one group launch (every task must own a spectrum slot).
template <int MR, int MC, int SR, int SC, int KF>
cudaError_t lines_launch(const CascadeLaunch& L, const FilterTable& F, int nimg, cudaStream_t stream) {
  using G = LinesGeom<MR, MC>;
  constexpr int NT = kLinesThreads;
  constexpr int LDB = SC % 2 == 0 ? SC + 1 : SC;
  constexpr size_t lp_smem = (size_t)SR * LDB * sizeof(float2);
  auto k_in = lines_rows_in_kernel<MR, MC, NT, KF>;
  auto k_cols = lines_cols_kernel<MR, MC, NT>;
  auto k_fwd = lines_rows_fwd_kernel<MR, MC, SR, SC, NT>;
  auto k_lp = lines_lowpass_kernel<MR, MC, SR, SC, NT>;
  static SmemOptin opt_in, opt_cols, opt_fwd;
  cudaError_t e = opt_in.ensure(k_in, (int)G::row_smem);
  if (e == cudaSuccess) e = opt_cols.ensure(k_cols, (int)G::col_smem);
  if (e == cudaSuccess) e = opt_fwd.ensure(k_fwd, (int)G::row_smem);
  if (e != cudaSuccess) return e;
  k_in<<<dim3(MR / G::RB, L.ntasks, nimg), NT, G::row_smem, stream>>>(L, F);
  k_cols<<<dim3(MC / G::CB, L.ntasks, nimg), NT, G::col_smem, stream>>>(L);
  if (L.modulus) k_fwd<<<dim3(MR / G::RB, L.ntasks, nimg), NT, G::row_smem, stream>>>(L, F);
  if (!L.skip_s) k_lp<<<dim3(L.ntasks, nimg), NT, lp_smem, stream>>>(L, F);
  return cudaGetLastError();
}

// Registry (ct_registry.cu): square sizes, fold kf as in ct_find.
void lines_register(int mr, int mc, int sr, int sc, int kf, LinesLauncher fn);
LinesLauncher lines_find(int mr, int mc, int sr, int sc, int kf);

template <int MR, int MC, int SR, int SC, int KF>
struct LinesRegistrar {
  LinesRegistrar() { lines_register(MR, MC, SR, SC, KF, &lines_launch<MR, MC, SR, SC, KF>); }
};

// A size with a runtime fold (any source), plus compile-time folds.
#define KYM_LINES_VARIANT(MR, MC, SR, SC) \
  static ::kym::LinesRegistrar<MR, MC, SR, SC, -1> kym_lines_reg_##MR##_##MC##_##SR##_##SC;
#define KYM_LINES_FOLD(MR, MC, SR, SC, KF) \
  static ::kym::LinesRegistrar<MR, MC, SR, SC, KF> kym_lines_regf_##MR##_##MC##_##SR##_##SC##_##KF;

}  // namespace kym
