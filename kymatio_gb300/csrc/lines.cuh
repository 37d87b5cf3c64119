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
constexpr int kLinesMinBlocks = 3;  // CTAs per SM the register budget is sized for (80 registers)
constexpr int kRowsFwdMinBlocks = 4;  // the row-FFT pass fits 64 registers (folds of at most 8 rows)

// Copy n <= N complex elements from global to shared memory with every load
// of a thread issued before its first store (N / NT loads in flight per
// thread): idx(e) gives the global offset, sidx(e) the shared one.
template <int N, int NT, class GI, class SI>
__device__ __forceinline__ void staged_copy(float2* __restrict__ dst, const float2* __restrict__ src, int n, GI idx,
                                            SI sidx) {
  constexpr int PER = (N + NT - 1) / NT;
  float2 v[PER];
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = threadIdx.x + i * NT;
    if (e < n) v[i] = src[idx(e)];
  }
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = threadIdx.x + i * NT;
    if (e < n) dst[sidx(e)] = v[i];
  }
}

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
    // reflect-padded image rows, every load of a thread in flight before the first store
    const float* x = L.x + (size_t)(L.img0 + img) * L.x_stride;
    constexpr int PER = (NEL + NT - 1) / NT;
    float xv[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int e = threadIdx.x + i * NT;
      if (e < NEL) {
        const int u = e / MC, v = e % MC;
        const int iy = ct_reflect(r0 + u - L.pad_t, L.img_M);
        const int ix = ct_reflect(v - L.pad_l, L.img_N);
        xv[i] = __ldg(x + (size_t)iy * L.img_N + ix);
      }
    }
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int e = threadIdx.x + i * NT;
      if (e < NEL) A[(e / MC) * LDR + e % MC] = make_float2(xv[i] * L.load_scale, 0.f);
    }
  } else if constexpr (KF > 0) {
    static_assert(MC % 2 == 0, "paired columns");
    constexpr int SCOLS = KF * MC;
    const float4* src4 = reinterpret_cast<const float4*>(L.src + (size_t)img * L.src_stride + t.src_off);
    const float2* psi2 = reinterpret_cast<const float2*>(F.f[t.psi]);
    const float sc = L.load_scale;
    if constexpr (KF == 1) {
      // the product src * psi: every load of a thread in flight before the first use
      constexpr int PER = (NEL / 2 + NT - 1) / NT;
      float4 sv[PER];
      float2 fv[PER];
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int e = threadIdx.x + i * NT;
        if (e < NEL / 2) {
          const size_t half = ((size_t)r0 * MC >> 1) + e;
          sv[i] = __ldg(src4 + half);
          fv[i] = __ldg(psi2 + half);
        }
      }
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int e = threadIdx.x + i * NT;
        if (e < NEL / 2) {
          const int u = (2 * e) / MC, v = (2 * e) % MC;
          A[u * LDR + v] = make_float2(sv[i].x * fv[i].x * sc, sv[i].y * fv[i].x * sc);
          A[u * LDR + v + 1] = make_float2(sv[i].z * fv[i].y * sc, sv[i].w * fv[i].y * sc);
        }
      }
    } else
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
  staged_copy<NEL, NT>(A, slot, NEL, [](int e) { return (size_t)(e / CB) * MC + e % CB; },
                       [](int e) { return (e / CB) * LDC + e % CB; });
  __syncthreads();
  const ct::ColLines<LDC> cols{A};
  if (L.modulus) {
    ct::fft_lines<MR, CB, NT>(cols, 0, L.pcol.tw, true);
    float2* ys = (L.ysave && t.y_off >= 0) ? L.ysave + (size_t)img * L.ysave_stride + t.y_off + c0 : nullptr;
    // U = |y| is real: the forward column FFT runs two columns per complex
    // line, Z = U[:, 2j] + i U[:, 2j+1] in column j (the moduli are held in
    // registers across the barrier, since column j is overwritten)
    static_assert(CB % 2 == 0, "column pairs");
    constexpr int NP = MR * (CB / 2);
    constexpr int PPT = (NP + NT - 1) / NT;
    float2 m[PPT];
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
      const int e = threadIdx.x + i * NT;
      if (e < NP) {
        const int r = e / (CB / 2), j = e % (CB / 2);
        const float2 z0 = A[r * LDC + 2 * j], z1 = A[r * LDC + 2 * j + 1];
        if (ys) {  // saved for the backward
          ys[(size_t)r * MC + 2 * j] = z0;
          ys[(size_t)r * MC + 2 * j + 1] = z1;
        }
        m[i] = make_float2(sqrtf(fmaf(z0.x, z0.x, z0.y * z0.y)), sqrtf(fmaf(z1.x, z1.x, z1.y * z1.y)));
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
      const int e = threadIdx.x + i * NT;
      if (e < NP) A[(e / (CB / 2)) * LDC + e % (CB / 2)] = m[i];
    }
    __syncthreads();
    ct::fft_lines<MR, CB / 2, NT>(cols, 0, L.pcol.tw, false);
    // unpack: X_2j[k] = (Z[k] + conj Z[-k]) / 2, X_2j+1[k] = -i (Z[k] - conj Z[-k]) / 2
    // (exactly Hermitian in k, which the next pass relies on)
    for (int e = threadIdx.x; e < NP; e += NT) {
      const int r = e / (CB / 2), j = e % (CB / 2);
      const float2 a = A[r * LDC + j], b = A[((MR - r) % MR) * LDC + j];
      const float2 x0 = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
      const float2 x1 = make_float2(0.5f * (a.y + b.y), 0.5f * (b.x - a.x));
      slot[(size_t)r * MC + 2 * j] = x0;
      slot[(size_t)r * MC + 2 * j + 1] = x1;
    }
    return;
  }
  ct::fft_lines<MR, CB, NT>(cols, 0, L.pcol.tw, false);
  for (int e = threadIdx.x; e < NEL; e += NT) {
    const int r = e / CB, j = e % CB;
    slot[(size_t)r * MC + j] = A[r * LDC + j];
  }
}

// ---- rows2: forward row FFT in place (modulus path), low-pass fold ------------
// The low-pass fold sums rows p + SR a (a < KSR): a block holds two such
// residue classes, so it also forms the complete folded rows of
// B = fold_ks(slot * phi) / ks^2 for them and leaves them at
// dst + img * dst_stride + bsum_off + task * SR * SC.
// The column pass left every column Hermitian (the FFT of the real modulus),
// so the final spectrum obeys F[MR - r][k] = conj(F[r][(MC - k) % MC]): a
// block pairs class c with its mirror class SR - c, runs the row FFTs of
// class c only and writes the mirror rows as conjugate reversals.  Block 0
// holds the two self-mirrored classes 0 and SR/2 and runs KSR + 1 of their
// rows.  Grid: SR / 2 blocks per task and image.
template <int MR, int MC, int SR, int SC>
struct RowsFwdGeom {
  static constexpr int KSR = MR / SR, KSC = MC / SC;
  static constexpr int RB = 2 * KSR;                      // rows per block
  static constexpr int LDR = MC % 2 == 0 ? MC + 1 : MC;
  static constexpr size_t smem = (size_t)RB * LDR * sizeof(float2);
  static constexpr int blocks = SR / 2;
  static_assert(SR % 2 == 0 && KSR % 2 == 0 && MR % 2 == 0, "mirror classes");
};

// Local row i of block b: its global row, and (for i >= the computed rows)
// the local row whose conjugate reversal it is.
template <int MR, int SR>
__device__ __forceinline__ void rows_fwd_map(int b, int i, int& grow, int& src, int& ncomp) {
  constexpr int KSR = MR / SR, H = KSR / 2;
  if (b > 0) {
    ncomp = KSR;
    if (i < KSR) {
      grow = b + SR * i;
      src = -1;
    } else {  // class SR - b, row (SR - b) + SR m mirrors b + SR (KSR - 1 - m)
      const int m = i - KSR;
      grow = (SR - b) + SR * m;
      src = KSR - 1 - m;
    }
  } else {
    // computed: class 0 rows SR a (a <= H), class SR/2 rows SR/2 + SR a (a < H)
    ncomp = KSR + 1;
    if (i <= H) {
      grow = SR * i;
      src = -1;
    } else if (i < KSR + 1) {
      grow = SR / 2 + SR * (i - H - 1);
      src = -1;
    } else if (i < KSR + 1 + (H - 1)) {  // class 0, a = H+1 .. KSR-1 mirrors a' = KSR - a
      const int a = H + 1 + (i - KSR - 1);
      grow = SR * a;
      src = KSR - a;
    } else {  // class SR/2, a = H .. KSR-1 mirrors a' = KSR - 1 - a (local H + 1 + a')
      const int a = H + (i - KSR - H);
      grow = SR / 2 + SR * a;
      src = H + 1 + (KSR - 1 - a);
    }
  }
}

template <int MR, int MC, int SR, int SC, int NT>
__global__ void __launch_bounds__(NT, MR / SR > 8 ? kLinesMinBlocks : kRowsFwdMinBlocks)
    lines_rows_fwd_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F) {
  using G = RowsFwdGeom<MR, MC, SR, SC>;
  constexpr int KSR = G::KSR, KSC = G::KSC, RB = G::RB, LDR = G::LDR;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  __shared__ int s_grow[RB], s_src[RB];
  __shared__ unsigned char s_loc[MR];  // global row -> local row (the block's rows only)
  const int task = blockIdx.y;
  const Task t = L.tasks[task];
  const int img = blockIdx.z;
  const int b = blockIdx.x;
  static_assert(RB <= NT, "one thread per local row for the row map");
  if (threadIdx.x < RB) {
    int g, src, nc;
    rows_fwd_map<MR, SR>(b, threadIdx.x, g, src, nc);
    s_grow[threadIdx.x] = g;
    s_src[threadIdx.x] = src;
    s_loc[g] = (unsigned char)threadIdx.x;
  }
  __syncthreads();
  const int ncomp = b > 0 ? KSR : KSR + 1;
  float2* slot = L.dst + (size_t)img * L.dst_stride + t.dst_off;
  staged_copy<(KSR + 1) * MC, NT>(A, slot, ncomp * MC, [&](int e) { return (size_t)s_grow[e / MC] * MC + e % MC; },
                                  [](int e) { return (e / MC) * LDR + e % MC; });
  __syncthreads();
  if (b > 0) ct::fft_lines<MC, KSR, NT>(ct::RowLines<LDR, false>{A}, 0, L.prow.tw, false);
  else ct::fft_lines<MC, KSR + 1, NT>(ct::RowLines<LDR, false>{A}, 0, L.prow.tw, false);
  // mirror rows: F[i][k] = conj(F[src][(MC - k) % MC])
  for (int e = threadIdx.x; e < (RB - ncomp) * MC; e += NT) {
    const int i = ncomp + e / MC, v = e % MC;
    const float2 z = A[s_src[i] * LDR + (MC - v) % MC];
    A[i * LDR + v] = make_float2(z.x, -z.y);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < RB * MC; e += NT) {
    const int u = e / MC, v = e % MC;
    slot[(size_t)s_grow[u] * MC + v] = A[u * LDR + v];
  }
  if (L.skip_s) return;
  const float* phi = F.f[t.phi];
  float2* bsum = L.dst + (size_t)img * L.dst_stride + L.bsum_off + (size_t)task * SR * SC;
  // The block's two classes c = cls[0], cls[1]: folded row c of B sums the
  // KSR rows c + SR a.  Four threads per output element each take KSR / 4
  // aliases (their loads unrolled and in flight together); a shuffle adds
  // the four partial sums.
  constexpr int SPL = 4, APT = KSR / SPL;
  static_assert(KSR % SPL == 0 && NT % 32 == 0, "split of the fold");
  const int cls[2] = {b > 0 ? b : 0, b > 0 ? SR - b : SR / 2};
  constexpr int NITEM = 2 * SC * SPL;
  for (int base = 0; base < NITEM; base += NT) {
    const int e = base + threadIdx.x;
    const int sub = e % SPL, o = e / SPL;
    const int ci = o / SC, q = o % SC;
    float2 acc = make_float2(0.f, 0.f);
    if (e < NITEM) {
      const int p = cls[ci];
#pragma unroll
      for (int k = 0; k < APT; ++k) {
        const int a = sub * APT + k;
        const int g = p + SR * a;  // its local row: the one of s_grow equal to g
        const float2* row = A + s_loc[g] * LDR;
        const float* frow = phi + (size_t)g * MC;
#pragma unroll
        for (int bb = 0; bb < KSC; ++bb) {
          const float2 z = row[q + SC * bb];
          const float f = __ldg(frow + q + SC * bb);
          acc.x = fmaf(z.x, f, acc.x);
          acc.y = fmaf(z.y, f, acc.y);
        }
      }
    }
#pragma unroll
    for (int m = 1; m < SPL; m <<= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, m);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, m);
    }
    if (e < NITEM && sub == 0) bsum[cls[ci] * SC + q] = cscale(acc, L.s_scale);
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
  using FG = RowsFwdGeom<MR, MC, SR, SC>;
  auto k_fwd = lines_rows_fwd_kernel<MR, MC, SR, SC, NT>;
  auto k_lp = lines_lowpass_kernel<MR, MC, SR, SC, NT>;
  static SmemOptin opt_in, opt_cols, opt_fwd;
  cudaError_t e = opt_in.ensure(k_in, (int)G::row_smem);
  if (e == cudaSuccess) e = opt_cols.ensure(k_cols, (int)G::col_smem);
  if (e == cudaSuccess) e = opt_fwd.ensure(k_fwd, (int)FG::smem);
  if (e != cudaSuccess) return e;
  if (L.lines_stage != 2) {
    k_in<<<dim3(MR / G::RB, L.ntasks, nimg), NT, G::row_smem, stream>>>(L, F);
    k_cols<<<dim3(MC / G::CB, L.ntasks, nimg), NT, G::col_smem, stream>>>(L);
    if (L.modulus) k_fwd<<<dim3(FG::blocks, L.ntasks, nimg), NT, FG::smem, stream>>>(L, F);
  }
  if (!L.skip_s && L.lines_stage != 1) k_lp<<<dim3(L.ntasks, nimg), NT, lp_smem, stream>>>(L, F);
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
