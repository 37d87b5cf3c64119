// DFT-GEMM form of a childless cascade task on the 5th-generation tensor
// cores: the inverse 2-D DFT of the folded spectrum, and the separable
// low-pass product, run as split-precision GEMMs against DFT / low-pass
// matrices (tcgen05, BF16 hi/lo operands, FP32 accumulation in TMEM).
//
// One task (kymatio/scattering2d/core/scattering2d.py:48-75 for one order-2
// path, :37-46 for an order-1 path without children) computes
//   A = fold_k(src * psi) / k^2 / M^2                 (cdgmm + subsample_fourier)
//   U = |W A W|,  W[v][y] = exp(+2 pi i v y / M)     (ifft2 + modulus)
//   S = T_r U T_c^T                                   (the low-pass branch)
// with the complex products written as real GEMMs over [Re | Im] halves:
//   step 1  Z = A W        D1[u][y | MP+y]  = sum_k Aop[u][k] Wop[y | MP+y][k]
//   step 2  U^T = Z^T W    D2[y][x | MP+x]  = sum_k Zop[y][k] Wop[x | MP+x][k]
//   step 3  T' = U^T T_r^T D3[y][p]         = sum_x U[x][y] T_r[p][x]
//   then    S[p][q] = sum_y T_c[q][y] T'[y][p]      (FP32 pipe)
// Wop = [[Re W, -Im W], [Im W, Re W]] is built once on the host in FP64,
// split into BF16 hi + lo, laid out as the shared-memory operand image and
// copied into shared memory with one TMA bulk copy per CTA; it stays resident
// while the CTA walks its tasks (persistent grid, one CTA per SM).  Every
// operand x enters as hi = bf16(x), lo = bf16(x - hi) and each GEMM sums
// A_hi B_hi + A_lo B_hi + A_hi B_lo.
//
// Shared memory (bytes, MP = M rounded up to 8; SBO = 32 MP):
//   [0, 4 MP^2)        operand A / Z^T, hi half (rows 0..MP-1)
//   [4 MP^2, 8 MP^2)   operand A / Z^T, lo half
//   [8 MP^2, 24 MP^2)  Wop hi | lo (2 MP rows each), resident
//   [24 MP^2, +32)     mbarriers, TMEM base
// The M = 128 tile reads rows MP..127 past each half: those rows hold other
// data and only produce accumulator rows that are never read.  Steps 3 and
// the T' read-back reuse [0, 8 MP^2).
#pragma once
#include "tc_cascade.cuh"

namespace kym {

template <int M, int NOUT>
struct DftGeom {
  static constexpr int MP = (M + 7) / 8 * 8;
  static constexpr int KP = 2 * MP;  // K: [Re | Im] halves
  static constexpr int NP = 2 * MP;  // N: [Re | Im] halves of the output
  static constexpr uint32_t SBO = (uint32_t)(KP / 8) * 128u;
  static constexpr size_t half_a = (size_t)(MP / 8) * SBO;
  static constexpr size_t off_ah = 0, off_al = half_a;
  static constexpr size_t w_half = (size_t)(NP / 8) * SBO;
  static constexpr size_t off_wh = 2 * half_a, off_wl = off_wh + w_half;
  static constexpr int K3 = (M + 15) / 16 * 16;
  static constexpr int N3 = NOUT < 16 ? 16 : (NOUT + 15) / 16 * 16;
  static constexpr uint32_t SBO3 = (uint32_t)(K3 / 8) * 128u;
  static constexpr size_t half_a3 = (size_t)(MP / 8) * SBO3;
  static constexpr size_t half_b3 = (size_t)(N3 / 8) * SBO3;
  static constexpr size_t off_a3h = 0, off_a3l = half_a3, off_b3h = 2 * half_a3, off_b3l = off_b3h + half_b3;
  static constexpr int TLD = N3 + 1;  // fp32 pitch of T'
  static constexpr size_t bar_off = off_wl + w_half;
  static constexpr size_t smem = bar_off + 32;
  static constexpr int C3 = (NP + 31) / 32 * 32;  // TMEM column of D3
  static constexpr int TMEM_COLS = 256;
  static constexpr uint32_t w_bytes = (uint32_t)(2 * w_half);
  static_assert(M % 4 == 0 && M <= 120, "work size");
  static_assert(NP <= 256 && C3 + N3 <= TMEM_COLS, "accumulator tile too wide");
  static_assert(off_b3l + half_b3 <= off_wh, "low-pass operands overlap the resident DFT matrix");
  static_assert((size_t)M * TLD * 4 <= off_wh, "T' overlaps the resident DFT matrix");
  static_assert(off_al + 16 * (size_t)SBO <= smem && off_a3l + 16 * (size_t)SBO3 <= smem,
                "M-tile reads stay inside the allocation");
};

namespace dft {

// 16-byte chunk of 8 K-consecutive bf16 values (hi and lo) at (row r, k0).
__device__ __forceinline__ void store_chunk(unsigned char* hi, unsigned char* lo, int r, int k0, int kp,
                                            const float (&v)[8]) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    __nv_bfloat16 h0, l0, h1, l1;
    tc::split_bf16(v[2 * i], h0, l0);
    tc::split_bf16(v[2 * i + 1], h1, l1);
    h[i] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
    l[i] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
  }
  const uint32_t off = tc::kmajor_offset(r, k0, kp);
  *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void store_one(unsigned char* hi, unsigned char* lo, int r, int k, int kp, float v) {
  __nv_bfloat16 h, l;
  tc::split_bf16(v, h, l);
  const uint32_t off = tc::kmajor_offset(r, k, kp);
  *reinterpret_cast<__nv_bfloat16*>(hi + off) = h;
  *reinterpret_cast<__nv_bfloat16*>(lo + off) = l;
}

// D (+)= A B^T over ksteps K-steps of 16, three split products per step.
__device__ __forceinline__ void split_gemm(uint32_t d, uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl,
                                           uint32_t sbo, uint32_t idesc, int ksteps) {
#pragma unroll 1
  for (int ks = 0; ks < ksteps; ++ks) {
    const uint32_t s = (uint32_t)ks * 256u;
    tc::mma_bf16(d, tc::smem_desc(ah + s, 128, sbo), tc::smem_desc(bh + s, 128, sbo), idesc, ks > 0);
    tc::mma_bf16(d, tc::smem_desc(al + s, 128, sbo), tc::smem_desc(bh + s, 128, sbo), idesc, true);
    tc::mma_bf16(d, tc::smem_desc(ah + s, 128, sbo), tc::smem_desc(bl + s, 128, sbo), idesc, true);
  }
}

// Every thread polls the barrier (bounded); the CTA agrees on the outcome.
// On a time-out the status word is flagged and the CTA waits once more
// (bounded) for the operations it issued before giving up.
__device__ __forceinline__ bool cta_wait(uint64_t* bar, uint32_t parity, unsigned* status) {
  bool ok = tc::mbar_wait_bounded(bar, parity, 1u << 22);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) atomicOr(status, tc::kErrMmaTimeout);
    tc::mbar_wait_bounded(bar, parity, 1u << 22);
    __syncthreads();
    return false;
  }
  return true;
}

// A = fold_KF(src * psi) * load_scale, written as the step-1 operand:
// row u, K chunk c (columns 8c..8c+7) for Re and chunk MP/8 + c for Im.
template <int M, int KF, int NT, int MP>
__device__ __forceinline__ void load_fold(unsigned char* ah, unsigned char* al, const CascadeLaunch& L,
                                          const FilterTable& F, const Task& t, int img) {
  constexpr int NCH = MP / 8, SCOLS = KF * M, KP = 2 * MP;
  const float4* src4 = reinterpret_cast<const float4*>(L.src + (size_t)img * L.src_stride + t.src_off);
  const float2* psi2 = reinterpret_cast<const float2*>(F.f[t.psi]);
  const float sc = L.load_scale;
  for (int e = threadIdx.x; e < M * NCH; e += NT) {
    const int u = e / NCH, c = e % NCH;
    const int v0 = 8 * c;
    const bool full = v0 + 8 <= M;  // M % 8 == 4: the last chunk holds 4 columns
    float re[8], im[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) re[i] = im[i] = 0.f;
#pragma unroll
    for (int a = 0; a < KF; ++a) {
#pragma unroll
      for (int b = 0; b < KF; ++b) {
        const size_t base = (size_t)(u + a * M) * SCOLS + v0 + b * M;  // a multiple of 4
        const float4* s = src4 + (base >> 1);
        const float2* f = psi2 + (base >> 1);
        const float4 s0 = __ldg(s), s1 = __ldg(s + 1);
        const float2 f0 = __ldg(f), f1 = __ldg(f + 1);
        re[0] = fmaf(s0.x, f0.x, re[0]); im[0] = fmaf(s0.y, f0.x, im[0]);
        re[1] = fmaf(s0.z, f0.y, re[1]); im[1] = fmaf(s0.w, f0.y, im[1]);
        re[2] = fmaf(s1.x, f1.x, re[2]); im[2] = fmaf(s1.y, f1.x, im[2]);
        re[3] = fmaf(s1.z, f1.y, re[3]); im[3] = fmaf(s1.w, f1.y, im[3]);
        if (full) {
          const float4 s2 = __ldg(s + 2), s3 = __ldg(s + 3);
          const float2 f2 = __ldg(f + 2), f3 = __ldg(f + 3);
          re[4] = fmaf(s2.x, f2.x, re[4]); im[4] = fmaf(s2.y, f2.x, im[4]);
          re[5] = fmaf(s2.z, f2.y, re[5]); im[5] = fmaf(s2.w, f2.y, im[5]);
          re[6] = fmaf(s3.x, f3.x, re[6]); im[6] = fmaf(s3.y, f3.x, im[6]);
          re[7] = fmaf(s3.z, f3.y, re[7]); im[7] = fmaf(s3.w, f3.y, im[7]);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      re[i] *= sc;
      im[i] *= sc;
    }
    store_chunk(ah, al, u, v0, KP, re);
    store_chunk(ah, al, u, MP + v0, KP, im);
  }
}

}  // namespace dft

template <int M, int NOUT, int KF, int NT>
__global__ void __launch_bounds__(NT, 1)
    tcdft_cascade_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F,
                         const __grid_constant__ LowpassTable LP, const unsigned char* __restrict__ wimg, int nimg,
                         unsigned* status) {
  using G = DftGeom<M, NOUT>;
  constexpr int MP = G::MP, KP = G::KP, NP = G::NP, K3 = G::K3, N3 = G::N3, TLD = G::TLD;
  constexpr int NCH = MP / 8;        // 8-column chunks of one [Re | Im] half
  constexpr int WPQ = NT / 128;      // warps per TMEM lane quarter
  static_assert(NT % 128 == 0, "whole lane quarters");
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* ah = smem + G::off_ah;
  unsigned char* al = smem + G::off_al;
  uint64_t* wbar = reinterpret_cast<uint64_t*>(smem + G::bar_off);
  uint64_t* mbar = wbar + 1;
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + G::bar_off + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, cgroup = warp >> 2;

  if (tid < 32) {
    tc::tmem_alloc(slot, G::TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(wbar, 1);
    tc::mbar_init(mbar, 1);
    tc::mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *slot;
  if (tid == 0) {
    // the resident DFT matrix: one TMA bulk copy, in 16 KB pieces
    tc::mbar_expect_tx(wbar, G::w_bytes);
    for (uint32_t o = 0; o < G::w_bytes; o += 16384u)
      tc::bulk_g2s(smem + G::off_wh + o, wimg + o, (G::w_bytes - o) < 16384u ? (G::w_bytes - o) : 16384u, wbar);
  }
  const uint32_t s_ah = tc::smem_addr(ah), s_al = tc::smem_addr(al);
  const uint32_t s_wh = tc::smem_addr(smem + G::off_wh), s_wl = tc::smem_addr(smem + G::off_wl);
  const uint32_t s_a3h = tc::smem_addr(smem + G::off_a3h), s_a3l = tc::smem_addr(smem + G::off_a3l);
  const uint32_t s_b3h = tc::smem_addr(smem + G::off_b3h), s_b3l = tc::smem_addr(smem + G::off_b3l);
  constexpr uint32_t idesc1 = tc::idesc_bf16_f32(128, NP);
  constexpr uint32_t idesc3 = tc::idesc_bf16_f32(128, N3);
  float* Tp = reinterpret_cast<float*>(smem);

  const int total = L.ntasks * nimg;
  uint32_t ph = 0;
  bool alive = dft::cta_wait(wbar, 0, status);
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    const int img = item / L.ntasks;
    const Task t = L.tasks[item - img * L.ntasks];
    float* out = L.out + (size_t)(L.img0 + img) * L.out_stride + (size_t)t.out_ch * NOUT * NOUT;
    if (!alive) {
      for (int o = tid; o < NOUT * NOUT; o += NT) out[o] = __int_as_float(0x7fc00000);
      continue;
    }
    // ---- step 1: Z = A W ---------------------------------------------------------
    dft::load_fold<M, KF, NT, MP>(ah, al, L, F, t, img);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      dft::split_gemm(taddr, s_ah, s_al, s_wh, s_wl, G::SBO, idesc1, KP / 16);
      tc::mma_commit(mbar);
    }
    alive = dft::cta_wait(mbar, ph, status);
    ph ^= 1u;
    if (!alive) {
      for (int o = tid; o < NOUT * NOUT; o += NT) out[o] = __int_as_float(0x7fc00000);
      continue;
    }
    tc::fence_after_sync();
    // ---- Z -> step-2 operand, transposed: row y, K = [Re Z[.][y] | Im Z[.][y]] -----
    if (32 * quarter < M) {
      const int u = 32 * quarter + lane;
      const uint32_t lrow = taddr + ((uint32_t)(32 * quarter) << 16);
      for (int c = cgroup; c < NCH; c += WPQ) {
        float re[8], im[8];
        tc::tmem_ld8(lrow + (uint32_t)(8 * c), re);
        tc::tmem_ld8(lrow + (uint32_t)(MP + 8 * c), im);
        tc::tmem_wait_ld();
        if (u < M) {
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int y = 8 * c + i;
            if (y < M) {
              dft::store_one(ah, al, y, u, KP, re[i]);
              dft::store_one(ah, al, y, MP + u, KP, im[i]);
            }
          }
        }
      }
    }
    if constexpr (MP > M) {
      // K padding of the valid rows: k in [M, MP) and [MP + M, 2 MP)
      for (int e = tid; e < M * (MP - M) * 2; e += NT) {
        const int y = e / (2 * (MP - M)), r = e % (2 * (MP - M));
        const int k = r < MP - M ? M + r : MP + M + (r - (MP - M));
        dft::store_one(ah, al, y, k, KP, 0.f);
      }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- step 2: U^T = Z^T W ------------------------------------------------------
    if (tid == 0) {
      dft::split_gemm(taddr, s_ah, s_al, s_wh, s_wl, G::SBO, idesc1, KP / 16);
      tc::mma_commit(mbar);
    }
    alive = dft::cta_wait(mbar, ph, status);
    ph ^= 1u;
    if (!alive) {
      for (int o = tid; o < NOUT * NOUT; o += NT) out[o] = __int_as_float(0x7fc00000);
      continue;
    }
    tc::fence_after_sync();
    // ---- modulus -> step-3 operand (row y, K = x); T_r -> B operand ------------------
    if (32 * quarter < M) {
      const int y = 32 * quarter + lane;
      const uint32_t lrow = taddr + ((uint32_t)(32 * quarter) << 16);
      for (int c = cgroup; c < K3 / 8; c += WPQ) {
        float v[8];
        if (c < NCH) {
          float re[8], im[8];
          tc::tmem_ld8(lrow + (uint32_t)(8 * c), re);
          tc::tmem_ld8(lrow + (uint32_t)(MP + 8 * c), im);
          tc::tmem_wait_ld();
#pragma unroll
          for (int i = 0; i < 8; ++i) v[i] = (8 * c + i < M) ? sqrtf(fmaf(re[i], re[i], im[i] * im[i])) : 0.f;
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) v[i] = 0.f;
        }
        if (y < M) dft::store_chunk(smem + G::off_a3h, smem + G::off_a3l, y, 8 * c, K3, v);
      }
    }
    {
      const float* trm = LP.r[t.phi];
      for (int e = tid; e < N3 * (K3 / 8); e += NT) {
        const int p = e % N3, c = e / N3;
        float v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int k = 8 * c + i;
          v[i] = (p < NOUT && k < M) ? __ldg(trm + p * M + k) : 0.f;
        }
        dft::store_chunk(smem + G::off_b3h, smem + G::off_b3l, p, 8 * c, K3, v);
      }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- step 3: T' = U^T T_r^T ------------------------------------------------------
    if (tid == 0) {
      dft::split_gemm(taddr + (uint32_t)G::C3, s_a3h, s_a3l, s_b3h, s_b3l, G::SBO3, idesc3, K3 / 16);
      tc::mma_commit(mbar);
    }
    alive = dft::cta_wait(mbar, ph, status);
    ph ^= 1u;
    if (!alive) {
      for (int o = tid; o < NOUT * NOUT; o += NT) out[o] = __int_as_float(0x7fc00000);
      continue;
    }
    tc::fence_after_sync();
    if (cgroup == 0 && 32 * quarter < M) {
      const int y = 32 * quarter + lane;
      const uint32_t lrow = taddr + ((uint32_t)(32 * quarter) << 16) + (uint32_t)G::C3;
#pragma unroll
      for (int c = 0; c < N3 / 8; ++c) {
        float v[8];
        tc::tmem_ld8(lrow + (uint32_t)(8 * c), v);
        tc::tmem_wait_ld();
        if (y < M)
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (8 * c + i < NOUT) Tp[y * TLD + 8 * c + i] = v[i];
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    // ---- S = T_c-contraction of T' on the FP32 pipe ------------------------------------
    {
      const float* tcm = LP.c[t.phi];
      for (int o = tid; o < NOUT * NOUT; o += NT) {
        const int p = o / NOUT, q = o % NOUT;
        const float* tq = tcm + q * M;
        float acc0 = 0.f, acc1 = 0.f;
#pragma unroll 4
        for (int y = 0; y < M; y += 2) {
          acc0 = fmaf(__ldg(tq + y), Tp[y * TLD + p], acc0);
          acc1 = fmaf(__ldg(tq + y + 1), Tp[(y + 1) * TLD + p], acc1);
        }
        out[o] = acc0 + acc1;
      }
    }
    __syncthreads();  // T' is overwritten by the next task's operands
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(taddr, G::TMEM_COLS);
}

// Launcher: the DFT operand image of size M for the current device
// (built once), a persistent grid of one CTA per SM.
const unsigned char* dft_operand_image(int m, size_t bytes);

template <int M, int NOUT, int KF, int NT>
cudaError_t tcdft_launch(const CascadeLaunch& L, const FilterTable& F, const LowpassTable& LP, unsigned* status,
                         int nimg, cudaStream_t stream) {
  using G = DftGeom<M, NOUT>;
  auto kern = tcdft_cascade_kernel<M, NOUT, KF, NT>;
  const unsigned char* w = dft_operand_image(M, G::w_bytes);
  if (!w) return cudaErrorMemoryAllocation;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::smem);
  if (e != cudaSuccess) return e;
  const int total = L.ntasks * nimg;
  if (total <= 0) return cudaSuccess;
  const int grid = total < sms ? total : sms;
  kern<<<grid, NT, G::smem, stream>>>(L, F, LP, w, nimg, status);
  return cudaGetLastError();
}

void tcdft_register(int mr, int mc, int nr, int nc, int kf, size_t smem, TcLauncher fn);
bool tcdft_find(int mr, int mc, int nr, int nc, int kf, size_t* smem, TcLauncher* fn);

template <int M, int NOUT, int KF, int NT>
struct TcDftRegistrar {
  TcDftRegistrar() { tcdft_register(M, M, NOUT, NOUT, KF, DftGeom<M, NOUT>::smem, &tcdft_launch<M, NOUT, KF, NT>); }
};

#define KYM_TCDFT_VARIANT(M, NOUT, KF, NT) \
  static ::kym::TcDftRegistrar<M, NOUT, KF, NT> kym_tcdft_reg_##M##_##NOUT##_##KF;

}  // namespace kym
