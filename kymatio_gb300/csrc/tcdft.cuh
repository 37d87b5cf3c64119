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
// copied into shared memory with TMA bulk copies; it stays resident while the
// CTA walks its paths (persistent grid, one CTA per SM).  Every operand x
// enters as hi = bf16(x), lo = bf16(x - hi) and each GEMM sums
// A_hi B_hi + A_lo B_hi + A_hi B_lo.
//
// The fold (the streaming read of the source spectrum and the wavelet) runs
// as a separate high-occupancy pass that writes each path's step-1 operand
// image to a slot in global memory; the GEMM kernel copies path k+1's image
// into its second buffer (TMA bulk copy) while path k is computed.
//
// Shared memory (bytes, MP = M rounded up to 8; SBO = 32 MP; slot = 8 MP^2):
//   [0, slot)             buffer 0: operand A / Z^T (hi rows, lo rows), then
//                         the step-3 operand and T'
//   [slot, 2 slot)        buffer 1
//   [2 slot, +16 MP^2)    Wop hi | lo (2 MP rows each), resident
//   then                  T_r as the step-3 B operand (hi | lo) and T_c (fp32),
//                         resident per low-pass filter; mbarriers, TMEM base
// The M = 128 tile reads rows MP..127 past each half: those rows hold other
// data and only produce accumulator rows that are never read.
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
  // one path's step-1 operand (hi rows, then lo rows): the unit the fold pass
  // writes to global memory and the kernel copies into one of two buffers
  static constexpr uint32_t slot_bytes = (uint32_t)(2 * half_a);
  static constexpr size_t w_half = (size_t)(NP / 8) * SBO;
  static constexpr size_t off_wh = 2 * (size_t)slot_bytes, off_wl = off_wh + w_half;
  static constexpr int K3 = (M + 15) / 16 * 16;
  static constexpr int N3 = NOUT < 16 ? 16 : (NOUT + 15) / 16 * 16;
  static constexpr uint32_t SBO3 = (uint32_t)(K3 / 8) * 128u;
  static constexpr size_t half_a3 = (size_t)(MP / 8) * SBO3;
  static constexpr size_t half_b3 = (size_t)(N3 / 8) * SBO3;
  static constexpr size_t off_a3l = half_a3;  // within the path's buffer
  static constexpr int TLD = N3 + 1;  // fp32 pitch of T'
  // resident low-pass factors of the group: T_r as the step-3 B operand, T_c in fp32
  static constexpr size_t off_b3h = off_wl + w_half, off_b3l = off_b3h + half_b3;
  static constexpr size_t off_tc = off_b3l + half_b3;
  static constexpr int TCLD = M + 1;  // fp32 pitch of T_c (conflict-free column reads)
  static constexpr int MAX_TASKS = 64;
  static constexpr size_t off_tasks = (off_tc + (size_t)NOUT * TCLD * 4 + 15) / 16 * 16;
  static constexpr size_t bar_off = off_tasks + (size_t)MAX_TASKS * sizeof(Task);
  static constexpr size_t smem = bar_off + 48;  // wbar, mbar[2], full[2], TMEM base
  static constexpr int C3 = (NP + 31) / 32 * 32;  // TMEM column of D3
  static constexpr int TMEM_COLS = 512;  // two groups, 256 columns each
  static constexpr uint32_t w_bytes = (uint32_t)(2 * w_half);
  static_assert(M % 4 == 0 && M <= 120, "work size");
  static_assert(NP <= 256 && C3 + N3 <= TMEM_COLS / 2, "accumulator tile too wide");
  static_assert(2 * half_a3 <= slot_bytes && (size_t)M * TLD * 4 <= slot_bytes,
                "step-3 operand and T' fit the path's buffer");
  static_assert(slot_bytes % 16 == 0, "TMA bulk copies move multiples of 16 bytes");
  static_assert(slot_bytes + half_a + 16 * (size_t)SBO <= smem && slot_bytes + off_a3l + 16 * (size_t)SBO3 <= smem,
                "M-tile reads of the second buffer stay inside the allocation");
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

// One 8-column chunk of A = fold_KF(src * psi) * load_scale: row u,
// columns 8c..8c+7 (columns at or beyond M are zero).
template <int M, int KF>
__device__ __forceinline__ void fold_chunk(const CascadeLaunch& L, const FilterTable& F, const Task& t, int img,
                                           int u, int c, float (&re)[8], float (&im)[8]) {
  constexpr int SCOLS = KF * M;
  const float4* src4 = reinterpret_cast<const float4*>(L.src + (size_t)img * L.src_stride + t.src_off);
  const float2* psi2 = reinterpret_cast<const float2*>(F.f[t.psi]);
  const int v0 = 8 * c;
  const bool full = v0 + 8 <= M;  // M % 8 == 4: the last chunk holds 4 columns
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
  const float sc = L.load_scale;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    re[i] *= sc;
    im[i] *= sc;
  }
}

}  // namespace dft

// Fold pass: A = fold_KF(src * psi) * load_scale for every path of the
// launch, written as each path's step-1 operand image (hi rows, lo rows;
// rows M..MP-1 are not written and only feed discarded accumulator rows).
// The paths form a P x Q grid: path p Q + q folds parent spectrum p (at
// tasks[p Q].src_off) with wavelet q (tasks[q].psi).  One CTA computes row u
// of every path of one image, so each source row and wavelet row it needs is
// read once (TMA bulk copies into shared memory) for all the paths sharing it.
template <int M, int KF, int P, int Q>
struct StripGeom {
  static constexpr int SC = KF * M;                      // source columns
  static constexpr uint32_t prow = (uint32_t)SC * 8u;     // bytes of one parent row
  static constexpr uint32_t frow = (uint32_t)SC * 4u;     // bytes of one wavelet row
  static constexpr uint32_t stage = P * prow + Q * frow;  // rows for one alias a
  static constexpr uint32_t tx = KF * stage;
  static constexpr size_t outs = (size_t)P * Q * M * 8;  // the outputs reuse the staging area
  static constexpr size_t bar_off = ((tx > outs ? (size_t)tx : outs) + 15) / 16 * 16;
  static constexpr size_t smem = bar_off + 16;
  static constexpr int NT = (M * P + 31) / 32 * 32;
  static_assert(prow % 16 == 0 && frow % 16 == 0, "bulk copies of whole 16-byte units");
};

template <int M, int KF, int P, int Q>
__global__ void __launch_bounds__(StripGeom<M, KF, P, Q>::NT)
    tcdft_fold_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F,
                      unsigned* status) {
  using G = DftGeom<M, 8>;
  using S = StripGeom<M, KF, P, Q>;
  constexpr int MP = G::MP, NCH = MP / 8, KP = G::KP, SC = S::SC, NT = S::NT;
  extern __shared__ __align__(16) unsigned char sm[];
  const float2* prow = reinterpret_cast<const float2*>(sm);               // [KF][P][SC]
  const float* frow = reinterpret_cast<const float*>(sm + KF * P * S::prow);  // [KF][Q][SC]
  float2* outs = reinterpret_cast<float2*>(sm);                           // [P Q][M], after the fold
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S::bar_off);
  const int u = blockIdx.x, img = blockIdx.y, tid = threadIdx.x;
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0) tc::mbar_expect_tx(bar, S::tx);
  __syncthreads();  // the expected byte count is set before any copy can complete
  if (tid < KF * (P + Q)) {
    // one row copy per thread: alias a, then parent p or wavelet q
    const int a = tid / (P + Q), w = tid - a * (P + Q);
    const size_t r = (size_t)(u + a * M) * SC;
    if (w < P)
      tc::bulk_g2s(sm + (size_t)(a * P + w) * S::prow,
                   L.src + (size_t)img * L.src_stride + L.tasks[w * Q].src_off + r, S::prow, bar);
    else
      tc::bulk_g2s(sm + (size_t)KF * P * S::prow + (size_t)(a * Q + (w - P)) * S::frow,
                   F.f[L.tasks[w - P].psi] + r, S::frow, bar);
  }
  bool ok = tc::mbar_wait_bounded(bar, 0, 1u << 22);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) atomicOr(status, tc::kErrMmaTimeout);
    tc::mbar_wait_bounded(bar, 0, 1u << 22);
    __syncthreads();
  }
  // thread (p, v): the Q paths of parent p at column v
  float2 acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = make_float2(0.f, 0.f);
  const int p = tid / M, v = tid - (tid / M) * M;
  if (tid < M * P) {
#pragma unroll
    for (int a = 0; a < KF; ++a)
#pragma unroll
      for (int b = 0; b < KF; ++b) {
        const float2 sv = prow[(a * P + p) * SC + v + b * M];
        const float* fr = frow + (size_t)a * Q * SC + v + b * M;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const float f = fr[q * SC];
          acc[q].x = fmaf(sv.x, f, acc[q].x);
          acc[q].y = fmaf(sv.y, f, acc[q].y);
        }
      }
  }
  __syncthreads();  // the staging area now holds the outputs
  const float sc = ok ? L.load_scale : __int_as_float(0x7fc00000);
  if (tid < M * P)
#pragma unroll
    for (int q = 0; q < Q; ++q) outs[(p * Q + q) * M + v] = make_float2(acc[q].x * sc, acc[q].y * sc);
  __syncthreads();
  // row u of every path's operand: 16-byte chunks (hi and lo) of [Re | Im]
  for (int e = tid; e < P * Q * 2 * NCH; e += NT) {
    const int t = e / (2 * NCH), r = e - t * (2 * NCH);
    const int part = r / NCH, c = r - part * NCH;
    float v8[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int x = 8 * c + i;
      const float2 z = x < M ? outs[t * M + x] : make_float2(0.f, 0.f);
      v8[i] = part ? z.y : z.x;
    }
    unsigned char* slot = L.opnd + ((size_t)img * L.ntasks + t) * G::slot_bytes;
    dft::store_chunk(slot, slot + G::half_a, u, part * MP + 8 * c, KP, v8);
  }
}

// The GEMM kernel: persistent, one CTA per SM, split into two independent
// groups of 8 warps.  Group g computes paths blockIdx.x + (2k + g) gridDim.x
// in its own operand buffer and its own half of tensor memory, with its own
// barriers, so one group's GEMMs run while the other reads back, and each
// group's next operand copy (TMA bulk copy) lands while the other computes.
namespace dft {
// named barrier of one group (ids 1 and 2; 0 is __syncthreads)
__device__ __forceinline__ void grp_sync(int g) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(256) : "memory");
}
__device__ __forceinline__ bool grp_any(int g, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(1 + g), "r"(256)
      : "memory");
  return r != 0;
}
// group-wide bounded wait; on a time-out the status word is flagged and the
// group waits once more (bounded) for the operations it issued
__device__ __forceinline__ bool grp_wait(int g, uint64_t* bar, uint32_t parity, unsigned* status) {
  const bool ok = tc::mbar_wait_bounded(bar, parity, 1u << 22);
  if (grp_any(g, !ok)) {
    if ((threadIdx.x & 255) == 0) atomicOr(status, tc::kErrMmaTimeout);
    tc::mbar_wait_bounded(bar, parity, 1u << 22);
    grp_sync(g);
    return false;
  }
  return true;
}
}  // namespace dft

template <int M, int NOUT, int KF, int NT>
__global__ void __launch_bounds__(NT, 1)
    tcdft_cascade_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ LowpassTable LP,
                         const unsigned char* __restrict__ wimg, int nimg, unsigned* status) {
  using G = DftGeom<M, NOUT>;
  constexpr int MP = G::MP, KP = G::KP, NP = G::NP, K3 = G::K3, N3 = G::N3, TLD = G::TLD;
  constexpr int NCH = MP / 8;  // 8-column chunks of one [Re | Im] half
  constexpr int GT = 256;      // threads per group
  constexpr int WPQ = 2;       // warps per TMEM lane quarter within a group
  static_assert(NT == 2 * GT, "two groups of 8 warps");
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* wbar = reinterpret_cast<uint64_t*>(smem + G::bar_off);
  uint64_t* mbar = wbar + 1;  // mbar[0], mbar[1]: GEMM completion per group
  uint64_t* full = wbar + 3;  // full[0], full[1]: operand arrival per group
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + G::bar_off + 40);
  const int tid = threadIdx.x;
  const int g = tid / GT, gtid = tid % GT;
  const int warp = gtid >> 5, lane = tid & 31;
  const int quarter = warp & 3, cgroup = warp >> 2;
  const int total = L.ntasks * nimg;

  if (tid < 32) {
    tc::tmem_alloc(slot, G::TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(wbar, 1);
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&mbar[i], 1);
      tc::mbar_init(&full[i], 1);
    }
    tc::mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *slot + (uint32_t)(g * (G::TMEM_COLS / 2));  // this group's half
  if (tid == 0) {
    // the resident DFT matrix, then each group's first operand
    tc::mbar_expect_tx(wbar, G::w_bytes);
    for (uint32_t o = 0; o < G::w_bytes; o += 16384u)
      tc::bulk_g2s(smem + G::off_wh + o, wimg + o, (G::w_bytes - o) < 16384u ? (G::w_bytes - o) : 16384u, wbar);
    for (int i = 0; i < 2; ++i) {
      const int first = (int)blockIdx.x + i * (int)gridDim.x;
      if (first < total) {
        tc::mbar_expect_tx(&full[i], G::slot_bytes);
        tc::bulk_g2s(smem + (size_t)i * G::slot_bytes, L.opnd + (size_t)first * G::slot_bytes, G::slot_bytes,
                     &full[i]);
      }
    }
  }
  // the group's low-pass factors (one filter per group, checked when the plan
  // was made): T_r split into the step-3 B operand, T_c kept in fp32; the task table
  float* tcs = reinterpret_cast<float*>(smem + G::off_tc);
  Task* tasks = reinterpret_cast<Task*>(smem + G::off_tasks);
  for (int i = tid; i < L.ntasks; i += NT) tasks[i] = L.tasks[i];
  {
    const int phi = L.tasks[0].phi;
    const float* trm = LP.r[phi];
    for (int e = tid; e < N3 * (K3 / 8); e += NT) {
      const int p = e % N3, c = e / N3;
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int kk = 8 * c + i;
        v[i] = (p < NOUT && kk < M) ? __ldg(trm + p * M + kk) : 0.f;
      }
      dft::store_chunk(smem + G::off_b3h, smem + G::off_b3l, p, 8 * c, K3, v);
    }
    const float* tcm = LP.c[phi];
    for (int e = tid; e < NOUT * M; e += NT) tcs[e / M * G::TCLD + e % M] = __ldg(tcm + e);
  }
  tc::fence_proxy_async();
  bool alive = dft::cta_wait(wbar, 0, status);  // CTA-wide: includes the barrier for the tables above

  const uint32_t s_wh = tc::smem_addr(smem + G::off_wh), s_wl = tc::smem_addr(smem + G::off_wl);
  const uint32_t s_b3h = tc::smem_addr(smem + G::off_b3h), s_b3l = tc::smem_addr(smem + G::off_b3l);
  constexpr uint32_t idesc1 = tc::idesc_bf16_f32(128, NP);
  constexpr uint32_t idesc3 = tc::idesc_bf16_f32(128, N3);
  unsigned char* buf = smem + (size_t)g * G::slot_bytes;
  unsigned char* ah = buf;
  unsigned char* al = buf + G::half_a;
  const uint32_t s_ah = tc::smem_addr(ah), s_al = tc::smem_addr(al);
  const uint32_t s_a3h = s_ah, s_a3l = s_ah + (uint32_t)G::off_a3l;
  float* Tp = reinterpret_cast<float*>(buf);
  uint32_t ph = 0, fph = 0;
  bool pending = (int)blockIdx.x + g * (int)gridDim.x < total;  // an operand copy is in flight
  for (int item = blockIdx.x + g * gridDim.x; item < total; item += 2 * gridDim.x) {
    const int img = item / L.ntasks;
    const Task t = tasks[item - img * L.ntasks];
    float* out = L.out + (size_t)(L.img0 + img) * L.out_stride + (size_t)t.out_ch * NOUT * NOUT;
    if (alive) {
      alive = dft::grp_wait(g, &full[g], fph, status);
      fph ^= 1u;
      pending = false;
    }
    if (!alive) {
      for (int o = gtid; o < NOUT * NOUT; o += GT) out[o] = __int_as_float(0x7fc00000);
      continue;
    }
    // ---- step 1: Z = A W ---------------------------------------------------------
    tc::fence_after_sync();
    if (gtid == 0) {
      dft::split_gemm(taddr, s_ah, s_al, s_wh, s_wl, G::SBO, idesc1, KP / 16);
      tc::mma_commit(&mbar[g]);
    }
    alive = dft::grp_wait(g, &mbar[g], ph, status);
    ph ^= 1u;
    if (!alive) {
      for (int o = gtid; o < NOUT * NOUT; o += GT) out[o] = __int_as_float(0x7fc00000);
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
      for (int e = gtid; e < M * (MP - M) * 2; e += GT) {
        const int y = e / (2 * (MP - M)), r = e % (2 * (MP - M));
        const int kk = r < MP - M ? M + r : MP + M + (r - (MP - M));
        dft::store_one(ah, al, y, kk, KP, 0.f);
      }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    dft::grp_sync(g);
    tc::fence_after_sync();
    // ---- step 2: U^T = Z^T W ------------------------------------------------------
    if (gtid == 0) {
      dft::split_gemm(taddr, s_ah, s_al, s_wh, s_wl, G::SBO, idesc1, KP / 16);
      tc::mma_commit(&mbar[g]);
    }
    alive = dft::grp_wait(g, &mbar[g], ph, status);
    ph ^= 1u;
    if (!alive) {
      for (int o = gtid; o < NOUT * NOUT; o += GT) out[o] = __int_as_float(0x7fc00000);
      continue;
    }
    tc::fence_after_sync();
    // ---- modulus -> step-3 operand (row y, K = x) -----------------------------------
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
          for (int i = 0; i < 8; ++i) v[i] = (8 * c + i < M) ? tc::sqrt_approx(fmaf(re[i], re[i], im[i] * im[i])) : 0.f;
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) v[i] = 0.f;
        }
        if (y < M) dft::store_chunk(buf, buf + G::off_a3l, y, 8 * c, K3, v);
      }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    dft::grp_sync(g);
    tc::fence_after_sync();
    // ---- step 3: T' = U^T T_r^T ------------------------------------------------------
    if (gtid == 0) {
      dft::split_gemm(taddr + (uint32_t)G::C3, s_a3h, s_a3l, s_b3h, s_b3l, G::SBO3, idesc3, K3 / 16);
      tc::mma_commit(&mbar[g]);
    }
    alive = dft::grp_wait(g, &mbar[g], ph, status);
    ph ^= 1u;
    if (!alive) {
      for (int o = gtid; o < NOUT * NOUT; o += GT) out[o] = __int_as_float(0x7fc00000);
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
    dft::grp_sync(g);
    // ---- S = T_c-contraction of T' on the FP32 pipe ------------------------------------
    // outputs o and o + NOUT^2 / 2 share q (and so their T_c row)
    constexpr int HALF = NOUT * NOUT / 2;
    static_assert((NOUT * NOUT) % 2 == 0 && HALF % NOUT == 0, "paired outputs share their column");
    for (int o = gtid; o < HALF; o += GT) {
      const int p = o / NOUT, q = o % NOUT, p2 = p + HALF / NOUT;
      const float* tq = tcs + q * G::TCLD;
      float acc0 = 0.f, acc1 = 0.f;
#pragma unroll 4
      for (int y = 0; y < M; ++y) {
        const float c = tq[y];
        acc0 = fmaf(c, Tp[y * TLD + p], acc0);
        acc1 = fmaf(c, Tp[y * TLD + p2], acc1);
      }
      out[o] = acc0;
      out[o + HALF] = acc1;
    }
    dft::grp_sync(g);  // T' is dead: the buffer takes the group's next operand
    const int next = item + 2 * gridDim.x;
    if (next < total) {
      if (gtid == 0) {
        tc::fence_proxy_async();
        tc::mbar_expect_tx(&full[g], G::slot_bytes);
        tc::bulk_g2s(buf, L.opnd + (size_t)next * G::slot_bytes, G::slot_bytes, &full[g]);
      }
      pending = true;
    }
  }
  // an operand copy still in flight (only after a time-out): wait for it (bounded)
  if (pending) tc::mbar_wait_bounded(&full[g], fph, 1u << 22);
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(*slot, G::TMEM_COLS);
}

// Launcher: the fold pass into the operand slots (L.opnd), then the GEMM
// kernel on a persistent grid of one CTA per SM with the DFT operand image
// of size M for the current device (built once).
const unsigned char* dft_operand_image(int m, size_t bytes);

template <int M, int KF, int P, int Q>
cudaError_t launch_fold(const CascadeLaunch& L, const FilterTable& F, unsigned* status, int nimg,
                        cudaStream_t stream) {
  using S = StripGeom<M, KF, P, Q>;
  auto kern = tcdft_fold_kernel<M, KF, P, Q>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::smem);
  if (e != cudaSuccess) return e;
  kern<<<dim3(M, nimg, 1), S::NT, S::smem, stream>>>(L, F, status);
  return cudaGetLastError();
}

template <int M, int NOUT, int KF, int NT>
cudaError_t tcdft_launch(const CascadeLaunch& L, const FilterTable& F, const LowpassTable& LP, unsigned* status,
                         int nimg, cudaStream_t stream) {
  using G = DftGeom<M, NOUT>;
  if (!L.opnd) return cudaErrorInvalidValue;
  const int total = L.ntasks * nimg;
  if (total <= 0) return cudaSuccess;
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
  // the fold pass over the P x Q grid of paths (Q = 8 wavelets; P = 1 or 8 sources)
  if (L.ntasks == 8) e = launch_fold<M, KF, 1, 8>(L, F, status, nimg, stream);
  else if (L.ntasks == 64) e = launch_fold<M, KF, 8, 8>(L, F, status, nimg, stream);
  else e = cudaErrorInvalidValue;
  if (e != cudaSuccess) return e;
  const int grid = total < sms ? total : sms;
  kern<<<grid, NT, G::smem, stream>>>(L, LP, w, nimg, status);
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
