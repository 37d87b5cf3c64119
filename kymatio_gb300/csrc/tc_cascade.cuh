// Tensor-core form of a childless cascade task (order-2 paths and the last
// order-1 scale): the modulus U = |IFFT2(fold(src * psi))| is computed as in
// the plain kernel, then the low-pass branch
//   S = unpad(Re IFFT2(fold_ks(FFT2(U) * phi)))
// runs as the separable product  S = T_r * U * T_c^T.  That identity holds
// because the low-pass filter phi (an isotropic Gaussian, periodised and
// masked per axis) is a rank-one outer product u v^T: T_r[p][x] =
// h_u[((p + r0) * ks - x) mod m] with h_u = IFFT(u), r0 the unpad offset
// (kymatio/scattering2d/filter_bank.py:45-51, torch_backend.py:92-180).
// U * T_c^T runs on tcgen05 from BF16 hi/lo operands (three products, FP32
// accumulation in tensor memory); T_r * (.) runs on the FP32 pipe.
#pragma once
#include "ct_cascade.cuh"
#include "tc.cuh"

namespace kym {

constexpr int kMaxLowpass = 32;

// Separable low-pass factors by low-pass filter index: rows (out_nr x mr)
// and columns (out_nc x mc), float32, row-major.
struct LowpassTable {
  const float* r[kMaxLowpass];
  const float* c[kMaxLowpass];
};

template <int MR, int MC, int NOUT>
struct TcGeom {
  static constexpr int LD = (MC % 2 == 0 ? MC + 1 : MC);
  static constexpr int MT = (MR + 127) / 128;          // M tiles of U
  static constexpr int KP = (MC + 15) / 16 * 16;       // K padded
  static constexpr int NP = (NOUT + 15) / 16 * 16;     // N padded (T_c rows)
  static constexpr size_t fft_bytes = (size_t)MR * LD * sizeof(float2);
  static constexpr size_t aop_bytes = (size_t)MT * 128 * KP * 2 * 2;  // hi + lo
  static constexpr size_t region0 = (fft_bytes > aop_bytes ? fft_bytes : aop_bytes);
  static constexpr size_t bop_off = (region0 + 1023) / 1024 * 1024;
  static constexpr size_t bop_bytes = (size_t)NP * KP * 2 * 2;
  static constexpr size_t t_off = bop_off + bop_bytes;
  static constexpr int TLD = NP + 1;                    // fp32 pitch of T = U T_c^T
  static constexpr size_t t_bytes = (size_t)MR * TLD * sizeof(float);
  static constexpr size_t bar_off = (t_off + t_bytes + 15) / 16 * 16;
  static constexpr size_t smem = bar_off + 16;
  // columns read back: tile mt occupies [mt*NP, mt*NP + NP); reads go 32 at a time
  static constexpr int TMEM_NEED = (MT - 1) * NP + (NP + 31) / 32 * 32;
  static constexpr int TMEM_COLS = TMEM_NEED <= 32 ? 32 : (TMEM_NEED <= 64 ? 64 : (TMEM_NEED <= 128 ? 128 : 256));
  static_assert(TMEM_NEED <= 256, "product tile too wide for the tensor-memory budget");
};

template <int MR, int MC, int NOUTR, int NOUTC, int KF, int NT>
__global__ void __launch_bounds__(NT, occupancy_blocks(TcGeom<MR, MC, NOUTC>::smem, NT))
    tc_cascade_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F,
                      const __grid_constant__ LowpassTable LP, unsigned* status) {
  using G = TcGeom<MR, MC, NOUTC>;
  constexpr int LD = G::LD, KP = G::KP, NP = G::NP, MT = G::MT, TLD = G::TLD;
  // M tile mt covers rows [tile_row0, tile_row0 + 128); the last tile of a
  // height above 128 is shifted back so that it ends at the last row group
  // (overlapping rows are computed twice, identically)
  auto tile_row0 = [](int mt) -> int {
    constexpr int MR8 = (MR + 7) / 8 * 8;
    const int r = mt * 128;
    return (MR > 128 && r + 128 > MR8) ? MR8 - 128 : r;
  };
  extern __shared__ __align__(1024) unsigned char smem[];
  float2* A = reinterpret_cast<float2*>(smem);
  unsigned char* aop = smem;
  unsigned char* bop = smem + G::bop_off;
  float* T = reinterpret_cast<float*>(smem + G::t_off);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + G::bar_off);
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + G::bar_off + 8);
  const int tid = threadIdx.x;
  const int img = blockIdx.y;
  const Task t = L.tasks[blockIdx.x];

  // tensor memory for the product tiles, allocated while the FFTs run
  if (tid < 32) {
    tc::tmem_alloc(slot, G::TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) tc::mbar_init(mbar, 1);

  // Operand B = T_c (NP x KP, rows beyond NOUTC and columns beyond MC zero):
  // its values are loaded into registers here and split into the operand
  // after the fold, so the loads' latency overlaps the fold's.
  constexpr int G8 = KP / 8;  // 16-byte chunks per operand row
  constexpr int BPER = (NP * G8 + NT - 1) / NT;
  const float* tcm = LP.c[t.phi];
  const size_t b_half = (size_t)NP * KP * 2;
  float bval[BPER][8];
#pragma unroll
  for (int i = 0; i < BPER; ++i) {
    const int g = tid + i * NT;
    const int r = g % NP, c = g / NP;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = 8 * c + q;
      bval[i][q] = (g < NP * G8 && r < NOUTC && k < MC) ? __ldg(tcm + r * MC + k) : 0.f;
    }
  }

  // ---- U = |IFFT2(fold(src * psi))| -----------------------------------------
  ct_load<MR, MC, 1, false, NT, KF, LD>(A, L, F, t, img, 0);
#pragma unroll
  for (int i = 0; i < BPER; ++i) {
    const int g = tid + i * NT;
    if (g < NP * G8) {
      const int r = g % NP, c = g / NP;
      uint32_t h[4], l[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) tc::split2_bf16(bval[i][2 * q], bval[i][2 * q + 1], h[q], l[q]);
      const uint32_t off = tc::kmajor_offset(r, 8 * c, KP);
      *reinterpret_cast<uint4*>(bop + off) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4*>(bop + b_half + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
  __syncthreads();
  ct::fft_lines<MC, MR, NT>(ct::RowLines<LD, false>{A}, 0, L.prow.tw, true);
  ct::fft_lines<MR, MC, NT>(ct::ColLines<LD>{A}, 0, L.pcol.tw, true);
  // Operand A = U in core-matrix layout, written as 16-byte chunks: item g
  // covers row r and the 8 columns 8c..8c+7 (one core-matrix row); eight
  // consecutive items are the 8 rows of one core matrix (128 contiguous
  // bytes).  Rows beyond MR are never written: they only feed output rows
  // that are discarded.  Columns beyond MC are zero.
  constexpr int MR8 = (MR + 7) / 8 * 8;   // rows rounded to whole core matrices
  constexpr int NIT = MR8 * G8;
  constexpr int PER = (NIT + NT - 1) / NT;
  uint4 hi4[PER], lo4[PER];
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int g = tid + i * NT;
    hi4[i] = make_uint4(0, 0, 0, 0);
    lo4[i] = make_uint4(0, 0, 0, 0);
    if (g < NIT) {
      const int r = (g / 8) % (MR8 / 8) * 8 + (g % 8);  // 8 consecutive items = 8 rows
      const int c = g / MR8;
      uint32_t h[4] = {0, 0, 0, 0}, l[4] = {0, 0, 0, 0};
      if (r < MR) {
        float uv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int k = 8 * c + q;
          uv[q] = 0.f;
          if (k < MC) {
            const float2 z = A[r * LD + k];
            uv[q] = tc::sqrt_approx(fmaf(z.x, z.x, z.y * z.y));
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) tc::split2_bf16(uv[2 * q], uv[2 * q + 1], h[q], l[q]);
      }
      hi4[i] = make_uint4(h[0], h[1], h[2], h[3]);
      lo4[i] = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
  __syncthreads();  // the FFT array is dead from here on; its space holds the operands
  const size_t a_half = (size_t)MT * 128 * KP * 2;
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int g = tid + i * NT;
    if (g < NIT) {
      const int r = (g / 8) % (MR8 / 8) * 8 + (g % 8);
      const int c = g / MR8;
      const uint32_t off = tc::kmajor_offset(r, 8 * c, KP);
      *reinterpret_cast<uint4*>(aop + off) = hi4[i];
      *reinterpret_cast<uint4*>(aop + a_half + off) = lo4[i];
    }
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *slot;

  // ---- T = U * T_c^T on the tensor cores ---------------------------------------
  if (tid == 0) {
    constexpr uint32_t sbo = (uint32_t)(KP / 8) * 128u;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, NP);
    const uint32_t a0 = tc::smem_addr(aop), a1 = a0 + (uint32_t)a_half;
    const uint32_t b0 = tc::smem_addr(bop), b1 = b0 + (uint32_t)b_half;
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
      const uint32_t d = taddr + (uint32_t)(mt * NP);
      const uint32_t at = (uint32_t)(tile_row0(mt) / 8) * sbo;
#pragma unroll 1
      for (int ks = 0; ks < KP / 16; ++ks) {
        const uint32_t step = (uint32_t)ks * 256u;
        tc::mma_bf16(d, tc::smem_desc(a0 + at + step, 128, sbo), tc::smem_desc(b0 + step, 128, sbo), idesc, ks > 0);
        tc::mma_bf16(d, tc::smem_desc(a1 + at + step, 128, sbo), tc::smem_desc(b0 + step, 128, sbo), idesc, true);
        tc::mma_bf16(d, tc::smem_desc(a0 + at + step, 128, sbo), tc::smem_desc(b1 + step, 128, sbo), idesc, true);
      }
    }
    tc::mma_commit(mbar);
  }
  // T_r (NOUTR x MR) is read by every output below: fetched into registers
  // while the tensor cores run, staged in the operand-A region once they finish
  constexpr int TRN = NOUTR * MR;
  constexpr int TRP = (TRN + NT - 1) / NT;
  static_assert((size_t)TRN * sizeof(float) <= G::region0, "T_r staging overlaps the product tile");
  const float* trm = LP.r[t.phi];
  float trv[TRP];
#pragma unroll
  for (int i = 0; i < TRP; ++i) trv[i] = (tid + i * NT < TRN) ? __ldg(trm + tid + i * NT) : 0.f;
  bool ok = tc::mbar_wait_bounded(mbar, 0, 1u << 24);
  if (!ok) {
    if (tid == 0) atomicOr(status, tc::kErrMmaTimeout);
    tc::mbar_wait_bounded(mbar, 0, 1u << 24);
  }
  tc::fence_after_sync();
  {
    const int w = tid >> 5, lane = tid & 31;
    if (w < 4 * MT) {
      const int mt = w >> 2, sub = w & 3;
      const int row = tile_row0(mt) + sub * 32 + lane;
#pragma unroll
      for (int c0 = 0; c0 < NP; c0 += 32) {
        float v[32];
        tc::tmem_ld32(taddr + ((uint32_t)(sub * 32) << 16) + (uint32_t)(mt * NP + c0), v);
        if (row < MR)
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (c0 + i < NP) T[row * TLD + c0 + i] = v[i];
      }
    }
  }
  float* trs = reinterpret_cast<float*>(smem);  // the operand-A region: the MMA has finished reading it
#pragma unroll
  for (int i = 0; i < TRP; ++i)
    if (tid + i * NT < TRN) trs[tid + i * NT] = trv[i];
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(taddr, G::TMEM_COLS);

  // ---- S = T_r * T on the FP32 pipe, written to the output channel -----------------
  float* out = L.out + (size_t)(L.img0 + img) * L.out_stride + (size_t)t.out_ch * NOUTR * NOUTC;
  // rows p and p + NOUTR / 2 share their T loads; four independent chains
  constexpr int HR = NOUTR / 2;
  static_assert(NOUTR % 2 == 0 && MR % 4 == 0, "paired rows and 16-byte T_r loads");
  for (int o = tid; o < HR * NOUTC; o += NT) {
    const int p = o / NOUTC, q = o % NOUTC;
    const float4* r0 = reinterpret_cast<const float4*>(trs + p * MR);
    const float4* r1 = reinterpret_cast<const float4*>(trs + (p + HR) * MR);
    float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
#pragma unroll 2
    for (int x4 = 0; x4 < MR / 4; ++x4) {
      const float4 u = r0[x4], w = r1[x4];
      const float* tq = T + 4 * x4 * TLD + q;
      const float t0 = tq[0], t1 = tq[TLD], t2 = tq[2 * TLD], t3 = tq[3 * TLD];
      a0 = fmaf(u.x, t0, a0);
      a1 = fmaf(u.y, t1, a1);
      b0 = fmaf(w.x, t0, b0);
      b1 = fmaf(w.y, t1, b1);
      a0 = fmaf(u.z, t2, a0);
      a1 = fmaf(u.w, t3, a1);
      b0 = fmaf(w.z, t2, b0);
      b1 = fmaf(w.w, t3, b1);
    }
    out[p * NOUTC + q] = ok ? a0 + a1 : __int_as_float(0x7fc00000);
    out[(p + HR) * NOUTC + q] = ok ? b0 + b1 : __int_as_float(0x7fc00000);
  }
}

using TcLauncher = cudaError_t (*)(const CascadeLaunch&, const FilterTable&, const LowpassTable&, unsigned*, int nimg,
                                   cudaStream_t);
void tc_register(int mr, int mc, int nr, int nc, int kf, size_t smem, TcLauncher fn);
bool tc_find(int mr, int mc, int nr, int nc, int kf, size_t* smem, TcLauncher* fn);

template <int MR, int MC, int NOUTR, int NOUTC, int KF, int NT>
cudaError_t tc_launch(const CascadeLaunch& L, const FilterTable& F, const LowpassTable& LP, unsigned* status, int nimg,
                      cudaStream_t stream) {
  using G = TcGeom<MR, MC, NOUTC>;
  auto kern = tc_cascade_kernel<MR, MC, NOUTR, NOUTC, KF, NT>;
  static SmemOptin optin;
  if (cudaError_t e = optin.ensure(kern, (int)G::smem); e != cudaSuccess) return e;
  kern<<<dim3(L.ntasks, nimg, 1), NT, G::smem, stream>>>(L, F, LP, status);
  return cudaGetLastError();
}

template <int MR, int MC, int NOUTR, int NOUTC, int KF, int NT>
struct TcRegistrar {
  TcRegistrar() { tc_register(MR, MC, NOUTR, NOUTC, KF, TcGeom<MR, MC, NOUTC>::smem, &tc_launch<MR, MC, NOUTR, NOUTC, KF, NT>); }
};

#define KYM_TC_VARIANT(MR, MC, NOUTR, NOUTC, KF, NT) \
  static ::kym::TcRegistrar<MR, MC, NOUTR, NOUTC, KF, NT> kym_tc_reg_##MR##_##MC##_##NOUTR##_##NOUTC##_##KF;

}  // namespace kym
