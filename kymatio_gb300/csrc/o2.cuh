// Line-split form of the childless groups whose paths form a P x Q grid
// (P parent spectra x Q wavelets: the L x L order-2 paths of a scale pair
// (j1, j2), or the L order-1 paths of one scale with P = 1), for sizes whose
// tasks read far more source than they compute on.
//
// In the fused task kernels every path folds its own copy of its parent
// spectrum times its wavelet, so a parent row crosses L2 once per child and a
// wavelet row once per parent and image.  Here the first pass folds each
// source row once for the whole group:
//   rows:  one CTA per (child row block, image) computes the folded rows
//          A = fold_k(src_p * psi_q) / k^2 of every path (p, q) of the group
//          from the P source rows and Q wavelet rows it needs (each loaded
//          once and reused from registers), runs their inverse row FFTs and
//          writes them to the paths' slots in the workspace.
// The slots then go through column passes:
//   plain form (the reference's algorithm, lines.cuh): column IFFT, modulus,
//          column FFT; row FFT with the low-pass fold; small IFFT2 -> output.
//   separable form (the low-pass of a childless path as S = T_r U T_c^T,
//          phi being a rank-one outer product; see tc_cascade.cuh):
//          cols:    column IFFT, modulus U, and W = T_r U for the column
//                   block, left in the block's first rows of the slot;
//          lowpass: S = W T_c^T -> output channel.
// A group runs in sub-launches of as many images as keep their slots in L2
// between the passes.  Operations per element and their order are those of
// ct_cascade_kernel / tc_cascade_kernel (kymatio/scattering2d/core/
// scattering2d.py:55-78 restated per path).
#pragma once
#include "lines.cuh"
#include "tc_cascade.cuh"

namespace kym {

constexpr int kO2Lines = 64;  // most folded lines per CTA of the rows pass

// child rows per CTA: the largest divisor of M that keeps P Q rows <= kO2Lines
__host__ __device__ constexpr int o2_rows_per_cta(int m, int pq) {
  int r = 1;
  for (int d = 1; d * pq <= kO2Lines; ++d)
    if (m % d == 0) r = d;
  return r;
}

template <int M, int KF, int P, int Q>
struct O2Geom {
  static constexpr int RPC = o2_rows_per_cta(M, P * Q);  // child rows per CTA
  static constexpr int NL = P * Q * RPC;                 // lines per CTA
  static constexpr int LD = M % 2 == 0 ? M + 1 : M;      // odd pitch
  static constexpr size_t smem = (size_t)NL * LD * sizeof(float2);
  static_assert(NL <= kO2Lines && M % RPC == 0, "rows per CTA");
  static_assert(M % 2 == 0, "paired columns");
};

// ---- rows: shared fold + inverse row FFT -> slots ------------------------------
// Task i = p * Q + q of the group folds source p (tasks[p * Q].src_off) with
// wavelet q (tasks[q].psi); its slot is dst + img * dst_stride +
// tasks[i].dst_off, M x M complex, row-major.  Line l of the CTA is path
// (p, q) at child row u0 + rr with l = (rr * P + p) * Q + q.
template <int M, int KF, int P, int Q, int NT>
__global__ void __launch_bounds__(NT, occupancy_blocks(O2Geom<M, KF, P, Q>::smem, NT) < 3
                                          ? occupancy_blocks(O2Geom<M, KF, P, Q>::smem, NT)
                                          : 3)
    o2_rows_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F) {
  using G = O2Geom<M, KF, P, Q>;
  constexpr int LD = G::LD, RPC = G::RPC;
  constexpr int SCOLS = KF * M;  // source row length
  constexpr int HALF = M / 2;    // column pairs per line
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  __shared__ long long s_src[P];
  __shared__ const float2* s_psi[Q];
  __shared__ long long s_dst[P * Q];
  const int img = blockIdx.y;
  const int u0 = blockIdx.x * RPC;
  for (int i = threadIdx.x; i < P * Q; i += NT) {
    const Task t = L.tasks[i];
    s_dst[i] = t.dst_off;
    if (i % Q == 0) s_src[i / Q] = t.src_off;
    if (i < Q) s_psi[i] = reinterpret_cast<const float2*>(F.f[t.psi]);
  }
  __syncthreads();
  const float2* srcimg = L.src + (size_t)img * L.src_stride;
  const float sc = L.load_scale;
  // item = (child row rr, source p, column pair h); consecutive threads take
  // consecutive column pairs, so every load of a warp is one contiguous run
  for (int it = threadIdx.x; it < RPC * P * HALF; it += NT) {
    const int h = it % HALF;
    const int rp = it / HALF;
    const int p = rp % P, rr = rp / P;
    const int u = u0 + rr, v = 2 * h;
    const float4* s4 = reinterpret_cast<const float4*>(srcimg + s_src[p]);
    float4 acc[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int a = 0; a < KF; ++a) {
#pragma unroll
      for (int b = 0; b < KF; ++b) {
        const size_t half = ((size_t)(u + a * M) * SCOLS + v + b * M) >> 1;
        const float4 x = __ldg(s4 + half);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const float2 f = __ldg(s_psi[q] + half);
          acc[q].x = fmaf(x.x, f.x, acc[q].x);
          acc[q].y = fmaf(x.y, f.x, acc[q].y);
          acc[q].z = fmaf(x.z, f.y, acc[q].z);
          acc[q].w = fmaf(x.w, f.y, acc[q].w);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      float2* row = A + ((rr * P + p) * Q + q) * LD + v;
      row[0] = make_float2(acc[q].x * sc, acc[q].y * sc);
      row[1] = make_float2(acc[q].z * sc, acc[q].w * sc);
    }
  }
  __syncthreads();
  ct::fft_lines<M, G::NL, NT>(ct::RowLines<LD, false>{A}, 0, L.prow.tw, true);
  for (int e = threadIdx.x; e < G::NL * M; e += NT) {
    const int l = e / M, v = e % M;
    const int q = l % Q, rp = l / Q, p = rp % P, rr = rp / P;
    float2* slot = L.dst + (size_t)img * L.dst_stride + s_dst[p * Q + q] + (size_t)(u0 + rr) * M;
    slot[v] = A[l * LD + v];
  }
}

// ---- separable form, cols: column IFFT, modulus, W = T_r U ----------------------
// One CTA per (column block of CB columns, task, image).  W (NOUTR x CB) goes
// to rows 0..NOUTR-1 of the block's own columns of the slot (real part), which
// only this CTA reads or writes.
template <int M, int CB, int NOUTR, int NT>
__global__ void __launch_bounds__(NT, 4)
    o2_cols_sep_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ LowpassTable LP) {
  constexpr int LDC = CB % 2 == 0 ? CB + 1 : CB;
  constexpr int NJ = NT / NOUTR;                 // column groups of the product
  constexpr int JPT = (CB + NJ - 1) / NJ;        // columns per thread
  static_assert(NT % NOUTR == 0 && M % 4 == 0 && NOUTR <= M, "product layout");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  const int c0 = blockIdx.x * CB;
  const Task t = L.tasks[blockIdx.y];
  const int img = blockIdx.z;
  float2* slot = L.dst + (size_t)img * L.dst_stride + t.dst_off + c0;
  for (int e = threadIdx.x; e < M * CB; e += NT) {
    const int r = e / CB, j = e % CB;
    A[r * LDC + j] = slot[(size_t)r * M + j];
  }
  __syncthreads();
  ct::fft_lines<M, CB, NT>(ct::ColLines<LDC>{A}, 0, L.pcol.tw, true);
  // U = |z| in place, in the real part: U[x][j] = A[x * LDC + j].x
  for (int e = threadIdx.x; e < M * CB; e += NT) {
    float2* z = A + (e / CB) * LDC + e % CB;
    const float2 v = *z;
    z->x = sqrtf(fmaf(v.x, v.x, v.y * v.y));
  }
  __syncthreads();
  const float* U = reinterpret_cast<const float*>(A);  // stride 2 floats per element
  const int p = threadIdx.x % NOUTR, jg = threadIdx.x / NOUTR;
  const float4* tr = reinterpret_cast<const float4*>(LP.r[t.phi] + (size_t)p * M);
  float acc[JPT];
#pragma unroll
  for (int k = 0; k < JPT; ++k) acc[k] = 0.f;
#pragma unroll 2
  for (int x4 = 0; x4 < M / 4; ++x4) {
    const float4 w = __ldg(tr + x4);
    const float* u = U + 2 * (4 * x4 * LDC);
#pragma unroll
    for (int k = 0; k < JPT; ++k) {
      const int j = 2 * (jg + k * NJ);
      if (jg + k * NJ < CB) {
        float a = acc[k];
        a = fmaf(w.x, u[j], a);
        a = fmaf(w.y, u[2 * LDC + j], a);
        a = fmaf(w.z, u[4 * LDC + j], a);
        a = fmaf(w.w, u[6 * LDC + j], a);
        acc[k] = a;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < JPT; ++k) {
    const int j = jg + k * NJ;
    if (j < CB) slot[(size_t)p * M + j] = make_float2(acc[k], 0.f);
  }
}

// ---- separable form, lowpass: S = W T_c^T -> output channel ---------------------
template <int M, int NOUTR, int NOUTC, int NT>
__global__ void __launch_bounds__(NT)
    o2_lowpass_sep_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ LowpassTable LP) {
  constexpr int LDW = M + 1;
  __shared__ float W[NOUTR * LDW];
  const Task t = L.tasks[blockIdx.x];
  const int img = blockIdx.y;
  const float2* slot = L.dst + (size_t)img * L.dst_stride + t.dst_off;
  for (int e = threadIdx.x; e < NOUTR * M; e += NT) W[(e / M) * LDW + e % M] = slot[e].x;
  __syncthreads();
  const float* tcm = LP.c[t.phi];
  float* out = L.out + (size_t)(L.img0 + img) * L.out_stride + (size_t)t.out_ch * NOUTR * NOUTC;
  for (int o = threadIdx.x; o < NOUTR * NOUTC; o += NT) {
    const int p = o / NOUTC, q = o % NOUTC;
    const float* w = W + p * LDW;
    const float* c = tcm + (size_t)q * M;
    float a0 = 0.f, a1 = 0.f;
#pragma unroll 4
    for (int x = 0; x < M; x += 2) {
      a0 = fmaf(w[x], __ldg(c + x), a0);
      a1 = fmaf(w[x + 1], __ldg(c + x + 1), a1);
    }
    out[p * NOUTC + q] = a0 + a1;
  }
}

// Launch of one sub-launch of a P x Q group: the rows pass, then the plain
// passes (LP == nullptr) or the separable ones.  L.dst / L.dst_stride: the
// slots; L.bsum_off: the folded low-pass blocks of the plain form, after the
// slots of each image; L.tasks: the group's tasks with their slot offsets.
using O2Launcher = cudaError_t (*)(const CascadeLaunch&, const FilterTable&, const LowpassTable*, int nimg,
                                   cudaStream_t);

template <int M, int KF, int P, int Q, int SR, int SC, int RB, int CB, int NTR, int NTC>
cudaError_t o2_launch(const CascadeLaunch& L, const FilterTable& F, const LowpassTable* LP, int nimg,
                      cudaStream_t stream) {
  using G = O2Geom<M, KF, P, Q>;
  using LG = LinesGeom<M, M, RB, CB>;
  constexpr int NOUTR = SR - 2, NOUTC = SC - 2;
  auto k_rows = o2_rows_kernel<M, KF, P, Q, NTR>;
  static SmemOptin opt_rows;
  cudaError_t e = opt_rows.ensure(k_rows, (int)G::smem);
  if (e != cudaSuccess) return e;
  k_rows<<<dim3(M / G::RPC, nimg, 1), NTR, G::smem, stream>>>(L, F);
  if (LP) {
    o2_cols_sep_kernel<M, CB, NOUTR, NTC><<<dim3(M / CB, L.ntasks, nimg), NTC, LG::col_smem, stream>>>(L, *LP);
    o2_lowpass_sep_kernel<M, NOUTR, NOUTC, 256><<<dim3(L.ntasks, nimg), 256, 0, stream>>>(L, *LP);
  } else {
    constexpr int LDB = SC % 2 == 0 ? SC + 1 : SC;
    constexpr size_t lp_smem = (size_t)SR * LDB * sizeof(float2);
    lines_cols_kernel<M, M, NTC, CB><<<dim3(M / CB, L.ntasks, nimg), NTC, LG::col_smem, stream>>>(L);
    lines_rows_fwd_kernel<M, M, SR, SC, NTC, RB>
        <<<dim3(M / RB, L.ntasks, nimg), NTC, LG::row_smem, stream>>>(L, F);
    lines_lowpass_kernel<M, M, SR, SC, 256><<<dim3(L.ntasks, nimg), 256, lp_smem, stream>>>(L, F);
  }
  return cudaGetLastError();
}

// Registry (ct_registry.cu), keyed by work size, fold, grid and low-pass size.
void o2_register(int m, int kf, int p, int q, int sr, O2Launcher fn);
O2Launcher o2_find(int m, int kf, int p, int q, int sr);

template <int M, int KF, int P, int Q, int SR, int SC, int RB, int CB, int NTR, int NTC>
struct O2Registrar {
  O2Registrar() { o2_register(M, KF, P, Q, SR, &o2_launch<M, KF, P, Q, SR, SC, RB, CB, NTR, NTC>); }
};

#define KYM_O2_VARIANT(M, KF, P, Q, SR, SC, RB, CB, NTR, NTC)                       \
  static ::kym::O2Registrar<M, KF, P, Q, SR, SC, RB, CB, NTR, NTC> kym_o2_reg_##M##_##KF##_##P##_##Q;

}  // namespace kym
