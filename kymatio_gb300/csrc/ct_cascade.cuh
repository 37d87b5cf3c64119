// Compile-time specialised variant of the fused cascade kernel (see
// cascade.cu for the algorithm).  MR x MC is the work size, SR x SC the
// low-pass output size, C the CTAs per task (rows split over a cluster),
// ONED a single row with a swizzled layout, NT the CTA size.
#pragma once
#include "cascade.cuh"
#include "ct_engine.cuh"

namespace kym {

using CtLauncher = cudaError_t (*)(const CascadeLaunch&, const FilterTable&, int nimg, cudaStream_t);

struct CtEntry {
  int mr, mc, sr, sc, c;
  bool oned;
  int kf;  // compile-time fold of the source: -1 runtime, 0 image source, k > 0 fold k x k
  size_t smem;
  CtLauncher fn;
};

// Registry of the instantiated variants (filled by static initialisers).
void ct_register(const CtEntry& e);
// Exact fold variant first, then the runtime-fold variant of the same size.
const CtEntry* ct_find(int mr, int mc, int sr, int sc, int c, bool oned, int kf);

__device__ __forceinline__ int ct_reflect(int i, int n) {
  if (n == 1) return 0;
  const int period = 2 * (n - 1);
  i %= period;
  if (i < 0) i += period;
  return i < n ? i : period - i;
}

// CTAs per SM a kernel's register budget is sized for: as many as 200 KB of
// shared memory holds, keeping at least 64 registers a thread.
__host__ __device__ constexpr int occupancy_blocks(size_t smem, int nt) {
  const int by_smem = (int)((size_t)200 * 1024 / (smem ? smem : 1));
  const int by_regs = 65536 / (nt * 64);
  const int b = by_smem < by_regs ? by_smem : by_regs;
  return b < 1 ? 1 : b;
}

template <int MR, int MC, int SR, int SC, int C, bool ONED, int NT>
struct CtGeom {
  static constexpr int RL = MR / C;                                  // rows per CTA
  static constexpr int LD = ONED ? MC + (MC >> 4) + 1 : (MC % 2 == 0 ? MC + 1 : MC);
  static constexpr int LDB = ONED ? SC + (SC >> 4) + 1 : (SC % 2 == 0 ? SC + 1 : SC);
  static constexpr size_t smem = ((size_t)RL * LD + (size_t)SR * LDB) * sizeof(float2);
  static constexpr int kMinBlocks = occupancy_blocks(smem, NT);
  static_assert(MR % C == 0 && MC % C == 0, "cluster split");
  static_assert(MR % SR == 0 && MC % SC == 0, "low-pass fold");
};

// Load phase of a task: the reflect-padded image (KF == 0), or the fold of
// src * psi over KF x KF aliases (KF > 0, paired float4 loads), or a
// runtime fold (KF < 0).  Writes the local rows of the work array A.
template <int MR, int MC, int C, bool ONED, int NT, int KF, int LD>
__device__ __forceinline__ void ct_load(float2* A, const CascadeLaunch& L, const FilterTable& F, const Task& t,
                                        int img, int row0) {
  constexpr int RL = MR / C;
  auto at = [&](int u, int v) -> float2* {
    if constexpr (ONED) return A + (v + (v >> 4));
    else return A + u * LD + v;
  };
  // ---- load ------------------------------------------------------------------
  constexpr int NLOC = RL * MC;
  if (KF == 0 || (KF < 0 && L.src_image)) {
    const float* x = L.x + (size_t)(L.img0 + img) * L.x_stride;
    for (int e = threadIdx.x; e < NLOC; e += NT) {
      const int u = e / MC, v = e % MC;
      // clusters take the image rows permuted (CTA c, local row u = row c + C u),
      // the layout the split column transform consumes
      const int grow = C > 1 ? row0 / RL + C * u : row0 + u;
      const int iy = ONED ? 0 : ct_reflect(grow - L.pad_t, L.img_M);
      const int ix = ct_reflect(v - L.pad_l, L.img_N);
      *at(u, v) = make_float2(__ldg(x + (size_t)iy * L.img_N + ix) * L.load_scale, 0.f);
    }
  } else if constexpr (KF > 0) {
    // fold KF x KF aliases of src * psi, two adjacent columns per item
    // (float4 / float2 loads: every offset is even because MC is even)
    static_assert(MC % 2 == 0, "paired columns");
    constexpr int KR = ONED ? 1 : KF;
    constexpr int SCOLS = KF * MC;
    const float4* src4 = reinterpret_cast<const float4*>(L.src + (size_t)img * L.src_stride + t.src_off);
    const float2* psi2 = reinterpret_cast<const float2*>(F.f[t.psi]);
    const float sc = L.load_scale;
    if constexpr (!ONED && C == 1 && MR % 2 == 0 && (MR / 2 + 1) * (MC / 2) >= 2 * NT) {
      // The source is the spectrum of a real image, P x Q = KF MR x KF MC:
      // X[P - r][(Q - c) % Q] = conj X[r][c].  The aliases of row u' = MR - u
      // are the mirrors of row u's, (r, c) = (u + a MR, v + b MC), so one pass
      // over row u's source values also gives
      //   Y[u'][(MC - v) % MC] = sum conj X[r][c] psi[P - r][(Q - c) % Q]
      // (and column v + 1 -> MC - 1 - v): half the source loads per output.
      // Rows 0 and MR / 2 are their own mirrors and are folded directly.
      // Taken where the half-size item set still gives every thread two
      // items (68x68 and up at 512 threads); below that, fewer threads with
      // longer load chains measured slower (20x20 and 40x40).
      constexpr int HC = MC / 2, NI = (MR / 2 + 1) * HC, P = KF * MR;
      const float* psi = F.f[t.psi];
#pragma unroll 2
      for (int e = threadIdx.x; e < NI; e += NT) {
        const int u = e / HC, v = 2 * (e % HC);
        const bool pair = u != 0 && u != MR / 2;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f), accp = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int a = 0; a < KF; ++a) {
          const int r = u + a * MR;
#pragma unroll
          for (int b = 0; b < KF; ++b) {
            const int c = v + b * MC;
            const size_t half = ((size_t)r * SCOLS + c) >> 1;
            const float4 s4 = __ldg(src4 + half);
            const float2 f2 = __ldg(psi2 + half);
            acc.x = fmaf(s4.x, f2.x, acc.x);
            acc.y = fmaf(s4.y, f2.x, acc.y);
            acc.z = fmaf(s4.z, f2.y, acc.z);
            acc.w = fmaf(s4.w, f2.y, acc.w);
            if (pair) {
              const float* prow = psi + (size_t)(P - r) * SCOLS;
              const float g0 = __ldg(prow + (c == 0 ? 0 : SCOLS - c));
              const float g1 = __ldg(prow + (SCOLS - 1 - c));
              accp.x = fmaf(s4.x, g0, accp.x);
              accp.y = fmaf(-s4.y, g0, accp.y);
              accp.z = fmaf(s4.z, g1, accp.z);
              accp.w = fmaf(-s4.w, g1, accp.w);
            }
          }
        }
        *at(u, v) = make_float2(acc.x * sc, acc.y * sc);
        *at(u, v + 1) = make_float2(acc.z * sc, acc.w * sc);
        if (pair) {
          *at(MR - u, (MC - v) % MC) = make_float2(accp.x * sc, accp.y * sc);
          *at(MR - u, MC - 1 - v) = make_float2(accp.z * sc, accp.w * sc);
        }
      }
      return;
    }
#pragma unroll 2
    for (int e = threadIdx.x; e < NLOC / 2; e += NT) {
      const int u = (2 * e) / MC, v = (2 * e) % MC;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int a = 0; a < KR; ++a) {
#pragma unroll
        for (int b = 0; b < KF; ++b) {
          const size_t half = ((size_t)(row0 + u + a * MR) * SCOLS + v + b * MC) >> 1;
          const float4 s4 = __ldg(src4 + half);
          const float2 f2 = __ldg(psi2 + half);
          acc.x = fmaf(s4.x, f2.x, acc.x);
          acc.y = fmaf(s4.y, f2.x, acc.y);
          acc.z = fmaf(s4.z, f2.y, acc.z);
          acc.w = fmaf(s4.w, f2.y, acc.w);
        }
      }
      *at(u, v) = make_float2(acc.x * sc, acc.y * sc);
      *at(u, v + 1) = make_float2(acc.z * sc, acc.w * sc);
    }
  } else {
    const float2* src = L.src + (size_t)img * L.src_stride + t.src_off;
    const float* psi = F.f[t.psi];
    const int kr = L.kr, kc = L.kc;
    const int scols = kc * MC;
    for (int e = threadIdx.x; e < NLOC; e += NT) {
      const int u = e / MC, v = e % MC;
      float2 acc = make_float2(0.f, 0.f);
      for (int a = 0; a < kr; ++a) {
        const size_t rb = (size_t)(row0 + u + a * MR) * scols + v;
#pragma unroll 4
        for (int b = 0; b < kc; ++b) {
          const size_t idx = rb + (size_t)b * MC;
          const float2 s = __ldg(src + idx);
          const float f = __ldg(psi + idx);
          acc.x = fmaf(s.x, f, acc.x);
          acc.y = fmaf(s.y, f, acc.y);
        }
      }
      *at(u, v) = cscale(acc, L.load_scale);
    }
  }
}

// Cluster column transforms split as MR = C x RL (C CTAs, RL local rows).
// DIF (natural rows in, CTA c holds rows RL c + n'):
//   X[k1 + C k2] = sum_n' W_RL^{n' k2} [ W_MR^{n' k1} sum_c x[RL c + n'] W_C^{c k1} ]
//   -> cross-CTA radix-C step (CTA k1 forms the bracket), then a local
//      RL-point FFT; CTA k1 ends with rows k1 + C k2 at local row k2.
// DIT (that permuted layout in):
//   X[k2 + RL k1] = sum_c W_C^{c k1} W_MR^{c k2} sum_g W_RL^{g k2} x[c + C g]
//   -> local RL-point FFT, then the cross-CTA step; CTA k1 ends with the
//      natural rows RL k1 + k2.
// Every remote element is read once; the in-place cross step runs in
// rounds with a cluster barrier between a round's reads and its writes.
template <int MR, int MC, int C, int LD, int NT, bool DIT>
__device__ __forceinline__ void ct_cross(float2* A, int rank, const float2* __restrict__ tw, bool inv) {
  constexpr int RL = MR / C;
  constexpr int NEL = RL * MC;
  constexpr int PER = 8;
  constexpr int ROUNDS = (NEL + NT * PER - 1) / (NT * PER);
  const uint32_t base = ct::smem_u32(A);
  float2 wc[C];  // W_C^{c rank}
#pragma unroll
  for (int c = 0; c < C; ++c) wc[c] = conj_if(__ldg(tw + ((c * rank) % C) * RL), inv);
#pragma unroll 1
  for (int rd = 0; rd < ROUNDS; ++rd) {
    float2 acc[PER];
#pragma unroll
    for (int it = 0; it < PER; ++it) {
      const int e = threadIdx.x + (rd * PER + it) * NT;
      acc[it] = make_float2(0.f, 0.f);
      if (e < NEL) {
        const int n = e / MC, col = e % MC;
        const uint32_t off = base + (uint32_t)((n * LD + col) * 8);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const float2 x = (c == rank) ? A[n * LD + col] : ct::ld_dsmem(ct::mapa(off, (uint32_t)c));
          float2 w = wc[c];
          if (DIT) w = cmul(w, conj_if(__ldg(tw + (c * n) % MR), inv));
          acc[it] = cadd(acc[it], cmul(x, w));
        }
        if (!DIT) acc[it] = cmul(acc[it], conj_if(__ldg(tw + (n * rank) % MR), inv));
      }
    }
    ct::cluster_sync();  // every CTA has read this round's elements
#pragma unroll
    for (int it = 0; it < PER; ++it) {
      const int e = threadIdx.x + (rd * PER + it) * NT;
      if (e < NEL) A[(e / MC) * LD + (e % MC)] = acc[it];
    }
  }
  __syncthreads();
}

// Column pass of the work array: local (C == 1) or split over the cluster.
// dif: natural rows in, permuted out (C > 1); !dif: permuted in, natural out.
template <int MR, int MC, int C, int LD, int NT>
__device__ __forceinline__ void ct_cols(float2* A, int rank, const float2* tw, const float2* tw_rl, bool inv,
                                        bool dif) {
  if constexpr (C == 1) {
    ct::fft_lines<MR, MC, NT>(ct::ColLines<LD>{A}, 0, tw, inv);
  } else {
    constexpr int RL = MR / C;
    ct::cluster_sync();  // rows of every CTA complete
    if (dif) {
      ct_cross<MR, MC, C, LD, NT, false>(A, rank, tw, inv);
      ct::fft_lines<RL, MC, NT>(ct::ColLines<LD>{A}, 0, tw_rl, inv);
    } else {
      ct::fft_lines<RL, MC, NT>(ct::ColLines<LD>{A}, 0, tw_rl, inv);
      ct::cluster_sync();
      ct_cross<MR, MC, C, LD, NT, true>(A, rank, tw, inv);
    }
  }
}

template <int MR, int MC, int SR, int SC, int C, bool ONED, int NT, int KF>
__global__ void __launch_bounds__(NT, (CtGeom<MR, MC, SR, SC, C, ONED, NT>::kMinBlocks))
    ct_cascade_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F) {
  using G = CtGeom<MR, MC, SR, SC, C, ONED, NT>;
  constexpr int RL = G::RL, LD = G::LD, LDB = G::LDB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  float2* B = A + RL * LD;
  int rank = 0;
  if constexpr (C > 1) rank = static_cast<int>(cg::this_cluster().block_rank());
  const int task_id = blockIdx.x / C;
  const int img = blockIdx.y;
  const Task t = L.tasks[task_id];
  const int row0 = rank * RL;

  auto at = [&](int u, int v) -> float2* {
    if constexpr (ONED) return A + (v + (v >> 4));
    else return A + u * LD + v;
  };

  ct_load<MR, MC, C, ONED, NT, KF, LD>(A, L, F, t, img, row0);
  __syncthreads();
  constexpr int NLOC = RL * MC;

  const ct::RowLines<LD, ONED> rows{A};
  if (KF != 0 && L.modulus) {
    // U = |IFFT2(A)| ; A = FFT2(U)  (a cluster leaves U in permuted rows)
    ct::fft_lines<MC, RL, NT>(rows, 0, L.prow.tw, true);
    if constexpr (!ONED) ct_cols<MR, MC, C, LD, NT>(A, rank, L.pcol.tw, L.tw_rl, true, true);
    // y saved for the backward in natural rows (a cluster holds row rank + C u)
    float2* ys = (L.ysave && t.y_off >= 0) ? L.ysave + (size_t)img * L.ysave_stride + t.y_off : nullptr;
    if constexpr (C == 1 && !ONED && MR % 2 == 0 && MC % 2 == 0) {
      // FFT2 of the real U: the column FFT runs two columns per complex line,
      // Z = U[:, 2j] + i U[:, 2j+1] in column j; the unpacked columns
      // X_2j[k] = (Z_k + conj Z_-k) / 2, X_2j+1[k] = -i (Z_k - conj Z_-k) / 2
      // are Hermitian in k to the bit, so the row FFTs of rows 0 .. MR/2 give
      // the rest as F[MR - k][v] = conj F[k][(MC - v) % MC].  In-place
      // rewrites read into registers, then write after a barrier.
      constexpr int HC = MC / 2, HR = MR / 2;
      constexpr int NPAIR = MR * HC, PP = (NPAIR + NT - 1) / NT;
      float2 m[PP];
#pragma unroll
      for (int i = 0; i < PP; ++i) {
        const int e = threadIdx.x + i * NT;
        if (e < NPAIR) {
          const int r = e / HC, j = e % HC;
          const float2 z0 = A[r * LD + 2 * j], z1 = A[r * LD + 2 * j + 1];
          if (ys) {  // saved for the backward
            ys[(size_t)r * MC + 2 * j] = z0;
            ys[(size_t)r * MC + 2 * j + 1] = z1;
          }
          m[i] = make_float2(sqrtf(fmaf(z0.x, z0.x, z0.y * z0.y)), sqrtf(fmaf(z1.x, z1.x, z1.y * z1.y)));
        }
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < PP; ++i) {
        const int e = threadIdx.x + i * NT;
        if (e < NPAIR) A[(e / HC) * LD + e % HC] = m[i];
      }
      __syncthreads();
      ct::fft_lines<MR, HC, NT>(ct::ColLines<LD>{A}, 0, L.pcol.tw, false);
      constexpr int NU = (HR + 1) * HC, PU = (NU + NT - 1) / NT;
      float2 za[PU], zb[PU];
#pragma unroll
      for (int i = 0; i < PU; ++i) {
        const int e = threadIdx.x + i * NT;
        if (e < NU) {
          const int k = e / HC, j = e % HC;
          za[i] = A[k * LD + j];
          zb[i] = A[((MR - k) % MR) * LD + j];
        }
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < PU; ++i) {
        const int e = threadIdx.x + i * NT;
        if (e < NU) {
          const int k = e / HC, j = e % HC, km = (MR - k) % MR;
          const float2 a = za[i], b = zb[i];
          const float2 x0 = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
          const float2 x1 = make_float2(0.5f * (a.y + b.y), 0.5f * (b.x - a.x));
          A[k * LD + 2 * j] = x0;
          A[k * LD + 2 * j + 1] = x1;
          if (km != k) {
            A[km * LD + 2 * j] = make_float2(x0.x, -x0.y);
            A[km * LD + 2 * j + 1] = make_float2(x1.x, -x1.y);
          }
        }
      }
      __syncthreads();
      ct::fft_lines<MC, HR + 1, NT>(rows, 0, L.prow.tw, false);
      for (int e = threadIdx.x; e < (MR - HR - 1) * MC; e += NT) {
        const int r = HR + 1 + e / MC, v = e % MC;
        const float2 z = A[(MR - r) * LD + (MC - v) % MC];
        A[r * LD + v] = make_float2(z.x, -z.y);
      }
      __syncthreads();
    } else {
      for (int e = threadIdx.x; e < NLOC; e += NT) {
        float2* p = at(e / MC, e % MC);
        const float2 z = *p;
        if (ys) ys[(size_t)(C > 1 ? rank + C * (e / MC) : e / MC) * MC + e % MC] = z;
        *p = make_float2(sqrtf(fmaf(z.x, z.x, z.y * z.y)), 0.f);
      }
      __syncthreads();
      if constexpr (!ONED) ct_cols<MR, MC, C, LD, NT>(A, rank, L.pcol.tw, L.tw_rl, false, false);
      ct::fft_lines<MC, RL, NT>(rows, 0, L.prow.tw, false);
    }
  } else {
    // the input stage: natural rows for one CTA, permuted rows for a cluster
    ct::fft_lines<MC, RL, NT>(rows, 0, L.prow.tw, false);
    if constexpr (!ONED) ct_cols<MR, MC, C, LD, NT>(A, rank, L.pcol.tw, L.tw_rl, false, false);
  }

  // ---- parent spectrum for the next order --------------------------------------
  if (t.dst_off >= 0) {
    float2* dst = L.dst + (size_t)img * L.dst_stride + t.dst_off + (size_t)row0 * MC;
    for (int e = threadIdx.x; e < NLOC; e += NT) dst[e] = *at(e / MC, e % MC);
  }

  if (L.skip_s) return;  // no remote shared-memory access follows the last cluster barrier

  // ---- low-pass: partial fold over local rows --------------------------------------
  constexpr int KSR = MR / SR, KSC = MC / SC;
  const float* phi = F.f[t.phi];
  for (int e = threadIdx.x; e < SR * SC; e += NT) {
    const int p = e / SC, q = e % SC;
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int a = 0; a < KSR; ++a) {
      const int g = p + a * SR;
      if (C > 1 && (g < row0 || g >= row0 + RL)) continue;
#pragma unroll
      for (int b = 0; b < KSC; ++b) {
        const int col = q + b * SC;
        const float2 z = *at(g - row0, col);
        const float f = __ldg(phi + (size_t)g * MC + col);
        acc.x = fmaf(z.x, f, acc.x);
        acc.y = fmaf(z.y, f, acc.y);
      }
    }
    float2* bp = ONED ? B + (q + (q >> 4)) : B + p * LDB + q;
    *bp = cscale(acc, L.s_scale);
  }
  if constexpr (C > 1) {
    ct::cluster_sync();
    if (rank == 0) {
      for (int e = threadIdx.x; e < SR * SC; e += NT) {
        float2* bp = B + (e / SC) * LDB + (e % SC);
        float2 acc = *bp;
        const uint32_t a = ct::smem_u32(bp);
#pragma unroll
        for (int r = 1; r < C; ++r) acc = cadd(acc, ct::ld_dsmem(ct::mapa(a, r)));
        *bp = acc;
      }
    }
    ct::cluster_sync();
    if (rank != 0) return;
  }
  __syncthreads();

  // ---- small inverse transform, real part, unpad ------------------------------------
  const ct::RowLines<LDB, ONED> brows{B};
  ct::fft_lines<SC, SR, NT>(brows, 0, L.psrow.tw, true);
  if constexpr (!ONED) {
    const ct::ColLines<LDB> bcols{B};
    ct::fft_lines<SR, SC, NT>(bcols, 0, L.pscol.tw, true);
  }
  float* out = L.out + (size_t)(L.img0 + img) * L.out_stride + (size_t)t.out_ch * L.out_nr * L.out_nc;
  for (int e = threadIdx.x; e < L.out_nr * L.out_nc; e += NT) {
    const int p = e / L.out_nc + L.out_r0, q = e % L.out_nc + L.out_c0;
    const float2* bp = ONED ? B + (q + (q >> 4)) : B + p * LDB + q;
    out[e] = bp->x;
  }
}

template <int MR, int MC, int SR, int SC, int C, bool ONED, int NT, int KF>
cudaError_t ct_launch(const CascadeLaunch& L, const FilterTable& F, int nimg, cudaStream_t stream) {
  using G = CtGeom<MR, MC, SR, SC, C, ONED, NT>;
  auto kern = ct_cascade_kernel<MR, MC, SR, SC, C, ONED, NT, KF>;
  static SmemOptin optin;
  if (cudaError_t e = optin.ensure(kern, (int)G::smem); e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(L.ntasks * C, nimg, 1);
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = G::smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  cfg.attrs = attr;
  cfg.numAttrs = 0;
  if (C > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kern, L, F);
}

template <int MR, int MC, int SR, int SC, int C, bool ONED, int NT, int KF>
struct CtRegistrar {
  CtRegistrar() {
    using G = CtGeom<MR, MC, SR, SC, C, ONED, NT>;
    ct_register(CtEntry{MR, MC, SR, SC, C, ONED, KF, G::smem, &ct_launch<MR, MC, SR, SC, C, ONED, NT, KF>});
  }
};

// A size with a runtime fold (any source), plus compile-time folds.
#define KYM_CT_VARIANT(MR, MC, SR, SC, C, ONED, NT) \
  static ::kym::CtRegistrar<MR, MC, SR, SC, C, ONED, NT, -1> kym_ct_reg_##MR##_##MC##_##SR##_##SC##_##C##_##ONED;
#define KYM_CT_FOLD(MR, MC, SR, SC, C, ONED, NT, KF) \
  static ::kym::CtRegistrar<MR, MC, SR, SC, C, ONED, NT, KF>  \
      kym_ct_regf_##MR##_##MC##_##SR##_##SC##_##C##_##ONED##_##KF;

}  // namespace kym
