// Hand-written backward of the fused cascade (adjoint of cascade.cu).
//
// Forward of one path, per image (all products pointwise, filters real):
//   Y = fold_k(P * psi) / k^2          P: parent spectrum (or U0^ for order 1)
//   y = IFFT2(Y) (normalised 1/m^2),  U = |y|,  U^ = FFT2(U)
//   S = unpad(Re IFFT2(fold_ks(U^ * phi) / ks^2))
// Adjoints (real inner product on complex vectors):
//   g_B  = FFT2(zeropad(g_S)) / s^2                    (unpad, Re, IFFT2)
//   g_U^ = phi * tile(g_B) / ks^2                      (fold: its adjoint tiles)
//        + sum over children c of psi_c * tile(g_Y_c) / k_c^2
//   g_U  = Re IFFT2u(g_U^)                             (FFT2 of a real signal; IFFT2u unnormalised)
//   g_y  = g_U * y / |y|, 0 where |y| == 0             (ModulusStable.backward,
//                                                       kymatio/backend/torch_backend.py:85-96)
//   g_Y  = FFT2(g_y) / m^2                             (normalised IFFT2)
// which the parent gathers through psi * tile(g_Y) / k^2.  The input stage
// ends with g_x = pad^T Re IFFT2u(g_U0^) (reflect-pad adjoint, a separate
// kernel).  The modulus phase y is recomputed from the parent spectrum.
#pragma once
#include "cascade.cuh"
#include "ct_cascade.cuh"
#include "ct_engine.cuh"

namespace kym {

struct BwdTask {
  long long src_off;  // parent spectrum within one image's block (recomputation)
  long long gy_off;   // this task's gradient block: g_U (real) then g_Y (complex); g_pad at level 0
  int psi;            // wavelet of the recomputation, -1 at level 0
  int phi;            // low-pass filter
  int out_ch;         // channel of the incoming gradient
  int gather_first;   // children in the gather table
  int gather_count;
  int y_off;          // saved modulus input y within one image's saved block (levels 1, 2)
};

struct GatherItem {
  long long gy_off;  // child's g_Y within one image's child block
  int psi;           // child's wavelet at the parent's resolution
  int mr, mc;        // child's work size
  int lkr, lkc;      // log2 of the fold factors parent -> child (powers of two)
  float w;           // 1 / (kr kc)
  int pad_;
  long long gy_pstride;  // parent sets: the same child of the next parent of the set is gy_pstride further
};

struct BwdLaunch {
  int mr, mc, kr, kc, ld, sr, sc, ldb, cluster, rows_local;
  FftPlan prow, pcol, psrow, pscol;
  int level;
  int out_r0, out_c0, out_nr, out_nc, out_channels;
  float rec_scale;  // recomputation load: 1/(kr kc) / (mr mc)
  float gb_scale;   // 1/(sr sc) / (ksr ksc)
  float gy_scale;   // 1/(mr mc)
  const float* gS;
  long long gS_stride;
  const float2* src;
  long long src_stride;
  float2* gy;
  long long gy_stride;
  const float2* gyc;
  long long gyc_stride;
  const BwdTask* tasks;
  int ntasks;
  const GatherItem* gather;
  int img0;
  const float2* tw_rl;  // local column length of a cluster split (mr / cluster)
  const float2* ysaved;  // non-null: y saved by the forward, read instead of recomputed
  long long ysaved_stride;
};

// ---------------------------------------------------------------------------
// FFT engines: compile-time stages or runtime plans, same call surface.
// ---------------------------------------------------------------------------
template <int MR, int MC, int SR, int SC, int C, bool ONED, int NT>
struct CtEngine {
  static constexpr int kC = C, kNT = NT;
  static constexpr bool kOned = ONED;
  static constexpr int RL = MR / C;
  static constexpr int LD = ONED ? MC + (MC >> 4) + 1 : (MC % 2 == 0 ? MC + 1 : MC);
  static constexpr int LDB = ONED ? SC + (SC >> 4) + 1 : (SC % 2 == 0 ? SC + 1 : SC);
  static constexpr size_t smem = ((size_t)RL * LD + (size_t)SR * LDB) * sizeof(float2);
  const BwdLaunch& L;
  float2* A;
  float2* B;
  int rank;
  __device__ int mr() const { return MR; }
  __device__ int mc() const { return MC; }
  __device__ int sr() const { return SR; }
  __device__ int sc() const { return SC; }
  __device__ int ld() const { return LD; }
  __device__ int ldb() const { return LDB; }
  __device__ int rl() const { return RL; }
  static constexpr bool kPerm = (C > 1);  // dif leaves rows permuted across the cluster
  // natural rows in; a cluster leaves row k1 + C k2 at CTA k1, local row k2
  __device__ __forceinline__ void fft2_dif(bool inv) const {
    ct::fft_lines<MC, RL, NT>(ct::RowLines<LD, ONED>{A}, 0, L.prow.tw, inv);
    if constexpr (!ONED) ct_cols<MR, MC, C, LD, NT>(A, rank, L.pcol.tw, L.tw_rl, inv, true);
  }
  // that permuted layout in, natural rows out
  __device__ __forceinline__ void fft2_dit(bool inv) const {
    if constexpr (!ONED) ct_cols<MR, MC, C, LD, NT>(A, rank, L.pcol.tw, L.tw_rl, inv, false);
    ct::fft_lines<MC, RL, NT>(ct::RowLines<LD, ONED>{A}, 0, L.prow.tw, inv);
  }
  __device__ __forceinline__ void small_fft2(bool inv) const {
    ct::fft_lines<SC, SR, NT>(ct::RowLines<LDB, ONED>{B}, 0, L.psrow.tw, inv);
    if constexpr (!ONED) ct::fft_lines<SR, SC, NT>(ct::ColLines<LDB>{B}, 0, L.pscol.tw, inv);
  }
  __device__ __forceinline__ void wide_sync() const {
    if constexpr (C > 1) ct::cluster_sync();
    else __syncthreads();
  }
};

template <bool CL, bool ONED>
struct RtEngine {
  static constexpr int kNT = kThreads;
  static constexpr bool kOned = ONED;
  const BwdLaunch& L;
  float2* A;
  float2* B;
  int rank;
  float2** rowp;
  __device__ int mr() const { return L.mr; }
  __device__ int mc() const { return L.mc; }
  __device__ int sr() const { return L.sr; }
  __device__ int sc() const { return L.sc; }
  __device__ int ld() const { return L.ld; }
  __device__ int ldb() const { return L.ldb; }
  __device__ int rl() const { return L.rows_local; }
  __device__ Slab slab() const {
    Slab w;
    w.local = A;
    w.rowp = rowp;
    w.rows = L.mr;
    w.cols = L.mc;
    w.ld = L.ld;
    w.rows_local = L.rows_local;
    w.row0 = rank * L.rows_local;
    w.nct = L.cluster;
    w.rank = rank;
    return w;
  }
  static constexpr bool kPerm = false;  // runtime plans keep natural rows
  __device__ void fft2(bool inv) const {
    const Slab w = slab();
    fft_pass<true, ONED, false>(w, L.rows_local, 0, L.prow, inv, Barrier{false});
    if constexpr (!ONED) {
      const int cpc = L.mc / L.cluster;
      if constexpr (CL) cg::this_cluster().sync();
      fft_pass<false, false, CL>(w, cpc, rank * cpc, L.pcol, inv, Barrier{CL});
    }
  }
  __device__ void fft2_dif(bool inv) const { fft2(inv); }
  __device__ void fft2_dit(bool inv) const { fft2(inv); }
  __device__ void small_fft2(bool inv) const {
    Slab w;
    w.local = B;
    w.rowp = nullptr;
    w.rows = L.sr;
    w.cols = L.sc;
    w.ld = L.ldb;
    w.rows_local = L.sr;
    w.row0 = 0;
    w.nct = 1;
    w.rank = 0;
    fft_pass<true, ONED, false>(w, L.sr, 0, L.psrow, inv, Barrier{false});
    if constexpr (!ONED) fft_pass<false, false, false>(w, L.sc, 0, L.pscol, inv, Barrier{false});
  }
  __device__ void wide_sync() const {
    if constexpr (CL) cg::this_cluster().sync();
    else __syncthreads();
  }
};

// Loop over n elements, NT threads, with the loads of UNR iterations of a
// thread issued before any of their uses (load(i) -> value, use(i, value)).
template <int UNR, int NT, class LoadF, class UseF>
__device__ __forceinline__ void staged_for(int n, LoadF load, UseF use) {
  using T = decltype(load(0));
  for (int base = 0; base < n; base += NT * UNR) {
    T v[UNR];
#pragma unroll
    for (int k = 0; k < UNR; ++k) {
      const int i = base + threadIdx.x + k * NT;
      if (i < n) v[k] = load(i);
    }
#pragma unroll
    for (int k = 0; k < UNR; ++k) {
      const int i = base + threadIdx.x + k * NT;
      if (i < n) use(i, v[k]);
    }
  }
}

struct PhiPre {
  float f;
  float2 y;
};

// ---------------------------------------------------------------------------
// The backward task kernel body.
// ---------------------------------------------------------------------------
template <class E>
__device__ __forceinline__ void bwd_body(const E& e, const BwdLaunch& L, const FilterTable& F) {
  constexpr bool ONED = E::kOned;
  constexpr int NT = E::kNT;
  const int task_id = blockIdx.x / L.cluster;
  const int img = blockIdx.y;
  const BwdTask t = L.tasks[task_id];
  const int MR = e.mr(), MC = e.mc(), SR = e.sr(), SC = e.sc(), LD = e.ld(), LDB = e.ldb(), RL = e.rl();
  const int row0 = e.rank * RL;
  float2* A = e.A;
  float2* B = e.B;
  auto at = [&](int u, int v) -> float2* {
    if constexpr (ONED) return A + (v + (v >> 4));
    else return A + u * LD + v;
  };
  auto bat = [&](int p, int q) -> float2* {
    if constexpr (ONED) return B + (q + (q >> 4));
    else return B + p * LDB + q;
  };

  // 1. g_B = FFT2(zeropad(g_S)) (scale folded into the tile below)
  const float* gS = L.gS + (size_t)(L.img0 + img) * L.gS_stride + (size_t)t.out_ch * L.out_nr * L.out_nc;
  for (int i = threadIdx.x; i < SR * SC; i += NT) {
    const int p = i / SC, q = i % SC;
    const int pr = p - L.out_r0, qc = q - L.out_c0;
    float g = 0.f;
    if (pr >= 0 && pr < L.out_nr && qc >= 0 && qc < L.out_nc) g = __ldg(gS + pr * L.out_nc + qc);
    *bat(p, q) = make_float2(g, 0.f);
  }
  __syncthreads();
  e.small_fft2(false);

  // 2. g_U^ = phi * tile(g_B) / ks^2 + sum_c psi_c * tile(g_Y_c) / k_c^2
  const float* phi = F.f[t.phi];
  const int nloc = RL * MC;
  // children's contributions, summed beforehand by bwd_gather_kernel into
  // this task's gradient block (complex, full m x m), added after the
  // low-pass term (same order as before: phi term, then the children's sum)
  const float2* pre =
      t.gather_count > 0 ? L.gy + (size_t)img * L.gy_stride + t.gy_off + (size_t)row0 * MC : nullptr;
  staged_for<8, NT>(
      nloc,
      [&](int i) {
        const int u = i / MC, v = i % MC;
        PhiPre r;
        r.f = __ldg(phi + (size_t)(row0 + u) * MC + v);
        r.y = pre ? __ldg(pre + i) : make_float2(0.f, 0.f);
        return r;
      },
      [&](int i, const PhiPre& r) {
        const int u = i / MC, v = i % MC;
        const int gu = row0 + u;
        const float f = r.f * L.gb_scale;
        const float2 b = *bat(gu % SR, v % SC);
        float2 z = make_float2(b.x * f, b.y * f);
        if (pre) {
          z.x += r.y.x;
          z.y += r.y.y;
        }
        *at(u, v) = z;
      });
  __syncthreads();

  // 3. g_U = Re IFFT2u(g_U^)
  e.fft2_dif(true);
  float* gu_base = reinterpret_cast<float*>(L.gy + (size_t)img * L.gy_stride + t.gy_off);
  float* gu_out = gu_base + (size_t)row0 * MC;
  if (L.level == 0) {
    // g_pad in natural rows for the reflect-pad adjoint
    for (int i = threadIdx.x; i < nloc; i += NT) {
      const int u = i / MC, v = i % MC;
      const int grow = E::kPerm ? e.rank + L.cluster * u : row0 + u;
      gu_base[(size_t)grow * MC + v] = at(u, v)->x;
    }
    return;
  }
  // levels 1 and 2 keep g_U in this CTA's (possibly permuted) rows
  for (int i = threadIdx.x; i < nloc; i += NT) gu_out[i] = at(i / MC, i % MC)->x;

  // 4. y = IFFT2(fold(P * psi)) for the modulus phase: saved by the forward
  // (natural rows), or recomputed from the parent spectrum
  __syncthreads();  // g_U stores visible to this CTA before they are re-read in step 5
  if (L.ysaved) {
    const float2* ys = L.ysaved + (size_t)img * L.ysaved_stride + t.y_off;
    staged_for<8, NT>(
        nloc,
        [&](int i) {
          const int u = i / MC, v = i % MC;
          const int grow = E::kPerm ? e.rank + L.cluster * u : row0 + u;
          return __ldg(ys + (size_t)grow * MC + v);
        },
        [&](int i, const float2& y) { *at(i / MC, i % MC) = y; });
    __syncthreads();
  } else {
    const float2* src = L.src + (size_t)img * L.src_stride + t.src_off;
    const float* psi = F.f[t.psi];
    const int scols = L.kc * MC;
    for (int i = threadIdx.x; i < nloc; i += NT) {
      const int u = i / MC, v = i % MC;
      float2 acc = make_float2(0.f, 0.f);
      for (int a = 0; a < L.kr; ++a) {
        const size_t rb = (size_t)(row0 + u + a * MR) * scols + v;
        for (int b = 0; b < L.kc; ++b) {
          const size_t idx = rb + (size_t)b * MC;
          const float2 s = __ldg(src + idx);
          const float w = __ldg(psi + idx);
          acc.x = fmaf(s.x, w, acc.x);
          acc.y = fmaf(s.y, w, acc.y);
        }
      }
      *at(u, v) = cscale(acc, L.rec_scale);
    }
    __syncthreads();
    e.fft2_dif(true);
  }

  // 5. g_y = g_U * y / |y|  (zero where |y| == 0)
  staged_for<8, NT>(
      nloc, [&](int i) { return gu_out[i]; },
      [&](int i, const float& g) {
        float2* p = at(i / MC, i % MC);
        const float2 y = *p;
        const float m = sqrtf(fmaf(y.x, y.x, y.y * y.y));
        *p = (m > 0.f) ? make_float2(g * y.x / m, g * y.y / m) : make_float2(0.f, 0.f);
      });
  __syncthreads();

  // 6. g_Y = FFT2(g_y) / m^2, written over g_U (already consumed)
  e.fft2_dit(false);
  float2* gy_out = L.gy + (size_t)img * L.gy_stride + t.gy_off + (size_t)row0 * MC;
  for (int i = threadIdx.x; i < nloc; i += NT) gy_out[i] = cscale(*at(i / MC, i % MC), L.gy_scale);
}

template <int MR, int MC, int SR, int SC, int C, bool ONED, int NT>
__global__ void __launch_bounds__(NT, occupancy_blocks(CtEngine<MR, MC, SR, SC, C, ONED, NT>::smem, NT))
    ct_bwd_kernel(const __grid_constant__ BwdLaunch L, const __grid_constant__ FilterTable F) {
  using E = CtEngine<MR, MC, SR, SC, C, ONED, NT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  int rank = 0;
  if constexpr (C > 1) rank = static_cast<int>(cg::this_cluster().block_rank());
  const E e{L, A, A + E::RL * E::LD, rank};
  bwd_body(e, L, F);
}

template <bool CL, bool ONED>
__global__ void __launch_bounds__(kThreads, 1)
    rt_bwd_kernel(const __grid_constant__ BwdLaunch L, const __grid_constant__ FilterTable F) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  float2* B = A + (size_t)L.rows_local * L.ld;
  float2** rowp = reinterpret_cast<float2**>(B + (size_t)L.sr * L.ldb);
  int rank = 0;
  if constexpr (CL) {
    cg::cluster_group cl = cg::this_cluster();
    rank = static_cast<int>(cl.block_rank());
    for (int g = threadIdx.x; g < L.mr; g += blockDim.x) {
      const int owner = g / L.rows_local;
      rowp[g] = cl.map_shared_rank(A, owner) + (size_t)(g - owner * L.rows_local) * L.ld;
    }
    __syncthreads();
  }
  const RtEngine<CL, ONED> e{L, A, B, rank, rowp};
  bwd_body(e, L, F);
}

// Children's contributions to a parent's spectrum gradient:
//   out[img][task][u][v] = sum_c psi_c[u][v] * g_Y_c[u mod mr_c][v mod mc_c] / (kr_c kc_c)
// written into each task's gradient block (complex, mr x mc).  One thread
// per column of a strip of kGatherRows rows; grid = (strips x column tiles,
// tasks, images).
constexpr int kGatherRows = 4;
constexpr int kGatherUnroll = 4;  // children whose loads are in flight together
constexpr int kGatherThreads = 256;
constexpr int kGatherLogs = 24;  // fold factors up to 2^23
// Parent sets: NP consecutive tasks whose children use the same wavelets and
// geometry (the L orientations theta1 of one scale j1, whose children are
// the same (j2, theta2) paths) are gathered by one block, so each wavelet
// value is loaded once for the NP parents; strips of kGatherSetRows rows.
constexpr int kGatherSetRows = 2;
// np in {2, 4, 8}; grid = (strips x column tiles, sets, images)
cudaError_t launch_gather_set(int np, dim3 grid, int threads, cudaStream_t stream, const BwdTask* tasks,
                              const GatherItem* gather, const FilterTable& F, int mr, int mc, float2* gy,
                              long long gy_stride, const float2* gyc, long long gyc_stride, int nimg);
__global__ void __launch_bounds__(kGatherThreads) bwd_gather_kernel(const BwdTask* __restrict__ tasks, const GatherItem* __restrict__ gather,
                                  FilterTable F, int mr, int mc, float2* __restrict__ gy, long long gy_stride,
                                  const float2* __restrict__ gyc, long long gyc_stride, int nimg);

// Reflect-pad adjoint: g_x[i][j] = sum of g_pad over the padded positions that
// reflect onto (i, j) (kymatio/scattering2d/backend/torch_backend.py:56-57,
// kymatio/scattering1d/backend/torch_backend.py:75-80).
__global__ void reflect_pad_adjoint_kernel(const float* __restrict__ gpad, long long gpad_stride, int Mp, int Np,
                                           float* __restrict__ gx, int M, int N, int pad_t, int pad_l, int nimg,
                                           int img0);

using BwdCtLauncher = cudaError_t (*)(const BwdLaunch&, const FilterTable&, int nimg, cudaStream_t);
void bwd_ct_register(int mr, int mc, int sr, int sc, int c, bool oned, size_t smem, BwdCtLauncher fn);
bool bwd_ct_find(int mr, int mc, int sr, int sc, int c, bool oned, size_t* smem, BwdCtLauncher* fn);

template <int MR, int MC, int SR, int SC, int C, bool ONED, int NT>
cudaError_t ct_bwd_launch(const BwdLaunch& L, const FilterTable& F, int nimg, cudaStream_t stream) {
  using E = CtEngine<MR, MC, SR, SC, C, ONED, NT>;
  auto kern = ct_bwd_kernel<MR, MC, SR, SC, C, ONED, NT>;
  static SmemOptin optin;
  if (cudaError_t err = optin.ensure(kern, (int)E::smem); err != cudaSuccess) return err;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(L.ntasks * C, nimg, 1);
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = E::smem;
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

template <int MR, int MC, int SR, int SC, int C, bool ONED, int NT>
struct BwdCtRegistrar {
  BwdCtRegistrar() {
    bwd_ct_register(MR, MC, SR, SC, C, ONED, CtEngine<MR, MC, SR, SC, C, ONED, NT>::smem,
                    &ct_bwd_launch<MR, MC, SR, SC, C, ONED, NT>);
  }
};

#define KYM_BWD_VARIANT(MR, MC, SR, SC, C, ONED, NT) \
  static ::kym::BwdCtRegistrar<MR, MC, SR, SC, C, ONED, NT> kym_bwd_reg_##MR##_##MC##_##SR##_##SC##_##C##_##ONED;

}  // namespace kym
