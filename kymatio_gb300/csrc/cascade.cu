// Fused scattering cascade kernels, their host-side plans and the C ABI of
// the forward transforms (include/kymatio_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include "../../include/kymatio_gb300.h"
#include "cascade.cuh"
#include "ct_cascade.cuh"
#include "bwd.cuh"
#include "tcdft.cuh"
#include "lines.cuh"
#include "plan_util.h"
#include "errors.h"

namespace kym {

__device__ __forceinline__ int reflect_idx(int i, int n) {
  if (n == 1) return 0;
  const int period = 2 * (n - 1);
  i %= period;
  if (i < 0) i += period;
  return i < n ? i : period - i;
}

// ---------------------------------------------------------------------------
// The fused task kernel.  grid = (ntasks * cluster, images), cluster = (C,1,1)
// CL: the work array is split over a cluster.  ONED: a single row (1-D).
// ---------------------------------------------------------------------------
template <bool CL, bool ONED>
__global__ void __launch_bounds__(kThreads, 1)
    cascade_kernel(const __grid_constant__ CascadeLaunch L, const __grid_constant__ FilterTable F) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  const int C = CL ? L.cluster : 1;
  int rank = 0;
  if constexpr (CL) rank = static_cast<int>(cg::this_cluster().block_rank());
  const int task_id = blockIdx.x / C;
  const int img = blockIdx.y;
  const Task t = L.tasks[task_id];
  const int rl = L.rows_local;
  const int row0 = rank * rl;
  const int mc = L.mc;
  float2* B = A + (size_t)rl * L.ld;
  float2** rowp = reinterpret_cast<float2**>(B + (size_t)L.sr * L.ldb);

  Slab w;
  w.local = A;
  w.rowp = rowp;
  w.rows = L.mr;
  w.cols = mc;
  w.ld = L.ld;
  w.rows_local = rl;
  w.row0 = row0;
  w.nct = C;
  w.rank = rank;
  const Barrier local_bar{false};
  const Barrier wide_bar{CL};

  if constexpr (CL) {
    cg::cluster_group cl = cg::this_cluster();
    for (int g = threadIdx.x; g < L.mr; g += blockDim.x) {
      const int owner = g / rl;
      float2* base = cl.map_shared_rank(A, owner);
      rowp[g] = base + (size_t)(g - owner * rl) * L.ld;
    }
  }

  auto elem = [&](int u, int v) -> float2* {
    if constexpr (ONED) return A + (v + (v >> 4));
    else return A + (size_t)u * L.ld + v;
  };

  // ---- load: reflect-padded image, or fold(src * psi) -----------------------
  const int nloc = rl * mc;
  if (L.src_image) {
    const float* x = L.x + (size_t)(L.img0 + img) * L.x_stride;
    for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
      const int u = e / mc, v = e - (e / mc) * mc;
      const int iy = ONED ? 0 : reflect_idx(row0 + u - L.pad_t, L.img_M);
      const int ix = reflect_idx(v - L.pad_l, L.img_N);
      *elem(u, v) = make_float2(__ldg(x + (size_t)iy * L.img_N + ix) * L.load_scale, 0.f);
    }
  } else {
    const float2* src = L.src + (size_t)img * L.src_stride + t.src_off;
    const float* psi = t.psi >= 0 ? F.f[t.psi] : nullptr;
    const int scols = L.kc * mc;
    for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
      const int u = e / mc, v = e - (e / mc) * mc;
      const int gu = row0 + u;
      float2 acc = make_float2(0.f, 0.f);
      for (int a = 0; a < L.kr; ++a) {
        const size_t rbase = (size_t)(gu + a * L.mr) * scols + v;
        for (int b = 0; b < L.kc; ++b) {
          const size_t idx = rbase + (size_t)b * mc;
          const float2 s = __ldg(src + idx);
          const float f = psi ? __ldg(psi + idx) : 1.f;
          acc.x = fmaf(s.x, f, acc.x);
          acc.y = fmaf(s.y, f, acc.y);
        }
      }
      *elem(u, v) = cscale(acc, L.load_scale);
    }
  }
  __syncthreads();

  const int cpc = mc / C;  // columns handled by this CTA in column passes
  if (L.modulus) {
    // U = |IFFT2(A)| ; A = FFT2(U)
    fft_pass<true, ONED, false>(w, rl, 0, L.prow, true, local_bar);
    if constexpr (!ONED) {
      if constexpr (CL) cg::this_cluster().sync();
      fft_pass<false, false, CL>(w, cpc, rank * cpc, L.pcol, true, wide_bar);
    }
    float2* ys = (L.ysave && t.y_off >= 0) ? L.ysave + (size_t)img * L.ysave_stride + t.y_off : nullptr;
    for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
      const int u = e / mc, v = e - (e / mc) * mc;
      float2* p = elem(u, v);
      const float2 z = *p;
      if (ys) ys[(size_t)(row0 + u) * mc + v] = z;  // saved for the backward
      *p = make_float2(sqrtf(z.x * z.x + z.y * z.y), 0.f);
    }
    if constexpr (!ONED) {
      wide_bar.sync();
      fft_pass<false, false, CL>(w, cpc, rank * cpc, L.pcol, false, wide_bar);
    } else {
      __syncthreads();
    }
    fft_pass<true, ONED, false>(w, rl, 0, L.prow, false, local_bar);
  } else {
    fft_pass<true, ONED, false>(w, rl, 0, L.prow, false, local_bar);
    if constexpr (!ONED) {
      if constexpr (CL) cg::this_cluster().sync();
      fft_pass<false, false, CL>(w, cpc, rank * cpc, L.pcol, false, wide_bar);
    }
  }

  // ---- store the spectrum for the next order --------------------------------
  if (t.dst_off >= 0) {
    float2* dst = L.dst + (size_t)img * L.dst_stride + t.dst_off + (size_t)row0 * mc;
    for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
      const int u = e / mc, v = e - (e / mc) * mc;
      dst[e] = *elem(u, v);
    }
  }

  if (L.skip_s) return;  // no remote shared-memory access follows the last cluster barrier

  // ---- low-pass branch: B = fold(A * phi) (partial over local rows) --------
  const float* phi = F.f[t.phi];
  const int sr = L.sr, sc = L.sc;
  const int ksr = L.mr / sr, ksc = mc / sc;
  for (int e = threadIdx.x; e < sr * sc; e += blockDim.x) {
    const int p = e / sc, q = e - (e / sc) * sc;
    float2 acc = make_float2(0.f, 0.f);
    for (int a = 0; a < ksr; ++a) {
      const int g = p + a * sr;
      if (g < row0 || g >= row0 + rl) continue;
      for (int b = 0; b < ksc; ++b) {
        const int col = q + b * sc;
        const float2 z = *elem(g - row0, col);
        const float f = __ldg(phi + (size_t)g * mc + col);
        acc.x = fmaf(z.x, f, acc.x);
        acc.y = fmaf(z.y, f, acc.y);
      }
    }
    float2* bp = ONED ? B + (q + (q >> 4)) : B + (size_t)p * L.ldb + q;
    *bp = cscale(acc, L.s_scale);
  }
  if constexpr (CL) {
    cg::cluster_group cl = cg::this_cluster();
    cl.sync();
    if (rank == 0) {
      for (int e = threadIdx.x; e < sr * sc; e += blockDim.x) {
        const int p = e / sc, q = e - (e / sc) * sc;
        float2* bp = B + (size_t)p * L.ldb + q;
        float2 acc = *bp;
        for (int r = 1; r < C; ++r) acc = cadd(acc, *cl.map_shared_rank(bp, r));
        *bp = acc;
      }
    }
    cl.sync();
    if (rank != 0) return;
  }
  __syncthreads();

  // ---- small inverse transform and unpadded real output ---------------------
  Slab wb;
  wb.local = B;
  wb.rowp = nullptr;
  wb.rows = sr;
  wb.cols = sc;
  wb.ld = L.ldb;
  wb.rows_local = sr;
  wb.row0 = 0;
  wb.nct = 1;
  wb.rank = 0;
  fft_pass<true, ONED, false>(wb, sr, 0, L.psrow, true, local_bar);
  if constexpr (!ONED) fft_pass<false, false, false>(wb, sc, 0, L.pscol, true, local_bar);

  float* out = L.out + (size_t)(L.img0 + img) * L.out_stride + (size_t)t.out_ch * L.out_nr * L.out_nc;
  for (int e = threadIdx.x; e < L.out_nr * L.out_nc; e += blockDim.x) {
    const int p = e / L.out_nc + L.out_r0, q = e % L.out_nc + L.out_c0;
    const float2* bp = ONED ? B + (q + (q >> 4)) : B + (size_t)p * L.ldb + q;
    out[e] = bp->x;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

namespace {

struct Group {
  CascadeLaunch L;       // pointers filled at launch
  bool has_ct = false;   // a compile-time specialised variant exists
  CtEntry ct{};
  bool has_tc = false;   // a tensor-core variant exists (childless tasks only)
  bool tc_on = true;     // kym_s2d_forward_tc uses it (kym_s2d_set_group_tc)
  size_t tc_smem = 0;
  TcLauncher tc = nullptr;
  TcLauncher tcdft = nullptr;     // DFT-GEMM tensor-core variant (childless tasks of the small sizes)
  LinesLauncher lines = nullptr;  // line-split passes (sizes above one CTA, every task owns a slot)
  std::vector<Task> tasks;
  size_t task_off = 0;   // offset into the device task array
  size_t smem = 0;
  bool oned = false;
  int level = 0;         // 0: input stage, 1: order 1, 2: order 2
  std::vector<std::pair<int, int>> out_runs;  // output channels it writes, as runs [first, end)
  int lane = 0;          // 0: the caller's stream, 1: the plan's side stream
};

int odd_pitch(int n) { return (n % 2 == 0) ? n + 1 : n; }
std::atomic<bool> g_use_ct{true};
std::atomic<bool> g_use_tcdft{false};
std::atomic<bool> g_use_side{true};
int swz_len(int n) { return n + (n >> 4) + 1; }

}  // namespace

struct DeviceState {
  Task* tasks = nullptr;
  float2* tw = nullptr;
  BwdTask* btasks = nullptr;
  GatherItem* gather = nullptr;
  // host transfers of kym_s2d_forward_host: input; output of the groups of
  // each launch lane (a lane's copies wait only for its own groups)
  cudaStream_t copy_in = nullptr, copy_out = nullptr, copy_out_side = nullptr;
  cudaStream_t side = nullptr;  // second lane of the forward's independent group chains
};

// Backward launch group: mirrors one forward group's geometry.
struct BwdGroup {
  int fwd = 0;                 // index of the forward group it mirrors
  int level = 0;
  std::vector<BwdTask> tasks;
  size_t task_off = 0;
  bool has_ct = false;
  size_t smem = 0;             // shared memory of the launched variant
  BwdCtLauncher ct = nullptr;
  int gather_np = 1;           // parents per gather block (sets of tasks sharing their children's wavelets)
};

struct CascadePlan {
  // geometry
  bool oned = false;
  int M = 0, N = 0, J = 0, L = 0, max_order = 2, pre_pad = 0;
  int Mp = 0, Np = 0;
  int channels = 0, out_nr = 0, out_nc = 0;
  int img_M = 0, img_N = 0, pad_t = 0, pad_l = 0;
  std::vector<int> filter_rows, filter_cols;  // expected filter shapes, by index
  long long u0_elems = 0;                     // per image
  long long u1_elems = 0;                     // per image
  size_t opnd_bytes = 0;                      // per image: DFT-GEMM operand slots of the largest such group
  int chunk = 0;
  std::vector<Group> groups;
  // launch order of the groups: the input stage, the order-1 groups that
  // store parent spectra, the order-2 groups, then the childless order-1
  // groups (they depend on nothing later, and a short group last leaves
  // little output to copy after the cascade in kym_s2d_forward_host)
  std::vector<int> order;
  std::vector<Task> all_tasks;
  // backward
  std::vector<BwdGroup> bgroups;
  std::vector<BwdTask> all_btasks;
  std::vector<GatherItem> all_gather;
  long long gy1_elems = 0, gy2_elems = 0;  // per image: order-1 / order-2 gradient blocks (complex)
  int bchunk = 0;
  TwiddleBank tw;
  std::mutex mu;                     // guards `dev` and `scratch_tables`
  std::map<int, DeviceState> dev;    // task and twiddle tables, per device
  // host image of the task and twiddle tables as the allocation-free forward
  // lays them out at the head of its scratch array; built on its first call
  // and kept for the plan's lifetime, so a copy from it never outlives it
  std::vector<unsigned char> scratch_tables;
  ~CascadePlan() {
    int cur = 0;
    const bool have = cudaGetDevice(&cur) == cudaSuccess;
    for (auto& kv : dev) {
      if (cudaSetDevice(kv.first) != cudaSuccess) continue;
      cudaFree(kv.second.tasks);
      cudaFree(kv.second.tw);
      cudaFree(kv.second.btasks);
      cudaFree(kv.second.gather);
      if (kv.second.copy_in) cudaStreamDestroy(kv.second.copy_in);
      if (kv.second.copy_out) cudaStreamDestroy(kv.second.copy_out);
      if (kv.second.copy_out_side) cudaStreamDestroy(kv.second.copy_out_side);
      if (kv.second.side) cudaStreamDestroy(kv.second.side);
    }
    if (have) cudaSetDevice(cur);
    cudaGetLastError();
  }
};

static int fail_cuda(cudaError_t e, const char* what) {
  set_error_message(what, cudaGetErrorString(e));
  return KYM_ERR_CUDA;
}

// Host-side finalisation: task offsets into one concatenated table.
static int finalize_groups(CascadePlan* P) {
  size_t total = 0;
  for (auto& g : P->groups) {
    // the line-split passes work in each task's spectrum slot
    for (const Task& t : g.tasks)
      if (t.dst_off < 0) g.lines = nullptr;
    g.task_off = total;
    total += g.tasks.size();
  }
  // the folded low-pass blocks of a line-split order-1 group sit after each
  // image's parent spectra, one region per such group (groups of different
  // launch lanes may run at the same time)
  long long lp = 0;
  for (auto& g : P->groups) {
    g.L.bsum_off = -1;
    if (g.lines && g.L.modulus && g.level == 1) {
      g.L.bsum_off = P->u1_elems + lp;
      lp += (long long)g.tasks.size() * g.L.sr * g.L.sc;
    }
  }
  P->u1_elems += lp;
  // per-image strides stay even (16-byte aligned complex64 pairs): bulk copies
  // of source rows read from them
  P->u0_elems += P->u0_elems & 1;
  P->u1_elems += P->u1_elems & 1;
  P->all_tasks.clear();
  for (auto& g : P->groups) P->all_tasks.insert(P->all_tasks.end(), g.tasks.begin(), g.tasks.end());
  // output channel runs, and the launch order
  for (auto& g : P->groups) {
    std::vector<int> ch;
    for (const Task& t : g.tasks)
      if (t.out_ch >= 0) ch.push_back(t.out_ch);
    std::sort(ch.begin(), ch.end());
    ch.erase(std::unique(ch.begin(), ch.end()), ch.end());
    g.out_runs.clear();
    for (size_t i = 0; i < ch.size(); ++i) {
      if (!g.out_runs.empty() && g.out_runs.back().second == ch[i]) ++g.out_runs.back().second;
      else g.out_runs.push_back({ch[i], ch[i] + 1});
    }
  }
  auto childless = [](const Group& g) {
    for (const Task& t : g.tasks)
      if (t.dst_off >= 0) return false;
    return true;
  };
  // launch lanes: an order-1 group and the order-2 groups reading its parent
  // spectra form a chain; the heaviest chain runs on the caller's stream,
  // the other chains with children on a side stream, where their blocks fill
  // the SMs the first chain leaves idle (its tails and narrow launches).  The
  // childless order-1 groups stay on the caller's stream, last: a short group
  // ends the forward, so little output is left to copy after the cascade
  // (kym_s2d_forward_host)
  {
    const int ng = (int)P->groups.size();
    std::vector<int> chain(ng, -1);
    for (int i = 0; i < ng; ++i)
      if (P->groups[i].level == 1) chain[i] = i;
    for (int i = 0; i < ng; ++i) {
      const Group& g = P->groups[i];
      if (g.level != 2 || g.tasks.empty()) continue;
      const long long src = g.tasks[0].src_off;
      for (int k = 0; k < ng && chain[i] < 0; ++k)
        if (P->groups[k].level == 1)
          for (const Task& t : P->groups[k].tasks)
            if (t.dst_off == src) {
              chain[i] = k;
              break;
            }
    }
    std::vector<double> weight(ng, 0.0);
    for (int i = 0; i < ng; ++i) {
      const Group& g = P->groups[i];
      if (chain[i] < 0) continue;
      const double area = (double)g.L.mr * g.L.mc;
      weight[chain[i]] += (double)g.tasks.size() * area * (std::log2(std::max(2.0, area)) + g.L.kr * g.L.kc);
    }
    int heavy = -1;
    for (int i = 0; i < ng; ++i)
      if (P->groups[i].level == 1 && (heavy < 0 || weight[i] > weight[heavy])) heavy = i;
    for (int i = 0; i < ng; ++i) {
      Group& g = P->groups[i];
      g.lane = (chain[i] >= 0 && chain[i] != heavy && !(g.level == 1 && childless(g))) ? 1 : 0;
    }
    for (int i = 0; i < ng; ++i)
      if (P->groups[i].level == 2 && chain[i] < 0) {
        for (auto& g : P->groups) g.lane = 0;  // unknown dependencies: one lane
        break;
      }
  }
  P->order.clear();
  for (int cls = 0; cls < 4; ++cls)
    for (size_t i = 0; i < P->groups.size(); ++i) {
      const Group& g = P->groups[i];
      const int c = g.level == 0 ? 0 : g.level == 2 ? 2 : (g.level == 1 && childless(g)) ? 3 : 1;
      if (c == cls) P->order.push_back((int)i);
    }
  return KYM_OK;
}

// The side lane of the forward on the current device (created on first use,
// at the lowest priority, the default streams' own; the plan's device tables
// must exist already).
static int side_stream(CascadePlan* P, cudaStream_t* side) {
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess) return fail_cuda(e, "side stream");
  std::lock_guard<std::mutex> lock(P->mu);
  auto it = P->dev.find(d);
  if (it == P->dev.end()) {
    set_error_message("side stream", "plan tables missing on this device");
    return KYM_ERR_INVALID;
  }
  DeviceState& s = it->second;
  if (!s.side) {
    int lo = 0, hi = 0;
    if ((e = cudaDeviceGetStreamPriorityRange(&lo, &hi)) != cudaSuccess ||
        (e = cudaStreamCreateWithPriority(&s.side, cudaStreamNonBlocking, lo)) != cudaSuccess)
      return fail_cuda(e, "side stream");
  }
  *side = s.side;
  return KYM_OK;
}

// The two copy streams of kym_s2d_forward_host on the current device
// (created on first use; the plan's device tables must exist already).
static int host_copy_streams(CascadePlan* P, cudaStream_t* in, cudaStream_t* out, cudaStream_t* out_side) {
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess) return fail_cuda(e, "host forward");
  std::lock_guard<std::mutex> lock(P->mu);
  auto it = P->dev.find(d);
  if (it == P->dev.end()) {
    set_error_message("host forward", "plan tables missing on this device");
    return KYM_ERR_INVALID;
  }
  DeviceState& s = it->second;
  if (!s.copy_in && (e = cudaStreamCreateWithFlags(&s.copy_in, cudaStreamNonBlocking)) != cudaSuccess)
    return fail_cuda(e, "copy stream");
  if (!s.copy_out && (e = cudaStreamCreateWithFlags(&s.copy_out, cudaStreamNonBlocking)) != cudaSuccess)
    return fail_cuda(e, "copy stream");
  if (!s.copy_out_side && (e = cudaStreamCreateWithFlags(&s.copy_out_side, cudaStreamNonBlocking)) != cudaSuccess)
    return fail_cuda(e, "copy stream");
  *in = s.copy_in;
  *out = s.copy_out;
  *out_side = s.copy_out_side;
  return KYM_OK;
}

// Upload the task and twiddle tables to the current device on first use.
static const DeviceState* device_state(CascadePlan* P) {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lock(P->mu);
  auto it = P->dev.find(d);
  if (it != P->dev.end()) return &it->second;
  DeviceState s;
  const size_t nt = P->all_tasks.size(), nw = P->tw.host().size();
  if (cudaMalloc(&s.tasks, std::max<size_t>(nt, 1) * sizeof(Task)) != cudaSuccess) return nullptr;
  if (cudaMalloc(&s.tw, std::max<size_t>(nw, 1) * sizeof(float2)) != cudaSuccess) {
    cudaFree(s.tasks);
    return nullptr;
  }
  const size_t nb = P->all_btasks.size(), ng = P->all_gather.size();
  if (cudaMalloc(&s.btasks, std::max<size_t>(nb, 1) * sizeof(BwdTask)) != cudaSuccess ||
      cudaMalloc(&s.gather, std::max<size_t>(ng, 1) * sizeof(GatherItem)) != cudaSuccess ||
      (nt && cudaMemcpy(s.tasks, P->all_tasks.data(), nt * sizeof(Task), cudaMemcpyHostToDevice) != cudaSuccess) ||
      (nw && cudaMemcpy(s.tw, P->tw.host().data(), nw * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess) ||
      (nb && cudaMemcpy(s.btasks, P->all_btasks.data(), nb * sizeof(BwdTask), cudaMemcpyHostToDevice) != cudaSuccess) ||
      (ng && cudaMemcpy(s.gather, P->all_gather.data(), ng * sizeof(GatherItem), cudaMemcpyHostToDevice) !=
                 cudaSuccess)) {
    cudaFree(s.tasks);
    cudaFree(s.tw);
    cudaFree(s.btasks);
    cudaFree(s.gather);
    return nullptr;
  }
  return &(P->dev[d] = s);
}

// Geometry of one group: work size (mr, mc), fold from the source, low-pass
// size.  Chooses the cluster size and shared-memory layout.
static int make_group(CascadePlan* P, Group& g, int mr, int mc, int kr, int kc, int sr, int sc, bool modulus,
                      bool src_image) {
  CascadeLaunch& L = g.L;
  std::memset(&L, 0, sizeof(L));
  g.oned = P->oned;
  L.mr = mr;
  L.mc = mc;
  L.kr = kr;
  L.kc = kc;
  L.sr = sr;
  L.sc = sc;
  L.modulus = modulus ? 1 : 0;
  L.src_image = src_image ? 1 : 0;
  L.bsum_off = -1;
  if (!make_fft_plan(mc, &L.prow, kThreads) || !make_fft_plan(mr, &L.pcol, kThreads) ||
      !make_fft_plan(sc, &L.psrow, kThreads) || !make_fft_plan(sr, &L.pscol, kThreads))
    return KYM_ERR_UNSUPPORTED;
  P->tw.add(mc);
  P->tw.add(mr);
  P->tw.add(sc);
  P->tw.add(sr);
  const size_t max_smem = max_dynamic_smem();
  if (P->oned) {
    L.ld = swz_len(mc);
    L.ldb = swz_len(sc);
    L.cluster = 1;
    L.rows_local = 1;
    g.smem = ((size_t)L.ld + L.ldb) * sizeof(float2);
    if (g.smem > max_smem) return KYM_ERR_UNSUPPORTED;
  } else {
    L.ld = odd_pitch(mc);
    L.ldb = odd_pitch(sc);
    int C = 0;
    for (int c : {1, 2, 4, 8}) {
      if (mr % c || mc % c) continue;
      size_t s = ((size_t)(mr / c) * L.ld + (size_t)sr * L.ldb) * sizeof(float2);
      if (c > 1) s += (size_t)mr * sizeof(void*);
      if (s <= max_smem) {
        C = c;
        g.smem = s;
        break;
      }
    }
    if (!C) return KYM_ERR_UNSUPPORTED;
    L.cluster = C;
    L.rows_local = mr / C;
    if (C > 1) P->tw.add(mr / C);
  }
  static_assert(sizeof(int) == 4, "");
  if (g_use_ct) {
    // image sources use fold 0; spectra fold kr x kr when square (2-D) or kc (1-D)
    const int kf = src_image ? 0 : (P->oned ? kc : (kr == kc ? kr : -2));
    const CtEntry* e = ct_find(mr, mc, sr, sc, L.cluster, P->oned, kf);
    if (e && e->smem <= max_smem) {
      g.has_ct = true;
      g.ct = *e;
      g.smem = e->smem;
    }
    if (!P->oned && L.cluster > 1) g.lines = lines_find(mr, mc, sr, sc, kf);
  }
  L.load_scale = src_image ? 1.f : (float)(1.0 / ((double)kr * kc) / (modulus ? (double)mr * mc : 1.0));
  L.s_scale = (float)(1.0 / ((double)(mr / sr) * (mc / sc)) / ((double)sr * sc));
  return KYM_OK;
}

template <bool CL, bool ONED>
static cudaError_t launch_group(const Group& g, const CascadeLaunch& L, const FilterTable& F, int nimg,
                                cudaStream_t stream) {
  auto kern = cascade_kernel<CL, ONED>;
  static SmemOptin optin;  // the largest dynamic shared memory, once per device
  if (cudaError_t e = optin.ensure(kern, (int)max_dynamic_smem()); e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(L.ntasks * L.cluster, nimg, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = g.smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  cfg.attrs = attr;
  cfg.numAttrs = 0;
  if (CL) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = L.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kern, L, F);
}

// Where one forward finds its tables and workspace.  ``stage0_per_chunk``
// runs the input stage chunk by chunk (the workspace then holds the input
// spectra of one chunk only).
struct RunArgs {
  const LowpassTable* lp = nullptr;  // non-null: tensor-core form for the groups that have one
  unsigned* status = nullptr;
  const DeviceState* ds = nullptr;
  float2* u0 = nullptr;
  float2* u1 = nullptr;
  int chunk = 1;
  bool stage0_per_chunk = false;
  float* group_ms = nullptr;
  int max_groups = 0;
  float2* ysave = nullptr;  // non-null: every path stores its modulus input (per image gy2 + gy1 elements)
  unsigned char* opnd = nullptr;  // DFT-GEMM operand slots (chunk images)
  // host transfers (kym_s2d_forward_host): the input is copied from x_host to
  // the device input in `parts` slices on copy_in, each output channel run is
  // copied to out_host on copy_out once the group writing it has finished
  const float* x_host = nullptr;
  float* out_host = nullptr;
  cudaStream_t copy_in = nullptr, copy_out = nullptr, copy_out_side = nullptr;
  int parts = 1;
  cudaEvent_t x_free = nullptr;  // non-null: the input copy waits for it instead of for `stream`
  // non-null: groups of lane 1 run here, forked from and joined back to the
  // caller's stream around every chunk
  cudaStream_t side = nullptr;
};

// Events of one host forward, destroyed when it returns (a recorded event may
// be destroyed before it completes; waits already enqueued on it stand).
struct EventPool {
  std::vector<cudaEvent_t> ev;
  cudaError_t make(cudaEvent_t* e) {
    const cudaError_t r = cudaEventCreateWithFlags(e, cudaEventDisableTiming);
    if (r == cudaSuccess) ev.push_back(*e);
    return r;
  }
  ~EventPool() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
};

static int make_filter_table(CascadePlan* P, const float* const* filters, int nfilters, FilterTable* F) {
  if (!filters || nfilters != (int)P->filter_rows.size() || nfilters > kMaxFilters) {
    set_error_message("filters", "filter count does not match the plan");
    return KYM_ERR_INVALID;
  }
  std::memset(F, 0, sizeof(*F));
  for (int i = 0; i < nfilters; ++i) {
    if (!filters[i]) {
      set_error_message("filters", "null filter pointer");
      return KYM_ERR_INVALID;
    }
    F->f[i] = filters[i];
  }
  return KYM_OK;
}

static int run_core(CascadePlan* P, const float* x, float* out, int batch, const FilterTable& F, const RunArgs& a,
                    cudaStream_t stream) {
  const DeviceState* ds = a.ds;
  // equal chunks: ceil(batch / n) images each for the fewest chunks n
  int chunk = std::max(1, std::min(batch, a.chunk));
  const int nch = (batch + chunk - 1) / chunk;
  chunk = (batch + nch - 1) / nch;
  const long long x_stride = (long long)P->img_M * P->img_N;
  const long long out_stride = (long long)P->channels * P->out_nr * P->out_nc;
  cudaError_t err = cudaSuccess;
  // optional timing: one event pair around every launch of every group
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> evs;
  const bool timed = a.group_ms && a.max_groups > 0;
  if (timed)
    for (int i = 0; i < a.max_groups; ++i) a.group_ms[i] = 0.f;
  // host transfers: input slices [part0[p], part0[p + 1]) copied on copy_in
  const bool hio = a.x_host && a.out_host && a.copy_in && a.copy_out && a.copy_out_side;
  EventPool pool;
  const int parts = hio ? std::max(1, std::min(a.parts, batch)) : 1;
  std::vector<int> part0(parts + 1);
  for (int p = 0; p <= parts; ++p) part0[p] = (int)((long long)batch * p / parts);
  std::vector<cudaEvent_t> in_ev(parts, nullptr);
  int waited = 0;  // input slices `stream` already waits for
  if (hio) {
    // the input copy overwrites the device input once its earlier users are
    // done: the work already on `stream`, or the caller's event (a staging
    // buffer the caller rotates, free while this stream still runs other
    // work).  The output copies follow the groups, hence that work too.
    cudaEvent_t start = a.x_free;
    if (!start && ((err = pool.make(&start)) != cudaSuccess || (err = cudaEventRecord(start, stream)) != cudaSuccess))
      return fail_cuda(err, "host forward");
    // (the caller's event also orders `stream`, for the device output, in
    // case the earlier call ran on another stream)
    if ((err = cudaStreamWaitEvent(a.copy_in, start, 0)) != cudaSuccess ||
        (a.x_free && (err = cudaStreamWaitEvent(stream, start, 0)) != cudaSuccess))
      return fail_cuda(err, "host forward");
    for (int p = 0; p < parts; ++p) {
      const size_t off = (size_t)part0[p] * x_stride;
      const size_t bytes = (size_t)(part0[p + 1] - part0[p]) * x_stride * sizeof(float);
      if ((err = cudaMemcpyAsync(const_cast<float*>(x) + off, a.x_host + off, bytes, cudaMemcpyHostToDevice,
                                 a.copy_in)) != cudaSuccess ||
          (err = pool.make(&in_ev[p])) != cudaSuccess || (err = cudaEventRecord(in_ev[p], a.copy_in)) != cudaSuccess)
        return fail_cuda(err, "host input copy");
    }
  }
  // make `stream` wait for the input slices that hold images below `end`
  auto wait_inputs = [&](int end) -> cudaError_t {
    cudaError_t r = cudaSuccess;
    while (hio && waited < parts && part0[waited] < end && r == cudaSuccess)
      r = cudaStreamWaitEvent(stream, in_ev[waited++], 0);
    return r;
  };
  for (int c0 = 0; c0 < batch; c0 += chunk) {
    const int nimg = std::min(chunk, batch - c0);
    bool forked = false;
    for (int gi : P->order) {
      const Group& g = P->groups[gi];
      if (g.level == 0 && c0 != 0 && !a.stage0_per_chunk) continue;  // input stage once over the batch
      if (a.side && g.level > 0 && !forked) {
        // the side lane starts once this chunk's inputs are ready: after
        // the work already on the caller's stream (input stage, earlier chunks)
        cudaEvent_t f;
        if ((err = pool.make(&f)) != cudaSuccess || (err = cudaEventRecord(f, stream)) != cudaSuccess ||
            (err = cudaStreamWaitEvent(a.side, f, 0)) != cudaSuccess)
          return fail_cuda(err, "side lane fork");
        forked = true;
      }
      const cudaStream_t gs = (a.side && g.lane == 1) ? a.side : stream;
      CascadeLaunch L = g.L;
      L.tasks = ds->tasks + g.task_off;
      L.ntasks = (int)g.tasks.size();
      L.prow.tw = ds->tw + P->tw.offset(L.prow.n);
      L.pcol.tw = ds->tw + P->tw.offset(L.pcol.n);
      L.psrow.tw = ds->tw + P->tw.offset(L.psrow.n);
      L.pscol.tw = ds->tw + P->tw.offset(L.pscol.n);
      L.tw_rl = L.cluster > 1 ? ds->tw + P->tw.offset(L.mr / L.cluster) : nullptr;
      L.x = x;
      L.x_stride = x_stride;
      L.opnd = a.opnd;
      L.out = out;
      L.out_stride = out_stride;
      if (a.ysave && g.level > 0) {
        L.ysave = a.ysave + (size_t)c0 * (P->gy1_elems + P->gy2_elems);
        L.ysave_stride = P->gy1_elems + P->gy2_elems;
      }
      int n = nimg;
      // image c of the chunk has its input spectrum at u0 + i * u0_elems, with
      // i = c0 + c when the input stage covers the whole batch, i = c otherwise
      const size_t u0_first = a.stage0_per_chunk ? 0 : (size_t)c0;
      if (g.level == 0) {
        n = a.stage0_per_chunk ? nimg : batch;
        L.img0 = a.stage0_per_chunk ? c0 : 0;
        L.dst = a.u0;
        L.dst_stride = P->u0_elems;
      } else if (g.level == 1) {
        L.img0 = c0;
        L.src = a.u0 + u0_first * P->u0_elems;
        L.src_stride = P->u0_elems;
        L.dst = a.u1;
        L.dst_stride = P->u1_elems;
      } else {
        L.img0 = c0;
        L.src = a.u1;
        L.src_stride = P->u1_elems;
      }
      // grid.y is limited to 65535 images per launch.  The line-split passes
      // round-trip their spectrum slots between passes: they run over as many
      // images as keep those slots within 64 MiB, so the slots stay in L2.
      int step = 65535;
      if (g.lines) {
        const double slot_bytes = (double)g.tasks.size() * g.L.mr * g.L.mc * sizeof(float2);
        step = (int)std::max(1.0, std::min(65535.0, 64.0 * 1024 * 1024 / slot_bytes));
      }
      // a line-split group runs its low-pass kernel once after all its
      // sub-launches: one wide launch instead of one narrow one per sub-launch
      const bool lp_after = g.lines && step < n;
      for (int i0 = 0; i0 < n;) {
        CascadeLaunch Li = L;
        if (lp_after) Li.lines_stage = 1;
        int ni = std::min(step, n - i0);
        if (hio && g.level == 0) {
          // the input stage runs slice by slice as the slices land
          const int first = L.img0 + i0;
          int p = 0;
          while (part0[p + 1] <= first) ++p;
          ni = std::min(ni, part0[p + 1] - first);
          if ((err = wait_inputs(first + ni)) != cudaSuccess) return fail_cuda(err, "host forward");
        }
        Li.img0 = L.img0 + i0;
        if (Li.src) Li.src = L.src + (size_t)i0 * L.src_stride;
        if (Li.dst) Li.dst = L.dst + (size_t)i0 * L.dst_stride;
        if (Li.ysave) Li.ysave = L.ysave + (size_t)i0 * L.ysave_stride;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (timed && (int)gi < a.max_groups) {
          cudaEventCreate(&e0);
          cudaEventCreate(&e1);
          cudaEventRecord(e0, gs);
        }
        if (a.lp && g.tc_on && g.tcdft && a.opnd) err = g.tcdft(Li, F, *a.lp, a.status, ni, gs);
        else if (a.lp && g.tc_on && g.has_tc) err = g.tc(Li, F, *a.lp, a.status, ni, gs);
        else if (g.lines) err = g.lines(Li, F, ni, gs);
        else if (g.has_ct) err = g.ct.fn(Li, F, ni, gs);
        else if (g.oned) err = launch_group<false, true>(g, Li, F, ni, gs);
        else if (Li.cluster > 1) err = launch_group<true, false>(g, Li, F, ni, gs);
        else err = launch_group<false, false>(g, Li, F, ni, gs);
        if (e0) {
          cudaEventRecord(e1, gs);
          evs.push_back({(int)gi, {e0, e1}});
        }
        if (err != cudaSuccess) {
          for (auto& e : evs) {
            cudaEventDestroy(e.second.first);
            cudaEventDestroy(e.second.second);
          }
          return fail_cuda(err, "cascade launch");
        }
        i0 += ni;
      }
      for (int i0 = 0; lp_after && i0 < n; i0 += 65535) {
        CascadeLaunch Li = L;
        Li.lines_stage = 2;
        const int ni = std::min(65535, n - i0);
        Li.img0 = L.img0 + i0;
        if (Li.src) Li.src = L.src + (size_t)i0 * L.src_stride;
        if (Li.dst) Li.dst = L.dst + (size_t)i0 * L.dst_stride;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (timed && gi < a.max_groups) {
          cudaEventCreate(&e0);
          cudaEventCreate(&e1);
          cudaEventRecord(e0, gs);
        }
        err = g.lines(Li, F, ni, gs);
        if (e0) {
          cudaEventRecord(e1, gs);
          evs.push_back({gi, {e0, e1}});
        }
        if (err != cudaSuccess) {
          for (auto& e : evs) {
            cudaEventDestroy(e.second.first);
            cudaEventDestroy(e.second.second);
          }
          return fail_cuda(err, "cascade launch");
        }
      }
      if (hio && !g.out_runs.empty()) {
        // this group's channels are final for its images: copy them out
        const int a0 = g.level == 0 ? L.img0 : c0;
        const cudaStream_t co = gs == stream ? a.copy_out : a.copy_out_side;
        cudaEvent_t done;
        if ((err = pool.make(&done)) != cudaSuccess || (err = cudaEventRecord(done, gs)) != cudaSuccess ||
            (err = cudaStreamWaitEvent(co, done, 0)) != cudaSuccess)
          return fail_cuda(err, "host forward");
        const size_t plane = (size_t)P->out_nr * P->out_nc;
        for (const auto& r : g.out_runs) {
          const size_t off = (size_t)a0 * out_stride + r.first * plane;
          err = cudaMemcpy2DAsync(a.out_host + off, out_stride * sizeof(float), out + off, out_stride * sizeof(float),
                                  (size_t)(r.second - r.first) * plane * sizeof(float), n, cudaMemcpyDeviceToHost,
                                  co);
          if (err != cudaSuccess) return fail_cuda(err, "host output copy");
        }
      }
    }
    if (forked) {
      // join: the next chunk reuses the parent-spectrum workspace
      cudaEvent_t jn;
      if ((err = pool.make(&jn)) != cudaSuccess || (err = cudaEventRecord(jn, a.side)) != cudaSuccess ||
          (err = cudaStreamWaitEvent(stream, jn, 0)) != cudaSuccess)
        return fail_cuda(err, "side lane join");
    }
  }
  if (hio) {
    // `stream` orders after every copy: later work on it sees out_host complete
    cudaEvent_t fin, fin_side;
    if ((err = wait_inputs(batch)) != cudaSuccess || (err = pool.make(&fin)) != cudaSuccess ||
        (err = cudaEventRecord(fin, a.copy_out)) != cudaSuccess || (err = cudaStreamWaitEvent(stream, fin, 0)) != cudaSuccess ||
        (err = pool.make(&fin_side)) != cudaSuccess || (err = cudaEventRecord(fin_side, a.copy_out_side)) != cudaSuccess ||
        (err = cudaStreamWaitEvent(stream, fin_side, 0)) != cudaSuccess)
      return fail_cuda(err, "host forward");
  }
  if (timed) {
    cudaError_t se = cudaStreamSynchronize(stream);
    for (auto& e : evs) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, e.second.first, e.second.second) == cudaSuccess) a.group_ms[e.first] += ms;
      cudaEventDestroy(e.second.first);
      cudaEventDestroy(e.second.second);
    }
    if (se != cudaSuccess) return fail_cuda(se, "timed forward");
  }
  return KYM_OK;
}

static int run_plan(CascadePlan* P, const float* x, float* out, int batch, const float* const* filters,
                    int nfilters, void* workspace, size_t ws_bytes, cudaStream_t stream,
                    float* group_ms = nullptr, int max_groups = 0, const LowpassTable* lp = nullptr,
                    unsigned* status = nullptr, float2* ysave = nullptr, const float* x_host = nullptr,
                    float* out_host = nullptr, int parts = 1, cudaEvent_t x_free = nullptr) {
  if (!P || !x || !out || batch < 0) {
    set_error_message("forward", "null plan, input or output");
    return KYM_ERR_INVALID;
  }
  if (batch == 0) return KYM_OK;
  FilterTable F;
  int rc = make_filter_table(P, filters, nfilters, &F);
  if (rc) return rc;
  const int chunk = std::min(batch, P->chunk);
  const size_t spectra = ((size_t)batch * P->u0_elems + (size_t)chunk * P->u1_elems) * sizeof(float2);
  // the DFT-GEMM groups of the tensor-core form keep their operand slots after the spectra
  const size_t opnd_off = (spectra + 255) & ~(size_t)255;
  // the fold pass copies source and wavelet rows with TMA: 16-byte-aligned bases
  bool aligned = (reinterpret_cast<uintptr_t>(workspace) & 15) == 0;
  for (int i = 0; aligned && i < nfilters; ++i) aligned = (reinterpret_cast<uintptr_t>(filters[i]) & 15) == 0;
  const bool dft = lp && !ysave && P->opnd_bytes && g_use_tcdft.load() && aligned;
  const size_t need = dft ? opnd_off + (size_t)chunk * P->opnd_bytes : spectra;
  if (!workspace || ws_bytes < need) {
    set_error_message("forward", "workspace missing or smaller than the plan requires");
    return KYM_ERR_WORKSPACE;
  }
  const DeviceState* ds = device_state(P);
  if (!ds) return fail_cuda(cudaGetLastError(), "plan table upload");
  RunArgs a;
  a.ds = ds;
  a.u0 = static_cast<float2*>(workspace);
  a.u1 = a.u0 + (size_t)batch * P->u0_elems;
  a.chunk = chunk;
  a.group_ms = group_ms;
  a.max_groups = max_groups;
  a.lp = ysave ? nullptr : lp;  // the tensor-core kernels do not save y
  a.status = status;
  a.ysave = ysave;
  if (dft) a.opnd = static_cast<unsigned char*>(workspace) + opnd_off;
  // independent group chains on the side lane (not while timing groups one
  // by one, nor with the DFT-GEMM form, whose groups share operand slots)
  bool lanes = g_use_side.load() && !group_ms && !a.opnd;
  if (lanes) {
    bool any = false;
    for (const Group& g : P->groups) any |= g.lane == 1;
    lanes = any;
  }
  if (lanes) {
    rc = side_stream(P, &a.side);
    if (rc) return rc;
  }
  if (x_host || out_host) {
    if (!x_host || !out_host) {
      set_error_message("host forward", "null host input or output");
      return KYM_ERR_INVALID;
    }
    rc = host_copy_streams(P, &a.copy_in, &a.copy_out, &a.copy_out_side);
    if (rc) return rc;
    a.x_host = x_host;
    a.out_host = out_host;
    a.parts = parts;
    a.x_free = x_free;
  }
  return run_core(P, x, out, batch, F, a, stream);
}

// Tensor-core variants for the childless groups (2-D, one CTA per task).
static void attach_tc(CascadePlan* P) {
  for (Group& g : P->groups) {
    g.has_tc = false;
    if (P->oned || g.level == 0 || g.L.cluster != 1 || g.L.kr != g.L.kc) continue;
    bool childless = true;
    for (const Task& t : g.tasks) childless &= t.dst_off < 0;
    if (!childless) continue;
    size_t smem = 0;
    TcLauncher fn = nullptr;
    if (tc_find(g.L.mr, g.L.mc, g.L.out_nr, g.L.out_nc, g.L.kr, &smem, &fn) && smem <= max_dynamic_smem()) {
      g.has_tc = true;
      g.tc_smem = smem;
      g.tc = fn;
      // the DFT-GEMM fold pass reads its paths as a P x 8 grid: path p * 8 + q
      // folds source p with wavelet q (sources and wavelets shared along rows
      // and columns), from 16-byte-aligned rows
      // the stride the fold reads per image: the input spectra for order 1,
      // the parent spectra for order 2
      const long long src_stride = g.level == 1 ? P->u0_elems : P->u1_elems;
      bool grid = (g.tasks.size() == 8 || g.tasks.size() == 64) && (src_stride % 2 == 0);
      for (size_t i = 0; grid && i < g.tasks.size(); ++i) {
        const Task& t = g.tasks[i];
        grid = t.src_off % 2 == 0 && t.src_off == g.tasks[i / 8 * 8].src_off && t.psi == g.tasks[i % 8].psi &&
               t.phi == g.tasks[0].phi;
      }
      if (grid && tcdft_find(g.L.mr, g.L.mc, g.L.out_nr, g.L.out_nc, g.L.kr, &smem, &fn) &&
          smem <= max_dynamic_smem()) {
        g.tcdft = fn;
        const size_t mp = (size_t)(g.L.mr + 7) / 8 * 8;
        P->opnd_bytes = std::max(P->opnd_bytes, g.tasks.size() * 8 * mp * mp);
      }
    }
  }
}

// Forward whose tables and workspace live in a caller-provided device buffer
// (the library's static scratch): the plan's task and twiddle tables are
// copied to its head on `stream`, then the batch runs in chunks whose input
// and parent spectra fit the rest.
int run_plan_in_scratch(CascadePlan* P, const float* x, float* out, int batch, const float* const* filters,
                        int nfilters, void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  if (!P || !x || !out || batch < 0 || !scratch) {
    set_error_message("forward_noalloc", "null plan, input, output or scratch");
    return KYM_ERR_INVALID;
  }
  if (batch == 0) return KYM_OK;
  FilterTable F;
  int rc = make_filter_table(P, filters, nfilters, &F);
  if (rc) return rc;
  const size_t nt = P->all_tasks.size(), nw = P->tw.host().size();
  const size_t tasks_bytes = (nt * sizeof(Task) + 255) & ~size_t(255);
  const size_t tw_bytes = (nw * sizeof(float2) + 255) & ~size_t(255);
  const size_t tables = tasks_bytes + tw_bytes;
  const size_t per_image = (size_t)(P->u0_elems + P->u1_elems) * sizeof(float2);
  if (tables + per_image > scratch_bytes) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "one image needs %zu bytes of scratch (tables %zu + spectra %zu), above the %zu-byte static "
                  "scratch of the allocation-free entry point",
                  tables + per_image, tables, per_image, scratch_bytes);
    set_error_message("forward_noalloc", msg);
    return KYM_ERR_WORKSPACE;
  }
  unsigned char* base = static_cast<unsigned char*>(scratch);
  // tables: copied on the stream, so earlier calls on the same stream finish
  // first.  The host image belongs to the plan (immutable once built).
  const unsigned char* img = nullptr;
  {
    std::lock_guard<std::mutex> lock(P->mu);
    if (P->scratch_tables.size() != tables) {
      P->scratch_tables.assign(tables, 0);
      if (nt) std::memcpy(P->scratch_tables.data(), P->all_tasks.data(), nt * sizeof(Task));
      if (nw) std::memcpy(P->scratch_tables.data() + tasks_bytes, P->tw.host().data(), nw * sizeof(float2));
    }
    img = P->scratch_tables.data();
  }
  cudaError_t e = cudaMemcpyAsync(base, img, tables, cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return fail_cuda(e, "scratch table copy");
  DeviceState ds;
  ds.tasks = reinterpret_cast<Task*>(base);
  ds.tw = reinterpret_cast<float2*>(base + tasks_bytes);
  const int fit = (int)std::min<size_t>((scratch_bytes - tables) / per_image, (size_t)1 << 20);
  RunArgs a;
  a.ds = &ds;
  a.chunk = std::max(1, std::min(fit, P->chunk));
  a.u0 = reinterpret_cast<float2*>(base + tables);
  a.u1 = a.u0 + (size_t)a.chunk * P->u0_elems;
  a.stage0_per_chunk = true;
  return run_core(P, x, out, batch, F, a, stream);
}

// ---------------------------------------------------------------------------
// backward: tables
// ---------------------------------------------------------------------------
static size_t rt_bwd_smem(const CascadeLaunch& L) {
  return ((size_t)L.rows_local * L.ld + (size_t)L.sr * L.ldb) * sizeof(float2) +
         (L.cluster > 1 ? (size_t)L.mr * sizeof(void*) : 0);
}

// Mirror every forward group with a backward group.  Order-2 tasks write
// g_Y into the per-image order-2 block; order-1 tasks gather their children
// (the order-2 tasks reading their spectrum) and write into the order-1
// block; the input stage gathers every order-1 task.
static int build_backward(CascadePlan* P) {
  P->bgroups.clear();
  P->all_btasks.clear();
  P->all_gather.clear();
  std::map<long long, std::vector<int>> children;  // parent spectrum offset -> (group<<20 | task)
  std::vector<std::vector<long long>> gy_of(P->groups.size());
  long long gy2 = 0, gy1 = 0;
  for (size_t gi = 0; gi < P->groups.size(); ++gi) {
    const Group& g = P->groups[gi];
    gy_of[gi].assign(g.tasks.size(), -1);
    if (g.level != 2) continue;
    for (size_t ti = 0; ti < g.tasks.size(); ++ti) {
      gy_of[gi][ti] = gy2;
      gy2 += (long long)g.L.mr * g.L.mc;
      children[g.tasks[ti].src_off].push_back((int)((gi << 20) | ti));
    }
  }
  for (size_t gi = 0; gi < P->groups.size(); ++gi) {
    const Group& g = P->groups[gi];
    if (g.level != 1) continue;
    for (size_t ti = 0; ti < g.tasks.size(); ++ti) {
      gy_of[gi][ti] = gy1;
      gy1 += (long long)g.L.mr * g.L.mc;
    }
  }
  P->gy1_elems = gy1;
  P->gy2_elems = gy2;
  auto item_of = [&](int gi, int ti) {
    const Group& c = P->groups[gi];
    GatherItem it;
    it.gy_off = gy_of[gi][ti];
    it.psi = c.tasks[ti].psi;
    it.mr = c.L.mr;
    it.mc = c.L.mc;
    auto lg = [](int k) {
      int q = 0;
      while ((1 << q) < k) ++q;
      return q;
    };
    it.lkr = lg(c.L.kr);
    it.lkc = lg(c.L.kc);
    it.w = (float)(1.0 / ((double)c.L.kr * c.L.kc));
    it.pad_ = 0;
    it.gy_pstride = 0;
    return it;
  };
  // the gather tabulates residues for power-of-two folds only (every fold of
  // the 1-D and 2-D cascades is one)
  for (const Group& g : P->groups)
    if ((g.L.kr & (g.L.kr - 1)) || (g.L.kc & (g.L.kc - 1)) || g.L.kr >= (1 << kGatherLogs) ||
        g.L.kc >= (1 << kGatherLogs)) {
      set_error_message("plan", "fold factor is not a power of two below 2^24");
      return KYM_ERR_UNSUPPORTED;
    }
  for (int level : {2, 1, 0}) {
    for (size_t gi = 0; gi < P->groups.size(); ++gi) {
      const Group& g = P->groups[gi];
      if (g.level != level) continue;
      BwdGroup b;
      b.fwd = (int)gi;
      b.level = level;
      for (size_t ti = 0; ti < g.tasks.size(); ++ti) {
        const Task& t = g.tasks[ti];
        BwdTask bt;
        bt.src_off = t.src_off;
        bt.gy_off = level == 0 ? 0 : gy_of[gi][ti];
        bt.psi = level == 0 ? -1 : t.psi;
        bt.phi = t.phi;
        bt.out_ch = t.out_ch;
        bt.gather_first = (int)P->all_gather.size();
        bt.gather_count = 0;
        bt.y_off = level == 0 ? -1 : (int)(gy_of[gi][ti] + (level == 1 ? P->gy2_elems : 0));
        if (level == 1 && t.dst_off >= 0) {
          auto it = children.find(t.dst_off);
          if (it != children.end())
            for (int code : it->second) P->all_gather.push_back(item_of(code >> 20, code & 0xFFFFF));
        } else if (level == 0) {
          for (size_t gj = 0; gj < P->groups.size(); ++gj)
            if (P->groups[gj].level == 1)
              for (size_t tj = 0; tj < P->groups[gj].tasks.size(); ++tj)
                P->all_gather.push_back(item_of((int)gj, (int)tj));
        }
        bt.gather_count = (int)P->all_gather.size() - bt.gather_first;
        b.tasks.push_back(bt);
      }
      size_t smem = 0;
      BwdCtLauncher fn = nullptr;
      if (g.has_ct && bwd_ct_find(g.L.mr, g.L.mc, g.L.sr, g.L.sc, g.L.cluster, g.oned, &smem, &fn)) {
        b.has_ct = true;
        b.ct = fn;
        b.smem = smem;
      } else {
        b.smem = rt_bwd_smem(g.L);
      }
      // parent sets for the gather: NP consecutive tasks with the same
      // children wavelets and geometry, each child's g_Y a fixed stride
      // further for the next parent of the set
      for (int np : {8, 4, 2}) {
        const int nt = (int)b.tasks.size();
        if (nt % np || b.tasks[0].gather_count == 0) continue;
        bool ok = true;
        std::vector<long long> stride(b.tasks[0].gather_count, 0);
        for (int s0 = 0; s0 < nt && ok; s0 += np) {
          const BwdTask& a = b.tasks[s0];
          for (int p = 1; p < np && ok; ++p) {
            const BwdTask& q = b.tasks[s0 + p];
            ok = q.gather_count == a.gather_count;
            for (int i = 0; ok && i < a.gather_count; ++i) {
              const GatherItem& x = P->all_gather[a.gather_first + i];
              const GatherItem& y = P->all_gather[q.gather_first + i];
              const long long d = y.gy_off - x.gy_off;
              if (p == 1 && s0 == 0) stride[i] = d;
              ok = y.psi == x.psi && y.mr == x.mr && y.mc == x.mc && y.lkr == x.lkr && y.lkc == x.lkc &&
                   d == (long long)p * stride[i] && stride[i] > 0;
            }
          }
        }
        if (!ok) continue;
        b.gather_np = np;
        for (int s0 = 0; s0 < nt; s0 += np)
          for (int i = 0; i < b.tasks[s0].gather_count; ++i) P->all_gather[b.tasks[s0].gather_first + i].gy_pstride = stride[i];
        break;
      }
      b.task_off = P->all_btasks.size();
      P->all_btasks.insert(P->all_btasks.end(), b.tasks.begin(), b.tasks.end());
      P->bgroups.push_back(b);
    }
  }
  // the forward tasks store y (the saved-activation form) at the same offsets:
  // per image [order-2 block | order-1 block]
  for (size_t gi = 0; gi < P->groups.size(); ++gi) {
    Group& g = P->groups[gi];
    for (size_t ti = 0; ti < g.tasks.size(); ++ti) {
      const int y = g.level == 0 ? -1 : (int)(gy_of[gi][ti] + (g.level == 1 ? P->gy2_elems : 0));
      g.tasks[ti].y_off = y;
      P->all_tasks[g.task_off + ti].y_off = y;
    }
  }
  const double budget = 1024.0 * 1024 * 1024;  // backward workspace per pass
  const double per = (double)(P->u0_elems + P->u1_elems + P->gy1_elems + P->gy2_elems) * sizeof(float2);
  P->bchunk = (int)std::max(1.0, std::min(budget / per, (double)(1 << 20)));
  return KYM_OK;
}

static size_t backward_bytes(const CascadePlan* P, int batch) {
  const int chunk = std::min(batch, P->bchunk);
  return (size_t)chunk * (P->u0_elems + P->u1_elems + P->gy1_elems + P->gy2_elems) * sizeof(float2);
}

template <bool CL, bool ONED>
static cudaError_t launch_rt_bwd(const BwdGroup& b, const BwdLaunch& L, const FilterTable& F, int nimg,
                                 cudaStream_t stream) {
  auto kern = rt_bwd_kernel<CL, ONED>;
  static SmemOptin optin;  // the largest dynamic shared memory, once per device
  if (cudaError_t e = optin.ensure(kern, (int)max_dynamic_smem()); e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(L.ntasks * L.cluster, nimg, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = b.smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  cfg.attrs = attr;
  cfg.numAttrs = 0;
  if (CL) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = L.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kern, L, F);
}

// g_x for a batch: per chunk, recompute the input and parent spectra, then
// run the order-2, order-1 and input-stage backward groups and the
// reflect-pad adjoint.
static int run_backward(CascadePlan* P, const float* x, const float* gout, float* gx, int batch,
                        const float* const* filters, int nfilters, void* workspace, size_t ws_bytes,
                        cudaStream_t stream, const float2* ysaved = nullptr) {
  if (!P || (!x && !ysaved) || !gout || !gx || batch < 0) {
    set_error_message("backward", "null plan, input, gradient or output");
    return KYM_ERR_INVALID;
  }
  if (batch == 0) return KYM_OK;
  FilterTable F;
  int rc = make_filter_table(P, filters, nfilters, &F);
  if (rc) return rc;
  if (!workspace || ws_bytes < backward_bytes(P, batch)) {
    set_error_message("backward", "workspace missing or smaller than the plan requires");
    return KYM_ERR_WORKSPACE;
  }
  const DeviceState* ds = device_state(P);
  if (!ds) return fail_cuda(cudaGetLastError(), "plan table upload");
  int chunk = std::min(batch, P->bchunk);
  const int nch = (batch + chunk - 1) / chunk;
  chunk = (batch + nch - 1) / nch;
  float2* u0 = static_cast<float2*>(workspace);
  float2* u1 = u0 + (size_t)chunk * P->u0_elems;
  float2* gy2 = u1 + (size_t)chunk * P->u1_elems;
  float2* gy1 = gy2 + (size_t)chunk * P->gy2_elems;
  const long long gs_stride = (long long)P->channels * P->out_nr * P->out_nc;
  cudaError_t err = cudaSuccess;
  for (int c0 = 0; c0 < batch; c0 += chunk) {
    const int nimg = std::min(chunk, batch - c0);
    const long long ystride = P->gy1_elems + P->gy2_elems;
    // 1. recompute the spectra the backward needs (input stage, parents),
    // unless the forward saved every path's modulus input
    RunArgs a;
    a.ds = ds;
    a.u0 = u0;
    a.u1 = u1;
    a.chunk = nimg;
    a.stage0_per_chunk = true;
    for (size_t gi = 0; gi < P->groups.size(); ++gi) {
      const Group& g = P->groups[gi];
      bool needed = g.level == 0;
      if (g.level == 1)
        for (const Task& t : g.tasks) needed |= t.dst_off >= 0;
      if (!needed || ysaved) continue;
      CascadeLaunch L = g.L;
      L.tasks = ds->tasks + g.task_off;
      L.ntasks = (int)g.tasks.size();
      L.prow.tw = ds->tw + P->tw.offset(L.prow.n);
      L.pcol.tw = ds->tw + P->tw.offset(L.pcol.n);
      L.psrow.tw = ds->tw + P->tw.offset(L.psrow.n);
      L.pscol.tw = ds->tw + P->tw.offset(L.pscol.n);
      L.tw_rl = L.cluster > 1 ? ds->tw + P->tw.offset(L.mr / L.cluster) : nullptr;
      L.x = x;
      L.x_stride = (long long)P->img_M * P->img_N;
      L.img0 = c0;
      L.skip_s = 1;
      if (g.level == 0) {
        L.dst = u0;
        L.dst_stride = P->u0_elems;
      } else {
        L.src = u0;
        L.src_stride = P->u0_elems;
        L.dst = u1;
        L.dst_stride = P->u1_elems;
      }
      if (g.lines) err = g.lines(L, F, nimg, stream);
      else if (g.has_ct) err = g.ct.fn(L, F, nimg, stream);
      else if (g.oned) err = launch_group<false, true>(g, L, F, nimg, stream);
      else if (L.cluster > 1) err = launch_group<true, false>(g, L, F, nimg, stream);
      else err = launch_group<false, false>(g, L, F, nimg, stream);
      if (err != cudaSuccess) return fail_cuda(err, "backward recomputation");
    }
    // 2. backward groups, order 2 then 1 then the input stage
    for (const BwdGroup& b : P->bgroups) {
      const Group& g = P->groups[b.fwd];
      BwdLaunch L;
      std::memset(&L, 0, sizeof(L));
      L.mr = g.L.mr;
      L.mc = g.L.mc;
      L.kr = g.L.kr;
      L.kc = g.L.kc;
      L.ld = g.L.ld;
      L.sr = g.L.sr;
      L.sc = g.L.sc;
      L.ldb = g.L.ldb;
      L.cluster = g.L.cluster;
      L.rows_local = g.L.rows_local;
      L.prow = g.L.prow;
      L.pcol = g.L.pcol;
      L.psrow = g.L.psrow;
      L.pscol = g.L.pscol;
      L.prow.tw = ds->tw + P->tw.offset(L.prow.n);
      L.pcol.tw = ds->tw + P->tw.offset(L.pcol.n);
      L.psrow.tw = ds->tw + P->tw.offset(L.psrow.n);
      L.pscol.tw = ds->tw + P->tw.offset(L.pscol.n);
      L.tw_rl = L.cluster > 1 ? ds->tw + P->tw.offset(L.mr / L.cluster) : nullptr;
      L.level = b.level;
      L.out_r0 = g.L.out_r0;
      L.out_c0 = g.L.out_c0;
      L.out_nr = g.L.out_nr;
      L.out_nc = g.L.out_nc;
      L.out_channels = P->channels;
      L.rec_scale = (float)(1.0 / ((double)L.kr * L.kc) / ((double)L.mr * L.mc));
      L.gb_scale = (float)(1.0 / ((double)L.sr * L.sc) / ((double)(L.mr / L.sr) * (L.mc / L.sc)));
      L.gy_scale = (float)(1.0 / ((double)L.mr * L.mc));
      L.gS = gout;
      L.gS_stride = gs_stride;
      L.tasks = ds->btasks + b.task_off;
      L.ntasks = (int)b.tasks.size();
      L.gather = ds->gather;
      L.img0 = c0;
      if (ysaved && b.level > 0) {
        L.ysaved = ysaved + (size_t)c0 * ystride;
        L.ysaved_stride = ystride;
      }
      if (b.level == 2) {
        L.src = u1;
        L.src_stride = P->u1_elems;
        L.gy = gy2;
        L.gy_stride = P->gy2_elems;
      } else if (b.level == 1) {
        L.src = u0;
        L.src_stride = P->u0_elems;
        L.gy = gy1;
        L.gy_stride = P->gy1_elems;
        L.gyc = gy2;
        L.gyc_stride = P->gy2_elems;
      } else {
        L.gy = u0;  // g_pad (real) over the input spectra, no longer needed
        L.gy_stride = P->u0_elems;
        L.gyc = gy1;
        L.gyc_stride = P->gy1_elems;
      }
      bool any_gather = false;
      for (const BwdTask& bt : b.tasks) any_gather |= bt.gather_count > 0;
      if (any_gather) {
        // one thread per column, at most kGatherThreads per block, tiles of equal width
        const int ntile = (L.mc + kGatherThreads - 1) / kGatherThreads;
        const int threads = ((L.mc + ntile - 1) / ntile + 31) / 32 * 32;
        const int ctiles = (L.mc + threads - 1) / threads;
        if (b.gather_np > 1) {
          dim3 grid((L.mr + kGatherSetRows - 1) / kGatherSetRows * ctiles, L.ntasks / b.gather_np, nimg);
          err = launch_gather_set(b.gather_np, grid, threads, stream, L.tasks, L.gather, F, L.mr, L.mc, L.gy,
                                  L.gy_stride, L.gyc, L.gyc_stride, nimg);
          if (err != cudaSuccess) return fail_cuda(err, "backward gather");
        } else {
          dim3 grid((L.mr + kGatherRows - 1) / kGatherRows * ctiles, L.ntasks, nimg);
          bwd_gather_kernel<<<grid, threads, 0, stream>>>(L.tasks, L.gather, F, L.mr, L.mc, L.gy, L.gy_stride, L.gyc,
                                                        L.gyc_stride, nimg);
        }
        err = cudaGetLastError();
        if (err != cudaSuccess) return fail_cuda(err, "backward gather");
      }
      if (b.has_ct) err = b.ct(L, F, nimg, stream);
      else if (g.oned) err = launch_rt_bwd<false, true>(b, L, F, nimg, stream);
      else if (L.cluster > 1) err = launch_rt_bwd<true, false>(b, L, F, nimg, stream);
      else err = launch_rt_bwd<false, false>(b, L, F, nimg, stream);
      if (err != cudaSuccess) return fail_cuda(err, "backward launch");
    }
    // 3. reflect-pad adjoint into g_x
    const int total = nimg * P->img_M * P->img_N;
    const int threads = 256;
    const int blocks = (total + threads - 1) / threads;
    reflect_pad_adjoint_kernel<<<blocks, threads, 0, stream>>>(
        reinterpret_cast<const float*>(u0), 2 * P->u0_elems, P->Mp, P->Np, gx, P->img_M, P->img_N, P->pad_t,
        P->pad_l, nimg, c0);
    err = cudaGetLastError();
    if (err != cudaSuccess) return fail_cuda(err, "reflect-pad adjoint");
  }
  return KYM_OK;
}

static size_t saved_bytes(const CascadePlan* P, int batch) {
  return (size_t)batch * (P->gy1_elems + P->gy2_elems) * sizeof(float2);
}

static int run_forward_save(CascadePlan* P, const float* x, float* out, int batch, const float* const* filters,
                            int nfilters, void* workspace, size_t ws_bytes, void* saved, size_t saved_size,
                            cudaStream_t stream) {
  if (batch > 0 && (!saved || saved_size < saved_bytes(P, batch))) {
    set_error_message("forward_save", "saved-activation buffer missing or smaller than the plan requires");
    return KYM_ERR_WORKSPACE;
  }
  return run_plan(P, x, out, batch, filters, nfilters, workspace, ws_bytes, stream, nullptr, 0, nullptr, nullptr,
                  static_cast<float2*>(saved));
}

static int run_backward_saved(CascadePlan* P, const void* saved, size_t saved_size, const float* gout, float* gx,
                              int batch, const float* const* filters, int nfilters, void* workspace,
                              size_t ws_bytes, cudaStream_t stream) {
  if (batch > 0 && (!saved || saved_size < saved_bytes(P, batch))) {
    set_error_message("backward_saved", "saved-activation buffer missing or smaller than the plan requires");
    return KYM_ERR_WORKSPACE;
  }
  return run_backward(P, nullptr, gout, gx, batch, filters, nfilters, workspace, ws_bytes, stream,
                      static_cast<const float2*>(saved));
}

// Images per chunk: as many as keep the chunk's parent spectra within 512 MiB.
// Large launches keep every SM busy through the tail of each group; the
// parents spill from L2 to HBM, but the children of a parent are adjacent
// tasks that run in the same wave and read it from L2, so HBM sees each
// parent about once per group (measured at 256x256 J=3, batch 64: the whole
// batch in one chunk runs 2.49 ms against 2.82 ms with 64 MiB chunks).
static void set_default_chunk(CascadePlan* P) {
  const double budget = 512.0 * 1024 * 1024;
  long long c = P->u1_elems ? (long long)(budget / (P->u1_elems * sizeof(float2))) : 1 << 20;
  P->chunk = (int)std::max<long long>(1, std::min<long long>(c, 1 << 20));
}

}  // namespace kym

using kym::CascadePlan;

// ---------------------------------------------------------------------------
// 2-D plan
// ---------------------------------------------------------------------------
struct kym_s2d_plan {
  CascadePlan p;
};

extern "C" int kym_s2d_plan_create(int M, int N, int J, int L, int max_order, int pre_pad, kym_s2d_plan** out) {
  using namespace kym;
  if (!out) return KYM_ERR_INVALID;
  *out = nullptr;
  if (M < 1 || N < 1 || J < 0 || L < 1 || max_order < 1 || max_order > 2) return KYM_ERR_INVALID;
  if ((1 << J) > M || (1 << J) > N) return KYM_ERR_INVALID;
  auto* h = new (std::nothrow) kym_s2d_plan;
  if (!h) return KYM_ERR_CUDA;
  CascadePlan* P = &h->p;
  P->M = M;
  P->N = N;
  P->J = J;
  P->L = L;
  P->max_order = max_order;
  P->pre_pad = pre_pad;
  const int k = 1 << J;
  P->Mp = ((M + k) / k + 1) * k;
  P->Np = ((N + k) / k + 1) * k;
  P->img_M = pre_pad ? P->Mp : M;
  P->img_N = pre_pad ? P->Np : N;
  P->pad_t = pre_pad ? 0 : (P->Mp - M) / 2;
  P->pad_l = pre_pad ? 0 : (P->Np - N) / 2;
  const int sr = P->Mp / k, sc = P->Np / k;
  P->out_nr = sr - 2;
  P->out_nc = sc - 2;
  // filter index layout: phi levels 0..J-1, then every psi's levels
  // (the order of the reference's registered buffers tensor0..tensorK)
  for (int r = 0; r < J; ++r) {
    P->filter_rows.push_back(P->Mp >> r);
    P->filter_cols.push_back(P->Np >> r);
  }
  std::vector<int> psi_first(J * L);
  for (int j = 0; j < J; ++j)
    for (int t = 0; t < L; ++t) {
      psi_first[j * L + t] = (int)P->filter_rows.size();
      const int nlev = std::min(j + 1, std::max(J - 1, 1));
      for (int r = 0; r < nlev; ++r) {
        P->filter_rows.push_back(P->Mp >> r);
        P->filter_cols.push_back(P->Np >> r);
      }
    }
  if ((int)P->filter_rows.size() > kMaxFilters) {
    delete h;
    return KYM_ERR_UNSUPPORTED;
  }
  P->u0_elems = (long long)P->Mp * P->Np;
  std::vector<long long> u1_off(J * L, -1);
  long long u1 = 0;
  if (max_order >= 2)
    for (int n1 = 0; n1 < J * L; ++n1) {
      const int j1 = n1 / L;
      if (j1 < J - 1) {
        u1_off[n1] = u1;
        u1 += (long long)(P->Mp >> j1) * (P->Np >> j1);
      }
    }
  P->u1_elems = u1;
  int rc = KYM_OK;
  // input stage
  {
    Group g;
    rc = make_group(P, g, P->Mp, P->Np, 1, 1, sr, sc, false, true);
    if (rc) goto fail;
    g.level = 0;
    g.L.out_r0 = 1;
    g.L.out_c0 = 1;
    g.L.out_nr = P->out_nr;
    g.L.out_nc = P->out_nc;
    g.L.img_M = P->img_M;
    g.L.img_N = P->img_N;
    g.L.pad_t = P->pad_t;
    g.L.pad_l = P->pad_l;
    g.tasks.push_back(Task{0, 0, -1, 0, 0, -1});
    P->groups.push_back(g);
  }
  // order 1, one launch per scale
  for (int j1 = 0; j1 < J; ++j1) {
    Group g;
    rc = make_group(P, g, P->Mp >> j1, P->Np >> j1, 1 << j1, 1 << j1, sr, sc, true, false);
    if (rc) goto fail;
    g.level = 1;
    g.L.out_r0 = 1;
    g.L.out_c0 = 1;
    g.L.out_nr = P->out_nr;
    g.L.out_nc = P->out_nc;
    for (int t = 0; t < L; ++t) {
      const int n1 = j1 * L + t;
      g.tasks.push_back(Task{0, u1_off[n1], psi_first[n1], j1, 1 + n1, -1});
    }
    P->groups.push_back(g);
  }
  // order 2, one launch per (j1, j2)
  if (max_order >= 2) {
    int ch = 1 + J * L;
    std::map<std::pair<int, int>, Group> byscale;
    std::vector<std::pair<int, int>> order;
    for (int n1 = 0; n1 < J * L; ++n1) {
      const int j1 = n1 / L;
      for (int n2 = 0; n2 < J * L; ++n2) {
        const int j2 = n2 / L;
        if (j2 <= j1) continue;
        auto key = std::make_pair(j1, j2);
        if (!byscale.count(key)) {
          Group g;
          rc = make_group(P, g, P->Mp >> j2, P->Np >> j2, 1 << (j2 - j1), 1 << (j2 - j1), sr, sc, true, false);
          if (rc) goto fail;
          g.level = 2;
          g.L.out_r0 = 1;
          g.L.out_c0 = 1;
          g.L.out_nr = P->out_nr;
          g.L.out_nc = P->out_nc;
          byscale[key] = g;
          order.push_back(key);
        }
        byscale[key].tasks.push_back(Task{u1_off[n1], -1, psi_first[n2] + j1, j2, ch++, -1});
      }
    }
    for (auto& key : order) P->groups.push_back(byscale[key]);
    P->channels = ch;
  } else {
    P->channels = 1 + J * L;
  }
  for (auto& g : P->groups) g.L.out_channels = P->channels;
  rc = finalize_groups(P);
  if (rc) goto fail;
  rc = build_backward(P);
  if (rc) goto fail;
  attach_tc(P);
  set_default_chunk(P);
  *out = h;
  return KYM_OK;
fail:
  delete h;
  return rc;
}

extern "C" int kym_set_specialized(int enable) {
  return kym::g_use_ct.exchange(enable != 0) ? 1 : 0;
}

extern "C" int kym_set_side_lane(int enable) {
  return kym::g_use_side.exchange(enable != 0) ? 1 : 0;
}

extern "C" int kym_set_tc_dft(int enable) {
  return kym::g_use_tcdft.exchange(enable != 0) ? 1 : 0;
}

extern "C" int kym_s2d_plan_destroy(kym_s2d_plan* plan) {
  delete plan;
  return KYM_OK;
}

extern "C" int kym_s2d_plan_info(const kym_s2d_plan* plan, int* M_padded, int* N_padded, int* channels,
                                 int* out_rows, int* out_cols, int* n_filters) {
  if (!plan) return KYM_ERR_INVALID;
  const CascadePlan& P = plan->p;
  if (M_padded) *M_padded = P.Mp;
  if (N_padded) *N_padded = P.Np;
  if (channels) *channels = P.channels;
  if (out_rows) *out_rows = P.out_nr;
  if (out_cols) *out_cols = P.out_nc;
  if (n_filters) *n_filters = (int)P.filter_rows.size();
  return KYM_OK;
}

extern "C" int kym_s2d_filter_shape(const kym_s2d_plan* plan, int index, int* rows, int* cols) {
  if (!plan || index < 0 || index >= (int)plan->p.filter_rows.size()) return KYM_ERR_INVALID;
  if (rows) *rows = plan->p.filter_rows[index];
  if (cols) *cols = plan->p.filter_cols[index];
  return KYM_OK;
}

extern "C" int kym_s2d_set_chunk(kym_s2d_plan* plan, int chunk) {
  if (!plan || chunk < 1) return KYM_ERR_INVALID;
  plan->p.chunk = chunk;
  return KYM_OK;
}

extern "C" int kym_s2d_get_chunk(const kym_s2d_plan* plan) { return plan ? plan->p.chunk : -1; }

extern "C" int kym_s2d_group_count(const kym_s2d_plan* plan) {
  return plan ? (int)plan->p.groups.size() : -1;
}

extern "C" int kym_s2d_group_info(const kym_s2d_plan* plan, int group, int* level, int* ntasks, int* rows,
                                  int* cols, int* fold, int* cluster) {
  if (!plan || group < 0 || group >= (int)plan->p.groups.size()) return KYM_ERR_INVALID;
  const kym::Group& g = plan->p.groups[group];
  if (level) *level = g.level;
  if (ntasks) *ntasks = (int)g.tasks.size();
  if (rows) *rows = g.L.mr;
  if (cols) *cols = g.L.mc;
  if (fold) *fold = g.L.kc;
  if (cluster) *cluster = g.L.cluster * (g.has_ct ? 1 : -1);
  return KYM_OK;
}

extern "C" int kym_s2d_forward_timed(const kym_s2d_plan* plan, const float* x, float* out, int batch,
                                     const float* const* filters, int n_filters, void* workspace,
                                     size_t workspace_bytes, void* stream, float* group_ms, int max_groups) {
  if (!plan || !group_ms || max_groups < 1) return KYM_ERR_INVALID;
  return kym::run_plan(const_cast<CascadePlan*>(&plan->p), x, out, batch, filters, n_filters, workspace,
                       workspace_bytes, static_cast<cudaStream_t>(stream), group_ms, max_groups);
}

extern "C" int kym_s2d_forward_tc(const kym_s2d_plan* plan, const float* x, float* out, int batch,
                                  const float* const* filters, int n_filters, const float* const* lowpass_rows,
                                  const float* const* lowpass_cols, int n_lowpass, void* workspace,
                                  size_t workspace_bytes, unsigned* status, void* stream, float* group_ms,
                                  int max_groups) {
  if (!plan || !lowpass_rows || !lowpass_cols || !status || n_lowpass < 1 || n_lowpass > kym::kMaxLowpass) {
    kym::set_error_message("forward_tc", "needs the separable low-pass factors and a status word");
    return KYM_ERR_INVALID;
  }
  kym::LowpassTable lp;
  std::memset(&lp, 0, sizeof(lp));
  for (int i = 0; i < n_lowpass; ++i) {
    lp.r[i] = lowpass_rows[i];
    lp.c[i] = lowpass_cols[i];
  }
  return kym::run_plan(const_cast<CascadePlan*>(&plan->p), x, out, batch, filters, n_filters, workspace,
                       workspace_bytes, static_cast<cudaStream_t>(stream), group_ms, group_ms ? max_groups : 0, &lp,
                       status);
}

extern "C" int kym_s2d_forward_host(const kym_s2d_plan* plan, const float* x_host, float* out_host, int batch,
                                    const float* const* filters, int n_filters, const float* const* lowpass_rows,
                                    const float* const* lowpass_cols, int n_lowpass, unsigned* status, float* x_dev,
                                    float* out_dev, void* workspace, size_t workspace_bytes, int parts,
                                    void* x_dev_free, void* stream) {
  if (!plan || !x_host || !out_host || !x_dev || !out_dev || parts < 1) {
    kym::set_error_message("forward_host", "null plan, host or device buffer, or parts < 1");
    return KYM_ERR_INVALID;
  }
  const bool tc = lowpass_rows || lowpass_cols || status;
  if (tc && (!lowpass_rows || !lowpass_cols || !status || n_lowpass < 1 || n_lowpass > kym::kMaxLowpass)) {
    kym::set_error_message("forward_host", "the tensor-core form needs the low-pass factors and a status word");
    return KYM_ERR_INVALID;
  }
  kym::LowpassTable lp;
  std::memset(&lp, 0, sizeof(lp));
  for (int i = 0; tc && i < n_lowpass; ++i) {
    lp.r[i] = lowpass_rows[i];
    lp.c[i] = lowpass_cols[i];
  }
  return kym::run_plan(const_cast<CascadePlan*>(&plan->p), x_dev, out_dev, batch, filters, n_filters, workspace,
                       workspace_bytes, static_cast<cudaStream_t>(stream), nullptr, 0, tc ? &lp : nullptr,
                       tc ? status : nullptr, nullptr, x_host, out_host, parts,
                       static_cast<cudaEvent_t>(x_dev_free));
}

extern "C" int kym_s2d_group_uses_tc(const kym_s2d_plan* plan, int group) {
  if (!plan || group < 0 || group >= (int)plan->p.groups.size()) return -1;
  const auto& g = plan->p.groups[group];
  if (!g.tc_on) return 0;
  if (g.tcdft && kym::g_use_tcdft.load()) return 2;
  return g.has_tc ? 1 : 0;
}

extern "C" int kym_s2d_set_group_tc(kym_s2d_plan* plan, int group, int enable) {
  if (!plan || group < 0 || group >= (int)plan->p.groups.size()) return -1;
  kym::Group& g = plan->p.groups[group];
  const int prev = g.tc_on ? 1 : 0;
  g.tc_on = enable != 0;
  return prev;
}

extern "C" int kym_s2d_group_lane(const kym_s2d_plan* plan, int group) {
  if (!plan || group < 0 || group >= (int)plan->p.groups.size()) return -1;
  return plan->p.groups[group].lane;
}

extern "C" int kym_s2d_group_kernels(const kym_s2d_plan* plan, int group, int tensor_cores) {
  if (!plan || group < 0 || group >= (int)plan->p.groups.size()) return -1;
  const kym::Group& g = plan->p.groups[group];
  if (tensor_cores && g.tc_on && g.tcdft && kym::g_use_tcdft.load()) return 2;  // fold pass, GEMM kernel
  if (tensor_cores && g.tc_on && g.has_tc) return 1;
  if (g.lines) return g.L.modulus ? 4 : 3;  // rows, columns, [rows + fold], low-pass (per sub-launch, or once after them)
  return 1;
}

extern "C" int kym_s2d_group_launches(const kym_s2d_plan* plan, int group, int batch, int tensor_cores) {
  if (!plan || group < 0 || group >= (int)plan->p.groups.size() || batch < 0) return -1;
  const CascadePlan& P = plan->p;
  const kym::Group& g = P.groups[group];
  if (batch == 0) return 0;
  // chunks and line-split sub-launches as run_core forms them
  int chunk = std::max(1, std::min(batch, P.chunk));
  const int nch = (batch + chunk - 1) / chunk;
  chunk = (batch + nch - 1) / nch;
  const int k = kym_s2d_group_kernels(plan, group, tensor_cores);
  const bool fused_tc = tensor_cores && g.tc_on && (g.has_tc || (g.tcdft && kym::g_use_tcdft.load()));
  auto sub = [&](int n) {
    if (!g.lines || fused_tc) return 1;
    const double slot_bytes = (double)g.tasks.size() * g.L.mr * g.L.mc * sizeof(float2);
    const int step = (int)std::max(1.0, std::min(65535.0, 64.0 * 1024 * 1024 / slot_bytes));
    return (n + step - 1) / step;
  };
  // with several sub-launches, the low-pass kernel runs once after them
  auto per = [&](int n) {
    const int s = sub(n);
    return s > 1 ? (k - 1) * s + (n + 65534) / 65535 : k * s;
  };
  if (g.level == 0) return per(batch);
  int tot = 0;
  for (int c0 = 0; c0 < batch; c0 += chunk) tot += per(std::min(chunk, batch - c0));
  return tot;
}

extern "C" size_t kym_s2d_workspace_bytes(const kym_s2d_plan* plan, int batch) {
  if (!plan || batch < 0) return 0;
  const CascadePlan& P = plan->p;
  const int chunk = std::min(batch, P.chunk);
  const size_t spectra = ((size_t)batch * P.u0_elems + (size_t)chunk * P.u1_elems) * sizeof(float2);
  if (!P.opnd_bytes) return spectra;
  return ((spectra + 255) & ~(size_t)255) + (size_t)chunk * P.opnd_bytes;
}

namespace kym {
CascadePlan* plan_of(const kym_s2d_plan* p) { return const_cast<CascadePlan*>(&p->p); }
}  // namespace kym

extern "C" int kym_s2d_set_backward_chunk(kym_s2d_plan* plan, int chunk) {
  if (!plan || chunk < 1) return KYM_ERR_INVALID;
  plan->p.bchunk = chunk;
  return KYM_OK;
}

extern "C" size_t kym_s2d_backward_workspace_bytes(const kym_s2d_plan* plan, int batch) {
  if (!plan || batch < 0) return 0;
  return kym::backward_bytes(&plan->p, batch);
}

extern "C" int kym_s2d_backward(const kym_s2d_plan* plan, const float* x, const float* grad_out, float* grad_x,
                                int batch, const float* const* filters, int n_filters, void* workspace,
                                size_t workspace_bytes, void* stream) {
  if (!plan) return KYM_ERR_INVALID;
  return kym::run_backward(const_cast<CascadePlan*>(&plan->p), x, grad_out, grad_x, batch, filters, n_filters,
                           workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" size_t kym_s2d_saved_bytes(const kym_s2d_plan* plan, int batch) {
  if (!plan || batch < 0) return 0;
  return kym::saved_bytes(&plan->p, batch);
}

extern "C" int kym_s2d_forward_save(const kym_s2d_plan* plan, const float* x, float* out, int batch,
                                    const float* const* filters, int n_filters, void* workspace,
                                    size_t workspace_bytes, void* saved, size_t saved_bytes, void* stream) {
  if (!plan) return KYM_ERR_INVALID;
  return kym::run_forward_save(const_cast<CascadePlan*>(&plan->p), x, out, batch, filters, n_filters, workspace,
                               workspace_bytes, saved, saved_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int kym_s2d_backward_saved(const kym_s2d_plan* plan, const void* saved, size_t saved_bytes,
                                      const float* grad_out, float* grad_x, int batch, const float* const* filters,
                                      int n_filters, void* workspace, size_t workspace_bytes, void* stream) {
  if (!plan) return KYM_ERR_INVALID;
  return kym::run_backward_saved(const_cast<CascadePlan*>(&plan->p), saved, saved_bytes, grad_out, grad_x, batch,
                                 filters, n_filters, workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int kym_s2d_forward(const kym_s2d_plan* plan, const float* x, float* out, int batch,
                               const float* const* filters, int n_filters, void* workspace,
                               size_t workspace_bytes, void* stream) {
  if (!plan) return KYM_ERR_INVALID;
  return kym::run_plan(const_cast<CascadePlan*>(&plan->p), x, out, batch, filters, n_filters, workspace,
                       workspace_bytes, static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// 1-D plan
// ---------------------------------------------------------------------------
struct kym_s1d_plan {
  CascadePlan p;
};

extern "C" int kym_s1d_plan_create(int N_padded, int N_input, int pad_left, int log2_stride, int max_order,
                                   int n_psi1, const int* psi1_j, const int* psi1_nlevels, int n_psi2,
                                   const int* psi2_j, const int* psi2_nlevels, int n_phi_levels, int out_start,
                                   int out_end, kym_s1d_plan** out) {
  using namespace kym;
  if (!out) return KYM_ERR_INVALID;
  *out = nullptr;
  if (N_padded < 2 || (N_padded & (N_padded - 1)) || N_input < 1 || log2_stride < 0 ||
      (1 << log2_stride) > N_padded || max_order < 1 || max_order > 2 || n_psi1 < 0 || n_psi2 < 0 ||
      (n_psi1 && (!psi1_j || !psi1_nlevels)) || (n_psi2 && (!psi2_j || !psi2_nlevels)) || n_phi_levels < 1 ||
      out_start < 0 || out_end <= out_start || out_end > (N_padded >> log2_stride))
    return KYM_ERR_INVALID;
  auto* h = new (std::nothrow) kym_s1d_plan;
  if (!h) return KYM_ERR_CUDA;
  CascadePlan* P = &h->p;
  P->oned = true;
  P->Mp = 1;
  P->Np = N_padded;
  P->img_M = 1;
  P->img_N = N_input;
  P->pad_t = 0;
  P->pad_l = pad_left;
  P->out_nr = 1;
  P->out_nc = out_end - out_start;
  const int S = N_padded >> log2_stride;
  int rc = KYM_OK;
  // filter index layout: phi levels, psi1 levels, psi2 levels
  std::vector<int> phi_idx, psi1_first, psi2_first;
  for (int l = 0; l < n_phi_levels; ++l) {
    phi_idx.push_back((int)P->filter_rows.size());
    P->filter_rows.push_back(1);
    P->filter_cols.push_back(N_padded >> l);
  }
  for (int n = 0; n < n_psi1; ++n) {
    psi1_first.push_back((int)P->filter_rows.size());
    for (int l = 0; l < psi1_nlevels[n]; ++l) {
      P->filter_rows.push_back(1);
      P->filter_cols.push_back(N_padded >> l);
    }
  }
  for (int n = 0; n < n_psi2; ++n) {
    psi2_first.push_back((int)P->filter_rows.size());
    for (int l = 0; l < psi2_nlevels[n]; ++l) {
      P->filter_rows.push_back(1);
      P->filter_cols.push_back(N_padded >> l);
    }
  }
  if ((int)P->filter_rows.size() > kMaxFilters) {
    delete h;
    return KYM_ERR_UNSUPPORTED;
  }
  auto mk = [&](Group& g, int m, int kfold, int level, bool modulus, bool image) -> int {
    int r = make_group(P, g, 1, m, 1, kfold, 1, S, modulus, image);
    if (r) return r;
    g.level = level;
    g.L.out_r0 = 0;
    g.L.out_c0 = out_start;
    g.L.out_nr = 1;
    g.L.out_nc = P->out_nc;
    g.L.img_M = 1;
    g.L.img_N = N_input;
    g.L.pad_t = 0;
    g.L.pad_l = pad_left;
    return KYM_OK;
  };
  P->u0_elems = N_padded;
  // parents that have children, by (k1) resolution
  std::vector<long long> u1_off(n_psi1, -1);
  long long u1 = 0;
  const bool second = max_order >= 2 && n_psi2 > 0;
  int ch = 0;
  std::map<std::tuple<int, int, int>, Group> groups;  // (level, m, fold) -> group
  std::vector<std::tuple<int, int, int>> order;
  auto group_for = [&](int level, int m, int kfold, bool modulus, bool image) -> Group* {
    auto key = std::make_tuple(level, m, kfold);
    if (!groups.count(key)) {
      Group g;
      if (mk(g, m, kfold, level, modulus, image)) return nullptr;
      groups[key] = g;
      order.push_back(key);
    }
    return &groups[key];
  };
  {
    Group* g = group_for(0, N_padded, 1, false, true);
    if (!g) { rc = KYM_ERR_UNSUPPORTED; goto fail; }
    // phi level 0 with the input stage; fold factor 2^log2_stride for S
    g->tasks.push_back(Task{0, 0, -1, phi_idx[0], ch++, -1});
  }
  for (int n1 = 0; n1 < n_psi1; ++n1) {
    const int j1 = psi1_j[n1];
    const int k1 = std::min(j1, log2_stride);
    bool has_child = false;
    if (second)
      for (int n2 = 0; n2 < n_psi2; ++n2) has_child |= psi2_j[n2] > j1;
    if (has_child) {
      u1_off[n1] = u1;
      u1 += N_padded >> k1;
    }
    if (k1 >= n_phi_levels) { rc = KYM_ERR_INVALID; goto fail; }
    Group* g = group_for(1, N_padded >> k1, 1 << k1, true, false);
    if (!g) { rc = KYM_ERR_UNSUPPORTED; goto fail; }
    g->tasks.push_back(Task{0, u1_off[n1], psi1_first[n1], phi_idx[k1], ch++, -1});
  }
  if (second) {
    for (int n1 = 0; n1 < n_psi1; ++n1) {
      const int j1 = psi1_j[n1];
      const int k1 = std::min(j1, log2_stride);
      for (int n2 = 0; n2 < n_psi2; ++n2) {
        const int j2 = psi2_j[n2];
        if (j2 <= j1) continue;
        const int sub2 = std::min(j2, log2_stride);
        const int k2 = std::max(sub2 - k1, 0);
        if (k1 >= psi2_nlevels[n2] || k1 + k2 >= n_phi_levels) { rc = KYM_ERR_INVALID; goto fail; }
        Group* g = group_for(2, N_padded >> (k1 + k2), 1 << k2, true, false);
        if (!g) { rc = KYM_ERR_UNSUPPORTED; goto fail; }
        g->tasks.push_back(Task{u1_off[n1], -1, psi2_first[n2] + k1, phi_idx[k1 + k2], ch++, -1});
      }
    }
  }
  for (auto& key : order) P->groups.push_back(groups[key]);
  P->channels = ch;
  P->u1_elems = u1;
  for (auto& g : P->groups) g.L.out_channels = P->channels;
  rc = finalize_groups(P);
  if (rc) goto fail;
  rc = build_backward(P);
  if (rc) goto fail;
  attach_tc(P);
  set_default_chunk(P);
  *out = h;
  return KYM_OK;
fail:
  delete h;
  return rc;
}

extern "C" int kym_s1d_plan_destroy(kym_s1d_plan* plan) {
  delete plan;
  return KYM_OK;
}

extern "C" int kym_s1d_plan_info(const kym_s1d_plan* plan, int* channels, int* out_len, int* n_filters) {
  if (!plan) return KYM_ERR_INVALID;
  if (channels) *channels = plan->p.channels;
  if (out_len) *out_len = plan->p.out_nc;
  if (n_filters) *n_filters = (int)plan->p.filter_rows.size();
  return KYM_OK;
}

extern "C" size_t kym_s1d_workspace_bytes(const kym_s1d_plan* plan, int batch) {
  if (!plan || batch < 0) return 0;
  const CascadePlan& P = plan->p;
  const int chunk = std::min(batch, P.chunk);
  return ((size_t)batch * P.u0_elems + (size_t)chunk * P.u1_elems) * sizeof(float2);
}

extern "C" int kym_s1d_set_chunk(kym_s1d_plan* plan, int chunk) {
  if (!plan || chunk < 1) return KYM_ERR_INVALID;
  plan->p.chunk = chunk;
  return KYM_OK;
}

extern "C" size_t kym_s1d_backward_workspace_bytes(const kym_s1d_plan* plan, int batch) {
  if (!plan || batch < 0) return 0;
  return kym::backward_bytes(&plan->p, batch);
}

extern "C" int kym_s1d_backward(const kym_s1d_plan* plan, const float* x, const float* grad_out, float* grad_x,
                                int batch, const float* const* filters, int n_filters, void* workspace,
                                size_t workspace_bytes, void* stream) {
  if (!plan) return KYM_ERR_INVALID;
  return kym::run_backward(const_cast<CascadePlan*>(&plan->p), x, grad_out, grad_x, batch, filters, n_filters,
                           workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" size_t kym_s1d_saved_bytes(const kym_s1d_plan* plan, int batch) {
  if (!plan || batch < 0) return 0;
  return kym::saved_bytes(&plan->p, batch);
}

extern "C" int kym_s1d_forward_save(const kym_s1d_plan* plan, const float* x, float* out, int batch,
                                    const float* const* filters, int n_filters, void* workspace,
                                    size_t workspace_bytes, void* saved, size_t saved_bytes, void* stream) {
  if (!plan) return KYM_ERR_INVALID;
  return kym::run_forward_save(const_cast<CascadePlan*>(&plan->p), x, out, batch, filters, n_filters, workspace,
                               workspace_bytes, saved, saved_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int kym_s1d_backward_saved(const kym_s1d_plan* plan, const void* saved, size_t saved_bytes,
                                      const float* grad_out, float* grad_x, int batch, const float* const* filters,
                                      int n_filters, void* workspace, size_t workspace_bytes, void* stream) {
  if (!plan) return KYM_ERR_INVALID;
  return kym::run_backward_saved(const_cast<CascadePlan*>(&plan->p), saved, saved_bytes, grad_out, grad_x, batch,
                                 filters, n_filters, workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int kym_s1d_forward(const kym_s1d_plan* plan, const float* x, float* out, int batch,
                               const float* const* filters, int n_filters, void* workspace,
                               size_t workspace_bytes, void* stream) {
  if (!plan) return KYM_ERR_INVALID;
  return kym::run_plan(const_cast<CascadePlan*>(&plan->p), x, out, batch, filters, n_filters, workspace,
                       workspace_bytes, static_cast<cudaStream_t>(stream));
}
