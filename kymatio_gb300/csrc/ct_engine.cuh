// Compile-time specialised shared-memory FFT stages.
//
// Same in-place Stockham scheme as fft_engine.cuh (reads at stride N/R,
// twiddles exp(-+2 pi i (j mod Ns) r / (Ns R)), radix-R DFT in registers,
// writes at stride Ns), but the length, radix schedule, number of lines and
// CTA size are template parameters: every index computation folds to
// constants, loops unroll, and nothing is called through the ABI, so the
// butterflies stay in registers.
#pragma once
#include "fft_engine.cuh"

namespace kym {
namespace ct {

// ---- radix schedule, evaluated at compile time -----------------------------
__host__ __device__ constexpr int next_radix(int m) {
  if (m % 16 == 0) return 16;
  if (m % 8 == 0) return 8;
  if (m % 4 == 0) return 4;
  if (m % 2 == 0) return 2;
  for (int f = 3; f <= m; f += 2)
    if (m % f == 0) return f;
  return m;
}
__host__ __device__ constexpr int stage_count(int n) {
  int s = 0;
  for (int m = n; m > 1; m /= next_radix(m)) ++s;
  return s;
}
__host__ __device__ constexpr int stage_radix(int n, int s) {
  int m = n;
  for (int i = 0; i < s; ++i) m /= next_radix(m);
  return next_radix(m);
}

// ---- shared-memory access helpers ------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint32_t mapa(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float2 ld_dsmem(uint32_t a) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void st_dsmem(uint32_t a, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Lines are rows of a local array (pitch LD); SWZ pads one slot every 16.
template <int LD, bool SWZ>
struct RowLines {
  float2* base;
  __device__ __forceinline__ float2 ld(int line, int i) const {
    if (SWZ) i += i >> 4;
    return base[line * LD + i];
  }
  __device__ __forceinline__ void st(int line, int i, float2 v) const {
    if (SWZ) i += i >> 4;
    base[line * LD + i] = v;
  }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
};

// Lines are columns of a local array (pitch LD).
template <int LD>
struct ColLines {
  float2* base;
  __device__ __forceinline__ float2 ld(int col, int i) const { return base[i * LD + col]; }
  __device__ __forceinline__ void st(int col, int i, float2 v) const { base[i * LD + col] = v; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
};

// Lines are columns of an array whose rows are split over the cluster:
// global row i lives in CTA i / RPC at local row i % RPC.
template <int LD, int RPC>
struct ClusterColLines {
  uint32_t base;  // shared-window address of this CTA's array
  __device__ __forceinline__ uint32_t addr(int col, int i) const {
    return mapa(base + (uint32_t)(((i % RPC) * LD + col) * 8), (uint32_t)(i / RPC));
  }
  __device__ __forceinline__ float2 ld(int col, int i) const { return ld_dsmem(addr(col, i)); }
  __device__ __forceinline__ void st(int col, int i, float2 v) const { st_dsmem(addr(col, i), v); }
  __device__ __forceinline__ void sync() const { cluster_sync(); }
};

// One stage over LINES lines (line index offset line0), CTA of NT threads.
template <int N, int R, int NS, int LINES, int NT, class Lines>
__device__ __forceinline__ void stage(const Lines& L, int line0, const float2* __restrict__ tw, bool inv) {
  constexpr int BPL = N / R;                      // butterflies per line
  constexpr int CAP = (36 / R) > 0 ? (36 / R) : 1;  // butterflies per thread (register budget)
  constexpr int NEED = (BPL + NT - 1) / NT;       // a line must fit one round
  static_assert(NEED <= CAP, "line too long for the CTA at this radix");
  constexpr int TOT = LINES * BPL;
  constexpr int WANT = (TOT + NT - 1) / NT;
  constexpr int ITEMS = WANT < CAP ? (WANT > NEED ? WANT : NEED) : CAP;
  constexpr int LPR0 = (NT * ITEMS) / BPL;
  constexpr int LPR = LPR0 < LINES ? LPR0 : LINES;  // lines per round
  constexpr int ROUNDS = (LINES + LPR - 1) / LPR;
  constexpr int TSTRIDE = N / (NS * R);
  float2 cs[(R & 1) ? (R - 1) / 2 + 1 : 1];
  if constexpr (R & 1) {
#pragma unroll
    for (int m = 0; m <= (R - 1) / 2; ++m) {
      const float2 t = __ldg(tw + m * (N / R));
      cs[m] = make_float2(t.x, -t.y);
    }
  }
#pragma unroll 1
  for (int rd = 0; rd < ROUNDS; ++rd) {
    const int l0 = rd * LPR;
    const int nl = (rd == ROUNDS - 1) ? (LINES - (ROUNDS - 1) * LPR) : LPR;
    float2 v[ITEMS][R];
    int jj[ITEMS], ln[ITEMS];
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const int b = threadIdx.x + it * NT;
      // the last round may hold fewer lines; its line count is still exact
      const bool full = (rd != ROUNDS - 1) || (LINES % LPR == 0);
      const int lines_here = full ? LPR : nl;
      jj[it] = -1;
      if (b < lines_here * BPL) {
        const int j = full ? b / LPR : b / nl;
        const int l = full ? b - j * LPR : b - j * nl;
        jj[it] = j;
        ln[it] = line0 + l0 + l;
#pragma unroll
        for (int r = 0; r < R; ++r) v[it][r] = L.ld(ln[it], j + r * BPL);
      }
    }
    L.sync();
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const int j = jj[it];
      if (j >= 0) {
        const int k = j % NS;
        if constexpr (NS > 1) {
#pragma unroll
          for (int r = 1; r < R; ++r) v[it][r] = cmul(v[it][r], conj_if(__ldg(tw + k * r * TSTRIDE), inv));
        }
        dft_any<R>(v[it], cs, inv);
        const int o = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) L.st(ln[it], o + r * NS, v[it][r]);
      }
    }
    if (rd + 1 < ROUNDS) {
      // the next round works on other lines: no barrier needed here
    }
  }
  L.sync();
}

template <int N, int S, int NS, int LINES, int NT, class Lines>
__device__ __forceinline__ void stages(const Lines& L, int line0, const float2* __restrict__ tw, bool inv) {
  if constexpr (S < stage_count(N)) {
    constexpr int R = stage_radix(N, S);
    stage<N, R, NS, LINES, NT, Lines>(L, line0, tw, inv);
    stages<N, S + 1, NS * R, LINES, NT, Lines>(L, line0, tw, inv);
  }
}

// Full 1-D transform of length N over LINES lines.
template <int N, int LINES, int NT, class Lines>
__device__ __forceinline__ void fft_lines(const Lines& L, int line0, const float2* __restrict__ tw, bool inv) {
  stages<N, 0, 1, LINES, NT, Lines>(L, line0, tw, inv);
}

}  // namespace ct
}  // namespace kym
