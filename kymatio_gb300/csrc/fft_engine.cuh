// Shared-memory mixed-radix FFT engine for the scattering cascade (sm_103a).
//
// A 2-D work array of complex fp32 lives in shared memory, either in one CTA
// or split by row slabs over the CTAs of a thread-block cluster (distributed
// shared memory).  Transforms run as in-place Stockham auto-sort stages
// (Govindaraju et al., "High performance discrete Fourier transforms on
// graphics processors", SC 2008): each stage reads R elements at stride n/R,
// applies the twiddles exp(-+2 pi i (j mod Ns) r / (Ns R)), runs a radix-R DFT
// in registers and writes the outputs at stride Ns.  Every thread holds its
// butterflies in registers between a barrier after the reads and the writes,
// so one buffer suffices.  Radices 2, 4, 8, 16 are hand-written; odd primes
// use the symmetric pair form (real/imag cosines and sines shared between
// outputs k and R-k).
//
// Direction: forward uses exp(-2 pi i k/n) (numpy/torch fft convention),
// inverse the conjugate; no normalisation is applied here.
#pragma once
#include <cuda_runtime.h>
#include <cooperative_groups.h>
#include <stdint.h>

namespace kym {

namespace cg = cooperative_groups;

constexpr int kMaxStages = 16;
constexpr int kThreads = 512;     // CTA size of the cascade kernels

// One axis of a transform: its length and radix schedule.  ``tw`` points to
// a device table exp(-2 pi i k / n), k in [0, n), built in FP64 on the host.
struct FftPlan {
  int n;
  int nstages;
  int radix[kMaxStages];
  const float2* tw;
};

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// a * (-i) for the forward direction, a * (+i) for the inverse
__device__ __forceinline__ float2 rot_q(float2 a, bool inv) {
  return inv ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
__device__ __forceinline__ float2 conj_if(float2 w, bool inv) { return inv ? make_float2(w.x, -w.y) : w; }

// ---------------------------------------------------------------------------
// radix kernels (in registers)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void dft2(float2& a, float2& b) {
  float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3, bool inv) {
  float2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
  float2 t2 = cadd(a1, a3), t3 = rot_q(csub(a1, a3), inv);
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

// exp(-2 pi i m / 16) for m in [0, 16), conjugated for the inverse.
__device__ __forceinline__ float2 w16(int m, bool inv) {
  constexpr float C[16] = {1.f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508978f,
                           0.f, -0.38268343236508978f, -0.70710678118654752f, -0.92387953251128674f,
                           -1.f, -0.92387953251128674f, -0.70710678118654752f, -0.38268343236508978f,
                           0.f, 0.38268343236508978f, 0.70710678118654752f, 0.92387953251128674f};
  float s = C[(m + 12) & 15];  // sin(2 pi m/16) = cos(2 pi (m - 4)/16)
  return make_float2(C[m & 15], inv ? s : -s);
}

// Composite radix R = R1 * R2 with R1 = 4 (inner DFT-4 over n1, stride R2),
// twiddle W_R^{n2 k1}, outer DFT over n2.  Output k = k1 + 4 k2.
template <int R2>
__device__ __forceinline__ void dft4xR2(float2 (&v)[4 * R2], bool inv);

template <>
__device__ __forceinline__ void dft4xR2<2>(float2 (&v)[8], bool inv) {
  // n = 2 n1 + n2: inner DFT-4 over n1 for n2 = 0, 1
#pragma unroll
  for (int n2 = 0; n2 < 2; ++n2) dft4(v[n2], v[2 + n2], v[4 + n2], v[6 + n2], inv);
  // now v[2 k1 + n2] = Y[n2][k1]; twiddle W8^{n2 k1} = W16^{2 n2 k1}
#pragma unroll
  for (int k1 = 1; k1 < 4; ++k1) v[2 * k1 + 1] = cmul(v[2 * k1 + 1], w16(2 * k1, inv));
  float2 o[8];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 a = v[2 * k1], b = v[2 * k1 + 1];
    dft2(a, b);
    o[k1] = a;
    o[k1 + 4] = b;
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = o[i];
}

template <>
__device__ __forceinline__ void dft4xR2<4>(float2 (&v)[16], bool inv) {
  // n = 4 n1 + n2
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4(v[n2], v[4 + n2], v[8 + n2], v[12 + n2], inv);
#pragma unroll
  for (int k1 = 1; k1 < 4; ++k1)
#pragma unroll
    for (int n2 = 1; n2 < 4; ++n2) v[4 * k1 + n2] = cmul(v[4 * k1 + n2], w16(n2 * k1, inv));
  float2 o[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 a0 = v[4 * k1], a1 = v[4 * k1 + 1], a2 = v[4 * k1 + 2], a3 = v[4 * k1 + 3];
    dft4(a0, a1, a2, a3, inv);
    o[k1] = a0;
    o[k1 + 4] = a1;
    o[k1 + 8] = a2;
    o[k1 + 12] = a3;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = o[i];
}

// Odd prime R: symmetric pair form.  cs[m] = (cos 2 pi m/R, sin 2 pi m/R),
// m in [1, (R-1)/2].
template <int R>
__device__ __forceinline__ void dft_odd(float2 (&v)[R], const float2 (&cs)[(R - 1) / 2 + 1], bool inv) {
  constexpr int H = (R - 1) / 2;
  float2 s[H], d[H];
  const float2 x0 = v[0];
  float2 X0 = x0;
#pragma unroll
  for (int n = 1; n <= H; ++n) {
    s[n - 1] = cadd(v[n], v[R - n]);
    d[n - 1] = csub(v[n], v[R - n]);
    X0 = cadd(X0, s[n - 1]);
  }
  v[0] = X0;
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    float2 A = x0, B = make_float2(0.f, 0.f);
#pragma unroll
    for (int n = 1; n <= H; ++n) {
      const int m = (n * k) % R;
      const float c = (m <= H) ? cs[m].x : cs[R - m].x;
      const float sn = (m <= H) ? cs[m].y : -cs[R - m].y;
      A.x = fmaf(s[n - 1].x, c, A.x);
      A.y = fmaf(s[n - 1].y, c, A.y);
      B.x = fmaf(d[n - 1].x, sn, B.x);
      B.y = fmaf(d[n - 1].y, sn, B.y);
    }
    // forward: X_k = A - iB, X_{R-k} = A + iB ; inverse swaps them
    float2 p = make_float2(A.x + B.y, A.y - B.x);
    float2 q = make_float2(A.x - B.y, A.y + B.x);
    v[k] = inv ? q : p;
    v[R - k] = inv ? p : q;
  }
}

template <int R>
struct Radix {
  static constexpr bool kOdd = (R & 1) != 0;
};

template <int R>
__device__ __forceinline__ void dft_any(float2 (&v)[R], const float2* cs, bool inv);

template <>
__device__ __forceinline__ void dft_any<2>(float2 (&v)[2], const float2*, bool) { dft2(v[0], v[1]); }
template <>
__device__ __forceinline__ void dft_any<4>(float2 (&v)[4], const float2*, bool inv) {
  dft4(v[0], v[1], v[2], v[3], inv);
}
template <>
__device__ __forceinline__ void dft_any<8>(float2 (&v)[8], const float2*, bool inv) { dft4xR2<2>(v, inv); }
template <>
__device__ __forceinline__ void dft_any<16>(float2 (&v)[16], const float2*, bool inv) { dft4xR2<4>(v, inv); }

#define KYM_ODD_RADIX(R)                                                                  \
  template <>                                                                             \
  __device__ __forceinline__ void dft_any<R>(float2(&v)[R], const float2* cs_in, bool inv) { \
    float2 cs[(R - 1) / 2 + 1];                                                           \
    _Pragma("unroll") for (int m = 0; m <= (R - 1) / 2; ++m) cs[m] = cs_in[m];            \
    dft_odd<R>(v, cs, inv);                                                               \
  }
KYM_ODD_RADIX(3)
KYM_ODD_RADIX(5)
KYM_ODD_RADIX(7)
KYM_ODD_RADIX(11)
KYM_ODD_RADIX(13)
KYM_ODD_RADIX(17)
KYM_ODD_RADIX(19)
KYM_ODD_RADIX(23)
#undef KYM_ODD_RADIX

// ---------------------------------------------------------------------------
// Work-array views
// ---------------------------------------------------------------------------

// A (rows x cols) complex array split by row slabs over `nct` CTAs.  Row g
// lives in CTA g / rows_local at local row g % rows_local.  ``rowp`` is a
// shared-memory table of generic pointers (valid across the cluster) to the
// start of every global row.  ``ld`` is the row pitch in complex elements;
// it is odd so that line-fastest thread mappings are bank-conflict free.
struct Slab {
  float2* local;
  float2* const* rowp;
  int rows, cols, ld;
  int rows_local, row0;
  int nct, rank;
};

struct Barrier {
  bool cluster;
  __device__ __forceinline__ void sync() const {
    if (cluster) cg::this_cluster().sync();
    else __syncthreads();
  }
};

// ---------------------------------------------------------------------------
// One Stockham stage over a set of lines.
//   ROWS=true : lines are this CTA's local rows (length cols); element i of
//               line l at local[l*ld + i] (i + (i>>4) when SWZ, used for the
//               single long line of the 1-D transform).
//   ROWS=false: lines are columns [line0, line0+nlines) (length rows).  With
//               CL the column spans the cluster and element i of column c is
//               rowp[i][c]; otherwise local[i*ld + c].
// Each thread owns up to ITEMS butterflies per round; rounds cover whole
// lines, so all reads of a line precede all its writes (in place).  The host
// guarantees n/R <= ITEMS * blockDim.x.
// ---------------------------------------------------------------------------
template <bool ROWS, bool SWZ, bool CL>
__device__ __forceinline__ float2* elem_ptr(const Slab& w, int line, int i) {
  if constexpr (ROWS) {
    if (SWZ) i += i >> 4;
    return w.local + (size_t)line * w.ld + i;
  } else if constexpr (CL) {
    return w.rowp[i] + line;
  } else {
    return w.local + (size_t)i * w.ld + line;
  }
}

template <int R, int ITEMS, bool ROWS, bool SWZ, bool CL>
__device__ __noinline__ void fft_stage(const Slab w, int nlines, int line0, int n, int Ns,
                                          const float2* __restrict__ tw, bool inv, const Barrier bar) {
  const int bpl = n / R;
  const int nthr = blockDim.x;
  int lpr = (nthr * ITEMS) / bpl;
  if (lpr < 1) lpr = 1;
  const int tstride = n / (Ns * R);
  float2 cs[Radix<R>::kOdd ? (R - 1) / 2 + 1 : 1];
  if constexpr (Radix<R>::kOdd) {
#pragma unroll
    for (int m = 0; m <= (R - 1) / 2; ++m) {
      float2 t = __ldg(tw + m * (n / R));
      cs[m] = make_float2(t.x, -t.y);  // the table holds exp(-i theta)
    }
  }
  const int rounds = (nlines + lpr - 1) / lpr;
  for (int rd = 0; rd < rounds; ++rd) {
    const int l0 = rd * lpr;
    const int nl = min(lpr, nlines - l0);
    const int nbf = nl * bpl;
    float2 v[ITEMS][R];
    int jj[ITEMS], ln[ITEMS];
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const int b = threadIdx.x + it * nthr;
      jj[it] = -1;
      ln[it] = 0;
      if (b < nbf) {
        ln[it] = line0 + l0 + b % nl;
        jj[it] = b / nl;
#pragma unroll
        for (int r = 0; r < R; ++r) v[it][r] = *elem_ptr<ROWS, SWZ, CL>(w, ln[it], jj[it] + r * bpl);
      }
    }
    bar.sync();
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const int j = jj[it];
      if (j >= 0) {
        const int k = j % Ns;
        if (Ns > 1) {
#pragma unroll
          for (int r = 1; r < R; ++r) v[it][r] = cmul(v[it][r], conj_if(__ldg(tw + k * r * tstride), inv));
        }
        dft_any<R>(v[it], cs, inv);
        const int o = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) *elem_ptr<ROWS, SWZ, CL>(w, ln[it], o + r * Ns) = v[it][r];
      }
    }
  }
  bar.sync();
}

// Fallback for prime radices without a specialisation (R <= 127): direct
// DFT from a local-memory copy.  One butterfly per thread per round.
template <bool ROWS, bool SWZ, bool CL>
__device__ __noinline__ void fft_stage_generic(const Slab w, int nlines, int line0, int n, int Ns, int R,
                                               const float2* __restrict__ tw, bool inv, const Barrier bar) {
  const int bpl = n / R;
  const int nthr = blockDim.x;
  int lpr = nthr / bpl;
  if (lpr < 1) lpr = 1;
  const int tstride = n / (Ns * R);
  const int step = n / R;  // W_R^q = W_n^(q n / R)
  const int rounds = (nlines + lpr - 1) / lpr;
  float2 v[128];
  for (int rd = 0; rd < rounds; ++rd) {
    const int l0 = rd * lpr;
    const int nl = min(lpr, nlines - l0);
    const int b = threadIdx.x;
    int line = 0, j = -1;
    if (b < nl * bpl) {
      line = line0 + l0 + b % nl;
      j = b / nl;
      for (int r = 0; r < R; ++r) v[r] = *elem_ptr<ROWS, SWZ, CL>(w, line, j + r * bpl);
    }
    bar.sync();
    if (j >= 0) {
      const int k = j % Ns;
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], conj_if(__ldg(tw + k * r * tstride), inv));
      const int o = (j / Ns) * Ns * R + k;
      for (int q = 0; q < R; ++q) {
        float2 acc = make_float2(0.f, 0.f);
        for (int r = 0; r < R; ++r) acc = cadd(acc, cmul(v[r], conj_if(__ldg(tw + ((q * r) % R) * step), inv)));
        *elem_ptr<ROWS, SWZ, CL>(w, line, o + q * Ns) = acc;
      }
    }
  }
  bar.sync();
}

// Run every stage of `p` over lines [line0, line0+nlines) of one axis.
template <bool ROWS, bool SWZ, bool CL>
__device__ __noinline__ void fft_pass(const Slab w, int nlines, int line0, const FftPlan p, bool inv,
                                      const Barrier bar) {
  int Ns = 1;
  const int nthr = blockDim.x;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s];
    const int items = (p.n / R + nthr - 1) / nthr;  // >1 only for long 1-D lines
#define KYM_STAGE(RR, IT) fft_stage<RR, IT, ROWS, SWZ, CL>(w, nlines, line0, p.n, Ns, p.tw, inv, bar)
    switch (R) {
      case 2:
        if (items <= 1) KYM_STAGE(2, 1);
        else if (items <= 2) KYM_STAGE(2, 2);
        else if (items <= 4) KYM_STAGE(2, 4);
        else if (items <= 8) KYM_STAGE(2, 8);
        else KYM_STAGE(2, 16);
        break;
      case 4:
        if (items <= 1) KYM_STAGE(4, 1);
        else if (items <= 2) KYM_STAGE(4, 2);
        else if (items <= 4) KYM_STAGE(4, 4);
        else KYM_STAGE(4, 8);
        break;
      case 8:
        if (items <= 1) KYM_STAGE(8, 1);
        else if (items <= 2) KYM_STAGE(8, 2);
        else KYM_STAGE(8, 4);
        break;
      case 16:
        if (items <= 1) KYM_STAGE(16, 1);
        else KYM_STAGE(16, 2);
        break;
      case 3: KYM_STAGE(3, 1); break;
      case 5: KYM_STAGE(5, 1); break;
      case 7: KYM_STAGE(7, 1); break;
      case 11: KYM_STAGE(11, 1); break;
      case 13: KYM_STAGE(13, 1); break;
      case 17: KYM_STAGE(17, 1); break;
      case 19: KYM_STAGE(19, 1); break;
      case 23: KYM_STAGE(23, 1); break;
      default: fft_stage_generic<ROWS, SWZ, CL>(w, nlines, line0, p.n, Ns, R, p.tw, inv, bar); break;
    }
#undef KYM_STAGE
    Ns *= R;
  }
}

}  // namespace kym
