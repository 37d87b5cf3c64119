/*
 * kymatio_gb300 -- C ABI of the GB300 scattering engine (sm_103a).
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*, a cudaStream_t; NULL is the legacy default stream), is
 * enqueued asynchronously on that stream, and returns an int status
 * (KYM_OK = 0).  No exception crosses this boundary.  The caller owns every
 * buffer: inputs, outputs, filters and workspaces are allocated by the caller
 * (the Python frontend allocates them with torch on the current device).
 * Tensors are contiguous, C order, float32; complex data is interleaved
 * (re, im) pairs, i.e. the reference's trailing dimension of 2.
 *
 * Plans are host objects holding the transform geometry; they upload small
 * task/twiddle tables to each device on first use and are safe to share
 * between threads and streams.
 */
#ifndef KYMATIO_GB300_H
#define KYMATIO_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KYM_OK 0
#define KYM_ERR_INVALID 1     /* bad argument, shape or pointer */
#define KYM_ERR_UNSUPPORTED 2 /* geometry the kernels cannot run (e.g. too large for shared memory) */
#define KYM_ERR_CUDA 3        /* a CUDA call failed (launch, copy, allocation of plan tables) */
#define KYM_ERR_WORKSPACE 4   /* workspace missing or smaller than required */

/* Library version, "major.minor.patch". */
const char* kym_version(void);
/* Message for the last CUDA error this thread saw inside the library. */
const char* kym_last_error(void);
/* Plans created after this call use the compile-time specialised kernels for
 * the sizes that have one (enable=1, the default) or the runtime-planned
 * kernels everywhere (enable=0, for cross-checks).  Returns the previous
 * setting. */
int kym_set_specialized(int enable);

/* In kym_s2d_forward_tc, run the small childless groups that have one
 * (68x68 at 256x256 J=3) in the DFT-GEMM form: the inverse 2-D DFT and the
 * low-pass product as split-precision tcgen05 GEMMs (enable=1), or in the
 * low-pass-only tensor-core form (enable=0, the default).  Takes effect at the
 * next call.  Returns the previous setting.  No counterpart in the
 * reference (a form of kymatio/scattering2d/core/scattering2d.py:48-75). */
int kym_set_tc_dft(int enable);

/* Forwards after this call run the launch groups that do not depend on the
 * heaviest order-1 scale (the other order-1 scales that have children, and
 * their order-2 groups) on a side stream of the plan, forked from and joined
 * back to the caller's stream around every chunk, so that their blocks fill
 * the SMs the main chain leaves idle (enable=1, the default), or every group
 * on the caller's stream (enable=0).  Results are identical either way.
 * Timed forwards and the DFT-GEMM form run on one stream.  The side stream
 * (and the copy streams of kym_s2d_forward_host) belong to the plan and are
 * shared by its callers: forwards of one plan from several host threads stay
 * correct, but while one thread captures a CUDA graph from a plan, another
 * must not run a forward of that plan.  Returns the previous setting.  No
 * counterpart in the reference. */
int kym_set_side_lane(int enable);

/* ------------------------------------------------------------------------
 * 2-D scattering (replaces the forward of ScatteringTorch2D,
 * kymatio/scattering2d/frontend/torch_frontend.py:72-111, driving
 * kymatio/scattering2d/core/scattering2d.py:1-88 over the op surface of
 * kymatio/scattering2d/backend/torch_backend.py:89-180).
 * ---------------------------------------------------------------------- */
typedef struct kym_s2d_plan kym_s2d_plan;

/* Geometry of ScatteringBase2D.build (kymatio/scattering2d/frontend/
 * base_frontend.py:19-32): padding to ((M+2^J)//2^J+1)*2^J.  Returns
 * KYM_ERR_INVALID when 2^J exceeds M or N (the reference raises
 * 'The smallest dimension should be larger than 2^J.'). */
int kym_s2d_plan_create(int M, int N, int J, int L, int max_order, int pre_pad, kym_s2d_plan** plan);
int kym_s2d_plan_destroy(kym_s2d_plan* plan);
/* Padded size, output channel count C = 1 + JL + L^2 J(J-1)/2 (max_order 2),
 * output spatial size and the number of filters the forward expects. */
int kym_s2d_plan_info(const kym_s2d_plan* plan, int* M_padded, int* N_padded, int* channels, int* out_rows,
                      int* out_cols, int* n_filters);
/* Shape of filter `index` in the order of the reference's registered buffers
 * tensor0..tensorK (kymatio/scattering2d/frontend/torch_frontend.py:28-43):
 * phi levels 0..J-1, then every psi's levels. */
int kym_s2d_filter_shape(const kym_s2d_plan* plan, int index, int* rows, int* cols);
/* Images per pass over the order-2 cascade (sizes the parent-spectrum workspace). */
int kym_s2d_set_chunk(kym_s2d_plan* plan, int chunk);
int kym_s2d_get_chunk(const kym_s2d_plan* plan);
size_t kym_s2d_workspace_bytes(const kym_s2d_plan* plan, int batch);
/* The forward runs as launch groups (input stage, one per order-1 scale, one
 * per order-2 scale pair); these describe them: level 0/1/2, tasks per
 * image, work size, fold factor from the parent spectrum, CTAs per task
 * (negative when the group runs the runtime-planned kernel). */
int kym_s2d_group_count(const kym_s2d_plan* plan);
int kym_s2d_group_info(const kym_s2d_plan* plan, int group, int* level, int* ntasks, int* rows, int* cols, int* fold,
                       int* cluster);
/* kym_s2d_forward with CUDA events around every launch; group_ms[g] receives
 * the summed device time of group g (synchronises the stream). */
int kym_s2d_forward_timed(const kym_s2d_plan* plan, const float* x, float* out, int batch, const float* const* filters,
                          int n_filters, void* workspace, size_t workspace_bytes, void* stream, float* group_ms,
                          int max_groups);
/* x: (batch, M, N) (or the padded size when pre_pad); out: (batch, C, out_rows,
 * out_cols); filters: host array of n_filters device pointers (real Fourier
 * filters, the reference's tensor{n} buffers without their trailing dim). */
int kym_s2d_forward(const kym_s2d_plan* plan, const float* x, float* out, int batch, const float* const* filters,
                    int n_filters, void* workspace, size_t workspace_bytes, void* stream);

/* Tensor-core split-precision forward (the reference has no counterpart; it
 * computes the same transform as kym_s2d_forward).  Every childless path
 * (order 2, and the last order-1 scale) runs its low-pass branch as the
 * separable product S = T_r U T_c^T: U T_c^T on tcgen05 from BF16 hi/lo
 * operands with FP32 accumulation, T_r (.) in FP32.  lowpass_rows[j] /
 * lowpass_cols[j] are the float32 factors (out_rows x M_padded/2^j and
 * out_cols x N_padded/2^j) of low-pass filter j; *status (device) gets bit 1
 * if a tensor-core completion wait ran out.  group_ms/max_groups as in
 * kym_s2d_forward_timed (pass NULL/0 to skip timing). */
int kym_s2d_forward_tc(const kym_s2d_plan* plan, const float* x, float* out, int batch, const float* const* filters,
                       int n_filters, const float* const* lowpass_rows, const float* const* lowpass_cols,
                       int n_lowpass, void* workspace, size_t workspace_bytes, unsigned* status, void* stream,
                       float* group_ms, int max_groups);
/* End-to-end forward between host buffers: x_host (batch, M, N) in,
 * out_host (batch, C, out_rows, out_cols) out, through the caller's device
 * buffers x_dev / out_dev of the same sizes.  The input is copied in `parts`
 * slices on a copy stream of the plan and the input stage of each slice starts
 * as it lands; each launch group's output channels are copied back on a second
 * copy stream as soon as the group has finished, so the transfers overlap the
 * cascade (host buffers page-locked; pageable ones give the same result
 * without the overlap).  lowpass_rows / lowpass_cols / status as in
 * kym_s2d_forward_tc select the tensor-core form; all three NULL the plain
 * form.  The input copy starts once the work already on `stream` is done, or,
 * when x_dev_free (a cudaEvent_t) is given, once that event has completed: a
 * caller that rotates two staging buffers passes the event it recorded after
 * the previous call on the same buffers (x_dev and out_dev), and the copy
 * then overlaps the cascade of the call in between.  Ordered on `stream`: work enqueued there
 * after this call sees out_host complete.  No counterpart in the reference,
 * whose frontend takes tensors on the module's device (kymatio/scattering2d/
 * frontend/torch_frontend.py:72-111). */
int kym_s2d_forward_host(const kym_s2d_plan* plan, const float* x_host, float* out_host, int batch,
                         const float* const* filters, int n_filters, const float* const* lowpass_rows,
                         const float* const* lowpass_cols, int n_lowpass, unsigned* status, float* x_dev,
                         float* out_dev, void* workspace, size_t workspace_bytes, int parts, void* x_dev_free,
                         void* stream);
/* Tensor-core form of launch group `group` in kym_s2d_forward_tc: 0 none
 * (FP32 kernel), 1 the low-pass product on tcgen05, 2 the DFT-GEMM form. */
int kym_s2d_group_uses_tc(const kym_s2d_plan* plan, int group);
/* Let kym_s2d_forward_tc run group `group` in its tensor-core kernel
 * (enable=1, the default) or in the plain FP32 kernel (enable=0; the plain
 * form is the more precise, so the result stays within the tensor-core form's
 * bar).  Used by the autotuner, which times both per group.  Returns the
 * previous setting, or -1 for a bad group.  No counterpart in the reference. */
int kym_s2d_set_group_tc(kym_s2d_plan* plan, int group, int enable);
/* Kernels that group `group` launches per chunk of images: 1 for a fused
 * cascade kernel; 3 or 4 for the line-split passes of the sizes above one
 * CTA, per sub-launch (a sub-launch covers as many images as keep the
 * group's spectrum slots within 64 MiB; with several sub-launches the
 * low-pass kernel runs once after them) (tensor_cores != 0: in
 * kym_s2d_forward_tc).  No counterpart in the reference (profiling). */
int kym_s2d_group_kernels(const kym_s2d_plan* plan, int group, int tensor_cores);
/* Kernel launches of group `group` in one forward over `batch` images (its
 * chunks and line-split sub-launches; tensor_cores as above).  No
 * counterpart in the reference (profiling). */
int kym_s2d_group_launches(const kym_s2d_plan* plan, int group, int batch, int tensor_cores);
/* Launch lane of group `group` in the forward (0: the caller's stream, 1: the
 * plan's side stream, see kym_set_side_lane), or -1 for a bad group.  No
 * counterpart in the reference (introspection). */
int kym_s2d_group_lane(const kym_s2d_plan* plan, int group);

/* Device build of the 2-D filter bank (replaces the host construction of
 * kymatio/scattering2d/filter_bank.py:5-175 called by ScatteringBase2D.
 * create_filters, kymatio/scattering2d/frontend/base_frontend.py:34-36):
 * the Gaussian low-pass phi and the J x L Morlet wavelets at the padded size,
 * every level cropped by the masked alias sum, computed in FP64 on the device
 * and rounded once to float32.  `out` receives
 * kym_s2d_filter_bank_floats() floats: the levels of phi, then of every psi
 * (j-major, theta-minor), each level row-major -- the order of the
 * reference's tensor{n} buffers.  The values agree with the reference's
 * complex64 build to float32 rounding, not bit for bit. */
long long kym_s2d_filter_bank_floats(int M_padded, int N_padded, int J, int L);
size_t kym_s2d_filter_bank_workspace_bytes(int M_padded, int N_padded, int J, int L);
int kym_s2d_filter_bank(int M_padded, int N_padded, int J, int L, float* out, long long out_floats, void* workspace,
                        size_t workspace_bytes, void* stream);

/* Hand-written backward: grad_x (batch, M, N) = (d forward / d x)^T grad_out,
 * grad_out shaped like the forward's output.  Replaces torch autograd through
 * the reference op surface (unpad, irfft, subsample_fourier, cdgmm, rfft,
 * ModulusStable.backward of kymatio/backend/torch_backend.py:85-96, ifft,
 * ReflectionPad2d).  Recomputes the input and parent spectra chunk by chunk
 * into the workspace (kym_s2d_backward_workspace_bytes). */
size_t kym_s2d_backward_workspace_bytes(const kym_s2d_plan* plan, int batch);
/* Images per backward pass (bounds its workspace: the recomputed input and
 * parent spectra and the per-path gradient blocks of one chunk; by default
 * as many images as fit 1 GiB). */
int kym_s2d_set_backward_chunk(kym_s2d_plan* plan, int chunk);
int kym_s2d_backward(const kym_s2d_plan* plan, const float* x, const float* grad_out, float* grad_x, int batch,
                     const float* const* filters, int n_filters, void* workspace, size_t workspace_bytes,
                     void* stream);

/* Saved-activation form of the forward/backward pair (what torch autograd
 * does with the reference's op graph: the forward keeps what the backward
 * needs, kymatio/backend/torch_backend.py:85-96 saves the modulus input).
 * kym_s2d_forward_save computes exactly kym_s2d_forward's output and also
 * stores every order-1 and order-2 path's modulus input y = IFFT2(...)
 * (complex64) into `saved` (kym_s2d_saved_bytes(plan, batch) bytes);
 * kym_s2d_backward_saved then needs neither x nor any recomputation.  The
 * frontend picks this form while batch x saved bytes per image stays under
 * its activation budget, and the recomputing kym_s2d_backward above it. */
size_t kym_s2d_saved_bytes(const kym_s2d_plan* plan, int batch);
int kym_s2d_forward_save(const kym_s2d_plan* plan, const float* x, float* out, int batch,
                         const float* const* filters, int n_filters, void* workspace, size_t workspace_bytes,
                         void* saved, size_t saved_bytes, void* stream);
int kym_s2d_backward_saved(const kym_s2d_plan* plan, const void* saved, size_t saved_bytes, const float* grad_out,
                           float* grad_x, int batch, const float* const* filters, int n_filters, void* workspace,
                           size_t workspace_bytes, void* stream);

/* Allocation-free forward.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory (a fixed memory pool reserved up
 * front, a host application that forbids allocation after start-up).  It
 * computes exactly what kym_s2d_forward computes, but needs no workspace
 * argument: the plan's tables and the spectra of one chunk of images live in
 * a static device array of KYM_NOALLOC_SCRATCH_BYTES inside the library,
 * which every GPU that loads the library holds until the process exits.  It
 * calls no cudaMalloc, cudaFree or allocating library routine.
 *   - The first call on a device looks the array's address up
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *   - Every call shares the one array: calls that overlap on the GPU (on
 *     different streams, or from different threads) race and corrupt each
 *     other's results; serialise them on one stream.
 *   - Returns KYM_ERR_WORKSPACE when one image's spectra plus the plan's tables
 *     exceed the array (kym_last_error() gives the sizes). */
#define KYM_NOALLOC_SCRATCH_BYTES (32u << 20)
int kym_s2d_forward_noalloc(const kym_s2d_plan* plan, const float* x, float* out, int batch,
                            const float* const* filters, int n_filters, void* stream);

/* Self-test of the tcgen05 split-precision GEMM (no reference counterpart):
 * D (M x N) = A (M x K) * B (N x K)^T from bf16 hi/lo operands with FP32
 * accumulation in tensor memory, one M=128 tile; M <= 128, N in
 * {16, 32, 48, 64}, K <= 256.  *status gets bit 1 if the completion wait ran
 * out (the result is then not written). */
int kym_tc_selftest(const float* A, const float* B, float* D, int M, int N, int K, unsigned* status, void* stream);

/* ------------------------------------------------------------------------
 * 1-D scattering, local averaging (replaces ScatteringBase1D.scattering with
 * average='local', kymatio/scattering1d/frontend/base_frontend.py:106-155,
 * and kymatio/scattering1d/core/scattering1d.py:2-107 over
 * kymatio/scattering1d/backend/torch_backend.py:18-141).  The geometry comes
 * from the frontend's build(): padded length (a power of two), reflect pad,
 * log2 of the stride, the j of every first/second-order wavelet and its
 * number of levels, and the unpad window at the output resolution.
 * ---------------------------------------------------------------------- */
typedef struct kym_s1d_plan kym_s1d_plan;

int kym_s1d_plan_create(int N_padded, int N_input, int pad_left, int log2_stride, int max_order, int n_psi1,
                        const int* psi1_j, const int* psi1_nlevels, int n_psi2, const int* psi2_j,
                        const int* psi2_nlevels, int n_phi_levels, int out_start, int out_end,
                        kym_s1d_plan** plan);
int kym_s1d_plan_destroy(kym_s1d_plan* plan);
int kym_s1d_plan_info(const kym_s1d_plan* plan, int* channels, int* out_len, int* n_filters);
int kym_s1d_set_chunk(kym_s1d_plan* plan, int chunk);
size_t kym_s1d_workspace_bytes(const kym_s1d_plan* plan, int batch);
/* x: (batch, N_input); out: (batch, channels, out_len); filters ordered as
 * the reference's tensor{n} buffers (phi levels, psi1 levels, psi2 levels,
 * kymatio/scattering1d/frontend/torch_frontend.py:30-56). */
int kym_s1d_forward(const kym_s1d_plan* plan, const float* x, float* out, int batch, const float* const* filters,
                    int n_filters, void* workspace, size_t workspace_bytes, void* stream);
/* Backward of kym_s1d_forward (ModulusStable.backward and the adjoints of the
 * 1-D op surface, kymatio/scattering1d/backend/torch_backend.py:18-141). */
size_t kym_s1d_backward_workspace_bytes(const kym_s1d_plan* plan, int batch);
int kym_s1d_backward(const kym_s1d_plan* plan, const float* x, const float* grad_out, float* grad_x, int batch,
                     const float* const* filters, int n_filters, void* workspace, size_t workspace_bytes,
                     void* stream);
/* Saved-activation form, as kym_s2d_saved_bytes / _forward_save / _backward_saved. */
size_t kym_s1d_saved_bytes(const kym_s1d_plan* plan, int batch);
int kym_s1d_forward_save(const kym_s1d_plan* plan, const float* x, float* out, int batch,
                         const float* const* filters, int n_filters, void* workspace, size_t workspace_bytes,
                         void* saved, size_t saved_bytes, void* stream);
int kym_s1d_backward_saved(const kym_s1d_plan* plan, const void* saved, size_t saved_bytes, const float* grad_out,
                           float* grad_x, int batch, const float* const* filters, int n_filters, void* workspace,
                           size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Operator surface (float32, interleaved complex), for driving the reference
 * frontend and core op by op.  batch counts the leading dimensions.
 * ---------------------------------------------------------------------- */
/* Batched 2-D DFT of M x N images (M = 1: 1-D lines of length N).  in_real:
 * input is real (trailing dim 1); out_real: write the real part only; inverse:
 * conjugate direction; every output is multiplied by scale.
 * rfft = (in_real, !out_real, fwd, 1); ifft = (!in_real, !out_real, inv,
 * 1/(MN)); irfft = (!in_real, out_real, inv, 1/(MN)).  Replaces
 * TorchBackend2D.rfft/ifft/irfft (kymatio/scattering2d/backend/torch_backend.py:
 * 131-155) and TorchBackend1D.rfft/ifft/irfft/cfft
 * (kymatio/scattering1d/backend/torch_backend.py:108-141). */
int kym_op_fft2(const float* in, float* out, int batch, int M, int N, int in_real, int out_real, int inverse,
                float scale, void* stream);
/* C[b, i] = A[b, i] * B[i] for i < n (B real, or complex when b_complex):
 * TorchBackend.cdgmm (kymatio/backend/torch_backend.py:147-219). */
int kym_op_cdgmm(const float* A, const float* B, float* C, long long batch, long long n, int b_complex, void* stream);
/* |x| and its adjoint x g / |x| (0 where |x| = 0): ModulusStable
 * (kymatio/backend/torch_backend.py:5-96). */
int kym_op_modulus(const float* x, float* y, long long n, void* stream);
int kym_op_modulus_backward(const float* x, const float* g, float* gx, long long n, void* stream);
/* Periodisation (mean of kr x kc aliases) of complex (batch, M, N) and its
 * adjoint (tiling / (kr kc)): subsample_fourier (kymatio/scattering2d/backend/
 * torch_backend.py:92-129, kymatio/scattering1d/backend/torch_backend.py:18-48). */
int kym_op_subsample(const float* x, float* y, int batch, int M, int N, int kr, int kc, void* stream);
int kym_op_subsample_adjoint(const float* g, float* gx, int batch, int M, int N, int kr, int kc, void* stream);
/* Reflect padding of real (batch, M, N) and its adjoint: Pad
 * (kymatio/scattering2d/backend/torch_backend.py:19-86) and TorchBackend1D.pad
 * (kymatio/scattering1d/backend/torch_backend.py:50-82). */
int kym_op_reflect_pad(const float* x, float* y, int batch, int M, int N, int top, int bottom, int left, int right,
                       void* stream);
int kym_op_reflect_pad_adjoint(const float* g, float* gx, int batch, int M, int N, int top, int bottom, int left,
                               int right, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* KYMATIO_GB300_H */
