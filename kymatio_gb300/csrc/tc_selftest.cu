// Self-test of the tcgen05 split-precision GEMM path: D = A * B^T for one
// M=128 tile (A: M x K, B: N x K, row-major float32), computed from bf16
// hi/lo operands in shared memory with FP32 accumulation in tensor memory.
// Used by the GPU tests to validate descriptors and data layouts.
#include <cuda_runtime.h>

#include "../../include/kymatio_gb300.h"
#include "errors.h"
#include "tc.cuh"

namespace kym {

__global__ void __launch_bounds__(128, 1)
    tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ D, int M, int N,
                       int K, int kp, unsigned* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + 8);
  unsigned char* a_hi = smem + 1024;
  unsigned char* a_lo = a_hi + 128 * kp * 2;
  unsigned char* b_hi = a_lo + 128 * kp * 2;
  unsigned char* b_lo = b_hi + N * kp * 2;
  const int tid = threadIdx.x;
  for (int e = tid; e < 128 * kp; e += blockDim.x) {
    const int r = e / kp, k = e % kp;
    const float v = (r < M && k < K) ? A[r * K + k] : 0.f;
    __nv_bfloat16 h, l;
    tc::split_bf16(v, h, l);
    const uint32_t off = tc::kmajor_offset(r, k, kp);
    *reinterpret_cast<__nv_bfloat16*>(a_hi + off) = h;
    *reinterpret_cast<__nv_bfloat16*>(a_lo + off) = l;
  }
  for (int e = tid; e < N * kp; e += blockDim.x) {
    const int r = e / kp, k = e % kp;
    const float v = (k < K) ? B[r * K + k] : 0.f;
    __nv_bfloat16 h, l;
    tc::split_bf16(v, h, l);
    const uint32_t off = tc::kmajor_offset(r, k, kp);
    *reinterpret_cast<__nv_bfloat16*>(b_hi + off) = h;
    *reinterpret_cast<__nv_bfloat16*>(b_lo + off) = l;
  }
  tc::fence_proxy_async();
  if (tid == 0) tc::mbar_init(mbar, 1);
  if (tid < 32) {
    tc::tmem_alloc(slot, 512);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *slot;
  if (tid == 0) {
    const uint32_t sbo = (uint32_t)(kp / 8) * 128u;
    const uint32_t idesc = tc::idesc_bf16_f32(128, N);
    const uint32_t a0 = tc::smem_addr(a_hi), a1 = tc::smem_addr(a_lo);
    const uint32_t b0 = tc::smem_addr(b_hi), b1 = tc::smem_addr(b_lo);
    for (int ks = 0; ks < kp / 16; ++ks) {
      const uint32_t step = (uint32_t)ks * 256u;
      tc::mma_bf16(taddr, tc::smem_desc(a0 + step, 128, sbo), tc::smem_desc(b0 + step, 128, sbo), idesc, ks > 0);
      tc::mma_bf16(taddr, tc::smem_desc(a1 + step, 128, sbo), tc::smem_desc(b0 + step, 128, sbo), idesc, true);
      tc::mma_bf16(taddr, tc::smem_desc(a0 + step, 128, sbo), tc::smem_desc(b1 + step, 128, sbo), idesc, true);
    }
    tc::mma_commit(mbar);
  }
  bool ok = tc::mbar_wait_bounded(mbar, 0, 1u << 22);
  if (!ok) {
    atomicOr(status, tc::kErrMmaTimeout);
    tc::mbar_wait_bounded(mbar, 0, 1u << 22);  // give the tensor core a second chance before releasing TMEM
  }
  tc::fence_after_sync();
  const int w = tid >> 5, lane = tid & 31;
  const int row = 32 * w + lane;
  for (int c0 = 0; c0 < N; c0 += 32) {
    float v[32];
    tc::tmem_ld32(taddr + ((uint32_t)(32 * w) << 16) + (uint32_t)c0, v);
    if (ok && row < M)
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (c0 + i < N) D[row * N + c0 + i] = v[i];
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(taddr, 512);
}

}  // namespace kym

extern "C" int kym_tc_selftest(const float* A, const float* B, float* D, int M, int N, int K, unsigned* status,
                               void* stream) {
  if (!A || !B || !D || !status || M < 1 || M > 128 || N < 16 || N > 64 || N % 16 || K < 1 || K > 256) {
    kym::set_error_message("tc_selftest", "needs M <= 128, N in {16, 32, 48, 64}, K <= 256");
    return KYM_ERR_INVALID;
  }
  const int kp = (K + 15) / 16 * 16;
  const size_t smem = 1024 + (size_t)(128 + N) * kp * 2 * 2;
  cudaError_t e = cudaFuncSetAttribute(kym::tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e == cudaSuccess) {
    kym::tc_selftest_kernel<<<1, 128, smem, static_cast<cudaStream_t>(stream)>>>(A, B, D, M, N, K, kp, status);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    kym::set_error_message("tc_selftest", cudaGetErrorString(e));
    return KYM_ERR_CUDA;
  }
  return KYM_OK;
}
