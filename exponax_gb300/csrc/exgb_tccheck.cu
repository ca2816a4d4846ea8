// exgb_tccheck.cu -- self-check of the tcgen05 layer (exgb_tc.cuh): one CTA
// computes D = A . B^T (M = 128, N <= 256, K <= 128, multiples of 16) from
// FP32 inputs, either with the inputs rounded to bf16 (one product per
// k-step) or in the split-BF16 three-product form, FP32 accumulation in
// tensor memory.  Exercises exactly the descriptors, the instruction
// descriptor, the TMEM allocation, commit/mbarrier and tcgen05.ld paths the
// DFT kernels use.
#include <cuda_runtime.h>

#include "exgb_internal.h"
#include "exgb_tc.cuh"

namespace exgb {

__global__ void __launch_bounds__(128, 1)
    tc_gemm_check_kernel(int N, int K, const float* __restrict__ A, const float* __restrict__ B, float* D,
                         int split, int* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* a_hi = smem;
  unsigned char* a_lo = a_hi + 128 * K * 2;
  unsigned char* b_hi = a_lo + 128 * K * 2;
  unsigned char* b_lo = b_hi + N * K * 2;
  const int KC = K / 8;
  for (int t = tid; t < 128 * KC; t += 128) {
    const int r = t / KC, c = t % KC;
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = A[(size_t)r * K + 8 * c + i];
    if (!split) {
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = __bfloat162float(__float2bfloat16_rn(v[i]));
    }
    tc::split8_store(v, a_hi, a_lo, tc::kmaj_chunk(r, c, K));
  }
  for (int t = tid; t < N * KC; t += 128) {
    const int r = t / KC, c = t % KC;
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = B[(size_t)r * K + 8 * c + i];
    if (!split) {
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = __bfloat162float(__float2bfloat16_rn(v[i]));
    }
    tc::split8_store(v, b_hi, b_lo, tc::kmaj_chunk(r, c, K));
  }
  uint32_t ncols = 32;
  while (ncols < (uint32_t)N) ncols <<= 1;
  if (warp == 0) {
    tc::tmem_alloc(&tbase, ncols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tbase;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, N);
    if (split) {
      tc::mma_split3(tmem, tc::smem_u32(a_hi), tc::smem_u32(a_lo), K, tc::smem_u32(b_hi), tc::smem_u32(b_lo), K, K,
                     idesc, false);
    } else {
      for (int s = 0; s < K / 16; ++s)
        tc::mma_bf16(tmem, tc::kmaj_desc(tc::smem_u32(a_hi), K, s), tc::kmaj_desc(tc::smem_u32(b_hi), K, s), idesc,
                     s > 0 ? 1u : 0u);
    }
    tc::mma_commit(&mbar);
  }
  bool ok = tc::mbar_wait(&mbar, 0, 4000000000LL);
  if (!ok) ok = tc::mbar_wait(&mbar, 0, 4000000000LL);  // let the MMAs drain before TMEM is released
  const int bad = __syncthreads_or(!ok);
  tc::fence_after_sync();
  if (!bad) {
    const int row = 32 * warp + lane;
    for (int c0 = 0; c0 < N; c0 += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 8; ++i) D[(size_t)row * N + c0 + i] = v[i];
    }
  } else if (tid == 0) {
    *status = EXGB_ETIMEOUT;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

}  // namespace exgb

extern "C" int exgb_tc_gemm_check(void* stream, int n, int k, const float* a, const float* b, float* d, int split) {
  using namespace exgb;
  if (!a || !b || !d) return fail(EXGB_EINVAL, "exgb_tc_gemm_check: NULL pointer");
  if (n < 16 || n > 256 || n % 16 || k < 16 || k > 128 || k % 16)
    return fail(EXGB_ESHAPE, "exgb_tc_gemm_check: need 16 <= n <= 256, 16 <= k <= 128, multiples of 16");
  int dev = 0, major = 0;
  EXGB_CUDA(cudaGetDevice(&dev));
  EXGB_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  if (major != 10) return fail(EXGB_EUNSUPPORTED, "exgb_tc_gemm_check: needs an sm_100-family GPU");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t smem = (size_t)(128 + n) * k * 4;
  EXGB_CUDA(cudaFuncSetAttribute(tc_gemm_check_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int* d_status = nullptr;
  EXGB_CUDA(cudaMallocAsync(&d_status, sizeof(int), st));
  EXGB_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int), st));
  tc_gemm_check_kernel<<<1, 128, smem, st>>>(n, k, a, b, d, split, d_status);
  EXGB_CUDA(cudaGetLastError());
  int h_status = 0;
  EXGB_CUDA(cudaMemcpyAsync(&h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  EXGB_CUDA(cudaFreeAsync(d_status, st));
  EXGB_CUDA(cudaStreamSynchronize(st));
  if (h_status) return fail(h_status, "exgb_tc_gemm_check: tensor-core wait timed out");
  return EXGB_OK;
}
