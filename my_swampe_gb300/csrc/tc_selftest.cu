// Self-check of the tcgen05 building blocks used by the tensor-core Legendre
// kernels: one D[128, N] = A[128, K] . B[N, K]^T GEMM (kind::tf32, FP32
// accumulation in TMEM), optionally in 3xTF32 split precision.  Exposed
// through the C ABI so the GPU test suite can pin the descriptor, instruction
// and TMEM-layout semantics numerically.
#include "swp_internal.h"
#include "tc_common.cuh"

namespace swp {

__global__ void __launch_bounds__(128) k_tc_selftest(const float* A, const float* B, float* D, int N, int K, int split3,
                                                     int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int M = 128;
  // every operand region is allocated twice its size and zeroed, so that a
  // mis-read descriptor stride still stays inside initialised shared memory
  float* sAh = (float*)sm;
  float* sAl = sAh + 2 * M * K;
  float* sBh = sAl + 2 * M * K;
  float* sBl = sBh + 2 * N * K;
  uint64_t* mbar = (uint64_t*)(sBl + 2 * N * K);
  uint32_t* tslot = (uint32_t*)(mbar + 1);
  const int tot = 4 * M * K + 4 * N * K;
  for (int i = threadIdx.x; i < tot; i += blockDim.x) sAh[i] = 0.f;
  __syncthreads();
  for (int i = threadIdx.x; i < M * K; i += blockDim.x) {
    int r = i / K, k = i % K;
    float hi, lo;
    tc::split_tf32(A[i], hi, lo);
    sAh[tc::cm_index(r, k, K)] = hi;
    sAl[tc::cm_index(r, k, K)] = lo;
  }
  for (int i = threadIdx.x; i < N * K; i += blockDim.x) {
    int r = i / K, k = i % K;
    float hi, lo;
    tc::split_tf32(B[i], hi, lo);
    sBh[tc::cm_index(r, k, K)] = hi;
    sBl[tc::cm_index(r, k, K)] = lo;
  }
  tc::fence_proxy_async();
  int ncols = 32;
  while (ncols < N) ncols *= 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    tc::tmem_alloc(tslot, ncols);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    tc::mbar_init(mbar, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  if (threadIdx.x == 0) {
    const uint32_t idesc = tc::idesc_tf32(M, N);
    const uint32_t aH = tc::smem_u32(sAh), aL = tc::smem_u32(sAl), bH = tc::smem_u32(sBh), bL = tc::smem_u32(sBl);
    const uint32_t sbo = (uint32_t)(K / 4) * 128u;
    uint32_t acc = 0;
    for (int kk = 0; kk < K / 8; ++kk) {
      uint32_t off = (uint32_t)kk * 256u;
      tc::mma_tf32(tbase, tc::make_desc(aH + off, 128, sbo), tc::make_desc(bH + off, 128, sbo), idesc, acc);
      acc = 1;
      if (split3) {
        tc::mma_tf32(tbase, tc::make_desc(aH + off, 128, sbo), tc::make_desc(bL + off, 128, sbo), idesc, 1);
        tc::mma_tf32(tbase, tc::make_desc(aL + off, 128, sbo), tc::make_desc(bH + off, 128, sbo), idesc, 1);
      }
    }
    tc::mma_commit(mbar);
  }
  const bool ok = tc::mbar_wait_bounded(mbar, 0);
  if (!ok && threadIdx.x == 0) atomicExch(status, 1);
  tc::fence_after_sync();
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(size_t)(32 * warp + lane) * N + c0 + i] = v[i];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

}  // namespace swp

extern "C" int swp_tc_selftest(const float* A, const float* B, float* D, int N, int K, int split3, void* stream) {
  using namespace swp;
  if (!A || !B || !D || N < 16 || N > 256 || (N % 16) != 0 || K < 8 || (K % 8) != 0 || K > 128) return SWP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  size_t smem = (size_t)(4 * 128 * K + 4 * N * K) * sizeof(float) + 64;
  if (smem > 227 * 1024) return SWP_ERR_ARG;
  int* dstat = nullptr;
  if (cudaMalloc(&dstat, sizeof(int)) != cudaSuccess) return SWP_ERR_CUDA;
  cudaMemsetAsync(dstat, 0, sizeof(int), s);
  cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  k_tc_selftest<<<1, 128, smem, s>>>(A, B, D, N, K, split3, dstat);
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, dstat, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dstat);
  if (e != cudaSuccess) return SWP_ERR_CUDA;
  return h ? SWP_ERR_NUMERIC : SWP_OK;
}
