// Tensor-core self-test and throughput probe (no counterpart in the
// reference): checks this library's tcgen05 operand layouts and descriptors
// against an exact host product, and measures the dense BF16 MMA rate that
// bounds the split-precision exchange.
//
//   hfg_tc_selftest : D = A B^T for M = 128, N <= 256 and `ksteps` K steps of
//                     16, bf16 operands staged in shared memory (K-major or
//                     MN-major), FP32 accumulation in tensor memory.
//   hfg_tc_peak     : back-to-back M = 128, N = 256, K = 16 MMAs on resident
//                     operands, `ctas_per_sm` CTAs per SM; returns TFLOP/s.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "smem_limit.hpp"
#include "tc.cuh"

namespace hfg {
namespace {

constexpr int kM = 128;

__global__ void __launch_bounds__(128) tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                          float* __restrict__ D, int N, int ksteps, int a_mn,
                                                          int b_mn, int swap, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int K = 16 * ksteps;
  unsigned char* At = sm;                                  // ksteps x 4 KB
  unsigned char* Bt = At + (size_t)ksteps * kM * 32;       // ksteps x N*32 B
  uint64_t* mbar = reinterpret_cast<uint64_t*>(Bt + (size_t)ksteps * N * 32);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  for (int idx = t; idx < kM * K; idx += blockDim.x) {
    const int m = idx / K, k = idx % K, ks = k >> 4, kk = k & 15;
    const uint32_t o = a_mn ? tc::off_mnmajor(m, kk) : tc::off_kmajor(m, kk);
    *reinterpret_cast<__nv_bfloat16*>(At + (size_t)ks * kM * 32 + o) = __float2bfloat16_rn(A[idx]);
  }
  for (int idx = t; idx < N * K; idx += blockDim.x) {
    const int n = idx / K, k = idx % K, ks = k >> 4, kk = k & 15;
    const uint32_t o = b_mn ? tc::off_mnmajor(n, kk) : tc::off_kmajor(n, kk);
    *reinterpret_cast<__nv_bfloat16*>(Bt + (size_t)ks * N * 32 + o) = __float2bfloat16_rn(B[idx]);
  }
  tc::fence_async_smem();
  if (w == 0) {
    tc::tmem_alloc(tslot, 256);
    tc::tmem_relinquish();
  }
  if (t == 0) tc::mbar_init(mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  if (t == 0) {
    const uint32_t idesc = tc::idesc_bf16(kM, N, a_mn, b_mn);
    const uint32_t lbo = swap ? tc::kSBO : tc::kLBO, sbo = swap ? tc::kLBO : tc::kSBO;
    for (int ks = 0; ks < ksteps; ++ks) {
      const uint64_t ad = tc::smem_desc(tc::smem_u32(At + (size_t)ks * kM * 32), lbo, sbo);
      const uint64_t bd = tc::smem_desc(tc::smem_u32(Bt + (size_t)ks * N * 32), lbo, sbo);
      tc::mma_bf16(taddr, ad, bd, idesc, ks > 0 ? 1u : 0u);
    }
    tc::mma_commit(mbar);
  }
  const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(mbar, 0));
  if (!ok && lane == 0) atomicExch(err, 1);
  tc::fence_after_sync();
  if (ok) {
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tc::tmem_ld16(taddr + ((uint32_t)(32 * w) << 16) + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(size_t)(32 * w + lane) * N + c + i] = v[i];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(taddr, 256);
}

__global__ void __launch_bounds__(128) tc_peak_kernel(int iters, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* At = sm;               // 128 x 16 bf16
  unsigned char* Bt = sm + kM * 32;     // 256 x 16 bf16
  uint64_t* mbar = reinterpret_cast<uint64_t*>(Bt + 256 * 32);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int t = threadIdx.x, w = t >> 5;
  // small exact values: the accumulators stay finite for any iteration count
  for (int i = t; i < (kM + 256) * 16; i += blockDim.x)
    reinterpret_cast<__nv_bfloat16*>(sm)[i] = __float2bfloat16_rn((float)((i * 7 + blockIdx.x) % 5 - 2) * 0.0625f);
  tc::fence_async_smem();
  if (w == 0) {
    tc::tmem_alloc(tslot, 256);
    tc::tmem_relinquish();
  }
  if (t == 0) tc::mbar_init(mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  if (t == 0) {
    const uint32_t idesc = tc::idesc_bf16(kM, 256, 0, 0);
    const uint64_t ad = tc::smem_desc(tc::smem_u32(At)), bd = tc::smem_desc(tc::smem_u32(Bt));
    for (int i = 0; i < iters; ++i) tc::mma_bf16(taddr, ad, bd, idesc, i > 0 ? 1u : 0u);
    tc::mma_commit(mbar);
  }
  if (!tc::mbar_wait(mbar, 0, 1u << 28) && (t & 31) == 0) atomicExch(err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(taddr, 256);
}

}  // namespace

cudaError_t tc_selftest(const float* A, const float* B, float* D, int N, int ksteps, int a_mn, int b_mn, int swap,
                        int* timed_out) {
  if (N < 16 || N > 256 || N % 16 != 0 || ksteps < 1 || ksteps > 8) return cudaErrorInvalidValue;
  const size_t smem = (size_t)ksteps * (kM + N) * 32 + 64;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* dErr = nullptr;
  cudaError_t e = cudaSuccess;
  const int K = 16 * ksteps;
  auto fail = [&](cudaError_t x) {
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dErr);
    return x;
  };
  if ((e = cudaMalloc(&dA, sizeof(float) * kM * K)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&dB, sizeof(float) * N * K)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&dD, sizeof(float) * kM * N)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&dErr, sizeof(int))) != cudaSuccess) return fail(e);
  cudaMemcpy(dA, A, sizeof(float) * kM * K, cudaMemcpyHostToDevice);
  cudaMemcpy(dB, B, sizeof(float) * N * K, cudaMemcpyHostToDevice);
  cudaMemset(dD, 0, sizeof(float) * kM * N);
  cudaMemset(dErr, 0, sizeof(int));
  if ((e = smem_limit(tc_selftest_kernel, smem)) != cudaSuccess) return fail(e);
  tc_selftest_kernel<<<1, 128, smem>>>(dA, dB, dD, N, ksteps, a_mn, b_mn, swap, dErr);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
  cudaMemcpy(D, dD, sizeof(float) * kM * N, cudaMemcpyDeviceToHost);
  cudaMemcpy(timed_out, dErr, sizeof(int), cudaMemcpyDeviceToHost);
  return fail(cudaGetLastError());
}

cudaError_t tc_peak(int ctas_per_sm, int iters, double* tflops, double* ms, int* timed_out) {
  // each CTA holds 256 of the SM's 512 tensor-memory columns
  if (ctas_per_sm < 1 || ctas_per_sm > 2 || iters < 1) return cudaErrorInvalidValue;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = (kM + 256) * 32 + 64;
  int* dErr = nullptr;
  cudaError_t e = cudaMalloc(&dErr, sizeof(int));
  if (e != cudaSuccess) return e;
  cudaMemset(dErr, 0, sizeof(int));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int grid = nsm * ctas_per_sm;
  tc_peak_kernel<<<grid, 128, smem>>>(iters / 8 + 1, dErr);  // warm-up
  cudaEventRecord(e0);
  tc_peak_kernel<<<grid, 128, smem>>>(iters, dErr);
  cudaEventRecord(e1);
  e = cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  *ms = t;
  *tflops = 2.0 * kM * 256 * 16 * (double)iters * grid / (t * 1e-3) / 1e12;
  cudaMemcpy(timed_out, dErr, sizeof(int), cudaMemcpyDeviceToHost);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(dErr);
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace hfg
