// Test-only probe of the UMMA operand layout: one CTA multiplies a 128x64
// fp16 tile A by a 64x64 fp16 tile B (both K-major, no swizzle, K = 64) with
// four K=16 tcgen05.mma steps into tensor memory and writes D (128x64 fp32).
// lbo/sbo are parameters so a wrong reading of the descriptor shows up as a
// wrong product; every address either reading stays inside the tiles.
#include <cuda_fp16.h>

#include "../amdat_gb300/csrc/umma.cuh"

using namespace amdat::umma;

extern "C" __global__ void __launch_bounds__(128) tc_probe_kernel(const __half* A, const __half* B,
                                                                  float* D, int lbo, int sbo,
                                                                  int* err) {
  __shared__ __align__(1024) unsigned char sA[128 * 64 * 2];
  __shared__ __align__(1024) unsigned char sB[64 * 64 * 2];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_ok;
  const int tid = threadIdx.x;
  for (int i = tid; i < 128 * 64; i += blockDim.x)
    *reinterpret_cast<__half*>(sA + kmajor_offset(i / 64, i % 64, 64)) = A[i];
  for (int i = tid; i < 64 * 64; i += blockDim.x)
    *reinterpret_cast<__half*>(sB + kmajor_offset(i / 64, i % 64, 64)) = B[i];
  if (tid == 0) {
    mbar_init(&mbar, 1);
    fence_mbarrier_init();
  }
  if (tid < 32) {
    tmem_alloc(&s_tmem, 64);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_tmem;
  if (tid == 0) {
    const uint32_t idesc = idesc_f16_f32(128, 64);
    for (int ks = 0; ks < 4; ++ks) {
      const uint64_t ad = smem_desc(smem_addr(sA) + ks * 256, (uint32_t)lbo, (uint32_t)sbo);
      const uint64_t bd = smem_desc(smem_addr(sB) + ks * 256, (uint32_t)lbo, (uint32_t)sbo);
      mma_f16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
    }
    mma_commit(&mbar);
    s_ok = mbar_wait(&mbar, 0, 1u << 22) ? 1 : 0;
  }
  __syncthreads();
  fence_after_sync();
  if (s_ok) {
    const int warp = tid / 32, lane = tid % 32;
    for (int c0 = 0; c0 < 64; c0 += 32) {
      uint32_t r[32];
      tmem_ld_32x32b_x32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, r);
      tmem_ld_wait();
      for (int j = 0; j < 32; ++j) D[(32 * warp + lane) * 64 + c0 + j] = __uint_as_float(r[j]);
    }
  } else if (tid == 0) {
    *err = 1;
  }
  fence_before_sync();
  __syncthreads();
  if (tid < 32) {
    fence_after_sync();
    tmem_dealloc(tmem, 64);
  }
}

extern "C" int tc_probe_run(const void* A, const void* B, void* D, int lbo, int sbo, void* err) {
  tc_probe_kernel<<<1, 128>>>((const __half*)A, (const __half*)B, (float*)D, lbo, sbo, (int*)err);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int)e;
}

// Test-only probe of the A-from-tensor-memory form: A (128 x 32 fp16) is
// written into tensor memory by tcgen05.st (row i in lane i, column c holding
// K elements 2c, 2c+1), B (32 x 32 fp16, K-major, no swizzle) sits in shared
// memory, and two K=16 tcgen05.mma steps (A address + 8 columns per step) give
// D = A B^T (128 x 32 fp32).
extern "C" __global__ void __launch_bounds__(128) tc_probe_tmem_a_kernel(const __half* A, const __half* B,
                                                                         float* D, int* err) {
  __shared__ __align__(1024) unsigned char sB[32 * 32 * 2];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_ok;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  for (int i = tid; i < 32 * 32; i += blockDim.x)
    *reinterpret_cast<__half*>(sB + kmajor_offset(i / 32, i % 32, 32)) = B[i];
  if (tid == 0) {
    mbar_init(&mbar, 1);
    fence_mbarrier_init();
  }
  if (tid < 32) {
    tmem_alloc(&s_tmem, 64);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_tmem;
  // A row (32 warp + lane) into lane (32 warp + lane), columns 32..47
  const int row = 32 * warp + lane;
  for (int c0 = 0; c0 < 16; c0 += 8) {
    uint32_t r[8];
    for (int c = 0; c < 8; ++c) {
      const __half2 h = __halves2half2(A[row * 32 + 2 * (c0 + c)], A[row * 32 + 2 * (c0 + c) + 1]);
      r[c] = *reinterpret_cast<const uint32_t*>(&h);
    }
    tmem_st_32x32b_x8(tmem + ((uint32_t)(32 * warp) << 16) + 32u + (uint32_t)c0, r);
  }
  tmem_st_wait();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (tid == 0) {
    const uint32_t idesc = idesc_f16_f32(128, 32);
    for (int ks = 0; ks < 2; ++ks) {
      const uint64_t bd = smem_desc(smem_addr(sB) + ks * 256, 128, 4 * 128);
      mma_f16_tmem_a(tmem, tmem + 32u + (uint32_t)(8 * ks), bd, idesc, ks > 0 ? 1u : 0u);
    }
    mma_commit(&mbar);
    s_ok = mbar_wait(&mbar, 0, 1u << 22) ? 1 : 0;
  }
  __syncthreads();
  fence_after_sync();
  if (s_ok) {
    uint32_t r[32];
    tmem_ld_32x32b_x32(tmem + ((uint32_t)(32 * warp) << 16), r);
    tmem_ld_wait();
    for (int j = 0; j < 32; ++j) D[row * 32 + j] = __uint_as_float(r[j]);
  } else if (tid == 0) {
    *err = 1;
  }
  fence_before_sync();
  __syncthreads();
  if (tid < 32) {
    fence_after_sync();
    tmem_dealloc(tmem, 64);
  }
}

extern "C" int tc_probe_tmem_a_run(const void* A, const void* B, void* D, void* err) {
  tc_probe_tmem_a_kernel<<<1, 128>>>((const __half*)A, (const __half*)B, (float*)D, (int*)err);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int)e;
}

// A bounded wait that runs out: an mbarrier nothing arrives on, polled with the
// engine's bounded try_wait (max_iter polls of <= 1 us).  The kernel records
// the outcome (1 = gave up) and returns normally, so the context stays usable.
extern "C" __global__ void wait_timeout_kernel(int* status, unsigned max_iter) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbarrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) *status = mbar_wait(&bar, 0, max_iter) ? 0 : 1;
}

extern "C" int wait_timeout_run(void* status, unsigned max_iter) {
  wait_timeout_kernel<<<1, 32>>>((int*)status, max_iter);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int)e;
}
