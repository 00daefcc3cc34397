// Self-test of the tcgen05 operand layouts that the library's tensor-core
// kernel sums rely on (fmca_gb300/csrc/umma.cuh): one 128 x 32 x 16 FP16
// product with A in tensor memory (row m in lane m, two K elements per
// column), B in shared memory as K-major core matrices without swizzle
// (LBO = 512 B between k groups, SBO = 128 B between n groups) and D in
// tensor memory, on small integers so that the FP32 result is exact.
// One CTA of 128 threads; every shared and global index stays inside the
// arrays declared here (B: 16 x 32 halves in 1 KB of an 8 KB buffer; out:
// 128 x 32 floats).
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "h2_gpu_kernels.cuh"
#include "umma.cuh"

using namespace fmca::gpu;

__device__ __host__ inline float probe_a(int m, int k) {
  return (float)(((m * 7 + k * 3) % 11) - 5);
}
__device__ __host__ inline float probe_b(int k, int n) {
  return (float)(((k * 5 + n) % 7) - 3);
}

__global__ void __launch_bounds__(128, 1) probe_kernel(float* out, int* status, int accumulate_twice) {
  __shared__ __align__(1024) unsigned char sb[8192];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int e = tid; e < 4096; e += 128) reinterpret_cast<uint16_t*>(sb)[e] = 0;
  __syncthreads();
  for (int e = tid; e < 16 * 32; e += 128) {
    const int k = e / 32, n = e % 32;
    const int off = (k / 8) * 512 + (n / 8) * 128 + (n % 8) * 16 + (k % 8) * 2;
    *reinterpret_cast<__half*>(sb + off) = __float2half(probe_b(k, n));
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(&tbase, 64);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t base = tbase;
  const uint32_t lanes = (uint32_t)(warp * 32) << 16;
  uint32_t a[8];
  for (int j = 0; j < 8; ++j) {
    __half2 h = __floats2half2_rn(probe_a(tid, 2 * j), probe_a(tid, 2 * j + 1));
    a[j] = *reinterpret_cast<uint32_t*>(&h);
  }
  tmem_st8(base + lanes + 32, a);
  tmem_wait_st();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid == 0) {
    const uint64_t bd = umma_desc(sb, 512, 128);
    umma_f16_ts(base, base + 32, bd, umma_idesc_f16(128, 32), 0);
    if (accumulate_twice) umma_f16_ts(base, base + 32, bd, umma_idesc_f16(128, 32), 1);
    umma_commit(&bar);
  }
  const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&bar, 0, 1000000000ull));
  tc_fence_after();
  if (ok) {
    uint32_t d[16];
    for (int c = 0; c < 32; c += 16) {
      tmem_ld16(base + lanes + c, d);
      tmem_wait_ld16(d);
      for (int j = 0; j < 16; ++j) out[tid * 32 + c + j] = __uint_as_float(d[j]);
    }
  } else if ((tid & 31) == 0) {
    atomicExch(status, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(base, 64);
}

// D (128 x 32, row-major) of A * B, or of 2 A * B with accumulate_twice;
// returns 0, 1 for a timed-out completion wait, or a CUDA error code + 100
extern "C" int umma_probe(float* host_out, int accumulate_twice) {
  float* d = nullptr;
  int* st = nullptr;
  int rc = 0;
  if (cudaMalloc(&d, 128 * 32 * sizeof(float)) != cudaSuccess) return 100 + (int)cudaGetLastError();
  if (cudaMalloc(&st, sizeof(int)) != cudaSuccess) {
    cudaFree(d);
    return 100 + (int)cudaGetLastError();
  }
  cudaMemset(d, 0, 128 * 32 * sizeof(float));
  cudaMemset(st, 0, sizeof(int));
  probe_kernel<<<1, 128>>>(d, st, accumulate_twice);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    rc = 100 + (int)e;
  } else {
    int s = 0;
    cudaMemcpy(&s, st, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(host_out, d, 128 * 32 * sizeof(float), cudaMemcpyDeviceToHost);
    rc = s;
  }
  cudaFree(d);
  cudaFree(st);
  return rc;
}
