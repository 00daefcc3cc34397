// Throughput of the special-function-unit operations that a kernel-sum pair
// costs (sqrt.approx and ex2.approx of FP32), alone and interleaved: every
// thread keeps 8 independent chains, 4 blocks of 512 threads per SM.
// sfu_probe(ms) fills ms[0..2] with the device time (ms) of 2^30 ex2, 2^30
// sqrt and 2^29 pairs (sqrt then ex2 of its negated result) per launch.
#include <cuda_runtime.h>

namespace {

template <int OP>
__global__ void sfu_loop(float* out, int iters) {
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = 0.3f + 0.001f * (float)(threadIdx.x + i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float y;
      if (OP == 0) {
        asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(v[i]));
        v[i] = y * -0.5f;
      } else if (OP == 1) {
        asm volatile("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(v[i]));
        v[i] = y + 0.5f;
      } else {
        float r;
        asm volatile("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v[i]));
        asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-r));
        v[i] = y * 0.5f + 0.75f;
      }
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += v[i];
  if (s == 12345.f) out[threadIdx.x] = s;
}

}  // namespace

extern "C" int sfu_probe(float* ms, int* sms) {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  *sms = nsm;
  float* out = nullptr;
  if (cudaMalloc(&out, 4096) != cudaSuccess) return 2;
  const int threads = 512, blocks = nsm * 4;
  // 2^30 operations per launch for one op per element, 2^29 pairs
  const int iters = (int)((1ll << 30) / ((long long)blocks * threads * 8));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int op = 0; op < 3; ++op) {
    const int it = op == 2 ? iters / 2 : iters;
    auto launch = [&] {
      if (op == 0) sfu_loop<0><<<blocks, threads>>>(out, it);
      else if (op == 1) sfu_loop<1><<<blocks, threads>>>(out, it);
      else sfu_loop<2><<<blocks, threads>>>(out, it);
    };
    launch();
    cudaEventRecord(e0);
    for (int r = 0; r < 3; ++r) launch();
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) return 3;
    cudaEventElapsedTime(&ms[op], e0, e1);
    ms[op] /= 3.f;
    // operations actually run: blocks x threads x it x 8
    ms[op] *= (float)((1ll << (op == 2 ? 29 : 30)) / ((double)blocks * threads * it * 8));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? 0 : 4;
}
