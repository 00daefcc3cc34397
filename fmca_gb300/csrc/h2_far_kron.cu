// Launches of the GAUSSIAN far field as Kronecker products.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "h2_far_kron.cuh"
#include "h2_far_kron.h"

namespace fmca {
namespace gpu {
namespace {

// Raises a kernel's dynamic shared-memory limit once per (kernel, device)
// and size; later calls (inside a stream capture, for instance) make no
// runtime call.
template <typename K>
void raise_smem(K kern, size_t bytes) {
  if (bytes <= 48 * 1024) return;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> raised;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = raised[{reinterpret_cast<const void*>(kern), dev}];
  if (cur >= bytes) return;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
      cudaSuccess)
    cur = bytes;
}

template <typename T, int DIM, int P>
cudaError_t go(const KGroup* groups, int ngroups, const uint32_t* ivl, const Pt4<T>* nodes_r,
               const Pt4<T>* nodes_c, const int* midx, T e, const T* t, int ldt, int tofs, T* s,
               int lds, int sofs, int rcount, cudaStream_t st) {
  constexpr int Q = DIM == 2 ? P * P : P * P * P;
  // columns per source-cluster slot: 32 / rw clusters contracted at once
  const int rw = rcount <= 1 ? 1 : (rcount <= 8 ? 8 : 32);
  const int sl = 32 / rw;
  if constexpr (std::is_same<T, float>::value && Q <= 64) {
    // coefficients in registers, one warp per group (far_kron_reg_kernel)
    const size_t rsmem = KronShape<DIM, P>::smem_bytes(rw);
    auto rlaunch = [&](auto kern) {
      raise_smem(kern, rsmem);
      kern<<<ngroups, 32, rsmem, st>>>(groups, ivl, nodes_r, nodes_c, midx, e, t, ldt, tofs, s,
                                       lds, sofs, rcount);
    };
    if (rw == 1)
      rlaunch(far_kron_reg_kernel<DIM, P, 1>);
    else if (rw == 8)
      rlaunch(far_kron_reg_kernel<DIM, P, 8>);
    else
      rlaunch(far_kron_reg_kernel<DIM, P, 32>);
    return cudaGetLastError();
  }
  const size_t smem = ((size_t)3 * Q * 32 + DIM * P + (size_t)sl * DIM * P * P) * sizeof(T) +
                      (size_t)(Q + sl) * sizeof(int);
  auto launch = [&](auto kern) {
    raise_smem(kern, smem);
    kern<<<ngroups, 256, smem, st>>>(groups, ivl, nodes_r, nodes_c, midx, e, t, ldt, tofs, s,
                                     lds, sofs, rcount);
  };
  if (rw == 1)
    launch(far_kron_kernel<T, DIM, P, 1>);
  else if (rw == 8)
    launch(far_kron_kernel<T, DIM, P, 8>);
  else
    launch(far_kron_kernel<T, DIM, P, 32>);
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_far_kron_kernel(int dim, int p1, const KGroup* groups, int ngroups,
                                   const uint32_t* ivl, const Pt4<T>* nodes_r,
                                   const Pt4<T>* nodes_c, const int* midx, T e, const T* t,
                                   int ldt, int tofs, T* s, int lds, int sofs, int rcount,
                                   cudaStream_t st) {
  if (ngroups == 0 || rcount <= 0) return cudaSuccess;
  if (rcount > 32) return cudaErrorInvalidValue;
#define FMCA_KRON(D, P)                                                                   \
  case D * 16 + P:                                                                        \
    return go<T, D, P>(groups, ngroups, ivl, nodes_r, nodes_c, midx, e, t, ldt, tofs, s, lds, \
                       sofs, rcount, st);
  switch (dim * 16 + p1) {
    FMCA_KRON(2, 3)
    FMCA_KRON(2, 4)
    FMCA_KRON(2, 5)
    FMCA_KRON(2, 6)
    FMCA_KRON(2, 7)
    FMCA_KRON(2, 8)
    FMCA_KRON(3, 3)
    FMCA_KRON(3, 4)
    FMCA_KRON(3, 5)
    FMCA_KRON(3, 6)
    default:
      return cudaErrorInvalidValue;
  }
#undef FMCA_KRON
}

template cudaError_t launch_far_kron_kernel<float>(int, int, const KGroup*, int, const uint32_t*,
                                                   const Pt4<float>*, const Pt4<float>*,
                                                   const int*, float, const float*, int, int,
                                                   float*, int, int, int, cudaStream_t);
template cudaError_t launch_far_kron_kernel<double>(int, int, const KGroup*, int,
                                                    const uint32_t*, const Pt4<double>*,
                                                    const Pt4<double>*, const int*, double,
                                                    const double*, int, int, double*, int, int,
                                                    int, cudaStream_t);

namespace {
__global__ void compact_columns_kernel(const float* __restrict__ src, int lds,
                                       float* __restrict__ dst, int ldd, int64_t rows, int cols) {
  const int64_t total = rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / cols;
    const int c = (int)(i - r * cols);
    dst[r * ldd + c] = src[r * lds + c];
  }
}
}  // namespace

cudaError_t launch_compact_columns(const float* src, int lds, float* dst, int ldd, int64_t rows,
                                   int cols, cudaStream_t st) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  if (cols > lds || cols > ldd) return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t blocks = std::min<int64_t>((rows * cols + 255) / 256, (int64_t)std::max(sms, 1) * 16);
  compact_columns_kernel<<<(int)blocks, 256, 0, st>>>(src, lds, dst, ldd, rows, cols);
  return cudaGetLastError();
}

}  // namespace gpu
}  // namespace fmca
