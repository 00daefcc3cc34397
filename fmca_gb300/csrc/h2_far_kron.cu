// Launches of the GAUSSIAN far field as Kronecker products.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
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
               const Pt4<T>* nodes_c, const int* midx, T e, const T* t, T* s, int ld, int rofs,
               int rcount, cudaStream_t st) {
  constexpr int Q = DIM == 2 ? P * P : P * P * P;
  // columns per source-cluster slot: 32 / rw clusters contracted at once
  const int rw = rcount <= 1 ? 1 : (rcount <= 8 ? 8 : 32);
  const int sl = 32 / rw;
  const size_t smem = ((size_t)3 * Q * 32 + DIM * P + (size_t)sl * DIM * P * P) * sizeof(T) +
                      (size_t)(Q + sl) * sizeof(int);
  auto launch = [&](auto kern) {
    raise_smem(kern, smem);
    kern<<<ngroups, 256, smem, st>>>(groups, ivl, nodes_r, nodes_c, midx, e, t, s, ld, rofs,
                                     rcount);
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
                                   T* s, int ld, int rofs, int rcount, cudaStream_t st) {
  if (ngroups == 0) return cudaSuccess;
  if (rcount > 32) return cudaErrorInvalidValue;
#define FMCA_KRON(D, P)                                                                   \
  case D * 16 + P:                                                                        \
    return go<T, D, P>(groups, ngroups, ivl, nodes_r, nodes_c, midx, e, t, s, ld, rofs,   \
                       rcount, st);
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
                                                   const int*, float, const float*, float*, int,
                                                   int, int, cudaStream_t);
template cudaError_t launch_far_kron_kernel<double>(int, int, const KGroup*, int,
                                                    const uint32_t*, const Pt4<double>*,
                                                    const Pt4<double>*, const int*, double,
                                                    const double*, double*, int, int, int,
                                                    cudaStream_t);

}  // namespace gpu
}  // namespace fmca
