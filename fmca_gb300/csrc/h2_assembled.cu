// Launches of the assembled H2 matrix, in a translation unit of their own so
// that their instantiations compile in parallel with h2_gpu.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "h2_assembled.h"
#include "h2_assembled_kernels.cuh"

namespace fmca {
namespace gpu {
namespace {

// Raises a kernel's dynamic shared-memory limit once per (kernel, device)
// and size (the kernels of one element type share a function type, so the
// key is the kernel's address).
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

template <typename T, int KT>
cudaError_t kstore_kt(const KGroup* groups, int ngroups, const uint32_t* ivl,
                      const uint64_t* koff, const Pt4<T>* tgt, const Pt4<T>* src,
                      const KParams<T>& kp, T* kstore, cudaStream_t st) {
  kstore_kernel<T, KT><<<ngroups, kAsmThreads, 0, st>>>(groups, ivl, koff, tgt, src, kp, kstore);
  return cudaGetLastError();
}

// Tile shape of the stream: about 16 KB of block values per stage (FP32, 3
// stages) or 32 KB (FP64, 3 stages), ts a multiple of 8 sources.
template <typename T>
void stream_shape(int kcap, int* ts, int* nst) {
  const int bytes = sizeof(T) == 4 ? 16384 : 32768;
  int t = bytes / (kcap * (int)sizeof(T));
  t = std::max(8, std::min(64, t & ~7));
  *ts = t;
  *nst = 3;
}

template <typename T, int TPT, int RB>
cudaError_t kstream_t(const KGroup* groups, int ngroups, int maxcount, const uint32_t* ivl,
                      const uint64_t* koff, const T* kstore, const T* sval, int ld, T* out,
                      int rofs, int rcount, unsigned long long wait_ns, int stall, int* errf,
                      cudaStream_t st) {
  const int kcap = (int)asm_row_stride((uint32_t)maxcount);
  int ts = 0, nst = 0;
  stream_shape<T>(kcap, &ts, &nst);
  auto kern = kstream_kernel<T, TPT, RB>;
  const size_t smem = 256 + (size_t)nst * ts * ((size_t)ld + kcap) * sizeof(T);
  raise_smem(kern, smem);
  int threads = (maxcount + TPT - 1) / TPT;
  threads = (threads + 31) / 32 * 32;
  threads = std::max(32, std::min(kAsmThreads, threads));
  kern<<<ngroups, threads, smem, st>>>(groups, ivl, koff, kstore, ts, kcap, nst, sval, ld, out,
                                       rofs, rcount, wait_ns, stall, errf);
  return cudaGetLastError();
}

template <typename T, int RB>
cudaError_t kstream_tpt(const KGroup* groups, int ngroups, int maxcount, const uint32_t* ivl,
                        const uint64_t* koff, const T* kstore, const T* sval, int ld, T* out,
                        int rofs, int rcount, unsigned long long wait_ns, int stall, int* errf,
                        cudaStream_t st) {
  if (maxcount > kAsmThreads)
    return kstream_t<T, 2, RB>(groups, ngroups, maxcount, ivl, koff, kstore, sval, ld, out, rofs,
                               rcount, wait_ns, stall, errf, st);
  return kstream_t<T, 1, RB>(groups, ngroups, maxcount, ivl, koff, kstore, sval, ld, out, rofs,
                             rcount, wait_ns, stall, errf, st);
}

}  // namespace

template <typename T>
cudaError_t launch_kstore(const KGroup* groups, int ngroups, const uint32_t* ivl,
                          const uint64_t* koff, const Pt4<T>* tgt, const Pt4<T>* src,
                          const KParams<T>& kp, T* kstore, cudaStream_t st) {
  if (ngroups == 0) return cudaSuccess;
  switch (kp.type) {
    case 0:
      return kstore_kt<T, 0>(groups, ngroups, ivl, koff, tgt, src, kp, kstore, st);
    case 1:
      return kstore_kt<T, 1>(groups, ngroups, ivl, koff, tgt, src, kp, kstore, st);
    case 2:
      return kstore_kt<T, 2>(groups, ngroups, ivl, koff, tgt, src, kp, kstore, st);
    case 3:
      return kstore_kt<T, 3>(groups, ngroups, ivl, koff, tgt, src, kp, kstore, st);
    default:
      return kstore_kt<T, -1>(groups, ngroups, ivl, koff, tgt, src, kp, kstore, st);
  }
}

template <typename T>
cudaError_t launch_kstream(int rb, const KGroup* groups, int ngroups, int maxcount,
                           const uint32_t* ivl, const uint64_t* koff, const T* kstore,
                           const T* sval, int ld, T* out, int rofs, int rcount,
                           unsigned long long wait_ns, int stall, int* errf, cudaStream_t st) {
  if (ngroups == 0) return cudaSuccess;
  if (maxcount > kAsmMaxTargets) return cudaErrorInvalidValue;
  switch (rb) {
    case 1:
      return kstream_tpt<T, 1>(groups, ngroups, maxcount, ivl, koff, kstore, sval, ld, out, rofs,
                               rcount, wait_ns, stall, errf, st);
    case 8:
      return kstream_tpt<T, 8>(groups, ngroups, maxcount, ivl, koff, kstore, sval, ld, out, rofs,
                               rcount, wait_ns, stall, errf, st);
    default:
      return kstream_tpt<T, 32>(groups, ngroups, maxcount, ivl, koff, kstore, sval, ld, out,
                                rofs, rcount, wait_ns, stall, errf, st);
  }
}

template cudaError_t launch_kstore<float>(const KGroup*, int, const uint32_t*, const uint64_t*,
                                          const Pt4<float>*, const Pt4<float>*,
                                          const KParams<float>&, float*, cudaStream_t);
template cudaError_t launch_kstore<double>(const KGroup*, int, const uint32_t*, const uint64_t*,
                                           const Pt4<double>*, const Pt4<double>*,
                                           const KParams<double>&, double*, cudaStream_t);
template cudaError_t launch_kstream<float>(int, const KGroup*, int, int, const uint32_t*,
                                           const uint64_t*, const float*, const float*, int,
                                           float*, int, int, unsigned long long, int, int*,
                                           cudaStream_t);
template cudaError_t launch_kstream<double>(int, const KGroup*, int, int, const uint32_t*,
                                            const uint64_t*, const double*, const double*, int,
                                            double*, int, int, unsigned long long, int, int*,
                                            cudaStream_t);

}  // namespace gpu
}  // namespace fmca
