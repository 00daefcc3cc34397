// Launches of the persistent tensor-core kernel sum (h2_umma_persistent.cuh),
// in a translation unit of their own so that their instantiations compile in
// parallel with h2_gpu.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "h2_umma_persistent.cuh"
#include "h2_plan.h"
#include "h2_umma_persistent.h"

namespace fmca {
namespace gpu {
namespace {

template <int KT, int H, bool REL, bool GRID>
cudaError_t launch_v(const KGroup* groups, int ngroups, const uint32_t* ivl,
                     const uint32_t* imask, const Pt4<float>* tgt, const float4* pairs,
                     const __half* vals, float* out, int rcount, const KParams<float>& kp,
                     int q, int* errf, const float* gexp, int nst, int F, int sms,
                     cudaStream_t st) {
  auto kern = ksum_um_persistent_kernel<KT, H, REL, GRID>;
  // the dynamic shared-memory limit, raised once per (kernel, device)
  static std::mutex mu;
  static std::map<int, bool> raised;
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!raised[dev] && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)um_smem_bytes(H, kUmMaxStages)) == cudaSuccess)
      raised[dev] = true;
  }
  kern<<<std::min(ngroups, sms), kUmThreads, um_smem_bytes(H, nst), st>>>(
      groups, ngroups, ivl, tgt, pairs, vals, out, kTcRhs, rcount, kp, q, errf, imask, gexp, nst,
      F);
  return cudaGetLastError();
}

template <int H, bool REL, bool GRID>
cudaError_t launch_k(int kt, const KGroup* groups, int ngroups, const uint32_t* ivl,
                     const uint32_t* imask, const Pt4<float>* tgt, const float4* pairs,
                     const __half* vals, float* out, int rcount, const KParams<float>& kp,
                     int q, int* errf, const float* gexp, int nst, int F, int sms,
                     cudaStream_t st) {
#define FMCA_PUM(KT)                                                                          \
  return launch_v<KT, H, REL, GRID>(groups, ngroups, ivl, imask, tgt, pairs, vals, out,     \
                                    rcount, kp, q, errf, gexp, nst, F, sms, st)
  switch (kt) {
    case 0:
      FMCA_PUM(0);
    case 1:
      FMCA_PUM(1);
    case 2:
      FMCA_PUM(2);
    case 3:
      FMCA_PUM(3);
    case 4:
      FMCA_PUM(4);
    case 5:
      FMCA_PUM(5);
    case K_DL_EXPONENTIAL:
      FMCA_PUM(K_DL_EXPONENTIAL);
    case K_DL_EXPONENTIAL + 1:
      FMCA_PUM(K_DL_EXPONENTIAL + 1);
    case K_DL_EXPONENTIAL + 2:
      FMCA_PUM(K_DL_EXPONENTIAL + 2);
    case K_DL_EXPONENTIAL + 3:
      FMCA_PUM(K_DL_EXPONENTIAL + 3);
    default:
      FMCA_PUM(-1);
  }
#undef FMCA_PUM
}

}  // namespace

cudaError_t launch_um_persistent(int kt, int H, bool rel, bool grid, const KGroup* groups,
                                 int ngroups, const uint32_t* ivl, const uint32_t* imask,
                                 const Pt4<float>* tgt, const float4* pairs, const __half* vals,
                                 float* out, int rcount, const KParams<float>& kp, int q,
                                 int* errf, float* gexp, int nst, int F, int sms,
                                 cudaStream_t st) {
  if (ngroups <= 0) return cudaSuccess;
  if (rel) {  // node sources: the groups' moment exponents first
    const int blocks = (ngroups * 32 + 255) / 256;
    if (grid)
      group_exponents_kernel<true, 2><<<blocks, 256, 0, st>>>(groups, ngroups, ivl, pairs, q,
                                                              imask, gexp);
    else if (H == 2)
      group_exponents_kernel<false, 2><<<blocks, 256, 0, st>>>(groups, ngroups, ivl, pairs, q,
                                                               imask, gexp);
    else
      group_exponents_kernel<false, 1><<<blocks, 256, 0, st>>>(groups, ngroups, ivl, pairs, q,
                                                               imask, gexp);
  }
#define FMCA_ARGS \
  kt, groups, ngroups, ivl, imask, tgt, pairs, vals, out, rcount, kp, q, errf, gexp, nst, F, sms, st
  if (grid) return launch_k<2, true, true>(FMCA_ARGS);
  if (H == 2) return rel ? launch_k<2, true, false>(FMCA_ARGS) : launch_k<2, false, false>(FMCA_ARGS);
  return rel ? launch_k<1, true, false>(FMCA_ARGS) : launch_k<1, false, false>(FMCA_ARGS);
#undef FMCA_ARGS
}

}  // namespace gpu
}  // namespace fmca
