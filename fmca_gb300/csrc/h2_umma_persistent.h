// The persistent launch of the tensor-core kernel sum (h2_umma_persistent.cu).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "h2_gpu_kernels.cuh"

namespace fmca {
namespace gpu {

// One CTA per SM (at most ngroups) running the groups in turn: kernel type
// kt, H target halves, rel: node sources with moment exponents (their
// per-group maxima are computed into gexp, 2 floats per group, first), grid:
// the sibling-paired tensor-grid far field; nst stages, units of F tiles.
cudaError_t launch_um_persistent(int kt, int H, bool rel, bool grid, const KGroup* groups,
                                 int ngroups, const uint32_t* ivl, const uint32_t* imask,
                                 const Pt4<float>* tgt, const float4* pairs, const __half* vals,
                                 float* out, int rcount, const KParams<float>& kp, int q,
                                 int* errf, float* gexp, int nst, int F, int sms,
                                 cudaStream_t st);

}  // namespace gpu
}  // namespace fmca
