// Launches of the assembled H2 matrix (h2_assembled.cu): storing the far- and
// near-field blocks and streaming them in a matvec.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "h2_gpu_kernels.cuh"

namespace fmca {
namespace gpu {

constexpr int kAsmMaxTargets = 256;  // targets per group of the stream (two per thread)

// row stride of a stored block: its target count rounded up to 4 (rows of
// 16-byte multiples for the bulk copies)
__host__ __device__ inline uint32_t asm_row_stride(uint32_t tcount) {
  return (tcount + 3u) & ~3u;
}

// Stores the block of every group at its offset koff[g] (elements of T):
// [j][i] = k(|tgt[tbegin + i] - src[s_j]|), row stride tcount rounded up to
// 4, zero padded.  Groups hold at most 256 targets.
template <typename T>
cudaError_t launch_kstore(const KGroup* groups, int ngroups, const uint32_t* ivl,
                          const uint64_t* koff, const Pt4<T>* tgt, const Pt4<T>* src,
                          const KParams<T>& kp, T* kstore, cudaStream_t st);

// out rows of every group = its stored block times the source rows of sval
// (chunk layout of the matvec: ld values per row, rcount of them from rofs);
// rb: right-hand sides per thread (1, 8 or 32); maxcount: largest group.
template <typename T>
cudaError_t launch_kstream(int rb, const KGroup* groups, int ngroups, int maxcount,
                           const uint32_t* ivl, const uint64_t* koff, const T* kstore,
                           const T* sval, int ld, T* out, int rofs, int rcount,
                           unsigned long long wait_ns, int stall, int* errf, cudaStream_t st);

}  // namespace gpu
}  // namespace fmca
