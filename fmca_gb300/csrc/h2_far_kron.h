// Launch of the GAUSSIAN far field as Kronecker products (h2_far_kron.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "h2_gpu_kernels.cuh"

namespace fmca {
namespace gpu {

// true if far_kron_kernel is compiled for the grid: 2-D with 3..8 nodes per
// dimension (p1), 3-D with 3..6
inline bool far_kron_grid(int dim, int p1) {
  return (dim == 2 && p1 >= 3 && p1 <= 8) || (dim == 3 && p1 >= 3 && p1 <= 6);
}

// s[tau] = sum over the admissible sigma of every far group (one row
// cluster of Q = p1^dim nodes each) of the Kronecker product of the
// Gaussian's 1-D factors applied to t[sigma]; e: the exponent scale (FP32:
// -log2(e) / (2 l^2) with ex2, FP64: -1 / (2 l^2) with exp); rcount <= 32
// right-hand sides, from column tofs of t (rows of ldt values) to column
// sofs of s (rows of lds values).  Returns the launch error;
// cudaErrorInvalidValue for a grid it is not compiled for.
template <typename T>
cudaError_t launch_far_kron_kernel(int dim, int p1, const KGroup* groups, int ngroups,
                                   const uint32_t* ivl, const Pt4<T>* nodes_r,
                                   const Pt4<T>* nodes_c, const int* midx, T e, const T* t,
                                   int ldt, int tofs, T* s, int lds, int sofs, int rcount,
                                   cudaStream_t st);

// dst[i][c] = src[i][c] for i < rows, c < cols: the first cols columns of
// rows of lds values into rows of ldd values
cudaError_t launch_compact_columns(const float* src, int lds, float* dst, int ldd, int64_t rows,
                                   int cols, cudaStream_t st);

}  // namespace gpu
}  // namespace fmca
