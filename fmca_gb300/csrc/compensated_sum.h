// Compensated summation for the FP32 leaf gather: the q terms of
// y_i = sum_k V[k][i] s[k] are added in blocks of kGatherBlock in plain FP32,
// and each block sum enters the running total through Kahan's compensated
// addition (Kahan 1965; Higham, Accuracy and Stability of Numerical
// Algorithms, 2nd ed., section 4.3). The rounding error of the total is then
// about kGatherBlock unit roundoffs instead of q. Plain C++ so that the same
// code is compiled for the device and for the host-side test
// (tests/test_compensated_sum.py).
#pragma once

#ifdef __CUDACC__
#define FMCA_HD __host__ __device__ __forceinline__
#else
#define FMCA_HD inline
#endif

namespace fmca {

constexpr int kGatherBlock = 8;  // terms per plain partial sum

// sum += x with the running compensation c (the negated low part lost so
// far); the operations must not be reassociated, so this is compiled
// without fast-math
template <typename T>
FMCA_HD void kahan_add(T& sum, T& c, T x) {
  const T y = x - c;
  const T t = sum + y;
  c = (t - sum) - y;
  sum = t;
}

}  // namespace fmca
