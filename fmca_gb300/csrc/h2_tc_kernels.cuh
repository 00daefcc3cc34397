// Mixed-precision matvec: kernel-value arithmetic and the scaling / split
// kernels around the tensor-core kernel sums (sm_103a).
//
// The kernel sums (h2_umma_kernels.cuh) compute
//   out[t][0..32) = sum_s a(t, s) v[s][0..32),  a(t, s) = k(|t - s|) 2^(w_s - E),
// with a and v split into FP16 halves (x = x_hi + x_lo) and three products
// a_hi v_hi + a_hi v_lo + a_lo v_hi on the tensor cores.
// Values are kept inside the FP16 range by exact power-of-two scalings:
// every right-hand side is divided by 2^ceil(log2 max|x_r|) before the
// product (and multiplied back at the end), and the interpolated moments of
// each column cluster by 2^e_sigma. The exponent e_sigma travels in the w
// field of the cluster's interpolation nodes and enters the exponential of
// the kernel, so the weight costs no multiplication; a group subtracts the
// largest exponent E of its sources (a <= 1) and multiplies its sums by 2^E.
// Coordinates are multiplied by a kernel-specific g so that the kernel
// argument needs no further scaling.
#pragma once

#include <type_traits>

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "h2_gpu_kernels.cuh"

namespace fmca {
namespace gpu {

__device__ __forceinline__ uint32_t h2_bits(__half2 h) {
  return *reinterpret_cast<uint32_t*>(&h);
}

constexpr int kTcRhs = 32;  // right-hand sides per product
constexpr float kLog2e = 1.44269504088896341f;
constexpr float kLn2 = 0.693147180559945309f;

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// 2^e for an integral e; 0 below the normal range (e = -inf included)
__device__ __forceinline__ float pow2i(float e) {
  const int i = __float2int_rz(fminf(fmaxf(e, -127.f), 127.f));
  return i <= -127 ? 0.f : __int_as_float((i + 127) << 23);
}

// a = k * 2^w of two squared distances in the coordinates scaled by g
// (make_kparams: g = log2(e) / l for EXPONENTIAL, log2(e) sqrt(3) / l,
// log2(e) sqrt(5) / l, log2(e) sqrt(7) / l and 3 log2(e) / l for MATERN32 /
// 52 / 72 / 92, so that r' = sqrt(r2) is the
// kernel argument times log2(e) and e^-argument = 2^-r'). FP32x2
// arithmetic, the square root and exponential per element on the SFU;
// sqrt(0) = 0, so coincident points need no guard. ZEROW: w = 0 (point
// sources), the exponent is -r' itself.
template <int KT, bool ZEROW = false>
__device__ __forceinline__ float2 kscaled2(float2 r2, float2 w, const KParams<float>& kp) {
  constexpr float c1 = kLn2;                         // argument per unit of r'
  constexpr float c2 = kLn2 * kLn2;
  if constexpr (KT == 3) {  // GAUSSIAN: 2^(w - r'^2)
    const float2 u = ZEROW ? f2(-r2.x, -r2.y) : __ffma2_rn(r2, f2(-1.f, -1.f), w);
    return f2(ex2_approx(u.x), ex2_approx(u.y));
  } else if constexpr (KT == 13) {  // l dk/dl of GAUSSIAN: 2 ln2 r'^2 2^-r'^2
    const float2 u = ZEROW ? f2(-r2.x, -r2.y) : __ffma2_rn(r2, f2(-1.f, -1.f), w);
    const float2 e = f2(ex2_approx(u.x), ex2_approx(u.y));
    return __fmul2_rn(__fmul2_rn(r2, f2(2.f * kLn2, 2.f * kLn2)), e);
  } else if constexpr (KT == 0 || KT == 1 || KT == 2 || KT == 4 || KT == 5 || KT == 10 ||
                       KT == 11 || KT == 12) {
    const float2 r = f2(sqrt_approx(r2.x), sqrt_approx(r2.y));
    const float2 u = ZEROW ? f2(-r.x, -r.y) : __ffma2_rn(r, f2(-1.f, -1.f), w);
    const float2 e = f2(ex2_approx(u.x), ex2_approx(u.y));
    if constexpr (KT == 0) {  // EXPONENTIAL: 2^(w - r')
      return e;
    } else if constexpr (KT == 1) {  // MATERN32: (1 + t) e^-t, t = ln2 r'
      return __fmul2_rn(__ffma2_rn(r, f2(c1, c1), f2(1.f, 1.f)), e);
    } else if constexpr (KT == 2) {  // MATERN52: (1 + t + t^2 / 3) e^-t
      const float2 p = __ffma2_rn(__ffma2_rn(r, f2(c2 / 3.f, c2 / 3.f), f2(c1, c1)), r,
                                  f2(1.f, 1.f));
      return __fmul2_rn(p, e);
    } else if constexpr (KT == 4) {  // MATERN72: (1 + t + 2 t^2 / 5 + t^3 / 15) e^-t
      constexpr float k2 = 0.4f * c2, k3 = c2 * c1 / 15.f;
      const float2 p = __ffma2_rn(__ffma2_rn(__ffma2_rn(r, f2(k3, k3), f2(k2, k2)), r,
                                             f2(c1, c1)),
                                  r, f2(1.f, 1.f));
      return __fmul2_rn(p, e);
    } else if constexpr (KT == 5) {  // MATERN92: (1 + t + 3 t^2 / 7 + 2 t^3 / 21 + t^4 / 105) e^-t
      constexpr float k2 = 3.f / 7.f * c2, k3 = 2.f / 21.f * c2 * c1, k4 = c2 * c2 / 105.f;
      const float2 p = __ffma2_rn(
          __ffma2_rn(__ffma2_rn(__ffma2_rn(r, f2(k4, k4), f2(k3, k3)), r, f2(k2, k2)), r,
                     f2(c1, c1)),
          r, f2(1.f, 1.f));
      return __fmul2_rn(p, e);
    } else if constexpr (KT == 10) {  // l dk/dl of EXPONENTIAL: t e^-t
      return __fmul2_rn(__fmul2_rn(r, f2(c1, c1)), e);
    } else if constexpr (KT == 11) {  // l dk/dl of MATERN32: t^2 e^-t
      return __fmul2_rn(__fmul2_rn(r2, f2(c2, c2)), e);
    } else {  // l dk/dl of MATERN52: t^2 / 3 (1 + t) e^-t
      const float2 p = __fmul2_rn(__fmul2_rn(r2, f2(c2 / 3.f, c2 / 3.f)),
                                  __ffma2_rn(r, f2(c1, c1), f2(1.f, 1.f)));
      return __fmul2_rn(p, e);
    }
  } else {
    return f2(keval_fast(kp.type, r2.x, kp) * pow2i(w.x),
              keval_fast(kp.type, r2.y, kp) * pow2i(w.y));
  }
}

// Source layouts of the tensor-core kernel sums (8 zero sources of padding
// after the last one):
//   pairs   record p = sources 2p, 2p + 1 as two float4
//           (-g x0, -g x1, -g y0, -g y1), (-g z0, -g z1, w0, w1);
//   values  FP16 hi and lo parts, element (s, r) of part p (0 hi, 1 lo) at
//           half index um_val_index(s, r, p): 1 KB per 8 sources, 8 x 8
//           blocks [r % 8][s % 8] ordered by p, r / 8 — the K-major core
//           matrices of a B operand of 64 columns (32 hi | 32 lo).
__host__ __device__ __forceinline__ size_t um_val_index(size_t s, int r, int p) {
  return (s >> 3) * 512 + (size_t)p * 256 + (size_t)(r >> 3) * 64 + (size_t)(r & 7) * 8 +
         (s & 7);
}
__host__ __device__ __forceinline__ size_t um_padded(size_t n) {
  return ((n + 7) & ~(size_t)7) + 8;
}

// per-column max |x| as FP32 bits (positive floats order like integers) for
// columns [c0, c0 + nc); a block reduces into shared memory first and
// flushes once per column
template <typename TI>
__global__ void colmax_kernel(int64_t n, int c0, int nc, const TI* __restrict__ x,
                              int64_t sxi, int64_t sxr, unsigned int* __restrict__ cmax) {
  // lane = column of a group of 32, warps stride over the rows; the maximum
  // is taken over the bit patterns of |x| (non-negative floating-point
  // numbers order like their bits) and converted to FP32 once: conversion
  // is monotone, so that equals the maximum of the converted elements
  extern __shared__ unsigned int smax[];
  for (int r = threadIdx.x; r < nc; r += blockDim.x) smax[r] = 0u;
  __syncthreads();
  using U = typename std::conditional<sizeof(TI) == 8, unsigned long long, unsigned int>::type;
  constexpr U kAbs = sizeof(TI) == 8 ? (U)0x7FFFFFFFFFFFFFFFull : (U)0x7FFFFFFFu;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int cg = 0; cg < nc; cg += 32) {
    const int r = cg + lane;
    if (r >= nc) continue;
    const U* p = reinterpret_cast<const U*>(x) + (int64_t)(c0 + r) * sxr + warp * sxi;
    const int64_t step = nwarps * sxi;
    U m = 0;
    for (int64_t i = warp; i < n; i += nwarps, p += step) {
      const U b = *p & kAbs;
      m = b > m ? b : m;
    }
    float mf;
    if constexpr (sizeof(TI) == 8)
      mf = (float)__longlong_as_double((long long)m);
    else
      mf = __uint_as_float(m);
    atomicMax(&smax[r], __float_as_uint(mf));
  }
  __syncthreads();
  for (int r = threadIdx.x; r < nc; r += blockDim.x)
    if (smax[r]) atomicMax(&cmax[c0 + r], smax[r]);
}

// power-of-two exponent that maps max |v| into (1/2, 1]; 0 for max = 0
__device__ __forceinline__ int scale_exp(float m) {
  if (!(m > 0.f) || !isfinite(m)) return 0;
  int e;
  frexpf(m, &e);  // m = f * 2^e, f in [0.5, 1)
  return e;
}

// gather for the mixed path: x' = x * 2^-e_r in cluster order, as FP32
// (chunk-major [chunk][n][32], for the CUDA-core tree passes) and as FP16
// hi / lo parts in the values layout ([chunk][um_padded(n) sources],
// padding zero)
// v * 2^-e, rounded once as ldexpf does: a multiply by an exact power of
// two while 2^-e is a normal FP32 number
__device__ __forceinline__ float scale_pow2(float v, int e) {
  return (e >= -127 && e <= 126) ? v * __int_as_float((127 - e) << 23) : ldexpf(v, -e);
}

template <typename TI>
__global__ void gather_split_kernel(const uint32_t* __restrict__ perm, int64_t n, int R,
                                    const TI* __restrict__ x, int64_t sxi, int64_t sxr,
                                    const unsigned int* __restrict__ cmax,
                                    float* __restrict__ xc, __half* __restrict__ xv) {
  // chunk blockIdx.y; one thread per 8 consecutive sources and right-hand
  // side of the chunk (the thread count of the grid is a multiple of 32, so
  // a thread keeps its right-hand side): the 8 FP16 hi (lo) values of a
  // core-matrix row are one 16-byte store
  const int64_t ch = blockIdx.y;
  const int64_t np = (int64_t)um_padded(n);
  const int64_t total = (np / 8) * kTcRhs;
  const int64_t first = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int rr = (int)(first & (kTcRhs - 1));
  const int r = (int)ch * kTcRhs + rr;
  const int ex = r < R ? scale_exp(__uint_as_float(cmax[r])) : 0;
  const TI* xr = x + (int64_t)r * sxr;
  float* xo = xc + ch * n * kTcRhs + rr;
  __half* o = xv + (size_t)ch * np * kTcRhs * 2;
  for (int64_t e = first; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t blk = e >> 5;
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int jj = 0; jj < 8; jj += 2) {
      float v[2];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int64_t i = blk * 8 + jj + t;
        v[t] = 0.f;
        if (r < R && i < n) {
          const int64_t src = perm ? (int64_t)perm[i] : i;
          v[t] = scale_pow2((float)xr[src * sxi], ex);
        }
        if (i < n) xo[i * kTcRhs] = v[t];
      }
      const __half2 h = __floats2half2_rn(v[0], v[1]);
      const float2 hf = __half22float2(h);
      hw[jj / 2] = h2_bits(h);
      lw[jj / 2] = h2_bits(__floats2half2_rn(v[0] - hf.x, v[1] - hf.y));
    }
    *reinterpret_cast<uint4*>(o + um_val_index((size_t)blk * 8, rr, 0)) =
        make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(o + um_val_index((size_t)blk * 8, rr, 1)) =
        make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

// pair records of n points (cluster order), coordinates multiplied by -g,
// w = 0; zero records up to um_padded(n)
// Kernels whose near field takes the squared distance in the dot-product
// form r^2 = (|t|^2 + |s|^2) - 2 t.s (four FP32x2 instructions per two
// sources instead of six). Its rounding error, a few ulp of |t|^2 + |s|^2
// in coordinates centred on the clouds' box, enters k through dk/d(r^2),
// which is bounded at r = 0 for these kernels (MATERN32..92, GAUSSIAN and
// their l dk/dl). EXPONENTIAL and its l dk/dl have dk/dr = -1/l at r = 0:
// there an error of d in r^2 moves k by about sqrt(d), so they keep the
// difference form.
__host__ __device__ constexpr bool um_near_dot(int kt) {
  return kt == 1 || kt == 2 || kt == 3 || kt == 4 || kt == 5 || kt == 11 || kt == 12 ||
         kt == 13;
}

// FP32 coordinate u of a point in the dot form: g (x - c), with the same
// two rounded operations for targets and sources
__device__ __forceinline__ float um_dot_coord(float x, float c, float g) {
  return __fmul_rn(g, __fsub_rn(x, c));
}
__device__ __forceinline__ float um_dot_norm(float ux, float uy, float uz) {
  return (float)((double)ux * ux + (double)uy * uy + (double)uz * uz);
}

// Point sources in the dot form: record p = sources 2p, 2p + 1 as
// (2 u_x0, 2 u_x1, 2 u_y0, 2 u_y1), (2 u_z0, 2 u_z1, |u_0|^2, |u_1|^2),
// u = g (x - c); zero records of padding
static __global__ void point_pairs_dot_kernel(int64_t n, const Pt4<float>* __restrict__ pts,
                                              KParams<float> kp, float4* __restrict__ pairs) {
  const int64_t np = (int64_t)um_padded(n) / 2;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float u[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}}, nn[2] = {0.f, 0.f};
    for (int k = 0; k < 2; ++k) {
      const int64_t s = 2 * p + k;
      if (s >= n) continue;
      const Pt4<float> a = pts[s];
      u[k][0] = um_dot_coord(a.x, kp.cx, kp.g);
      u[k][1] = um_dot_coord(a.y, kp.cy, kp.g);
      u[k][2] = um_dot_coord(a.z, kp.cz, kp.g);
      nn[k] = um_dot_norm(u[k][0], u[k][1], u[k][2]);
    }
    pairs[2 * p] = make_float4(2.f * u[0][0], 2.f * u[1][0], 2.f * u[0][1], 2.f * u[1][1]);
    pairs[2 * p + 1] = make_float4(2.f * u[0][2], 2.f * u[1][2], nn[0], nn[1]);
  }
}

static __global__ void point_pairs_kernel(int64_t n, const Pt4<float>* __restrict__ pts, float g,
                                   float4* __restrict__ pairs) {
  const int64_t np = (int64_t)um_padded(n) / 2;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s0 = 2 * p, s1 = 2 * p + 1;
    Pt4<float> a{0.f, 0.f, 0.f, 0.f}, b{0.f, 0.f, 0.f, 0.f};
    if (s0 < n) a = pts[s0];
    if (s1 < n) b = pts[s1];
    pairs[2 * p] = make_float4(-g * a.x, -g * b.x, -g * a.y, -g * b.y);
    pairs[2 * p + 1] = make_float4(-g * a.z, -g * b.z, 0.f, 0.f);
  }
}

// per column cluster c (one block each): e = exponent of max |t|, the
// moments t'' = t * 2^-e split into FP16 hi / lo in the values layout, and
// the pair-record entries of the cluster's q nodes with coordinates
// multiplied by -g and w = e (-1000 for a cluster without moments). The
// last block also zeroes the padding after node C q.
static __global__ void tscale_kernel(int C, int q, int rcount, const float* __restrict__ t,
                              const Pt4<float>* __restrict__ nodes, float g,
                              __half* __restrict__ tv, float* __restrict__ pairs) {
  const int c = blockIdx.x;
  if (c >= C) return;
  __shared__ float red[32];
  const size_t base = (size_t)c * q * kTcRhs;
  float m = 0.f;
  for (int e = threadIdx.x; e < q * kTcRhs; e += blockDim.x)
    if ((e % kTcRhs) < rcount) m = fmaxf(m, fabsf(t[base + e]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const float mx = red[0];
  const int ex = scale_exp(mx);
  const float w = mx > 0.f && isfinite(mx) ? (float)ex : -1000.f;
  for (int e = threadIdx.x; e < q * kTcRhs; e += blockDim.x) {
    const int r = e % kTcRhs;
    const float v = r < rcount ? ldexpf(t[base + e], -ex) : 0.f;
    const __half h = __float2half_rn(v);
    const size_t sidx = (size_t)c * q + e / kTcRhs;
    tv[um_val_index(sidx, r, 0)] = h;
    tv[um_val_index(sidx, r, 1)] = __float2half_rn(v - __half2float(h));
  }
  for (int k = threadIdx.x; k < q; k += blockDim.x) {
    const size_t s = (size_t)c * q + k;
    const Pt4<float> p = nodes[s];
    float* rec = pairs + (s >> 1) * 8 + (s & 1);
    rec[0] = -g * p.x;
    rec[2] = -g * p.y;
    rec[4] = -g * p.z;
    rec[6] = w;
  }
  if (c == C - 1) {
    const size_t n = (size_t)C * q, np = um_padded(n);
    for (size_t s = n + threadIdx.x; s < np; s += blockDim.x) {
      float* rec = pairs + (s >> 1) * 8 + (s & 1);
      rec[0] = rec[2] = rec[4] = rec[6] = 0.f;
      for (int r = 0; r < kTcRhs; ++r) {
        tv[um_val_index(s, r, 0)] = __float2half_rn(0.f);
        tv[um_val_index(s, r, 1)] = __float2half_rn(0.f);
      }
    }
  }
}

// Far-field sources on tensor grids (dimension 3, kGridP1^3 nodes per
// cluster): cluster c owns value rows [c * 128, c * 128 + 128) in grid order
// (node with digits (a, b, c') at row (a P1 + b) P1 + c'), rows past P1^3
// zero; and a 64-byte record rec[c] = (X[0][0..P1), X[1][0..P1),
// X[2][0..P1), w): the coordinate -g x of each grid line and the moment
// exponent w (-1000 for a cluster without moments).
constexpr int kGridP1 = 5;
constexpr int kGridRows = 128;

// per column cluster c (one block each, q = kGridP1^3 nodes): moments t in
// the plan's node order, midx = digits of each node (3 per node)
static __global__ void tscale_grid_kernel(int C, int rcount, const float* __restrict__ t,
                                   const Pt4<float>* __restrict__ nodes,
                                   const int* __restrict__ midx, float g,
                                   __half* __restrict__ tv, float* __restrict__ rec) {
  constexpr int q = kGridP1 * kGridP1 * kGridP1;
  const int c = blockIdx.x;
  if (c >= C) return;
  __shared__ float red[32];
  __shared__ int node_of_row[kGridRows];  // node index of each grid row, -1 past q
  const size_t base = (size_t)c * q * kTcRhs;
  for (int k = threadIdx.x; k < kGridRows; k += blockDim.x) node_of_row[k] = -1;
  __syncthreads();
  for (int k = threadIdx.x; k < q; k += blockDim.x)
    node_of_row[(midx[3 * k] * kGridP1 + midx[3 * k + 1]) * kGridP1 + midx[3 * k + 2]] = k;
  float m = 0.f;
  const float4* t4 = reinterpret_cast<const float4*>(t + base);
  for (int e = threadIdx.x; e < q * kTcRhs / 4; e += blockDim.x) {
    const float4 v = t4[e];
    const int r0 = (4 * e) % kTcRhs;
    if (r0 + 0 < rcount) m = fmaxf(m, fabsf(v.x));
    if (r0 + 1 < rcount) m = fmaxf(m, fabsf(v.y));
    if (r0 + 2 < rcount) m = fmaxf(m, fabsf(v.z));
    if (r0 + 3 < rcount) m = fmaxf(m, fabsf(v.w));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const float mx = red[0];
  const int ex = scale_exp(mx);
  // one thread per 8 grid rows and right-hand side: the 8 FP16 hi (lo)
  // values of a core-matrix row are one 16-byte store
  const size_t row0 = (size_t)c * kGridRows;
  for (int task = threadIdx.x; task < (kGridRows / 8) * kTcRhs; task += blockDim.x) {
    const int rb = task / kTcRhs, r = task % kTcRhs;
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int jj = 0; jj < 8; jj += 2) {
      float v[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int k = node_of_row[rb * 8 + jj + u];
        v[u] = (k >= 0 && r < rcount) ? scale_pow2(t[base + (size_t)k * kTcRhs + r], ex) : 0.f;
      }
      const __half2 h = __floats2half2_rn(v[0], v[1]);
      const float2 hf = __half22float2(h);
      hw[jj / 2] = h2_bits(h);
      lw[jj / 2] = h2_bits(__floats2half2_rn(v[0] - hf.x, v[1] - hf.y));
    }
    *reinterpret_cast<uint4*>(tv + um_val_index(row0 + rb * 8, r, 0)) =
        make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(tv + um_val_index(row0 + rb * 8, r, 1)) =
        make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
  // grid lines: the nodes with digits (i, 0, 0), (0, i, 0), (0, 0, i) give
  // X[d][i] (every node of a line shares that coordinate)
  float* rc = rec + (size_t)c * 16;
  for (int k = threadIdx.x; k < q; k += blockDim.x) {
    const int a = midx[3 * k], b = midx[3 * k + 1], cc = midx[3 * k + 2];
    const Pt4<float> p = nodes[(size_t)c * q + k];
    if (b == 0 && cc == 0) rc[a] = -g * p.x;
    if (a == 0 && cc == 0) rc[kGridP1 + b] = -g * p.y;
    if (a == 0 && b == 0) rc[2 * kGridP1 + cc] = -g * p.z;
  }
  if (threadIdx.x == 0) rc[15] = mx > 0.f && isfinite(mx) ? (float)ex : -1000.f;
}

// y (natural order) = sigma2 * 2^e_r * (ynear + yfar): the two FP32 parts
// added in FP32 (one rounding, 6e-8 relative), the scaling in FP64. FP64
// arithmetic is scarce on this part (two operations per clock and SM), so
// an element costs one conversion and one multiply; the column's scale
// sigma2 * 2^e_r is formed from its exponent bits once per thread (v *
// (sigma2 2^e) rounds once, like ldexp(sigma2 v, e)). Lane = column of a
// group of 32, warps stride over the rows.
template <typename TO>
__global__ void scatter_scaled_kernel(const uint32_t* __restrict__ perm, int64_t n, int R,
                                      const float* __restrict__ ynear,
                                      const float* __restrict__ yfar,
                                      const unsigned int* __restrict__ cmax, double sigma2,
                                      TO* __restrict__ y, int64_t syi, int64_t syr) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int cg = 0; cg < R; cg += kTcRhs) {
    const int r = cg + lane;
    if (r >= R) continue;
    const int ex = scale_exp(__uint_as_float(cmax[r]));
    const double sc = sigma2 * __longlong_as_double((long long)(ex + 1023) << 52);
    const int64_t off = (int64_t)(r / kTcRhs) * n * kTcRhs + r % kTcRhs;
    const float* yn = ynear + off;
    const float* yf = yfar + off;
    TO* yr = y + (int64_t)r * syr;
    for (int64_t i = warp; i < n; i += nwarps) {
      const float v = yn[i * kTcRhs] + yf[i * kTcRhs];
      const int64_t dst = perm ? (int64_t)perm[i] : i;
      yr[dst * syi] = (TO)((double)v * sc);
    }
  }
}

}  // namespace gpu
}  // namespace fmca
