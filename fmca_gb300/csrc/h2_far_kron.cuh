// Far field of the GAUSSIAN kernel as Kronecker products.  The kernels below
// are instantiated only in h2_far_kron.cu, a translation unit of its own, so
// that their instantiations compile in parallel with h2_gpu.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "h2_gpu_kernels.cuh"

namespace fmca {
namespace gpu {

// Far field of the GAUSSIAN kernel on tensor-product nodes, as Kronecker
// products.  exp(e |u - v|^2) = prod_d exp(e (u_d - v_d)^2), so the coupling
// matrix of an admissible block (tau, sigma), K at the node pairs
// (NystromEvaluator.h:40-56 with invV = I), is the Kronecker product of DIM
// factors S_d[a][b] = exp(e (x^tau_d(a) - x^sigma_d(b))^2) of P x P, and
//   s_tau = sum_sigma (S_0 (x) ... (x) S_{DIM-1}) t_sigma
// costs DIM contractions of P terms per coefficient instead of Q kernel
// values and Q terms.  x_d(a) are the node coordinates of the plan (the
// node whose digits are a in dimension d and 0 elsewhere), e = -1 / (2 l^2)
// (FP64) or -log2(e) / (2 l^2) applied with ex2 (FP32, as keval_fast).
// Block = one far group (the nodes of one row cluster, Q <= 256).  A lane
// holds right-hand side r = lane % RW of source cluster slot lane / RW:
// 32 / RW source clusters are contracted at once (RW = 32, 8 or 1 columns),
// coefficients in tensor order in shared memory like transfer_sf_kernel;
// the slots' sums are added at the end.  Writes s[tau] (every row cluster
// has a group; those without admissible blocks write zeros).
// shared: X, Y, Z [Q][32] T, xt [DIM][P] T, ef [SL][DIM][P][P] T, sidx [Q]
// ints, scl [SL] ints
template <typename T, int DIM, int P, int RW>
__global__ void __launch_bounds__(256)
    far_kron_kernel(const KGroup* __restrict__ groups, const uint32_t* __restrict__ ivl,
                    const Pt4<T>* __restrict__ nodes_r, const Pt4<T>* __restrict__ nodes_c,
                    const int* __restrict__ midx_g, T e, const T* __restrict__ t, int ldt,
                    int tofs, T* __restrict__ s, int lds, int sofs, int rcount) {
  constexpr int Q = DIM == 1 ? P : DIM == 2 ? P * P : P * P * P;
  constexpr int NC = Q / P;
  constexpr int SL = 32 / RW;          // source clusters per step
  constexpr int NF = DIM * P * P;      // factor entries per source cluster
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* X = reinterpret_cast<T*>(smem_raw);
  T* Y = X + Q * 32;
  T* Z = Y + Q * 32;
  T* xt = Z + Q * 32;     // [DIM][P]
  T* ef = xt + DIM * P;   // [SL][DIM][P][P]
  int* sidx = reinterpret_cast<int*>(ef + SL * NF);  // tensor position -> storage index
  int* scl = sidx + Q;                               // [SL] source clusters of the step
  const KGroup g = groups[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int slot = lane / RW, col = lane % RW;
  const bool live = col < rcount;
  const int r = tofs + col;
  for (int k = threadIdx.x; k < Q; k += blockDim.x) {
    int pos = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) pos = pos * P + midx_g[k * 3 + d];
    sidx[pos] = k;
  }
  for (int i = threadIdx.x; i < Q * 32; i += blockDim.x) Z[i] = T(0);
  __syncthreads();
  // stride of digit d in tensor order
  auto stride_of = [](int d) { return d == DIM - 1 ? 1 : (d == DIM - 2 ? P : P * P); };
  auto coord = [](const Pt4<T>& p, int d) { return d == 0 ? p.x : (d == 1 ? p.y : p.z); };
  for (int i = threadIdx.x; i < DIM * P; i += blockDim.x) {
    const int d = i / P, a = i - d * P;
    xt[i] = coord(nodes_r[g.tbegin + sidx[a * stride_of(d)]], d);
  }
  // source clusters: the group's node intervals, cluster by cluster
  int iv = g.ivl_begin;
  uint32_t cur = iv < g.ivl_end ? ivl[2 * iv] / Q : 0u;
  constexpr int U = 8;
  while (true) {
    __syncthreads();  // the previous step is done with X, Y, ef and scl
    if (threadIdx.x == 0) {
      for (int j = 0; j < SL; ++j) {
        while (iv < g.ivl_end && cur >= ivl[2 * iv + 1] / Q) {
          ++iv;
          if (iv < g.ivl_end) cur = ivl[2 * iv] / Q;
        }
        scl[j] = iv < g.ivl_end ? (int)cur++ : -1;
      }
    }
    __syncthreads();
    if (scl[0] < 0) break;
    for (int i = threadIdx.x; i < SL * NF; i += blockDim.x) {
      const int j = i / NF, f = i - j * NF;
      const int d = f / (P * P), a = (f / P) % P, b = f % P;
      T v = T(0);
      if (scl[j] >= 0) {
        const T dv = xt[d * P + a] -
                     coord(nodes_c[(size_t)scl[j] * Q + sidx[b * stride_of(d)]], d);
        if constexpr (sizeof(T) == 4)
          v = ex2_approx(dv * dv * e);
        else
          v = exp(dv * dv * e);
      }
      ef[i] = v;
    }
    const int sc = scl[slot];
    for (int t0 = warp; t0 < Q; t0 += nw * U) {
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int q = t0 + nw * u;
        v[u] = (q < Q && live && sc >= 0) ? t[((size_t)sc * Q + sidx[q]) * ldt + r] : T(0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (t0 + nw * u < Q) X[(t0 + nw * u) * 32 + lane] = v[u];
    }
    __syncthreads();
    T* in = X;
    T* out = Y;
    const T* efs = ef + slot * NF;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int stride = stride_of(d);
      T f[P][P];
#pragma unroll
      for (int a = 0; a < P; ++a)
#pragma unroll
        for (int b = 0; b < P; ++b) f[a][b] = efs[(d * P + a) * P + b];
      const bool last = d == DIM - 1;
      for (int c = warp; c < NC; c += nw) {
        const int hi = c / stride, lo = c % stride;
        const int base = hi * stride * P + lo;
        T v[P];
#pragma unroll
        for (int j = 0; j < P; ++j) v[j] = in[(base + j * stride) * 32 + lane];
#pragma unroll
        for (int a = 0; a < P; ++a) {
          T acc = T(0);
#pragma unroll
          for (int j = 0; j < P; ++j) acc = fma(f[a][j], v[j], acc);
          const int o = (base + a * stride) * 32 + lane;
          if (!last)
            out[o] = acc;
          else
            Z[o] += acc;
        }
      }
      if (!last) __syncthreads();
      T* tmp = in;
      in = out;
      out = tmp;
    }
  }
  // every lane's last contraction wrote Z before the loop's final barrier
  for (int i = threadIdx.x; i < Q * RW; i += blockDim.x) {
    const int q = i / RW, c = i - q * RW;
    if (c < rcount) {
      T sum = T(0);
#pragma unroll
      for (int j = 0; j < SL; ++j) sum += Z[q * 32 + j * RW + c];
      s[((size_t)g.tbegin + sidx[q]) * lds + sofs + c] = sum;
    }
  }
}

// The same far field in FP32 for grids of Q <= 64 nodes: one warp per far
// group, no barrier but __syncwarp.  Each lane holds one right-hand side
// (r = lane % RW) of one source cluster (slot lane / RW, SL = 32 / RW
// clusters per step) as Q registers: every index of the contractions is a
// compile-time constant once the loops are unrolled, so the DIM
// contractions run in place on the registers, fibre by fibre, and the last
// one is added into the lane's column of the accumulator Z in shared
// memory.  Lanes of unused columns load a used one (their sums are never
// read); slots past the group's last source cluster load its first one and
// get zero factors.  At the end the slots' columns of Z are added.
// Every source cluster's coefficients are read once per admissible block
// (about 50 times): the columns should fill the rows of t (ldt = the
// columns in use), so that t stays in L2 for the re-reads.
// shared: sidx, soff [Q4] ints, sb [DP4] ints, xt [DP4], Z [Q][32],
// xs [SL][DP], ef [SL][NFS] floats, scls [SL] ints
template <int DIM, int P>
struct KronShape {
  static constexpr int Q = DIM == 2 ? P * P : P * P * P;
  static constexpr int DP = DIM * P;      // 1-D nodes of all dimensions
  static constexpr int NF = DIM * P * P;  // factor entries per source cluster
  static constexpr int NFS = NF | 1;      // odd slot stride: slots on distinct banks
  static constexpr int Q4 = (Q + 3) / 4 * 4;
  static constexpr int DP4 = (DP + 3) / 4 * 4;
  // shared-memory bytes for RW columns per slot
  static constexpr size_t smem_bytes(int rw) {
    return sizeof(int) * (2 * Q4 + DP4) +
           sizeof(float) * (DP4 + Q * 32 + (32 / rw) * (DP + NFS)) + sizeof(int) * (32 / rw);
  }
  // stride of digit d in tensor order (digit 0 most significant)
  static constexpr int stride(int d) { return d == DIM - 1 ? 1 : (d == DIM - 2 ? P : P * P); }
};

template <int DIM, int P, int RW>
__global__ void __launch_bounds__(32)
    far_kron_reg_kernel(const KGroup* __restrict__ groups, const uint32_t* __restrict__ ivl,
                        const Pt4<float>* __restrict__ nodes_r,
                        const Pt4<float>* __restrict__ nodes_c, const int* __restrict__ midx_g,
                        float e, const float* __restrict__ t, int ldt, int tofs,
                        float* __restrict__ s, int lds, int sofs, int rcount) {
  using S = KronShape<DIM, P>;
  constexpr int Q = S::Q, DP = S::DP, NF = S::NF, NFS = S::NFS;
  constexpr int SL = 32 / RW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* sidx = reinterpret_cast<int*>(smem_raw);  // tensor position -> storage index
  int* soff = sidx + S::Q4;                      // sidx * ldt
  int* sb = soff + S::Q4;  // [DIM][P] storage index of the node with digit d = b, others 0
  float* xt = reinterpret_cast<float*>(sb + S::DP4);  // [DIM][P] target node coordinates
  float* Z = xt + S::DP4;                             // [Q][32]
  float* xs = Z + Q * 32;                             // [SL][DIM][P] source node coordinates
  float* ef = xs + SL * DP;                           // [SL][NFS] factors [d][a][b]
  int* scls = reinterpret_cast<int*>(ef + SL * NFS);  // [SL] clusters of the step
  const KGroup g = groups[blockIdx.x];
  const int lane = threadIdx.x;
  const int slot = lane / RW, col = lane % RW;
  auto coord = [](const Pt4<float>& p, int d) { return d == 0 ? p.x : (d == 1 ? p.y : p.z); };
  for (int k = lane; k < Q; k += 32) {
    int pos = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) pos = pos * P + midx_g[k * 3 + d];
    sidx[pos] = k;
  }
#pragma unroll
  for (int q = 0; q < Q; ++q) Z[q * 32 + lane] = 0.f;
  __syncwarp();
  for (int q = lane; q < Q; q += 32) soff[q] = sidx[q] * ldt;
  for (int i = lane; i < DP; i += 32) {
    const int d = i / P, b = i - d * P;
    const int k = sidx[b * S::stride(d)];
    sb[i] = k;
    xt[i] = coord(nodes_r[g.tbegin + k], d);
  }
  __syncwarp();
  // the walk over the group's source clusters (uniform over the warp):
  // interval iv, next cluster cur of it
  int iv = g.ivl_begin;
  uint32_t cur = 0, cend = 0;
  if (iv < g.ivl_end) {
    cur = ivl[2 * iv] / Q;
    cend = ivl[2 * iv + 1] / Q;
  }
  auto next_cluster = [&]() -> int {
    while (iv < g.ivl_end && cur >= cend) {
      if (++iv < g.ivl_end) {
        cur = ivl[2 * iv] / Q;
        cend = ivl[2 * iv + 1] / Q;
      }
    }
    return iv < g.ivl_end ? (int)cur++ : -1;
  };
  const int cc = tofs + (col < rcount ? col : rcount - 1);
  while (true) {
    int sc = -1, sc0 = -1;
#pragma unroll
    for (int j = 0; j < SL; ++j) {
      const int c = next_cluster();
      if (j == 0) sc0 = c;
      if (j == slot) sc = c;
    }
    if (sc0 < 0) break;
    // this lane's column of its source cluster's coefficients; the loads
    // are issued before the factors are computed
    float x[Q];
    {
      const float* tc = t + (size_t)(sc < 0 ? sc0 : sc) * Q * ldt + cc;
#pragma unroll
      for (int q = 0; q < Q; ++q) x[q] = __ldg(tc + soff[q]);
    }
    __syncwarp();  // the previous step is done with scls, xs and ef
    if (col == 0) scls[slot] = sc;
    __syncwarp();
    for (int i = lane; i < SL * DP; i += 32) {
      const int j = i / DP, f = i - j * DP;
      const int sj = scls[j];
      xs[i] = coord(nodes_c[(size_t)(sj < 0 ? sc0 : sj) * Q + sb[f]], f / P);
    }
    __syncwarp();
    // factor rows (slot j, dimension d, target node a), P entries each
    for (int i = lane; i < SL * DP; i += 32) {
      const int j = i / DP, f = i - j * DP, d = f / P;
      const bool used = scls[j] >= 0;
      const float xa = xt[f];
      const float* xr = xs + j * DP + d * P;
      float* er = ef + j * NFS + f * P;
#pragma unroll
      for (int b = 0; b < P; ++b) {
        const float dv = xa - xr[b];
        er[b] = used ? ex2_approx(dv * dv * e) : 0.f;
      }
    }
    __syncwarp();
    const float* efs = ef + slot * NFS;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      constexpr int NC = Q / P;
      const int stride = S::stride(d);
      float f[P][P];
#pragma unroll
      for (int a = 0; a < P; ++a)
#pragma unroll
        for (int b = 0; b < P; ++b) f[a][b] = efs[(d * P + a) * P + b];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const int base = (c / stride) * stride * P + c % stride;
        float v[P];
#pragma unroll
        for (int j = 0; j < P; ++j) v[j] = x[base + j * stride];
#pragma unroll
        for (int a = 0; a < P; ++a) {
          const int o = base + a * stride;
          float acc = d == DIM - 1 ? Z[o * 32 + lane] : 0.f;
#pragma unroll
          for (int j = 0; j < P; ++j) acc = fmaf(f[a][j], v[j], acc);
          if (d == DIM - 1)
            Z[o * 32 + lane] = acc;
          else
            x[o] = acc;
        }
      }
    }
  }
  __syncwarp();
  for (int i = lane; i < Q * RW; i += 32) {
    const int q = i / RW, c = i - q * RW;
    if (c < rcount) {
      float sum = 0.f;
#pragma unroll
      for (int j = 0; j < SL; ++j) sum += Z[q * 32 + j * RW + c];
      s[((size_t)g.tbegin + sidx[q]) * lds + sofs + c] = sum;
    }
  }
}

}  // namespace gpu
}  // namespace fmca

