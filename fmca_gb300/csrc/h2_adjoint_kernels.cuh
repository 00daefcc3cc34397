// Device code of the H2 adjoint: gradients of f = sum_r y_r^T K_H2 x_r with
// respect to the point coordinates, the cluster tree and the boxes held fixed.
//
// K_H2 = Near + V_r^T A V_c, where A (transfers and couplings at the fixed
// interpolation nodes) does not depend on the points.  With U^x = A V_c x
// (the leaf expansions the leaf gather consumes, one q x R block per row
// leaf):
//   df/dp_i (near) = sum_j c_ij g(|p_i - q_j|) (p_i - q_j),
//                    c_ij = sum_r y_ir x_jr, g(r) = k'(r) / r
//   df/dp_i (far)  = sum_k grad V_r[k, i](p_i) . sum_r U^x[k, r] y_ir
// The column-side terms are the same expressions with x and y exchanged
// (and U^y = A^T V_r y); for one point cloud both add up.
#pragma once

#include "h2_gpu_kernels.cuh"
#include "h2_tc_kernels.cuh"

namespace fmca {
namespace gpu {

// g(r) = k'(r) / r of the four covariance kernels (0 at r = 0, where the
// pair's gradient vanishes because p_i - q_j = 0)
__device__ __forceinline__ double kgrad_ref(int type, double r2, const KParams<double>& kp) {
  if (!(r2 > 0.)) return 0.;
  const double r = sqrt(r2), l = kp.l;
  switch (type) {
    case 0:
      return -exp(-r / l) / (l * r);
    case 1:
      return -kp.a * kp.a * exp(-kp.a * r);
    case 2:
      return -(kp.a * kp.a / 3.) * (1. + kp.a * r) * exp(-kp.a * r);
    case 3:
      return -exp(-0.5 * r2 / (l * l)) / (l * l);
  }
  return 0.;
}

__device__ __forceinline__ float kgrad_fast(int type, float r2, const KParams<float>& kp) {
  if (!(r2 > 0.f)) return 0.f;
  switch (type) {
    case 0: {
      const float r = sqrt_approx(r2);
      return -ex2_approx(r * kp.e2) * kp.il / r;
    }
    case 1: {
      const float r = sqrt_approx(r2);
      return -kp.a * kp.a * ex2_approx(r * kp.e2);
    }
    case 2: {
      const float r = sqrt_approx(r2);
      return -(kp.a * kp.a * 0.333333343f) * fmaf(kp.a, r, 1.f) * ex2_approx(r * kp.e2);
    }
    case 3:
      return -ex2_approx(r2 * kp.e2) * kp.il * kp.il;
  }
  return 0.f;
}

template <typename T>
__device__ __forceinline__ T kgrad(int type, T r2, const KParams<T>& kp);
template <>
__device__ __forceinline__ double kgrad<double>(int type, double r2, const KParams<double>& kp) {
  return kgrad_ref(type, r2, kp);
}
template <>
__device__ __forceinline__ float kgrad<float>(int type, float r2, const KParams<float>& kp) {
  return kgrad_fast(type, r2, kp);
}

// Near-field gradient: G[t] += scale * sum_s c_ts g(|p_t - q_s|) (p_t - q_s)
// (accumulated pair by pair from the differences),
// c_ts = sum_r tval[t][r] * colscale[r] * sval[s][r] over the RHS chunk.
// SYM (one point cloud, where every dense pair (t, s) is also one (s, t)):
// c_ts also takes sum_r tval2[t][r] * colscale[r] * sval2[s][r], so that the
// two sides of the adjoint (y_t x_s and x_t y_s) share one evaluation of g.
// The values of a side start at a column offset of its rows (ofs: tval,
// sval, tval2, sval2), so both sides may live in one buffer; sval2 ==
// sval then stages the source rows once.
// One thread per target; sources stream through shared memory like ksum.
template <typename T, int RB, int TS, int STAGES, bool SYM = false>
__global__ void near_grad_kernel(const KGroup* __restrict__ groups,
                                 const uint32_t* __restrict__ ivl,
                                 const Pt4<T>* __restrict__ tgt, const Pt4<T>* __restrict__ src,
                                 const T* __restrict__ tval, const T* __restrict__ sval, int ld,
                                 const double* __restrict__ colscale, int rcount,
                                 KParams<T> kp, double scale, double* __restrict__ G,
                                 int* err, const T* __restrict__ tval2 = nullptr,
                                 const T* __restrict__ sval2 = nullptr, int4 ofs = {0, 0, 0, 0}) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
  int* scnt = reinterpret_cast<int*>(smem_raw + 8 * STAGES);
  Pt4<T>* spts = reinterpret_cast<Pt4<T>*>(smem_raw + 128);
  T* svals = reinterpret_cast<T*>(smem_raw + 128 + STAGES * TS * sizeof(Pt4<T>));
  // SYM with a second source buffer: its tiles after the first one's
  const bool two = SYM && sval2 != sval;
  T* svals2 = two ? svals + (size_t)STAGES * TS * ld : svals;

  const KGroup g = groups[blockIdx.x];
  const int tid = threadIdx.x;
  const bool active = (uint32_t)tid < g.tcount;
  Pt4<T> p{T(0), T(0), T(0), T(0)};
  T yv[RB], xv[SYM ? RB : 1];
#pragma unroll
  for (int r = 0; r < RB; ++r) yv[r] = T(0);
#pragma unroll
  for (int r = 0; r < (SYM ? RB : 1); ++r) xv[r] = T(0);
  if (active) {
    p = tgt[g.tbegin + tid];
    const T* tv = tval + (size_t)(g.tbegin + tid) * ld + ofs.x;
#pragma unroll
    for (int r = 0; r < RB; ++r)
      if (r < rcount) yv[r] = (T)((double)tv[r] * colscale[r]);
    if constexpr (SYM) {
      const T* tv2 = tval2 + (size_t)(g.tbegin + tid) * ld + ofs.z;
#pragma unroll
      for (int r = 0; r < RB; ++r)
        if (r < rcount) xv[r] = (T)((double)tv2[r] * colscale[r]);
    }
  }
  T ax = T(0), ay = T(0), az = T(0);

  int ntiles = 0;
  for (int i = g.ivl_begin; i < g.ivl_end; ++i)
    ntiles += (int)((ivl[2 * i + 1] - ivl[2 * i] + TS - 1) / TS);
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  int pi = g.ivl_begin;
  uint32_t poff = 0;
  int issued = 0;
  auto issue = [&](int stage) {
    const uint32_t b = ivl[2 * pi], e = ivl[2 * pi + 1];
    const uint32_t s0 = b + poff;
    const uint32_t cnt = (e - s0) < (uint32_t)TS ? (e - s0) : (uint32_t)TS;
    scnt[stage] = (int)cnt;
    const uint32_t bp = cnt * (uint32_t)sizeof(Pt4<T>);
    const uint32_t bv = cnt * (uint32_t)ld * (uint32_t)sizeof(T);
    mbar_expect_tx(&bars[stage], bp + (two ? 2u : 1u) * bv);
    bulk_g2s(spts + stage * TS, src + s0, bp, &bars[stage]);
    bulk_g2s(svals + (size_t)stage * TS * ld, sval + (size_t)s0 * ld, bv, &bars[stage]);
    if (two)
      bulk_g2s(svals2 + (size_t)stage * TS * ld, sval2 + (size_t)s0 * ld, bv, &bars[stage]);
    poff += cnt;
    if (b + poff >= e) {
      ++pi;
      poff = 0;
    }
    ++issued;
  };
  if (tid == 0)
    for (int s = 0; s < STAGES && s < ntiles; ++s) issue(s);
  bool aborted = false;
  for (int k = 0; k < ntiles; ++k) {
    const int stage = k % STAGES;
    const bool ok = mbar_wait_bounded(&bars[stage], (uint32_t)((k / STAGES) & 1), kWaitLimitNs);
    if (ok && active) {
      const int cnt = scnt[stage];
      const Pt4<T>* P = spts + stage * TS;
      const T* V = svals + (size_t)stage * TS * ld;
      const T* V2 = svals2 + (size_t)stage * TS * ld;
      for (int j = 0; j < cnt; ++j) {
        const Pt4<T> s = P[j];
        // only the rcount columns from the offset are read: with a column
        // offset, columns past them may lie beyond the row (and the stage)
        const T* v = V + (size_t)j * ld + ofs.y;
        T c = T(0);
#pragma unroll
        for (int r = 0; r < RB; ++r)
          if (r < rcount) c += yv[r] * v[r];
        if constexpr (SYM) {
          const T* v2 = V2 + (size_t)j * ld + ofs.w;
#pragma unroll
          for (int r = 0; r < RB; ++r)
            if (r < rcount) c += xv[r] * v2[r];
        }
        const T dx = p.x - s.x, dy = p.y - s.y, dz = p.z - s.z;
        const T w = c * kgrad<T>(kp.type, dx * dx + dy * dy + dz * dz, kp);
        // accumulate w (p - q) directly: p sum(w) - sum(w q) cancels badly
        ax += w * dx;
        ay += w * dy;
        az += w * dz;
      }
    }
    if (__syncthreads_or(ok ? 0 : 1)) {
      aborted = true;
      break;
    }
    if (tid == 0 && k + STAGES < ntiles) issue(stage);
  }
  if (aborted) {
    if (tid == 0) {
      atomicExch(err, 1);
      for (int k = 0; k < issued; ++k)
        mbar_wait_bounded(&bars[k % STAGES], (uint32_t)((k / STAGES) & 1), kWaitLimitNs / 4);
    }
    return;
  }
  if (active) {
    double* o = G + (size_t)(g.tbegin + tid) * 4;
    o[0] += scale * (double)ax;
    o[1] += scale * (double)ay;
    o[2] += scale * (double)az;
  }
}

// 1-D barycentric Lagrange factors and their derivatives
// l_a'(x) = l_a(x) sum_{b != a} 1 / (x - xi_b)  (the logarithmic derivative
// of prod_{b != a} (x - xi_b); summed without the a term, so nothing cancels
// when x is close to xi_a); at a node xi_m the differentiation-matrix values
// l_a'(xi_m) = (w_a / w_m) / (xi_m - xi_a), l_m'(xi_m) = -sum of those
template <typename T>
__device__ __forceinline__ void lagrange1d_deriv(const InterpDev<T>& ip, T x, T* f, T* df) {
  int m = -1;
  for (int a = 0; a < ip.p1; ++a)
    if (fabs(x - ip.xi[a]) <= T(kDblEps)) m = a;
  if (m < 0) {
    T W = T(0);
    T inv[8];
    for (int b = 0; b < ip.p1; ++b) {
      inv[b] = T(1) / (x - ip.xi[b]);
      W += ip.w[b] * inv[b];
    }
    for (int a = 0; a < ip.p1; ++a) {
      T s = T(0);
      for (int b = 0; b < ip.p1; ++b)
        if (b != a) s += inv[b];
      f[a] = ip.w[a] * inv[a] / W;
      df[a] = f[a] * s;
    }
  } else {
    T s = T(0);
    for (int a = 0; a < ip.p1; ++a) {
      f[a] = a == m ? T(1) : T(0);
      if (a != m) {
        df[a] = (ip.w[a] / ip.w[m]) / (ip.xi[m] - ip.xi[a]);
        s += df[a];
      }
    }
    df[m] = -s;
  }
}

// Far-field gradient: for every point i of a row leaf c,
//   G[i] += scale * sum_k grad V_c[k, i] * sum_r U[c][k][r] tval[i][r] colscale[r]
// blockDim 128; shared: F[128][3][8], D[128][3][8], S[64][RB], midx q*3
template <typename T, int RB>
__global__ void far_grad_kernel(const int32_t* __restrict__ leaves,
                                const uint32_t* __restrict__ cbegin,
                                const uint32_t* __restrict__ csize,
                                const T* __restrict__ bbmin, const T* __restrict__ bbext,
                                const Pt4<T>* __restrict__ pts, const T* __restrict__ U,
                                const T* __restrict__ tval, int ld,
                                const double* __restrict__ colscale, int rcount,
                                const int* __restrict__ midx_g, InterpDev<T> ip,
                                double scale, double* __restrict__ G,
                                const T* __restrict__ U2 = nullptr,
                                const T* __restrict__ tval2 = nullptr,
                                int4 ofs = {0, 0, 0, 0}) {
  // U2 / tval2 given: the second side of the adjoint (its expansions U2 and
  // point values tval2) with the same basis derivatives; ofs: column
  // offsets of U, tval, U2, tval2 in their rows
  constexpr int KC = 64;
  const bool sym = U2 != nullptr;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* F = reinterpret_cast<T*>(smem_raw);  // blockDim x 24
  T* D = F + blockDim.x * 24;             // blockDim x 24
  T* S = D + blockDim.x * 24;             // KC x RB
  T* S2 = S + KC * RB;                    // KC x RB (sym)
  int* midx = reinterpret_cast<int*>(S2 + (sym ? KC * RB : 0));
  const int c = leaves[blockIdx.x];
  const uint32_t b = cbegin[c], n = csize[c];
  const int q = ip.q, tid = threadIdx.x;
  for (int i = tid; i < q * 3; i += blockDim.x) midx[i] = midx_g[i];
  T lo[3], ex[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = d < ip.dim ? bbmin[c * 3 + d] : T(0);
    ex[d] = d < ip.dim ? bbext[c * 3 + d] : T(1);
  }
  T* f = F + tid * 24;
  T* df = D + tid * 24;
  for (uint32_t i0 = 0; i0 < n; i0 += blockDim.x) {
    const bool valid = i0 + tid < n;
    T yv[RB], xv[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) yv[r] = xv[r] = T(0);
    if (valid) {
      const Pt4<T> p = pts[b + i0 + tid];
      const T pc[3] = {p.x, p.y, p.z};
      for (int d = 0; d < 3; ++d) {
        if (d < ip.dim) {
          lagrange1d_deriv(ip, (pc[d] - lo[d]) / ex[d], f + d * 8, df + d * 8);
        } else {
          f[d * 8] = T(1);
          df[d * 8] = T(0);
        }
      }
      const T* tv = tval + (size_t)(b + i0 + tid) * ld + ofs.y;
#pragma unroll
      for (int r = 0; r < RB; ++r)
        if (r < rcount) yv[r] = (T)((double)tv[r] * colscale[r]);
      if (sym) {
        const T* tv2 = tval2 + (size_t)(b + i0 + tid) * ld + ofs.w;
#pragma unroll
        for (int r = 0; r < RB; ++r)
          if (r < rcount) xv[r] = (T)((double)tv2[r] * colscale[r]);
      }
    }
    T gx = T(0), gy = T(0), gz = T(0);
    for (int k0 = 0; k0 < q; k0 += KC) {
      const int cnt = (q - k0) < KC ? (q - k0) : KC;
      __syncthreads();
      for (int e = tid; e < cnt * RB; e += blockDim.x) {
        const int k = e / RB, r = e % RB;
        const size_t row = ((size_t)c * q + k0 + k) * ld;
        S[e] = (r < rcount) ? U[row + ofs.x + r] : T(0);
        if (sym) S2[e] = (r < rcount) ? U2[row + ofs.z + r] : T(0);
      }
      __syncthreads();
      if (valid) {
        for (int k = 0; k < cnt; ++k) {
          T h = T(0);
#pragma unroll
          for (int r = 0; r < RB; ++r) h += S[k * RB + r] * yv[r];
          if (sym) {
#pragma unroll
            for (int r = 0; r < RB; ++r) h += S2[k * RB + r] * xv[r];
          }
          const int kk = k0 + k;
          const int m0 = midx[kk * 3], m1 = midx[kk * 3 + 1], m2 = midx[kk * 3 + 2];
          const T f0 = f[m0], f1 = f[8 + m1], f2 = f[16 + m2];
          gx += h * df[m0] * f1 * f2;
          gy += h * f0 * df[8 + m1] * f2;
          gz += h * f0 * f1 * df[16 + m2];
        }
      }
    }
    if (valid) {
      double* o = G + (size_t)(b + i0 + tid) * 4;
      o[0] += scale * (double)gx / (double)ex[0];
      if (ip.dim > 1) o[1] += scale * (double)gy / (double)ex[1];
      if (ip.dim > 2) o[2] += scale * (double)gz / (double)ex[2];
    }
    __syncthreads();
  }
}

// partial sums of sum_{i, r} a[i, r] * b[i, r] (strided, any dtypes), one
// partial per block, reduced deterministically by dot_final_kernel
template <typename TA, typename TB>
__global__ void dot_partial_kernel(int64_t n, int R, const TA* __restrict__ a, int64_t sai,
                                   int64_t sar, const TB* __restrict__ b, int64_t sbi,
                                   int64_t sbr, double* __restrict__ partial) {
  __shared__ double red[32];
  double s = 0.;
  const int64_t total = n * (int64_t)R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R;
    const int r = (int)(e % R);
    s += (double)a[i * sai + r * sar] * (double)b[i * sbi + r * sbr];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
  }
}

// out[idx] = scale * sum(partial[0..n)), one block of 256 threads
__global__ void dot_final_kernel(const double* __restrict__ partial, int n, double scale,
                                 double* __restrict__ out, int idx) {
  __shared__ double red[256];
  double s = 0.;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[idx] = scale * red[0];
}

// out[idx] = a * in[src]  (small scalar moves on the device)
__global__ void scalar_axpy_kernel(const double* __restrict__ in, int src, double a,
                                   double* __restrict__ out, int idx) {
  if (threadIdx.x == 0 && blockIdx.x == 0) out[idx] = a * in[src];
}

// colscale[r] = 2^(e_x[r] + e_y[r]) from the column maxima of the two
// scaled inputs (1 where a maxima array is absent)
__global__ void colscale_kernel(int R, const unsigned int* __restrict__ cx,
                                const unsigned int* __restrict__ cy,
                                double* __restrict__ out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x) {
    int e = 0;
    if (cx) e += scale_exp(__uint_as_float(cx[r]));
    if (cy) e += scale_exp(__uint_as_float(cy[r]));
    out[r] = ldexp(1.0, e);
  }
}

// dX (natural order, strides) = G (cluster order, 4 doubles per point)
template <typename TO>
__global__ void grad_scatter_kernel(const uint32_t* __restrict__ perm, int64_t n, int dim,
                                    const double* __restrict__ G, TO* __restrict__ dX,
                                    int64_t sdi, int64_t sdd) {
  const int64_t total = n * (int64_t)dim;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / dim;
    const int d = (int)(e % dim);
    dX[(int64_t)perm[i] * sdi + d * sdd] = (TO)G[i * 4 + d];
  }
}

// y (strides) = a * x (contiguous n x R column-major), same dtype
template <typename T>
__global__ void scale_copy_kernel(int64_t n, int R, const T* __restrict__ x, double a,
                                  T* __restrict__ y, int64_t syi, int64_t syr) {
  const int64_t total = n * (int64_t)R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n;
    const int r = (int)(e / n);
    y[i * syi + (int64_t)r * syr] = (T)(a * (double)x[e]);
  }
}

// out (n x 2R, column-major, leading dimension n) = [x | y] from two
// strided n x R inputs
template <typename T>
__global__ void pack_pair_kernel(int64_t n, int R, const T* __restrict__ x, int64_t sxi,
                                 int64_t sxr, const T* __restrict__ y, int64_t syi, int64_t syr,
                                 T* __restrict__ out) {
  const int64_t total = n * (int64_t)R * 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n;
    const int c = (int)(e / n);
    out[e] = c < R ? x[i * sxi + (int64_t)c * sxr] : y[i * syi + (int64_t)(c - R) * syr];
  }
}

}  // namespace gpu
}  // namespace fmca
