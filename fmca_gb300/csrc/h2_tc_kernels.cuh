// Tensor-core kernel sums of the mixed-precision matvec (sm_103a).
//
// ksum_tc computes out[t][0..32) = sum_s a(t, s) * v[s][0..32) for one
// group of targets per CTA, like ksum_kernel, with the contraction on the
// tensor cores:
//   * a(t, s) = k(|tgt_t - src_s|) * 2^(w_s - E) is evaluated in FP32 by the
//     warp that owns the targets, directly in the register layout of the
//     A operand of mma.m16n8k16 (no shared-memory round trip), and split
//     into two FP16 halves a = a_hi + a_lo (a_hi = a with its low 13
//     mantissa bits cleared, a_lo = the exact rest rounded to FP16);
//   * the source values arrive pre-split (v = v_hi + v_lo, FP16) in shared
//     memory through cp.async.bulk copies completed on mbarriers, and are
//     read as B fragments with ldmatrix.trans;
//   * three products a_hi v_hi + a_hi v_lo + a_lo v_hi accumulate in FP32.
//     The tensor cores round the accumulation toward zero, so a long sum
//     drifts toward zero; the MMA accumulators are therefore emptied into
//     separate FP32 registers (round-to-nearest adds) after every tile of
//     kTcTile sources and restart from zero.
// Values are kept inside the FP16 range by exact power-of-two scalings:
// every right-hand side is divided by 2^ceil(log2 max|x_r|) before the
// product (and multiplied back at the end), and the interpolated moments of
// each column cluster by 2^e_sigma. The exponent e_sigma travels in the w
// field of the cluster's interpolation nodes and enters the exponential of
// the kernel, so the weight costs no multiplication; a group subtracts the
// largest exponent E of its sources (a <= 1) and multiplies its sums by 2^E.
//
// Per-pair FP32 work is kept small by three layouts: coordinates are
// multiplied by a kernel-specific g so the kernel argument needs no further
// scaling; each source tile is rewritten in shared memory as records of two
// sources (x0 x1 y0 y1 | z0 z1 w0 w1, coordinates negated) so that packed
// FP32x2 operands load directly; and rows past the end of a tile get w = -inf
// (a = 0) once per tile instead of a select per pair.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "h2_gpu_kernels.cuh"

namespace fmca {
namespace gpu {

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, "
      "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4_trans(uint32_t& r0, uint32_t& r1, uint32_t& r2,
                                              uint32_t& r3, const void* p) {
  asm volatile(
      "ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
      : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
      : "r"(smem_u32(p)));
}

__device__ __forceinline__ uint32_t h2_bits(__half2 h) {
  return *reinterpret_cast<uint32_t*>(&h);
}

constexpr int kTcTile = 128;  // sources per pipeline stage
constexpr int kTcStages = 3;
constexpr int kTcRhs = 32;    // right-hand sides per product (4 n-tiles of 8)
constexpr float kLog2e = 1.44269504088896341f;

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// 2^e for an integral e; 0 below the normal range (e = -inf included)
__device__ __forceinline__ float pow2i(float e) {
  const int i = __float2int_rz(fminf(fmaxf(e, -127.f), 127.f));
  return i <= -127 ? 0.f : __int_as_float((i + 127) << 23);
}

// a = k * 2^w of two squared distances in the coordinates scaled by g;
// FP32x2 arithmetic, the square root and exponential per element on the SFU
template <int KT>
__device__ __forceinline__ float2 kscaled2(float2 r2, float2 w, const KParams<float>& kp) {
  if constexpr (KT == 3) {  // GAUSSIAN: 2^(w - r'^2)
    const float2 u = __ffma2_rn(r2, f2(-1.f, -1.f), w);
    return f2(ex2_approx(u.x), ex2_approx(u.y));
  } else if constexpr (KT == 0 || KT == 1 || KT == 2) {
    const float2 r = f2(sqrt_approx(r2.x), sqrt_approx(r2.y));
    if constexpr (KT == 0) {  // EXPONENTIAL: 2^(w - r')
      const float2 u = __ffma2_rn(r, f2(-1.f, -1.f), w);
      return f2(ex2_approx(u.x), ex2_approx(u.y));
    } else {
      const float2 u = __ffma2_rn(r, f2(-kLog2e, -kLog2e), w);
      const float2 e = f2(ex2_approx(u.x), ex2_approx(u.y));
      if constexpr (KT == 1) return __ffma2_rn(r, e, e);  // MATERN32: (1 + r') e
      // MATERN52: (1 + r' + r'^2 / 3) e
      const float2 p = __ffma2_rn(__ffma2_rn(r, f2(0.333333343f, 0.333333343f), f2(1.f, 1.f)),
                                  r, f2(1.f, 1.f));
      return __fmul2_rn(p, e);
    }
  } else {
    return f2(keval_fast(kp.type, r2.x, kp) * pow2i(w.x),
              keval_fast(kp.type, r2.y, kp) * pow2i(w.y));
  }
}

// Shared memory: [bars | counts] (128 B) | STAGES x TS source points |
// STAGES x TS x 32 FP16 v_hi | STAGES x TS x 32 FP16 v_lo.
// Each point stage arrives as TS records (x, y, z, w) and is rewritten in
// place, warp by warp (a warp's 32 points and their 16 pair records occupy
// the same 512 bytes), as pair records (-g x0, -g x1, -g y0, -g y1, -g z0,
// -g z1, w0 - E, w1 - E).
// REL: the sources are interpolation nodes whose w holds their cluster's
// moment exponent; clusters are q consecutive nodes. Otherwise w = 0.
template <int KT, int MT, bool REL>
__global__ void __launch_bounds__(128, 4)
    ksum_tc_kernel(const KGroup* __restrict__ groups, const uint32_t* __restrict__ ivl,
                   const Pt4<float>* __restrict__ tgt, const Pt4<float>* __restrict__ src,
                   const __half* __restrict__ vhi, const __half* __restrict__ vlo,
                   float* __restrict__ out, int ldo, int rcount, KParams<float> kp, int q,
                   int* err) {
  constexpr int TS = kTcTile, STAGES = kTcStages;
  static_assert(TS == 128, "the in-place pair layout assumes one point per thread");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
  int* scnt = reinterpret_cast<int*>(smem_raw + 8 * STAGES);
  float* sred = reinterpret_cast<float*>(smem_raw + 64);
  Pt4<float>* spts = reinterpret_cast<Pt4<float>*>(smem_raw + 128);
  __half* shi = reinterpret_cast<__half*>(smem_raw + 128 + STAGES * TS * 16);
  __half* slo = shi + STAGES * TS * kTcRhs;

  const KGroup g = groups[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  const float gs = kp.g;

  // zero the source buffers once, so rows past a partial tile always hold
  // finite data; the proxy fence orders these generic writes before the
  // bulk copies
  {
    uint4* z = reinterpret_cast<uint4*>(spts);
    const int n16 = STAGES * TS * (16 + kTcRhs * 2 * 2) / 16;
    for (int i = tid; i < n16; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }

  // targets of this thread: rows gid and gid + 8 of each of the warp's
  // m-tiles, scaled by g and duplicated into both halves of a packed pair
  float2 tx[MT][2], ty[MT][2], tz[MT][2];
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t i = (uint32_t)(warp * MT * 16 + m * 16 + gid + 8 * h);
      float px = 0.f, py = 0.f, pz = 0.f;
      if (i < g.tcount) {
        const Pt4<float> p = tgt[g.tbegin + i];
        px = gs * p.x;
        py = gs * p.y;
        pz = gs * p.z;
      }
      tx[m][h] = f2(px, px);
      ty[m][h] = f2(py, py);
      tz[m][h] = f2(pz, pz);
    }
  float acc[MT][4][4], tot[MT][4][4];
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[m][n][c] = tot[m][n][c] = 0.f;

  int ntiles = 0;
  for (int i = g.ivl_begin; i < g.ivl_end; ++i)
    ntiles += (int)((ivl[2 * i + 1] - ivl[2 * i] + TS - 1) / TS);

  // largest moment exponent E of the group's source clusters
  float E = 0.f;
  if constexpr (REL) {
    float m = -CUDART_INF_F;
    for (int i = g.ivl_begin + tid; i < g.ivl_end; i += blockDim.x)
      for (uint32_t s = ivl[2 * i], e = ivl[2 * i + 1]; s < e; s = (s / q + 1) * q)
        m = fmaxf(m, src[s].w);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) sred[warp] = m;
  }

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if constexpr (REL) {
    E = fmaxf(fmaxf(sred[0], sred[1]), fmaxf(sred[2], sred[3]));
    E = fmaxf(E, -1000.f);  // groups without sources
  }

  int pi = g.ivl_begin;
  uint32_t poff = 0;
  int issued = 0;
  auto issue = [&](int stage) {
    const uint32_t b = ivl[2 * pi], e = ivl[2 * pi + 1];
    const uint32_t s0 = b + poff;
    const uint32_t cnt = (e - s0) < (uint32_t)TS ? (e - s0) : (uint32_t)TS;
    scnt[stage] = (int)cnt;
    const uint32_t bp = cnt * 16u, bv = cnt * (uint32_t)kTcRhs * 2u;
    mbar_expect_tx(&bars[stage], bp + 2 * bv);
    bulk_g2s(spts + stage * TS, src + s0, bp, &bars[stage]);
    bulk_g2s(shi + (size_t)stage * TS * kTcRhs, vhi + (size_t)s0 * kTcRhs, bv, &bars[stage]);
    bulk_g2s(slo + (size_t)stage * TS * kTcRhs, vlo + (size_t)s0 * kTcRhs, bv, &bars[stage]);
    poff += cnt;
    if (b + poff >= e) {
      ++pi;
      poff = 0;
    }
    ++issued;
  };
  if (tid == 0)
    for (int s = 0; s < STAGES && s < ntiles; ++s) issue(s);

  // ldmatrix row / column of this lane inside a 16 x 16 block
  const int lrow = (lane & 7) + ((lane >> 3) & 1) * 8;
  const int lcol = (lane >> 4) * 8;

  bool aborted = false;
  for (int k = 0; k < ntiles; ++k) {
    const int stage = k % STAGES;
    const uint32_t parity = (uint32_t)((k / STAGES) & 1);
    const bool ok = mbar_wait_bounded(&bars[stage], parity, kWaitLimitNs);
    const int cnt = scnt[stage];
    if (ok) {
      // rewrite this warp's 32 points as 16 pair records, in place
      float4* P4 = reinterpret_cast<float4*>(spts + stage * TS);
      const float4 p = P4[tid];
      __syncwarp();
      float* rec = reinterpret_cast<float*>(P4) + (tid >> 1) * 8 + (tid & 1);
      // rows past the tile's end hold stale records: zero coordinates keep
      // their (zero) kernel values finite
      const bool valid = tid < cnt;
      rec[0] = valid ? -gs * p.x : 0.f;
      rec[2] = valid ? -gs * p.y : 0.f;
      rec[4] = valid ? -gs * p.z : 0.f;
      rec[6] = valid ? (REL ? p.w - E : 0.f) : -CUDART_INF_F;
      // these generic writes precede the next bulk copy into the stage
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (__syncthreads_or(ok ? 0 : 1)) {
      aborted = true;
      break;
    }
    {
      const float4* R4 = reinterpret_cast<const float4*>(spts + stage * TS);
      const __half* H = shi + (size_t)stage * TS * kTcRhs;
      const __half* L = slo + (size_t)stage * TS * kTcRhs;
      for (int ks = 0; ks < cnt; ks += 16) {
        // B fragments of the 4 n-tiles, hi and lo
        uint32_t bh[4][2], bl[4][2];
        const __half* hrow = H + (size_t)(ks + lrow) * kTcRhs + lcol;
        const __half* lrowp = L + (size_t)(ks + lrow) * kTcRhs + lcol;
        ldsm_x4_trans(bh[0][0], bh[0][1], bh[1][0], bh[1][1], hrow);
        ldsm_x4_trans(bh[2][0], bh[2][1], bh[3][0], bh[3][1], hrow + 16);
        ldsm_x4_trans(bl[0][0], bl[0][1], bl[1][0], bl[1][1], lrowp);
        ldsm_x4_trans(bl[2][0], bl[2][1], bl[3][0], bl[3][1], lrowp + 16);
        // this thread's source columns as two pair records:
        // pair 0 = (2 tig, 2 tig + 1), pair 1 = (2 tig + 8, 2 tig + 9)
        float2 nsx[2], nsy[2], nsz[2], wv[2];
#pragma unroll
        for (int pp = 0; pp < 2; ++pp) {
          const int jp = (ks >> 1) + tig + 4 * pp;
          const float4 a = R4[2 * jp], b = R4[2 * jp + 1];
          nsx[pp] = f2(a.x, a.y);
          nsy[pp] = f2(a.z, a.w);
          nsz[pp] = f2(b.x, b.y);
          wv[pp] = f2(b.z, b.w);
        }
#pragma unroll
        for (int m = 0; m < MT; ++m) {
          uint32_t ahi[4], alo[4];
#pragma unroll
          for (int pp = 0; pp < 2; ++pp)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const float2 dx = __fadd2_rn(tx[m][h], nsx[pp]);
              const float2 dy = __fadd2_rn(ty[m][h], nsy[pp]);
              const float2 dz = __fadd2_rn(tz[m][h], nsz[pp]);
              const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
              const float2 av = kscaled2<KT>(r2, wv[pp], kp);
              // register 2 pp + h of the A fragment: row gid + 8 h, pair pp;
              // hi keeps the top 11 significant bits (exact in FP16 for
              // |a| >= 2^-14), lo = a - hi exactly in FP32
              const float2 hi = f2(__uint_as_float(__float_as_uint(av.x) & 0xffffe000u),
                                   __uint_as_float(__float_as_uint(av.y) & 0xffffe000u));
              const float2 lo = __ffma2_rn(hi, f2(-1.f, -1.f), av);
              ahi[2 * pp + h] = h2_bits(__floats2half2_rn(hi.x, hi.y));
              alo[2 * pp + h] = h2_bits(__floats2half2_rn(lo.x, lo.y));
            }
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            mma16816(acc[m][n], ahi, bh[n][0], bh[n][1]);
            mma16816(acc[m][n], ahi, bl[n][0], bl[n][1]);
            mma16816(acc[m][n], alo, bh[n][0], bh[n][1]);
          }
        }
      }
      // empty the tensor-core accumulators into the FP32 totals
#pragma unroll
      for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int n = 0; n < 4; ++n)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            tot[m][n][c] += acc[m][n][c];
            acc[m][n][c] = 0.f;
          }
    }
    __syncthreads();
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
  const int eo = (int)E;
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t i = (uint32_t)(warp * MT * 16 + m * 16 + gid + 8 * h);
      if (i >= g.tcount) continue;
      float* o = out + (size_t)(g.tbegin + i) * ldo;
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const int c = n * 8 + 2 * tig;
        const float v0 = REL ? ldexpf(tot[m][n][2 * h], eo) : tot[m][n][2 * h];
        const float v1 = REL ? ldexpf(tot[m][n][2 * h + 1], eo) : tot[m][n][2 * h + 1];
        if (c < rcount) o[c] = v0;
        if (c + 1 < rcount) o[c + 1] = v1;
      }
    }
}

// per-column max |x| as float bits (positive floats order like integers).
// Columns [c0, c0 + nc) of this launch; a block reduces into shared memory
// first (per-thread running maxima when the grid stride is a multiple of
// nc, so every thread stays on one column) and flushes once per column.
template <typename TI>
__global__ void colmax_kernel(int64_t n, int c0, int nc, const TI* __restrict__ x,
                              int64_t sxi, int64_t sxr, unsigned int* __restrict__ cmax) {
  extern __shared__ unsigned int smax[];
  for (int r = threadIdx.x; r < nc; r += blockDim.x) smax[r] = 0u;
  __syncthreads();
  const int64_t total = n * (int64_t)nc;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t first = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (stride % nc == 0) {
    unsigned int m = 0u;
    const int r = (int)(first % nc);
    for (int64_t e = first; e < total; e += stride) {
      const int64_t i = e / nc;
      m = max(m, __float_as_uint(fabsf((float)x[i * sxi + (int64_t)(c0 + r) * sxr])));
    }
    if (first < total) atomicMax(&smax[r], m);
  } else {
    for (int64_t e = first; e < total; e += stride) {
      const int64_t i = e / nc;
      const int r = (int)(e % nc);
      atomicMax(&smax[r], __float_as_uint(fabsf((float)x[i * sxi + (int64_t)(c0 + r) * sxr])));
    }
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

// gather for the mixed path: x' = x * 2^-e_r (cluster order, chunk-major
// [chunk][n][32]) in FP32 and split into FP16 hi / lo parts
template <typename TI>
__global__ void gather_split_kernel(const uint32_t* __restrict__ perm, int64_t n, int R,
                                   const TI* __restrict__ x, int64_t sxi, int64_t sxr,
                                   const unsigned int* __restrict__ cmax,
                                   float* __restrict__ xc, __half* __restrict__ xh,
                                   __half* __restrict__ xl) {
  const int nchunks = (R + kTcRhs - 1) / kTcRhs;
  const int64_t per = n * (int64_t)kTcRhs;
  const int64_t total = per * nchunks;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ch = e / per, rem = e % per;
    const int64_t i = rem / kTcRhs;
    const int r = (int)ch * kTcRhs + (int)(rem % kTcRhs);
    float v = 0.f;
    if (r < R) {
      const int64_t src = perm ? (int64_t)perm[i] : i;
      const int ex = scale_exp(__uint_as_float(cmax[r]));
      v = ldexpf((float)x[src * sxi + (int64_t)r * sxr], -ex);
    }
    xc[e] = v;
    const __half h = __float2half_rn(v);
    xh[e] = h;
    xl[e] = __float2half_rn(v - __half2float(h));
  }
}

// per column cluster: e = exponent of max |t|, t'' = t * 2^-e split into
// FP16 hi / lo, and the cluster's node coordinates with w = e (the moment
// exponent; -1000 for a cluster without moments)
__global__ void tscale_kernel(int C, int q, int rcount, const float* __restrict__ t,
                              const Pt4<float>* __restrict__ nodes,
                              __half* __restrict__ th, __half* __restrict__ tl,
                              Pt4<float>* __restrict__ nodes_s) {
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
    const float v = (e % kTcRhs) < rcount ? ldexpf(t[base + e], -ex) : 0.f;
    const __half h = __float2half_rn(v);
    th[base + e] = h;
    tl[base + e] = __float2half_rn(v - __half2float(h));
  }
  for (int k = threadIdx.x; k < q; k += blockDim.x) {
    Pt4<float> p = nodes[(size_t)c * q + k];
    p.w = w;
    nodes_s[(size_t)c * q + k] = p;
  }
}

// y (natural order) = sigma2 * 2^e_r * (ynear + yfar), combined in FP64
template <typename TO>
__global__ void scatter_scaled_kernel(const uint32_t* __restrict__ perm, int64_t n, int R,
                                      const float* __restrict__ ynear,
                                      const float* __restrict__ yfar,
                                      const unsigned int* __restrict__ cmax, double sigma2,
                                      TO* __restrict__ y, int64_t syi, int64_t syr) {
  const int64_t total = n * (int64_t)R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R;
    const int r = (int)(e % R);
    const int64_t k = ((int64_t)(r / kTcRhs) * n + i) * kTcRhs + r % kTcRhs;
    const int64_t dst = perm ? (int64_t)perm[i] : i;
    const double v = (double)ynear[k] + (double)yfar[k];
    const int ex = scale_exp(__uint_as_float(cmax[r]));
    y[dst * syi + (int64_t)r * syr] = (TO)(ldexp(sigma2 * v, ex));
  }
}

}  // namespace gpu
}  // namespace fmca
