// Device code of the H2 matvec (sm_103a).
//
// Stages of one product y = K_H2 x (FMCA/src/H2Matrix/H2MatrixBase.h:113-152):
//   gather      x (natural order, any strides) -> xc (cluster order, ld = ldv)
//   leafmom     t_tau = V_tau xc_tau for column leaves, V generated from the
//               points on the fly (forward_transform_impl.h:31-33,
//               NystromMoments.h:24-34)
//   m2m         t_dad = sum_sons E_son t_son, one launch per level, bottom-up
//               (forward_transform_impl.h:24-30)
//   ksum far    s_tau = sum_sigma K(xi_tau, xi_sigma) t_sigma over the
//               admissible list of every row cluster (NystromEvaluator.h:
//               40-56 + H2MatrixBase.h:140-142); with total-degree
//               interpolation between two changes of basis (t to the nodal
//               basis by invV^T, s back by invV)
//   l2l         s_son += E_son^T s_dad, one launch per level, top-down
//               (backward_transform_impl.h:21-28)
//   leafgather  yfar_tau = V_tau^T s_tau for row leaves, compensated in FP32
//               (backward_transform_impl.h:29-31)
//   ksum near   ynear_tau = sum K(X_tau, X_sigma) xc_sigma over the dense
//               list of every row leaf (NystromEvaluator.h:61-71 +
//               H2MatrixBase.h:143-146)
//   scatter     y = sigma2 * (ynear + yfar), combined in FP64, natural order
//
// ksum is the hot kernel: one CTA owns a group of targets (points of a row
// leaf, or interpolation nodes of a row cluster) and streams the group's
// source intervals through shared memory with cp.async.bulk copies completed
// on mbarriers (3-stage ring).  Each thread keeps TPT targets x RB
// right-hand sides in registers; every source costs one broadcast load of
// its coordinates and RB/4 broadcast vector loads of its values.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "compensated_sum.h"

namespace fmca {
namespace gpu {

constexpr double kDblEps = 2.220446049250313080847263336181640625e-16;
constexpr int kLeafChunk = 128;      // points per shared-memory chunk of leafmom_kernel
constexpr int kTransferChunk = 128;  // source coefficients per chunk of transfer_kernel

template <typename T>
struct alignas(4 * sizeof(T)) Pt4 {
  T x, y, z, w;
};

// target group of ksum: targets [tbegin, tbegin + tcount) of the target
// array, sources = union of intervals ivl[2*ivl_begin .. 2*ivl_end)
struct KGroup {
  uint32_t tbegin, tcount;
  int32_t ivl_begin, ivl_end;
};

template <typename T>
struct KParams {
  int type;
  T l, c;
  T a;   // sqrt(3)/l, sqrt(5)/l, ... (per type)
  T e2;  // scale of the exponent in base 2 (FP32 path)
  T il;  // 1 / l
  T g;   // coordinate scale of the tensor-core path (1 for generic kernels)
  // centre subtracted from every coordinate before the scaling by g in the
  // near field's dot-product distance form (um_near_dot)
  T cx = 0, cy = 0, cz = 0;
  unsigned long long wait_ns;  // limit of the kernel sums' bounded waits
  // test hook (fmca_plan_set_stalled_wait): the first wait of every
  // kernel-sum CTA is on a barrier that nothing completes, so it runs out
  int stall;
};

// kind 0: Chebyshev tensor product (Lagrange factors from xi, w); kind 1:
// total degree (L2-normalised Legendre factors)
template <typename T>
struct InterpDev {
  int kind, dim, p1, q;
  T xi[8], w[8];
};

// ---------------------------------------------------------------------------
// PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kLn2f = 0.693147180559945309f;
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], "
      "%2;\n selp.u32 %0, 1, 0, p;\n}" : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for a phase of an mbarrier for at most limit_ns; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_timer_ns() - t0 > limit_ns) return false;
  }
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per wait

// ---------------------------------------------------------------------------
// radial kernels, evaluated from the squared distance.
// KT >= 0: compile-time kernel type; KT < 0: runtime switch on kp.type.
// FP64: operation order of FMCA/src/CovarianceKernel/CovarianceKernel.h.
__device__ __forceinline__ double keval_ref(int type, double r2,
                                           const KParams<double>& kp) {
  const double r = sqrt(r2);
  const double l = kp.l;
  switch (type) {
    case 0:
      return exp(-r / l);
    case 1:
      return (1. + kp.a * r) * exp(-1.7320508075688772 * r / l);
    case 2:
      return (1. + kp.a * r + 5 * r * r / (3 * l * l)) *
             exp(-2.23606797749979 * r / l);
    case 3:
      return exp(-0.5 * r * r / (l * l));
    case 4: {
      const double t = r / l;
      return (1. + kp.a * r + 14. / 5 * (t * t) +
              7. * 2.6457513110645907 / 15. * (t * t * t)) *
             exp(-2.6457513110645907 * r / l);
    }
    case 5: {
      const double t = r / l;
      return (1. + 3. / l * r + 27. / 7. * (t * t) + 18. / 7. * (t * t * t) +
              27. / 35. * (t * t * t * t)) *
             exp(-3 * r / l);
    }
    case 6:
      return 1. / sqrt((r / l) * (r / l) + kp.c * kp.c);
    case 7:
      return sqrt((r / l) * (r / l) + kp.c * kp.c);
    case 8:
      return r / l;
    case 9:
      return (r / l) * (r / l) * (r / l);
    // length-scale derivatives, returned as l * dk/dl (dimensionless; the
    // driver divides the result by l)
    case 10: {
      const double t = r / l;
      return t * exp(-t);
    }
    case 11: {
      const double u = kp.a * r;
      return u * u * exp(-u);
    }
    case 12: {
      const double u = kp.a * r;
      return u * u / 3. * (1. + u) * exp(-u);
    }
    case 13: {
      const double t2 = r2 / (l * l);
      return t2 * exp(-0.5 * t2);
    }
    case 14:  // BIHARMONIC2D, 0 below r = DBL_EPSILON
      return r < 2.220446049250313e-16 ? 0. : log(r / l) * (r / l) * (r / l);
    case 15:  // TPS2D
      return r > 0. ? r * r * log(r) : 0.;
  }
  return 0.;
}

// FP32: approximate sqrt / exp2 on the SFU, FP32 FMA elsewhere.
__device__ __forceinline__ float keval_fast(int type, float r2,
                                            const KParams<float>& kp) {
  switch (type) {
    case 0: {  // exp(-r/l)
      const float r = sqrt_approx(r2);
      return ex2_approx(r * kp.e2);
    }
    case 1: {  // (1 + a r) exp(-a r)
      const float r = sqrt_approx(r2);
      const float e = ex2_approx(r * kp.e2);
      return fmaf(kp.a * r, e, e);
    }
    case 2: {  // (1 + a r + (a r)^2 / 3) exp(-a r)
      const float r = sqrt_approx(r2);
      const float t = kp.a * r;
      const float e = ex2_approx(r * kp.e2);
      return fmaf(fmaf(t, 0.333333343f, 1.f), t, 1.f) * e;
    }
    case 3:  // exp(-r^2 / (2 l^2))
      return ex2_approx(r2 * kp.e2);
    case 4: {
      const float r = sqrt_approx(r2);
      const float t = r / kp.l;
      const float e = ex2_approx(r * kp.e2);
      const float p = fmaf(fmaf(fmaf(t, 1.2346839451789856f, 2.8f), t,
                                2.6457513110645907f),
                           t, 1.f);
      return p * e;
    }
    case 5: {
      const float r = sqrt_approx(r2);
      const float t = r / kp.l;
      const float e = ex2_approx(r * kp.e2);
      const float p =
          fmaf(fmaf(fmaf(fmaf(t, 0.77142857f, 2.5714285f), t, 3.857142857f), t,
                    3.f),
               t, 1.f);
      return p * e;
    }
    case 6: {
      const float t2 = r2 / (kp.l * kp.l);
      return rsqrt_approx(t2 + kp.c * kp.c);
    }
    case 7: {
      const float t2 = r2 / (kp.l * kp.l);
      return sqrt_approx(t2 + kp.c * kp.c);
    }
    case 8:
      return sqrt_approx(r2) / kp.l;
    case 9: {
      const float t = sqrt_approx(r2) / kp.l;
      return t * t * t;
    }
    // l * dk/dl of kernels 0..3 (bounded by 1)
    case 10: {
      const float r = sqrt_approx(r2);
      return r * kp.il * ex2_approx(r * kp.e2);
    }
    case 11: {
      const float r = sqrt_approx(r2);
      const float u = kp.a * r;
      return u * u * ex2_approx(r * kp.e2);
    }
    case 12: {
      const float r = sqrt_approx(r2);
      const float u = kp.a * r;
      return u * u * 0.333333343f * (1.f + u) * ex2_approx(r * kp.e2);
    }
    case 13:
      return r2 * kp.il * kp.il * ex2_approx(r2 * kp.e2);
    // thin-plate kernels from r^2: t^2 log t = (ln 2 / 2) t^2 log2(t^2)
    case 14: {
      const float t2 = r2 * (kp.il * kp.il);
      return t2 > 0.f ? (0.5f * kLn2f) * t2 * lg2_approx(t2) : 0.f;
    }
    case 15:
      return r2 > 0.f ? (0.5f * kLn2f) * r2 * lg2_approx(r2) : 0.f;
  }
  return 0.f;
}

template <typename T, int KT>
__device__ __forceinline__ T keval(T r2, const KParams<T>& kp);
template <>
__device__ __forceinline__ double keval<double, -1>(double r2,
                                                    const KParams<double>& kp) {
  return keval_ref(kp.type, r2, kp);
}
template <>
__device__ __forceinline__ double keval<double, 0>(double r2,
                                                   const KParams<double>& kp) {
  return keval_ref(0, r2, kp);
}
template <>
__device__ __forceinline__ double keval<double, 1>(double r2,
                                                   const KParams<double>& kp) {
  return keval_ref(1, r2, kp);
}
template <>
__device__ __forceinline__ double keval<double, 2>(double r2,
                                                   const KParams<double>& kp) {
  return keval_ref(2, r2, kp);
}
template <>
__device__ __forceinline__ double keval<double, 3>(double r2,
                                                   const KParams<double>& kp) {
  return keval_ref(3, r2, kp);
}
template <>
__device__ __forceinline__ float keval<float, -1>(float r2,
                                                  const KParams<float>& kp) {
  return keval_fast(kp.type, r2, kp);
}
template <>
__device__ __forceinline__ float keval<float, 0>(float r2,
                                                 const KParams<float>& kp) {
  return keval_fast(0, r2, kp);
}
template <>
__device__ __forceinline__ float keval<float, 1>(float r2,
                                                 const KParams<float>& kp) {
  return keval_fast(1, r2, kp);
}
template <>
__device__ __forceinline__ float keval<float, 2>(float r2,
                                                 const KParams<float>& kp) {
  return keval_fast(2, r2, kp);
}
template <>
__device__ __forceinline__ float keval<float, 3>(float r2,
                                                 const KParams<float>& kp) {
  return keval_fast(3, r2, kp);
}

// ---------------------------------------------------------------------------
// ksum: out[t][rofs + r] (+)= sum_s k(|tgt_t - src_s|) * sval[s][rofs + r]
// Shared memory: [bars | counts] (128 B), then STAGES tiles of TS source
// coordinates, then STAGES tiles of TS x ldv source values.
template <typename T, int KT, int TPT, int RB, int TS, int STAGES>
__global__ void ksum_kernel(const KGroup* __restrict__ groups,
                            const uint32_t* __restrict__ ivl,
                            const Pt4<T>* __restrict__ tgt,
                            const Pt4<T>* __restrict__ src,
                            const T* __restrict__ sval, int ldv,
                            T* __restrict__ out, int rofs, int rcount,
                            KParams<T> kp, int accumulate, int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
  int* scnt = reinterpret_cast<int*>(smem_raw + 8 * STAGES);
  Pt4<T>* spts = reinterpret_cast<Pt4<T>*>(smem_raw + 128);
  T* svals = reinterpret_cast<T*>(smem_raw + 128 + STAGES * TS * sizeof(Pt4<T>));

  const KGroup g = groups[blockIdx.x];
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;

  T tx[TPT], ty[TPT], tz[TPT];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const uint32_t i = tid + t * nthr;
    if (i < g.tcount) {
      const Pt4<T> p = tgt[g.tbegin + i];
      tx[t] = p.x;
      ty[t] = p.y;
      tz[t] = p.z;
    } else {
      tx[t] = ty[t] = tz[t] = T(0);
    }
  }
  T acc[TPT][RB];
#pragma unroll
  for (int t = 0; t < TPT; ++t)
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[t][r] = T(0);

  int ntiles = 0;
  for (int i = g.ivl_begin; i < g.ivl_end; ++i)
    ntiles += (int)((ivl[2 * i + 1] - ivl[2 * i] + TS - 1) / TS);

  // a barrier nothing arrives on (the stalled-wait test hook waits on it)
  uint64_t* never = reinterpret_cast<uint64_t*>(smem_raw + 64);
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
    mbar_init(never, 1);
    fence_mbar_init();
  }
  __syncthreads();

  // producer cursor (thread 0 only)
  int pi = g.ivl_begin;
  uint32_t poff = 0;
  int issued = 0;
  auto issue = [&](int stage) {
    const uint32_t b = ivl[2 * pi], e = ivl[2 * pi + 1];
    const uint32_t s0 = b + poff;
    const uint32_t cnt = (e - s0) < (uint32_t)TS ? (e - s0) : (uint32_t)TS;
    scnt[stage] = (int)cnt;
    const uint32_t bp = cnt * (uint32_t)sizeof(Pt4<T>);
    const uint32_t bv = cnt * (uint32_t)ldv * (uint32_t)sizeof(T);
    mbar_expect_tx(&bars[stage], bp + bv);
    bulk_g2s(spts + stage * TS, src + s0, bp, &bars[stage]);
    bulk_g2s(svals + (size_t)stage * TS * ldv, sval + (size_t)s0 * ldv, bv,
             &bars[stage]);
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
    const uint32_t parity = (uint32_t)((k / STAGES) & 1);
    const bool ok =
        mbar_wait_bounded((kp.stall && k == 0) ? never : &bars[stage], parity, kp.wait_ns);
    if (ok) {
      const int cnt = scnt[stage];
      const Pt4<T>* P = spts + stage * TS;
      const T* V = svals + (size_t)stage * TS * ldv + rofs;
      int j = 0;
      if constexpr (sizeof(T) == 4 && RB % 4 == 0) {
        // FP32: two sources per step in packed FP32x2 arithmetic (the
        // squared distances of both, and every accumulator pair of
        // columns (r, r + 1) updated by one FFMA2 per source); the same
        // operations per element as the scalar loop below
        for (; j + 1 < cnt; j += 2) {
          const Pt4<T> s0 = P[j], s1 = P[j + 1];
          const float2 sx = make_float2(s0.x, s1.x), sy = make_float2(s0.y, s1.y),
                       sz = make_float2(s0.z, s1.z);
          float2 ka[TPT], kb[TPT];
#pragma unroll
          for (int t = 0; t < TPT; ++t) {
            const float2 m1 = make_float2(-1.f, -1.f);
            const float2 dx = __ffma2_rn(sx, m1, make_float2(tx[t], tx[t]));
            const float2 dy = __ffma2_rn(sy, m1, make_float2(ty[t], ty[t]));
            const float2 dz = __ffma2_rn(sz, m1, make_float2(tz[t], tz[t]));
            const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
            const T k0 = keval<T, KT>(r2.x, kp), k1 = keval<T, KT>(r2.y, kp);
            ka[t] = make_float2(k0, k0);
            kb[t] = make_float2(k1, k1);
          }
          const T* v0 = V + (size_t)j * ldv;
          const T* v1 = v0 + ldv;
#pragma unroll
          for (int r = 0; r < RB; r += 4) {
            const float4 a = *reinterpret_cast<const float4*>(v0 + r);
            const float4 b = *reinterpret_cast<const float4*>(v1 + r);
            const float2 a01 = make_float2(a.x, a.y), a23 = make_float2(a.z, a.w);
            const float2 b01 = make_float2(b.x, b.y), b23 = make_float2(b.z, b.w);
#pragma unroll
            for (int t = 0; t < TPT; ++t) {
              float2 p01 = make_float2(acc[t][r + 0], acc[t][r + 1]);
              float2 p23 = make_float2(acc[t][r + 2], acc[t][r + 3]);
              p01 = __ffma2_rn(ka[t], a01, p01);
              p23 = __ffma2_rn(ka[t], a23, p23);
              p01 = __ffma2_rn(kb[t], b01, p01);
              p23 = __ffma2_rn(kb[t], b23, p23);
              acc[t][r + 0] = p01.x;
              acc[t][r + 1] = p01.y;
              acc[t][r + 2] = p23.x;
              acc[t][r + 3] = p23.y;
            }
          }
        }
      }
#pragma unroll 2
      for (; j < cnt; ++j) {
        const Pt4<T> s = P[j];
        T kv[TPT];
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
          const T dx = tx[t] - s.x, dy = ty[t] - s.y, dz = tz[t] - s.z;
          kv[t] = keval<T, KT>(dx * dx + dy * dy + dz * dz, kp);
        }
        const T* v = V + (size_t)j * ldv;
        if constexpr (RB % 4 == 0 && sizeof(T) == 4) {
#pragma unroll
          for (int r = 0; r < RB; r += 4) {
            const float4 vv = *reinterpret_cast<const float4*>(v + r);
#pragma unroll
            for (int t = 0; t < TPT; ++t) {
              acc[t][r + 0] = fmaf(kv[t], vv.x, acc[t][r + 0]);
              acc[t][r + 1] = fmaf(kv[t], vv.y, acc[t][r + 1]);
              acc[t][r + 2] = fmaf(kv[t], vv.z, acc[t][r + 2]);
              acc[t][r + 3] = fmaf(kv[t], vv.w, acc[t][r + 3]);
            }
          }
        } else if constexpr (RB % 2 == 0 && sizeof(T) == 8) {
#pragma unroll
          for (int r = 0; r < RB; r += 2) {
            const double2 vv = *reinterpret_cast<const double2*>(v + r);
#pragma unroll
            for (int t = 0; t < TPT; ++t) {
              acc[t][r + 0] = fma(kv[t], vv.x, acc[t][r + 0]);
              acc[t][r + 1] = fma(kv[t], vv.y, acc[t][r + 1]);
            }
          }
        } else {
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            const T vv = v[r];
#pragma unroll
            for (int t = 0; t < TPT; ++t) acc[t][r] += kv[t] * vv;
          }
        }
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
      // drain the copies this CTA still has in flight, again bounded
      const int consumed_max = issued;
      for (int k = 0; k < consumed_max; ++k)
        mbar_wait_bounded(&bars[k % STAGES], (uint32_t)((k / STAGES) & 1),
                          kWaitLimitNs / 4);
    }
    return;
  }
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const uint32_t i = tid + t * nthr;
    if (i < g.tcount) {
      T* o = out + (size_t)(g.tbegin + i) * ldv + rofs;
#pragma unroll
      for (int r = 0; r < RB; ++r)
        if (r < rcount) o[r] = accumulate ? o[r] + acc[t][r] : acc[t][r];
    }
  }
}

// ---------------------------------------------------------------------------
// 1-D barycentric Lagrange factors, same guard and operation order as the
// host (TensorProductInterpolator.h:65-81); factor a is stored at f[a * stride]
template <typename T>
__device__ __forceinline__ void lagrange1d(const InterpDev<T>& ip, T x, T* f,
                                           int stride = 1) {
  T weight = T(0);
  for (int k = 0; k < ip.p1; ++k) weight += ip.w[k] / (x - ip.xi[k]);
  for (int a = 0; a < ip.p1; ++a) {
    const T dxa = x - ip.xi[a];
    f[a * stride] = (fabs(dxa) > T(kDblEps)) ? ip.w[a] / dxa / weight : T(1);
  }
}

// the p1 one-dimensional factors of the interpolator's basis at x in [0, 1]:
// Lagrange factors, or Legendre polynomials scaled to unit L2 norm
// (evalPolynomials.h:19-38: the three-term recurrence on the unscaled
// polynomials, each scaled by sqrt(2 i + 1))
template <typename T>
__device__ __forceinline__ void basis1d(const InterpDev<T>& ip, T x, T* f, int stride = 1) {
  if (ip.kind == 0) {
    lagrange1d(ip, x, f, stride);
    return;
  }
  T p0 = T(0), p1 = T(1);
  f[0] = T(1);
  for (int i = 1; i < ip.p1; ++i) {
    const T v = T(2 * i - 1) / T(i) * (T(2) * x - T(1)) * p1 - T(i - 1) / T(i) * p0;
    p0 = p1;
    p1 = v;
    f[i * stride] = v * sqrt(T(2 * i + 1));
  }
}

// multi-index k -> (k0, k1, k2) packed as k0 | k1 << 8 | k2 << 16 (digits < 256)
__device__ __forceinline__ void pack_digits(const int* __restrict__ midx_g, int q,
                                            int* __restrict__ pk) {
  for (int i = threadIdx.x; i < q; i += blockDim.x)
    pk[i] = midx_g[i * 3] | (midx_g[i * 3 + 1] << 8) | (midx_g[i * 3 + 2] << 16);
}

// Copies rows [0, cnt) of a block with leading dimension ldv, columns
// rofs .. rofs + rcount - 1, into a dense cnt x RB tile in shared memory and
// zero-fills columns rcount .. RB - 1.  Each thread issues U loads before it
// stores any of them, so that their latencies overlap; full rows at 16-byte
// aligned addresses move as 16-byte vectors.
template <typename T, int RB>
__device__ __forceinline__ void stage_rows(T* __restrict__ dst, const T* src, int cnt,
                                           int ldv, int rofs, int rcount) {
  constexpr int U = 8;
  constexpr int VW = 16 / (int)sizeof(T);
  const int nthr = blockDim.x, tid = threadIdx.x;
  if constexpr (RB % VW == 0) {
    if (rcount == RB && (ldv % VW) == 0 && (rofs % VW) == 0 &&
        (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
      constexpr int VPR = RB / VW;
      const int total = cnt * VPR, ld4 = ldv / VW;
      const uint4* s4 = reinterpret_cast<const uint4*>(src + rofs);
      uint4* d4 = reinterpret_cast<uint4*>(dst);
      for (int i0 = tid; i0 < total; i0 += U * nthr) {
        uint4 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = i0 + u * nthr;
          v[u] = i < total ? s4[(size_t)(i / VPR) * ld4 + i % VPR] : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (i0 + u * nthr < total) d4[i0 + u * nthr] = v[u];
      }
      return;
    }
  }
  const int total = cnt * RB;
  for (int i0 = tid; i0 < total; i0 += U * nthr) {
    T v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u * nthr, r = i % RB;
      v[u] = (i < total && r < rcount) ? src[(size_t)(i / RB) * ldv + rofs + r] : T(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (i0 + u * nthr < total) dst[i0 + u * nthr] = v[u];
  }
}

// acc[r] += v * row[r] for r < RB; FP32 with RB a multiple of 4: packed
// FP32x2 FMAs on column pairs fed by 16-byte loads (row 16-byte aligned),
// the same rounding per element as the scalar loop
template <typename T, int RB>
__device__ __forceinline__ void axpy_row(T (&acc)[RB], T v, const T* __restrict__ row) {
  if constexpr (sizeof(T) == 4 && RB % 4 == 0) {
    const float2 vv = make_float2(v, v);
#pragma unroll
    for (int r = 0; r < RB; r += 4) {
      const float4 x = *reinterpret_cast<const float4*>(row + r);
      const float2 p01 = __ffma2_rn(vv, make_float2(x.x, x.y), make_float2(acc[r], acc[r + 1]));
      const float2 p23 =
          __ffma2_rn(vv, make_float2(x.z, x.w), make_float2(acc[r + 2], acc[r + 3]));
      acc[r] = p01.x;
      acc[r + 1] = p01.y;
      acc[r + 2] = p23.x;
      acc[r + 3] = p23.y;
    }
  } else {
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[r] = fma(v, row[r], acc[r]);
  }
}

// o[r] = acc[r] (ADD: o[r] += acc[r]) for r < rc, as 16-byte vectors when the
// row is full and aligned
template <typename T, int RB, bool ADD>
__device__ __forceinline__ void store_row(T* o, const T (&acc)[RB], int rc) {
  if (rc == RB && (reinterpret_cast<uintptr_t>(o) & 15) == 0) {
    if constexpr (sizeof(T) == 4 && RB % 4 == 0) {
#pragma unroll
      for (int r = 0; r < RB; r += 4) {
        float4 v = make_float4(acc[r], acc[r + 1], acc[r + 2], acc[r + 3]);
        if (ADD) {
          const float4 u = *reinterpret_cast<const float4*>(o + r);
          v = make_float4(u.x + v.x, u.y + v.y, u.z + v.z, u.w + v.w);
        }
        *reinterpret_cast<float4*>(o + r) = v;
      }
      return;
    } else if constexpr (sizeof(T) == 8 && RB % 2 == 0) {
#pragma unroll
      for (int r = 0; r < RB; r += 2) {
        double2 v = make_double2(acc[r], acc[r + 1]);
        if (ADD) {
          const double2 u = *reinterpret_cast<const double2*>(o + r);
          v = make_double2(u.x + v.x, u.y + v.y);
        }
        *reinterpret_cast<double2*>(o + r) = v;
      }
      return;
    }
  }
#pragma unroll
  for (int r = 0; r < RB; ++r)
    if (r < rc) o[r] = ADD ? o[r] + acc[r] : acc[r];
}

// leaf moments: t[c][k][r] = sum_i V_c[k][i] x[i][r]
// blockDim 128; shared: F[CH][3][FS], X[CH][RB], packed digits q ints.  FS:
// slots for the 1-D factors of one dimension, 8 (degree <= 7) or 16 (the
// total-degree bases of higher degree)
template <typename T, int RB, int FS = 8>
__global__ void leafmom_kernel(const int32_t* __restrict__ leaves,
                               const uint32_t* __restrict__ cbegin,
                               const uint32_t* __restrict__ csize,
                               const T* __restrict__ bbmin,
                               const T* __restrict__ bbext,
                               const Pt4<T>* __restrict__ pts,
                               const T* __restrict__ xc, int ldv, int rofs,
                               int rcount, const int* __restrict__ midx_g,
                               InterpDev<T> ip, T* __restrict__ tout) {
  constexpr int CH = kLeafChunk;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* F = reinterpret_cast<T*>(smem_raw);  // CH x 3 x FS
  T* X = F + CH * 3 * FS;                 // CH x RB
  int* pk = reinterpret_cast<int*>(X + CH * RB);
  const int c = leaves[blockIdx.x];
  const uint32_t b = cbegin[c], n = csize[c];
  const int q = ip.q, tid = threadIdx.x, nthr = blockDim.x;
  pack_digits(midx_g, q, pk);
  T lo[3], ex[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = d < ip.dim ? bbmin[c * 3 + d] : T(0);
    ex[d] = d < ip.dim ? bbext[c * 3 + d] : T(1);
  }
  for (int kc = 0; kc < q; kc += nthr) {
    const int k = kc + tid;
    const bool valid = k < q;
    __syncthreads();
    const int kd = valid ? pk[k] : 0;
    const int m0 = kd & 255, m1 = FS + ((kd >> 8) & 255), m2 = kd >> 16;
    T acc[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[r] = T(0);
    for (uint32_t i0 = 0; i0 < n; i0 += CH) {
      const int cnt = (int)((n - i0) < (uint32_t)CH ? (n - i0) : CH);
      for (int t = tid; t < cnt * 3; t += nthr) {
        const int i = t / 3, d = t - 3 * i;
        T* f = F + t * FS;
        if (d < ip.dim) {
          const T x = reinterpret_cast<const T*>(pts + b + i0 + i)[d];
          const T lod = d == 0 ? lo[0] : (d == 1 ? lo[1] : lo[2]);
          const T exd = d == 0 ? ex[0] : (d == 1 ? ex[1] : ex[2]);
          basis1d(ip, (x - lod) / exd, f);
        } else {
          f[0] = T(1);
        }
      }
      stage_rows<T, RB>(X, xc + (size_t)(b + i0) * ldv, cnt, ldv, rofs, rcount);
      __syncthreads();
      if (valid) {
        for (int i = 0; i < cnt; ++i) {
          const T* f = F + i * 3 * FS;
          const T v = f[m0] * f[m1] * f[2 * FS + m2];
          axpy_row<T, RB>(acc, v, X + i * RB);
        }
      }
      __syncthreads();
    }
    if (valid) store_row<T, RB, false>(tout + ((size_t)c * q + k) * ldv + rofs, acc, rcount);
  }
}

// one transfer level.  up == true (M2M): for each cluster c in list,
//   t[c][k] = sum_sons sum_j E_son[k][j] t[son][j]
// up == false (L2L): for each cluster c in list (level >= 1),
//   s[c][j] += sum_k E_c[k][j] s[parent][k]
// E_c[k][j] = e_c[0][k0][j0] * e_c[1][k1][j1] * e_c[2][k2][j2]
// blockIdx.y selects right-hand sides rofs + RB * blockIdx.y onwards, so that
// a level with few clusters still spreads over many SMs.
// shared: e[3][8][8], S[JC][RB], packed digits q ints
template <typename T, int RB, bool UP>
__global__ void transfer_kernel(const int32_t* __restrict__ clist,
                                const int32_t* __restrict__ son0,
                                const int32_t* __restrict__ nsons,
                                const int32_t* __restrict__ parent,
                                const T* __restrict__ E,
                                const int* __restrict__ midx_g, InterpDev<T> ip,
                                T* buf, int ldv, int rofs, int rcount) {
  constexpr int JC = kTransferChunk;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* e = reinterpret_cast<T*>(smem_raw);  // 3 x 8 x 8
  T* S = e + 192;                         // JC x RB
  int* pk = reinterpret_cast<int*>(S + JC * RB);
  const int c = clist[blockIdx.x];
  const int q = ip.q, p1 = ip.p1, tid = threadIdx.x, nthr = blockDim.x;
  const int rofs_b = rofs + (int)blockIdx.y * RB;
  const int rc = min(RB, rcount - (int)blockIdx.y * RB);
  pack_digits(midx_g, q, pk);
  const int nsrc = UP ? nsons[c] : 1;
  for (int kc = 0; kc < q; kc += nthr) {
    const int k = kc + tid;  // output index
    const bool valid = k < q;
    __syncthreads();
    const int kd = valid ? pk[k] : 0;
    // UP: E_son[k][jj] = e[d][k_d][j_d]; DOWN: E_c[jj][k] = e[d][j_d][k_d]
    const int b0 = UP ? (kd & 255) * 8 : (kd & 255);
    const int b1 = 64 + (UP ? ((kd >> 8) & 255) * 8 : ((kd >> 8) & 255));
    const int b2 = 128 + (UP ? (kd >> 16) * 8 : (kd >> 16));
    const int sh = UP ? 0 : 3;
    T acc[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[r] = T(0);
    for (int si = 0; si < nsrc; ++si) {
      const int ec = UP ? son0[c] + si : c;          // cluster whose E is used
      const int sc = UP ? son0[c] + si : parent[c];  // source moments
      for (int j0 = 0; j0 < q; j0 += JC) {
        const int cnt = (q - j0) < JC ? (q - j0) : JC;
        __syncthreads();
        if (j0 == 0) {
          for (int i = tid; i < 192; i += nthr) {
            const int d = i / 64, a = (i / 8) % 8, bb = i % 8;
            e[i] = (d < ip.dim && a < p1 && bb < p1)
                       ? E[(((size_t)ec * ip.dim + d) * p1 + a) * p1 + bb]
                       : ((a == 0 && bb == 0) ? T(1) : T(0));
          }
        }
        stage_rows<T, RB>(S, buf + ((size_t)sc * q + j0) * ldv, cnt, ldv, rofs_b, rc);
        __syncthreads();
        if (valid) {
          for (int j = 0; j < cnt; ++j) {
            const int jd = pk[j0 + j];
            const T ev = e[b0 + ((jd & 255) << sh)] * e[b1 + (((jd >> 8) & 255) << sh)] *
                         e[b2 + ((jd >> 16) << sh)];
#pragma unroll
            for (int r = 0; r < RB; ++r) acc[r] += ev * S[j * RB + r];
          }
        }
      }
    }
    if (valid) store_row<T, RB, !UP>(buf + ((size_t)c * q + k) * ldv + rofs_b, acc, rc);
  }
}

// elements of a q x q matrix in shared memory rounded up to a multiple of
// 4, so that the rows staged after it start on a 16-byte boundary (the
// 16-byte vector stores of stage_rows)
__host__ __device__ constexpr size_t dense_pad(int q) { return ((size_t)q * q + 3) & ~(size_t)3; }

// One transfer level with dense per-cluster matrices E_c (q x q, row-major;
// total-degree interpolation):
//   UP (M2M):   t[c][k] = sum_sons sum_j E_son[k][j] t[son][j]
//   DOWN (L2L): s[c][j] += sum_k E_c[k][j] s[parent][k]
// Block = one cluster and a slice of RB right-hand sides (blockIdx.y), one
// thread per output coefficient (q <= blockDim); E and the source rows
// staged in shared memory. shared: E [q][q] (padded), S [q][RB]
template <typename T, int RB, bool UP>
__global__ void transfer_dense_kernel(const int32_t* __restrict__ clist,
                                      const int32_t* __restrict__ son0,
                                      const int32_t* __restrict__ nsons,
                                      const int32_t* __restrict__ parent,
                                      const T* __restrict__ E, int q, T* buf, int ldv,
                                      int rofs, int rcount) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* e = reinterpret_cast<T*>(smem_raw);  // q x q
  T* S = e + dense_pad(q);                 // q x RB, 16-byte aligned
  const int c = clist[blockIdx.x];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int rofs_b = rofs + (int)blockIdx.y * RB;
  const int rc = min(RB, rcount - (int)blockIdx.y * RB);
  const int nsrc = UP ? nsons[c] : 1;
  const int k = tid;  // output coefficient (q <= blockDim)
  T acc[RB];
#pragma unroll
  for (int r = 0; r < RB; ++r) acc[r] = T(0);
  for (int si = 0; si < nsrc; ++si) {
    const int ec = UP ? son0[c] + si : c;          // cluster whose E is used
    const int sc = UP ? son0[c] + si : parent[c];  // source coefficients
    __syncthreads();
    for (int i = tid; i < q * q; i += nthr) e[i] = E[(size_t)ec * q * q + i];
    stage_rows<T, RB>(S, buf + (size_t)sc * q * ldv, q, ldv, rofs_b, rc);
    __syncthreads();
    if (k < q) {
      for (int j = 0; j < q; ++j) {
        const T ev = UP ? e[k * q + j] : e[j * q + k];
#pragma unroll
        for (int r = 0; r < RB; ++r) acc[r] += ev * S[j * RB + r];
      }
    }
  }
  if (k < q) store_row<T, RB, !UP>(buf + ((size_t)c * q + k) * ldv + rofs_b, acc, rc);
}

// Change of basis of every cluster's coefficients, in place:
//   buf[c][k] = sum_j M[k][j] buf[c][j]   (M: q x q, row-major)
// for clusters 0 .. ncl - 1. With total-degree interpolation the moments of
// the upward pass are taken to the nodal basis by M = invV^T before the
// far field, and the far-field expansions back by M = invV after it, so that
// the coupling invV K invV^T (NystromEvaluator.h:40-56) becomes a kernel sum
// over the interpolation nodes. shared: M [q][q] (padded), S [q][RB]
template <typename T, int RB>
__global__ void basis_change_kernel(int ncl, const T* __restrict__ M, int q, T* buf, int ldv,
                                    int rofs, int rcount) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* m = reinterpret_cast<T*>(smem_raw);  // q x q
  T* S = m + dense_pad(q);                 // q x RB, 16-byte aligned
  const int c = blockIdx.x;
  if (c >= ncl) return;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int rofs_b = rofs + (int)blockIdx.y * RB;
  const int rc = min(RB, rcount - (int)blockIdx.y * RB);
  for (int i = tid; i < q * q; i += nthr) m[i] = M[i];
  stage_rows<T, RB>(S, buf + (size_t)c * q * ldv, q, ldv, rofs_b, rc);
  __syncthreads();
  for (int k = tid; k < q; k += nthr) {
    T acc[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[r] = T(0);
    for (int j = 0; j < q; ++j) {
      const T mv = m[k * q + j];
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r] += mv * S[j * RB + r];
    }
    store_row<T, RB, false>(buf + ((size_t)c * q + k) * ldv + rofs_b, acc, rc);
  }
}

// One transfer level, sum-factorised (FP32, 32 right-hand sides):
// E_c = e_c[0] (x) e_c[1] (x) ... applied as DIM contractions of P terms
// each, on the coefficients held in tensor order (node with digits
// (i_0, .., i_{DIM-1}) at position (i_0 P + i_1) P + ..). Block = one
// cluster, 4 or 8 warps, lane = right-hand side rofs + lane; a contraction over
// dimension d hands every warp whole columns (the P coefficients that
// differ in digit d): P loads, P^2 FMAs and P stores per column.
//   UP (M2M):   t[c] = sum_sons (e_son[0] (x) ..) t[son]   (e[k][j], k: c)
//   DOWN (L2L): s[c] += (e_c[0] (x) ..)^T s[parent]        (e[k][j], j: c)
// The same sums as transfer_kernel, in another order of the terms. Global
// rows move in batches of 8 loads per lane, so that their latencies overlap.
// shared: X, Y, Z [P^DIM][32] floats, sidx [P^DIM] ints, e [DIM][P][P]
template <int DIM, int P, bool UP>
__global__ void __launch_bounds__(256)
    transfer_sf_kernel(const int32_t* __restrict__ clist, const int32_t* __restrict__ son0,
                       const int32_t* __restrict__ nsons, const int32_t* __restrict__ parent,
                       const float* __restrict__ E, const int* __restrict__ midx_g,
                       float* buf, int ldv, int rofs, int rcount) {
  constexpr int Q = DIM == 1 ? P : DIM == 2 ? P * P : P * P * P;
  constexpr int NC = Q / P;  // columns of one contraction
  extern __shared__ __align__(16) float smf[];
  float* X = smf;
  float* Y = X + Q * 32;
  float* Z = Y + Q * 32;
  int* sidx = reinterpret_cast<int*>(Z + Q * 32);  // tensor position -> storage index
  float* ef = reinterpret_cast<float*>(sidx + Q);  // [DIM][P][P]
  const int c = clist[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const bool live = lane < rcount;
  const int r = rofs + lane;
  for (int k = threadIdx.x; k < Q; k += blockDim.x) {
    int pos = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) pos = pos * P + midx_g[k * 3 + d];
    sidx[pos] = k;
  }
  for (int e = threadIdx.x; e < Q * 32; e += blockDim.x) Z[e] = 0.f;
  constexpr int U = 8;
  const int nsrc = UP ? nsons[c] : 1;
  for (int si = 0; si < nsrc; ++si) {
    const int ec = UP ? son0[c] + si : c;
    const int sc = UP ? son0[c] + si : parent[c];
    __syncthreads();  // previous source done with X, Y and ef; sidx ready
    for (int e = threadIdx.x; e < DIM * P * P; e += blockDim.x) ef[e] = E[(size_t)ec * DIM * P * P + e];
    for (int t0 = warp; t0 < Q; t0 += nw * U) {
      float v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int t = t0 + nw * u;
        v[u] = (t < Q && live) ? buf[((size_t)sc * Q + sidx[t]) * ldv + r] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (t0 + nw * u < Q) X[(t0 + nw * u) * 32 + lane] = v[u];
    }
    __syncthreads();
    float* in = X;
    float* out = Y;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      // stride of digit d and the factor, oriented output x input
      const int stride = d == DIM - 1 ? 1 : (d == DIM - 2 ? P : P * P);
      float f[P][P];
#pragma unroll
      for (int a = 0; a < P; ++a)
#pragma unroll
        for (int b = 0; b < P; ++b)
          f[a][b] = UP ? ef[(d * P + a) * P + b] : ef[(d * P + b) * P + a];
      const bool last = d == DIM - 1;
      for (int col = warp; col < NC; col += nw) {
        // base position of the column: digits other than d from col
        const int hi = col / stride, lo = col % stride;
        const int base = hi * stride * P + lo;
        float v[P];
#pragma unroll
        for (int j = 0; j < P; ++j) v[j] = in[(base + j * stride) * 32 + lane];
#pragma unroll
        for (int a = 0; a < P; ++a) {
          float acc = 0.f;
#pragma unroll
          for (int j = 0; j < P; ++j) acc = fmaf(f[a][j], v[j], acc);
          const int o = (base + a * stride) * 32 + lane;
          if (!last)
            out[o] = acc;
          else
            Z[o] += acc;
        }
      }
      __syncthreads();
      float* tmp = in;
      in = out;
      out = tmp;
    }
  }
  // UP: t[c] = Z; DOWN: s[c] += Z
  if (live)
    for (int t0 = warp; t0 < Q; t0 += nw * U) {
      float v[U];
      if (!UP) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int t = t0 + nw * u;
          v[u] = t < Q ? buf[((size_t)c * Q + sidx[t]) * ldv + r] : 0.f;
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int t = t0 + nw * u;
        if (t < Q)
          buf[((size_t)c * Q + sidx[t]) * ldv + r] = UP ? Z[t * 32 + lane] : v[u] + Z[t * 32 + lane];
      }
    }
}

// leaf gather: yfar[i][r] = sum_k V_c[k][i] s[c][k][r] for row leaves; in
// FP32 the sum over k is compensated (compensated_sum.h)
// shared: F[3 FS][blockDim] (one column per thread), S[q][RB], packed digits
// q ints; FS as for leafmom_kernel
template <typename T, int RB, int FS = 8>
__global__ void leafgather_kernel(const int32_t* __restrict__ leaves,
                                  const uint32_t* __restrict__ cbegin,
                                  const uint32_t* __restrict__ csize,
                                  const T* __restrict__ bbmin,
                                  const T* __restrict__ bbext,
                                  const Pt4<T>* __restrict__ pts,
                                  const T* __restrict__ s, int ldv, int rofs,
                                  int rcount, const int* __restrict__ midx_g,
                                  InterpDev<T> ip, T* __restrict__ yout) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int q = ip.q, tid = threadIdx.x, nthr = blockDim.x;
  T* F = reinterpret_cast<T*>(smem_raw);  // 3 FS x blockDim
  T* S = F + nthr * 3 * FS;               // q x RB
  int* pk = reinterpret_cast<int*>(S + (size_t)q * RB);
  const int c = leaves[blockIdx.x];
  const uint32_t b = cbegin[c], n = csize[c];
  pack_digits(midx_g, q, pk);
  T lo[3], ex[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = d < ip.dim ? bbmin[c * 3 + d] : T(0);
    ex[d] = d < ip.dim ? bbext[c * 3 + d] : T(1);
  }
  stage_rows<T, RB>(S, s + (size_t)c * q * ldv, q, ldv, rofs, rcount);
  __syncthreads();
  T* f = F + tid;
  for (uint32_t i0 = 0; i0 < n; i0 += nthr) {
    if (i0 + tid >= n) break;
    const Pt4<T> p = pts[b + i0 + tid];
    const T pc[3] = {p.x, p.y, p.z};
    for (int d = 0; d < 3; ++d) {
      if (d < ip.dim)
        basis1d(ip, (pc[d] - lo[d]) / ex[d], f + d * FS * nthr, nthr);
      else
        f[d * FS * nthr] = T(1);
    }
    T acc[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[r] = T(0);
    if constexpr (sizeof(T) == 4) {
      // compensated: plain partial sums of kGatherBlock terms, each added
      // into the total with Kahan's compensation (compensated_sum.h)
      T cmp[RB];
#pragma unroll
      for (int r = 0; r < RB; ++r) cmp[r] = T(0);
      for (int k0 = 0; k0 < q; k0 += kGatherBlock) {
        const int k1 = min(q, k0 + kGatherBlock);
        T part[RB];
#pragma unroll
        for (int r = 0; r < RB; ++r) part[r] = T(0);
        for (int k = k0; k < k1; ++k) {
          const int kd = pk[k];
          const T v = f[(kd & 255) * nthr] * f[(FS + ((kd >> 8) & 255)) * nthr] *
                      f[(2 * FS + (kd >> 16)) * nthr];
          axpy_row<T, RB>(part, v, S + k * RB);
        }
#pragma unroll
        for (int r = 0; r < RB; ++r) kahan_add(acc[r], cmp[r], part[r]);
      }
    } else {
      for (int k = 0; k < q; ++k) {
        const int kd = pk[k];
        const T v = f[(kd & 255) * nthr] * f[(FS + ((kd >> 8) & 255)) * nthr] *
                    f[(2 * FS + (kd >> 16)) * nthr];
        axpy_row<T, RB>(acc, v, S + k * RB);
      }
    }
    store_row<T, RB, false>(yout + (size_t)(b + i0 + tid) * ldv + rofs, acc, rcount);
  }
}

// x (natural order, strides) -> xc (cluster order).  Buffers are chunk-major:
// right-hand side r of row i lives at [(r / rb) * n + i] * ld + r % rb, with
// ld >= rb; padding columns are zero.
template <typename TI, typename T>
__global__ void gather_kernel(const uint32_t* __restrict__ perm, int64_t n,
                              int R, int rb, int ld, const TI* __restrict__ x,
                              int64_t sxi, int64_t sxr, T* __restrict__ xc) {
  const int nchunks = (R + rb - 1) / rb;
  const int64_t per = n * (int64_t)ld;
  const int64_t total = per * nchunks;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ch = e / per, rem = e % per;
    const int64_t i = rem / ld;
    const int rr = (int)(rem % ld);
    const int r = (int)ch * rb + rr;
    const int64_t src = perm ? (int64_t)perm[i] : i;
    xc[e] = (rr < rb && r < R) ? (T)x[src * sxi + (int64_t)r * sxr] : T(0);
  }
}

// y (natural order) = sigma2 * (ynear + yfar), combined in FP64
template <typename T, typename TO>
__global__ void scatter_kernel(const uint32_t* __restrict__ perm, int64_t n,
                               int R, int rb, int ld, const T* __restrict__ ynear,
                               const T* __restrict__ yfar, double sigma2,
                               TO* __restrict__ y, int64_t syi, int64_t syr) {
  const int64_t total = n * (int64_t)R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R;
    const int r = (int)(e % R);
    const int64_t k = ((int64_t)(r / rb) * n + i) * ld + r % rb;
    const int64_t dst = perm ? (int64_t)perm[i] : i;
    const double v = (double)ynear[k] + (double)yfar[k];
    y[dst * syi + (int64_t)r * syr] = (TO)(sigma2 * v);
  }
}

// dense FP64 kernel matrix (CovarianceKernel::eval), column-major n_r x n_c
static __global__ void dense_eval_kernel(int dim, const double* __restrict__ PR,
                                  int64_t nr, const double* __restrict__ PC,
                                  int64_t nc, KParams<double> kp, double sigma2,
                                  double* __restrict__ out) {
  const int64_t total = nr * nc;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % nr, j = e / nr;
    double r2 = 0;
    for (int d = 0; d < dim; ++d) {
      const double dd = PR[i * dim + d] - PC[j * dim + d];
      r2 = d == 0 ? dd * dd : r2 + dd * dd;
    }
    out[e] = sigma2 * keval_ref(kp.type, r2, kp);
  }
}

}  // namespace gpu
}  // namespace fmca
