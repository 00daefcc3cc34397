// Device code of the assembled H2 matrix: the stored far-field and near-field
// blocks of FMCA's computeH2Matrix (FMCA/src/H2Matrix/H2MatrixBase.h:222-255)
// and the matvec that streams them (operator*, matrix_vector_product_impl.h:
// 17-98).
//
// Storage.  The blocks are kept per target group of the matrix-free kernel
// sums (the same group lists: far groups = interpolation nodes of one row
// cluster against the nodes of its admissible column clusters, near groups =
// points of one row leaf against its merged dense column intervals).  Group g
// owns one dense block [j][i] = k(|target_i - source_j|), source-major, j
// running over the group's source sequence (its intervals in order) and i
// over its targets with the row stride tp = tcount rounded up to 4 (rows of
// 16-byte multiples, zero padded), at element offset koff[g].  A source tile
// of a group is therefore one contiguous stretch of memory that a single
// cp.async.bulk copy moves into shared memory.
//
// kstore_kernel writes the blocks (the kernel evaluated exactly as the
// matrix-free CUDA-core kernel sum evaluates it); kstream_kernel is the
// kernel sum with the evaluation replaced by the stored values: a producer
// thread streams tiles of (block rows, source values) through a ring of
// shared-memory stages completed on mbarriers, every thread accumulates TPT
// targets x RB right-hand sides in registers (FP32: packed FP32x2 FMAs).
// The stream reads every stored value once per right-hand-side chunk, so the
// kernel is bound by HBM bandwidth for FP32 and by the FP64 FMA pipe for
// FP64 with many right-hand sides.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "h2_assembled.h"
#include "h2_gpu_kernels.cuh"

namespace fmca {
namespace gpu {

constexpr int kAsmThreads = 128;

// Evaluates and stores the block of every group (grid = groups, 128
// threads; thread i owns targets i and i + 128).
template <typename T, int KT>
__global__ void __launch_bounds__(kAsmThreads)
    kstore_kernel(const KGroup* __restrict__ groups, const uint32_t* __restrict__ ivl,
                  const uint64_t* __restrict__ koff, const Pt4<T>* __restrict__ tgt,
                  const Pt4<T>* __restrict__ src, KParams<T> kp, T* __restrict__ kstore) {
  const KGroup g = groups[blockIdx.x];
  const uint32_t tp = asm_row_stride(g.tcount);
  T* __restrict__ blk = kstore + koff[blockIdx.x];
  T tx[2], ty[2], tz[2];
  bool live[2], inrow[2];
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const uint32_t i = threadIdx.x + t * kAsmThreads;
    live[t] = i < g.tcount;
    inrow[t] = i < tp;
    tx[t] = ty[t] = tz[t] = T(0);
    if (live[t]) {
      const Pt4<T> p = tgt[g.tbegin + i];
      tx[t] = p.x;
      ty[t] = p.y;
      tz[t] = p.z;
    }
  }
  uint64_t row = 0;
  for (int k = g.ivl_begin; k < g.ivl_end; ++k) {
    const uint32_t b = ivl[2 * k], e = ivl[2 * k + 1];
#pragma unroll 4
    for (uint32_t s = b; s < e; ++s) {
      const Pt4<T> p = src[s];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        if (inrow[t]) {
          T v = T(0);
          if (live[t]) {
            const T dx = tx[t] - p.x, dy = ty[t] - p.y, dz = tz[t] - p.z;
            v = keval<T, KT>(dx * dx + dy * dy + dz * dz, kp);
          }
          blk[row + threadIdx.x + t * kAsmThreads] = v;
        }
      }
      row += tp;
    }
  }
}

// out[t][rofs + r] = sum_j block[g][j][t] * sval[s_j][rofs + r] for every
// group (grid = groups).  Shared memory: 256 bytes of barriers and tile
// counts, then nst tiles of ts x ldv source values, then nst tiles of
// ts x kcap block values (kcap >= tp of every group).
template <typename T, int TPT, int RB>
__global__ void __launch_bounds__(kAsmThreads)
    kstream_kernel(const KGroup* __restrict__ groups, const uint32_t* __restrict__ ivl,
                   const uint64_t* __restrict__ koff, const T* __restrict__ kstore, int ts,
                   int kcap, int nst, const T* __restrict__ sval, int ldv,
                   T* __restrict__ out, int rofs, int rcount, unsigned long long wait_ns,
                   int stall, int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* never = reinterpret_cast<uint64_t*>(smem_raw + 64);
  int* scnt = reinterpret_cast<int*>(smem_raw + 128);
  T* svals = reinterpret_cast<T*>(smem_raw + 256);
  T* sblk = svals + (size_t)nst * ts * ldv;

  const KGroup g = groups[blockIdx.x];
  const uint32_t tp = asm_row_stride(g.tcount);
  const T* gblk = kstore + koff[blockIdx.x];
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  bool live[TPT];
#pragma unroll
  for (int t = 0; t < TPT; ++t) live[t] = (uint32_t)(tid + t * nthr) < g.tcount;

  constexpr bool kPacked = sizeof(T) == 4 && RB % 4 == 0;
  constexpr int kAcc = kPacked ? RB / 2 : RB;
  using Acc = typename std::conditional<kPacked, float2, T>::type;
  Acc acc[TPT][kAcc];
#pragma unroll
  for (int t = 0; t < TPT; ++t)
#pragma unroll
    for (int r = 0; r < kAcc; ++r) {
      if constexpr (kPacked)
        acc[t][r] = make_float2(0.f, 0.f);
      else
        acc[t][r] = T(0);
    }

  int ntiles = 0;
  for (int i = g.ivl_begin; i < g.ivl_end; ++i)
    ntiles += (int)((ivl[2 * i + 1] - ivl[2 * i] + ts - 1) / ts);

  if (tid == 0) {
    for (int s = 0; s < nst; ++s) mbar_init(&bars[s], 1);
    mbar_init(never, 1);
    fence_mbar_init();
  }
  __syncthreads();

  // producer cursor (thread 0 only): interval, offset in it, position in
  // the group's source sequence
  int pi = g.ivl_begin;
  uint32_t poff = 0;
  uint64_t pj = 0;
  int issued = 0;
  auto issue = [&](int stage) {
    const uint32_t b = ivl[2 * pi], e = ivl[2 * pi + 1];
    const uint32_t s0 = b + poff;
    const uint32_t cnt = (e - s0) < (uint32_t)ts ? (e - s0) : (uint32_t)ts;
    scnt[stage] = (int)cnt;
    const uint32_t bv = cnt * (uint32_t)ldv * (uint32_t)sizeof(T);
    const uint32_t bk = cnt * tp * (uint32_t)sizeof(T);
    mbar_expect_tx(&bars[stage], bv + bk);
    bulk_g2s(svals + (size_t)stage * ts * ldv, sval + (size_t)s0 * ldv, bv, &bars[stage]);
    bulk_g2s(sblk + (size_t)stage * ts * kcap, gblk + pj * tp, bk, &bars[stage]);
    poff += cnt;
    pj += cnt;
    if (b + poff >= e) {
      ++pi;
      poff = 0;
    }
    ++issued;
  };
  if (tid == 0)
    for (int s = 0; s < nst && s < ntiles; ++s) issue(s);

  bool aborted = false;
  int stage = 0;
  uint32_t parity = 0;
  for (int k = 0; k < ntiles; ++k) {
    const bool ok = mbar_wait_bounded((stall && k == 0) ? never : &bars[stage], parity, wait_ns);
    if (ok) {
      const int cnt = scnt[stage];
      const T* V = svals + (size_t)stage * ts * ldv + rofs;
      const T* B = sblk + (size_t)stage * ts * kcap;
#pragma unroll 2
      for (int j = 0; j < cnt; ++j) {
        T kv[TPT];
#pragma unroll
        for (int t = 0; t < TPT; ++t) kv[t] = live[t] ? B[(size_t)j * tp + tid + t * nthr] : T(0);
        const T* v = V + (size_t)j * ldv;
        if constexpr (kPacked) {
#pragma unroll
          for (int r = 0; r < RB; r += 4) {
            const float4 vv = *reinterpret_cast<const float4*>(v + r);
            const float2 v01 = make_float2(vv.x, vv.y), v23 = make_float2(vv.z, vv.w);
#pragma unroll
            for (int t = 0; t < TPT; ++t) {
              const float2 kk = make_float2(kv[t], kv[t]);
              acc[t][r / 2] = __ffma2_rn(kk, v01, acc[t][r / 2]);
              acc[t][r / 2 + 1] = __ffma2_rn(kk, v23, acc[t][r / 2 + 1]);
            }
          }
        } else if constexpr (RB % 2 == 0 && sizeof(T) == 8) {
#pragma unroll
          for (int r = 0; r < RB; r += 2) {
            const double2 vv = *reinterpret_cast<const double2*>(v + r);
#pragma unroll
            for (int t = 0; t < TPT; ++t) {
              acc[t][r] = fma(kv[t], vv.x, acc[t][r]);
              acc[t][r + 1] = fma(kv[t], vv.y, acc[t][r + 1]);
            }
          }
        } else {
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            const T vv = v[r];
#pragma unroll
            for (int t = 0; t < TPT; ++t) acc[t][r] = fma(kv[t], vv, acc[t][r]);
          }
        }
      }
    }
    if (__syncthreads_or(ok ? 0 : 1)) {
      aborted = true;
      break;
    }
    if (tid == 0 && k + nst < ntiles) issue(stage);
    if (++stage == nst) {
      stage = 0;
      parity ^= 1u;
    }
  }
  if (aborted) {
    if (tid == 0) {
      atomicExch(err, 1);
      // drain the copies this CTA still has in flight, again bounded
      for (int k = 0; k < issued; ++k)
        mbar_wait_bounded(&bars[k % nst], (uint32_t)((k / nst) & 1), kWaitLimitNs / 4);
    }
    return;
  }
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    if (!live[t]) continue;
    T* o = out + (size_t)(g.tbegin + tid + t * nthr) * ldv + rofs;
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      if (r < rcount) {
        if constexpr (kPacked)
          o[r] = (r & 1) ? acc[t][r / 2].y : acc[t][r / 2].x;
        else
          o[r] = acc[t][r];
      }
    }
  }
}

}  // namespace gpu
}  // namespace fmca
