// Kernel sums of the mixed-precision matvec on the fifth-generation tensor
// cores (tcgen05, sm_103a).
//
// ksum_um computes out[t][0..32) = sum_s a(t, s) v[s][0..32) for one group
// of up to 128 H targets per CTA (one CTA per SM), with
//   a(t, s) = k(|t - s|) 2^(w_s - E)
// (w_s: the source's moment exponent, 0 for points; E: the largest w_s of
// the group; the scaling of h2_tc_kernels.cuh),
// split into FP16 halves a = a_hi + a_lo and contracted as
//   a_hi v_hi + a_hi v_lo + a_lo v_hi
// by two tcgen05.mma per 16 sources and target half (M = 128 targets,
// K = 16 sources): a_hi x [v_hi | v_lo] with N = 64 and a_lo x v_hi with
// N = 32 (a product costs the same below N = 64, so merging the hi and lo
// values saves a third of them), A in tensor memory, B in shared memory,
// FP32 accumulators in tensor memory. Warp roles:
//   warp 0       producer: packs the group's source intervals into tiles of
//                128 sources (pieces aligned to 8 sources, rows outside the
//                intervals masked) and loads them with cp.async.bulk;
//   warp 1       one thread issues the tensor-core products;
//   warps 2..    NSETS sets of 4 evaluation warps. Warp w owns tensor-memory
//                lanes 32 (w % 4) .. + 31, i.e. targets h * 128 + lane for
//                each half h < H. Set s evaluates the 16-source chunks
//                kk = s, s + NSETS, ... of every tile into a ring of A
//                slots in tensor memory, and the set of tile k adds that
//                tile's accumulator into the running total once the total
//                holds tile k - 1 (the tensor cores round accumulations
//                toward zero, so totals are kept with round-to-nearest FP32
//                adds per tile of 128 sources).
// Every wait is bounded (2 s); on a timeout the CTA raises the error flag,
// drains its copies and products, frees tensor memory and returns, and
// CTAs that start after the flag was raised return at once.
//
// Sources arrive as pair records and FP16 values in the layouts described
// in h2_tc_kernels.cuh (pieces of whole 8-source blocks).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "h2_gpu_kernels.cuh"
#include "h2_tc_kernels.cuh"
#include "umma.cuh"

namespace fmca {
namespace gpu {

constexpr int kUmTile = 128;  // sources per stage: 8 chunks of 16
constexpr int kUmStages = 6;
constexpr int kUmPtsBytes = kUmTile * 16;
constexpr int kUmValBytes = kUmTile * kTcRhs * 2 * 2;  // hi and lo, interleaved
constexpr int kUmStageBytes = kUmPtsBytes + kUmValBytes;
constexpr int kUmHeader = 1024;
// slack after the last stage, and enough shared memory that no second CTA
// fits on the SM (each CTA allocates all 512 tensor-memory columns)
constexpr int kUmPad = 6144;
constexpr size_t kUmSmemBytes = kUmHeader + (size_t)kUmStages * kUmStageBytes + kUmPad;
constexpr uint32_t kUmCols = 512;

__device__ __forceinline__ void mbar_expect_tx_only(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(
                   umma_smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive1(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma_smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// bounded wait that also gives up when another role of the CTA aborted
__device__ __forceinline__ bool um_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (global_timer_ns() - t0 > kWaitLimitNs) {
      *abort = 1;
      return false;
    }
  }
}

// kernel values of one 16-source chunk (8 pair records) for the H targets
// of this thread, split into FP16 hi / lo registers (two sources each)
template <int KT, int H, bool MASKED, bool REL>
__device__ __forceinline__ void um_eval_chunk(const float4* __restrict__ rec, uint32_t m16,
                                              const float2 (&tx)[H], const float2 (&ty)[H],
                                              const float2 (&tz)[H], float E,
                                              const KParams<float>& kp, uint32_t (&hi)[H][8],
                                              uint32_t (&lo)[H][8]) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float4 a = rec[2 * j], b = rec[2 * j + 1];
    const float2 sx = f2(a.x, a.y), sy = f2(a.z, a.w), sz = f2(b.x, b.y);
    float2 sw = REL ? __fadd2_rn(f2(b.z, b.w), f2(-E, -E)) : f2(b.z, b.w);
    if constexpr (MASKED) {
      if (!((m16 >> (2 * j)) & 1u)) sw.x = -CUDART_INF_F;
      if (!((m16 >> (2 * j + 1)) & 1u)) sw.y = -CUDART_INF_F;
    }
#pragma unroll
    for (int h = 0; h < H; ++h) {
      const float2 dx = __fadd2_rn(tx[h], sx);
      const float2 dy = __fadd2_rn(ty[h], sy);
      const float2 dz = __fadd2_rn(tz[h], sz);
      const float2 r2 =
          __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __ffma2_rn(dx, dx, f2(1e-30f, 1e-30f))));
      const float2 av = kscaled2<KT>(r2, sw, kp);
      const float2 hv = f2(__uint_as_float(__float_as_uint(av.x) & 0xffffe000u),
                           __uint_as_float(__float_as_uint(av.y) & 0xffffe000u));
      const float2 lv = __ffma2_rn(hv, f2(-1.f, -1.f), av);
      hi[h][j] = h2_bits(__floats2half2_rn(hv.x, hv.y));
      lo[h][j] = h2_bits(__floats2half2_rn(lv.x, lv.y));
    }
  }
}

// Tensor-grid sources (one column cluster per tile, nodes in grid order):
// kernel values of the chunks 2 S and 2 S + 1 (grid rows 32 S .. 32 S + 31)
// for target (tx, ty, tz) (scaled by g). With the grid lines X (scaled by
// -g) the squared distance to node (a, b, c) is ux[a] + uy[b] + uz[c], so a
// thread squares 3 x kGridP1 differences per tile instead of three per
// pair, and the source positions are compile-time constants. wv = w - E of
// the cluster; rows past kGridP1^3 give a = 0.
template <int KT, int S>
__device__ __forceinline__ void grid_eval_pair(float tx, float ty, float tz,
                                               const float* __restrict__ X, float wv,
                                               const KParams<float>& kp, uint32_t (&hi)[2][8],
                                               uint32_t (&lo)[2][8]) {
  constexpr int P = kGridP1, Q = P * P * P;
  float ux[P], uy[P], uz[P];
#pragma unroll
  for (int i = 0; i < P; ++i) {
    const float dx = tx + X[i], dy = ty + X[P + i], dz = tz + X[2 * P + i];
    ux[i] = dx * dx;
    uy[i] = dy * dy;
    uz[i] = fmaf(dz, dz, 1e-30f);
  }
#pragma unroll
  for (int cc = 0; cc < 2; ++cc)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int p0 = 32 * S + 16 * cc + 2 * j, p1 = p0 + 1;
      if (p0 >= Q) {
        hi[cc][j] = lo[cc][j] = 0u;
        continue;
      }
      const float r0 = (ux[p0 / (P * P)] + uy[(p0 / P) % P]) + uz[p0 % P];
      float r1 = 1.f, w1 = -CUDART_INF_F;
      if (p1 < Q) {
        r1 = (ux[p1 / (P * P)] + uy[(p1 / P) % P]) + uz[p1 % P];
        w1 = wv;
      }
      const float2 av = kscaled2<KT>(f2(r0, r1), f2(wv, w1), kp);
      const float2 hv = f2(__uint_as_float(__float_as_uint(av.x) & 0xffffe000u),
                           __uint_as_float(__float_as_uint(av.y) & 0xffffe000u));
      const float2 lv = __ffma2_rn(hv, f2(-1.f, -1.f), av);
      hi[cc][j] = h2_bits(__floats2half2_rn(hv.x, hv.y));
      lo[cc][j] = h2_bits(__floats2half2_rn(lv.x, lv.y));
    }
}

// bits of rows [vb, ve) inside the 32-row word starting at row w0
__device__ __forceinline__ uint32_t row_bits(uint32_t vb, uint32_t ve, uint32_t w0) {
  const uint32_t lo = max(vb, w0), hi = min(ve, w0 + 32u);
  if (lo >= hi) return 0u;
  const uint32_t n = hi - lo;
  return (n == 32u ? 0xffffffffu : ((1u << n) - 1u)) << (lo - w0);
}

// H: target halves of 128 (groups of up to 128 H targets); NSETS: sets of
// 4 evaluation warps; REL: sources are interpolation nodes (q per cluster)
// weighted by their cluster's moment exponent, else points of weight 1.
template <int KT, int H, int NSETS, bool REL>
__global__ void __launch_bounds__(32 * (3 + 4 * NSETS), 1)
    ksum_um_kernel(const KGroup* __restrict__ groups, const uint32_t* __restrict__ ivl,
                   const Pt4<float>* __restrict__ tgt, const float4* __restrict__ pairs,
                   const __half* __restrict__ vals, float* __restrict__ out, int ldo, int rcount,
                   KParams<float> kp, int q, int* err) {
  constexpr int NST = kUmStages;
  constexpr int NEVAL = 4 * NSETS;  // evaluation warps
  // Two product threads (one tcgen05.mma takes ~70 cycles to issue from a
  // thread, so one thread cannot keep the tensor cores busy): with two target
  // halves thread j issues half j, with one half thread j issues the chunks
  // kk = j mod 2 into its own accumulator.
  // tensor-memory columns: accumulators [buffer][thread] x 64 (0..31: the
  // a_hi v_hi + a_lo v_hi products, 32..63: a_hi v_lo), the running total
  // [half] x 32 shared by all sets, A slots [slot][half] x (8 hi + 8 lo)
  constexpr int ACC0 = 0;
  constexpr int TOT0 = 2 * 2 * 64;
  constexpr int A0 = TOT0 + H * 32;
  // A slots: at most one tile (8 chunks). Parity waits are exact only while
  // a waiter is at most one phase ahead of its barrier; a longer ring would
  // let a set finish the chunks of tile k + 1 before the products of tile
  // k - 2 complete, and its accumulator wait for tile k could then pass on
  // the parity of tile k - 4.
  constexpr int NSLOT_FIT = ((int)kUmCols - A0) / (H * 16);
  constexpr int NSLOT = NSLOT_FIT >= 8 ? 8 : NSLOT_FIT;
  static_assert(NSLOT_FIT >= 4, "tensor-memory budget");
  constexpr uint32_t IDESC64 = umma_idesc_f16(128, 64);
  constexpr uint32_t IDESC32 = umma_idesc_f16(128, 32);

  if (*reinterpret_cast<volatile int*>(err)) return;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);          // [NST]
  uint64_t* empty = full + NST;                                      // [NST]
  uint64_t* afull = empty + NST;                                     // [16]
  uint64_t* aempty = afull + 16;                                     // [16]
  // tile accumulators complete on accf[k % 4] (two buffers, four barriers):
  // with one product thread up to a tile behind the other, a flush of tile
  // k may start before tile k - 2 completes, never before tile k - 4
  uint64_t* accf = aempty + 16;                                      // [4]
  uint64_t* acce = accf + 4;                                         // [2]
  uint64_t* done = acce + 2;                                         // [2]
  uint64_t* tdone = done + 2;   // one phase per flush into the shared total
  static_assert(8 * (2 * NST + 16 + 16 + 4 + 2 + 2 + 1) <= 512, "barrier area");
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + 512);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + 516);
  uint32_t* masks = reinterpret_cast<uint32_t*>(smem_raw + 528);   // [NST][4]
  float* ered = reinterpret_cast<float*>(smem_raw + 640);           // [NEVAL]
  unsigned char* stages = smem_raw + kUmHeader;

  const KGroup g = groups[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // tiles of the group: its intervals widened to multiples of 8 sources
  int ntiles;
  {
    uint32_t rows = 0;
    for (int i = g.ivl_begin + lane; i < g.ivl_end; i += 32)
      rows += ((ivl[2 * i + 1] + 7u) & ~7u) - (ivl[2 * i] & ~7u);
    for (int o = 16; o > 0; o >>= 1) rows += __shfl_xor_sync(0xffffffffu, rows, o);
    ntiles = (int)((rows + kUmTile - 1) / kUmTile);
  }

  // zero the stages once (rows past the last piece of a tile hold finite
  // data); the proxy fence orders these writes before the bulk copies
  {
    uint4* z = reinterpret_cast<uint4*>(stages);
    const int n16 = (NST * kUmStageBytes + kUmPad) / 16;
    for (int i = tid; i < n16; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NEVAL + 2);
    }
    for (int s = 0; s < 16; ++s) {
      mbar_init(&afull[s], 4);
      mbar_init(&aempty[s], H == 2 ? 2 : 1);
    }
    for (int b = 0; b < 4; ++b) mbar_init(&accf[b], 2);
    for (int b = 0; b < 2; ++b) mbar_init(&acce[b], 4);
    mbar_init(&done[0], 1);
    mbar_init(&done[1], 1);
    mbar_init(tdone, 4);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(tslot, kUmCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (warp == 0) {
    // ---------------- producer
    if (lane == 0) {
      int pi = g.ivl_begin;
      uint32_t pos = 0xffffffffu;  // aligned start inside interval pi (none yet)
      int issued = 0;
      bool ok = true;
      for (int k = 0; k < ntiles; ++k) {
        const int stage = k % NST;
        if (k >= NST && !um_wait(&empty[stage], (uint32_t)((k / NST - 1) & 1), abort_flag)) {
          ok = false;
          break;
        }
        unsigned char* sp = stages + (size_t)stage * kUmStageBytes;
        // pieces: the group's intervals widened to multiples of 8 sources,
        // packed into the tile's 128 rows; every piece posts its bytes on
        // the stage barrier before its copies, and the final arrival (after
        // the row mask is written) lets the phase complete
        uint32_t row = 0, m0 = 0u, m1 = 0u, m2 = 0u, m3 = 0u;
        while (row < (uint32_t)kUmTile && pi < g.ivl_end) {
          const uint32_t b = ivl[2 * pi], e = ivl[2 * pi + 1];
          const uint32_t a0 = pos != 0xffffffffu ? pos : (b & ~7u);
          const uint32_t ae = (e + 7u) & ~7u;
          const uint32_t take = min(ae - a0, (uint32_t)kUmTile - row);
          if (take > 0) {
            mbar_expect_tx_only(&full[stage], take * (16u + 2u * kTcRhs * 2u));
            bulk_g2s(sp + row * 16, pairs + a0, take * 16, &full[stage]);
            bulk_g2s(sp + kUmPtsBytes + row * 128, vals + (size_t)a0 * 2 * kTcRhs, take * 128,
                     &full[stage]);
            // rows [vb, ve) hold sources of the interval
            const uint32_t vb = max(b, a0) - a0 + row;
            const uint32_t ve = e > a0 ? min(e, a0 + take) - a0 + row : vb;
            m0 |= row_bits(vb, ve, 0);
            m1 |= row_bits(vb, ve, 32);
            m2 |= row_bits(vb, ve, 64);
            m3 |= row_bits(vb, ve, 96);
          }
          row += take;
          if (a0 + take >= ae) {
            ++pi;
            pos = 0xffffffffu;
          } else {
            pos = a0 + take;
          }
        }
        masks[stage * 4 + 0] = m0;
        masks[stage * 4 + 1] = m1;
        masks[stage * 4 + 2] = m2;
        masks[stage * 4 + 3] = m3;
        mbar_arrive1(&full[stage]);
        ++issued;
      }
      if (!ok) {
        atomicExch(err, 1);
        // copies still in flight land before the CTA frees its memory
        for (int k = issued > NST ? issued - NST : 0; k < issued; ++k)
          mbar_wait_bounded(&full[k % NST], (uint32_t)((k / NST) & 1), kWaitLimitNs / 8);
      }
    }
    __syncwarp();
  } else if (warp == 1 || warp == 2) {
    // ---------------- tensor-core products (thread j of two)
    const int j = warp - 1;
    if (lane == 0) {
      bool ok = true;
      for (int k = 0; k < ntiles && ok; ++k) {
        const int stage = k % NST, b = k & 1;
        if (!um_wait(&full[stage], (uint32_t)((k / NST) & 1), abort_flag) ||
            (k >= 2 && !um_wait(&acce[b], (uint32_t)(((k >> 1) - 1) & 1), abort_flag))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const unsigned char* vt = stages + (size_t)stage * kUmStageBytes + kUmPtsBytes;
        const int h = H == 2 ? j : 0;
        const uint32_t d = tbase + ACC0 + (b * 2 + j) * 64;
        for (int kk = (H == 2 ? 0 : j); kk < 8; kk += (H == 2 ? 1 : 2)) {
          const int c = k * 8 + kk, slot = c % NSLOT;
          if (!um_wait(&afull[slot], (uint32_t)((c / NSLOT) & 1), abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          // B: 16 sources x (32 hi | 32 lo) columns; the N = 32 product
          // reads the hi half only
          const uint64_t bd = umma_desc(vt + kk * 2048, 1024, 128);
          const uint32_t a = tbase + A0 + (slot * H + h) * 16;
          umma_f16_ts(d, a, bd, IDESC64, kk > (H == 2 ? 0 : j) ? 1u : 0u);
          umma_f16_ts(d, a + 8, bd, IDESC32, 1u);
          umma_commit(&aempty[slot]);
        }
        if (!ok) break;
        umma_commit(&empty[stage]);
        umma_commit(&accf[k % 4]);
      }
      if (!ok) {
        atomicExch(err, 1);
        // products already issued complete before tensor memory is freed
        umma_commit(&done[j]);
        mbar_wait_bounded(&done[j], 0, kWaitLimitNs / 8);
      }
    }
    __syncwarp();
  } else {
    // ---------------- evaluation warps
    const int ew = warp - 3, set = ew >> 2;
    const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
    const int row = (warp & 3) * 32 + lane;
    const float gs = kp.g;
    float2 tx[H], ty[H], tz[H];
#pragma unroll
    for (int h = 0; h < H; ++h) {
      const uint32_t i = (uint32_t)(h * 128 + row);
      float px = 0.f, py = 0.f, pz = 0.f;
      if (i < g.tcount) {
        const Pt4<float> p = tgt[g.tbegin + i];
        px = gs * p.x;
        py = gs * p.y;
        pz = gs * p.z;
      }
      tx[h] = f2(px, px);
      ty[h] = f2(py, py);
      tz[h] = f2(pz, pz);
    }
    // largest moment exponent E of the group's source clusters
    float E = 0.f;
    if constexpr (REL) {
      float mx = -CUDART_INF_F;
      for (int i = g.ivl_begin + ew * 32 + lane; i < g.ivl_end; i += NEVAL * 32)
        for (uint32_t s = ivl[2 * i], e = ivl[2 * i + 1]; s < e; s = (s / q + 1) * q) {
          const float4 r = pairs[2 * (s >> 1) + 1];
          mx = fmaxf(mx, (s & 1u) ? r.w : r.z);
        }
      for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0) ered[ew] = mx;
      named_sync(1, NEVAL * 32);
      float all = -CUDART_INF_F;
      for (int w = 0; w < NEVAL; ++w) all = fmaxf(all, ered[w]);
      E = fmaxf(all, -1000.f);  // groups without sources
    }

    bool ok = true;
    // flushes run tile after tile (each waits for the previous one on
    // tdone), so all sets share one running total
    auto flush = [&](int k) {
      const int b = k & 1;
      if (!__all_sync(0xffffffffu, um_wait(&accf[k % 4], (uint32_t)((k / 4) & 1), abort_flag)) ||
          (k >= 1 &&
           !__all_sync(0xffffffffu, um_wait(tdone, (uint32_t)((k - 1) & 1), abort_flag)))) {
        ok = false;
        return;
      }
      tc_fence_after();
#pragma unroll
      for (int h = 0; h < H; ++h)
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 16) {
          // two target halves: accumulator of thread h; one half: the sum
          // of both threads' accumulators
          uint32_t v[16], u[16], t[16];
          tmem_ld16(tbase + lanes + ACC0 + (b * 2 + h) * 64 + c0, v);
          tmem_ld16(tbase + lanes + ACC0 + (b * 2 + h) * 64 + 32 + c0, u);
          tmem_wait_ld16(u);
          tmem_wait_ld16(v);
#pragma unroll
          for (int i = 0; i < 16; ++i)
            v[i] = __float_as_uint(__uint_as_float(v[i]) + __uint_as_float(u[i]));
          if (H == 1) {
            tmem_ld16(tbase + lanes + ACC0 + (b * 2 + 1) * 64 + c0, t);
            tmem_ld16(tbase + lanes + ACC0 + (b * 2 + 1) * 64 + 32 + c0, u);
            tmem_wait_ld16(t);
            tmem_wait_ld16(u);
#pragma unroll
            for (int i = 0; i < 16; ++i)
              v[i] = __float_as_uint(__uint_as_float(v[i]) +
                                     (__uint_as_float(t[i]) + __uint_as_float(u[i])));
          }
          if (k > 0) {
            tmem_ld16(tbase + lanes + TOT0 + h * 32 + c0, t);
            tmem_wait_ld16(t);
#pragma unroll
            for (int i = 0; i < 16; ++i)
              v[i] = __float_as_uint(__uint_as_float(v[i]) + __uint_as_float(t[i]));
          }
          tmem_st8(tbase + lanes + TOT0 + h * 32 + c0, v);
          tmem_st8(tbase + lanes + TOT0 + h * 32 + c0 + 8, v + 8);
        }
      tmem_wait_st();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive1(&acce[b]);
        mbar_arrive1(tdone);
      }
    };

    for (int k = 0; k < ntiles && ok; ++k) {
      const int stage = k % NST;
      if (!__all_sync(0xffffffffu, um_wait(&full[stage], (uint32_t)((k / NST) & 1), abort_flag))) {
        ok = false;
        break;
      }
      const float4* R4 = reinterpret_cast<const float4*>(stages + (size_t)stage * kUmStageBytes);
      for (int kk = set; kk < 8; kk += NSETS) {
        const int c = k * 8 + kk, slot = c % NSLOT;
        if (c >= NSLOT &&
            !__all_sync(0xffffffffu,
                        um_wait(&aempty[slot], (uint32_t)((c / NSLOT - 1) & 1), abort_flag))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t m16 = (masks[stage * 4 + (kk >> 1)] >> ((kk & 1) * 16)) & 0xffffu;
        uint32_t hi[H][8], lo[H][8];
        if (m16 == 0xffffu) {
          um_eval_chunk<KT, H, false, REL>(R4 + kk * 16, m16, tx, ty, tz, E, kp, hi, lo);
        } else if (m16 == 0u) {
#pragma unroll
          for (int h = 0; h < H; ++h)
#pragma unroll
            for (int j = 0; j < 8; ++j) hi[h][j] = lo[h][j] = 0u;
        } else {
          um_eval_chunk<KT, H, true, REL>(R4 + kk * 16, m16, tx, ty, tz, E, kp, hi, lo);
        }
#pragma unroll
        for (int h = 0; h < H; ++h) {
          const uint32_t a = tbase + lanes + A0 + (slot * H + h) * 16;
          tmem_st8(a, hi[h]);
          tmem_st8(a + 8, lo[h]);
        }
        tmem_wait_st();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive1(&afull[slot]);
      }
      if (!ok) break;
      __syncwarp();
      if (lane == 0) mbar_arrive1(&empty[stage]);
      if (k >= 1 && (k - 1) % NSETS == set) {
        flush(k - 1);
        if (!ok) break;
      }
    }
    if (ok && ntiles >= 1 && (ntiles - 1) % NSETS == set) flush(ntiles - 1);
    if (!ok) atomicExch(err, 1);

    // every set's totals are complete: set 0 adds them and writes the rows
    named_sync(1, NEVAL * 32);
    if (set == 0 && !*abort_flag) {
      tc_fence_after();
      const int eo = (int)E;
#pragma unroll 1
      for (int h = 0; h < H; ++h) {
        const uint32_t i = (uint32_t)(h * 128 + row);
        float acc[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[j] = 0.f;
        if (ntiles > 0)
#pragma unroll
          for (int c0 = 0; c0 < 32; c0 += 16) {
            uint32_t t[16];
            tmem_ld16(tbase + lanes + TOT0 + h * 32 + c0, t);
            tmem_wait_ld16(t);
#pragma unroll
            for (int j = 0; j < 16; ++j) acc[c0 + j] += __uint_as_float(t[j]);
          }
        if (i < g.tcount) {
          float* o = out + (size_t)(g.tbegin + i) * ldo;
          if (REL)
#pragma unroll
            for (int j = 0; j < 32; ++j) acc[j] = ldexpf(acc[j], eo);
          if (rcount == 32 && ldo == 32) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              *reinterpret_cast<float4*>(o + j) = make_float4(acc[j], acc[j + 1], acc[j + 2], acc[j + 3]);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (j < rcount) o[j] = acc[j];
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tbase, kUmCols);
  }
}

// ---------------------------------------------------------------------------
// Far field on tensor grids (dimension 3, kGridP1^3 nodes per cluster): one
// CTA per row cluster (its nodes are the up to 128 targets, one target
// half) and one tile per admissible source cluster, in the
// tscale_grid_kernel layout (a 64-byte grid-line record and 128 value rows
// in grid order). Roles as in ksum_um_kernel (warp 0 producer, warps 1-2 the
// product threads, warps 3-18 four sets of evaluation warps), with a
// protocol that keeps the evaluation sets off the products' critical path:
//   set s evaluates the chunks 2 s and 2 s + 1 of every tile (grid rows
//     32 s .. 32 s + 31) into the A pair slot (4 k + s) mod 8, so the ring
//     holds two tiles;
//   product thread j issues the pairs of sets j and j + 2 of every tile into
//     its own accumulator of buffer k & 1, commits each pair (aempty) and
//     the tile (accf[k % 4]);
//   set k mod 4 adds both accumulators of tile k into its own running total
//     in shared memory (round-to-nearest FP32 adds per 128 sources, as the
//     tensor cores truncate their accumulations) after it has written its
//     A pair of tile k + 1, and then frees the accumulator buffer (acce) and
//     the stage (empty): the products of tile k completing implies that
//     every set has read the tile's grid lines. (Flushing before that A
//     pair instead delays the products of tile k + 1, measured slower.)
// The four totals are added at the end. Every wait is bounded as in
// ksum_um_kernel.
constexpr int kGridSets = 4;
constexpr size_t kGridTotBytes = (size_t)kGridSets * kTcRhs * 128 * sizeof(float);
constexpr size_t kGridSmemBytes = kUmHeader + (size_t)kUmStages * kUmStageBytes + kGridTotBytes;

template <int KT>
__global__ void __launch_bounds__(32 * (3 + 4 * kGridSets), 1)
    ksum_grid_kernel(const KGroup* __restrict__ groups, const uint32_t* __restrict__ ivl,
                     const Pt4<float>* __restrict__ tgt, const float4* __restrict__ rec,
                     const __half* __restrict__ vals, float* __restrict__ out, int ldo,
                     int rcount, KParams<float> kp, int* err) {
  constexpr int NST = kUmStages;
  constexpr int NSETS = kGridSets, NEVAL = 4 * NSETS;
  constexpr uint32_t q = kGridP1 * kGridP1 * kGridP1;
  // tensor-memory columns: accumulators [buffer][thread] x 64 (0..31: the
  // a_hi v_hi + a_lo v_hi products, 32..63: a_hi v_lo), then NPS pair slots
  // of 32 (chunk 2 s: hi, lo; chunk 2 s + 1: hi, lo; 8 columns each)
  constexpr int ACC0 = 0, A0 = 256, NPS = 8;
  static_assert(A0 + NPS * 32 <= (int)kUmCols, "tensor-memory budget");
  constexpr uint32_t IDESC64 = umma_idesc_f16(128, 64);
  constexpr uint32_t IDESC32 = umma_idesc_f16(128, 32);

  if (*reinterpret_cast<volatile int*>(err)) return;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);  // [NST]
  uint64_t* empty = full + NST;                              // [NST]
  uint64_t* afull = empty + NST;                             // [NPS]
  uint64_t* aempty = afull + NPS;                            // [NPS]
  uint64_t* accf = aempty + NPS;                             // [4]
  uint64_t* acce = accf + 4;                                 // [2]
  uint64_t* done = acce + 2;                                 // [2]
  static_assert(8 * (2 * NST + 2 * NPS + 4 + 2 + 2) <= 512, "barrier area");
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + 512);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + 516);
  float* ered = reinterpret_cast<float*>(smem_raw + 640);  // [NEVAL]
  unsigned char* stages = smem_raw + kUmHeader;
  // running totals [set][column][target]
  float* tot = reinterpret_cast<float*>(stages + (size_t)NST * kUmStageBytes);

  const KGroup g = groups[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  int ntiles;  // source clusters of the group
  {
    uint32_t n = 0;
    for (int i = g.ivl_begin + lane; i < g.ivl_end; i += 32)
      n += (ivl[2 * i + 1] - ivl[2 * i]) / q;
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    ntiles = (int)n;
  }
  {
    float4* z = reinterpret_cast<float4*>(tot);
    for (int i = tid; i < (int)(kGridTotBytes / 16); i += blockDim.x)
      z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int s = 0; s < NPS; ++s) {
      mbar_init(&afull[s], 4);
      mbar_init(&aempty[s], 1);
    }
    for (int b = 0; b < 4; ++b) mbar_init(&accf[b], 2);
    for (int b = 0; b < 2; ++b) mbar_init(&acce[b], 4);
    mbar_init(&done[0], 1);
    mbar_init(&done[1], 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(tslot, kUmCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (warp == 0) {
    // ---------------- producer: one source cluster per stage
    if (lane == 0) {
      int pi = g.ivl_begin;
      uint32_t pos = 0xffffffffu;  // next cluster inside interval pi (none yet)
      int issued = 0;
      bool ok = true;
      for (int k = 0; k < ntiles; ++k) {
        const int stage = k % NST;
        if (k >= NST && !um_wait(&empty[stage], (uint32_t)((k / NST - 1) & 1), abort_flag)) {
          ok = false;
          break;
        }
        while (pos == 0xffffffffu || pos >= ivl[2 * pi + 1] / q) {
          if (pos != 0xffffffffu) ++pi;
          pos = ivl[2 * pi] / q;
        }
        const uint32_t sigma = pos++;
        unsigned char* sp = stages + (size_t)stage * kUmStageBytes;
        mbar_expect_tx(&full[stage], 64u + (uint32_t)kUmValBytes);
        bulk_g2s(sp, rec + (size_t)sigma * 4, 64u, &full[stage]);
        bulk_g2s(sp + kUmPtsBytes, vals + (size_t)sigma * kGridRows * 2 * kTcRhs,
                 (uint32_t)kUmValBytes, &full[stage]);
        ++issued;
      }
      if (!ok) {
        atomicExch(err, 1);
        // copies still in flight land before the CTA frees its memory
        for (int k = issued > NST ? issued - NST : 0; k < issued; ++k)
          mbar_wait_bounded(&full[k % NST], (uint32_t)((k / NST) & 1), kWaitLimitNs / 8);
      }
    }
    __syncwarp();
  } else if (warp == 1 || warp == 2) {
    // ---------------- tensor-core products (thread j of two)
    const int j = warp - 1;
    if (lane == 0) {
      bool ok = true;
      for (int k = 0; k < ntiles && ok; ++k) {
        const int stage = k % NST, b = k & 1;
        if (!um_wait(&full[stage], (uint32_t)((k / NST) & 1), abort_flag) ||
            (k >= 2 && !um_wait(&acce[b], (uint32_t)(((k >> 1) - 1) & 1), abort_flag))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const unsigned char* vt = stages + (size_t)stage * kUmStageBytes + kUmPtsBytes;
        const uint32_t d = tbase + ACC0 + (b * 2 + j) * 64;
        for (int s = j; s < NSETS; s += 2) {
          const int p = 4 * k + s, slot = p % NPS;
          if (!um_wait(&afull[slot], (uint32_t)((p / NPS) & 1), abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int cc = 0; cc < 2; ++cc) {
            // B: 16 sources x (32 hi | 32 lo) columns; the N = 32 product
            // reads the hi half only
            const uint64_t bd = umma_desc(vt + (2 * s + cc) * 2048, 1024, 128);
            const uint32_t a = tbase + A0 + slot * 32 + cc * 16;
            umma_f16_ts(d, a, bd, IDESC64, (s == j && cc == 0) ? 0u : 1u);
            umma_f16_ts(d, a + 8, bd, IDESC32, 1u);
          }
          umma_commit(&aempty[slot]);
        }
        if (!ok) break;
        umma_commit(&accf[k % 4]);
      }
      if (!ok) {
        atomicExch(err, 1);
        // products already issued complete before tensor memory is freed
        umma_commit(&done[j]);
        mbar_wait_bounded(&done[j], 0, kWaitLimitNs / 8);
      }
    }
    __syncwarp();
  } else {
    // ---------------- evaluation warps
    const int ew = warp - 3, set = ew >> 2;
    const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
    const int row = (warp & 3) * 32 + lane;
    float tx = 0.f, ty = 0.f, tz = 0.f;
    if ((uint32_t)row < g.tcount) {
      const Pt4<float> pt = tgt[g.tbegin + row];
      tx = kp.g * pt.x;
      ty = kp.g * pt.y;
      tz = kp.g * pt.z;
    }
    // largest moment exponent E of the group's source clusters
    float E;
    {
      float mx = -CUDART_INF_F;
      for (int i = g.ivl_begin + ew * 32 + lane; i < g.ivl_end; i += NEVAL * 32)
        for (uint32_t c = ivl[2 * i] / q, ce = ivl[2 * i + 1] / q; c < ce; ++c)
          mx = fmaxf(mx, rec[(size_t)c * 4 + 3].w);
      for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0) ered[ew] = mx;
      named_sync(1, NEVAL * 32);
      float all = -CUDART_INF_F;
      for (int w = 0; w < NEVAL; ++w) all = fmaxf(all, ered[w]);
      E = fmaxf(all, -1000.f);  // groups without sources
    }
    float* mytot = tot + (size_t)set * kTcRhs * 128 + row;

    bool ok = true;
    auto flush = [&](int k) {
      const int b = k & 1;
      if (!__all_sync(0xffffffffu, um_wait(&accf[k % 4], (uint32_t)((k / 4) & 1), abort_flag))) {
        ok = false;
        return;
      }
      tc_fence_after();
#pragma unroll
      for (int c0 = 0; c0 < 32; c0 += 16) {
        uint32_t v[16], u[16], t[16], w[16];
        tmem_ld16(tbase + lanes + ACC0 + b * 128 + c0, v);
        tmem_ld16(tbase + lanes + ACC0 + b * 128 + 32 + c0, u);
        tmem_ld16(tbase + lanes + ACC0 + b * 128 + 64 + c0, t);
        tmem_ld16(tbase + lanes + ACC0 + b * 128 + 96 + c0, w);
        tmem_wait_ld16(v);
        tmem_wait_ld16(u);
        tmem_wait_ld16(t);
        tmem_wait_ld16(w);
#pragma unroll
        for (int i = 0; i < 16; ++i)
          mytot[(c0 + i) * 128] += (__uint_as_float(v[i]) + __uint_as_float(u[i])) +
                                   (__uint_as_float(t[i]) + __uint_as_float(w[i]));
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive1(&acce[b]);
        if ((warp & 3) == 0) mbar_arrive1(&empty[k % NST]);
      }
    };

    for (int k = 0; k < ntiles && ok; ++k) {
      const int stage = k % NST;
      if (!__all_sync(0xffffffffu, um_wait(&full[stage], (uint32_t)((k / NST) & 1), abort_flag))) {
        ok = false;
        break;
      }
      const float* X = reinterpret_cast<const float*>(stages + (size_t)stage * kUmStageBytes);
      const float wv = X[15] - E;
      uint32_t gh[2][8], gl[2][8];
      switch (set) {
        case 0:
          grid_eval_pair<KT, 0>(tx, ty, tz, X, wv, kp, gh, gl);
          break;
        case 1:
          grid_eval_pair<KT, 1>(tx, ty, tz, X, wv, kp, gh, gl);
          break;
        case 2:
          grid_eval_pair<KT, 2>(tx, ty, tz, X, wv, kp, gh, gl);
          break;
        default:
          grid_eval_pair<KT, 3>(tx, ty, tz, X, wv, kp, gh, gl);
          break;
      }
      const int p = 4 * k + set, slot = p % NPS;
      if (p >= NPS &&
          !__all_sync(0xffffffffu,
                      um_wait(&aempty[slot], (uint32_t)((p / NPS - 1) & 1), abort_flag))) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t a = tbase + lanes + A0 + slot * 32;
      tmem_st8(a, gh[0]);
      tmem_st8(a + 8, gl[0]);
      tmem_st8(a + 16, gh[1]);
      tmem_st8(a + 24, gl[1]);
      tmem_wait_st();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive1(&afull[slot]);
      if (k >= 1 && (k - 1) % NSETS == set) {
        flush(k - 1);
        if (!ok) break;
      }
    }
    if (ok && ntiles >= 1 && (ntiles - 1) % NSETS == set) flush(ntiles - 1);
    if (!ok) atomicExch(err, 1);

    // all totals are complete: set s adds the four totals of columns
    // 8 s .. 8 s + 7 and writes them
    named_sync(1, NEVAL * 32);
    if (!*abort_flag && (uint32_t)row < g.tcount) {
      const int eo = (int)E;
      float acc[8];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const float* t = tot + (size_t)(8 * set + jj) * 128 + row;
        acc[jj] = ldexpf(((t[0] + t[kTcRhs * 128]) + t[2 * kTcRhs * 128]) + t[3 * kTcRhs * 128],
                         eo);
      }
      float* o = out + (size_t)(g.tbegin + row) * ldo + 8 * set;
      if (rcount == 32 && ldo == 32) {
        *reinterpret_cast<float4*>(o) = make_float4(acc[0], acc[1], acc[2], acc[3]);
        *reinterpret_cast<float4*>(o + 4) = make_float4(acc[4], acc[5], acc[6], acc[7]);
      } else {
#pragma unroll
        for (int jj = 0; jj < 8; ++jj)
          if (8 * set + jj < rcount) o[jj] = acc[jj];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tbase, kUmCols);
  }
}

}  // namespace gpu
}  // namespace fmca
