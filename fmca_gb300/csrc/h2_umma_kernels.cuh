// Kernel sums of the mixed-precision matvec on the fifth-generation tensor
// cores (tcgen05, sm_103a).
//
// ksum_um computes out[t][0..32) = sum_s a(t, s) v[s][0..32) for one group
// of up to 128 H targets per CTA (one CTA per SM), with
//   a(t, s) = k(|t - s|) 2^(w_s - E)
// (w_s: the source's moment exponent, 0 for points; E: the largest w_s of
// the sources that serve the target half; the scaling of h2_tc_kernels.cuh),
// split into FP16 halves a = a_hi + a_lo and contracted as
//   a_hi v_hi + a_hi v_lo + a_lo v_hi
// by two tcgen05.mma per 16 sources and target half (M = 128 targets,
// K = 16 sources): a_hi x [v_hi | v_lo] with N = 64 and a_lo x v_hi with
// N = 32 (a product costs the same below N = 64, so merging the hi and lo
// values saves a third of them), A in tensor memory, B in shared memory,
// FP32 accumulators in tensor memory. Warp roles:
//   warp 0       producer: loads tiles of 128 sources with cp.async.bulk
//                (the group's source intervals packed in pieces aligned to
//                8 sources, rows outside the intervals masked; or, on
//                tensor grids, one source cluster per tile);
//   warps 1, 2   one thread each issues tensor-core products: with two
//                target halves thread j issues half j of every chunk, with
//                one half thread j issues the chunk pairs of sets j and
//                j + 2 (one tcgen05.mma takes ~70 cycles to issue, so one
//                thread cannot keep up with the evaluation warps);
//   warps 3..18  four sets of 4 evaluation warps. Warp w owns tensor-memory
//                lanes 32 (w % 4) .. + 31, i.e. targets h * 128 + lane for
//                each half h < H. Set s evaluates the chunks 2 s and 2 s + 1
//                of every tile into the A pair slot (4 k + s) mod NPS;
//   warps 19..22 flush warps, one per tensor-memory lane quarter (below).
// On tensor grids the two halves are two sibling row clusters (targets
// g.tbegin + h q + lane, lane < q) over the union of their admissible column
// clusters: every interval of the union carries the halves it serves
// (imask), and a half that a source cluster does not serve gets zero A
// values without an evaluation.
// The products of F consecutive tiles (a unit) accumulate in one of two
// accumulator buffers. The flush warps take the units in order: they add a
// unit's accumulators into the running total in shared memory
// (round-to-nearest FP32 adds per unit, as the tensor cores truncate their
// accumulations), free the accumulator buffer and the unit's stages (the
// products of a unit completing implies that every set has read the unit's
// source records), and at the end scale and write the totals. Flushing in
// separate warps keeps the evaluation sets, which run within a tile of
// each other, from waiting on one set's flush (4-5 % faster than a flush by
// the set of the unit).
// Every wait is bounded (2 s); on a timeout the CTA raises the error flag,
// drains its copies and products, frees tensor memory and returns, and
// CTAs that start after the flag was raised return at once.
// The barrier protocol is modelled in tests/test_umma_protocol.py.
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
constexpr int kUmPtsBytes = kUmTile * 16;
constexpr int kUmValBytes = kUmTile * kTcRhs * 2 * 2;  // hi and lo, interleaved
constexpr int kUmStageBytes = kUmPtsBytes + kUmValBytes;
constexpr int kUmHeader = 1024;
constexpr int kUmSets = 4;        // sets of 4 evaluation warps
constexpr int kUmFlushWarps = 4;  // one per tensor-memory lane quarter
constexpr int kUmThreads = 32 * (3 + 4 * kUmSets + kUmFlushWarps);
// floats per target row of the running total: 32 columns and a pad of 4,
// so that a quarter warp's 16-byte accesses to 8 rows hit 32 banks
constexpr int kUmTotStride = kTcRhs + 4;
// stages (a launch parameter from 2 to kUmMaxStages; the defaults were the
// fastest at n = 1e6), and the shared memory of a CTA: header, stages,
// running total [target][column]. Every size leaves no room for a second
// CTA on the SM, which matters as each CTA allocates all 512 tensor-memory
// columns.
constexpr int kUmMaxStages = 7;
__host__ __device__ constexpr int um_stages(int H) { return H == 2 ? 5 : 6; }
__host__ __device__ constexpr size_t um_smem_bytes(int H, int nst) {
  return kUmHeader + (size_t)nst * kUmStageBytes + (size_t)128 * H * kUmTotStride * sizeof(float);
}
// tiles per accumulation unit: at most 3 (4 starved the stage ring)
constexpr int kUmMaxUnit = 3;
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

// bounded wait (limit_ns) that also gives up when another role of the CTA
// aborted
__device__ __forceinline__ bool um_wait(uint64_t* bar, uint32_t parity, volatile int* abort,
                                        uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (global_timer_ns() - t0 > limit_ns) {
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
      const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
      const float2 av = kscaled2<KT, !REL && !MASKED>(r2, sw, kp);
      const float2 hv = f2(__uint_as_float(__float_as_uint(av.x) & 0xffffe000u),
                           __uint_as_float(__float_as_uint(av.y) & 0xffffe000u));
      const float2 lv = __ffma2_rn(hv, f2(-1.f, -1.f), av);
      hi[h][j] = h2_bits(__floats2half2_rn(hv.x, hv.y));
      lo[h][j] = h2_bits(__floats2half2_rn(lv.x, lv.y));
    }
  }
}

// The near field in the dot form (um_near_dot): records from
// point_pairs_dot_kernel, targets as nx = (-u_x, -u_x), ... and tn = |u|^2
// (um_targets), so r^2 = tn + |s|^2 - 2 u.s in four FP32x2 instructions.
// Masked rows get w = -inf (a = 0). Kernels with a square root take it of
// |r^2|: rounding can leave r^2 slightly below 0 for coincident points.
template <int KT, int H, bool MASKED>
__device__ __forceinline__ void um_eval_chunk_dot(const float4* __restrict__ rec, uint32_t m16,
                                                  const float2 (&nx)[H], const float2 (&ny)[H],
                                                  const float2 (&nz)[H], const float2 (&tn)[H],
                                                  const KParams<float>& kp, uint32_t (&hi)[H][8],
                                                  uint32_t (&lo)[H][8]) {
  constexpr bool kSqrt = KT != 3 && KT != 13;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float4 a = rec[2 * j], b = rec[2 * j + 1];
    const float2 sx = f2(a.x, a.y), sy = f2(a.z, a.w), sz = f2(b.x, b.y), sn = f2(b.z, b.w);
    float2 sw = f2(0.f, 0.f);
    if constexpr (MASKED) {
      if (!((m16 >> (2 * j)) & 1u)) sw.x = -CUDART_INF_F;
      if (!((m16 >> (2 * j + 1)) & 1u)) sw.y = -CUDART_INF_F;
    }
#pragma unroll
    for (int h = 0; h < H; ++h) {
      float2 r2 = __ffma2_rn(nx[h], sx, __ffma2_rn(ny[h], sy,
                                                   __ffma2_rn(nz[h], sz, __fadd2_rn(tn[h], sn))));
      if constexpr (kSqrt) r2 = f2(fabsf(r2.x), fabsf(r2.y));
      const float2 av = kscaled2<KT, !MASKED>(r2, sw, kp);
      const float2 hv = f2(__uint_as_float(__float_as_uint(av.x) & 0xffffe000u),
                           __uint_as_float(__float_as_uint(av.y) & 0xffffe000u));
      const float2 lv = __ffma2_rn(hv, f2(-1.f, -1.f), av);
      hi[h][j] = h2_bits(__floats2half2_rn(hv.x, hv.y));
      lo[h][j] = h2_bits(__floats2half2_rn(lv.x, lv.y));
    }
  }
}

// The evaluation warps' target registers for the H halves of group g (row
// = tensor-memory lane, HS targets per half): (g t, g t) per coordinate, or
// in the near field's dot form (-u, -u) with u = g (t - c) and tn = |u|^2.
// Lanes without a target get zeros.
template <int H, bool DOT>
__device__ __forceinline__ void um_targets(const Pt4<float>* __restrict__ tgt, const KGroup& g,
                                           int row, int HS, const KParams<float>& kp,
                                           float2 (&tx)[H], float2 (&ty)[H], float2 (&tz)[H],
                                           float2 (&tn)[H]) {
#pragma unroll
  for (int h = 0; h < H; ++h) {
    const uint32_t i = (uint32_t)(h * HS + row);
    float px = 0.f, py = 0.f, pz = 0.f, pn = 0.f;
    if (row < HS && i < g.tcount) {
      const Pt4<float> pt = tgt[g.tbegin + i];
      if constexpr (DOT) {
        const float ux = um_dot_coord(pt.x, kp.cx, kp.g);
        const float uy = um_dot_coord(pt.y, kp.cy, kp.g);
        const float uz = um_dot_coord(pt.z, kp.cz, kp.g);
        pn = um_dot_norm(ux, uy, uz);
        px = -ux;
        py = -uy;
        pz = -uz;
      } else {
        px = kp.g * pt.x;
        py = kp.g * pt.y;
        pz = kp.g * pt.z;
      }
    }
    tx[h] = f2(px, px);
    ty[h] = f2(py, py);
    tz[h] = f2(pz, pz);
    tn[h] = f2(pn, pn);
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
  float ux[P], uy[P], uz[P], uxy[P * P];
#pragma unroll
  for (int i = 0; i < P; ++i) {
    const float dx = tx + X[i], dy = ty + X[P + i], dz = tz + X[2 * P + i];
    ux[i] = dx * dx;
    uy[i] = dy * dy;
    uz[i] = dz * dz;
  }
  // the (a, b) line sums this set's 32 rows touch (about 7 of P^2; the
  // others are dead code), so a node costs one add instead of two
#pragma unroll
  for (int i = 0; i < P * P; ++i) uxy[i] = ux[i / P] + uy[i % P];
#pragma unroll
  for (int cc = 0; cc < 2; ++cc)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int p0 = 32 * S + 16 * cc + 2 * j, p1 = p0 + 1;
      if (p0 >= Q) {
        hi[cc][j] = lo[cc][j] = 0u;
        continue;
      }
      const float r0 = uxy[p0 / P] + uz[p0 % P];
      float r1 = 1.f, w1 = -CUDART_INF_F;
      if (p1 < Q) {
        r1 = uxy[p1 / P] + uz[p1 % P];
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

// H: target halves of 128 (groups of up to 128 H targets); REL: sources are
// interpolation nodes (q per cluster) weighted by their cluster's moment
// exponent, else points of weight 1; GRID (with REL, H = 1, 3-D, q =
// kGridP1^3): every tile is one source cluster on its tensor grid
// (tscale_grid_kernel layout; `pairs` holds the clusters' 64-byte grid-line
// records). nst: stages of the ring (2 .. kUmMaxStages). F: tiles per
// accumulation unit (1 .. min(kUmMaxUnit, nst); the tensor cores
// accumulate F tiles before a flush adds them into a running total): 2 by
// default on tensor grids and with two target halves. 256 sources per flush
// made the far field 5 % and the near field 2 % faster, and the far field's
// rounding error 1.5x larger (5e-7 relative at n = 1e6, measured against
// FP64). Both are chosen per plan by the autotuner when it is enabled.
// split (point sources, one half; null otherwise): the group's targets are
// rows of up to two leaves, rows [0, split[g]) of the first and the rest of
// the second, over the union of the leaves' source intervals; imask[i] holds
// the leaves interval i serves (bit 0: the first, bit 1: the second), the
// producer posts one row mask per leaf and every target takes its leaf's.
template <int KT, int H, bool REL, bool GRID>
__global__ void __launch_bounds__(kUmThreads, 1)
    ksum_um_kernel(const KGroup* __restrict__ groups, const uint32_t* __restrict__ ivl,
                   const Pt4<float>* __restrict__ tgt, const float4* __restrict__ pairs,
                   const __half* __restrict__ vals, float* __restrict__ out, int ldo, int rcount,
                   KParams<float> kp, int q, int* err, const uint32_t* __restrict__ imask,
                   int nst, int F, const uint32_t* __restrict__ split) {
  const int NST = nst;
  constexpr int NSETS = kUmSets, NEVAL = 4 * NSETS;
  constexpr int NT = 128 * H;  // targets of a group
  // tensor-memory columns: accumulators [buffer][thread] x 64 (0..31: the
  // a_hi v_hi + a_lo v_hi products, 32..63: a_hi v_lo), then NPS A pair
  // slots of H x 32 columns ([chunk of the pair][half] x (8 hi + 8 lo)):
  // two tiles of slots with one half, one tile with two
  constexpr int ACC0 = 0, A0 = 256;
  constexpr int NPS = ((int)kUmCols - A0) / (H * 32);
  static_assert(NPS % NSETS == 0, "pair slots: whole tiles (parity waits)");
  constexpr uint32_t IDESC64 = umma_idesc_f16(128, 64);
  constexpr uint32_t IDESC32 = umma_idesc_f16(128, 32);
  static_assert(!GRID || REL, "grid tiles: node sources");
  // targets of half h: g.tbegin + h HS + row for row < HS (on tensor grids
  // every half is one row cluster of q nodes; imask[interval] holds the
  // halves a source cluster serves)
  const int HS = GRID ? q : 128;
  // point sources of a kernel smooth at r = 0: the dot-product distance form
  constexpr bool DOT = !REL && !GRID && um_near_dot(KT);

  if (*reinterpret_cast<volatile int*>(err)) return;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);  // [NST]
  uint64_t* empty = full + NST;                              // [NST]
  uint64_t* afull = empty + NST;                             // [NPS]
  uint64_t* aempty = afull + NPS;                            // [NPS]
  // unit accumulators complete on accf[u % 4] (two buffers; a product
  // thread may run a tile ahead of the other, but starts unit u + 2 only
  // after unit u was flushed, so two barriers would do)
  uint64_t* accf = aempty + NPS;                             // [4]
  uint64_t* acce = accf + 4;                                 // [2]
  uint64_t* done = acce + 2;                                 // [2]
  uint64_t* never = done + 2;  // nothing arrives (the stalled-wait test hook)
  static_assert(8 * (2 * kUmMaxStages + 2 * NPS + 4 + 2 + 2 + 1) <= 512, "barrier area");
  static_assert(528 + 16 * kUmMaxStages <= 640, "stage masks");
  static_assert(640 + (int)sizeof(float) * NEVAL * H <= 768 &&
                    768 + 16 * kUmMaxStages <= kUmHeader,
                "second-leaf masks after the exponent maxima");
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + 512);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + 516);
  uint32_t* masks = reinterpret_cast<uint32_t*>(smem_raw + 528);  // [kUmMaxStages][4]
  float* ered = reinterpret_cast<float*>(smem_raw + 640);          // [NEVAL][H]
  // row masks of the second leaf of packed groups [kUmMaxStages][4]
  uint32_t* masks2 = reinterpret_cast<uint32_t*>(smem_raw + 768);
  // packed groups of two leaves (point sources, one half only)
  constexpr bool PKOK = H == 1 && !REL && !GRID;
  const bool pk = PKOK && split != nullptr;
  unsigned char* stages = smem_raw + kUmHeader;
  float* tot = reinterpret_cast<float*>(stages + (size_t)NST * kUmStageBytes);

  const KGroup g = groups[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t wlim = kp.wait_ns;  // limit of the waits below (not of the drains)

  // tiles of the group: its intervals widened to multiples of 8 sources
  // (grid: one tile per source cluster)
  int ntiles;
  {
    uint32_t rows = 0;
    for (int i = g.ivl_begin + lane; i < g.ivl_end; i += 32)
      rows += GRID ? (ivl[2 * i + 1] - ivl[2 * i]) / (uint32_t)q
                   : ((ivl[2 * i + 1] + 7u) & ~7u) - (ivl[2 * i] & ~7u);
    for (int o = 16; o > 0; o >>= 1) rows += __shfl_xor_sync(0xffffffffu, rows, o);
    ntiles = GRID ? (int)rows : (int)((rows + kUmTile - 1) / kUmTile);
  }

  // zero the stages (rows past the last piece of a tile hold finite data)
  // and the totals; the proxy fence orders these writes before the copies
  {
    uint4* z = reinterpret_cast<uint4*>(stages);
    const int n16 = (int)((um_smem_bytes(H, NST) - kUmHeader) / 16);
    for (int i = tid; i < n16; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int s = 0; s < NPS; ++s) {
      mbar_init(&afull[s], 4);
      mbar_init(&aempty[s], H == 2 ? 2 : 1);
    }
    for (int b = 0; b < 4; ++b) mbar_init(&accf[b], 2);
    for (int b = 0; b < 2; ++b) mbar_init(&acce[b], 4);
    mbar_init(&done[0], 1);
    mbar_init(&done[1], 1);
    mbar_init(never, 1);
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
      uint32_t pos = 0xffffffffu;  // next source inside interval pi (none yet)
      int issued = 0;
      bool ok = !kp.stall || um_wait(never, 0, abort_flag, wlim);
      // ring position of tile k: stage = k % NST, phase = (k / NST) & 1,
      // kept as counters (NST is a launch parameter; no divisions per tile)
      int stage = -1;
      uint32_t ph = 1;
      for (int k = 0; k < ntiles && ok; ++k) {
        if (++stage == NST) stage = 0;
        if (stage == 0) ph ^= 1u;
        if (k >= NST && !um_wait(&empty[stage], ph ^ 1u, abort_flag, wlim)) {
          ok = false;
          break;
        }
        unsigned char* sp = stages + (size_t)stage * kUmStageBytes;
        if constexpr (GRID) {
          // the next source cluster: its grid-line record and 128 value rows
          while (pos == 0xffffffffu || pos >= ivl[2 * pi + 1] / (uint32_t)q) {
            if (pos != 0xffffffffu) ++pi;
            pos = ivl[2 * pi] / (uint32_t)q;
          }
          const uint32_t sigma = pos++;
          masks[stage * 4] = imask ? imask[pi] : 1u;
          mbar_expect_tx(&full[stage], 64u + (uint32_t)kUmValBytes);
          bulk_g2s(sp, pairs + (size_t)sigma * 4, 64u, &full[stage]);
          bulk_g2s(sp + kUmPtsBytes, vals + (size_t)sigma * kGridRows * 2 * kTcRhs,
                   (uint32_t)kUmValBytes, &full[stage]);
          ++issued;
          continue;
        }
        // pieces: the group's intervals widened to multiples of 8 sources,
        // packed into the tile's 128 rows; every piece posts its bytes on
        // the stage barrier before its copies, and the final arrival (after
        // the row mask is written) lets the phase complete
        uint32_t row = 0, m0 = 0u, m1 = 0u, m2 = 0u, m3 = 0u;
        uint32_t n0 = 0u, n1 = 0u, n2 = 0u, n3 = 0u;  // second leaf (packed groups)
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
            const uint32_t r0 = row_bits(vb, ve, 0), r1 = row_bits(vb, ve, 32);
            const uint32_t r2 = row_bits(vb, ve, 64), r3 = row_bits(vb, ve, 96);
            const uint32_t sv = pk ? imask[pi] : 1u;  // leaves the interval serves
            if (sv & 1u) {
              m0 |= r0;
              m1 |= r1;
              m2 |= r2;
              m3 |= r3;
            }
            if (sv & 2u) {
              n0 |= r0;
              n1 |= r1;
              n2 |= r2;
              n3 |= r3;
            }
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
        if (pk) {
          masks2[stage * 4 + 0] = n0;
          masks2[stage * 4 + 1] = n1;
          masks2[stage * 4 + 2] = n2;
          masks2[stage * 4 + 3] = n3;
        }
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
      const int h = H == 2 ? j : 0;
      // ring position (stage, ph) and accumulation unit (u, tile kin of
      // the unit) of tile k, kept as counters
      int stage = -1, u = 0, kin = -1;
      uint32_t ph = 1;
      for (int k = 0; k < ntiles && ok; ++k) {
        if (++stage == NST) stage = 0;
        if (stage == 0) ph ^= 1u;
        if (++kin == F) {
          kin = 0;
          ++u;
        }
        const int b = u & 1;
        const bool first = kin == 0;
        if (!um_wait(&full[stage], ph, abort_flag, wlim) ||
            (first && u >= 2 &&
             !um_wait(&acce[b], (uint32_t)(((u >> 1) - 1) & 1), abort_flag, wlim))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const unsigned char* vt = stages + (size_t)stage * kUmStageBytes + kUmPtsBytes;
        const uint32_t d = tbase + ACC0 + (b * 2 + j) * 64;
        const int s0 = H == 2 ? 0 : j;
        for (int s = s0; s < NSETS; s += H == 2 ? 1 : 2) {
          const int p = 4 * k + s, slot = p % NPS;
          if (!um_wait(&afull[slot], (uint32_t)((p / NPS) & 1), abort_flag, wlim)) {
            ok = false;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int cc = 0; cc < 2; ++cc) {
            // B: 16 sources x (32 hi | 32 lo) columns; the N = 32 product
            // reads the hi half only
            const uint64_t bd = umma_desc(vt + (2 * s + cc) * 2048, 1024, 128);
            const uint32_t a = tbase + A0 + slot * (H * 32) + (cc * H + h) * 16;
            umma_f16_ts(d, a, bd, IDESC64, (first && s == s0 && cc == 0) ? 0u : 1u);
            umma_f16_ts(d, a + 8, bd, IDESC32, 1u);
          }
          umma_commit(&aempty[slot]);
        }
        if (!ok) break;
        if (kin == F - 1 || k == ntiles - 1) umma_commit(&accf[u % 4]);
      }
      if (!ok) {
        atomicExch(err, 1);
        // products already issued complete before tensor memory is freed
        umma_commit(&done[j]);
        mbar_wait_bounded(&done[j], 0, kWaitLimitNs / 8);
      }
    }
    __syncwarp();
  } else if (warp < 3 + NEVAL) {
    // ---------------- evaluation warps
    const int ew = warp - 3, set = ew >> 2;
    const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
    const int row = (warp & 3) * 32 + lane;
    // packed groups: this target belongs to the second leaf
    const bool second = pk && (uint32_t)row >= split[blockIdx.x];
    float2 tx[H], ty[H], tz[H], tn[H];
    um_targets<H, DOT>(tgt, g, row, HS, kp, tx, ty, tz, tn);
    // largest moment exponent E of the group's source clusters, per target
    // half (Eh: over the intervals that serve the half) and overall (E)
    float E = 0.f, Eh[H];
#pragma unroll
    for (int h = 0; h < H; ++h) Eh[h] = 0.f;
    if constexpr (REL) {
      float mx[H];
#pragma unroll
      for (int h = 0; h < H; ++h) mx[h] = -CUDART_INF_F;
      for (int i = g.ivl_begin + ew * 32 + lane; i < g.ivl_end; i += NEVAL * 32) {
        float mi = -CUDART_INF_F;
        for (uint32_t s = ivl[2 * i], e = ivl[2 * i + 1]; s < e; s = (s / q + 1) * q) {
          if constexpr (GRID) {
            mi = fmaxf(mi, pairs[(size_t)(s / q) * 4 + 3].w);
          } else {
            const float4 r = pairs[2 * (s >> 1) + 1];
            mi = fmaxf(mi, (s & 1u) ? r.w : r.z);
          }
        }
        const uint32_t msk = imask ? imask[i] : (1u << H) - 1u;
#pragma unroll
        for (int h = 0; h < H; ++h)
          if ((msk >> h) & 1u) mx[h] = fmaxf(mx[h], mi);
      }
#pragma unroll
      for (int h = 0; h < H; ++h) {
        for (int o = 16; o > 0; o >>= 1)
          mx[h] = fmaxf(mx[h], __shfl_xor_sync(0xffffffffu, mx[h], o));
        if (lane == 0) ered[ew * H + h] = mx[h];
      }
      named_sync(1, (NEVAL + kUmFlushWarps) * 32);
      E = -1000.f;  // groups without sources
#pragma unroll
      for (int h = 0; h < H; ++h) {
        float all = -CUDART_INF_F;
        for (int w = 0; w < NEVAL; ++w) all = fmaxf(all, ered[w * H + h]);
        Eh[h] = fmaxf(all, -1000.f);
        E = fmaxf(E, Eh[h]);
      }
    }
    bool ok = true;
    int stage = -1;  // k % NST and (k / NST) & 1, kept as counters
    uint32_t ph = 1;
    for (int k = 0; k < ntiles && ok; ++k) {
      if (++stage == NST) stage = 0;
      if (stage == 0) ph ^= 1u;
      if (!__all_sync(0xffffffffu, um_wait(&full[stage], ph, abort_flag, wlim))) {
        ok = false;
        break;
      }
      const unsigned char* sp = stages + (size_t)stage * kUmStageBytes;
      const int p = 4 * k + set, slot = p % NPS;
      auto slot_free = [&]() {
        return p < NPS ||
               __all_sync(0xffffffffu,
                          um_wait(&aempty[slot], (uint32_t)((p / NPS - 1) & 1), abort_flag, wlim));
      };
      const uint32_t a = tbase + lanes + A0 + slot * (H * 32);
      if constexpr (GRID) {
        // one source cluster: both chunks of this set from the grid lines,
        // half after half; a half the cluster does not serve gets zeros
        const float* X = reinterpret_cast<const float*>(sp);
        const uint32_t hm = masks[stage * 4];
        // one copy of each set's evaluation code: the half is a loop
        // variable and its target is selected by value
#pragma unroll 1
        for (int h = 0; h < H; ++h) {
          uint32_t gh[2][8], gl[2][8];
          const float hx = h ? tx[H - 1].x : tx[0].x;
          const float hy = h ? ty[H - 1].x : ty[0].x;
          const float hz = h ? tz[H - 1].x : tz[0].x;
          const float wv = X[15] - (h ? Eh[H - 1] : Eh[0]);
          if ((hm >> h) & 1u) {
            switch (set) {
              case 0:
                grid_eval_pair<KT, 0>(hx, hy, hz, X, wv, kp, gh, gl);
                break;
              case 1:
                grid_eval_pair<KT, 1>(hx, hy, hz, X, wv, kp, gh, gl);
                break;
              case 2:
                grid_eval_pair<KT, 2>(hx, hy, hz, X, wv, kp, gh, gl);
                break;
              default:
                grid_eval_pair<KT, 3>(hx, hy, hz, X, wv, kp, gh, gl);
                break;
            }
          } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) gh[0][i] = gh[1][i] = gl[0][i] = gl[1][i] = 0u;
          }
          if (h == 0) {
            if (!slot_free()) {
              ok = false;
              break;
            }
            tc_fence_after();
          }
#pragma unroll
          for (int cc = 0; cc < 2; ++cc) tmem_st8x2(a + (cc * H + h) * 16, gh[cc], gl[cc]);
        }
        if (!ok) break;
      } else {
        // chunk 2 s, then (once the slot is free) its A, chunk 2 s + 1 and
        // its A: one chunk of values in registers at a time
        const float4* R4 = reinterpret_cast<const float4*>(sp);
#pragma unroll
        for (int cc = 0; cc < 2; ++cc) {
          const int kk = 2 * set + cc;
          uint32_t m16 = (masks[stage * 4 + (kk >> 1)] >> ((kk & 1) * 16)) & 0xffffu;
          bool full16 = m16 == 0xffffu, none16 = m16 == 0u;
          if constexpr (PKOK) {
            if (pk) {  // the target's own leaf's mask; the paths by vote
              if (second)
                m16 = (masks2[stage * 4 + (kk >> 1)] >> ((kk & 1) * 16)) & 0xffffu;
              full16 = __all_sync(0xffffffffu, m16 == 0xffffu);
              none16 = __all_sync(0xffffffffu, m16 == 0u);
            }
          }
          uint32_t hi[H][8], lo[H][8];
          if (full16) {
            if constexpr (DOT)
              um_eval_chunk_dot<KT, H, false>(R4 + kk * 16, m16, tx, ty, tz, tn, kp, hi, lo);
            else
              um_eval_chunk<KT, H, false, REL>(R4 + kk * 16, m16, tx, ty, tz, E, kp, hi, lo);
          } else if (none16) {
#pragma unroll
            for (int h = 0; h < H; ++h)
#pragma unroll
              for (int i = 0; i < 8; ++i) hi[h][i] = lo[h][i] = 0u;
          } else {
            if constexpr (DOT)
              um_eval_chunk_dot<KT, H, true>(R4 + kk * 16, m16, tx, ty, tz, tn, kp, hi, lo);
            else
              um_eval_chunk<KT, H, true, REL>(R4 + kk * 16, m16, tx, ty, tz, E, kp, hi, lo);
          }
          if (cc == 0) {
            if (!slot_free()) {
              ok = false;
              break;
            }
            tc_fence_after();
          }
#pragma unroll
          for (int h = 0; h < H; ++h) tmem_st8x2(a + (cc * H + h) * 16, hi[h], lo[h]);
        }
        if (!ok) break;
      }
      tmem_wait_st();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive1(&afull[slot]);
    }
    if (!ok) atomicExch(err, 1);
  } else {
    // ---------------- flush warps: warp w owns tensor-memory lanes
    // 32 (w % 4) .. + 31 and adds the accumulators of every unit, in order,
    // into the running total of its targets
    const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
    const int row = (warp & 3) * 32 + lane;
    float Eh[H];
#pragma unroll
    for (int h = 0; h < H; ++h) Eh[h] = 0.f;
    if constexpr (REL) {
      // the evaluation warps' per-warp maxima of the moment exponents
      named_sync(1, (NEVAL + kUmFlushWarps) * 32);
#pragma unroll
      for (int h = 0; h < H; ++h) {
        float all = -CUDART_INF_F;
        for (int w = 0; w < NEVAL; ++w) all = fmaxf(all, ered[w * H + h]);
        Eh[h] = fmaxf(all, -1000.f);
      }
    }
    float* mytot = tot + (size_t)row * kUmTotStride;
    bool ok = true;
    const int nunits = (ntiles + F - 1) / F;
    int fstage = 0;  // stage of the first tile of unit u
    for (int u = 0; u < nunits; ++u) {
      const int b = u & 1;
      if (!__all_sync(0xffffffffu, um_wait(&accf[u % 4], (uint32_t)((u / 4) & 1), abort_flag, wlim))) {
        ok = false;
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int h = 0; h < H; ++h)
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 16) {
          // two target halves: the accumulator of thread h; one half: the
          // sum of both threads' accumulators
          uint32_t v[16], w[16];
          tmem_ld16(tbase + lanes + ACC0 + (b * 2 + h) * 64 + c0, v);
          tmem_ld16(tbase + lanes + ACC0 + (b * 2 + h) * 64 + 32 + c0, w);
          tmem_wait_ld16(v);
          tmem_wait_ld16(w);
          float x[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) x[i] = __uint_as_float(v[i]) + __uint_as_float(w[i]);
          if (H == 1) {
            tmem_ld16(tbase + lanes + ACC0 + (b * 2 + 1) * 64 + c0, v);
            tmem_ld16(tbase + lanes + ACC0 + (b * 2 + 1) * 64 + 32 + c0, w);
            tmem_wait_ld16(v);
            tmem_wait_ld16(w);
#pragma unroll
            for (int i = 0; i < 16; ++i)
              x[i] += __uint_as_float(v[i]) + __uint_as_float(w[i]);
          }
          float4* t4 = reinterpret_cast<float4*>(mytot + (size_t)h * 128 * kUmTotStride + c0);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float4 t = t4[i];
            t.x += x[4 * i];
            t.y += x[4 * i + 1];
            t.z += x[4 * i + 2];
            t.w += x[4 * i + 3];
            t4[i] = t;
          }
        }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive1(&acce[b]);
        if ((warp & 3) == 0)
          for (int t = u * F, st = fstage; t < u * F + F && t < ntiles; ++t) {
            mbar_arrive1(&empty[st]);
            if (++st == NST) st = 0;
          }
      }
      fstage += F;
      if (fstage >= NST) fstage -= NST;
    }
    if (!ok) atomicExch(err, 1);
    if (ok && !*abort_flag) {
#pragma unroll 1
      for (int h = 0; h < H; ++h) {
        const int eo = (int)(h ? Eh[H - 1] : Eh[0]);
        const uint32_t i = (uint32_t)(h * HS + row);  // target
        if (row >= HS || i >= g.tcount) continue;
        const float4* t4 = reinterpret_cast<const float4*>(mytot + (size_t)h * 128 * kUmTotStride);
        float* o = out + (size_t)(g.tbegin + i) * ldo;
        const bool whole = rcount == 32 && ldo == 32;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          float4 t = t4[c];
          if (REL) {
            t.x = ldexpf(t.x, eo);
            t.y = ldexpf(t.y, eo);
            t.z = ldexpf(t.z, eo);
            t.w = ldexpf(t.w, eo);
          }
          if (whole) {
            reinterpret_cast<float4*>(o)[c] = t;
          } else {
            if (4 * c + 0 < rcount) o[4 * c + 0] = t.x;
            if (4 * c + 1 < rcount) o[4 * c + 1] = t.y;
            if (4 * c + 2 < rcount) o[4 * c + 2] = t.z;
            if (4 * c + 3 < rcount) o[4 * c + 3] = t.w;
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

}  // namespace gpu
}  // namespace fmca
