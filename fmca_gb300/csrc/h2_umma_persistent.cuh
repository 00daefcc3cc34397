// The tensor-core kernel sum (ksum_um_kernel, h2_umma_kernels.cuh) as one
// persistent launch over a flattened group list: one CTA per SM, each running
// its share of the groups (of every point cloud of a batched plan) in turn.
// Measured at n = 1e6 (3-D, p = 4, R = 32) the per-group launch is as fast or
// faster (the item loop costs instructions and code size in every tile), so
// the autotuner picks this form only where it measures it faster.
#pragma once

#include "h2_umma_kernels.cuh"

namespace fmca {
namespace gpu {

// Largest moment exponent of every group's source clusters, per target half
// (over the intervals that serve the half; imask NULL: all halves), at
// least -1000 (groups without sources): gexp[2 g + h]. One warp per group.
// Node sources carry their cluster's exponent in the w fields of their pair
// records, grid tiles in the w of the 64-byte grid record.
template <bool GRID, int H>
__global__ void group_exponents_kernel(const KGroup* __restrict__ groups, int ngroups,
                                       const uint32_t* __restrict__ ivl,
                                       const float4* __restrict__ pairs, int q,
                                       const uint32_t* __restrict__ imask,
                                       float* __restrict__ gexp) {
  const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (gw >= ngroups) return;
  const KGroup g = groups[gw];
  float mx[H];
#pragma unroll
  for (int h = 0; h < H; ++h) mx[h] = -CUDART_INF_F;
  for (int i = g.ivl_begin + lane; i < g.ivl_end; i += 32) {
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
    for (int o = 16; o > 0; o >>= 1) mx[h] = fmaxf(mx[h], __shfl_xor_sync(0xffffffffu, mx[h], o));
    if (lane == 0) gexp[(size_t)gw * 2 + h] = fmaxf(mx[h], -1000.f);
  }
}

// ksum_um_kernel as a persistent launch: CTA b runs groups b, b + gridDim.x,
// ... in turn, through one copy ring, one barrier set and one tensor-memory
// allocation. The ring, pair-slot and unit counters run on over the groups;
// the last accumulation unit of every group closes early (units never span
// two groups), and the flush warps write a group's totals and clear them
// before the next group's first unit. Target coordinates are loaded and the
// moment exponents E read (from group_exponents_kernel) where a group
// begins. Roles, barriers, bounded waits and the abort path are those of
// ksum_um_kernel; the protocol over several groups is modelled in
// tests/test_umma_protocol.py.
template <int KT, int H, bool REL, bool GRID>
__global__ void __launch_bounds__(kUmThreads, 1)
    ksum_um_persistent_kernel(const KGroup* __restrict__ groups, int ngroups, const uint32_t* __restrict__ ivl,
                   const Pt4<float>* __restrict__ tgt, const float4* __restrict__ pairs,
                   const __half* __restrict__ vals, float* __restrict__ out, int ldo, int rcount,
                   KParams<float> kp, int q, int* err, const uint32_t* __restrict__ imask,
                   const float* __restrict__ gexp, int nst, int F) {
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
  constexpr bool DOT = !REL && !GRID && um_near_dot(KT);  // near-field distance form

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
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + 512);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + 516);
  uint32_t* masks = reinterpret_cast<uint32_t*>(smem_raw + 528);  // [kUmMaxStages][4]
  unsigned char* stages = smem_raw + kUmHeader;
  float* tot = reinterpret_cast<float*>(stages + (size_t)NST * kUmStageBytes);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t wlim = kp.wait_ns;  // limit of the waits below (not of the drains)
  // tiles of group g (warp-collective): its intervals widened to multiples
  // of 8 sources (grid: one tile per source cluster)
  auto group_tiles = [&](const KGroup& g) {
    uint32_t rows = 0;
    for (int i = g.ivl_begin + lane; i < g.ivl_end; i += 32)
      rows += GRID ? (ivl[2 * i + 1] - ivl[2 * i]) / (uint32_t)q
                   : ((ivl[2 * i + 1] + 7u) & ~7u) - (ivl[2 * i] & ~7u);
    for (int o = 16; o > 0; o >>= 1) rows += __shfl_xor_sync(0xffffffffu, rows, o);
    return GRID ? (int)rows : (int)((rows + kUmTile - 1) / kUmTile);
  };
  // the groups of this CTA: blockIdx.x, + gridDim.x, ... (one group per CTA
  // when the grid has one CTA per group; a persistent grid of one CTA per SM
  // runs several in turn through the same ring, barriers and tensor memory)
  const int g0 = blockIdx.x, gstep = gridDim.x;

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
    int issued = 0;
    bool ok = true;
    if (lane == 0) ok = !kp.stall || um_wait(never, 0, abort_flag, wlim);
    ok = __shfl_sync(0xffffffffu, ok, 0);
    // ring position of tile k: stage = k % NST, phase = (k / NST) & 1, kept
    // as counters (NST is a launch parameter; no divisions per tile); k runs
    // on over the groups of the CTA
    int stage = -1, k = 0;
    uint32_t ph = 1;
    for (int gi = g0; gi < ngroups && ok; gi += gstep) {
      const KGroup g = groups[gi];
      const int ntiles = group_tiles(g);
      if (lane == 0) {
        int pi = g.ivl_begin;
        uint32_t pos = 0xffffffffu;  // next source inside interval pi (none yet)
        for (int kt = 0; kt < ntiles && ok; ++kt, ++k) {
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
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
    }
    if (lane == 0 && !ok) {
      atomicExch(err, 1);
      // copies still in flight land before the CTA frees its memory
      for (int kk = issued > NST ? issued - NST : 0; kk < issued; ++kk)
        mbar_wait_bounded(&full[kk % NST], (uint32_t)((kk / NST) & 1), kWaitLimitNs / 8);
    }
    __syncwarp();
  } else if (warp == 1 || warp == 2) {
    // ---------------- tensor-core products (thread j of two)
    const int j = warp - 1;
    bool ok = true;
    const int h = H == 2 ? j : 0;
    // ring position (stage, ph), tile k and accumulation unit u of the CTA's
    // tile stream (units never span two groups) and tile kin of the unit,
    // kept as counters
    int stage = -1, u = -1, kin = 0, k = 0;
    uint32_t ph = 1;
    for (int gi = g0; gi < ngroups && ok; gi += gstep) {
      const int ntiles = group_tiles(groups[gi]);
      if (lane == 0) {
        for (int kt = 0; kt < ntiles && ok; ++kt, ++k) {
          if (++stage == NST) stage = 0;
          if (stage == 0) ph ^= 1u;
          if (kt == 0 || ++kin == F) {
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
          if (kin == F - 1 || kt == ntiles - 1) umma_commit(&accf[u % 4]);
        }
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
    }
    if (lane == 0 && !ok) {
      atomicExch(err, 1);
      // products already issued complete before tensor memory is freed
      umma_commit(&done[j]);
      mbar_wait_bounded(&done[j], 0, kWaitLimitNs / 8);
    }
    __syncwarp();
  } else if (warp < 3 + NEVAL) {
    // ---------------- evaluation warps
    const int ew = warp - 3, set = ew >> 2;
    const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
    const int row = (warp & 3) * 32 + lane;
    bool ok = true;
    int stage = -1, k = 0;  // k % NST and (k / NST) & 1, kept as counters
    uint32_t ph = 1;
    for (int gi = g0; gi < ngroups && ok; gi += gstep) {
    const KGroup g = groups[gi];
    const int ntiles = group_tiles(g);
    float2 tx[H], ty[H], tz[H], tn[H];
    um_targets<H, DOT>(tgt, g, row, HS, kp, tx, ty, tz, tn);
    // largest moment exponent of the group's source clusters per target half
    // (Eh, over the intervals that serve the half: group_exponents_kernel)
    // and overall (E)
    float E = 0.f, Eh[H];
#pragma unroll
    for (int h = 0; h < H; ++h) Eh[h] = 0.f;
    if constexpr (REL) {
      E = -1000.f;  // groups without sources
#pragma unroll
      for (int h = 0; h < H; ++h) {
        Eh[h] = gexp[(size_t)gi * 2 + h];
        E = fmaxf(E, Eh[h]);
      }
    }
    for (int kt = 0; kt < ntiles && ok; ++kt, ++k) {
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
          const uint32_t m16 = (masks[stage * 4 + (kk >> 1)] >> ((kk & 1) * 16)) & 0xffffu;
          uint32_t hi[H][8], lo[H][8];
          if (m16 == 0xffffu) {
            if constexpr (DOT)
              um_eval_chunk_dot<KT, H, false>(R4 + kk * 16, m16, tx, ty, tz, tn, kp, hi, lo);
            else
              um_eval_chunk<KT, H, false, REL>(R4 + kk * 16, m16, tx, ty, tz, E, kp, hi, lo);
          } else if (m16 == 0u) {
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
    }
    if (!ok) atomicExch(err, 1);
  } else {
    // ---------------- flush warps: warp w owns tensor-memory lanes
    // 32 (w % 4) .. + 31 and adds the accumulators of every unit, in order,
    // into the running total of its targets; at the end of every group it
    // scales and writes the totals and clears them for the next group
    const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
    const int row = (warp & 3) * 32 + lane;
    float* mytot = tot + (size_t)row * kUmTotStride;
    bool ok = true;
    int u = 0;       // unit of the CTA's tile stream
    int fstage = 0;  // stage of the first tile of unit u
    for (int gi = g0; gi < ngroups && ok; gi += gstep) {
      const KGroup g = groups[gi];
      const int ntiles = group_tiles(g);
      float Eh[H];
#pragma unroll
      for (int h = 0; h < H; ++h) Eh[h] = REL ? gexp[(size_t)gi * 2 + h] : 0.f;
      for (int t0 = 0; t0 < ntiles; t0 += F, ++u) {
        const int b = u & 1, c = min(F, ntiles - t0);  // tiles of the unit
        if (!__all_sync(0xffffffffu,
                        um_wait(&accf[u % 4], (uint32_t)((u / 4) & 1), abort_flag, wlim))) {
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
            for (int t = 0, st = fstage; t < c; ++t) {
              mbar_arrive1(&empty[st]);
              if (++st == NST) st = 0;
            }
        }
        fstage += c;
        if (fstage >= NST) fstage -= NST;
      }
      if (!ok || *abort_flag) {
        ok = false;
        break;
      }
      // the group's results: totals x 2^E, then cleared for the next group
#pragma unroll 1
      for (int h = 0; h < H; ++h) {
        const int eo = (int)(h ? Eh[H - 1] : Eh[0]);
        const uint32_t i = (uint32_t)(h * HS + row);  // target
        float4* t4 = reinterpret_cast<float4*>(mytot + (size_t)h * 128 * kUmTotStride);
        if (row < HS && i < g.tcount) {
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
#pragma unroll
        for (int c = 0; c < 8; ++c) t4[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    if (!ok) atomicExch(err, 1);
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
