// Cluster-tree construction on the GPU: the level sorter of Tree::build_with.
//
// The reference splits a cluster by sorting its index range along the
// longest edge of its box with std::sort and halving it
// (FMCA/src/Clustering/ClusterTreeSplitter.h:60-81, called level after level
// by ClusterTreeInitializer_ClusterTree.h:56-86).  When the coordinates of a
// range are distinct, its sorted order is unique, so any sort gives the
// reference's permutation; only equal coordinates are ordered by
// libstdc++'s introsort.  Here every level is one segmented sort of all the
// splitting clusters' ranges:
//   1. gather: the level's ranges packed into one array of (key, index,
//      segment) records, key = the order-preserving 64-bit image of the
//      coordinate;
//   2. a stable least-significant-digit radix sort of the records, eight
//      8-bit passes on the key, then one or two passes on the segment (so the
//      ranges come out whole, each in coordinate order); every pass is a
//      block histogram, one scan over the [block][digit] counts and a
//      scatter that ranks equal digits of a warp with __match_any_sync in
//      position order;
//   3. scatter back into the permutation, the coordinates at the split
//      (offsets size / 2 - 1 and size / 2) per segment, and a scan for equal
//      neighbouring coordinates (compared as doubles, as std::sort's
//      comparator does; NaN counts as equal).  Any equal pair sends the
//      whole tree back to the host build.
// Bounding boxes, shrinking and numbering stay on the host (h2_plan.cpp):
// they are O(clusters) once the splits are known, plus one pass over the
// points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "h2_gpu.h"

namespace fmca {
namespace gpu {
namespace {

constexpr int kRxThreads = 256;
constexpr int kRxWarps = kRxThreads / 32;
constexpr int kRxTile = 4096;                     // records per block
constexpr int kRxWarpItems = kRxTile / kRxWarps;  // 512 consecutive records per warp

__device__ __forceinline__ uint64_t ord_bits(double x) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

struct SegDev {
  uint32_t begin, size, cbeg;
  int coord;
};

// compact position p -> segment (binary search over the packed offsets)
__device__ __forceinline__ int seg_of(const SegDev* segs, int m, uint32_t p) {
  int lo = 0, hi = m - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].cbeg <= p)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void gather_records_kernel(const SegDev* __restrict__ segs, int m, uint32_t total,
                                      const uint32_t* __restrict__ idx,
                                      const double* __restrict__ P, int dim,
                                      uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                      uint32_t* __restrict__ sid) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += gridDim.x * blockDim.x) {
    const int s = seg_of(segs, m, p);
    const SegDev sg = segs[s];
    const uint32_t v = idx[sg.begin + (p - sg.cbeg)];
    keys[p] = ord_bits(P[(size_t)v * dim + sg.coord]);
    vals[p] = v;
    sid[p] = (uint32_t)s;
  }
}

__device__ __forceinline__ uint32_t rx_digit(const uint64_t* keys, const uint32_t* sid, uint32_t p,
                                             int shift, int on_seg) {
  return on_seg ? (sid[p] >> shift) & 255u : (uint32_t)(keys[p] >> shift) & 255u;
}

// hist[b * 256 + d] = records of block b with digit d
__global__ void rx_hist_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ sid,
                               uint32_t n, int shift, int on_seg, uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  const uint32_t b0 = blockIdx.x * (uint32_t)kRxTile;
  const uint32_t b1 = min(n, b0 + (uint32_t)kRxTile);
  for (uint32_t p = b0 + threadIdx.x; p < b1; p += blockDim.x)
    atomicAdd(&cnt[rx_digit(keys, sid, p, shift, on_seg)], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(size_t)blockIdx.x * 256 + d] = cnt[d];
}

// in place: hist[b * 256 + d] = (records of digits < d in all blocks) +
// (records of digit d in blocks < b), the start of block b's digit-d
// records after the pass.  One block of 256 threads, thread d walks its
// digit over the blocks (consecutive threads read consecutive words).
__global__ void rx_scan_kernel(uint32_t* __restrict__ hist, int nblocks) {
  __shared__ uint32_t base[256];
  const int d = threadIdx.x;
  uint32_t run = 0;
  for (int b = 0; b < nblocks; ++b) {
    const uint32_t c = hist[(size_t)b * 256 + d];
    hist[(size_t)b * 256 + d] = run;
    run += c;
  }
  base[d] = run;
  __syncthreads();
  // exclusive scan of the digit totals (Hillis-Steele over 256 entries)
  for (int o = 1; o < 256; o <<= 1) {
    const uint32_t v = d >= o ? base[d - o] : 0u;
    __syncthreads();
    base[d] += v;
    __syncthreads();
  }
  const uint32_t off = base[d] - run;
  for (int b = 0; b < nblocks; ++b) hist[(size_t)b * 256 + d] += off;
}

// stable scatter of one radix pass: records of block b with digit d go to
// offs[b * 256 + d] + their rank among the block's digit-d records in
// position order (warps own consecutive runs of 512 records; in every round
// of 32 the lanes with equal digits rank by __match_any_sync)
__global__ void rx_scatter_kernel(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                  const uint32_t* __restrict__ sin, uint64_t* __restrict__ kout,
                                  uint32_t* __restrict__ vout, uint32_t* __restrict__ sout,
                                  uint32_t n, const uint32_t* __restrict__ offs, int shift,
                                  int on_seg) {
  __shared__ uint32_t cnt[kRxWarps][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < kRxWarps * 256; i += blockDim.x) (&cnt[0][0])[i] = 0u;
  __syncthreads();
  const uint32_t base = blockIdx.x * (uint32_t)kRxTile + (uint32_t)warp * kRxWarpItems;
  for (int r = 0; r < kRxWarpItems / 32; ++r) {
    const uint32_t p = base + (uint32_t)(r * 32 + lane);
    const bool valid = p < n;
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      const uint32_t d = rx_digit(kin, sin, p, shift, on_seg);
      const unsigned peers = __match_any_sync(act, d);
      if (lane == __ffs(peers) - 1) cnt[warp][d] += __popc(peers);
    }
    __syncwarp();
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) {
    uint32_t run = 0;
    for (int w = 0; w < kRxWarps; ++w) {
      const uint32_t c = cnt[w][d];
      cnt[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  for (int r = 0; r < kRxWarpItems / 32; ++r) {
    const uint32_t p = base + (uint32_t)(r * 32 + lane);
    const bool valid = p < n;
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    uint32_t d = 0;
    unsigned peers = 0;
    if (valid) {
      d = rx_digit(kin, sin, p, shift, on_seg);
      peers = __match_any_sync(act, d);
      const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
      const uint32_t dst = offs[(size_t)blockIdx.x * 256 + d] + cnt[warp][d] + rank;
      kout[dst] = kin[p];
      vout[dst] = vin[p];
      sout[dst] = sin[p];
    }
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) cnt[warp][d] += __popc(peers);
    __syncwarp();
  }
}

// sorted records back into the permutation; per segment the coordinates at
// the split; a flag for equal (or NaN) neighbouring coordinates
__global__ void scatter_back_kernel(const SegDev* __restrict__ segs, uint32_t total,
                                    const uint32_t* __restrict__ vals,
                                    const uint32_t* __restrict__ sid,
                                    const double* __restrict__ P, int dim,
                                    uint32_t* __restrict__ idx, int* __restrict__ ties) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += gridDim.x * blockDim.x) {
    const SegDev sg = segs[sid[p]];
    const uint32_t v = vals[p];
    idx[sg.begin + (p - sg.cbeg)] = v;
    const double c = P[(size_t)v * dim + sg.coord];
    bool tie = !(c == c);
    if (p > sg.cbeg) tie = tie || c == P[(size_t)vals[p - 1] * dim + sg.coord];
    if (tie) atomicExch(ties, 1);
  }
}

__global__ void split_values_kernel(const SegDev* __restrict__ segs, int m,
                                    const uint32_t* __restrict__ vals,
                                    const double* __restrict__ P, int dim,
                                    double* __restrict__ cut) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m; s += gridDim.x * blockDim.x) {
    const SegDev sg = segs[s];
    const uint32_t h = sg.cbeg + sg.size / 2;
    cut[2 * s] = P[(size_t)vals[h - 1] * dim + sg.coord];
    cut[2 * s + 1] = P[(size_t)vals[h] * dim + sg.coord];
  }
}

// Stable LSD radix sort of (key, val, sid) records on one stream: ping-pong
// buffers of a fixed capacity; sort() runs 8-bit passes over the low
// key_bits of the key, then over the low sid_bits of sid, and leaves the
// sorted records in buffer cur.
struct RecordSort {
  cudaStream_t st = nullptr;
  size_t cap = 0;
  uint64_t* k[2] = {nullptr, nullptr};
  uint32_t* v[2] = {nullptr, nullptr};
  uint32_t* s[2] = {nullptr, nullptr};
  uint32_t* hist = nullptr;
  int cur = 0;

  void release() {
    for (int b = 0; b < 2; ++b) {
      cudaFree(k[b]);
      cudaFree(v[b]);
      cudaFree(s[b]);
      k[b] = nullptr;
      v[b] = nullptr;
      s[b] = nullptr;
    }
    cudaFree(hist);
    hist = nullptr;
    cap = 0;
  }
  // capacity for n records (buffer cur keeps its first `keep` records)
  bool reserve(size_t n, size_t keep = 0) {
    if (n <= cap) return true;
    size_t nc = std::max<size_t>(n, cap * 2);
    uint64_t* nk[2] = {nullptr, nullptr};
    uint32_t* nv[2] = {nullptr, nullptr};
    uint32_t* ns[2] = {nullptr, nullptr};
    uint32_t* nh = nullptr;
    bool ok = true;
    for (int b = 0; b < 2; ++b)
      ok = ok && cudaMalloc(&nk[b], nc * 8) == cudaSuccess &&
           cudaMalloc(&nv[b], nc * 4) == cudaSuccess && cudaMalloc(&ns[b], nc * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&nh, (size_t)256 * 4 * ((nc + kRxTile - 1) / kRxTile + 1)) == cudaSuccess;
    if (ok && keep)
      ok = cudaMemcpyAsync(nk[0], k[cur], keep * 8, cudaMemcpyDeviceToDevice, st) == cudaSuccess &&
           cudaMemcpyAsync(nv[0], v[cur], keep * 4, cudaMemcpyDeviceToDevice, st) == cudaSuccess &&
           cudaMemcpyAsync(ns[0], s[cur], keep * 4, cudaMemcpyDeviceToDevice, st) == cudaSuccess &&
           cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) {
      for (int b = 0; b < 2; ++b) {
        cudaFree(nk[b]);
        cudaFree(nv[b]);
        cudaFree(ns[b]);
      }
      cudaFree(nh);
      return false;
    }
    release();
    for (int b = 0; b < 2; ++b) {
      k[b] = nk[b];
      v[b] = nv[b];
      s[b] = ns[b];
    }
    hist = nh;
    cap = nc;
    cur = 0;
    return true;
  }
  void sort(uint32_t n, int key_bits, int sid_bits) {
    if (n == 0) return;
    const int nb = (int)((n + kRxTile - 1) / kRxTile);
    auto pass = [&](int shift, int on_seg) {
      rx_hist_kernel<<<nb, kRxThreads, 0, st>>>(k[cur], s[cur], n, shift, on_seg, hist);
      rx_scan_kernel<<<1, 256, 0, st>>>(hist, nb);
      rx_scatter_kernel<<<nb, kRxThreads, 0, st>>>(k[cur], v[cur], s[cur], k[cur ^ 1], v[cur ^ 1],
                                                   s[cur ^ 1], n, hist, shift, on_seg);
      cur ^= 1;
    };
    for (int shift = 0; shift < key_bits; shift += 8) pass(shift, 0);
    for (int shift = 0; shift < sid_bits; shift += 8) pass(shift, 1);
  }
};

class GpuLevelSorter final : public LevelSorter {
 public:
  GpuLevelSorter() = default;
  GpuLevelSorter(const GpuLevelSorter&) = delete;
  GpuLevelSorter& operator=(const GpuLevelSorter&) = delete;
  ~GpuLevelSorter() override {
    if (st_) cudaStreamSynchronize(st_);
    for (void* p : bufs_) cudaFree(p);
    if (segdev_) cudaFree(segdev_);
    if (cut_) cudaFree(cut_);
    rs_.release();
    if (st_) cudaStreamDestroy(st_);
  }

  bool start(const double* P, int dim, uint32_t n) override {
    dim_ = dim;
    n_ = n;
    if (cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking) != cudaSuccess) return false;
    rs_.st = st_;
    if (!alloc(&P_, (size_t)dim * n) || !alloc(&idx_, n) || !alloc(&ties_, 1) ||
        !rs_.reserve(std::max<uint32_t>(1, n)))
      return false;
    std::vector<uint32_t> iota(n);
    for (uint32_t i = 0; i < n; ++i) iota[i] = i;
    return cudaMemcpyAsync(P_, P, sizeof(double) * dim * n, cudaMemcpyHostToDevice, st_) ==
               cudaSuccess &&
           cudaMemcpyAsync(idx_, iota.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice,
                           st_) == cudaSuccess &&
           cudaStreamSynchronize(st_) == cudaSuccess;
  }

  bool sort_level(const std::vector<SortSegment>& segs, std::vector<double>* cut,
                  bool* ties) override {
    const int m = (int)segs.size();
    std::vector<SegDev> hs(m);
    uint32_t total = 0;
    for (int i = 0; i < m; ++i) {
      hs[i] = SegDev{segs[i].begin, segs[i].size, total, segs[i].coord};
      total += segs[i].size;
    }
    if (m == 0 || total == 0) {
      cut->assign(2 * (size_t)m, 0.);
      *ties = false;
      return true;
    }
    if ((size_t)m > seg_cap_) {
      if (segdev_) cudaFree(segdev_);
      if (cut_) cudaFree(cut_);
      segdev_ = nullptr;
      cut_ = nullptr;
      seg_cap_ = 0;
      if (cudaMalloc(&segdev_, sizeof(SegDev) * m) != cudaSuccess ||
          cudaMalloc(&cut_, sizeof(double) * 2 * m) != cudaSuccess)
        return false;
      seg_cap_ = m;
    }
    const int grid = std::min<int>(4096, (int)((total + 255) / 256));
    bool ok = cudaMemcpyAsync(segdev_, hs.data(), sizeof(SegDev) * m, cudaMemcpyHostToDevice,
                              st_) == cudaSuccess &&
              cudaMemsetAsync(ties_, 0, sizeof(int), st_) == cudaSuccess;
    if (!ok) return false;
    rs_.cur = 0;
    gather_records_kernel<<<grid, 256, 0, st_>>>(segdev_, m, total, idx_, P_, dim_, rs_.k[0],
                                                 rs_.v[0], rs_.s[0]);
    int sid_bits = 0;
    while (m > 1 && ((uint32_t)(m - 1) >> sid_bits) != 0) sid_bits += 8;
    rs_.sort(total, 64, sid_bits);
    const int c = rs_.cur;
    scatter_back_kernel<<<grid, 256, 0, st_>>>(segdev_, total, rs_.v[c], rs_.s[c], P_, dim_,
                                               idx_, ties_);
    split_values_kernel<<<(m + 255) / 256, 256, 0, st_>>>(segdev_, m, rs_.v[c], P_, dim_, cut_);
    if (cudaGetLastError() != cudaSuccess) return false;
    cut->resize(2 * (size_t)m);
    int t = 0;
    ok = cudaMemcpyAsync(cut->data(), cut_, sizeof(double) * 2 * m, cudaMemcpyDeviceToHost,
                         st_) == cudaSuccess &&
         cudaMemcpyAsync(&t, ties_, sizeof(int), cudaMemcpyDeviceToHost, st_) == cudaSuccess &&
         cudaStreamSynchronize(st_) == cudaSuccess;
    *ties = t != 0;
    return ok;
  }

  bool finish(std::vector<uint32_t>* perm) override {
    perm->resize(n_);
    return cudaMemcpyAsync(perm->data(), idx_, sizeof(uint32_t) * n_, cudaMemcpyDeviceToHost,
                           st_) == cudaSuccess &&
           cudaStreamSynchronize(st_) == cudaSuccess;
  }

 private:
  template <typename V>
  bool alloc(V** p, size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(1, count) * sizeof(V)) != cudaSuccess) return false;
    bufs_.push_back(q);
    *p = static_cast<V*>(q);
    return true;
  }

  int dim_ = 0;
  uint32_t n_ = 0;
  cudaStream_t st_ = nullptr;
  std::vector<void*> bufs_;
  double* P_ = nullptr;
  uint32_t* idx_ = nullptr;
  RecordSort rs_;
  int* ties_ = nullptr;
  SegDev* segdev_ = nullptr;
  double* cut_ = nullptr;
  size_t seg_cap_ = 0;
};

// ---------------------------------------------------------------------------
// Block pattern (H2MatrixBase::computePattern, H2MatrixBase.h:160-191) level
// by level: every pair of the current level is compared
// (Admissibility.h:19-29,95-115, in the reference's FP64 operation order
// with rounded operations only, so that every decision equals the host's)
// and becomes a far leaf (low-rank and cheaper than dense, 32-bit unsigned
// products like the reference's Index), a near leaf, or four son pairs of
// the next level.  Every pair carries its path from the root, two bits per
// level: the rank of the son pair in the order the reference's stack pops
// them (the last pushed, sons (1, 1), first).  Sorting the leaves by the
// left-aligned path gives exactly the order of the depth-first recursion.
struct TreeDev {
  const double *bbmin, *bbmax, *radius;
  const uint32_t* size;
  const int32_t *son0, *nsons;
};

struct PairList {
  uint64_t* key;
  int32_t *i, *j;
};

__global__ void pattern_level_kernel(const uint64_t* __restrict__ fkey,
                                     const int32_t* __restrict__ fi,
                                     const int32_t* __restrict__ fj, uint32_t nf, int depth,
                                     TreeDev R, TreeDev Cl, int dim, double eta, uint32_t qq,
                                     PairList far, PairList near, PairList next,
                                     unsigned int* __restrict__ counts) {
  for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
    const int i = fi[f], j = fj[f];
    const uint64_t key = fkey[f];
    double s2 = 0.0;
    for (int d = 0; d < dim; ++d) {
      double a = __dsub_rn(R.bbmin[(size_t)i * dim + d], Cl.bbmin[(size_t)j * dim + d]);
      a = __dadd_rn(a, R.bbmax[(size_t)i * dim + d]);
      a = __dsub_rn(a, Cl.bbmax[(size_t)j * dim + d]);
      const double v = __dmul_rn(0.5, a);
      const double sq = __dmul_rn(v, v);
      s2 = d == 0 ? sq : __dadd_rn(s2, sq);
    }
    const double r1 = R.radius[i], r2 = Cl.radius[j];
    double dist = __dsub_rn(__dsub_rn(__dsqrt_rn(s2), r1), r2);
    dist = dist > 0 ? dist : 0;
    const double radius = r1 > r2 ? r1 : r2;
    if (radius > __dmul_rn(eta, dist)) {
      const int ni = R.nsons[i], nj = Cl.nsons[j];
      if (!ni || !nj) {
        const unsigned int o = atomicAdd(&counts[1], 1u);
        near.key[o] = key;
        near.i[o] = i;
        near.j[o] = j;
      } else {
        const unsigned int o = atomicAdd(&counts[2], (unsigned int)(ni * nj));
        const int shift = 62 - 2 * depth;
        for (int b = 0; b < nj; ++b)
          for (int a = 0; a < ni; ++a) {
            const int t = b * ni + a;  // push index
            const uint64_t rank = (uint64_t)(ni * nj - 1 - t);
            next.key[o + t] = key | (rank << shift);
            next.i[o + t] = R.son0[i] + a;
            next.j[o + t] = Cl.son0[j] + b;
          }
      }
    } else {
      const uint32_t dense = R.size[i] * Cl.size[j];
      const int which = qq < dense ? 0 : 1;
      const unsigned int o = atomicAdd(&counts[which], 1u);
      PairList& out = which ? near : far;
      out.key[o] = key;
      out.i[o] = i;
      out.j[o] = j;
    }
  }
}

// leaves packed as sort records (key, i, j)
__global__ void pack_leaves_kernel(const uint64_t* __restrict__ key, const int32_t* __restrict__ i,
                                   const int32_t* __restrict__ j, uint32_t n,
                                   uint64_t* __restrict__ k, uint32_t* __restrict__ v,
                                   uint32_t* __restrict__ s) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    k[p] = key[p];
    v[p] = (uint32_t)i[p];
    s[p] = (uint32_t)j[p];
  }
}

// device buffer of one array type with a host-side capacity
template <typename V>
struct DevBuf {
  V* p = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { cudaFree(p); }
  void swap(DevBuf& o) {
    std::swap(p, o.p);
    std::swap(cap, o.cap);
  }
  // grows to n elements, keeping the first `keep`
  bool reserve(size_t n, size_t keep, cudaStream_t st) {
    if (n <= cap) return true;
    const size_t nc = std::max(n, cap * 2);
    V* q = nullptr;
    if (cudaMalloc(&q, nc * sizeof(V)) != cudaSuccess) return false;
    if (keep && (cudaMemcpyAsync(q, p, keep * sizeof(V), cudaMemcpyDeviceToDevice, st) !=
                     cudaSuccess ||
                 cudaStreamSynchronize(st) != cudaSuccess)) {
      cudaFree(q);
      return false;
    }
    cudaFree(p);
    p = q;
    cap = nc;
    return true;
  }
};

struct PairBufs {
  DevBuf<uint64_t> key;
  DevBuf<int32_t> i, j;
  bool reserve(size_t n, size_t keep, cudaStream_t st) {
    return key.reserve(n, keep, st) && i.reserve(n, keep, st) && j.reserve(n, keep, st);
  }
  PairList list() { return PairList{key.p, i.p, j.p}; }
  void swap(PairBufs& o) {
    key.swap(o.key);
    i.swap(o.i);
    j.swap(o.j);
  }
};

class GpuPatternBuilder final : public PatternBuilder {
 public:
  GpuPatternBuilder() = default;
  GpuPatternBuilder(const GpuPatternBuilder&) = delete;
  GpuPatternBuilder& operator=(const GpuPatternBuilder&) = delete;
  ~GpuPatternBuilder() override {
    if (st_) cudaStreamSynchronize(st_);
    for (void* p : bufs_) cudaFree(p);
    rs_.release();
    if (st_) cudaStreamDestroy(st_);
  }

  bool build(const Tree& rows, const Tree& cols, uint32_t qq, double eta,
             std::vector<int32_t>* far_row, std::vector<int32_t>* far_col,
             std::vector<int32_t>* near_row, std::vector<int32_t>* near_col) override {
    const int dim = rows.dim;
    if (cols.dim != dim || rows.nclusters() < 1 || cols.nclusters() < 1) return false;
    // binary trees of at most 32 levels: two bits of path per level
    for (const Tree* t : {&rows, &cols}) {
      if (t->nlevels() > 32) return false;
      for (int32_t ns : t->nsons)
        if (ns != 0 && ns != 2) return false;
    }
    if (!st_) {
      if (cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking) != cudaSuccess) return false;
      rs_.st = st_;
    }
    TreeDev R, Cl;
    if (!upload_tree(rows, &R) || !upload_tree(cols, &Cl)) return false;
    unsigned int* counts = nullptr;
    if (!alloc(&counts, 3)) return false;
    PairBufs cur, nxt, far, near;
    const uint64_t zero = 0;
    const int32_t root = 0;
    if (!cur.reserve(1, 0, st_) ||
        cudaMemcpyAsync(cur.key.p, &zero, 8, cudaMemcpyHostToDevice, st_) != cudaSuccess ||
        cudaMemcpyAsync(cur.i.p, &root, 4, cudaMemcpyHostToDevice, st_) != cudaSuccess ||
        cudaMemcpyAsync(cur.j.p, &root, 4, cudaMemcpyHostToDevice, st_) != cudaSuccess)
      return false;
    unsigned int h[3] = {0, 0, 0};
    uint32_t nf = 1;
    for (int depth = 0; nf > 0; ++depth) {
      if (depth > 31) return false;
      if (!far.reserve((size_t)h[0] + nf, h[0], st_) ||
          !near.reserve((size_t)h[1] + nf, h[1], st_) || !nxt.reserve((size_t)4 * nf, 0, st_))
        return false;
      unsigned int c3[3] = {h[0], h[1], 0};
      if (cudaMemcpyAsync(counts, c3, sizeof(c3), cudaMemcpyHostToDevice, st_) != cudaSuccess)
        return false;
      const int grid = (int)std::min<uint32_t>(4096, (nf + 255) / 256);
      pattern_level_kernel<<<grid, 256, 0, st_>>>(cur.key.p, cur.i.p, cur.j.p, nf, depth, R, Cl,
                                                  dim, eta, qq, far.list(), near.list(),
                                                  nxt.list(), counts);
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, st_) != cudaSuccess ||
          cudaStreamSynchronize(st_) != cudaSuccess)
        return false;
      nf = h[2];
      cur.swap(nxt);
    }
    return sorted(far, h[0], far_row, far_col) && sorted(near, h[1], near_row, near_col);
  }

 private:
  // the leaves in depth-first order: sorted by their left-aligned paths
  bool sorted(PairBufs& b, uint32_t n, std::vector<int32_t>* ri, std::vector<int32_t>* rj) {
    ri->resize(n);
    rj->resize(n);
    if (n == 0) return true;
    if (!rs_.reserve(n)) return false;
    rs_.cur = 0;
    const int grid = (int)std::min<uint32_t>(4096, (n + 255) / 256);
    pack_leaves_kernel<<<grid, 256, 0, st_>>>(b.key.p, b.i.p, b.j.p, n, rs_.k[0], rs_.v[0],
                                              rs_.s[0]);
    rs_.sort(n, 64, 0);
    return cudaGetLastError() == cudaSuccess &&
           cudaMemcpyAsync(ri->data(), rs_.v[rs_.cur], 4 * (size_t)n, cudaMemcpyDeviceToHost,
                           st_) == cudaSuccess &&
           cudaMemcpyAsync(rj->data(), rs_.s[rs_.cur], 4 * (size_t)n, cudaMemcpyDeviceToHost,
                           st_) == cudaSuccess &&
           cudaStreamSynchronize(st_) == cudaSuccess;
  }

  bool upload_tree(const Tree& t, TreeDev* d) {
    const int C = t.nclusters(), dim = t.dim;
    // cluster radii as the host compare forms them: 0.5 * |extent|, the
    // squares summed in dimension order
    std::vector<double> rad(C);
    for (int c = 0; c < C; ++c) {
      const double* e = t.bbext.data() + (size_t)c * dim;
      double s2 = e[0] * e[0];
      for (int k = 1; k < dim; ++k) s2 += e[k] * e[k];
      rad[c] = 0.5 * std::sqrt(s2);
    }
    double *bmin, *bmax, *r;
    uint32_t* sz;
    int32_t *s0, *ns;
    if (!put(&bmin, t.bbmin) || !put(&bmax, t.bbmax) || !put(&r, rad) || !put(&sz, t.size) ||
        !put(&s0, t.son0) || !put(&ns, t.nsons))
      return false;
    *d = TreeDev{bmin, bmax, r, sz, s0, ns};
    return true;
  }
  template <typename V>
  bool alloc(V** p, size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(1, count) * sizeof(V)) != cudaSuccess) return false;
    bufs_.push_back(q);
    *p = static_cast<V*>(q);
    return true;
  }
  template <typename V>
  bool put(V** p, const std::vector<V>& h) {
    return alloc(p, h.size()) &&
           cudaMemcpyAsync(*p, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice, st_) ==
               cudaSuccess;
  }

  cudaStream_t st_ = nullptr;
  std::vector<void*> bufs_;
  RecordSort rs_;
};

}  // namespace

std::unique_ptr<LevelSorter> make_gpu_level_sorter() {
  return std::unique_ptr<LevelSorter>(new GpuLevelSorter());
}

std::unique_ptr<PatternBuilder> make_gpu_pattern_builder() {
  return std::unique_ptr<PatternBuilder>(new GpuPatternBuilder());
}

}  // namespace gpu
}  // namespace fmca
