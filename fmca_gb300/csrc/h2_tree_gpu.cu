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
//      block histogram, one scan over [digit][block] and a scatter that ranks
//      equal digits of a warp with __match_any_sync in position order;
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

// hist[d * nblocks + b] = records of block b with digit d
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
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(size_t)d * gridDim.x + blockIdx.x] = cnt[d];
}

// exclusive scan of len entries in place, one block of 1024 threads
__global__ void rx_scan_kernel(uint32_t* __restrict__ a, uint32_t len) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (len + blockDim.x - 1) / blockDim.x;
  const uint32_t b0 = threadIdx.x * per, b1 = min(len, b0 + per);
  uint32_t s = 0;
  for (uint32_t i = b0; i < b1; ++i) s += a[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const uint32_t v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - s;  // exclusive prefix of this thread's chunk
  for (uint32_t i = b0; i < b1; ++i) {
    const uint32_t v = a[i];
    a[i] = run;
    run += v;
  }
}

// stable scatter of one radix pass: records of block b with digit d go to
// offs[d * nblocks + b] + their rank among the block's digit-d records in
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
      const uint32_t dst = offs[(size_t)d * gridDim.x + blockIdx.x] + cnt[warp][d] + rank;
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
    if (st_) cudaStreamDestroy(st_);
  }

  bool start(const double* P, int dim, uint32_t n) override {
    dim_ = dim;
    n_ = n;
    if (cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking) != cudaSuccess) return false;
    const uint32_t nb = std::max<uint32_t>(1, (n + kRxTile - 1) / kRxTile);
    if (!alloc(&P_, (size_t)dim * n) || !alloc(&idx_, n) || !alloc(&k_[0], n) ||
        !alloc(&k_[1], n) || !alloc(&v_[0], n) || !alloc(&v_[1], n) || !alloc(&s_[0], n) ||
        !alloc(&s_[1], n) || !alloc(&hist_, (size_t)256 * nb) || !alloc(&ties_, 1))
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
    const int nb = (int)((total + kRxTile - 1) / kRxTile);
    const int grid = std::min<int>(4096, (int)((total + 255) / 256));
    bool ok = cudaMemcpyAsync(segdev_, hs.data(), sizeof(SegDev) * m, cudaMemcpyHostToDevice,
                              st_) == cudaSuccess &&
              cudaMemsetAsync(ties_, 0, sizeof(int), st_) == cudaSuccess;
    if (!ok) return false;
    gather_records_kernel<<<grid, 256, 0, st_>>>(segdev_, m, total, idx_, P_, dim_, k_[0], v_[0],
                                                 s_[0]);
    int cur = 0;
    auto pass = [&](int shift, int on_seg) {
      rx_hist_kernel<<<nb, kRxThreads, 0, st_>>>(k_[cur], s_[cur], total, shift, on_seg, hist_);
      rx_scan_kernel<<<1, 1024, 0, st_>>>(hist_, (uint32_t)(256 * nb));
      rx_scatter_kernel<<<nb, kRxThreads, 0, st_>>>(k_[cur], v_[cur], s_[cur], k_[cur ^ 1],
                                                    v_[cur ^ 1], s_[cur ^ 1], total, hist_, shift,
                                                    on_seg);
      cur ^= 1;
    };
    for (int shift = 0; shift < 64; shift += 8) pass(shift, 0);
    for (int shift = 0; m > 1 && ((uint32_t)(m - 1) >> shift) != 0; shift += 8) pass(shift, 1);
    scatter_back_kernel<<<grid, 256, 0, st_>>>(segdev_, total, v_[cur], s_[cur], P_, dim_, idx_,
                                               ties_);
    split_values_kernel<<<(m + 255) / 256, 256, 0, st_>>>(segdev_, m, v_[cur], P_, dim_, cut_);
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
  uint64_t* k_[2] = {nullptr, nullptr};
  uint32_t* v_[2] = {nullptr, nullptr};
  uint32_t* s_[2] = {nullptr, nullptr};
  uint32_t* hist_ = nullptr;
  int* ties_ = nullptr;
  SegDev* segdev_ = nullptr;
  double* cut_ = nullptr;
  size_t seg_cap_ = 0;
};

}  // namespace

std::unique_ptr<LevelSorter> make_gpu_level_sorter() {
  return std::unique_ptr<LevelSorter>(new GpuLevelSorter());
}

}  // namespace gpu
}  // namespace fmca
