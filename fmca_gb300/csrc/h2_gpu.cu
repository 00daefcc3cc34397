// Device plan and matvec driver.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

#include "../../include/fmca_gb300.h"
#include "h2_gpu.h"
#include "h2_adjoint_kernels.cuh"
#include "h2_assembled.h"
#include "h2_far_kron.h"
#include "near_pack.h"
#include "h2_gpu_kernels.cuh"
#include "h2_tc_kernels.cuh"
#include "h2_umma_kernels.cuh"
#include "h2_umma_persistent.h"

namespace fmca {
namespace gpu {

namespace {

#define FMCA_CK(expr)                                                        \
  do {                                                                       \
    cudaError_t e_ = (expr);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      *err = std::string(#expr) + " failed: " + cudaGetErrorString(e_);     \
      return e_ == cudaErrorMemoryAllocation ? FMCA_ERR_OUT_OF_MEMORY        \
                                             : FMCA_ERR_CUDA;                \
    }                                                                        \
  } while (0)

constexpr int kGroupCap = 256;    // targets per ksum CTA (128 threads x 2)
constexpr int kTcGroupCap = 128;  // targets per far-field tensor-core CTA
constexpr int kStages = 3;
template <typename T>
struct TileSize;
template <>
struct TileSize<double> {
  static constexpr int value = 64;
};
template <>
struct TileSize<float> {
  static constexpr int value = 128;
};

template <typename T>
struct DevSet {
  bool ready = false;
  Pt4<T>* pts_r = nullptr;
  Pt4<T>* pts_c = nullptr;
  Pt4<T>* nodes_r = nullptr;
  Pt4<T>* nodes_c = nullptr;
  T* bbmin_r = nullptr;
  T* bbext_r = nullptr;
  T* bbmin_c = nullptr;
  T* bbext_c = nullptr;
  T* E_r = nullptr;
  T* E_c = nullptr;
  T* to_nodal = nullptr;    // total degree: invV^T (row-major q x q)
  T* from_nodal = nullptr;  // total degree: invV
  InterpDev<T> ip;
  // centre of the box of both point clouds (the near field's dot-product
  // distance form measures coordinates from it)
  float ctr[3] = {0.f, 0.f, 0.f};
};

// midpoint of the bounding box of the row and column points (dim <= 3)
void cloud_centre(const Plan& plan, float ctr[3]) {
  const int dim = plan.interp.dim;
  for (int d = 0; d < 3; ++d) {
    double lo = 0, hi = 0;
    bool any = false;
    for (const std::vector<double>* P : {&plan.points_r, &plan.points_c}) {
      for (size_t i = 0; d < dim && i + dim <= P->size(); i += dim) {
        const double v = (*P)[i + d];
        if (!std::isfinite(v)) continue;
        if (!any || v < lo) lo = v;
        if (!any || v > hi) hi = v;
        any = true;
      }
    }
    ctr[d] = any ? (float)(0.5 * (lo + hi)) : 0.f;
  }
}

struct GroupList {
  KGroup* groups = nullptr;
  uint32_t* ivl = nullptr;
  // per interval: target halves it serves (paired grid lists), or the leaves
  // it serves (packed near lists)
  uint32_t* imask = nullptr;
  uint32_t* split = nullptr;  // packed near lists: rows of a group's first leaf
  int ngroups = 0;
  int maxcount = 0;
};

// Launch shapes of the kernel sums (stages of the copy ring, tiles per
// accumulation unit).
struct UmCfg {
  int nst, F;
  int persist = 0;  // 1: one CTA per SM running groups in turn; 0: one CTA per group
};
// Transfer level thresholds (cluster counts): levels with fewer than
// wide_below clusters run the sum-factorised transfer with 8 warps per
// cluster, levels with fewer than slice_below clusters split the
// right-hand sides over blockIdx.y in slices of 8.
struct TrCfg {
  int wide_below, slice_below;
};
// Every launch-shape choice of one matvec: the defaults (measured fastest at
// n = 1e6, 3-D, p = 4, 32 right-hand sides) or what the autotuner measured
// fastest on a plan for one (precision, kernel, right-hand sides) key.
struct TuneCfg {
  UmCfg near{um_stages(2), 2};       // near field
  int near_halves = 2;  // near field: target groups of two halves (256) or one (128)
  UmCfg far_grid{um_stages(2), 2};   // far field on sibling-paired tensor grids
  UmCfg far_nodes{um_stages(1), 1};  // far field on interpolation nodes
  int far_pairs = 1;  // 3-D plans of degree kGridP1 - 1: paired grids (1) or nodes (0)
  TrCfg tr{4 * 152, 2 * 152};
  int small_tc = 0;   // mixed precision, nrhs <= 16: tensor cores (1) or FP32 CUDA cores (0)
  // tensor-core path, GAUSSIAN on tensor-product nodes: the far field as
  // Kronecker products on the CUDA cores (1) or the tensor-core kernel sum (0)
  int far_kron = 1;
  // near field with one half: target rows of up to two leaves per group
  // over the union of their sources (1), or one leaf per group (0)
  int near_pack = 0;
  int tuned = 0;      // 1 if the autotuner chose these values
  float tune_ms = 0;  // time the tuning took
  static TuneCfg defaults(int sms) {
    TuneCfg c;
    c.tr = TrCfg{4 * sms, 2 * sms};
    return c;
  }
};

// Stored far- and near-field blocks of an assembled plan
// (fmca_plan_assemble): FP64 values for FMCA_PREC_FP64, FP32 values
// otherwise, one block per group of the CUDA-core group lists dp->far and
// dp->near at the per-group element offsets far_off / near_off.
struct AsmStore {
  int precision = -1;  // -1: not assembled
  KernelDesc k{};
  void* far = nullptr;
  void* near = nullptr;
  uint64_t* far_off = nullptr;
  uint64_t* near_off = nullptr;
  size_t bytes = 0;  // device bytes of the four arrays
};

void release_store(AsmStore* a) {
  for (void* p : {a->far, a->near, (void*)a->far_off, (void*)a->near_off})
    if (p) cudaFree(p);
  *a = AsmStore();
}

}  // namespace

struct DevPlan {
  int device = -1;
  int sms = 152;  // multiprocessors of the device (read at upload)
  std::vector<void*> allocs;
  size_t alloc_bytes = 0;  // sum of the sizes of allocs
  // launch shapes of the current call, and those the autotuner chose per
  // (precision, kernel, right-hand sides) key
  TuneCfg cfg;
  bool autotune = false;
  std::map<uint64_t, TuneCfg> tuned;
  int64_t tunings = 0;  // tuning runs on this plan
  DevSet<double> d;
  DevSet<float> f;
  int* midx = nullptr;
  uint32_t* perm_r = nullptr;
  uint32_t* perm_c = nullptr;
  uint32_t *cbegin_r = nullptr, *csize_r = nullptr;
  uint32_t *cbegin_c = nullptr, *csize_c = nullptr;
  int32_t *son0_c = nullptr, *nsons_c = nullptr, *parent_r = nullptr;
  int32_t *leaves_r = nullptr, *leaves_c = nullptr;
  int nleaves_r = 0, nleaves_c = 0;
  int32_t* m2m_list = nullptr;  // col clusters with sons, by level
  std::vector<int> m2m_ptr;
  int32_t* l2l_list = nullptr;  // row clusters of level >= 1, by level
  std::vector<int> l2l_ptr;
  GroupList far, near;  // chunked to kGroupCap targets (near: also the tensor-core list)
  GroupList near_h1;    // near field chunked to kTcGroupCap targets (one target half)
  GroupList near_pk;    // near field, one target half, rows of up to two leaves per group
  float* gexp = nullptr;  // per far group and target half: the moment exponent E
  GroupList far_tc;     // chunked to kTcGroupCap targets
  GroupList far_grid2;  // tensor grids: sibling row clusters paired as two target halves
  int* err_flag = nullptr;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  AsmStore as;  // stored blocks of fmca_plan_assemble
  std::mutex mu;
  // options of the current call; stage profiling: events recorded at stage
  // boundaries of the last matvec
  CallOpts opts;
  bool profile = false;
  std::vector<cudaEvent_t> events;
  std::vector<int> event_stage;
  int nevents = 0;
  int64_t launches = 0;  // kernels launched by the last matvec
  void mark(int stage, cudaStream_t st) {
    if (!profile) return;
    if (nevents >= (int)events.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return;
      events.push_back(e);
      event_stage.push_back(0);
    }
    cudaEventRecord(events[nevents], st);
    event_stage[nevents] = stage;
    ++nevents;
  }
  void reset_marks() {
    nevents = 0;
    launches = 0;
  }
};

namespace {

template <typename V>
int to_device(DevPlan* dp, const V* host, size_t count, V** out,
              std::string* err) {
  *out = nullptr;
  if (count == 0) return FMCA_OK;
  void* p = nullptr;
  FMCA_CK(cudaMalloc(&p, count * sizeof(V)));
  dp->allocs.push_back(p);
  dp->alloc_bytes += count * sizeof(V);
  FMCA_CK(cudaMemcpy(p, host, count * sizeof(V), cudaMemcpyHostToDevice));
  *out = static_cast<V*>(p);
  return FMCA_OK;
}

#define FMCA_TRY(expr)            \
  do {                            \
    int s_ = (expr);              \
    if (s_ != FMCA_OK) return s_; \
  } while (0)

// Builds target groups for ksum.  Each entry of src_lists is the interval
// list of one logical target range [tb, tb + tc); ranges are chunked to at
// most kGroupCap targets; groups are ordered by decreasing work.
struct HostGroups {
  std::vector<KGroup> groups;
  std::vector<uint32_t> ivl;
  std::vector<uint32_t> imask;  // optional, one per interval
  int maxcount = 0;
};

void add_target_range(HostGroups* hg, uint32_t tb, uint32_t tc, int ib, int ie,
                      uint32_t cap) {
  for (uint32_t o = 0; o < tc; o += cap) {
    KGroup g;
    g.tbegin = tb + o;
    g.tcount = std::min<uint32_t>(cap, tc - o);
    g.ivl_begin = ib;
    g.ivl_end = ie;
    hg->groups.push_back(g);
    hg->maxcount = std::max<int>(hg->maxcount, (int)g.tcount);
  }
}

void sort_groups(HostGroups* hg) {
  std::vector<uint64_t> work(hg->groups.size());
  for (size_t i = 0; i < hg->groups.size(); ++i) {
    uint64_t s = 0;
    for (int k = hg->groups[i].ivl_begin; k < hg->groups[i].ivl_end; ++k)
      s += hg->ivl[2 * k + 1] - hg->ivl[2 * k];
    work[i] = s * hg->groups[i].tcount;
  }
  std::vector<size_t> order(hg->groups.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return work[a] > work[b]; });
  std::vector<KGroup> g2(hg->groups.size());
  for (size_t i = 0; i < order.size(); ++i) g2[i] = hg->groups[order[i]];
  hg->groups.swap(g2);
}

int upload_groups(DevPlan* dp, const HostGroups& hg, GroupList* gl,
                  std::string* err) {
  FMCA_TRY(to_device(dp, hg.groups.data(), hg.groups.size(), &gl->groups, err));
  FMCA_TRY(to_device(dp, hg.ivl.data(), hg.ivl.size(), &gl->ivl, err));
  if (!hg.imask.empty())
    FMCA_TRY(to_device(dp, hg.imask.data(), hg.imask.size(), &gl->imask, err));
  gl->ngroups = (int)hg.groups.size();
  gl->maxcount = hg.maxcount;
  return FMCA_OK;
}

template <typename T>
int upload_set(const Plan& plan, DevPlan* dp, DevSet<T>* s, std::string* err) {
  if (s->ready) return FMCA_OK;
  const int dim = plan.interp.dim, q = plan.interp.q;
  // points in cluster order
  auto make_pts = [&](const std::vector<double>& Pnat, const Tree& t,
                      std::vector<Pt4<T>>* out) {
    out->assign(t.n, Pt4<T>{T(0), T(0), T(0), T(0)});
    for (uint32_t i = 0; i < t.n; ++i) {
      const double* p = Pnat.data() + (size_t)t.perm[i] * dim;
      Pt4<T>& o = (*out)[i];
      o.x = (T)p[0];
      o.y = dim > 1 ? (T)p[1] : T(0);
      o.z = dim > 2 ? (T)p[2] : T(0);
      o.w = T(1);  // source weight of the tensor-core kernel sum
    }
  };
  auto make_nodes = [&](const std::vector<double>& nd, int C,
                        std::vector<Pt4<T>>* out) {
    out->assign((size_t)C * q, Pt4<T>{T(0), T(0), T(0), T(0)});
    for (size_t k = 0; k < (size_t)C * q; ++k) {
      (*out)[k].x = (T)nd[k * dim];
      (*out)[k].y = dim > 1 ? (T)nd[k * dim + 1] : T(0);
      (*out)[k].z = dim > 2 ? (T)nd[k * dim + 2] : T(0);
    }
  };
  auto make_bb = [&](const std::vector<double>& v, int C, std::vector<T>* out) {
    out->assign((size_t)C * 3, T(0));
    for (int c = 0; c < C; ++c)
      for (int d = 0; d < dim; ++d) (*out)[(size_t)c * 3 + d] = (T)v[(size_t)c * dim + d];
  };
  std::vector<Pt4<T>> hp;
  std::vector<T> hv;
  cloud_centre(plan, s->ctr);
  make_pts(plan.points_r, plan.rows, &hp);
  FMCA_TRY(to_device(dp, hp.data(), hp.size(), &s->pts_r, err));
  make_pts(plan.points_c, plan.cols, &hp);
  FMCA_TRY(to_device(dp, hp.data(), hp.size(), &s->pts_c, err));
  make_nodes(plan.row_nodes, plan.rows.nclusters(), &hp);
  FMCA_TRY(to_device(dp, hp.data(), hp.size(), &s->nodes_r, err));
  make_nodes(plan.col_nodes, plan.cols.nclusters(), &hp);
  FMCA_TRY(to_device(dp, hp.data(), hp.size(), &s->nodes_c, err));
  make_bb(plan.rows.bbmin, plan.rows.nclusters(), &hv);
  FMCA_TRY(to_device(dp, hv.data(), hv.size(), &s->bbmin_r, err));
  make_bb(plan.rows.bbext, plan.rows.nclusters(), &hv);
  FMCA_TRY(to_device(dp, hv.data(), hv.size(), &s->bbext_r, err));
  make_bb(plan.cols.bbmin, plan.cols.nclusters(), &hv);
  FMCA_TRY(to_device(dp, hv.data(), hv.size(), &s->bbmin_c, err));
  make_bb(plan.cols.bbext, plan.cols.nclusters(), &hv);
  FMCA_TRY(to_device(dp, hv.data(), hv.size(), &s->bbext_c, err));
  hv.assign(plan.row_E.begin(), plan.row_E.end());
  FMCA_TRY(to_device(dp, hv.data(), hv.size(), &s->E_r, err));
  hv.assign(plan.col_E.begin(), plan.col_E.end());
  FMCA_TRY(to_device(dp, hv.data(), hv.size(), &s->E_c, err));
  if (plan.interp.kind == kInterpTotalDegree) {
    hv.assign((size_t)q * q, T(0));
    for (int k = 0; k < q; ++k)
      for (int j = 0; j < q; ++j) hv[(size_t)k * q + j] = (T)plan.interp.invV[(size_t)j * q + k];
    FMCA_TRY(to_device(dp, hv.data(), hv.size(), &s->to_nodal, err));
    hv.assign(plan.interp.invV.begin(), plan.interp.invV.end());
    FMCA_TRY(to_device(dp, hv.data(), hv.size(), &s->from_nodal, err));
  }
  s->ip.kind = plan.interp.kind;
  s->ip.dim = dim;
  s->ip.p1 = plan.interp.deg + 1;
  s->ip.q = q;
  for (int k = 0; k < 8; ++k) {
    s->ip.xi[k] = k <= plan.interp.deg ? (T)plan.interp.xi[k] : T(0);
    s->ip.w[k] = k <= plan.interp.deg ? (T)plan.interp.w[k] : T(0);
  }
  s->ready = true;
  return FMCA_OK;
}

int upload_common(const Plan& plan, DevPlan* dp, std::string* err) {
  const Interp& ip = plan.interp;
  std::vector<int> midx((size_t)ip.q * 3, 0);
  for (int k = 0; k < ip.q; ++k)
    for (int d = 0; d < ip.dim; ++d) midx[(size_t)k * 3 + d] = ip.midx[(size_t)k * ip.dim + d];
  FMCA_TRY(to_device(dp, midx.data(), midx.size(), &dp->midx, err));
  FMCA_TRY(to_device(dp, plan.rows.perm.data(), plan.rows.perm.size(), &dp->perm_r, err));
  FMCA_TRY(to_device(dp, plan.cols.perm.data(), plan.cols.perm.size(), &dp->perm_c, err));
  FMCA_TRY(to_device(dp, plan.rows.begin.data(), plan.rows.begin.size(), &dp->cbegin_r, err));
  FMCA_TRY(to_device(dp, plan.rows.size.data(), plan.rows.size.size(), &dp->csize_r, err));
  FMCA_TRY(to_device(dp, plan.cols.begin.data(), plan.cols.begin.size(), &dp->cbegin_c, err));
  FMCA_TRY(to_device(dp, plan.cols.size.data(), plan.cols.size.size(), &dp->csize_c, err));
  FMCA_TRY(to_device(dp, plan.cols.son0.data(), plan.cols.son0.size(), &dp->son0_c, err));
  FMCA_TRY(to_device(dp, plan.cols.nsons.data(), plan.cols.nsons.size(), &dp->nsons_c, err));
  FMCA_TRY(to_device(dp, plan.rows.parent.data(), plan.rows.parent.size(), &dp->parent_r, err));
  FMCA_TRY(to_device(dp, plan.row_leaves.data(), plan.row_leaves.size(), &dp->leaves_r, err));
  FMCA_TRY(to_device(dp, plan.col_leaves.data(), plan.col_leaves.size(), &dp->leaves_c, err));
  dp->nleaves_r = (int)plan.row_leaves.size();
  dp->nleaves_c = (int)plan.col_leaves.size();
  // transfer level lists, bucketed by level (a batched plan holds a forest
  // whose clusters of one level are not contiguous)
  auto by_level = [](const Tree& t, bool up, std::vector<int32_t>* lst, std::vector<int>* ptr) {
    const int L = t.nlevels();
    std::vector<std::vector<int32_t>> b(L);
    for (int c = 0; c < t.nclusters(); ++c) {
      if (up ? t.nsons[c] > 0 : t.level[c] >= 1) b[t.level[c]].push_back(c);
    }
    ptr->assign(L + 1, 0);
    lst->clear();
    for (int l = 0; l < L; ++l) {
      lst->insert(lst->end(), b[l].begin(), b[l].end());
      (*ptr)[l + 1] = (int)lst->size();
    }
  };
  {
    std::vector<int32_t> lst;
    by_level(plan.cols, true, &lst, &dp->m2m_ptr);
    FMCA_TRY(to_device(dp, lst.data(), lst.size(), &dp->m2m_list, err));
  }
  {
    std::vector<int32_t> lst;
    by_level(plan.rows, false, &lst, &dp->l2l_ptr);
    FMCA_TRY(to_device(dp, lst.data(), lst.size(), &dp->l2l_list, err));
  }
  // far groups: targets = nodes of every row cluster, sources = node ranges
  // of the admissible column clusters, consecutive clusters merged.
  // Two chunkings: kGroupCap targets (CUDA-core kernel sum) and kTcGroupCap
  // (tensor-core kernel sum).
  for (int pass = 0; pass < 2; ++pass) {
    const uint32_t cap = pass == 0 ? kGroupCap : kTcGroupCap;
    HostGroups hg;
    const int q = ip.q;
    const Pattern& P = plan.pat;
    for (int c = 0; c < plan.rows.nclusters(); ++c) {
      const int ib = (int)(hg.ivl.size() / 2);
      for (int k = P.far_ptr[c]; k < P.far_ptr[c + 1]; ++k) {
        const uint32_t b = (uint32_t)P.far_idx[k] * q, e = b + q;
        if (hg.ivl.size() > (size_t)2 * ib && hg.ivl.back() == b)
          hg.ivl.back() = e;
        else {
          hg.ivl.push_back(b);
          hg.ivl.push_back(e);
        }
      }
      add_target_range(&hg, (uint32_t)c * q, q, ib, (int)(hg.ivl.size() / 2), cap);
    }
    sort_groups(&hg);
    FMCA_TRY(upload_groups(dp, hg, pass == 0 ? &dp->far : &dp->far_tc, err));
  }
  // far groups on tensor grids, two sibling row clusters a, a + 1 per group
  // (target halves of q nodes each): sources = the union of their
  // admissible column clusters, consecutive clusters with the same halves
  // merged into one interval, imask = the halves an interval serves
  if (plan.interp.kind == kInterpTensor && plan.interp.dim == 3 &&
      plan.interp.deg + 1 == kGridP1) {
    HostGroups hg;
    const int q = ip.q;
    const Pattern& P = plan.pat;
    const Tree& T = plan.rows;
    std::vector<std::pair<int, int>> pairs;  // (first cluster, clusters in the group)
    for (int c = 0; c < T.nclusters(); ++c) {
      if (T.parent[c] < 0) pairs.push_back({c, 1});
      for (int i = 0; i < T.nsons[c]; i += 2)
        pairs.push_back({T.son0[c] + i, std::min(2, T.nsons[c] - i)});
    }
    for (const auto& pr : pairs) {
      const int a = pr.first, m = pr.second;
      std::vector<std::pair<int, uint32_t>> u;  // (column cluster, halves)
      for (int h = 0; h < m; ++h)
        for (int k = P.far_ptr[a + h]; k < P.far_ptr[a + h + 1]; ++k)
          u.push_back({P.far_idx[k], 1u << h});
      // groups without sources stay: the kernel writes their zero locals
      std::sort(u.begin(), u.end());
      const int ib = (int)(hg.ivl.size() / 2);
      for (size_t i = 0; i < u.size();) {
        uint32_t mask = u[i].second;
        size_t j = i + 1;
        if (j < u.size() && u[j].first == u[i].first) mask |= u[j++].second;
        const uint32_t b = (uint32_t)u[i].first * q, e = b + q;
        if (hg.ivl.size() > (size_t)2 * ib && hg.ivl.back() == b && hg.imask.back() == mask) {
          hg.ivl.back() = e;
        } else {
          hg.ivl.push_back(b);
          hg.ivl.push_back(e);
          hg.imask.push_back(mask);
        }
        i = j;
      }
      KGroup g;
      g.tbegin = (uint32_t)a * q;
      g.tcount = (uint32_t)(m * q);
      g.ivl_begin = ib;
      g.ivl_end = (int)(hg.ivl.size() / 2);
      hg.groups.push_back(g);
      hg.maxcount = std::max<int>(hg.maxcount, (int)g.tcount);
    }
    // most work first (the imask array stays aligned with the intervals)
    sort_groups(&hg);
    FMCA_TRY(upload_groups(dp, hg, &dp->far_grid2, err));
  }
  // near groups: targets = points of every row leaf, sources = merged
  // column point intervals; kGroupCap = 256 targets suits both the CUDA-core
  // kernel sum and the tensor-core one with two halves of 128, kTcGroupCap
  // = 128 the tensor-core one with one half (small leaves; an autotuner
  // choice)
  for (int pass = 0; pass < 2; ++pass) {
    HostGroups hg;
    const Pattern& P = plan.pat;
    hg.ivl = P.near_ivl;
    for (size_t l = 0; l < plan.row_leaves.size(); ++l) {
      const int c = plan.row_leaves[l];
      add_target_range(&hg, plan.rows.begin[c], plan.rows.size[c], P.near_ptr[l],
                       P.near_ptr[l + 1], pass == 0 ? kGroupCap : kTcGroupCap);
    }
    sort_groups(&hg);
    FMCA_TRY(upload_groups(dp, hg, pass == 0 ? &dp->near : &dp->near_h1, err));
  }
  {
    // near field with one half: the rows of up to two leaves per group
    // (near_pack.cpp), where that saves a tenth of the groups
    PackedNear pk;
    if (build_near_packed(plan, kTcGroupCap, &pk)) {
      HostGroups hg;
      for (size_t i = 0; i < pk.ngroups(); ++i) {
        KGroup g;
        g.tbegin = pk.tbegin[i];
        g.tcount = pk.tcount[i];
        g.ivl_begin = pk.ivl_begin[i];
        g.ivl_end = pk.ivl_end[i];
        hg.groups.push_back(g);
        hg.maxcount = std::max<int>(hg.maxcount, (int)g.tcount);
      }
      hg.ivl.swap(pk.ivl);
      hg.imask.swap(pk.imask);
      FMCA_TRY(upload_groups(dp, hg, &dp->near_pk, err));
      FMCA_TRY(to_device(dp, pk.split.data(), pk.split.size(), &dp->near_pk.split, err));
    }
  }
  {
    void* p = nullptr;
    FMCA_CK(cudaMalloc(&p, sizeof(int)));
    dp->allocs.push_back(p);
    dp->alloc_bytes += sizeof(int);
    FMCA_CK(cudaMemset(p, 0, sizeof(int)));
    dp->err_flag = static_cast<int*>(p);
  }
  {
    const size_t ng = std::max<size_t>({(size_t)1, (size_t)dp->far_tc.ngroups,
                                        (size_t)dp->far_grid2.ngroups});
    void* p = nullptr;
    FMCA_CK(cudaMalloc(&p, sizeof(float) * 2 * ng));
    dp->allocs.push_back(p);
    dp->alloc_bytes += sizeof(float) * 2 * ng;
    dp->gexp = static_cast<float*>(p);
  }
  return FMCA_OK;
}

// right-hand-side blocking: RB accumulators per target; every per-row buffer
// is chunk-major ([R / RB][rows][ld]) so one chunk is contiguous and a source
// tile of ksum copies only its chunk.  ld = max(RB, 16 bytes / sizeof(T))
// keeps every row of a chunk 16-byte aligned for the bulk copies.
int rhs_block(int nrhs) { return nrhs <= 1 ? 1 : (nrhs <= 8 ? 8 : 32); }
template <typename T>
int ld_for(int nrhs) {
  const int rb = rhs_block(nrhs);
  const int minld = 16 / (int)sizeof(T);
  return rb < minld ? minld : rb;
}
int nchunks_for(int nrhs) {
  const int rb = rhs_block(nrhs);
  return (nrhs + rb - 1) / rb;
}

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

template <typename T>
struct Workspace {
  T *xc, *t, *s, *ynear, *yfar;
};

template <typename T>
size_t ws_layout(const Plan& plan, int nrhs, void* base, Workspace<T>* w) {
  const size_t ld = ld_for<T>(nrhs), nch = nchunks_for(nrhs);
  const size_t q = plan.interp.q;
  size_t off = 0;
  auto take = [&](size_t elems) {
    T* p = base ? reinterpret_cast<T*>(static_cast<char*>(base) + off) : nullptr;
    off += align_up(elems * sizeof(T));
    return p;
  };
  Workspace<T> tmp;
  tmp.xc = take((size_t)plan.cols.n * ld * nch);
  tmp.t = take((size_t)plan.cols.nclusters() * q * ld * nch);
  tmp.s = take((size_t)plan.rows.nclusters() * q * ld * nch);
  tmp.ynear = take((size_t)plan.rows.n * ld * nch);
  tmp.yfar = take((size_t)plan.rows.n * ld * nch);
  if (w) *w = tmp;
  return off;
}

template <typename T>
KParams<T> make_kparams(const KernelDesc& k, const CallOpts& opts = CallOpts()) {
  KParams<T> kp;
  const double l = k.l, log2e = 1.4426950408889634;
  double a = 0, e2 = 0;
  // the length-scale derivative kernels share the constants of their kernel
  const int base = is_dl_kernel(k.type) ? k.type - K_DL_EXPONENTIAL : k.type;
  switch (base) {
    case FMCA_KERNEL_EXPONENTIAL:
      e2 = -log2e / l;
      break;
    case FMCA_KERNEL_MATERN32:
      a = std::sqrt(3.) / l;
      e2 = -a * log2e;
      break;
    case FMCA_KERNEL_MATERN52:
      a = std::sqrt(5.) / l;
      e2 = -a * log2e;
      break;
    case FMCA_KERNEL_GAUSSIAN:
      e2 = -0.5 * log2e / (l * l);
      break;
    case FMCA_KERNEL_MATERN72:
      a = std::sqrt(7.) / l;
      e2 = -a * log2e;
      break;
    case FMCA_KERNEL_MATERN92:
      e2 = -3. / l * log2e;
      break;
    default:
      break;
  }
  kp.type = k.type;
  kp.l = (T)l;
  kp.c = (T)k.c;
  kp.a = (T)a;
  kp.e2 = (T)e2;
  kp.il = (T)(1. / l);
  // tensor-core path: coordinates multiplied by g turn the distance into
  // r' = g r, the kernel argument t times log2(e): k = 2^-r' (EXPONENTIAL),
  // (1 + t) 2^-r' (MATERN32), (1 + t + t^2/3) 2^-r' (MATERN52) with
  // t = ln(2) r', or 2^-r'^2 (GAUSSIAN)
  double g = 1;
  switch (base) {  // l dk/dl kernels use the coordinates of their kernel
    case FMCA_KERNEL_EXPONENTIAL:
      g = log2e / l;
      break;
    case FMCA_KERNEL_MATERN32:
    case FMCA_KERNEL_MATERN52:
    case FMCA_KERNEL_MATERN72:
      g = log2e * a;
      break;
    case FMCA_KERNEL_MATERN92:
      g = log2e * 3. / l;
      break;
    case FMCA_KERNEL_GAUSSIAN:
      g = std::sqrt(0.5 * log2e) / l;
      break;
    default:
      break;
  }
  kp.g = (T)g;
  kp.wait_ns = opts.wait_ns ? opts.wait_ns : kWaitLimitNs;
  kp.stall = opts.stall;
  return kp;
}

// kernel parameters of the tensor-core path: with the centre of the set's
// point clouds for the near field's dot-product distance form
KParams<float> tc_kparams(const DevSet<float>& S, const KernelDesc& k, const CallOpts& opts) {
  KParams<float> kp = make_kparams<float>(k, opts);
  kp.cx = S.ctr[0];
  kp.cy = S.ctr[1];
  kp.cz = S.ctr[2];
  return kp;
}

// scale applied to the assembled product: sigma2, divided by l for the
// length-scale derivative kernels (their device values are l * dk/dl)
double output_scale(const KernelDesc& k) {
  return is_dl_kernel(k.type) ? k.sigma2 / k.l : k.sigma2;
}

// Raises a kernel's dynamic shared-memory limit once per (kernel, device):
// later calls (for instance inside a stream capture) make no runtime call.
template <typename K>
void ensure_smem(K kern, size_t bytes) {
  if (bytes <= 48 * 1024) return;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = done[{reinterpret_cast<const void*>(kern), dev}];
  if (cur >= bytes) return;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
      cudaSuccess)
    cur = bytes;
}

template <typename T, int KT, int TPT, int RB>
cudaError_t launch_ksum_t(const GroupList& gl, const Pt4<T>* tgt,
                          const Pt4<T>* src, const T* sval, int ld, T* out,
                          int rofs, int rcount, const KParams<T>& kp, int accum,
                          int* errf, cudaStream_t st) {
  constexpr int TS = TileSize<T>::value;
  auto kern = ksum_kernel<T, KT, TPT, RB, TS, kStages>;
  const size_t smem = 128 + (size_t)kStages * TS * (sizeof(Pt4<T>) + (size_t)ld * sizeof(T));
  ensure_smem(kern, smem);
  int threads = (gl.maxcount + TPT - 1) / TPT;
  threads = (threads + 31) / 32 * 32;
  threads = std::max(32, std::min(128, threads));
  kern<<<gl.ngroups, threads, smem, st>>>(gl.groups, gl.ivl, tgt, src, sval, ld,
                                          out, rofs, rcount, kp, accum, errf);
  return cudaGetLastError();
}

template <typename T, int KT, int RB>
cudaError_t launch_ksum_tpt(const GroupList& gl, const Pt4<T>* tgt,
                            const Pt4<T>* src, const T* sval, int ld, T* out,
                            int rofs, int rcount, const KParams<T>& kp,
                            int accum, int* errf, cudaStream_t st) {
  if (gl.maxcount > 128)
    return launch_ksum_t<T, KT, 2, RB>(gl, tgt, src, sval, ld, out, rofs, rcount,
                                       kp, accum, errf, st);
  return launch_ksum_t<T, KT, 1, RB>(gl, tgt, src, sval, ld, out, rofs, rcount,
                                     kp, accum, errf, st);
}

template <typename T, int RB>
cudaError_t launch_ksum_kt(const GroupList& gl, const Pt4<T>* tgt,
                           const Pt4<T>* src, const T* sval, int ld, T* out,
                           int rofs, int rcount, const KParams<T>& kp, int accum,
                           int* errf, cudaStream_t st) {
  switch (kp.type) {
    case 0:
      return launch_ksum_tpt<T, 0, RB>(gl, tgt, src, sval, ld, out, rofs, rcount, kp, accum, errf, st);
    case 1:
      return launch_ksum_tpt<T, 1, RB>(gl, tgt, src, sval, ld, out, rofs, rcount, kp, accum, errf, st);
    case 2:
      return launch_ksum_tpt<T, 2, RB>(gl, tgt, src, sval, ld, out, rofs, rcount, kp, accum, errf, st);
    case 3:
      return launch_ksum_tpt<T, 3, RB>(gl, tgt, src, sval, ld, out, rofs, rcount, kp, accum, errf, st);
    default:
      return launch_ksum_tpt<T, -1, RB>(gl, tgt, src, sval, ld, out, rofs, rcount, kp, accum, errf, st);
  }
}

template <typename T>
cudaError_t launch_ksum(int rb, const GroupList& gl, const Pt4<T>* tgt,
                        const Pt4<T>* src, const T* sval, int ld, T* out,
                        int rofs, int rcount, const KParams<T>& kp, int accum,
                        int* errf, cudaStream_t st) {
  if (gl.ngroups == 0) return cudaSuccess;
  switch (rb) {
    case 1:
      return launch_ksum_kt<T, 1>(gl, tgt, src, sval, ld, out, rofs, rcount, kp, accum, errf, st);
    case 8:
      return launch_ksum_kt<T, 8>(gl, tgt, src, sval, ld, out, rofs, rcount, kp, accum, errf, st);
    default:
      return launch_ksum_kt<T, 32>(gl, tgt, src, sval, ld, out, rofs, rcount, kp, accum, errf, st);
  }
}

// one transfer level (M2M when UP, else L2L) over the nb clusters of list.
// A level with fewer than tc.slice_below clusters (default: two per SM)
// splits the right-hand sides over blockIdx.y in slices of 8, so that it
// still spreads over the GPU; the sum-factorised kernel runs 8 warps per
// cluster on levels with fewer than tc.wide_below clusters (default: four
// per SM).
template <int DIM, int P, bool UP>
void launch_transfer_sf(int nb, const int32_t* list, const int32_t* son0,
                        const int32_t* nsons, const int32_t* parent, const float* E,
                        const int* midx, float* buf, int ld, int rofs, int rcount,
                        const TrCfg& tc, cudaStream_t st) {
  constexpr int Q = DIM == 2 ? P * P : P * P * P;
  auto kern = transfer_sf_kernel<DIM, P, UP>;
  const size_t smem = (size_t)(3 * Q * 32 + Q + DIM * P * P) * sizeof(float);
  ensure_smem(kern, smem);
  // levels with few clusters: 8 warps per cluster shorten its latency chain
  const int threads = nb < tc.wide_below ? 256 : 128;
  kern<<<nb, threads, smem, st>>>(list, son0, nsons, parent, E, midx, buf, ld, rofs, rcount);
}

// the sum-factorised transfer for the tensor grids it is instantiated for
// (2-D with 4..8 nodes per dimension, 3-D with 4..6; FP32, up to 32
// right-hand sides); false: use transfer_kernel
template <bool UP>
bool launch_transfer_sf_any(int nb, const int32_t* list, const int32_t* son0,
                            const int32_t* nsons, const int32_t* parent, const float* E,
                            const int* midx, const InterpDev<float>& ip, float* buf, int ld,
                            int rofs, int rcount, const TrCfg& tc, cudaStream_t st) {
  if (rcount > 32) return false;
#define FMCA_SF(D, P)                                                                    \
  case D * 16 + P:                                                                       \
    launch_transfer_sf<D, P, UP>(nb, list, son0, nsons, parent, E, midx, buf, ld, rofs, \
                                 rcount, tc, st);                                        \
    return true;
  switch (ip.dim * 16 + ip.p1) {
    FMCA_SF(2, 4)
    FMCA_SF(2, 5)
    FMCA_SF(2, 6)
    FMCA_SF(2, 7)
    FMCA_SF(2, 8)
    FMCA_SF(3, 4)
    FMCA_SF(3, 5)
    FMCA_SF(3, 6)
    default:
      return false;
  }
#undef FMCA_SF
}

template <typename T, int RB, bool UP>
void launch_transfer(int nb, const int32_t* list, const int32_t* son0,
                     const int32_t* nsons, const int32_t* parent, const T* E,
                     const int* midx, const InterpDev<T>& ip, T* buf, int ld,
                     int rofs, int rcount, const TrCfg& tc, cudaStream_t st) {
  if (ip.kind == kInterpTotalDegree) {
    // dense E per cluster; levels with few clusters split the right-hand
    // sides in slices of 8
    const int q = ip.q;
    if (nb < tc.slice_below && rcount > 8 && RB > 8) {
      auto kern = transfer_dense_kernel<T, 8, UP>;
      const size_t smem = (dense_pad(q) + (size_t)q * 8) * sizeof(T);
      ensure_smem(kern, smem);
      kern<<<dim3(nb, (rcount + 7) / 8), 128, smem, st>>>(list, son0, nsons, parent, E, q,
                                                           buf, ld, rofs, rcount);
    } else {
      auto kern = transfer_dense_kernel<T, RB, UP>;
      const size_t smem = (dense_pad(q) + (size_t)q * RB) * sizeof(T);
      ensure_smem(kern, smem);
      kern<<<dim3(nb, (rcount + RB - 1) / RB), 128, smem, st>>>(list, son0, nsons, parent, E,
                                                                 q, buf, ld, rofs, rcount);
    }
    return;
  }
  if constexpr (std::is_same<T, float>::value && RB == 32) {
    if (launch_transfer_sf_any<UP>(nb, list, son0, nsons, parent, E, midx, ip, buf, ld, rofs,
                                   rcount, tc, st))
      return;
  }
  const size_t tail = (size_t)ip.q * sizeof(int);
  if constexpr (RB > 8) {
    if (nb < tc.slice_below && rcount > 8) {
      constexpr int RS = 8;
      auto kern = transfer_kernel<T, RS, UP>;
      const size_t smem = (192 + kTransferChunk * RS) * sizeof(T) + tail;
      ensure_smem(kern, smem);
      kern<<<dim3(nb, (rcount + RS - 1) / RS), 128, smem, st>>>(
          list, son0, nsons, parent, E, midx, ip, buf, ld, rofs, rcount);
      return;
    }
  }
  auto kern = transfer_kernel<T, RB, UP>;
  const size_t smem = (192 + kTransferChunk * RB) * sizeof(T) + tail;
  ensure_smem(kern, smem);
  kern<<<nb, 128, smem, st>>>(list, son0, nsons, parent, E, midx, ip, buf, ld, rofs,
                              rcount);
}

// The far field of the GAUSSIAN kernel on tensor-product nodes as Kronecker
// products (far_kron_reg_kernel, far_kron_kernel), for the grids they are
// instantiated for: 2-D with 3..8 nodes per dimension, 3-D with 3..6.
// false: not applicable (another kernel, total degree, other grids); the
// caller runs the dense kernel sum.
template <typename T>
bool far_kron_ok(const DevPlan* dp, const DevSet<T>& S, int type, int rcount) {
  return type == FMCA_KERNEL_GAUSSIAN && S.ip.kind == kInterpTensor && rcount <= 32 &&
         far_kron_grid(S.ip.dim, S.ip.p1) && dp->far.ngroups > 0 && dp->far.maxcount == S.ip.q;
}
template <typename T>
bool launch_far_kron(const DevPlan* dp, const DevSet<T>& S, const KParams<T>& kp, const T* t,
                     int ldt, int tofs, T* s, int lds, int sofs, int rcount, cudaStream_t st,
                     cudaError_t* err) {
  if (!far_kron_ok(dp, S, kp.type, rcount)) return false;
  const T e = sizeof(T) == 4 ? kp.e2 : T(-0.5) / (kp.l * kp.l);
  *err = launch_far_kron_kernel<T>(S.ip.dim, S.ip.p1, dp->far.groups, dp->far.ngroups,
                                   dp->far.ivl, S.nodes_r, S.nodes_c, dp->midx, e, t, ldt, tofs,
                                   s, lds, sofs, rcount, st);
  return true;
}

// total degree: coefficients of clusters 0 .. ncl - 1 to (M = invV^T) or
// from (M = invV) the nodal basis of the far field; one launch (or none for
// the tensor product, whose basis is nodal already)
template <typename T, int RB>
bool launch_basis_change(const InterpDev<T>& ip, int ncl, const T* M, T* buf, int ld, int rofs,
                         int rcount, cudaStream_t st) {
  if (ip.kind != kInterpTotalDegree || ncl == 0) return false;
  auto kern = basis_change_kernel<T, RB>;
  const size_t smem = (dense_pad(ip.q) + (size_t)ip.q * RB) * sizeof(T);
  ensure_smem(kern, smem);
  kern<<<dim3(ncl, (rcount + RB - 1) / RB), 128, smem, st>>>(ncl, M, ip.q, buf, ld, rofs,
                                                              rcount);
  return true;
}

template <typename T, int RB, int FS>
size_t leafmom_smem(int q) {
  return (size_t)kLeafChunk * (3 * FS + RB) * sizeof(T) + (size_t)q * sizeof(int);
}
template <typename T, int RB, int FS>
size_t leafgather_smem(int q) {
  return ((size_t)128 * 3 * FS + (size_t)q * RB) * sizeof(T) + (size_t)q * sizeof(int);
}

// The leaf passes (upward: moments of the column leaves into t; downward:
// the row leaves' far-field values from s) with 8 factor slots per
// dimension, or 16 for the total-degree bases of degree 8 and above.
template <typename T, int RB, int FS>
cudaError_t leafmom_fs(int nb, const DevPlan* dp, const DevSet<T>& S, const T* xc, int ld,
                       int rofs, int rcount, T* t, cudaStream_t st) {
  auto kern = leafmom_kernel<T, RB, FS>;
  const size_t smem = leafmom_smem<T, RB, FS>(S.ip.q);
  ensure_smem(kern, smem);
  kern<<<nb, 128, smem, st>>>(dp->leaves_c, dp->cbegin_c, dp->csize_c, S.bbmin_c, S.bbext_c,
                              S.pts_c, xc, ld, rofs, rcount, dp->midx, S.ip, t);
  return cudaGetLastError();
}
template <typename T, int RB>
cudaError_t launch_leafmom(const DevPlan* dp, const DevSet<T>& S, const T* xc, int ld, int rofs,
                           int rcount, T* t, cudaStream_t st) {
  if (!dp->nleaves_c) return cudaSuccess;
  if (S.ip.p1 > 8)
    return leafmom_fs<T, RB, 16>(dp->nleaves_c, dp, S, xc, ld, rofs, rcount, t, st);
  return leafmom_fs<T, RB, 8>(dp->nleaves_c, dp, S, xc, ld, rofs, rcount, t, st);
}
template <typename T, int RB, int FS>
cudaError_t leafgather_fs(int nb, const DevPlan* dp, const DevSet<T>& S, const T* s, int ld,
                          int rofs, int rcount, T* y, cudaStream_t st) {
  auto kern = leafgather_kernel<T, RB, FS>;
  const size_t smem = leafgather_smem<T, RB, FS>(S.ip.q);
  ensure_smem(kern, smem);
  kern<<<nb, 128, smem, st>>>(dp->leaves_r, dp->cbegin_r, dp->csize_r, S.bbmin_r, S.bbext_r,
                              S.pts_r, s, ld, rofs, rcount, dp->midx, S.ip, y);
  return cudaGetLastError();
}
template <typename T, int RB>
cudaError_t launch_leafgather(const DevPlan* dp, const DevSet<T>& S, const T* s, int ld,
                              int rofs, int rcount, T* y, cudaStream_t st) {
  if (!dp->nleaves_r) return cudaSuccess;
  if (S.ip.p1 > 8)
    return leafgather_fs<T, RB, 16>(dp->nleaves_r, dp, S, s, ld, rofs, rcount, y, st);
  return leafgather_fs<T, RB, 8>(dp->nleaves_r, dp, S, s, ld, rofs, rcount, y, st);
}

// as: stored blocks of an assembled plan (the far field streams them instead
// of evaluating the kernel), or null
template <typename T, int RB>
cudaError_t run_tree_stages(const Plan& plan, DevPlan* dp, DevSet<T>& S,
                            Workspace<T>& w, int ld, int rofs, int rcount,
                            const KParams<T>& kp, cudaStream_t st,
                            const AsmStore* as = nullptr) {
  const int q = plan.interp.q;
  // upward pass: leaf moments
  {
    dp->launches += dp->nleaves_c ? 1 : 0;
    cudaError_t e = launch_leafmom<T, RB>(dp, S, w.xc, ld, rofs, rcount, w.t, st);
    if (e != cudaSuccess) return e;
    dp->mark(FMCA_STAGE_LEAFMOM, st);
  }
  // M2M, bottom-up
  for (int l = plan.cols.nlevels() - 1; l >= 0; --l) {
    const int nb = dp->m2m_ptr[l + 1] - dp->m2m_ptr[l];
    if (nb) {
      launch_transfer<T, RB, true>(nb, dp->m2m_list + dp->m2m_ptr[l], dp->son0_c,
                                   dp->nsons_c, nullptr, S.E_c, dp->midx, S.ip, w.t, ld,
                                   rofs, rcount, dp->cfg.tr, st);
      ++dp->launches;
    }
  }
  dp->launches += launch_basis_change<T, RB>(S.ip, plan.cols.nclusters(), S.to_nodal, w.t, ld,
                                             rofs, rcount, st);
  dp->mark(FMCA_STAGE_M2M, st);
  // far-field coupling: stored blocks, the Gaussian's Kronecker factors, or
  // the kernel sum over the node pairs
  cudaError_t e = cudaSuccess;
  if (as)
    e = launch_kstream<T>(RB, dp->far.groups, dp->far.ngroups, dp->far.maxcount, dp->far.ivl,
                          as->far_off, static_cast<const T*>(as->far), w.t, ld, w.s, rofs,
                          rcount, kp.wait_ns, kp.stall, dp->err_flag, st);
  else if (!launch_far_kron<T>(dp, S, kp, w.t, ld, rofs, w.s, ld, rofs, rcount, st, &e))
    e = launch_ksum<T>(RB, dp->far, S.nodes_r, S.nodes_c, w.t, ld, w.s, rofs, rcount, kp, 0,
                       dp->err_flag, st);
  if (e != cudaSuccess) return e;
  dp->launches += dp->far.ngroups ? 1 : 0;
  dp->launches += launch_basis_change<T, RB>(S.ip, plan.rows.nclusters(), S.from_nodal, w.s,
                                             ld, rofs, rcount, st);
  dp->mark(FMCA_STAGE_FAR, st);
  // L2L, top-down
  for (int l = 1; l < plan.rows.nlevels(); ++l) {
    const int nb = dp->l2l_ptr[l + 1] - dp->l2l_ptr[l];
    if (nb) {
      launch_transfer<T, RB, false>(nb, dp->l2l_list + dp->l2l_ptr[l], nullptr, nullptr,
                                    dp->parent_r, S.E_r, dp->midx, S.ip, w.s, ld, rofs,
                                    rcount, dp->cfg.tr, st);
      ++dp->launches;
    }
  }
  dp->mark(FMCA_STAGE_L2L, st);
  // leaf gather
  {
    cudaError_t eg = launch_leafgather<T, RB>(dp, S, w.s, ld, rofs, rcount, w.yfar, st);
    if (eg != cudaSuccess) return eg;
    dp->launches += dp->nleaves_r ? 1 : 0;
    dp->mark(FMCA_STAGE_LEAFGATHER, st);
  }
  return cudaGetLastError();
}

// near field of one right-hand-side chunk (the last stage of the chunk; it
// fills the GPU on its own, so running it concurrently with the far-field
// chain on a second stream gained nothing at n = 1e6)
template <typename T, int RB>
cudaError_t run_near(DevPlan* dp, DevSet<T>& S, Workspace<T>& w, int ld, int rcount,
                     const KParams<T>& kp, cudaStream_t st, const AsmStore* as = nullptr) {
  cudaError_t e =
      as ? launch_kstream<T>(RB, dp->near.groups, dp->near.ngroups, dp->near.maxcount,
                             dp->near.ivl, as->near_off, static_cast<const T*>(as->near), w.xc,
                             ld, w.ynear, 0, rcount, kp.wait_ns, kp.stall, dp->err_flag, st)
         : launch_ksum<T>(RB, dp->near, S.pts_r, S.pts_c, w.xc, ld, w.ynear, 0, rcount, kp, 0,
                          dp->err_flag, st);
  dp->launches += dp->near.ngroups ? 1 : 0;
  dp->mark(FMCA_STAGE_NEAR, st);
  return e;
}

// caller workspace if given, else the plan's own (grown on demand)
int acquire_ws(DevPlan* dp, size_t need, void** ws, size_t wsb, cudaStream_t st,
               std::string* err) {
  if (!*ws) {
    if (dp->ws_bytes < need) {
      if (dp->ws) {
        FMCA_CK(cudaStreamSynchronize(st));
        cudaFree(dp->ws);
        dp->ws = nullptr;
        dp->ws_bytes = 0;
      }
      FMCA_CK(cudaMalloc(&dp->ws, need));
      dp->ws_bytes = need;
    }
    *ws = dp->ws;
  } else if (wsb < need) {
    *err = "workspace too small: need " + std::to_string(need) + " bytes";
    return FMCA_ERR_INVALID_ARGUMENT;
  }
  return FMCA_OK;
}

// Where a finished matvec left its cluster-ordered input and leaf expansions
// (used by the adjoint).  All buffers are chunk-major [nch][rows][ld].
struct MatvecState {
  const void* xc = nullptr;        // input in cluster order (T)
  const void* s = nullptr;         // downward-pass expansions per row cluster (T)
  const unsigned int* cmax = nullptr;  // column maxima of the scaled path, or null
  int ld = 0, rb = 0, nch = 0;
  bool fp64 = false;
  int cofs = 0;  // first column of this product's right-hand sides in the buffers
};

template <typename T>
int matvec_t(const Plan& plan, DevPlan* dp, DevSet<T>& S, const KernelDesc& k,
             int dtype, int order, int nrhs, const void* x, int64_t sxi,
             int64_t sxr, void* y, int64_t syi, int64_t syr, void* ws,
             size_t wsb, cudaStream_t st, std::string* err,
             MatvecState* state = nullptr, const AsmStore* as = nullptr) {
  const int ld = ld_for<T>(nrhs);
  const int rb = rhs_block(nrhs);
  const size_t need = ws_layout<T>(plan, nrhs, nullptr, nullptr);
  FMCA_TRY(acquire_ws(dp, need, &ws, wsb, st, err));
  Workspace<T> w;
  ws_layout<T>(plan, nrhs, ws, &w);
  if (state) {
    state->xc = w.xc;
    state->s = w.s;
    state->cmax = nullptr;
    state->ld = ld;
    state->rb = rb;
    state->nch = nchunks_for(nrhs);
    state->fp64 = sizeof(T) == 8;
  }
  dp->reset_marks();
  dp->mark(-1, st);
  const KParams<T> kp = make_kparams<T>(k, dp->opts);
  const uint32_t* pc = order == FMCA_ORDER_NATURAL ? dp->perm_c : nullptr;
  const uint32_t* pr = order == FMCA_ORDER_NATURAL ? dp->perm_r : nullptr;
  const int nthr = 256;
  auto blocks = [&](int64_t total) {
    int64_t b = (total + nthr - 1) / nthr;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)dp->sms * 32));
  };
  if (dtype == FMCA_DTYPE_F64)
    gather_kernel<double, T><<<blocks((int64_t)plan.cols.n * ld * nchunks_for(nrhs)), nthr, 0,
                               st>>>(pc, plan.cols.n, nrhs, rb, ld,
                                     static_cast<const double*>(x), sxi, sxr, w.xc);
  else
    gather_kernel<float, T><<<blocks((int64_t)plan.cols.n * ld * nchunks_for(nrhs)), nthr, 0,
                              st>>>(pc, plan.cols.n, nrhs, rb, ld,
                                    static_cast<const float*>(x), sxi, sxr, w.xc);
  FMCA_CK(cudaGetLastError());
  ++dp->launches;
  dp->mark(FMCA_STAGE_GATHER, st);
  const size_t q = plan.interp.q;
  for (int ch = 0; ch * rb < nrhs; ++ch) {
    const int rcount = std::min(rb, nrhs - ch * rb);
    Workspace<T> wc;
    wc.xc = w.xc + (size_t)ch * plan.cols.n * ld;
    wc.t = w.t + (size_t)ch * plan.cols.nclusters() * q * ld;
    wc.s = w.s + (size_t)ch * plan.rows.nclusters() * q * ld;
    wc.ynear = w.ynear + (size_t)ch * plan.rows.n * ld;
    wc.yfar = w.yfar + (size_t)ch * plan.rows.n * ld;
    cudaError_t e;
    switch (rb) {
      case 1:
        e = run_tree_stages<T, 1>(plan, dp, S, wc, ld, 0, rcount, kp, st, as);
        if (e == cudaSuccess) e = run_near<T, 1>(dp, S, wc, ld, rcount, kp, st, as);
        break;
      case 8:
        e = run_tree_stages<T, 8>(plan, dp, S, wc, ld, 0, rcount, kp, st, as);
        if (e == cudaSuccess) e = run_near<T, 8>(dp, S, wc, ld, rcount, kp, st, as);
        break;
      default:
        e = run_tree_stages<T, 32>(plan, dp, S, wc, ld, 0, rcount, kp, st, as);
        if (e == cudaSuccess) e = run_near<T, 32>(dp, S, wc, ld, rcount, kp, st, as);
        break;
    }
    FMCA_CK(e);
    FMCA_CK(cudaGetLastError());
  }
  if (dtype == FMCA_DTYPE_F64)
    scatter_kernel<T, double><<<blocks((int64_t)plan.rows.n * nrhs), nthr, 0, st>>>(
        pr, plan.rows.n, nrhs, rb, ld, w.ynear, w.yfar, output_scale(k), static_cast<double*>(y),
        syi, syr);
  else
    scatter_kernel<T, float><<<blocks((int64_t)plan.rows.n * nrhs), nthr, 0, st>>>(
        pr, plan.rows.n, nrhs, rb, ld, w.ynear, w.yfar, output_scale(k), static_cast<float*>(y),
        syi, syr);
  ++dp->launches;
  dp->mark(FMCA_STAGE_SCATTER, st);
  FMCA_CK(cudaGetLastError());
  return FMCA_OK;
}

// ---------------------------------------------------------------------------
// mixed precision with tensor-core kernel sums
struct TcWorkspace {
  float *xc, *t, *s, *ynear, *yfar;
  __half *xv, *tv;            // tensor-core values layout (hi and lo parts)
  float4* pairs_c;            // column points as pair records
  float4* pairs_n;            // column interpolation nodes as pair records
  unsigned int* cmax;
};

size_t tc_ws_layout(const Plan& plan, int nrhs, void* base, TcWorkspace* w) {
  const size_t nch = (nrhs + kTcRhs - 1) / kTcRhs, ld = kTcRhs;
  const size_t q = plan.interp.q;
  const size_t Cr = plan.rows.nclusters(), Cc = plan.cols.nclusters();
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* p = base ? static_cast<char*>(base) + off : nullptr;
    off += align_up(bytes);
    return p;
  };
  TcWorkspace t;
  // far values: the tensor-grid layout (128 rows per cluster) or the general one
  const size_t npc = um_padded(plan.cols.n);
  const size_t npn = std::max(um_padded(Cc * q), Cc * (size_t)kGridRows);
  t.xc = (float*)take(plan.cols.n * ld * nch * 4);
  t.xv = (__half*)take(npc * ld * nch * 2 * 2);
  t.t = (float*)take(Cc * q * ld * nch * 4);
  t.tv = (__half*)take(npn * ld * 2 * 2);
  t.pairs_c = (float4*)take(npc * 16);
  t.pairs_n = (float4*)take(npn * 16);
  t.s = (float*)take(Cr * q * ld * nch * 4);
  t.ynear = (float*)take(plan.rows.n * ld * nch * 4);
  t.yfar = (float*)take(plan.rows.n * ld * nch * 4);
  t.cmax = (unsigned int*)take((size_t)nrhs * 4);
  if (w) *w = t;
  return off;
}

// kernels whose values lie in [0, 1] (the FP16 split needs a bounded range):
// the six covariance kernels and l * dk/dl of the first four
// fewer than 17 right-hand sides take the CUDA-core FP32 path unless the
// autotuner found the tensor-core path (columns padded to 32) faster
bool tc_bounded(int type) {
  return (type >= FMCA_KERNEL_EXPONENTIAL && type <= FMCA_KERNEL_MATERN92) ||
         (type >= K_DL_EXPONENTIAL && type <= K_DL_GAUSSIAN);
}
bool tc_supported(int type, int nrhs, int small_tc) {
  return tc_bounded(type) && (nrhs > 16 || small_tc);
}

// Tensor-core kernel sum over a group list: H target halves of 128 per
// CTA (groups of up to 128 H targets). q > 0: the sources are
// interpolation nodes (q per cluster) weighted by their cluster's moment
// exponent; q = 0: points of weight 1. grid: nodes on tensor grids
// (tscale_grid_kernel layout). uc: stages and tiles per accumulation unit.

template <int KT, int H, bool REL, bool GRID>
cudaError_t launch_um_v(const GroupList& gl, const Pt4<float>* tgt, const float4* pairs,
                        const __half* vals, float* out, int rcount,
                        const KParams<float>& kp, int q, int* errf, cudaStream_t st,
                        const UmCfg& uc, float* gexp, int sms) {
  if (uc.persist) {
    if (gl.split) return cudaErrorInvalidValue;  // packed lists: one CTA per group only
    return launch_um_persistent(KT, H, REL, GRID, gl.groups, gl.ngroups, gl.ivl, gl.imask, tgt,
                                pairs, vals, out, rcount, kp, q, errf, gexp, uc.nst, uc.F, sms,
                                st);
  }
  auto kern = ksum_um_kernel<KT, H, REL, GRID>;
  const size_t smem = um_smem_bytes(H, kUmMaxStages);
  ensure_smem(kern, smem);
  kern<<<gl.ngroups, kUmThreads, um_smem_bytes(H, uc.nst), st>>>(
      gl.groups, gl.ivl, tgt, pairs, vals, out, kTcRhs, rcount, kp, q, errf, gl.imask, uc.nst,
      uc.F, gl.split);
  return cudaGetLastError();
}

template <int KT, int H>
cudaError_t launch_um_t(const GroupList& gl, const Pt4<float>* tgt, const float4* pairs,
                        const __half* vals, float* out, int rcount,
                        const KParams<float>& kp, int q, int* errf, cudaStream_t st,
                        bool grid, const UmCfg& uc, float* gexp, int sms) {
  if constexpr (H == 2) {  // tensor grids: sibling row clusters as the two halves
    if (grid)
      return launch_um_v<KT, 2, true, true>(gl, tgt, pairs, vals, out, rcount, kp, q, errf, st,
                                            uc, gexp, sms);
  }
  if (q > 0)
    return launch_um_v<KT, H, true, false>(gl, tgt, pairs, vals, out, rcount, kp, q, errf, st,
                                           uc, gexp, sms);
  return launch_um_v<KT, H, false, false>(gl, tgt, pairs, vals, out, rcount, kp, 0, errf, st,
                                          uc, nullptr, sms);
}

template <int H>
cudaError_t launch_um_k(const GroupList& gl, const Pt4<float>* tgt, const float4* pairs,
                        const __half* vals, float* out, int rcount,
                        const KParams<float>& kp, int q, int* errf, cudaStream_t st,
                        bool grid, const UmCfg& uc, float* gexp, int sms) {
#define FMCA_UM(KT) \
  launch_um_t<KT, H>(gl, tgt, pairs, vals, out, rcount, kp, q, errf, st, grid, uc, gexp, sms)
  switch (kp.type) {
    case 0:
      return FMCA_UM(0);
    case 1:
      return FMCA_UM(1);
    case 2:
      return FMCA_UM(2);
    case 3:
      return FMCA_UM(3);
    case 4:
      return FMCA_UM(4);
    case 5:
      return FMCA_UM(5);
    case K_DL_EXPONENTIAL:
      return FMCA_UM(K_DL_EXPONENTIAL);
    case K_DL_EXPONENTIAL + 1:
      return FMCA_UM(K_DL_EXPONENTIAL + 1);
    case K_DL_EXPONENTIAL + 2:
      return FMCA_UM(K_DL_EXPONENTIAL + 2);
    case K_DL_EXPONENTIAL + 3:
      return FMCA_UM(K_DL_EXPONENTIAL + 3);
    default:
      return FMCA_UM(-1);
  }
#undef FMCA_UM
}

// grid: the far field of a 3-D plan of degree kGridP1 - 1 (sources in the
// tscale_grid_kernel layout). uc is checked here: 2 <= nst <= kUmMaxStages,
// 1 <= F <= min(kUmMaxUnit, nst) (a unit's tiles must fit in the ring).
template <int H>
cudaError_t launch_um(const GroupList& gl, const Pt4<float>* tgt, const float4* pairs,
                      const __half* vals, float* out, int rcount,
                      const KParams<float>& kp, int q, int* errf, cudaStream_t st,
                      bool grid, const UmCfg& uc, float* gexp, int sms) {
  if (gl.ngroups == 0) return cudaSuccess;
  if (uc.nst < 2 || uc.nst > kUmMaxStages || uc.F < 1 || uc.F > kUmMaxUnit || uc.F > uc.nst)
    return cudaErrorInvalidValue;
  return launch_um_k<H>(gl, tgt, pairs, vals, out, rcount, kp, q, errf, st, grid, uc, gexp, sms);
}

bool grid_far(const Plan& plan) {
  return plan.interp.kind == kInterpTensor && plan.interp.dim == 3 &&
         plan.interp.deg + 1 == kGridP1;
}

// The stages of one right-hand-side chunk (32 columns) of the mixed
// precision matvec, each callable on its own (the autotuner times them one
// by one with different launch shapes).  Every stage records its event and
// counts its launches.
struct TcChunk {
  const Plan* plan;
  DevPlan* dp;
  DevSet<float>* S;
  KParams<float> kp;
  int rcount, q, Cc, Cr;
  int64_t npc;
  float *xc, *t, *s, *yfar, *ynear;
  const __half* xv;
  TcWorkspace w;
  cudaStream_t st;

  // The leaf passes accumulate only the chunk's rcount columns (1, 8 or 32
  // per thread): every later reader of t and s (moment scaling, transfers,
  // gradient terms) and of yfar (scatter) takes rcount columns too
  cudaError_t leafmom() {
    cudaError_t e =
        rcount <= 1   ? launch_leafmom<float, 1>(dp, *S, xc, kTcRhs, 0, rcount, t, st)
        : rcount <= 8 ? launch_leafmom<float, 8>(dp, *S, xc, kTcRhs, 0, rcount, t, st)
                      : launch_leafmom<float, kTcRhs>(dp, *S, xc, kTcRhs, 0, rcount, t, st);
    if (e != cudaSuccess) return e;
    dp->launches += dp->nleaves_c ? 1 : 0;
    dp->mark(FMCA_STAGE_LEAFMOM, st);
    return cudaGetLastError();
  }
  cudaError_t m2m(const TrCfg& tr) {
    for (int l = plan->cols.nlevels() - 1; l >= 0; --l) {
      const int nb = dp->m2m_ptr[l + 1] - dp->m2m_ptr[l];
      if (nb) {
        launch_transfer<float, kTcRhs, true>(nb, dp->m2m_list + dp->m2m_ptr[l], dp->son0_c,
                                             dp->nsons_c, nullptr, S->E_c, dp->midx, S->ip, t,
                                             kTcRhs, 0, rcount, tr, st);
        ++dp->launches;
      }
    }
    dp->launches +=
        launch_basis_change<float, kTcRhs>(S->ip, Cc, S->to_nodal, t, kTcRhs, 0, rcount, st);
    dp->mark(FMCA_STAGE_M2M, st);
    return cudaGetLastError();
  }
  // far field: moments scaled into the FP16 value layout, then the kernel
  // sum, on the sibling-paired tensor grids (3-D plans of degree
  // kGridP1 - 1, unless cfg.far_pairs is 0) or on interpolation nodes
  cudaError_t far(const TuneCfg& cfg) {
    // the Gaussian's far field as Kronecker products (FP32 CUDA cores on the
    // unscaled moments), when the grid is one it is compiled for
    cudaError_t ek = cudaSuccess;
    if (cfg.far_kron && far_kron_ok(dp, *S, kp.type, rcount)) {
      // up to 8 columns in use: the moments are read from a compact copy
      // (in the idle FP16 value buffer), rows of 1 or 8 values instead of
      // 32, which stays in L2 for the re-reads of each source cluster
      const int rb = rhs_block(rcount);
      const float* tk = t;
      if (rb < kTcRhs) {
        float* tc = reinterpret_cast<float*>(w.tv);
        ek = launch_compact_columns(t, kTcRhs, tc, rb, (int64_t)Cc * q, rcount, st);
        if (ek != cudaSuccess) return ek;
        ++dp->launches;
        tk = tc;
      }
      launch_far_kron<float>(dp, *S, kp, tk, rb < kTcRhs ? rb : kTcRhs, 0, s, kTcRhs, 0, rcount,
                             st, &ek);
      ++dp->launches;
      if (ek != cudaSuccess) return ek;
      dp->mark(FMCA_STAGE_FAR, st);
      return cudaGetLastError();
    }
    const bool grid = grid_far(*plan) && cfg.far_pairs;
    if (grid)
      tscale_grid_kernel<<<Cc, 128, 0, st>>>(Cc, rcount, t, S->nodes_c, dp->midx, kp.g, w.tv,
                                              reinterpret_cast<float*>(w.pairs_n));
    else
      tscale_kernel<<<Cc, 128, 0, st>>>(Cc, q, rcount, t, S->nodes_c, kp.g, w.tv,
                                         reinterpret_cast<float*>(w.pairs_n));
    ++dp->launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const GroupList& fl = grid ? dp->far_grid2 : dp->far_tc;
    e = grid ? launch_um<2>(fl, S->nodes_r, w.pairs_n, w.tv, s, rcount, kp, q, dp->err_flag, st,
                            true, cfg.far_grid, dp->gexp, dp->sms)
             : launch_um<1>(fl, S->nodes_r, w.pairs_n, w.tv, s, rcount, kp, q, dp->err_flag, st,
                            false, cfg.far_nodes, dp->gexp, dp->sms);
    if (e != cudaSuccess) return e;
    // the persistent form computes the groups' exponents in a launch first
    const bool persist = grid ? cfg.far_grid.persist : cfg.far_nodes.persist;
    dp->launches += fl.ngroups ? (persist ? 2 : 1) : 0;
    dp->launches +=
        launch_basis_change<float, kTcRhs>(S->ip, Cr, S->from_nodal, s, kTcRhs, 0, rcount, st);
    dp->mark(FMCA_STAGE_FAR, st);
    return cudaGetLastError();
  }
  cudaError_t l2l(const TrCfg& tr) {
    for (int l = 1; l < plan->rows.nlevels(); ++l) {
      const int nb = dp->l2l_ptr[l + 1] - dp->l2l_ptr[l];
      if (nb) {
        launch_transfer<float, kTcRhs, false>(nb, dp->l2l_list + dp->l2l_ptr[l], nullptr,
                                              nullptr, dp->parent_r, S->E_r, dp->midx, S->ip, s,
                                              kTcRhs, 0, rcount, tr, st);
        ++dp->launches;
      }
    }
    dp->mark(FMCA_STAGE_L2L, st);
    return cudaGetLastError();
  }
  cudaError_t leafgather() {
    cudaError_t e =
        rcount <= 1   ? launch_leafgather<float, 1>(dp, *S, s, kTcRhs, 0, rcount, yfar, st)
        : rcount <= 8 ? launch_leafgather<float, 8>(dp, *S, s, kTcRhs, 0, rcount, yfar, st)
                      : launch_leafgather<float, kTcRhs>(dp, *S, s, kTcRhs, 0, rcount, yfar, st);
    if (e != cudaSuccess) return e;
    dp->launches += dp->nleaves_r ? 1 : 0;
    dp->mark(FMCA_STAGE_LEAFGATHER, st);
    return cudaGetLastError();
  }
  // near field: groups of up to 256 targets as two halves of 128, or of up
  // to 128 targets as one half (halves = 1), one leaf per group or (pack,
  // one CTA per group) the rows of up to two leaves
  cudaError_t near(const UmCfg& uc, int halves, int pack = 0) {
    const bool pk = pack && halves == 1 && !uc.persist && dp->near_pk.ngroups > 0;
    const GroupList& gl = pk ? dp->near_pk : halves == 1 ? dp->near_h1 : dp->near;
    cudaError_t e =
        halves == 1
            ? launch_um<1>(gl, S->pts_r, w.pairs_c, xv, ynear, rcount, kp, 0, dp->err_flag, st,
                           false, uc, nullptr, dp->sms)
            : launch_um<2>(gl, S->pts_r, w.pairs_c, xv, ynear, rcount, kp, 0, dp->err_flag, st,
                           false, uc, nullptr, dp->sms);
    dp->launches += gl.ngroups ? 1 : 0;
    dp->mark(FMCA_STAGE_NEAR, st);
    return e;
  }
};

TcChunk tc_chunk(const Plan& plan, DevPlan* dp, DevSet<float>& S, const TcWorkspace& w,
                 const KParams<float>& kp, int nrhs, int ch, cudaStream_t st) {
  const int RB = kTcRhs, ld = kTcRhs;
  const int64_t nc = plan.cols.n, nr = plan.rows.n;
  const size_t q = plan.interp.q;
  TcChunk c;
  c.plan = &plan;
  c.dp = dp;
  c.S = &S;
  c.kp = kp;
  c.rcount = std::min(RB, nrhs - ch * RB);
  c.q = (int)q;
  c.Cc = plan.cols.nclusters();
  c.Cr = plan.rows.nclusters();
  c.npc = (int64_t)um_padded(nc);
  c.xc = w.xc + (size_t)ch * nc * ld;
  c.t = w.t + (size_t)ch * c.Cc * q * ld;
  c.s = w.s + (size_t)ch * c.Cr * q * ld;
  c.yfar = w.yfar + (size_t)ch * nr * ld;
  c.ynear = w.ynear + (size_t)ch * nr * ld;
  c.xv = w.xv + (size_t)ch * c.npc * ld * 2;
  c.w = w;
  c.st = st;
  return c;
}

int matvec_tc(const Plan& plan, DevPlan* dp, DevSet<float>& S, const KernelDesc& k,
              int dtype, int order, int nrhs, const void* x, int64_t sxi, int64_t sxr,
              void* y, int64_t syi, int64_t syr, void* ws, size_t wsb, cudaStream_t st,
              std::string* err, MatvecState* state = nullptr) {
  constexpr int RB = kTcRhs;
  const int ld = kTcRhs;
  const size_t need = tc_ws_layout(plan, nrhs, nullptr, nullptr);
  FMCA_TRY(acquire_ws(dp, need, &ws, wsb, st, err));
  TcWorkspace w;
  tc_ws_layout(plan, nrhs, ws, &w);
  if (state) {
    state->xc = w.xc;
    state->s = w.s;
    state->cmax = w.cmax;
    state->ld = ld;
    // up to 8 right-hand sides (tensor cores chosen by the autotuner): the
    // gradient terms read only the occupied columns of the 32-column layout
    state->rb = nrhs <= 8 ? rhs_block(nrhs) : RB;
    state->nch = (nrhs + RB - 1) / RB;
    state->fp64 = false;
  }
  dp->reset_marks();
  dp->mark(-1, st);
  const KParams<float> kp = tc_kparams(S, k, dp->opts);
  const uint32_t* pc = order == FMCA_ORDER_NATURAL ? dp->perm_c : nullptr;
  const uint32_t* pr = order == FMCA_ORDER_NATURAL ? dp->perm_r : nullptr;
  const int nthr = 256;
  auto blocks = [&](int64_t total) {
    int64_t b = (total + nthr - 1) / nthr;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)dp->sms * 32));
  };
  const int64_t nc = plan.cols.n, nr = plan.rows.n;
  const int nch = (nrhs + RB - 1) / RB;
  FMCA_CK(cudaMemsetAsync(w.cmax, 0, sizeof(unsigned int) * nrhs, st));
  constexpr int kColChunk = 4096;  // columns per colmax launch (16 KB shared)
  for (int c0 = 0; c0 < nrhs; c0 += kColChunk) {
    const int ncol = std::min(kColChunk, nrhs - c0);
    const size_t smem = sizeof(unsigned int) * ncol;
    if (dtype == FMCA_DTYPE_F64)
      colmax_kernel<double><<<dp->sms * 4, nthr, smem, st>>>(
          nc, c0, ncol, static_cast<const double*>(x), sxi, sxr, w.cmax);
    else
      colmax_kernel<float><<<dp->sms * 4, nthr, smem, st>>>(
          nc, c0, ncol, static_cast<const float*>(x), sxi, sxr, w.cmax);
    ++dp->launches;
  }
  const int64_t npc = (int64_t)um_padded(nc);
  const dim3 ggrid(blocks(npc / 8 * RB), nch);
  if (dtype == FMCA_DTYPE_F64)
    gather_split_kernel<double><<<ggrid, nthr, 0, st>>>(
        pc, nc, nrhs, static_cast<const double*>(x), sxi, sxr, w.cmax, w.xc, w.xv);
  else
    gather_split_kernel<float><<<ggrid, nthr, 0, st>>>(
        pc, nc, nrhs, static_cast<const float*>(x), sxi, sxr, w.cmax, w.xc, w.xv);
  if (um_near_dot(kp.type))
    point_pairs_dot_kernel<<<blocks(npc / 2), nthr, 0, st>>>(nc, S.pts_c, kp, w.pairs_c);
  else
    point_pairs_kernel<<<blocks(npc / 2), nthr, 0, st>>>(nc, S.pts_c, kp.g, w.pairs_c);
  FMCA_CK(cudaGetLastError());
  dp->launches += 2;
  dp->mark(FMCA_STAGE_GATHER, st);
  for (int ch = 0; ch < nch; ++ch) {
    TcChunk c = tc_chunk(plan, dp, S, w, kp, nrhs, ch, st);
    FMCA_CK(c.leafmom());
    FMCA_CK(c.m2m(dp->cfg.tr));
    FMCA_CK(c.far(dp->cfg));
    FMCA_CK(c.l2l(dp->cfg.tr));
    FMCA_CK(c.leafgather());
    FMCA_CK(c.near(dp->cfg.near, dp->cfg.near_halves, dp->cfg.near_pack));
  }
  if (dtype == FMCA_DTYPE_F64)
    scatter_scaled_kernel<double><<<blocks(nr * nrhs), nthr, 0, st>>>(
        pr, nr, nrhs, w.ynear, w.yfar, w.cmax, output_scale(k), static_cast<double*>(y), syi, syr);
  else
    scatter_scaled_kernel<float><<<blocks(nr * nrhs), nthr, 0, st>>>(
        pr, nr, nrhs, w.ynear, w.yfar, w.cmax, output_scale(k), static_cast<float*>(y), syi, syr);
  FMCA_CK(cudaGetLastError());
  ++dp->launches;
  dp->mark(FMCA_STAGE_SCATTER, st);
  return FMCA_OK;
}

}  // namespace

int upload(const Plan& plan, int precision, DevPlan** dev, std::string* err) {
  int cur = 0;
  FMCA_CK(cudaGetDevice(&cur));
  DevPlan* dp = *dev;
  if (!dp) {
    dp = new DevPlan();
    dp->device = cur;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cur) == cudaSuccess &&
        sms > 0)
      dp->sms = sms;
    dp->cfg = TuneCfg::defaults(dp->sms);
    int s = upload_common(plan, dp, err);
    if (s != FMCA_OK) {
      destroy(dp);
      return s;
    }
    *dev = dp;
  } else if (dp->device != cur) {
    *err = "plan was uploaded to device " + std::to_string(dp->device) +
           " but the current device is " + std::to_string(cur);
    return FMCA_ERR_INVALID_ARGUMENT;
  }
  if (precision == FMCA_PREC_FP64) return upload_set<double>(plan, dp, &dp->d, err);
  return upload_set<float>(plan, dp, &dp->f, err);
}

void destroy(DevPlan* dp) {
  if (!dp) return;
  int cur = -1;
  cudaGetDevice(&cur);
  if (dp->device >= 0 && dp->device != cur) cudaSetDevice(dp->device);
  for (void* p : dp->allocs) cudaFree(p);
  release_store(&dp->as);
  for (cudaEvent_t e : dp->events) cudaEventDestroy(e);
  if (dp->ws) cudaFree(dp->ws);
  if (dp->device >= 0 && dp->device != cur && cur >= 0) cudaSetDevice(cur);
  delete dp;
}

size_t workspace_bytes(const Plan& plan, int precision, int nrhs) {
  if (precision == FMCA_PREC_FP64) return ws_layout<double>(plan, nrhs, nullptr, nullptr);
  const size_t f = ws_layout<float>(plan, nrhs, nullptr, nullptr);
  if (precision == FMCA_PREC_FP32) return f;
  return std::max(f, tc_ws_layout(plan, nrhs, nullptr, nullptr));
}

namespace {

uint64_t tune_key(int precision, int type, int nrhs) {
  return (uint64_t)precision | ((uint64_t)type << 8) | ((uint64_t)std::min(nrhs, 33) << 16);
}

// the cached launch shapes of a key, or the defaults
TuneCfg config_for(const DevPlan* dp, int precision, int type, int nrhs) {
  auto it = dp->tuned.find(tune_key(precision, type, nrhs));
  return it != dp->tuned.end() ? it->second : TuneCfg::defaults(dp->sms);
}

bool stream_capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return true;
  return cs != cudaStreamCaptureStatusNone;
}

// The autotuner: measures the launch shapes of the mixed-precision matvec on
// this plan with CUDA events on the caller's stream and keeps the fastest in
// dp->cfg.  Steps (each trial timed twice, the faster counts):
//  1. fewer than 17 right-hand sides: one whole matvec on the FP32 CUDA
//     cores against the faster of two on the tensor cores (columns padded
//     to 32; near-field groups of two target halves and of one);
//  2. on the tensor-core path, after one matvec with the defaults has
//     filled the workspace, the stages of the first right-hand-side chunk
//     one by one: the near-field kernel sum with two target halves over
//     stage counts 4..7 and units of 1..3 tiles and with one half over 5..7
//     and 1..2; the far field (moment scaling + kernel sum) on
//     paired tensor grids (stages 4..6, units 1..3) and on nodes (stages
//     5..7, units 1..2); the upward and downward transfer passes over the
//     level thresholds {0, 2, 4, 8} x SMs (8 warps per cluster) and
//     {0, 1, 2, 4} x SMs (right-hand-side slices).
// The trials overwrite the workspace; the caller runs the real matvec with
// the chosen shapes afterwards.  Other precisions keep the defaults.
int tune(const Plan& plan, DevPlan* dp, const KernelDesc& k, int precision, int dtype,
         int order, int nrhs, const void* x, int64_t sxi, int64_t sxr, void* y, int64_t syi,
         int64_t syr, void* ws, size_t wsb, cudaStream_t st, std::string* err) {
  const auto t_begin = std::chrono::steady_clock::now();
  TuneCfg best = TuneCfg::defaults(dp->sms);
  dp->cfg = best;
  if (precision == FMCA_PREC_MIXED && tc_bounded(k.type)) {
    cudaEvent_t e0, e1;
    FMCA_CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      *err = "cudaEventCreate failed";
      return FMCA_ERR_CUDA;
    }
    const bool prof = dp->profile;
    dp->profile = false;  // no stage events inside the trials
    int status = FMCA_OK;
    // fastest of two runs of fn (ms); negative on a failure
    auto timed = [&](auto&& fn) -> float {
      float bestms = -1.f;
      for (int r = 0; r < 2; ++r) {
        if (cudaEventRecord(e0, st) != cudaSuccess) return -1.f;
        if (fn() != FMCA_OK) return -1.f;
        float ms = 0.f;
        if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
          return -1.f;
        if (bestms < 0.f || ms < bestms) bestms = ms;
      }
      return bestms;
    };
    auto run_tc = [&]() {
      return matvec_tc(plan, dp, dp->f, k, dtype, order, nrhs, x, sxi, sxr, y, syi, syr, ws, wsb,
                       st, err);
    };
    auto run_cc = [&]() {
      return matvec_t<float>(plan, dp, dp->f, k, dtype, order, nrhs, x, sxi, sxr, y, syi, syr,
                             ws, wsb, st, err);
    };
    auto ok_cuda = [](cudaError_t e) { return e == cudaSuccess ? FMCA_OK : FMCA_ERR_CUDA; };
    bool use_tc = nrhs > 16;
    if (!use_tc) {
      dp->cfg.small_tc = 0;
      const float t_cc = timed(run_cc);
      dp->cfg.small_tc = 1;
      const float t_tc = timed(run_tc);
      // the near field with one target half of 128 as well: leaves of up to
      // 128 points fill a third of two halves
      dp->cfg.near_halves = 1;
      dp->cfg.near = UmCfg{um_stages(1), 1};
      const float t_tc1 = timed(run_tc);
      dp->cfg = best;
      if (t_cc < 0.f || t_tc < 0.f || t_tc1 < 0.f) status = FMCA_ERR_CUDA;
      use_tc = std::min(t_tc, t_tc1) < t_cc;
      best.small_tc = use_tc ? 1 : 0;
    }
    if (status == FMCA_OK && use_tc) {
      dp->cfg = best;
      status = run_tc();
      if (status == FMCA_OK) {
        TcWorkspace w;
        tc_ws_layout(plan, nrhs, ws ? ws : dp->ws, &w);
        TcChunk c = tc_chunk(plan, dp, dp->f, w, tc_kparams(dp->f, k, dp->opts), nrhs, 0, st);
        float bt = -1.f;
        // one half: also the groups of two leaves' rows (packed)
        const int max_pack = dp->near_pk.ngroups > 0 ? 1 : 0;
        for (int halves = 2; halves >= 1 && status == FMCA_OK; --halves)
          for (int nst = halves == 2 ? 4 : 5; nst <= kUmMaxStages && status == FMCA_OK; ++nst)
            for (int F = 1; F <= (halves == 2 ? kUmMaxUnit : 2) && status == FMCA_OK; ++F)
              for (int pack = 0; pack <= (halves == 1 ? max_pack : 0); ++pack) {
                const UmCfg uc{nst, F};
                const float ms = timed([&]() { return ok_cuda(c.near(uc, halves, pack)); });
                if (ms < 0.f) {
                  status = FMCA_ERR_CUDA;
                  break;
                }
                if (bt < 0.f || ms < bt) {
                  bt = ms;
                  best.near = uc;
                  best.near_halves = halves;
                  best.near_pack = pack;
                }
              }
        if (status == FMCA_OK) {  // the fastest shape as a persistent launch (one leaf per group)
          UmCfg uc = best.near;
          uc.persist = 1;
          const float ms = timed([&]() { return ok_cuda(c.near(uc, best.near_halves)); });
          if (ms < 0.f) {
            status = FMCA_ERR_CUDA;
          } else if (ms < bt) {
            best.near = uc;
            best.near_pack = 0;
          }
        }
        bt = -1.f;
        // the Gaussian's Kronecker far field first (the default where it
        // applies), then the tensor-core kernel sums
        best.far_kron = 0;
        if (far_kron_ok(dp, dp->f, k.type, std::min(nrhs, kTcRhs))) {
          TuneCfg cand = best;
          cand.far_kron = 1;
          const float ms = timed([&]() { return ok_cuda(c.far(cand)); });
          if (ms < 0.f)
            status = FMCA_ERR_CUDA;
          else {
            bt = ms;
            best.far_kron = 1;
          }
        }
        const bool grid = grid_far(plan);
        for (int pairs = grid ? 1 : 0; pairs >= 0 && status == FMCA_OK; --pairs)
          for (int nst = pairs ? 4 : 5; nst <= (pairs ? 6 : 7); ++nst)
            for (int F = 1; F <= (pairs ? 3 : 2); ++F) {
              TuneCfg cand = best;
              cand.far_kron = 0;
              cand.far_pairs = pairs;
              (pairs ? cand.far_grid : cand.far_nodes) = UmCfg{nst, F};
              const float ms = timed([&]() { return ok_cuda(c.far(cand)); });
              if (ms < 0.f) {
                status = FMCA_ERR_CUDA;
                break;
              }
              if (bt < 0.f || ms < bt) {
                bt = ms;
                best.far_kron = 0;
                best.far_pairs = cand.far_pairs;
                best.far_grid = cand.far_grid;
                best.far_nodes = cand.far_nodes;
              }
            }
        if (status == FMCA_OK && !best.far_kron) {  // the fastest shape as a persistent launch
          TuneCfg cand = best;
          (cand.far_pairs && grid ? cand.far_grid : cand.far_nodes).persist = 1;
          const float ms = timed([&]() { return ok_cuda(c.far(cand)); });
          if (ms < 0.f) {
            status = FMCA_ERR_CUDA;
          } else if (ms < bt) {
            best.far_grid = cand.far_grid;
            best.far_nodes = cand.far_nodes;
          }
        }
        bt = -1.f;
        for (int wide : {0, 2, 4, 8})
          for (int slice : {0, 1, 2, 4}) {
            if (status != FMCA_OK) break;
            const TrCfg tr{wide * dp->sms, slice * dp->sms};
            const float ms = timed([&]() {
              cudaError_t e = c.m2m(tr);
              return ok_cuda(e == cudaSuccess ? c.l2l(tr) : e);
            });
            if (ms < 0.f) {
              status = FMCA_ERR_CUDA;
              break;
            }
            if (bt < 0.f || ms < bt) {
              bt = ms;
              best.tr = tr;
            }
          }
      }
    }
    dp->profile = prof;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status != FMCA_OK) {
      if (err->empty()) *err = std::string("autotuner: ") + cudaGetErrorString(cudaGetLastError());
      return status;
    }
  }
  best.tuned = 1;
  best.tune_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() -
                                                          t_begin).count();
  dp->tuned[tune_key(precision, k.type, nrhs)] = best;
  ++dp->tunings;
  dp->cfg = best;
  return FMCA_OK;
}

// sets the call's options and launch shapes (tuning them first if the
// autotuner is on and this key has none yet, outside stream captures)
int prepare_call(const Plan& plan, DevPlan* dp, const KernelDesc& k, int precision, int dtype,
                 int order, int nrhs, const void* x, int64_t sxi, int64_t sxr, void* y,
                 int64_t syi, int64_t syr, void* ws, size_t wsb, cudaStream_t st,
                 std::string* err, const CallOpts& opts, bool may_tune) {
  dp->opts = opts;
  dp->profile = opts.profile;
  dp->cfg = config_for(dp, precision, k.type, nrhs);
  if (may_tune && opts.autotune && !dp->cfg.tuned && !stream_capturing(st))
    return tune(plan, dp, k, precision, dtype, order, nrhs, x, sxi, sxr, y, syi, syr, ws, wsb,
                st, err);
  return FMCA_OK;
}

}  // namespace

int matvec(const Plan& plan, DevPlan* dp, const KernelDesc& k, int precision,
           int dtype, int order, int nrhs, const void* x, int64_t sxi,
           int64_t sxr, void* y, int64_t syi, int64_t syr, void* ws,
           size_t ws_bytes, cudaStream_t st, std::string* err, const CallOpts& opts) {
  std::lock_guard<std::mutex> lock(dp->mu);
  FMCA_TRY(prepare_call(plan, dp, k, precision, dtype, order, nrhs, x, sxi, sxr, y, syi, syr,
                        ws, ws_bytes, st, err, opts, true));
  if (precision == FMCA_PREC_FP64)
    return matvec_t<double>(plan, dp, dp->d, k, dtype, order, nrhs, x, sxi, sxr, y,
                            syi, syr, ws, ws_bytes, st, err);
  if (precision == FMCA_PREC_MIXED && tc_supported(k.type, nrhs, dp->cfg.small_tc))
    return matvec_tc(plan, dp, dp->f, k, dtype, order, nrhs, x, sxi, sxr, y, syi, syr, ws,
                     ws_bytes, st, err);
  return matvec_t<float>(plan, dp, dp->f, k, dtype, order, nrhs, x, sxi, sxr, y, syi,
                         syr, ws, ws_bytes, st, err);
}

// ---------------------------------------------------------------------------
// assembled plans (fmca_plan_assemble, fmca_matvec_assembled)
namespace {

// Stored elements and groups of the assembled blocks, from the host plan:
// the groups of the CUDA-core lists (far: the nodes of every row cluster,
// near: the points of every row leaf, both chunked to kGroupCap targets),
// each a block of (its sources) x (its targets rounded up to 4).
void asm_counts(const Plan& plan, uint64_t* elems, uint64_t* groups) {
  auto chunks = [](uint32_t tc, uint64_t* ng) {
    uint64_t rows = 0;
    for (uint32_t o = 0; o < tc; o += kGroupCap) {
      rows += asm_row_stride(std::min<uint32_t>(kGroupCap, tc - o));
      ++*ng;
    }
    return rows;
  };
  const Pattern& P = plan.pat;
  const uint64_t q = plan.interp.q;
  uint64_t e = 0, ng = 0;
  for (int c = 0; c < plan.rows.nclusters(); ++c)
    e += (uint64_t)(P.far_ptr[c + 1] - P.far_ptr[c]) * q * chunks((uint32_t)q, &ng);
  for (size_t l = 0; l < plan.row_leaves.size(); ++l) {
    uint64_t ns = 0;
    for (int k = P.near_ptr[l]; k < P.near_ptr[l + 1]; ++k)
      ns += P.near_ivl[2 * k + 1] - P.near_ivl[2 * k];
    e += ns * chunks(plan.rows.size[plan.row_leaves[l]], &ng);
  }
  *elems = e;
  *groups = ng;
}

// per-group element offsets of one device group list's blocks and their sum
int asm_offsets(const GroupList& gl, std::vector<uint64_t>* off, uint64_t* total,
                std::string* err) {
  off->assign(gl.ngroups, 0);
  *total = 0;
  if (!gl.ngroups) return FMCA_OK;
  std::vector<KGroup> g(gl.ngroups);
  FMCA_CK(cudaMemcpy(g.data(), gl.groups, sizeof(KGroup) * g.size(), cudaMemcpyDeviceToHost));
  int nivl = 0;
  for (const KGroup& x : g) nivl = std::max(nivl, x.ivl_end);
  std::vector<uint32_t> iv((size_t)2 * nivl);
  if (nivl)
    FMCA_CK(cudaMemcpy(iv.data(), gl.ivl, sizeof(uint32_t) * iv.size(), cudaMemcpyDeviceToHost));
  uint64_t o = 0;
  for (int i = 0; i < gl.ngroups; ++i) {
    uint64_t ns = 0;
    for (int k = g[i].ivl_begin; k < g[i].ivl_end; ++k) ns += iv[2 * k + 1] - iv[2 * k];
    (*off)[i] = o;
    o += ns * asm_row_stride(g[i].tcount);
  }
  *total = o;
  return FMCA_OK;
}

template <typename T>
int assemble_t(DevPlan* dp, DevSet<T>& S, const KernelDesc& k, int precision,
               cudaStream_t st, std::string* err) {
  std::vector<uint64_t> foff, noff;
  uint64_t fe = 0, ne = 0;
  FMCA_TRY(asm_offsets(dp->far, &foff, &fe, err));
  FMCA_TRY(asm_offsets(dp->near, &noff, &ne, err));
  AsmStore& a = dp->as;
  auto grab = [&](size_t bytes, void** out) -> int {
    *out = nullptr;
    if (!bytes) return FMCA_OK;
    FMCA_CK(cudaMalloc(out, bytes));
    a.bytes += bytes;
    return FMCA_OK;
  };
  int s = grab(fe * sizeof(T), &a.far);
  if (s == FMCA_OK) s = grab(ne * sizeof(T), &a.near);
  if (s == FMCA_OK) s = grab(foff.size() * sizeof(uint64_t), (void**)&a.far_off);
  if (s == FMCA_OK) s = grab(noff.size() * sizeof(uint64_t), (void**)&a.near_off);
  if (s == FMCA_OK && !foff.empty() &&
      cudaMemcpy(a.far_off, foff.data(), foff.size() * sizeof(uint64_t),
                 cudaMemcpyHostToDevice) != cudaSuccess)
    s = FMCA_ERR_CUDA;
  if (s == FMCA_OK && !noff.empty() &&
      cudaMemcpy(a.near_off, noff.data(), noff.size() * sizeof(uint64_t),
                 cudaMemcpyHostToDevice) != cudaSuccess)
    s = FMCA_ERR_CUDA;
  const KParams<T> kp = make_kparams<T>(k, dp->opts);
  cudaError_t e = cudaSuccess;
  if (s == FMCA_OK)
    e = launch_kstore<T>(dp->far.groups, dp->far.ngroups, dp->far.ivl, a.far_off, S.nodes_r,
                         S.nodes_c, kp, static_cast<T*>(a.far), st);
  if (s == FMCA_OK && e == cudaSuccess)
    e = launch_kstore<T>(dp->near.groups, dp->near.ngroups, dp->near.ivl, a.near_off, S.pts_r,
                         S.pts_c, kp, static_cast<T*>(a.near), st);
  if (s == FMCA_OK && e != cudaSuccess) {
    *err = std::string("storing the blocks failed: ") + cudaGetErrorString(e);
    s = FMCA_ERR_CUDA;
  }
  if (s != FMCA_OK) {
    if (err->empty()) *err = "assembling the plan failed (device memory)";
    release_store(&dp->as);
    return s;
  }
  dp->launches = (dp->far.ngroups ? 1 : 0) + (dp->near.ngroups ? 1 : 0);
  a.precision = precision;
  a.k = k;
  return FMCA_OK;
}

}  // namespace

size_t assembled_bytes(const Plan& plan, int precision) {
  uint64_t e = 0, g = 0;
  asm_counts(plan, &e, &g);
  return (size_t)(e * (precision == FMCA_PREC_FP64 ? 8 : 4) + g * sizeof(uint64_t));
}

int assemble(const Plan& plan, DevPlan* dp, const KernelDesc& k, int precision,
             cudaStream_t st, std::string* err, const CallOpts& opts) {
  (void)plan;
  std::lock_guard<std::mutex> lock(dp->mu);
  if (dp->far.maxcount > kAsmMaxTargets || dp->near.maxcount > kAsmMaxTargets) {
    *err = "group larger than the assembled stream supports";
    return FMCA_ERR_UNSUPPORTED;
  }
  release_store(&dp->as);
  dp->opts = opts;
  dp->profile = false;
  if (precision == FMCA_PREC_FP64) return assemble_t<double>(dp, dp->d, k, precision, st, err);
  return assemble_t<float>(dp, dp->f, k, precision, st, err);
}

void release_assembled(DevPlan* dp) {
  if (!dp) return;
  std::lock_guard<std::mutex> lock(dp->mu);
  release_store(&dp->as);
}

int assembled_precision(DevPlan* dp) {
  if (!dp) return -1;
  std::lock_guard<std::mutex> lock(dp->mu);
  return dp->as.precision;
}

int matvec_assembled(const Plan& plan, DevPlan* dp, int precision, int dtype, int order,
                     int nrhs, const void* x, int64_t sxi, int64_t sxr, void* y, int64_t syi,
                     int64_t syr, void* ws, size_t ws_bytes, cudaStream_t st, std::string* err,
                     const CallOpts& opts) {
  std::lock_guard<std::mutex> lock(dp->mu);
  if (dp->as.precision < 0) {
    *err = "the plan holds no assembled blocks (fmca_plan_assemble)";
    return FMCA_ERR_INVALID_ARGUMENT;
  }
  if ((precision == FMCA_PREC_FP64) != (dp->as.precision == FMCA_PREC_FP64)) {
    *err = "the plan's blocks were assembled in another precision (FP64 blocks serve "
           "FMCA_PREC_FP64, FP32 blocks FMCA_PREC_FP32 and FMCA_PREC_MIXED)";
    return FMCA_ERR_INVALID_ARGUMENT;
  }
  dp->opts = opts;
  dp->profile = opts.profile;
  dp->cfg = TuneCfg::defaults(dp->sms);
  if (precision == FMCA_PREC_FP64)
    return matvec_t<double>(plan, dp, dp->d, dp->as.k, dtype, order, nrhs, x, sxi, sxr, y, syi,
                            syr, ws, ws_bytes, st, err, nullptr, &dp->as);
  return matvec_t<float>(plan, dp, dp->f, dp->as.k, dtype, order, nrhs, x, sxi, sxr, y, syi,
                         syr, ws, ws_bytes, st, err, nullptr, &dp->as);
}

void tuned_config(DevPlan* dp, int precision, int type, int nrhs, int32_t* out) {
  for (int i = 0; i < FMCA_TUNE_COUNT; ++i) out[i] = 0;
  TuneCfg c = TuneCfg::defaults(dp ? dp->sms : 152);
  if (dp) {
    std::lock_guard<std::mutex> lock(dp->mu);
    c = config_for(dp, precision, type, nrhs);
    out[FMCA_TUNE_TUNINGS] = (int32_t)dp->tunings;
  }
  const bool pairs = c.far_pairs != 0;
  out[FMCA_TUNE_TUNED] = c.tuned;
  out[FMCA_TUNE_NEAR_STAGES] = c.near.nst;
  out[FMCA_TUNE_NEAR_UNIT] = c.near.F;
  out[FMCA_TUNE_FAR_PAIRS] = c.far_pairs;
  out[FMCA_TUNE_FAR_GRID_STAGES] = c.far_grid.nst;
  out[FMCA_TUNE_FAR_GRID_UNIT] = c.far_grid.F;
  out[FMCA_TUNE_FAR_NODE_STAGES] = c.far_nodes.nst;
  out[FMCA_TUNE_FAR_NODE_UNIT] = c.far_nodes.F;
  out[FMCA_TUNE_WIDE_BELOW] = c.tr.wide_below;
  out[FMCA_TUNE_SLICE_BELOW] = c.tr.slice_below;
  out[FMCA_TUNE_SMALL_R_TENSOR] = c.small_tc;
  out[FMCA_TUNE_NEAR_HALVES] = c.near_halves;
  out[FMCA_TUNE_NEAR_PERSIST] = c.near.persist;
  // the tuner sets it on the far-field form the plan uses
  out[FMCA_TUNE_FAR_PERSIST] = c.far_grid.persist | c.far_nodes.persist;
  out[FMCA_TUNE_US] = (int32_t)(c.tune_ms * 1000.f);
  out[FMCA_TUNE_FAR_KRON] = c.far_kron;
  out[FMCA_TUNE_NEAR_PACK] = c.near_pack;
  (void)pairs;
}

int set_tuned_config(DevPlan* dp, int precision, int type, int nrhs, const int32_t* in,
                     std::string* err) {
  auto um_ok = [](int nst, int F) {
    return nst >= 2 && nst <= kUmMaxStages && F >= 1 && F <= kUmMaxUnit && F <= nst;
  };
  if (!um_ok(in[FMCA_TUNE_NEAR_STAGES], in[FMCA_TUNE_NEAR_UNIT]) ||
      !um_ok(in[FMCA_TUNE_FAR_GRID_STAGES], in[FMCA_TUNE_FAR_GRID_UNIT]) ||
      !um_ok(in[FMCA_TUNE_FAR_NODE_STAGES], in[FMCA_TUNE_FAR_NODE_UNIT]) ||
      (in[FMCA_TUNE_FAR_PAIRS] != 0 && in[FMCA_TUNE_FAR_PAIRS] != 1) ||
      (in[FMCA_TUNE_SMALL_R_TENSOR] != 0 && in[FMCA_TUNE_SMALL_R_TENSOR] != 1) ||
      (in[FMCA_TUNE_NEAR_HALVES] != 1 && in[FMCA_TUNE_NEAR_HALVES] != 2) ||
      (in[FMCA_TUNE_NEAR_PERSIST] != 0 && in[FMCA_TUNE_NEAR_PERSIST] != 1) ||
      (in[FMCA_TUNE_FAR_PERSIST] != 0 && in[FMCA_TUNE_FAR_PERSIST] != 1) ||
      (in[FMCA_TUNE_FAR_KRON] != 0 && in[FMCA_TUNE_FAR_KRON] != 1) ||
      (in[FMCA_TUNE_NEAR_PACK] != 0 && in[FMCA_TUNE_NEAR_PACK] != 1) ||
      in[FMCA_TUNE_WIDE_BELOW] < 0 || in[FMCA_TUNE_SLICE_BELOW] < 0) {
    *err = "launch shapes out of range (stages 2..7, units 1..min(3, stages), flags 0/1, "
           "halves 1/2, thresholds >= 0)";
    return FMCA_ERR_INVALID_ARGUMENT;
  }
  if (in[FMCA_TUNE_NEAR_PACK] && dp->near_pk.ngroups == 0) {
    *err = "near_pack: this plan has no packed near groups (they would not save a tenth of "
           "the groups of one leaf each)";
    return FMCA_ERR_INVALID_ARGUMENT;
  }
  TuneCfg c = TuneCfg::defaults(dp->sms);
  c.near = UmCfg{in[FMCA_TUNE_NEAR_STAGES], in[FMCA_TUNE_NEAR_UNIT], in[FMCA_TUNE_NEAR_PERSIST]};
  c.near_halves = in[FMCA_TUNE_NEAR_HALVES];
  c.far_pairs = in[FMCA_TUNE_FAR_PAIRS];
  c.far_grid = UmCfg{in[FMCA_TUNE_FAR_GRID_STAGES], in[FMCA_TUNE_FAR_GRID_UNIT],
                     in[FMCA_TUNE_FAR_PERSIST]};
  c.far_nodes = UmCfg{in[FMCA_TUNE_FAR_NODE_STAGES], in[FMCA_TUNE_FAR_NODE_UNIT],
                      in[FMCA_TUNE_FAR_PERSIST]};
  c.tr = TrCfg{in[FMCA_TUNE_WIDE_BELOW], in[FMCA_TUNE_SLICE_BELOW]};
  c.small_tc = in[FMCA_TUNE_SMALL_R_TENSOR];
  c.far_kron = in[FMCA_TUNE_FAR_KRON];
  c.near_pack = in[FMCA_TUNE_NEAR_PACK];
  c.tuned = 1;
  std::lock_guard<std::mutex> lock(dp->mu);
  dp->tuned[tune_key(precision, type, nrhs)] = c;
  return FMCA_OK;
}

// ---------------------------------------------------------------------------
// adjoint
namespace {

// blocks of the dot-product reduction (its partial sums live in the
// workspace, so the count is fixed: 4 per SM of a 152-SM GB300)
constexpr int kDotBlocks = 152 * 4;

// z (contiguous n_r x R column-major, dtype of x) = K x
int matvec_state(const Plan& plan, DevPlan* dp, const KernelDesc& k, int precision,
                 int dtype, int nrhs, const void* x, int64_t sxi, int64_t sxr, void* z,
                 void* ws, size_t wsb, cudaStream_t st, std::string* err, MatvecState* state) {
  const int64_t nr = plan.rows.n;
  if (precision == FMCA_PREC_FP64)
    return matvec_t<double>(plan, dp, dp->d, k, dtype, FMCA_ORDER_NATURAL, nrhs, x, sxi, sxr,
                            z, 1, nr, ws, wsb, st, err, state);
  if (precision == FMCA_PREC_MIXED && tc_supported(k.type, nrhs, dp->cfg.small_tc))
    return matvec_tc(plan, dp, dp->f, k, dtype, FMCA_ORDER_NATURAL, nrhs, x, sxi, sxr, z, 1, nr,
                     ws, wsb, st, err, state);
  return matvec_t<float>(plan, dp, dp->f, k, dtype, FMCA_ORDER_NATURAL, nrhs, x, sxi, sxr, z,
                         1, nr, ws, wsb, st, err, state);
}

// out[idx] = scale * sum_{i,r} a[i, r] b[i, r]; a strided, b contiguous
// (n x R column-major); both of dtype
cudaError_t launch_dot(int dtype, int64_t n, int R, const void* a, int64_t sai, int64_t sar,
                       const void* b, double* partial, double scale, double* out, int idx,
                       cudaStream_t st) {
  if (dtype == FMCA_DTYPE_F64)
    dot_partial_kernel<double, double><<<kDotBlocks, 256, 0, st>>>(
        n, R, static_cast<const double*>(a), sai, sar, static_cast<const double*>(b), 1, n,
        partial);
  else
    dot_partial_kernel<float, float><<<kDotBlocks, 256, 0, st>>>(
        n, R, static_cast<const float*>(a), sai, sar, static_cast<const float*>(b), 1, n,
        partial);
  dot_final_kernel<<<1, 256, 0, st>>>(partial, kDotBlocks, scale, out, idx);
  return cudaGetLastError();
}

__global__ void set_scalar_kernel(double* out, int idx, double v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) out[idx] = v;
}

// tval2 / sval2 given: the symmetric form (both sides of the adjoint from one
// evaluation per pair; one point cloud)
// ofs: column offsets of tval, sval, tval2, sval2 in their rows
template <typename T, int RB>
cudaError_t launch_near_grad(const GroupList& gl, const Pt4<T>* tgt, const Pt4<T>* src,
                             const T* tval, const T* sval, int ld, const double* cs,
                             int rcount, const KParams<T>& kp, double scale, double* G,
                             int* errf, cudaStream_t st, const T* tval2 = nullptr,
                             const T* sval2 = nullptr, int4 ofs = {0, 0, 0, 0}) {
  if (gl.ngroups == 0) return cudaSuccess;
  constexpr int TS = TileSize<T>::value;
  const bool sym = tval2 && sval2;
  const bool two = sym && sval2 != sval;
  const size_t smem =
      128 + (size_t)kStages * TS * (sizeof(Pt4<T>) + (two ? 2 : 1) * (size_t)ld * sizeof(T));
  const int threads = std::max(32, (gl.maxcount + 31) / 32 * 32);
  if (sym) {
    auto kern = near_grad_kernel<T, RB, TS, kStages, true>;
    ensure_smem(kern, smem);
    kern<<<gl.ngroups, threads, smem, st>>>(gl.groups, gl.ivl, tgt, src, tval, sval, ld, cs,
                                            rcount, kp, scale, G, errf, tval2, sval2, ofs);
  } else {
    auto kern = near_grad_kernel<T, RB, TS, kStages, false>;
    ensure_smem(kern, smem);
    kern<<<gl.ngroups, threads, smem, st>>>(gl.groups, gl.ivl, tgt, src, tval, sval, ld, cs,
                                            rcount, kp, scale, G, errf, nullptr, nullptr, ofs);
  }
  return cudaGetLastError();
}

// U2 / tval2 given: both sides of the adjoint in one pass; ofs: column
// offsets of U, tval, U2, tval2 in their rows
template <typename T, int RB>
cudaError_t launch_far_grad(const Plan& plan, DevPlan* dp, DevSet<T>& S, const T* U,
                            const T* tval, int ld, const double* cs, int rcount,
                            double scale, double* G, cudaStream_t st, const T* U2 = nullptr,
                            const T* tval2 = nullptr, int4 ofs = {0, 0, 0, 0}) {
  if (!dp->nleaves_r) return cudaSuccess;
  auto kern = far_grad_kernel<T, RB>;
  const size_t smem = (128 * 48 + (U2 ? 2 : 1) * 64 * RB) * sizeof(T) +
                      (size_t)plan.interp.q * 3 * sizeof(int);
  ensure_smem(kern, smem);
  kern<<<dp->nleaves_r, 128, smem, st>>>(dp->leaves_r, dp->cbegin_r, dp->csize_r, S.bbmin_r,
                                         S.bbext_r, S.pts_r, U, tval, ld, cs, rcount,
                                         dp->midx, S.ip, scale, G, U2, tval2, ofs);
  return cudaGetLastError();
}

template <typename T>
int grad_terms(const Plan& plan, DevPlan* dp, DevSet<T>& S, const KernelDesc& k,
               const MatvecState& A, const MatvecState& B, int nrhs, const double* cs,
               double scale, double* G, cudaStream_t st, std::string* err) {
  const KParams<T> kp = make_kparams<T>(k);
  const size_t q = plan.interp.q;
  const int64_t nr = plan.rows.n, nc = plan.cols.n;
  const size_t Cr = plan.rows.nclusters();
  const int ld = A.ld, rb = A.rb;
  // the two sides (x: A, y: B) may share buffers at different column offsets
  const int4 nofs = {B.cofs, A.cofs, A.cofs, B.cofs};  // near: y_t, x_s, x_t, y_s
  const int4 fofs = {A.cofs, B.cofs, B.cofs, A.cofs};  // far: U_x, y_t, U_y, x_t
  for (int ch = 0; ch < A.nch; ++ch) {
    const int rcount = std::min(rb, nrhs - ch * rb);
    const T* xa = static_cast<const T*>(A.xc) + (size_t)ch * nc * ld;
    const T* yb = static_cast<const T*>(B.xc) + (size_t)ch * nr * ld;
    const T* ua = static_cast<const T*>(A.s) + (size_t)ch * Cr * q * ld;
    const T* ub = static_cast<const T*>(B.s) + (size_t)ch * Cr * q * ld;
    const double* csc = cs + ch * rb;
    // one point cloud (the adjoint refuses point gradients otherwise): both
    // sides, y_t x_s and x_t y_s, in one pass over the dense pairs and one
    // over the row leaves
    cudaError_t e = cudaSuccess;
    switch (rb) {
      case 1:
        e = launch_near_grad<T, 1>(dp->near, S.pts_r, S.pts_c, yb, xa, ld, csc, rcount, kp,
                                   scale, G, dp->err_flag, st, xa, yb, nofs);
        if (e == cudaSuccess)
          e = launch_far_grad<T, 1>(plan, dp, S, ua, yb, ld, csc, rcount, scale, G, st, ub, xa,
                                    fofs);
        break;
      case 8:
        e = launch_near_grad<T, 8>(dp->near, S.pts_r, S.pts_c, yb, xa, ld, csc, rcount, kp,
                                   scale, G, dp->err_flag, st, xa, yb, nofs);
        if (e == cudaSuccess)
          e = launch_far_grad<T, 8>(plan, dp, S, ua, yb, ld, csc, rcount, scale, G, st, ub, xa,
                                    fofs);
        break;
      default:
        e = launch_near_grad<T, 32>(dp->near, S.pts_r, S.pts_c, yb, xa, ld, csc, rcount, kp,
                                    scale, G, dp->err_flag, st, xa, yb, nofs);
        if (e == cudaSuccess)
          e = launch_far_grad<T, 32>(plan, dp, S, ua, yb, ld, csc, rcount, scale, G, st, ub,
                                     xa, fofs);
        break;
    }
    FMCA_CK(e);
  }
  return FMCA_OK;
}

struct AdjointWorkspace {
  void *wsA, *wsB;
  size_t mv;
  void* z;   // dtype of the inputs, n x 2 nrhs
  void* xy;  // [x | y] for the joint product K [x | y] (n x 2 nrhs), dtype
  double *G, *partial, *colscale, *scal;
};

// K x and K y run as one product of 2 nrhs columns when those fit one
// 32-column chunk (every kernel value then serves both)
bool adjoint_joint(int nrhs) { return 2 * nrhs <= 32; }

size_t adjoint_layout(const Plan& plan, int precision, int nrhs, void* base,
                      AdjointWorkspace* w) {
  size_t mvb = workspace_bytes(plan, precision, nrhs);
  if (adjoint_joint(nrhs)) mvb = std::max(mvb, workspace_bytes(plan, precision, 2 * nrhs));
  const size_t mv = align_up(mvb);
  const size_t n = std::max<size_t>(plan.rows.n, plan.cols.n);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* p = base ? static_cast<char*>(base) + off : nullptr;
    off += align_up(bytes);
    return p;
  };
  AdjointWorkspace t;
  t.mv = mv;
  t.wsA = take(mv);
  t.wsB = take(mv);
  t.z = take(sizeof(double) * n * 2 * nrhs);
  t.xy = adjoint_joint(nrhs) ? take(sizeof(double) * n * 2 * nrhs) : nullptr;
  t.G = (double*)take(sizeof(double) * 4 * std::max<size_t>(plan.rows.n, plan.cols.n));
  t.partial = (double*)take(sizeof(double) * kDotBlocks);
  t.colscale = (double*)take(sizeof(double) * nrhs);
  t.scal = (double*)take(sizeof(double) * 8);
  if (w) *w = t;
  return off;
}

}  // namespace

size_t adjoint_workspace_bytes(const Plan& plan, int precision, int nrhs) {
  return adjoint_layout(plan, precision, nrhs, nullptr, nullptr);
}

int adjoint(const Plan& plan, DevPlan* dp, const KernelDesc& k, int precision, int dtype,
            int nrhs, const void* x, int64_t sxi, int64_t sxr, const void* y, int64_t syi,
            int64_t syr, double* values, void* dX, int64_t sdi, int64_t sdd, void* Kx, void* Ky,
            void* ws, size_t wsb, cudaStream_t st, std::string* err, const CallOpts& opts) {
  std::lock_guard<std::mutex> lock(dp->mu);
  // launch shapes: those tuned for this key by matvecs, if any (the adjoint
  // does not tune)
  FMCA_TRY(prepare_call(plan, dp, k, precision, dtype, FMCA_ORDER_NATURAL, nrhs, x, sxi, sxr,
                        nullptr, 0, 0, ws, wsb, st, err, opts, false));
  const bool base_kernel = k.type >= FMCA_KERNEL_EXPONENTIAL && k.type <= FMCA_KERNEL_GAUSSIAN;
  if ((dX || Ky) && !plan.same_tree) {
    *err = "gradients w.r.t. the points and K^T y need one point cloud (Pr == Pc)";
    return FMCA_ERR_UNSUPPORTED;
  }
  if (dX && !base_kernel) {
    *err = "point gradients are implemented for EXPONENTIAL, MATERN32, MATERN52, GAUSSIAN";
    return FMCA_ERR_UNSUPPORTED;
  }
  const size_t need = adjoint_layout(plan, precision, nrhs, nullptr, nullptr);
  FMCA_TRY(acquire_ws(dp, need, &ws, wsb, st, err));
  AdjointWorkspace w;
  adjoint_layout(plan, precision, nrhs, ws, &w);
  KernelDesc k1 = k;
  k1.sigma2 = 1.0;
  const int64_t nr = plan.rows.n, nc = plan.cols.n;
  const int nthr = 256;
  auto blocks = [&](int64_t total) {
    int64_t b = (total + nthr - 1) / nthr;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)dp->sms * 32));
  };
  MatvecState A, B;
  // with point gradients or K y on one point cloud and few right-hand
  // sides, K x and K y come from one product of [x | y]: its first nrhs
  // columns are the x side (state A), the others the y side (state B)
  const bool joint = (dX || Ky) && plan.same_tree && adjoint_joint(nrhs);
  if (joint) {
    if (dtype == FMCA_DTYPE_F64)
      pack_pair_kernel<double><<<blocks(nr * 2 * nrhs), nthr, 0, st>>>(
          nr, nrhs, static_cast<const double*>(x), sxi, sxr, static_cast<const double*>(y), syi,
          syr, static_cast<double*>(w.xy));
    else
      pack_pair_kernel<float><<<blocks(nr * 2 * nrhs), nthr, 0, st>>>(
          nr, nrhs, static_cast<const float*>(x), sxi, sxr, static_cast<const float*>(y), syi,
          syr, static_cast<float*>(w.xy));
    FMCA_CK(cudaGetLastError());
    FMCA_TRY(matvec_state(plan, dp, k1, precision, dtype, 2 * nrhs, w.xy, 1, nr, w.z, w.wsA,
                          w.mv, st, err, &A));
    B = A;
    B.cofs = nrhs;
  } else {
    // z = K x with unit variance
    FMCA_TRY(matvec_state(plan, dp, k1, precision, dtype, nrhs, x, sxi, sxr, w.z, w.wsA, w.mv,
                          st, err, &A));
  }
  // f = sigma2 * y . K x, df/dsigma2 = y . K x
  FMCA_CK(launch_dot(dtype, nr, nrhs, y, syi, syr, w.z, w.partial, 1.0, w.scal, 0, st));
  if (values) {
    scalar_axpy_kernel<<<1, 32, 0, st>>>(w.scal, 0, k.sigma2, values, 0);
    scalar_axpy_kernel<<<1, 32, 0, st>>>(w.scal, 0, 1.0, values, 2);
  }
  if (Kx) {
    if (dtype == FMCA_DTYPE_F64)
      scale_copy_kernel<double><<<blocks(nr * nrhs), nthr, 0, st>>>(
          nr, nrhs, static_cast<const double*>(w.z), k.sigma2, static_cast<double*>(Kx), syi,
          syr);
    else
      scale_copy_kernel<float><<<blocks(nr * nrhs), nthr, 0, st>>>(
          nr, nrhs, static_cast<const float*>(w.z), k.sigma2, static_cast<float*>(Kx), syi,
          syr);
  }
  // K y of the joint product, before z is reused below
  if (joint && Ky) {
    const size_t zofs = (size_t)nr * nrhs * (dtype == FMCA_DTYPE_F64 ? 8 : 4);
    const void* zy = static_cast<const char*>(w.z) + zofs;
    if (dtype == FMCA_DTYPE_F64)
      scale_copy_kernel<double><<<blocks(nc * nrhs), nthr, 0, st>>>(
          nc, nrhs, static_cast<const double*>(zy), k.sigma2, static_cast<double*>(Ky), sxi,
          sxr);
    else
      scale_copy_kernel<float><<<blocks(nc * nrhs), nthr, 0, st>>>(
          nc, nrhs, static_cast<const float*>(zy), k.sigma2, static_cast<float*>(Ky), sxi, sxr);
  }
  // df/dl = sigma2 * y . H2[dk/dl] x
  if (values) {
    if (base_kernel) {
      KernelDesc kd = k1;
      kd.type = k.type + K_DL_EXPONENTIAL;
      FMCA_TRY(matvec_state(plan, dp, kd, precision, dtype, nrhs, x, sxi, sxr, w.z, w.wsB,
                            w.mv, st, err, nullptr));
      FMCA_CK(launch_dot(dtype, nr, nrhs, y, syi, syr, w.z, w.partial, k.sigma2, values, 1,
                         st));
    } else {
      set_scalar_kernel<<<1, 32, 0, st>>>(values, 1, std::nan(""));
    }
  }
  if ((dX || Ky) && !joint) {
    // the y-side product (K is symmetric for one point cloud)
    FMCA_TRY(matvec_state(plan, dp, k1, precision, dtype, nrhs, y, syi, syr, w.z, w.wsB, w.mv,
                          st, err, &B));
    if (Ky) {
      if (dtype == FMCA_DTYPE_F64)
        scale_copy_kernel<double><<<blocks(nc * nrhs), nthr, 0, st>>>(
            nc, nrhs, static_cast<const double*>(w.z), k.sigma2, static_cast<double*>(Ky),
            sxi, sxr);
      else
        scale_copy_kernel<float><<<blocks(nc * nrhs), nthr, 0, st>>>(
            nc, nrhs, static_cast<const float*>(w.z), k.sigma2, static_cast<float*>(Ky), sxi,
            sxr);
    }
  }
  if (dX) {
    FMCA_CK(cudaMemsetAsync(w.G, 0, sizeof(double) * 4 * nr, st));
    colscale_kernel<<<1, 256, 0, st>>>(nrhs, A.cmax ? A.cmax + A.cofs : nullptr,
                                       B.cmax ? B.cmax + B.cofs : nullptr, w.colscale);
    if (A.fp64)
      FMCA_TRY(grad_terms<double>(plan, dp, dp->d, k1, A, B, nrhs, w.colscale, k.sigma2, w.G,
                                  st, err));
    else
      FMCA_TRY(grad_terms<float>(plan, dp, dp->f, k1, A, B, nrhs, w.colscale, k.sigma2, w.G,
                                 st, err));
    if (dtype == FMCA_DTYPE_F64)
      grad_scatter_kernel<double><<<blocks(nr * plan.interp.dim), nthr, 0, st>>>(
          dp->perm_r, nr, plan.interp.dim, w.G, static_cast<double*>(dX), sdi, sdd);
    else
      grad_scatter_kernel<float><<<blocks(nr * plan.interp.dim), nthr, 0, st>>>(
          dp->perm_r, nr, plan.interp.dim, w.G, static_cast<float*>(dX), sdi, sdd);
  }
  FMCA_CK(cudaGetLastError());
  return FMCA_OK;
}

int update_points(const Plan& plan, DevPlan* dp, std::string* err) {
  if (!dp) return FMCA_OK;
  auto refresh = [&](auto& S) -> int {
    using T = std::remove_reference_t<decltype(S.ip.xi[0])>;
    if (!S.ready) return FMCA_OK;
    const int dim = plan.interp.dim;
    for (int side = 0; side < 2; ++side) {
      const Tree& t = side == 0 ? plan.rows : plan.cols;
      const std::vector<double>& Pn = side == 0 ? plan.points_r : plan.points_c;
      std::vector<Pt4<T>> hp(t.n);
      for (uint32_t i = 0; i < t.n; ++i) {
        const double* p = Pn.data() + (size_t)t.perm[i] * dim;
        hp[i] = Pt4<T>{(T)p[0], dim > 1 ? (T)p[1] : T(0), dim > 2 ? (T)p[2] : T(0), T(1)};
      }
      FMCA_CK(cudaMemcpy(side == 0 ? S.pts_r : S.pts_c, hp.data(), sizeof(Pt4<T>) * t.n,
                         cudaMemcpyHostToDevice));
    }
    cloud_centre(plan, S.ctr);
    return FMCA_OK;
  };
  std::lock_guard<std::mutex> lock(dp->mu);
  int cur = -1;
  FMCA_CK(cudaGetDevice(&cur));
  if (cur != dp->device) FMCA_CK(cudaSetDevice(dp->device));
  int s = refresh(dp->d);
  if (s == FMCA_OK) s = refresh(dp->f);
  if (cur != dp->device) cudaSetDevice(cur);
  return s;
}

int check_device_error(DevPlan* dp, std::string* err) {
  if (!dp || !dp->err_flag) return FMCA_OK;
  FMCA_CK(cudaDeviceSynchronize());
  int h = 0;
  FMCA_CK(cudaMemcpy(&h, dp->err_flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    FMCA_CK(cudaMemset(dp->err_flag, 0, sizeof(int)));
    *err = "a kernel gave up a bounded wait on a shared-memory copy";
    return FMCA_ERR_TIMEOUT;
  }
  return FMCA_OK;
}

int dense_eval(const KernelDesc& k, int dim, const double* PR, int64_t nr,
               const double* PC, int64_t nc, double* out, std::string* err) {
  double *dr = nullptr, *dc = nullptr, *dout = nullptr;
  FMCA_CK(cudaMalloc(&dr, sizeof(double) * (size_t)(dim * nr + 1)));
  FMCA_CK(cudaMalloc(&dc, sizeof(double) * (size_t)(dim * nc + 1)));
  FMCA_CK(cudaMalloc(&dout, sizeof(double) * (size_t)(nr * nc + 1)));
  FMCA_CK(cudaMemcpy(dr, PR, sizeof(double) * dim * nr, cudaMemcpyHostToDevice));
  FMCA_CK(cudaMemcpy(dc, PC, sizeof(double) * dim * nc, cudaMemcpyHostToDevice));
  const KParams<double> kp = make_kparams<double>(k);
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 152;
  dense_eval_kernel<<<sms * 16, 256>>>(dim, dr, nr, dc, nc, kp, output_scale(k), dout);
  FMCA_CK(cudaGetLastError());
  FMCA_CK(cudaMemcpy(out, dout, sizeof(double) * nr * nc, cudaMemcpyDeviceToHost));
  cudaFree(dr);
  cudaFree(dc);
  cudaFree(dout);
  return FMCA_OK;
}

int device_of(const DevPlan* dp) { return dp ? dp->device : -1; }

size_t device_bytes(const DevPlan* dp) {
  return dp ? dp->alloc_bytes + dp->ws_bytes + dp->as.bytes : 0;
}

bool resident(const DevPlan* dp, int precision) {
  int cur = -1;
  if (!dp || cudaGetDevice(&cur) != cudaSuccess || cur != dp->device) return false;
  return precision == FMCA_PREC_FP64 ? dp->d.ready : dp->f.ready;
}

int profile(DevPlan* dp, double* stage_ms, int64_t* launches, std::string* err) {
  for (int i = 0; i < FMCA_STAGE_COUNT; ++i) stage_ms[i] = 0;
  if (launches) *launches = dp ? dp->launches : 0;
  if (!dp || dp->nevents < 2) return FMCA_OK;
  FMCA_CK(cudaEventSynchronize(dp->events[dp->nevents - 1]));
  for (int k = 1; k < dp->nevents; ++k) {
    float ms = 0;
    FMCA_CK(cudaEventElapsedTime(&ms, dp->events[k - 1], dp->events[k]));
    const int sid = dp->event_stage[k];
    if (sid >= 0 && sid < FMCA_STAGE_COUNT) stage_ms[sid] += ms;
  }
  return FMCA_OK;
}

}  // namespace gpu
}  // namespace fmca
