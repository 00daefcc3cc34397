// Device plan and matvec driver.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/fmca_gb300.h"
#include "h2_gpu.h"
#include "h2_gpu_kernels.cuh"
#include "h2_tc_kernels.cuh"

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
constexpr int kTcGroupCap = 128;  // targets per ksum_tc CTA (4 warps x 32)
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
  InterpDev<T> ip;
};

struct GroupList {
  KGroup* groups = nullptr;
  uint32_t* ivl = nullptr;
  int ngroups = 0;
  int maxcount = 0;
};

}  // namespace

struct DevPlan {
  int device = -1;
  std::vector<void*> allocs;
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
  GroupList far, near;        // chunked to kGroupCap targets
  GroupList far_tc, near_tc;  // chunked to kTcGroupCap targets
  int* err_flag = nullptr;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  std::mutex mu;
  // stage profiling: events recorded at stage boundaries of the last matvec
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
  // transfer level lists
  {
    const Tree& t = plan.cols;
    std::vector<int32_t> lst;
    dp->m2m_ptr.assign(t.nlevels() + 1, 0);
    for (int l = 0; l < t.nlevels(); ++l) {
      for (int c = t.level_ptr[l]; c < t.level_ptr[l + 1]; ++c)
        if (t.nsons[c]) lst.push_back(c);
      dp->m2m_ptr[l + 1] = (int)lst.size();
    }
    FMCA_TRY(to_device(dp, lst.data(), lst.size(), &dp->m2m_list, err));
  }
  {
    const Tree& t = plan.rows;
    std::vector<int32_t> lst;
    dp->l2l_ptr.assign(t.nlevels() + 1, 0);
    for (int l = 0; l < t.nlevels(); ++l) {
      if (l >= 1)
        for (int c = t.level_ptr[l]; c < t.level_ptr[l + 1]; ++c) lst.push_back(c);
      dp->l2l_ptr[l + 1] = (int)lst.size();
    }
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
  // near groups: targets = points of every row leaf, sources = merged
  // column point intervals
  for (int pass = 0; pass < 2; ++pass) {
    const uint32_t cap = pass == 0 ? kGroupCap : kTcGroupCap;
    HostGroups hg;
    const Pattern& P = plan.pat;
    hg.ivl = P.near_ivl;
    for (size_t l = 0; l < plan.row_leaves.size(); ++l) {
      const int c = plan.row_leaves[l];
      add_target_range(&hg, plan.rows.begin[c], plan.rows.size[c], P.near_ptr[l],
                       P.near_ptr[l + 1], cap);
    }
    sort_groups(&hg);
    FMCA_TRY(upload_groups(dp, hg, pass == 0 ? &dp->near : &dp->near_tc, err));
  }
  {
    void* p = nullptr;
    FMCA_CK(cudaMalloc(&p, sizeof(int)));
    dp->allocs.push_back(p);
    FMCA_CK(cudaMemset(p, 0, sizeof(int)));
    dp->err_flag = static_cast<int*>(p);
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
KParams<T> make_kparams(const KernelDesc& k) {
  KParams<T> kp;
  const double l = k.l, log2e = 1.4426950408889634;
  double a = 0, e2 = 0;
  switch (k.type) {
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
  return kp;
}

template <typename K>
void ensure_smem(K kern, size_t bytes) {
  if (bytes > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)bytes);
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

template <typename T, int RB>
cudaError_t run_tree_stages(const Plan& plan, DevPlan* dp, DevSet<T>& S,
                            Workspace<T>& w, int ld, int rofs, int rcount,
                            const KParams<T>& kp, cudaStream_t st) {
  const int q = plan.interp.q;
  const size_t midx_bytes = (size_t)q * 3 * sizeof(int);
  // upward pass: leaf moments
  {
    dp->launches += dp->nleaves_c ? 1 : 0;
    auto kern = leafmom_kernel<T, RB>;
    const size_t smem = (64 * 24 + 64 * RB) * sizeof(T) + midx_bytes;
    ensure_smem(kern, smem);
    if (dp->nleaves_c)
      kern<<<dp->nleaves_c, 128, smem, st>>>(dp->leaves_c, dp->cbegin_c, dp->csize_c,
                                             S.bbmin_c, S.bbext_c, S.pts_c, w.xc, ld,
                                             rofs, rcount, dp->midx, S.ip, w.t);
    dp->mark(FMCA_STAGE_LEAFMOM, st);
  }
  // M2M, bottom-up
  {
    auto kern = transfer_kernel<T, RB, true>;
    const size_t smem = (192 + 64 * RB) * sizeof(T) + midx_bytes;
    ensure_smem(kern, smem);
    for (int l = plan.cols.nlevels() - 1; l >= 0; --l) {
      const int nb = dp->m2m_ptr[l + 1] - dp->m2m_ptr[l];
      if (nb) {
        kern<<<nb, 128, smem, st>>>(dp->m2m_list + dp->m2m_ptr[l], dp->son0_c,
                                    dp->nsons_c, nullptr, S.E_c, dp->midx, S.ip,
                                    w.t, ld, rofs, rcount);
        ++dp->launches;
      }
    }
    dp->mark(FMCA_STAGE_M2M, st);
  }
  // far-field coupling
  cudaError_t e = launch_ksum<T>(RB, dp->far, S.nodes_r, S.nodes_c, w.t, ld, w.s,
                                 rofs, rcount, kp, 0, dp->err_flag, st);
  if (e != cudaSuccess) return e;
  dp->launches += dp->far.ngroups ? 1 : 0;
  dp->mark(FMCA_STAGE_FAR, st);
  // L2L, top-down
  {
    auto kern = transfer_kernel<T, RB, false>;
    const size_t smem = (192 + 64 * RB) * sizeof(T) + midx_bytes;
    ensure_smem(kern, smem);
    for (int l = 1; l < plan.rows.nlevels(); ++l) {
      const int nb = dp->l2l_ptr[l + 1] - dp->l2l_ptr[l];
      if (nb) {
        kern<<<nb, 128, smem, st>>>(dp->l2l_list + dp->l2l_ptr[l], nullptr, nullptr,
                                    dp->parent_r, S.E_r, dp->midx, S.ip, w.s, ld,
                                    rofs, rcount);
        ++dp->launches;
      }
    }
    dp->mark(FMCA_STAGE_L2L, st);
  }
  // leaf gather
  {
    auto kern = leafgather_kernel<T, RB>;
    const size_t smem = (128 * 24 + 64 * RB) * sizeof(T) + midx_bytes;
    ensure_smem(kern, smem);
    if (dp->nleaves_r)
      kern<<<dp->nleaves_r, 128, smem, st>>>(dp->leaves_r, dp->cbegin_r, dp->csize_r,
                                             S.bbmin_r, S.bbext_r, S.pts_r, w.s, ld,
                                             rofs, rcount, dp->midx, S.ip, w.yfar);
    dp->launches += dp->nleaves_r ? 1 : 0;
    dp->mark(FMCA_STAGE_LEAFGATHER, st);
  }
  // near field
  e = launch_ksum<T>(RB, dp->near, S.pts_r, S.pts_c, w.xc, ld, w.ynear, rofs, rcount,
                     kp, 0, dp->err_flag, st);
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

template <typename T>
int matvec_t(const Plan& plan, DevPlan* dp, DevSet<T>& S, const KernelDesc& k,
             int dtype, int order, int nrhs, const void* x, int64_t sxi,
             int64_t sxr, void* y, int64_t syi, int64_t syr, void* ws,
             size_t wsb, cudaStream_t st, std::string* err) {
  const int ld = ld_for<T>(nrhs);
  const int rb = rhs_block(nrhs);
  const size_t need = ws_layout<T>(plan, nrhs, nullptr, nullptr);
  FMCA_TRY(acquire_ws(dp, need, &ws, wsb, st, err));
  Workspace<T> w;
  ws_layout<T>(plan, nrhs, ws, &w);
  dp->nevents = 0;
  dp->launches = 0;
  dp->mark(-1, st);
  const KParams<T> kp = make_kparams<T>(k);
  const uint32_t* pc = order == FMCA_ORDER_NATURAL ? dp->perm_c : nullptr;
  const uint32_t* pr = order == FMCA_ORDER_NATURAL ? dp->perm_r : nullptr;
  const int nthr = 256;
  auto blocks = [&](int64_t total) {
    int64_t b = (total + nthr - 1) / nthr;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32));
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
        e = run_tree_stages<T, 1>(plan, dp, S, wc, ld, 0, rcount, kp, st);
        break;
      case 8:
        e = run_tree_stages<T, 8>(plan, dp, S, wc, ld, 0, rcount, kp, st);
        break;
      default:
        e = run_tree_stages<T, 32>(plan, dp, S, wc, ld, 0, rcount, kp, st);
        break;
    }
    FMCA_CK(e);
    FMCA_CK(cudaGetLastError());
  }
  if (dtype == FMCA_DTYPE_F64)
    scatter_kernel<T, double><<<blocks((int64_t)plan.rows.n * nrhs), nthr, 0, st>>>(
        pr, plan.rows.n, nrhs, rb, ld, w.ynear, w.yfar, k.sigma2, static_cast<double*>(y),
        syi, syr);
  else
    scatter_kernel<T, float><<<blocks((int64_t)plan.rows.n * nrhs), nthr, 0, st>>>(
        pr, plan.rows.n, nrhs, rb, ld, w.ynear, w.yfar, k.sigma2, static_cast<float*>(y),
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
  __half *xh, *xl, *th, *tl;
  Pt4<float>* nodes_s;
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
  t.xc = (float*)take(plan.cols.n * ld * nch * 4);
  t.xh = (__half*)take(plan.cols.n * ld * nch * 2);
  t.xl = (__half*)take(plan.cols.n * ld * nch * 2);
  t.t = (float*)take(Cc * q * ld * nch * 4);
  t.th = (__half*)take(Cc * q * ld * 2);
  t.tl = (__half*)take(Cc * q * ld * 2);
  t.nodes_s = (Pt4<float>*)take(Cc * q * sizeof(Pt4<float>));
  t.s = (float*)take(Cr * q * ld * nch * 4);
  t.ynear = (float*)take(plan.rows.n * ld * nch * 4);
  t.yfar = (float*)take(plan.rows.n * ld * nch * 4);
  t.cmax = (unsigned int*)take((size_t)nrhs * 4);
  if (w) *w = t;
  return off;
}

bool tc_supported(int type, int nrhs) {
  return type >= FMCA_KERNEL_EXPONENTIAL && type <= FMCA_KERNEL_MATERN92 && nrhs > 16;
}

template <int KT, int MT>
cudaError_t launch_tc_t(const GroupList& gl, const Pt4<float>* tgt, const Pt4<float>* src,
                        const __half* vh, const __half* vl, float* out, int rcount,
                        const KParams<float>& kp, int* errf, cudaStream_t st) {
  auto kern = ksum_tc_kernel<KT, MT>;
  const size_t smem = 128 + (size_t)kTcStages * kTcTile * (16 + 4 * kTcRhs);
  ensure_smem(kern, smem);
  kern<<<gl.ngroups, 128, smem, st>>>(gl.groups, gl.ivl, tgt, src, vh, vl, out, kTcRhs,
                                       rcount, kp, errf);
  return cudaGetLastError();
}

// groups hold at most kTcGroupCap = 4 warps x 2 m-tiles x 16 targets
template <int KT>
cudaError_t launch_tc_mt(const GroupList& gl, const Pt4<float>* tgt, const Pt4<float>* src,
                         const __half* vh, const __half* vl, float* out, int rcount,
                         const KParams<float>& kp, int* errf, cudaStream_t st) {
  return launch_tc_t<KT, 2>(gl, tgt, src, vh, vl, out, rcount, kp, errf, st);
}

cudaError_t launch_tc(const GroupList& gl, const Pt4<float>* tgt, const Pt4<float>* src,
                      const __half* vh, const __half* vl, float* out, int rcount,
                      const KParams<float>& kp, int* errf, cudaStream_t st) {
  if (gl.ngroups == 0) return cudaSuccess;
  switch (kp.type) {
    case 0:
      return launch_tc_mt<0>(gl, tgt, src, vh, vl, out, rcount, kp, errf, st);
    case 1:
      return launch_tc_mt<1>(gl, tgt, src, vh, vl, out, rcount, kp, errf, st);
    case 2:
      return launch_tc_mt<2>(gl, tgt, src, vh, vl, out, rcount, kp, errf, st);
    case 3:
      return launch_tc_mt<3>(gl, tgt, src, vh, vl, out, rcount, kp, errf, st);
    default:
      return launch_tc_mt<-1>(gl, tgt, src, vh, vl, out, rcount, kp, errf, st);
  }
}

int matvec_tc(const Plan& plan, DevPlan* dp, DevSet<float>& S, const KernelDesc& k,
              int dtype, int order, int nrhs, const void* x, int64_t sxi, int64_t sxr,
              void* y, int64_t syi, int64_t syr, void* ws, size_t wsb, cudaStream_t st,
              std::string* err) {
  constexpr int RB = kTcRhs;
  const int ld = kTcRhs;
  const size_t need = tc_ws_layout(plan, nrhs, nullptr, nullptr);
  FMCA_TRY(acquire_ws(dp, need, &ws, wsb, st, err));
  TcWorkspace w;
  tc_ws_layout(plan, nrhs, ws, &w);
  dp->nevents = 0;
  dp->launches = 0;
  dp->mark(-1, st);
  const KParams<float> kp = make_kparams<float>(k);
  const uint32_t* pc = order == FMCA_ORDER_NATURAL ? dp->perm_c : nullptr;
  const uint32_t* pr = order == FMCA_ORDER_NATURAL ? dp->perm_r : nullptr;
  const int nthr = 256;
  auto blocks = [&](int64_t total) {
    int64_t b = (total + nthr - 1) / nthr;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32));
  };
  const int64_t nc = plan.cols.n, nr = plan.rows.n;
  const int nch = (nrhs + RB - 1) / RB;
  FMCA_CK(cudaMemsetAsync(w.cmax, 0, sizeof(unsigned int) * nrhs, st));
  constexpr int kColChunk = 4096;  // columns per colmax launch (16 KB shared)
  for (int c0 = 0; c0 < nrhs; c0 += kColChunk) {
    const int ncol = std::min(kColChunk, nrhs - c0);
    const size_t smem = sizeof(unsigned int) * ncol;
    if (dtype == FMCA_DTYPE_F64)
      colmax_kernel<double><<<152 * 4, nthr, smem, st>>>(
          nc, c0, ncol, static_cast<const double*>(x), sxi, sxr, w.cmax);
    else
      colmax_kernel<float><<<152 * 4, nthr, smem, st>>>(
          nc, c0, ncol, static_cast<const float*>(x), sxi, sxr, w.cmax);
    ++dp->launches;
  }
  if (dtype == FMCA_DTYPE_F64)
    gather_split_kernel<double><<<blocks(nc * RB * nch), nthr, 0, st>>>(
        pc, nc, nrhs, static_cast<const double*>(x), sxi, sxr, w.cmax, w.xc, w.xh, w.xl);
  else
    gather_split_kernel<float><<<blocks(nc * RB * nch), nthr, 0, st>>>(
        pc, nc, nrhs, static_cast<const float*>(x), sxi, sxr, w.cmax, w.xc, w.xh, w.xl);
  FMCA_CK(cudaGetLastError());
  dp->launches += 1;
  dp->mark(FMCA_STAGE_GATHER, st);
  const size_t q = plan.interp.q;
  const size_t midx_bytes = q * 3 * sizeof(int);
  const int Cc = plan.cols.nclusters(), Cr = plan.rows.nclusters();
  for (int ch = 0; ch < nch; ++ch) {
    const int rcount = std::min(RB, nrhs - ch * RB);
    float* xc = w.xc + (size_t)ch * nc * ld;
    const __half* xh = w.xh + (size_t)ch * nc * ld;
    const __half* xl = w.xl + (size_t)ch * nc * ld;
    float* t = w.t + (size_t)ch * Cc * q * ld;
    float* s = w.s + (size_t)ch * Cr * q * ld;
    float* ynear = w.ynear + (size_t)ch * nr * ld;
    float* yfar = w.yfar + (size_t)ch * nr * ld;
    {
      auto kern = leafmom_kernel<float, RB>;
      const size_t smem = (64 * 24 + 64 * RB) * sizeof(float) + midx_bytes;
      ensure_smem(kern, smem);
      if (dp->nleaves_c) {
        kern<<<dp->nleaves_c, 128, smem, st>>>(dp->leaves_c, dp->cbegin_c, dp->csize_c,
                                               S.bbmin_c, S.bbext_c, S.pts_c, xc, ld, 0,
                                               rcount, dp->midx, S.ip, t);
        ++dp->launches;
      }
      dp->mark(FMCA_STAGE_LEAFMOM, st);
    }
    {
      auto kern = transfer_kernel<float, RB, true>;
      const size_t smem = (192 + 64 * RB) * sizeof(float) + midx_bytes;
      ensure_smem(kern, smem);
      for (int l = plan.cols.nlevels() - 1; l >= 0; --l) {
        const int nb = dp->m2m_ptr[l + 1] - dp->m2m_ptr[l];
        if (nb) {
          kern<<<nb, 128, smem, st>>>(dp->m2m_list + dp->m2m_ptr[l], dp->son0_c, dp->nsons_c,
                                      nullptr, S.E_c, dp->midx, S.ip, t, ld, 0, rcount);
          ++dp->launches;
        }
      }
      dp->mark(FMCA_STAGE_M2M, st);
    }
    tscale_kernel<<<Cc, 128, 0, st>>>(Cc, (int)q, rcount, t, S.nodes_c, w.th, w.tl,
                                       w.nodes_s);
    ++dp->launches;
    FMCA_CK(launch_tc(dp->far_tc, S.nodes_r, w.nodes_s, w.th, w.tl, s, rcount, kp,
                      dp->err_flag, st));
    dp->launches += dp->far_tc.ngroups ? 1 : 0;
    dp->mark(FMCA_STAGE_FAR, st);
    {
      auto kern = transfer_kernel<float, RB, false>;
      const size_t smem = (192 + 64 * RB) * sizeof(float) + midx_bytes;
      ensure_smem(kern, smem);
      for (int l = 1; l < plan.rows.nlevels(); ++l) {
        const int nb = dp->l2l_ptr[l + 1] - dp->l2l_ptr[l];
        if (nb) {
          kern<<<nb, 128, smem, st>>>(dp->l2l_list + dp->l2l_ptr[l], nullptr, nullptr,
                                      dp->parent_r, S.E_r, dp->midx, S.ip, s, ld, 0, rcount);
          ++dp->launches;
        }
      }
      dp->mark(FMCA_STAGE_L2L, st);
    }
    {
      auto kern = leafgather_kernel<float, RB>;
      const size_t smem = (128 * 24 + 64 * RB) * sizeof(float) + midx_bytes;
      ensure_smem(kern, smem);
      if (dp->nleaves_r) {
        kern<<<dp->nleaves_r, 128, smem, st>>>(dp->leaves_r, dp->cbegin_r, dp->csize_r,
                                               S.bbmin_r, S.bbext_r, S.pts_r, s, ld, 0,
                                               rcount, dp->midx, S.ip, yfar);
        ++dp->launches;
      }
      dp->mark(FMCA_STAGE_LEAFGATHER, st);
    }
    FMCA_CK(launch_tc(dp->near_tc, S.pts_r, S.pts_c, xh, xl, ynear, rcount, kp,
                      dp->err_flag, st));
    dp->launches += dp->near_tc.ngroups ? 1 : 0;
    dp->mark(FMCA_STAGE_NEAR, st);
  }
  if (dtype == FMCA_DTYPE_F64)
    scatter_scaled_kernel<double><<<blocks(nr * nrhs), nthr, 0, st>>>(
        pr, nr, nrhs, w.ynear, w.yfar, w.cmax, k.sigma2, static_cast<double*>(y), syi, syr);
  else
    scatter_scaled_kernel<float><<<blocks(nr * nrhs), nthr, 0, st>>>(
        pr, nr, nrhs, w.ynear, w.yfar, w.cmax, k.sigma2, static_cast<float*>(y), syi, syr);
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

int matvec(const Plan& plan, DevPlan* dp, const KernelDesc& k, int precision,
           int dtype, int order, int nrhs, const void* x, int64_t sxi,
           int64_t sxr, void* y, int64_t syi, int64_t syr, void* ws,
           size_t ws_bytes, cudaStream_t st, std::string* err) {
  std::lock_guard<std::mutex> lock(dp->mu);
  if (precision == FMCA_PREC_FP64)
    return matvec_t<double>(plan, dp, dp->d, k, dtype, order, nrhs, x, sxi, sxr, y,
                            syi, syr, ws, ws_bytes, st, err);
  if (precision == FMCA_PREC_MIXED && tc_supported(k.type, nrhs))
    return matvec_tc(plan, dp, dp->f, k, dtype, order, nrhs, x, sxi, sxr, y, syi, syr, ws,
                     ws_bytes, st, err);
  return matvec_t<float>(plan, dp, dp->f, k, dtype, order, nrhs, x, sxi, sxr, y, syi,
                         syr, ws, ws_bytes, st, err);
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
  dense_eval_kernel<<<152 * 16, 256>>>(dim, dr, nr, dc, nc, kp, k.sigma2, dout);
  FMCA_CK(cudaGetLastError());
  FMCA_CK(cudaMemcpy(out, dout, sizeof(double) * nr * nc, cudaMemcpyDeviceToHost));
  cudaFree(dr);
  cudaFree(dc);
  cudaFree(dout);
  return FMCA_OK;
}

int device_of(const DevPlan* dp) { return dp ? dp->device : -1; }

void set_profiling(DevPlan* dp, bool on) {
  if (dp) dp->profile = on;
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
