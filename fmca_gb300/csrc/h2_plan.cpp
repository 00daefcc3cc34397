// Host-side H2 plan construction.  Compile with -ffp-contract=off.
#include "h2_plan.h"

#include <algorithm>
#include <atomic>
#include <exception>
#include <thread>
#include <cctype>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <stdexcept>

namespace fmca {

namespace {
constexpr double kEps = std::numeric_limits<double>::epsilon();
constexpr double kInf = std::numeric_limits<double>::infinity();
}  // namespace

// ---------------------------------------------------------------------------
// kernels
int kernel_type_from_name(const std::string& name) {
  std::string s(name);
  for (auto& ch : s) ch = (char)std::toupper((unsigned char)ch);
  static const char* names[] = {"EXPONENTIAL",     "MATERN32",       "MATERN52",
                                "GAUSSIAN",        "MATERN72",       "MATERN92",
                                "INVMULTIQUADRIC", "MULTIQUADRIC",   "BIHARMONIC3D",
                                "TRIHARMONIC3D",   "DL_EXPONENTIAL", "DL_MATERN32",
                                "DL_MATERN52",     "DL_GAUSSIAN",    "BIHARMONIC2D",
                                "TPS2D"};
  for (int i = 0; i < K_NUM_KERNELS; ++i)
    if (s == names[i]) return i;
  return -1;
}

const char* kernel_type_name(int type) {
  static const char* names[] = {"EXPONENTIAL",     "MATERN32",       "MATERN52",
                                "GAUSSIAN",        "MATERN72",       "MATERN92",
                                "INVMULTIQUADRIC", "MULTIQUADRIC",   "BIHARMONIC3D",
                                "TRIHARMONIC3D",   "DL_EXPONENTIAL", "DL_MATERN32",
                                "DL_MATERN52",     "DL_GAUSSIAN",    "BIHARMONIC2D",
                                "TPS2D"};
  return (type >= 0 && type < K_NUM_KERNELS) ? names[type] : "UNKNOWN";
}

// Expression order follows FMCA/src/CovarianceKernel/CovarianceKernel.h:56-118.
double kernel_eval_host(int type, double l, double c, double r) {
  switch (type) {
    case K_EXPONENTIAL:
      return std::exp(-r / l);
    case K_MATERN32:
      return (1. + std::sqrt(3.) / l * r) * std::exp(-std::sqrt(3.) * r / l);
    case K_MATERN52:
      return (1. + std::sqrt(5.) / l * r + 5 * r * r / (3 * l * l)) *
             std::exp(-std::sqrt(5.) * r / l);
    case K_GAUSSIAN:
      return std::exp(-0.5 * r * r / (l * l));
    case K_MATERN72:
      return (1. + std::sqrt(7.) / l * r + 14. / 5 * std::pow(r / l, 2.) +
              7. * std::sqrt(7.) / 15. * std::pow(r / l, 3.)) *
             std::exp(-std::sqrt(7.) * r / l);
    case K_MATERN92:
      return (1. + 3. / l * r + 27. / 7. * std::pow(r / l, 2.) +
              18. / 7. * std::pow(r / l, 3.) + 27. / 35. * std::pow(r / l, 4.)) *
             std::exp(-3 * r / l);
    case K_INVMULTIQUADRIC:
      return 1. / std::sqrt((r / l) * (r / l) + c * c);
    case K_MULTIQUADRIC:
      return std::sqrt((r / l) * (r / l) + c * c);
    case K_BIHARMONIC3D:
      return r / l;
    case K_TRIHARMONIC3D:
      return (r / l) * (r / l) * (r / l);
    case K_DL_EXPONENTIAL:  // d/dl exp(-r/l) = (r/l^2) exp(-r/l)
      return r / (l * l) * std::exp(-r / l);
    case K_DL_MATERN32: {  // (3 r^2 / l^3) exp(-sqrt(3) r / l)
      const double a = std::sqrt(3.) / l;
      return a * a * r * r / l * std::exp(-a * r);
    }
    case K_DL_MATERN52: {  // (a^2 r^2 / (3 l)) (1 + a r) exp(-a r), a = sqrt(5)/l
      const double a = std::sqrt(5.) / l;
      return a * a * r * r / (3. * l) * (1. + a * r) * std::exp(-a * r);
    }
    case K_DL_GAUSSIAN:  // (r^2 / l^3) exp(-r^2 / (2 l^2))
      return r * r / (l * l * l) * std::exp(-0.5 * r * r / (l * l));
    case K_BIHARMONIC2D:
      return r < std::numeric_limits<double>::epsilon() ? 0. : std::log(r / l) * (r / l) * (r / l);
    case K_TPS2D:
      return r > 0 ? r * r * std::log(r) : 0.;
  }
  return std::numeric_limits<double>::quiet_NaN();
}

// ---------------------------------------------------------------------------
// interpolation (TensorProductInterpolator.h:39-61, TotalDegreeInterpolator.h:
// 26-47, MultiIndexSet.h:39-100)
namespace {
// the multi-indices of the tensor (max entry <= deg) or total-degree (sum
// <= deg) set, ordered by 1-norm, then lexicographically (FMCA_Compare)
std::vector<std::vector<int>> index_set(int dim, int deg, bool total) {
  std::vector<std::vector<int>> set;
  std::vector<int> cur(dim, 0);
  int count = 1;
  for (int i = 0; i < dim; ++i) count *= (deg + 1);
  for (int k = 0; k < count; ++k) {
    int r = k, sum = 0;
    for (int i = dim - 1; i >= 0; --i) {
      cur[i] = r % (deg + 1);
      r /= (deg + 1);
      sum += cur[i];
    }
    if (!total || sum <= deg) set.push_back(cur);
  }
  std::sort(set.begin(), set.end(), [](const std::vector<int>& a, const std::vector<int>& b) {
    int na = 0, nb = 0;
    for (int v : a) na += v;
    for (int v : b) nb += v;
    if (na != nb) return na < nb;
    return std::lexicographical_compare(a.begin(), a.end(), b.begin(), b.end());
  });
  return set;
}

// radical inverse of m in base b: the digits of m mirrored at the radix
// point, as one correctly rounded division of two exact integers (the
// Halton sequence of HaltonSet.h:30-55)
double radical_inverse(uint64_t m, uint64_t b) {
  uint64_t num = 0, den = 1;
  while (m) {
    num = num * b + m % b;
    den *= b;
    m /= b;
  }
  return (double)num / (double)den;
}

// DeMarchi points (DeMarchiPoints.h:20-43): the Halton points 100 ..
// 100 + 10 q - 1 (HaltonSet<100>: 100 points skipped) are candidates; the
// nodes are the first q columns chosen by a column-pivoted QR
// factorisation of the q x 10 q matrix of polynomial values, in the order
// chosen. Householder reflections; the remaining column norms are
// recomputed at every step instead of downdated.
void demarchi_nodes(const Interp& ip, std::vector<double>* nodes) {
  const int q = ip.q, dim = ip.dim, M = 10 * q;
  static const uint64_t primes[3] = {2, 3, 5};
  std::vector<double> cand((size_t)M * dim), A((size_t)q * M);
  for (int m = 0; m < M; ++m) {
    for (int d = 0; d < dim; ++d)
      cand[(size_t)m * dim + d] = radical_inverse((uint64_t)(100 + m), primes[d]);
    ip.poly(&cand[(size_t)m * dim], &A[(size_t)m * q]);
  }
  std::vector<int> col(M);
  for (int m = 0; m < M; ++m) col[m] = m;
  std::vector<double> v(q);
  for (int s = 0; s < q; ++s) {
    int best = s;
    double bn = -1.;
    for (int j = s; j < M; ++j) {
      double n2 = 0;
      for (int i = s; i < q; ++i) n2 += A[(size_t)j * q + i] * A[(size_t)j * q + i];
      if (n2 > bn) {
        bn = n2;
        best = j;
      }
    }
    if (best != s) {
      std::swap(col[s], col[best]);
      for (int i = 0; i < q; ++i) std::swap(A[(size_t)s * q + i], A[(size_t)best * q + i]);
    }
    // reflector H = I - 2 v v^T / (v^T v) mapping column s onto e_s
    const double alpha = A[(size_t)s * q + s] >= 0 ? -std::sqrt(bn) : std::sqrt(bn);
    double vv = 0;
    for (int i = s; i < q; ++i) {
      v[i] = A[(size_t)s * q + i] - (i == s ? alpha : 0.);
      vv += v[i] * v[i];
    }
    if (vv == 0) continue;
    for (int j = s; j < M; ++j) {
      double dot = 0;
      for (int i = s; i < q; ++i) dot += v[i] * A[(size_t)j * q + i];
      const double f = 2. * dot / vv;
      for (int i = s; i < q; ++i) A[(size_t)j * q + i] -= f * v[i];
    }
  }
  nodes->assign((size_t)q * dim, 0.);
  for (int k = 0; k < q; ++k)
    for (int d = 0; d < dim; ++d) (*nodes)[(size_t)k * dim + d] = cand[(size_t)col[k] * dim + d];
}

// inverse of the n x n row-major matrix a (Gauss-Jordan, partial pivoting)
std::vector<double> invert(std::vector<double> a, int n) {
  std::vector<double> b((size_t)n * n, 0.);
  for (int i = 0; i < n; ++i) b[(size_t)i * n + i] = 1.;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::abs(a[(size_t)r * n + c]) > std::abs(a[(size_t)piv * n + c])) piv = r;
    if (piv != c)
      for (int j = 0; j < n; ++j) {
        std::swap(a[(size_t)c * n + j], a[(size_t)piv * n + j]);
        std::swap(b[(size_t)c * n + j], b[(size_t)piv * n + j]);
      }
    const double d = a[(size_t)c * n + c];
    for (int j = 0; j < n; ++j) {
      a[(size_t)c * n + j] /= d;
      b[(size_t)c * n + j] /= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[(size_t)r * n + c];
      if (f == 0) continue;
      for (int j = 0; j < n; ++j) {
        a[(size_t)r * n + j] -= f * a[(size_t)c * n + j];
        b[(size_t)r * n + j] -= f * b[(size_t)c * n + j];
      }
    }
  }
  return b;
}
}  // namespace

void Interp::init(int dim_, int deg_, int kind_) {
  kind = kind_;
  dim = dim_;
  deg = deg_;
  const double weight = 2. * M_PI / (2. * double(deg) + 2.);
  xi.assign(deg + 1, 0.);
  w.assign(deg + 1, 0.);
  for (int k = 0; k <= deg; ++k) {
    xi[k] = std::cos(weight * (double(k) + 0.5));
    xi[k] = 0.5 * (xi[k] + 1);
    w[k] = std::sin(weight * (double(k) + 0.5));
    if (k % 2 == 1) w[k] *= -1.;
  }
  const std::vector<std::vector<int>> set = index_set(dim, deg, kind == kInterpTotalDegree);
  q = (int)set.size();
  midx.assign((size_t)q * dim, 0);
  for (int k = 0; k < q; ++k)
    for (int i = 0; i < dim; ++i) midx[(size_t)k * dim + i] = set[k][i];
  Xi.assign((size_t)q * dim, 0.);
  invV.clear();
  if (kind == kInterpTotalDegree) {
    demarchi_nodes(*this, &Xi);
    std::vector<double> V((size_t)q * q);
    for (int i = 0; i < q; ++i) poly(&Xi[(size_t)i * dim], &V[(size_t)i * q]);
    invV = invert(V, q);
  } else {
    for (int k = 0; k < q; ++k)
      for (int i = 0; i < dim; ++i) Xi[(size_t)k * dim + i] = xi[set[k][i]];
  }
}

void Interp::legendre1d(double x, double* f) const {
  double p0 = 0., p1 = 1.;
  f[0] = 1.;
  for (int i = 1; i <= deg; ++i) {
    const double v = double(2 * i - 1) / double(i) * (2. * x - 1.) * p1 -
                     double(i - 1) / double(i) * p0;
    p0 = p1;
    p1 = v;
    f[i] = v * std::sqrt(double(2 * i + 1));
  }
}

void Interp::poly(const double* u, double* out) const {
  double f[3][32];
  for (int d = 0; d < dim; ++d) legendre1d(u[d], f[d]);
  for (int k = 0; k < q; ++k) {
    double v = 1.;
    for (int d = 0; d < dim; ++d) v *= f[d][midx[(size_t)k * dim + d]];
    out[k] = v;
  }
}

// Barycentric Lagrange basis in one variable (TensorProductInterpolator.h:65-81).
// The multivariate basis value of multi-index k is the product over the
// dimensions, taken in dimension order starting from 1.
void Interp::lagrange1d(double x, double* f) const {
  double weight = 0;
  for (int k = 0; k <= deg; ++k) weight += w[k] / (x - xi[k]);
  for (int a = 0; a <= deg; ++a)
    f[a] = (std::abs(x - xi[a]) > kEps) ? w[a] / (x - xi[a]) / weight : 1.;
}

// ---------------------------------------------------------------------------
// cluster tree
namespace {
struct TmpNode {
  uint32_t begin, size;
  int level;
  int sons[2];
  int nsons;
  std::vector<double> bb;  // min[dim], max[dim], ext[dim]
};

struct TreeBuilder {
  const double* P;
  int dim;
  uint32_t split_threshold;
  std::vector<uint32_t>* idx;
  std::vector<TmpNode> nodes;

  double coord(uint32_t i, int d) const { return P[(size_t)i * dim + d]; }

  // ClusterTreeInitializer<ClusterTree>::init_ClusterTree_impl + the
  // CardinalityBisection splitter, for one node: sorts the node's index
  // range along the longest edge of its (propagated) box and halves it.
  // Reads nodes[me] and writes only its own index range and sons, so nodes
  // of one level split concurrently. False: the node is a leaf.
  // longest edge of a (propagated) box, first maximum
  int longest_edge(const TmpNode& f) const {
    int longest = 0;
    for (int d = 1; d < dim; ++d)
      if (f.bb[2 * dim + d] > f.bb[2 * dim + longest]) longest = d;
    return longest;
  }

  bool split(int me, TmpNode* sons) const {
    const TmpNode& f = nodes[me];
    if (f.size <= split_threshold) return false;
    TmpNode s0 = f, s1 = f;
    s0.level = s1.level = f.level + 1;
    s0.nsons = s1.nsons = 0;
    const int longest = longest_edge(f);
    // std::sort of the index range by the coordinate, done on (coordinate,
    // index) records: the algorithm makes the same comparisons and moves
    // whatever the element type, so the index order is that of sorting the
    // indices with an indirect comparator, without a cache miss per
    // comparison
    uint32_t* ids = idx->data();
    struct Rec {
      double key;
      uint32_t id;
    };
    std::vector<Rec> rec(s0.size);
    for (uint32_t i = 0; i < s0.size; ++i)
      rec[i] = Rec{coord(ids[s0.begin + i], longest), ids[s0.begin + i]};
    std::sort(rec.begin(), rec.end(), [](const Rec& a, const Rec& b) { return a.key < b.key; });
    for (uint32_t i = 0; i < s0.size; ++i) ids[s0.begin + i] = rec[i].id;
    s0.size /= 2;
    s1.size -= s0.size;
    s1.begin += s0.size;
    s0.bb[dim + longest] = coord(ids[s0.begin + s0.size - 1], longest);
    s0.bb[2 * dim + longest] = s0.bb[dim + longest] - s0.bb[longest];
    s1.bb[longest] = coord(ids[s1.begin], longest);
    s1.bb[2 * dim + longest] = s1.bb[dim + longest] - s1.bb[longest];
    sons[0] = std::move(s0);
    sons[1] = std::move(s1);
    return true;
  }

  // the whole refinement, level by level: the nodes of a level split in
  // parallel (each std::sort on its own index range, the same calls on the
  // same data as the reference's depth-first recursion, so the permutation
  // is identical), then their sons are appended in order. Node storage order
  // differs from the recursion's; the ids are assigned afterwards in level
  // order, so they do not depend on it.
  void refine_all(int nthreads) {
    std::vector<int> cur{0};
    while (!cur.empty()) {
      const size_t m = cur.size();
      std::vector<TmpNode> out(2 * m);
      std::vector<char> did(m, 0);
      uint64_t work = 0;
      for (int c : cur) work += nodes[c].size;
      const int nt = (work < (1u << 16)) ? 1 : (int)std::min<size_t>((size_t)nthreads, m);
      if (nt <= 1) {
        for (size_t i = 0; i < m; ++i) did[i] = split(cur[i], &out[2 * i]);
      } else {
        // a failure (bad_alloc) in a worker is rethrown here, after the join
        std::atomic<size_t> next(0);
        std::vector<std::exception_ptr> errs(nt);
        auto body = [&](int t) {
          try {
            for (size_t i; (i = next.fetch_add(1)) < m;) did[i] = split(cur[i], &out[2 * i]);
          } catch (...) {
            errs[t] = std::current_exception();
            next.store(m);
          }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; ++t) pool.emplace_back(body, t);
        body(0);
        for (auto& th : pool) th.join();
        for (auto& e : errs)
          if (e) std::rethrow_exception(e);
      }
      std::vector<int> nxt;
      for (size_t i = 0; i < m; ++i) {
        if (!did[i]) continue;
        const int i0 = (int)nodes.size();
        nodes.push_back(std::move(out[2 * i]));
        nodes.push_back(std::move(out[2 * i + 1]));
        nodes[cur[i]].sons[0] = i0;
        nodes[cur[i]].sons[1] = i0 + 1;
        nodes[cur[i]].nsons = 2;
        nxt.push_back(i0);
        nxt.push_back(i0 + 1);
      }
      cur.swap(nxt);
    }
  }

  // refine_all with every level's sorts done by a LevelSorter: the same
  // splits (a sorted range is unique when its coordinates are distinct),
  // the son boxes from the coordinates the sorter returns at the split.
  // false: a sorted range held equal coordinates, or the sorter failed.
  bool refine_with(LevelSorter* so) {
    std::vector<int> cur{0};
    std::vector<SortSegment> segs;
    std::vector<int> who;
    std::vector<double> cut;
    while (!cur.empty()) {
      segs.clear();
      who.clear();
      for (int c : cur) {
        const TmpNode& f = nodes[c];
        if (f.size <= split_threshold) continue;
        segs.push_back(SortSegment{f.begin, f.size, longest_edge(f)});
        who.push_back(c);
      }
      if (segs.empty()) break;
      bool ties = false;
      if (!so->sort_level(segs, &cut, &ties) || ties) return false;
      std::vector<int> nxt;
      for (size_t i = 0; i < who.size(); ++i) {
        const int longest = segs[i].coord;
        TmpNode s0 = nodes[who[i]], s1 = nodes[who[i]];
        s0.level = s1.level = nodes[who[i]].level + 1;
        s0.nsons = s1.nsons = 0;
        s0.size /= 2;
        s1.size -= s0.size;
        s1.begin += s0.size;
        s0.bb[dim + longest] = cut[2 * i];
        s0.bb[2 * dim + longest] = s0.bb[dim + longest] - s0.bb[longest];
        s1.bb[longest] = cut[2 * i + 1];
        s1.bb[2 * dim + longest] = s1.bb[dim + longest] - s1.bb[longest];
        const int i0 = (int)nodes.size();
        nodes.push_back(std::move(s0));
        nodes.push_back(std::move(s1));
        nodes[who[i]].sons[0] = i0;
        nodes[who[i]].sons[1] = i0 + 1;
        nodes[who[i]].nsons = 2;
        nxt.push_back(i0);
        nxt.push_back(i0 + 1);
      }
      cur.swap(nxt);
    }
    return so->finish(idx);
  }

  // shrinkToFit_impl (ClusterTreeInitializer_ClusterTree.h:88-132)
  void shrink(int me) {
    std::vector<double> bb(3 * dim);
    TmpNode& nd = nodes[me];
    if (nd.size) {
      const uint32_t* ids = idx->data();
      for (int d = 0; d < dim; ++d) bb[d] = bb[dim + d] = coord(ids[nd.begin], d);
      if (nd.nsons) {
        for (int s = 0; s < nd.nsons; ++s) {
          shrink(nodes[me].sons[s]);
          const TmpNode& sn = nodes[nodes[me].sons[s]];
          if (sn.size)
            for (int d = 0; d < dim; ++d) {
              bb[d] = std::min(bb[d], sn.bb[d]);
              bb[dim + d] = std::max(bb[dim + d], sn.bb[dim + d]);
            }
        }
      } else {
        for (uint32_t i = 0; i < nd.size; ++i)
          for (int d = 0; d < dim; ++d) {
            const double v = coord(ids[nd.begin + i], d);
            bb[d] = std::min(v, bb[d]);
            bb[dim + d] = std::max(v, bb[dim + d]);
          }
      }
    } else {
      for (int d = 0; d < dim; ++d) {
        bb[d] = kInf;
        bb[dim + d] = -kInf;
      }
    }
    for (int d = 0; d < dim; ++d) bb[2 * dim + d] = bb[dim + d] - bb[d];
    for (int d = 0; d < dim; ++d)
      if (bb[dim + d] - bb[d] < 2e2 * kEps) {
        bb[dim + d] += 1e2 * kEps;
        bb[d] -= 1e2 * kEps;
        bb[2 * dim + d] = bb[dim + d] - bb[d];
      }
    nodes[me].bb = std::move(bb);
  }
};

// init_BoundingBox_impl and the root of the refinement
void start_builder(TreeBuilder* tb, Tree* t, const double* P, int dim, uint32_t n,
                   uint32_t min_csize) {
  t->dim = dim;
  t->n = n;
  t->perm.resize(n);
  std::iota(t->perm.begin(), t->perm.end(), 0u);
  tb->P = P;
  tb->dim = dim;
  tb->split_threshold = min_csize >= 1 ? (2 * min_csize - 1) : 1;
  tb->idx = &t->perm;
  TmpNode root;
  root.begin = 0;
  root.size = n;
  root.level = 0;
  root.nsons = 0;
  root.bb.assign(3 * dim, 0.);
  // init_BoundingBox_impl: box of all points, inflated by an epsilon layer
  for (int d = 0; d < dim; ++d) {
    double lo = n ? P[d] : 0., hi = n ? P[d] : 0.;
    for (uint32_t i = 1; i < n; ++i) {
      lo = std::min(lo, P[(size_t)i * dim + d]);
      hi = std::max(hi, P[(size_t)i * dim + d]);
    }
    lo -= kEps * std::abs(lo);
    hi += kEps * std::abs(hi);
    root.bb[d] = lo;
    root.bb[dim + d] = hi;
    root.bb[2 * dim + d] = hi - lo;
  }
  tb->nodes.reserve(2 * (n / std::max<uint32_t>(1, min_csize)) + 8);
  tb->nodes.push_back(std::move(root));
}

// shrinkToFit and the level-order numbering of a refined tree
void finish_tree(TreeBuilder& tb, Tree* t) {
  const int dim = t->dim;
  std::vector<uint32_t>& begin = t->begin;
  std::vector<uint32_t>& size = t->size;
  std::vector<int32_t>& level = t->level;
  std::vector<int32_t>& parent = t->parent;
  std::vector<int32_t>& son0 = t->son0;
  std::vector<int32_t>& nsons = t->nsons;
  std::vector<double>& bbmin = t->bbmin;
  std::vector<double>& bbmax = t->bbmax;
  std::vector<double>& bbext = t->bbext;
  std::vector<int32_t>& level_ptr = t->level_ptr;
  tb.shrink(0);
  // level-order numbering (IDDFSForwardIterator): breadth first, sons in order
  const int C = (int)tb.nodes.size();
  std::vector<int> order;
  order.reserve(C);
  order.push_back(0);
  for (size_t h = 0; h < order.size(); ++h)
    for (int s = 0; s < tb.nodes[order[h]].nsons; ++s)
      order.push_back(tb.nodes[order[h]].sons[s]);
  std::vector<int> newid(C);
  for (int i = 0; i < C; ++i) newid[order[i]] = i;
  begin.resize(C);
  size.resize(C);
  level.resize(C);
  parent.assign(C, -1);
  son0.assign(C, -1);
  nsons.assign(C, 0);
  bbmin.resize((size_t)C * dim);
  bbmax.resize((size_t)C * dim);
  bbext.resize((size_t)C * dim);
  int maxlev = 0;
  for (int i = 0; i < C; ++i) {
    const TmpNode& nd = tb.nodes[order[i]];
    begin[i] = nd.begin;
    size[i] = nd.size;
    level[i] = nd.level;
    maxlev = std::max(maxlev, nd.level);
    nsons[i] = nd.nsons;
    if (nd.nsons) {
      son0[i] = newid[nd.sons[0]];
      for (int s = 0; s < nd.nsons; ++s) parent[newid[nd.sons[s]]] = i;
    }
    for (int d = 0; d < dim; ++d) {
      bbmin[(size_t)i * dim + d] = nd.bb[d];
      bbmax[(size_t)i * dim + d] = nd.bb[dim + d];
      bbext[(size_t)i * dim + d] = nd.bb[2 * dim + d];
    }
  }
  level_ptr.assign(maxlev + 2, 0);
  for (int i = 0; i < C; ++i) level_ptr[level[i] + 1] = i + 1;
  for (int l = 1; l <= maxlev + 1; ++l)
    level_ptr[l] = std::max(level_ptr[l], level_ptr[l - 1]);
}
}  // namespace

void Tree::build(const double* P, int dim_, uint32_t n_, uint32_t min_csize, int threads) {
  TreeBuilder tb;
  start_builder(&tb, this, P, dim_, n_, min_csize);
  if (threads <= 0) threads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  tb.refine_all(threads);
  finish_tree(tb, this);
}

bool Tree::build_with(LevelSorter* sorter, const double* P, int dim_, uint32_t n_,
                      uint32_t min_csize) {
  TreeBuilder tb;
  start_builder(&tb, this, P, dim_, n_, min_csize);
  if (!sorter->start(P, dim_, n_) || !tb.refine_with(sorter)) {
    *this = Tree();
    return false;
  }
  finish_tree(tb, this);
  return true;
}

// ---------------------------------------------------------------------------
// cluster bases
void compute_transfer_factors(const Tree& t, const Interp& ip,
                              std::vector<double>* E) {
  const int C = t.nclusters(), dim = t.dim, p1 = ip.deg + 1;
  if (ip.kind == kInterpTotalDegree) {
    // E = P(son nodes in the father's cell) invV^T
    // (compute_cluster_bases_impl.h:36-50), row-major q x q per son
    const int q = ip.q;
    E->assign((size_t)C * q * q, 0.);
    std::vector<double> u(dim), P((size_t)q * q);
    for (int c = 1; c < C; ++c) {
      const int fa = t.parent[c];
      if (fa < 0 || t.size[c] == 0) continue;  // E stays zero for empty sons
      for (int j = 0; j < q; ++j) {
        for (int d = 0; d < dim; ++d)
          u[d] = ip.Xi[(size_t)j * dim + d] * t.bbext[(size_t)c * dim + d] /
                     t.bbext[(size_t)fa * dim + d] +
                 (t.bbmin[(size_t)c * dim + d] - t.bbmin[(size_t)fa * dim + d]) /
                     t.bbext[(size_t)fa * dim + d];
        ip.poly(u.data(), &P[(size_t)j * q]);  // P[j][k]: polynomial k at node j
      }
      double* e = E->data() + (size_t)c * q * q;
      for (int k = 0; k < q; ++k)
        for (int jj = 0; jj < q; ++jj) {
          double acc = 0;
          for (int j = 0; j < q; ++j) acc += P[(size_t)j * q + k] * ip.invV[(size_t)jj * q + j];
          e[(size_t)k * q + jj] = acc;
        }
    }
    return;
  }
  const size_t per = (size_t)dim * p1 * p1;
  E->assign((size_t)C * per, 0.);
  std::vector<double> f(p1);
  for (int c = 1; c < C; ++c) {
    const int fa = t.parent[c];
    if (fa < 0 || t.size[c] == 0) continue;  // E stays zero for empty sons
    double* e = E->data() + (size_t)c * per;
    for (int d = 0; d < dim; ++d) {
      const double sc = t.bbext[(size_t)c * dim + d];
      const double sf = t.bbext[(size_t)fa * dim + d];
      const double mc = t.bbmin[(size_t)c * dim + d];
      const double mf = t.bbmin[(size_t)fa * dim + d];
      for (int b = 0; b < p1; ++b) {
        // compute_cluster_bases_impl.h:134-139
        const double u = ip.xi[b] * sc / sf + (mc - mf) / sf;
        ip.lagrange1d(u, f.data());
        for (int a = 0; a < p1; ++a) e[((size_t)d * p1 + a) * p1 + b] = f[a];
      }
    }
  }
}

// interpolation nodes of a cluster: Xi .* ext + min (NystromEvaluator.h:44-49)
void compute_node_coords(const Tree& t, const Interp& ip,
                         std::vector<double>* nodes) {
  const int C = t.nclusters(), dim = t.dim, q = ip.q;
  nodes->assign((size_t)C * q * dim, 0.);
  for (int c = 0; c < C; ++c)
    for (int k = 0; k < q; ++k)
      for (int d = 0; d < dim; ++d)
        (*nodes)[((size_t)c * q + k) * dim + d] =
            ip.Xi[(size_t)k * dim + d] * t.bbext[(size_t)c * dim + d] +
            t.bbmin[(size_t)c * dim + d];
}

// ---------------------------------------------------------------------------
// admissibility (Admissibility.h:19-29, 95-115)
namespace {
enum Adm { kRefine = 0, kLowRank = 1, kDense = 2 };

inline double norm_seq(const double* v, int dim) {
  double s = v[0] * v[0];
  for (int d = 1; d < dim; ++d) s += v[d] * v[d];
  return std::sqrt(s);
}

Adm compare(const Tree& r, int i, const Tree& c, int j, double eta) {
  const int dim = r.dim;
  double tmp[16];
  std::vector<double> big;
  double* v = tmp;
  if (dim > 16) {
    big.resize(dim);
    v = big.data();
  }
  const double radius1 = 0.5 * norm_seq(r.bbext.data() + (size_t)i * dim, dim);
  const double radius2 = 0.5 * norm_seq(c.bbext.data() + (size_t)j * dim, dim);
  for (int d = 0; d < dim; ++d)
    v[d] = 0.5 * (r.bbmin[(size_t)i * dim + d] - c.bbmin[(size_t)j * dim + d] +
                  r.bbmax[(size_t)i * dim + d] - c.bbmax[(size_t)j * dim + d]);
  double dist = norm_seq(v, dim) - radius1 - radius2;
  dist = dist > 0 ? dist : 0;
  const double radius = radius1 > radius2 ? radius1 : radius2;
  if (radius > eta * dist) {
    if (!r.nsons[i] || !c.nsons[j]) return kDense;
    return kRefine;
  }
  return kLowRank;
}
}  // namespace

void Plan::build(const double* Pr, uint32_t nr, const double* Pc, uint32_t nc,
                 int dim, int deg, double eta_, uint32_t min_leaf, bool same,
                 int interp_kind, LevelSorter* sorter, PatternBuilder* pattern_builder) {
  interp.init(dim, deg, interp_kind);
  eta = eta_;
  points_r.assign(Pr, Pr + (size_t)dim * nr);
  if (same)
    points_c = points_r;
  else
    points_c.assign(Pc, Pc + (size_t)dim * nc);
  same_tree = same;
  const uint32_t mincsize =
      min_leaf > (uint32_t)interp.q ? min_leaf : (uint32_t)interp.q;
  // trees: level sorts on the sorter when one is given, else (and when a
  // sorted range holds equal coordinates) on the host
  trees_sorted_elsewhere = 0;
  auto make_tree = [&](Tree* t, const double* P, uint32_t n) {
    if (sorter && t->build_with(sorter, P, dim, n, mincsize))
      ++trees_sorted_elsewhere;
    else
      t->build(P, dim, n, mincsize, build_threads);
  };
  make_tree(&rows, Pr, nr);
  if (same)
    cols = rows;
  else
    make_tree(&cols, Pc, nc);
  compute_transfer_factors(rows, interp, &row_E);
  compute_node_coords(rows, interp, &row_nodes);
  if (same) {
    col_E = row_E;
    col_nodes = row_nodes;
  } else {
    compute_transfer_factors(cols, interp, &col_E);
    compute_node_coords(cols, interp, &col_nodes);
  }
  // leaves in cluster (point) order
  auto leaves_of = [](const Tree& t, std::vector<int32_t>* out) {
    out->clear();
    for (int c = 0; c < t.nclusters(); ++c)
      if (!t.nsons[c]) out->push_back(c);
    std::sort(out->begin(), out->end(), [&t](int a, int b) {
      return t.begin[a] != t.begin[b] ? t.begin[a] < t.begin[b] : a < b;
    });
  };
  leaves_of(rows, &row_leaves);
  leaves_of(cols, &col_leaves);

  // pattern: depth-first stack over cluster pairs (H2MatrixBase.h:160-191),
  // or the same leaves in the same order from the pattern builder
  Pattern& P = pat;
  P = Pattern();
  const uint32_t qq = (uint32_t)interp.q * (uint32_t)interp.q;  // Index arithmetic
  pattern_built_elsewhere = 0;
  if (pattern_builder && pattern_builder->build(rows, cols, qq, eta, &P.far_row, &P.far_col,
                                                &P.near_row, &P.near_col))
    pattern_built_elsewhere = 1;
  else
    P = Pattern();
  std::vector<std::pair<int32_t, int32_t>> stack;
  if (!pattern_built_elsewhere) stack.emplace_back(0, 0);
  while (!stack.empty()) {
    const auto blk = stack.back();
    stack.pop_back();
    const int i = blk.first, j = blk.second;
    const Adm adm = compare(rows, i, cols, j, eta);
    if (adm == kLowRank) {
      // only low-rank if cheaper than the dense block; 32-bit unsigned
      // products exactly like the reference's Index type
      const uint32_t dense = rows.size[i] * cols.size[j];
      if (qq < dense) {
        P.far_row.push_back(i);
        P.far_col.push_back(j);
      } else {
        P.near_row.push_back(i);
        P.near_col.push_back(j);
      }
    } else if (adm == kRefine) {
      for (int b = 0; b < cols.nsons[j]; ++b)
        for (int a = 0; a < rows.nsons[i]; ++a)
          stack.emplace_back(rows.son0[i] + a, cols.son0[j] + b);
    } else {
      P.near_row.push_back(i);
      P.near_col.push_back(j);
    }
  }
  // far field CSR by row cluster, column clusters ascending
  const int Cr = rows.nclusters();
  P.far_ptr.assign(Cr + 1, 0);
  for (int32_t r : P.far_row) P.far_ptr[r + 1]++;
  for (int c = 0; c < Cr; ++c) P.far_ptr[c + 1] += P.far_ptr[c];
  P.far_idx.assign(P.far_row.size(), 0);
  {
    std::vector<int32_t> fill(P.far_ptr.begin(), P.far_ptr.end() - 1);
    for (size_t b = 0; b < P.far_row.size(); ++b)
      P.far_idx[fill[P.far_row[b]]++] = P.far_col[b];
    for (int c = 0; c < Cr; ++c)
      std::sort(P.far_idx.begin() + P.far_ptr[c], P.far_idx.begin() + P.far_ptr[c + 1]);
  }
  // near field: split dense blocks onto row leaves, merge column intervals
  const int nleaf = (int)row_leaves.size();
  std::vector<uint32_t> leaf_begin(nleaf);
  for (int l = 0; l < nleaf; ++l) leaf_begin[l] = rows.begin[row_leaves[l]];
  std::vector<std::vector<std::pair<uint32_t, uint32_t>>> per_leaf(nleaf);
  P.near_pairs = 0;
  for (size_t b = 0; b < P.near_row.size(); ++b) {
    const int i = P.near_row[b], j = P.near_col[b];
    P.near_pairs += (uint64_t)rows.size[i] * cols.size[j];
    if (rows.size[i] == 0 || cols.size[j] == 0) continue;
    const uint32_t lo = rows.begin[i], hi = rows.begin[i] + rows.size[i];
    int l = (int)(std::lower_bound(leaf_begin.begin(), leaf_begin.end(), lo) -
                  leaf_begin.begin());
    for (; l < nleaf && leaf_begin[l] < hi; ++l) {
      if (rows.size[row_leaves[l]] == 0) continue;
      per_leaf[l].emplace_back(cols.begin[j], cols.begin[j] + cols.size[j]);
    }
  }
  P.near_ptr.assign(nleaf + 1, 0);
  P.near_ivl.clear();
  for (int l = 0; l < nleaf; ++l) {
    auto& v = per_leaf[l];
    std::sort(v.begin(), v.end());
    size_t start = P.near_ivl.size();
    for (const auto& iv : v) {
      if (P.near_ivl.size() > start && P.near_ivl.back() == iv.first)
        P.near_ivl.back() = iv.second;
      else {
        P.near_ivl.push_back(iv.first);
        P.near_ivl.push_back(iv.second);
      }
    }
    P.near_ptr[l + 1] = (int32_t)(P.near_ivl.size() / 2);
    std::vector<std::pair<uint32_t, uint32_t>>().swap(v);
  }
}

namespace {
// appends tree b to a with cluster ids offset by a's cluster count and point
// indices by a's point count
void append_tree(Tree* a, const Tree& b) {
  const int32_t co = a->nclusters();
  const uint32_t po = a->n;
  a->dim = b.dim;
  for (uint32_t v : b.perm) a->perm.push_back(v + po);
  for (int c = 0; c < b.nclusters(); ++c) {
    a->begin.push_back(b.begin[c] + po);
    a->size.push_back(b.size[c]);
    a->level.push_back(b.level[c]);
    a->parent.push_back(b.parent[c] >= 0 ? b.parent[c] + co : -1);
    a->son0.push_back(b.son0[c] >= 0 ? b.son0[c] + co : -1);
    a->nsons.push_back(b.nsons[c]);
  }
  a->bbmin.insert(a->bbmin.end(), b.bbmin.begin(), b.bbmin.end());
  a->bbmax.insert(a->bbmax.end(), b.bbmax.begin(), b.bbmax.end());
  a->bbext.insert(a->bbext.end(), b.bbext.begin(), b.bbext.end());
  const size_t L = std::max(a->level_ptr.size(), b.level_ptr.size());
  a->level_ptr.assign(L, 0);  // only the number of levels is meaningful
  a->n += b.n;
}
}  // namespace

void Plan::merge(const std::vector<const Plan*>& parts) {
  *this = Plan();
  if (parts.empty()) return;
  interp = parts[0]->interp;
  eta = parts[0]->eta;
  same_tree = true;
  cloud_offsets.assign(1, 0);
  const int dim = interp.dim;
  const int q = interp.q;
  pat.far_ptr.assign(1, 0);
  pat.near_ptr.assign(1, 0);
  for (const Plan* p : parts) {
    same_tree = same_tree && p->same_tree;
    const int32_t rco = rows.nclusters(), cco = cols.nclusters();
    const uint32_t cpo = cols.n;
    // block lists
    for (size_t b = 0; b < p->pat.far_row.size(); ++b) {
      pat.far_row.push_back(p->pat.far_row[b] + rco);
      pat.far_col.push_back(p->pat.far_col[b] + cco);
    }
    for (size_t b = 0; b < p->pat.near_row.size(); ++b) {
      pat.near_row.push_back(p->pat.near_row[b] + rco);
      pat.near_col.push_back(p->pat.near_col[b] + cco);
    }
    const int32_t fo = (int32_t)pat.far_idx.size();
    for (int c = 0; c < p->rows.nclusters(); ++c) pat.far_ptr.push_back(p->pat.far_ptr[c + 1] + fo);
    for (int32_t v : p->pat.far_idx) pat.far_idx.push_back(v + cco);
    const int32_t io = (int32_t)(pat.near_ivl.size() / 2);
    for (size_t l = 0; l + 1 < p->pat.near_ptr.size(); ++l)
      pat.near_ptr.push_back(p->pat.near_ptr[l + 1] + io);
    for (uint32_t v : p->pat.near_ivl) pat.near_ivl.push_back(v + cpo);
    pat.near_pairs += p->pat.near_pairs;
    for (int32_t c : p->row_leaves) row_leaves.push_back(c + rco);
    for (int32_t c : p->col_leaves) col_leaves.push_back(c + cco);
    row_E.insert(row_E.end(), p->row_E.begin(), p->row_E.end());
    col_E.insert(col_E.end(), p->col_E.begin(), p->col_E.end());
    row_nodes.insert(row_nodes.end(), p->row_nodes.begin(), p->row_nodes.end());
    col_nodes.insert(col_nodes.end(), p->col_nodes.begin(), p->col_nodes.end());
    points_r.insert(points_r.end(), p->points_r.begin(), p->points_r.end());
    points_c.insert(points_c.end(), p->points_c.begin(), p->points_c.end());
    append_tree(&rows, p->rows);
    append_tree(&cols, p->cols);
    cloud_offsets.push_back(rows.n);
  }
  (void)dim;
  (void)q;
}

void Plan::statistics(double out[6]) const {
  size_t mem = 0;
  const uint32_t qq = (uint32_t)interp.q * (uint32_t)interp.q;
  for (size_t b = 0; b < pat.far_row.size(); ++b) mem += qq;
  for (size_t b = 0; b < pat.near_row.size(); ++b)
    mem += (uint32_t)(rows.size[pat.near_row[b]] * cols.size[pat.near_col[b]]);
  out[0] = rows.n;
  out[1] = cols.n;
  out[2] = (double)pat.far_row.size();
  out[3] = (double)pat.near_row.size();
  out[4] = std::round(double(mem) / rows.n);
  out[5] = double(mem * sizeof(double)) / 1e9;
}

}  // namespace fmca
