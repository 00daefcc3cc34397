// ORACLE — test infrastructure only; never part of the product path.
//
// FP64 CPU restatement of FMCA's matrix-free H2 kernel matvec, written in the
// reference's own recursive shape (explicit leaf bases V, explicit transfer
// matrices E, a column-bucket scheduler with one OpenMP loop per bucket).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load
// it, and only as a checker / baseline.
//
// Parity status: the reference (muchip/fmca) is a header-only Eigen library;
// Eigen is not available here, so it cannot be compiled or run and there are
// no reference outputs to compare with.  Its tests ship no golden vectors for
// this path.  This restatement is pinned to the reference's own known-answer
// checks only: the transfer-matrix identity < 1e-13
// (FMCA/src/H2Matrix/compute_cluster_bases_impl.h:59-80, run by
// tests/test_H2Matrix.cpp:46-49), permutation completeness
// (tests/test_ClusterTree.cpp:50-57) and the H2-vs-dense compression error
// measured the way tests/test_H2Matrix.cpp:59-74 does.  Value-level parity
// with the reference binary is therefore unpinned.
//
// Followed, function by function:
//   tree       ClusterTreeInitializer_ClusterTree.h:24-132 (init, bounding
//              box, refinement, shrinkToFit), ClusterTreeSplitter.h:60-81
//              (CardinalityBisection), IDDFSForwardIterator.h:37-63 (ids)
//   interp     TensorProductInterpolator.h:39-81, MultiIndexSet.h:87-187;
//              TotalDegreeInterpolator.h:26-47, DeMarchiPoints.h:20-43,
//              evalPolynomials.h:19-63, HaltonSet.h:30-55 (total degree)
//   bases      NystromMoments.h:24-34, compute_cluster_bases_impl.h:28-57
//   pattern    H2MatrixBase.h:160-191, Admissibility.h:19-29,95-115
//   statistics H2MatrixBase.h:70-105
//   action     H2MatrixBase.h:113-152, forward_transform_impl.h:21-43,
//              NystromEvaluator.h:40-56 (S = invV K invV^T, total degree),
//              backward_transform_impl.h:21-33, unsymmetricNystromEvaluator.h:
//              42-73, pyH2Matrix::action py/FMCA.cpp:230-240
//   kernel     CovarianceKernel.h:56-143
//
// Build with -ffp-contract=off (see oracle/build.py).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <set>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using Index = unsigned int;
using Scalar = double;
const Scalar kZeroTol = std::numeric_limits<Scalar>::epsilon();
const Scalar kInf = std::numeric_limits<Scalar>::infinity();

// column-major dense matrix
struct Mat {
  int r = 0, c = 0;
  std::vector<Scalar> a;
  Mat() {}
  Mat(int r_, int c_) : r(r_), c(c_), a((size_t)r_ * c_, 0.) {}
  Scalar& operator()(int i, int j) { return a[(size_t)j * r + i]; }
  Scalar operator()(int i, int j) const { return a[(size_t)j * r + i]; }
};

// C += A * B   (A: m x k, B: k x n)
void gemm_acc(const Mat& A, const Scalar* B, int ldb, int n, Scalar* C, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < A.c; ++k) {
      const Scalar b = B[(size_t)j * ldb + k];
      const Scalar* ak = &A.a[(size_t)k * A.r];
      Scalar* cj = C + (size_t)j * ldc;
      for (int i = 0; i < A.r; ++i) cj[i] += ak[i] * b;
    }
}
// C += A^T * B   (A: k x m, B: k x n)
void gemmT_acc(const Mat& A, const Scalar* B, int ldb, int n, Scalar* C, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < A.c; ++i) {
      const Scalar* ai = &A.a[(size_t)i * A.r];
      const Scalar* bj = B + (size_t)j * ldb;
      Scalar s = 0;
      for (int k = 0; k < A.r; ++k) s += ai[k] * bj[k];
      C[(size_t)j * ldc + i] += s;
    }
}

// ---------------------------------------------------------------------------
struct Interpolator {
  Index dim = 0, deg = 0;
  bool td = false;  // TotalDegreeInterpolator instead of TensorProductInterpolator
  std::vector<Scalar> xi, w;
  std::vector<std::vector<Index>> idcs;  // multi-index set in set order
  Mat TP_xi;                             // dim x q nodes
  Mat invV;                              // total degree: inverse Vandermonde
  void init(Index d, Index p, bool total_degree = false) {
    dim = d;
    deg = p;
    td = total_degree;
    const Scalar weight = 2. * M_PI / (2. * Scalar(deg) + 2.);
    xi.resize(deg + 1);
    w.resize(deg + 1);
    for (Index k = 0; k <= deg; ++k) {
      xi[k] = std::cos(weight * (Scalar(k) + 0.5));
      w[k] = std::sin(weight * (Scalar(k) + 0.5));
    }
    for (auto& v : xi) v = 0.5 * (v + 1);
    for (Index i = 1; i < w.size(); i += 2) w[i] *= -1.;
    // std::set with the graded lexicographic order; generated recursively
    // (MultiIndexSet.h:147-187) under the set's criterion: max entry <= deg
    // (tensor product) or entry sum <= deg (total degree)
    struct Cmp {
      bool operator()(const std::vector<Index>& a, const std::vector<Index>& b) const {
        Index na = 0, nb = 0;
        for (auto v : a) na += v;
        for (auto v : b) nb += v;
        if (na != nb) return na < nb;
        return std::lexicographical_compare(a.begin(), a.end(), b.begin(), b.end());
      }
    };
    std::set<std::vector<Index>, Cmp> s;
    std::vector<Index> index(dim, 0);
    std::function<void(Index)> add = [&](Index max_bit) {
      for (Index i = max_bit; i < dim; ++i) {
        index[i] += 1;
        Index mx = 0, sum = 0;
        for (auto v : index) {
          mx = std::max(mx, v);
          sum += v;
        }
        if ((td ? sum : mx) <= deg) {
          s.insert(index);
          add(i);
        }
        index[i] -= 1;
      }
    };
    s.insert(index);
    add(0);
    idcs.assign(s.begin(), s.end());
    TP_xi = Mat(dim, (int)idcs.size());
    if (td) {
      demarchi();
    } else {
      for (size_t k = 0; k < idcs.size(); ++k)
        for (Index i = 0; i < dim; ++i) TP_xi(i, (int)k) = xi[idcs[k][i]];
    }
  }
  int q() const { return (int)idcs.size(); }

  // L2-normalised Legendre polynomials on [0, 1] (evalPolynomials.h:19-38)
  void legendre(Scalar x, Scalar* f) const {
    Scalar p0 = 0, p1 = 1;
    f[0] = 1;
    for (Index i = 1; i <= deg; ++i) {
      const Scalar v = Scalar(2 * i - 1) / Scalar(i) * (2 * x - 1) * p1 -
                       Scalar(i - 1) / Scalar(i) * p0;
      p0 = p1;
      p1 = v;
      f[i] = v * std::sqrt(Scalar(2 * i + 1));
    }
  }

  // i-th point of the Halton sequence in base b, by Horner's scheme in long
  // double on the b-adic digits (HaltonSet.h:30-55)
  static Scalar halton(unsigned long i, unsigned long b) {
    std::vector<unsigned long> dig;
    while (i) {
      dig.push_back(i % b);
      i /= b;
    }
    if (dig.empty()) return 0;
    const long double binv = (long double)1 / (long double)b;
    long double r = dig.back();
    for (int j = (int)dig.size() - 2; j >= 0; --j) r = binv * r + dig[j];
    r *= binv;
    return (Scalar)r;
  }

  // DeMarchi points (DeMarchiPoints.h:20-43): greedy selection among the
  // Halton points 100 .. 100 + 10 q - 1 of the candidate whose polynomial
  // vector has the largest component orthogonal to the ones chosen (the
  // pivot order of a column-pivoted QR), here by modified Gram-Schmidt
  // with a second orthogonalisation pass; then invV = V^{-1}, V(i, k) =
  // polynomial k at node i, by LU with partial pivoting
  // (TotalDegreeInterpolator.h:40-45)
  void demarchi() {
    const int n = q(), M = 10 * n;
    static const unsigned long primes[3] = {2, 3, 5};
    std::vector<std::vector<Scalar>> cand(M, std::vector<Scalar>(dim));
    std::vector<std::vector<Scalar>> R(M, std::vector<Scalar>(n));
    for (int m = 0; m < M; ++m) {
      for (Index d = 0; d < dim; ++d) cand[m][d] = halton(100 + m, primes[d]);
      eval(cand[m].data(), R[m].data());
    }
    std::vector<char> used(M, 0);
    for (int s = 0; s < n; ++s) {
      int best = -1;
      Scalar bn = -1;
      for (int m = 0; m < M; ++m) {
        if (used[m]) continue;
        Scalar n2 = 0;
        for (int k = 0; k < n; ++k) n2 += R[m][k] * R[m][k];
        if (n2 > bn) {
          bn = n2;
          best = m;
        }
      }
      used[best] = 1;
      for (Index d = 0; d < dim; ++d) TP_xi(d, s) = cand[best][d];
      std::vector<Scalar> u = R[best];
      const Scalar nu = std::sqrt(bn);
      for (auto& v : u) v /= nu;
      for (int m = 0; m < M; ++m) {
        if (used[m]) continue;
        for (int pass = 0; pass < 2; ++pass) {
          Scalar dot = 0;
          for (int k = 0; k < n; ++k) dot += u[k] * R[m][k];
          for (int k = 0; k < n; ++k) R[m][k] -= dot * u[k];
        }
      }
    }
    Mat V(n, n);
    std::vector<Scalar> row(n);
    for (int i = 0; i < n; ++i) {
      std::vector<Scalar> pt(dim);
      for (Index d = 0; d < dim; ++d) pt[d] = TP_xi(d, i);
      eval(pt.data(), row.data());
      for (int k = 0; k < n; ++k) V(i, k) = row[k];
    }
    // LU with partial pivoting, then one solve per unit vector
    std::vector<int> piv(n);
    Mat LU = V;
    for (int k = 0; k < n; ++k) piv[k] = k;
    for (int k = 0; k < n; ++k) {
      int pr = k;
      for (int i = k + 1; i < n; ++i)
        if (std::abs(LU(i, k)) > std::abs(LU(pr, k))) pr = i;
      if (pr != k) {
        for (int j = 0; j < n; ++j) std::swap(LU(k, j), LU(pr, j));
        std::swap(piv[k], piv[pr]);
      }
      for (int i = k + 1; i < n; ++i) {
        LU(i, k) /= LU(k, k);
        for (int j = k + 1; j < n; ++j) LU(i, j) -= LU(i, k) * LU(k, j);
      }
    }
    invV = Mat(n, n);
    std::vector<Scalar> b(n);
    for (int c = 0; c < n; ++c) {
      for (int i = 0; i < n; ++i) b[i] = piv[i] == c ? 1. : 0.;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) b[i] -= LU(i, j) * b[j];
      for (int i = n - 1; i >= 0; --i) {
        for (int j = i + 1; j < n; ++j) b[i] -= LU(i, j) * b[j];
        b[i] /= LU(i, i);
      }
      for (int i = 0; i < n; ++i) invV(i, c) = b[i];
    }
  }

  // full multivariate evaluation, like evalPolynomials / the Lagrange basis
  void eval(const Scalar* pt, Scalar* out) const {
    if (td) {
      std::vector<std::vector<Scalar>> f(dim, std::vector<Scalar>(deg + 1));
      for (Index i = 0; i < dim; ++i) legendre(pt[i], f[i].data());
      for (size_t k = 0; k < idcs.size(); ++k) {
        Scalar v = 1;
        for (Index i = 0; i < dim; ++i) v *= f[i][idcs[k][i]];
        out[k] = v;
      }
      return;
    }
    std::vector<Scalar> weight(dim);
    for (Index i = 0; i < dim; ++i) {
      Scalar s = 0;
      for (Index k = 0; k <= deg; ++k) s += w[k] / (pt[i] - xi[k]);
      weight[i] = s;
    }
    for (size_t k = 0; k < idcs.size(); ++k) {
      Scalar v = 1;
      for (Index i = 0; i < dim; ++i)
        if (std::abs(pt[i] - xi[idcs[k][i]]) > kZeroTol)
          v *= w[idcs[k][i]] / (pt[i] - xi[idcs[k][i]]) / weight[i];
      out[k] = v;
    }
  }
};

// ---------------------------------------------------------------------------
struct Node {
  std::vector<Node> sons;
  Node* dad = nullptr;
  Index level = 0;
  Index begin = 0, size = 0;
  Index block_id = 0;
  std::vector<Scalar> bmin, bmax, bext;
  Mat V;               // leaves: q x size
  std::vector<Mat> E;  // per son: q x q
};

struct Tree {
  Node root;
  std::vector<Index> indices;
  std::vector<Node*> by_id;
  Index dim = 0;
  const Scalar* P = nullptr;

  Scalar p(Index i, Index d) const { return P[(size_t)i * dim + d]; }

  void refine(Node& nd, Index min_csize) {
    const Index thr = min_csize >= 1 ? (2 * min_csize - 1) : 1;
    if (nd.size <= thr) return;
    nd.sons.resize(2);
    for (auto& s : nd.sons) {
      s.dad = &nd;
      s.level = nd.level + 1;
      s.bmin = nd.bmin;
      s.bmax = nd.bmax;
      s.bext = nd.bext;
      s.begin = nd.begin;
      s.size = nd.size;
    }
    Node& c1 = nd.sons[0];
    Node& c2 = nd.sons[1];
    Index longest = 0;
    for (Index d = 1; d < dim; ++d)
      if (c1.bext[d] > c1.bext[longest]) longest = d;
    const Tree* self = this;
    std::sort(indices.begin() + c1.begin, indices.begin() + c1.begin + c1.size,
              [self, longest](Index i, Index j) { return self->p(i, longest) < self->p(j, longest); });
    c1.size /= 2;
    c2.size -= c1.size;
    c2.begin += c1.size;
    c1.bmax[longest] = p(indices[c1.begin + c1.size - 1], longest);
    c1.bext[longest] = c1.bmax[longest] - c1.bmin[longest];
    c2.bmin[longest] = p(indices[c2.begin], longest);
    c2.bext[longest] = c2.bmax[longest] - c2.bmin[longest];
    for (auto& s : nd.sons) refine(s, min_csize);
  }

  void shrink(Node& nd) {
    std::vector<Scalar> lo(dim), hi(dim);
    if (nd.size) {
      for (Index d = 0; d < dim; ++d) lo[d] = hi[d] = p(indices[nd.begin], d);
      if (nd.sons.size()) {
        for (auto& s : nd.sons) {
          shrink(s);
          if (s.size)
            for (Index d = 0; d < dim; ++d) {
              lo[d] = std::min(lo[d], s.bmin[d]);
              hi[d] = std::max(hi[d], s.bmax[d]);
            }
        }
      } else {
        for (Index i = 0; i < nd.size; ++i)
          for (Index d = 0; d < dim; ++d) {
            lo[d] = std::min(p(indices[nd.begin + i], d), lo[d]);
            hi[d] = std::max(p(indices[nd.begin + i], d), hi[d]);
          }
      }
    } else {
      for (Index d = 0; d < dim; ++d) {
        lo[d] = kInf;
        hi[d] = -kInf;
      }
    }
    std::vector<Scalar> ex(dim);
    for (Index d = 0; d < dim; ++d) ex[d] = hi[d] - lo[d];
    for (Index d = 0; d < dim; ++d)
      if (hi[d] - lo[d] < 2e2 * kZeroTol) {
        hi[d] += 1e2 * kZeroTol;
        lo[d] -= 1e2 * kZeroTol;
        ex[d] = hi[d] - lo[d];
      }
    nd.bmin = lo;
    nd.bmax = hi;
    nd.bext = ex;
  }

  // level-wise numbering by iterative deepening
  void number() {
    by_id.clear();
    Index depth = 0;
    while (true) {
      size_t before = by_id.size();
      std::function<void(Node&)> visit = [&](Node& nd) {
        if (nd.level == depth) {
          nd.block_id = (Index)by_id.size();
          by_id.push_back(&nd);
          return;
        }
        for (auto& s : nd.sons) visit(s);
      };
      visit(root);
      if (by_id.size() == before) break;
      ++depth;
    }
  }

  void init(const Scalar* P_, Index d, Index n, Index min_csize) {
    P = P_;
    dim = d;
    root.bmin.resize(dim);
    root.bmax.resize(dim);
    root.bext.resize(dim);
    for (Index k = 0; k < dim; ++k) {
      Scalar lo = P[k], hi = P[k];
      for (Index i = 1; i < n; ++i) {
        lo = std::min(lo, p(i, k));
        hi = std::max(hi, p(i, k));
      }
      root.bmin[k] = lo - kZeroTol * std::abs(lo);
      root.bmax[k] = hi + kZeroTol * std::abs(hi);
      root.bext[k] = root.bmax[k] - root.bmin[k];
    }
    root.begin = 0;
    root.size = n;
    indices.resize(n);
    for (Index i = 0; i < n; ++i) indices[i] = i;
    refine(root, min_csize);
    shrink(root);
    number();
  }

  // leaf moment matrix (NystromMoments::moment_matrix) of any node
  Mat moments(const Node& nd, const Interpolator& ip) const {
    Mat M(ip.q(), (int)nd.size);
    std::vector<Scalar> pt(dim);
    for (Index i = 0; i < nd.size; ++i) {
      for (Index d = 0; d < dim; ++d)
        pt[d] = (p(indices[nd.begin + i], d) - nd.bmin[d]) / nd.bext[d];
      ip.eval(pt.data(), &M.a[(size_t)i * M.r]);
    }
    return M;
  }

  void bases(Node& nd, const Interpolator& ip) {
    nd.V = Mat();
    nd.E.clear();
    if (nd.sons.size()) {
      for (auto& s : nd.sons) bases(s, ip);
      const int q = ip.q();
      std::vector<Scalar> pt(dim);
      for (auto& s : nd.sons) {
        Mat E(q, q);
        if (s.size)
          for (int j = 0; j < q; ++j) {
            for (Index d = 0; d < dim; ++d)
              pt[d] = ip.TP_xi(d, j) * s.bext[d] / nd.bext[d] +
                      (s.bmin[d] - nd.bmin[d]) / nd.bext[d];
            ip.eval(pt.data(), &E.a[(size_t)j * q]);
          }
        if (ip.td) {  // E = E invV^T (compute_cluster_bases_impl.h:50)
          Mat F(q, q);
          for (int jj = 0; jj < q; ++jj)
            for (int j = 0; j < q; ++j) {
              const Scalar v = ip.invV(jj, j);
              for (int k = 0; k < q; ++k) F(k, jj) += E(k, j) * v;
            }
          E = std::move(F);
        }
        nd.E.push_back(std::move(E));
      }
    } else {
      nd.V = moments(nd, ip);
    }
  }
};

// ---------------------------------------------------------------------------
using KernelFn = std::function<Scalar(Scalar)>;

KernelFn make_kernel(int type, Scalar l, Scalar c) {
  switch (type) {
    case 0: return [l](Scalar r) { return std::exp(-r / l); };
    case 1: return [l](Scalar r) { return (1. + std::sqrt(3.) / l * r) * std::exp(-std::sqrt(3.) * r / l); };
    case 2:
      return [l](Scalar r) {
        return (1. + std::sqrt(5.) / l * r + 5 * r * r / (3 * l * l)) * std::exp(-std::sqrt(5.) * r / l);
      };
    case 3: return [l](Scalar r) { return std::exp(-0.5 * r * r / (l * l)); };
    case 4:
      return [l](Scalar r) {
        return (1. + std::sqrt(7.) / l * r + 14. / 5 * std::pow(r / l, 2.) +
                7. * std::sqrt(7.) / 15. * std::pow(r / l, 3.)) *
               std::exp(-std::sqrt(7.) * r / l);
      };
    case 5:
      return [l](Scalar r) {
        return (1. + 3. / l * r + 27. / 7. * std::pow(r / l, 2.) + 18. / 7. * std::pow(r / l, 3.) +
                27. / 35. * std::pow(r / l, 4.)) *
               std::exp(-3 * r / l);
      };
    case 6: return [l, c](Scalar r) { return 1. / std::sqrt((r / l) * (r / l) + c * c); };
    case 7: return [l, c](Scalar r) { return std::sqrt((r / l) * (r / l) + c * c); };
    case 8: return [l](Scalar r) { return r / l; };
    case 9: return [l](Scalar r) { return (r / l) * (r / l) * (r / l); };
    // length-scale derivatives dk/dl of kernels 0..3
    case 10: return [l](Scalar r) { return r / (l * l) * std::exp(-r / l); };
    case 11:
      return [l](Scalar r) {
        const Scalar a = std::sqrt(3.) / l;
        return a * a * r * r / l * std::exp(-a * r);
      };
    case 12:
      return [l](Scalar r) {
        const Scalar a = std::sqrt(5.) / l;
        return a * a * r * r / (3. * l) * (1. + a * r) * std::exp(-a * r);
      };
    case 13: return [l](Scalar r) { return r * r / (l * l * l) * std::exp(-0.5 * r * r / (l * l)); };
    // BIHARMONIC2D and TPS2D (CovarianceKernel.h:56-59, 117-118)
    case 14:
      return [l](Scalar r) {
        return r < std::numeric_limits<Scalar>::epsilon() ? 0 : std::log(r / l) * (r / l) * (r / l);
      };
    case 15: return [](Scalar r) { return r > 0 ? r * r * std::log(r) : 0; };
  }
  return [](Scalar) { return std::numeric_limits<Scalar>::quiet_NaN(); };
}

inline Scalar dist(const Scalar* x, const Scalar* y, Index dim) {
  Scalar s = 0;
  for (Index d = 0; d < dim; ++d) {
    const Scalar t = x[d] - y[d];
    s = d == 0 ? t * t : s + t * t;
  }
  return std::sqrt(s);
}

struct Block {
  Node* row;
  Node* col;
  bool low_rank;
};

struct OPlan {
  Index dim = 0;
  Interpolator ip;
  Tree rt, ct;
  std::vector<Scalar> Pr, Pc;
  std::vector<Block> blocks;  // leaves of the block tree, in DFS pop order
  Scalar eta = 0.8;
  // kept by oracle_action when asked (keep != 0), for oracle_action_part:
  // x in cluster order and the column clusters' moments of that call
  std::vector<Scalar> kept_srhs;
  std::vector<Mat> kept_t;
  int kept_R = 0;
  bool keep = false;
};

enum { kRefine = 0, kLowRank = 1, kDense = 2 };

int compare(const Node& a, const Node& b, Index dim, Scalar eta) {
  auto nrm = [dim](const std::vector<Scalar>& v) {
    Scalar s = 0;
    for (Index d = 0; d < dim; ++d) s = d == 0 ? v[d] * v[d] : s + v[d] * v[d];
    return std::sqrt(s);
  };
  const Scalar r1 = 0.5 * nrm(a.bext);
  const Scalar r2 = 0.5 * nrm(b.bext);
  std::vector<Scalar> m(dim);
  for (Index d = 0; d < dim; ++d) m[d] = 0.5 * (a.bmin[d] - b.bmin[d] + a.bmax[d] - b.bmax[d]);
  Scalar dd = nrm(m) - r1 - r2;
  dd = dd > 0 ? dd : 0;
  const Scalar radius = r1 > r2 ? r1 : r2;
  if (radius > eta * dd) return (!a.sons.size() || !b.sons.size()) ? kDense : kRefine;
  return kLowRank;
}

void pattern(OPlan* P) {
  const Index q = (Index)P->ip.q();
  std::vector<std::pair<Node*, Node*>> stack;
  stack.emplace_back(&P->rt.root, &P->ct.root);
  while (!stack.empty()) {
    auto b = stack.back();
    stack.pop_back();
    const int adm = compare(*b.first, *b.second, P->dim, P->eta);
    if (adm == kLowRank) {
      const Index brows = q, bcols = q;
      P->blocks.push_back({b.first, b.second, brows * bcols < b.first->size * b.second->size});
    } else if (adm == kRefine) {
      for (size_t j = 0; j < b.second->sons.size(); ++j)
        for (size_t i = 0; i < b.first->sons.size(); ++i)
          stack.emplace_back(&b.first->sons[i], &b.second->sons[j]);
    } else {
      P->blocks.push_back({b.first, b.second, false});
    }
  }
}

void forward(const Node& nd, const Tree& t, const Scalar* x, int ldx, int R,
             std::vector<Mat>* tv) {
  Mat& out = (*tv)[nd.block_id];
  const int q = nd.sons.size() ? nd.E[0].r : nd.V.r;
  out = Mat(q, R);
  if (nd.sons.size()) {
    for (size_t i = 0; i < nd.sons.size(); ++i) {
      forward(nd.sons[i], t, x, ldx, R, tv);
      gemm_acc(nd.E[i], (*tv)[nd.sons[i].block_id].a.data(), q, R, out.a.data(), q);
    }
  } else {
    gemm_acc(nd.V, x + nd.begin, ldx, R, out.a.data(), q);
  }
}

void backward(const Node& nd, Scalar* y, int ldy, int R, std::vector<Mat>& tv) {
  if (nd.sons.size()) {
    for (size_t i = 0; i < nd.sons.size(); ++i) {
      const Mat& dad = tv[nd.block_id];
      gemmT_acc(nd.E[i], dad.a.data(), dad.r, R, tv[nd.sons[i].block_id].a.data(),
                tv[nd.sons[i].block_id].r);
      backward(nd.sons[i], y, ldy, R, tv);
    }
  } else {
    const Mat& s = tv[nd.block_id];
    gemmT_acc(nd.V, s.a.data(), s.r, R, y + nd.begin, ldy);
  }
}

// backward() for a subtree whose rows start at row0 of y
void backward_part(const Node& nd, Index row0, Scalar* y, int ldy, int R, std::vector<Mat>& tv) {
  if (nd.sons.size()) {
    for (size_t i = 0; i < nd.sons.size(); ++i) {
      const Mat& dad = tv[nd.block_id];
      gemmT_acc(nd.E[i], dad.a.data(), dad.r, R, tv[nd.sons[i].block_id].a.data(),
                tv[nd.sons[i].block_id].r);
      backward_part(nd.sons[i], row0, y, ldy, R, tv);
    }
  } else {
    const Mat& s = tv[nd.block_id];
    gemmT_acc(nd.V, s.a.data(), s.r, R, y + (nd.begin - row0), ldy);
  }
}

Scalar check_transfer(Node& nd, const Tree& t, const Interpolator& ip, Mat* Vout) {
  if (!nd.sons.size()) {
    *Vout = nd.V;
    return 0;
  }
  Scalar worst = 0;
  std::vector<Mat> sonV(nd.sons.size());
  for (size_t i = 0; i < nd.sons.size(); ++i)
    worst = std::max(worst, check_transfer(nd.sons[i], t, ip, &sonV[i]));
  Mat V = t.moments(nd, ip);
  Mat W(ip.q(), 0);
  for (size_t i = 0; i < nd.sons.size(); ++i) {
    Mat part(ip.q(), sonV[i].c);
    gemm_acc(nd.E[i], sonV[i].a.data(), sonV[i].r, sonV[i].c, part.a.data(), part.r);
    W.a.insert(W.a.end(), part.a.begin(), part.a.end());
    W.c += part.c;
  }
  Scalar num = 0, den = 0;
  for (size_t k = 0; k < V.a.size(); ++k) {
    num += (V.a[k] - W.a[k]) * (V.a[k] - W.a[k]);
    den += V.a[k] * V.a[k];
  }
  *Vout = std::move(W);
  return std::max(worst, std::sqrt(num) / std::sqrt(den));
}

}  // namespace

extern "C" {

void* oracle_plan_create_ex(const double* Pr, int dim, int64_t nr, const double* Pc,
                            int64_t nc, int deg, double eta, int64_t min_leaf,
                            int total_degree) {
  OPlan* P = new OPlan();
  P->dim = (Index)dim;
  P->eta = eta;
  P->ip.init((Index)dim, (Index)deg, total_degree != 0);
  const bool same = (Pc == nullptr || Pc == Pr);
  P->Pr.assign(Pr, Pr + (size_t)dim * nr);
  if (same) {
    P->Pc = P->Pr;
    nc = nr;
  } else {
    P->Pc.assign(Pc, Pc + (size_t)dim * nc);
  }
  const Index q = (Index)P->ip.q();
  const Index m = (Index)min_leaf > q ? (Index)min_leaf : q;
  P->rt.init(P->Pr.data(), (Index)dim, (Index)nr, m);
  P->ct.init(P->Pc.data(), (Index)dim, (Index)nc, m);
  P->rt.bases(P->rt.root, P->ip);
  P->ct.bases(P->ct.root, P->ip);
  pattern(P);
  return P;
}

void* oracle_plan_create(const double* Pr, int dim, int64_t nr, const double* Pc,
                         int64_t nc, int deg, double eta, int64_t min_leaf) {
  return oracle_plan_create_ex(Pr, dim, nr, Pc, nc, deg, eta, min_leaf, 0);
}

// total degree: the q nodes (dim x q, column-major) and invV (q x q,
// column-major); returns q
int oracle_interp(void* h, double* nodes, double* invV) {
  const Interpolator& ip = static_cast<OPlan*>(h)->ip;
  const int q = ip.q();
  if (nodes) std::copy(ip.TP_xi.a.begin(), ip.TP_xi.a.end(), nodes);
  if (invV && ip.td) std::copy(ip.invV.a.begin(), ip.invV.a.end(), invV);
  return q;
}

void oracle_plan_destroy(void* h) { delete static_cast<OPlan*>(h); }

// counts: [row clusters, col clusters, far blocks, dense blocks, q,
//          dense point pairs]
void oracle_counts(void* h, int64_t* out) {
  OPlan* P = static_cast<OPlan*>(h);
  int64_t nf = 0, nd = 0, pairs = 0;
  for (auto& b : P->blocks) {
    (b.low_rank ? nf : nd)++;
    if (!b.low_rank) pairs += (int64_t)b.row->size * (int64_t)b.col->size;
  }
  out[0] = (int64_t)P->rt.by_id.size();
  out[1] = (int64_t)P->ct.by_id.size();
  out[2] = nf;
  out[3] = nd;
  out[4] = P->ip.q();
  out[5] = pairs;
}

void oracle_perm(void* h, int side, uint32_t* out) {
  OPlan* P = static_cast<OPlan*>(h);
  const Tree& t = side == 0 ? P->rt : P->ct;
  std::memcpy(out, t.indices.data(), sizeof(uint32_t) * t.indices.size());
}

// meta: (begin, size, level, parent id) per cluster; bb: (min, max, ext)
void oracle_clusters(void* h, int side, int32_t* meta, double* bb) {
  OPlan* P = static_cast<OPlan*>(h);
  const Tree& t = side == 0 ? P->rt : P->ct;
  const Index dim = P->dim;
  for (size_t c = 0; c < t.by_id.size(); ++c) {
    const Node& nd = *t.by_id[c];
    meta[4 * c + 0] = (int32_t)nd.begin;
    meta[4 * c + 1] = (int32_t)nd.size;
    meta[4 * c + 2] = (int32_t)nd.level;
    meta[4 * c + 3] = nd.dad ? (int32_t)nd.dad->block_id : -1;
    for (Index d = 0; d < dim; ++d) {
      bb[c * 3 * dim + d] = nd.bmin[d];
      bb[c * 3 * dim + dim + d] = nd.bmax[d];
      bb[c * 3 * dim + 2 * dim + d] = nd.bext[d];
    }
  }
}

// kind 0: low-rank, 1: dense
void oracle_blocks(void* h, int kind, int32_t* rows, int32_t* cols) {
  OPlan* P = static_cast<OPlan*>(h);
  size_t k = 0;
  for (auto& b : P->blocks)
    if (b.low_rank == (kind == 0)) {
      rows[k] = (int32_t)b.row->block_id;
      cols[k] = (int32_t)b.col->block_id;
      ++k;
    }
}

// statistics() of the reference
void oracle_statistics(void* h, double* out) {
  OPlan* P = static_cast<OPlan*>(h);
  const Index q = (Index)P->ip.q();
  size_t lr = 0, f = 0, mem = 0;
  for (auto& b : P->blocks) {
    if (b.low_rank) {
      ++lr;
      mem += q * q;
    } else {
      ++f;
      mem += b.row->size * b.col->size;
    }
  }
  out[0] = P->rt.root.size;
  out[1] = P->ct.root.size;
  out[2] = (double)lr;
  out[3] = (double)f;
  out[4] = std::round(double(mem) / P->rt.root.size);
  out[5] = double(mem * sizeof(double)) / 1e9;
}

// largest relative error of the transfer identity over both trees
double oracle_check_transfer(void* h) {
  OPlan* P = static_cast<OPlan*>(h);
  Mat V;
  const double a = check_transfer(P->rt.root, P->rt, P->ip, &V);
  const double b = check_transfer(P->ct.root, P->ct, P->ip, &V);
  return std::max(a, b);
}

// y (n_r x R, column-major, natural order) = sigma2 * H2(x).
// bucket_stride > 1 processes only every bucket_stride-th column bucket
// (a bounded sample for timing); work[0..1] receive the dense pairs and the
// interpolated pairs (q^2 per low-rank block) processed.
static void action_impl(OPlan* P, int ktype, double l, double c, double sigma2,
                        const double* x, int R, double* y, int bucket_stride, double* work,
                        std::vector<Mat>* leaf_expansions);

void oracle_action(void* h, int ktype, double l, double c, double sigma2,
                   const double* x, int R, double* y, int bucket_stride,
                   int nthreads, double* work) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  action_impl(static_cast<OPlan*>(h), ktype, l, c, sigma2, x, R, y, bucket_stride, work,
              nullptr);
}

}  // extern "C"

// One leaf of the block tree applied to the product (the body of the
// column-bucket loop of H2MatrixBase::action, H2MatrixBase.h:127-148):
// low-rank blocks add S t_sigma to the row cluster's expansion, dense blocks
// S x_sigma to the rows of lhs (row i of the product at lhs[i - row0], column
// stride ldl).
static void apply_block(const OPlan* P, const KernelFn& kern, const Block& b,
                        const Scalar* srhs, int nc, int R, const std::vector<Mat>& trhs,
                        std::vector<Mat>* tlhs_p, Scalar* lhs, Index row0, int ldl,
                        double* dense_pairs, double* lr_pairs) {
  const Index dim = P->dim;
  const int q = P->ip.q();
  std::vector<Mat>& tlhs = *tlhs_p;
  // node coordinates of a cluster (XiX in NystromEvaluator::interpolate_kernel)
  auto nodes = [&](const Node& nd) {
    Mat X(dim, q);
    for (int k = 0; k < q; ++k)
      for (Index d = 0; d < dim; ++d) X(d, k) = P->ip.TP_xi(d, k) * nd.bext[d] + nd.bmin[d];
    return X;
  };
  const Node& row = *b.row;
  const Node& col = *b.col;
  if (b.low_rank) {
    const Mat XiX = nodes(row), XiY = nodes(col);
    Mat S(q, q);
    for (int j = 0; j < q; ++j)
      for (int i = 0; i < q; ++i)
        S(i, j) = kern(dist(&XiX.a[(size_t)i * dim], &XiY.a[(size_t)j * dim], dim));
    if (P->ip.td) {  // S = invV S invV^T (NystromEvaluator.h:50-54)
      Mat A(q, q), B(q, q);
      for (int j = 0; j < q; ++j)
        for (int m = 0; m < q; ++m) {
          const Scalar v = S(m, j);
          for (int i = 0; i < q; ++i) A(i, j) += P->ip.invV(i, m) * v;
        }
      for (int j = 0; j < q; ++j)
        for (int m = 0; m < q; ++m) {
          const Scalar v = P->ip.invV(j, m);
          for (int i = 0; i < q; ++i) B(i, j) += A(i, m) * v;
        }
      S = std::move(B);
    }
    const Mat& t = trhs[col.block_id];
    gemm_acc(S, t.a.data(), q, R, tlhs[row.block_id].a.data(), q);
    *lr_pairs += (double)q * q;
  } else {
    Mat S((int)row.size, (int)col.size);
    for (Index j = 0; j < col.size; ++j)
      for (Index i = 0; i < row.size; ++i)
        S((int)i, (int)j) =
            kern(dist(&P->Pr[(size_t)P->rt.indices[row.begin + i] * dim],
                      &P->Pc[(size_t)P->ct.indices[col.begin + j] * dim], dim));
    gemm_acc(S, srhs + col.begin, nc, R, lhs + (row.begin - row0), ldl);
    *dense_pairs += (double)row.size * col.size;
  }
}

// the action; optionally returns the row-cluster expansions after the
// downward pass (at the leaves: what V^T multiplies)
static void action_impl(OPlan* P, int ktype, double l, double c, double sigma2,
                        const double* x, int R, double* y, int bucket_stride, double* work,
                        std::vector<Mat>* leaf_expansions) {
  const KernelFn kern = make_kernel(ktype, l, c);
  const int nr = (int)P->rt.root.size, nc = (int)P->ct.root.size;
  const int q = P->ip.q();
  // srhs = P^T rhs: cluster order
  std::vector<Scalar> srhs((size_t)nc * R);
  for (int r = 0; r < R; ++r)
    for (int i = 0; i < nc; ++i)
      srhs[(size_t)r * nc + i] = x[(size_t)r * nc + P->ct.indices[i]];
  std::vector<Scalar> lhs((size_t)nr * R, 0.);
  std::vector<Mat> trhs(P->ct.by_id.size());
  forward(P->ct.root, P->ct, srhs.data(), nc, R, &trhs);
  std::vector<Mat> tlhs(P->rt.by_id.size());
  for (auto* nd : P->rt.by_id) tlhs[nd->block_id] = Mat(q, R);
  std::vector<std::vector<const Block*>> sched(P->ct.by_id.size());
  for (auto& b : P->blocks) sched[b.col->block_id].push_back(&b);
  double dense_pairs = 0, lr_pairs = 0;
  const int stride = bucket_stride > 1 ? bucket_stride : 1;
  for (size_t bj = 0; bj < sched.size(); ++bj) {
    if ((int)(bj % stride) != 0) continue;
    const auto& bucket = sched[bj];
#pragma omp parallel for schedule(dynamic) reduction(+ : dense_pairs, lr_pairs)
    for (long k = 0; k < (long)bucket.size(); ++k)
      apply_block(P, kern, *bucket[k], srhs.data(), nc, R, trhs, &tlhs, lhs.data(), 0, nr,
                  &dense_pairs, &lr_pairs);
  }
  backward(P->rt.root, lhs.data(), nr, R, tlhs);
  for (int r = 0; r < R; ++r)
    for (int i = 0; i < nr; ++i)
      y[(size_t)r * nr + P->rt.indices[i]] = sigma2 * lhs[(size_t)r * nr + i];
  if (work) {
    work[0] = dense_pairs;
    work[1] = lr_pairs;
  }
  if (leaf_expansions) *leaf_expansions = std::move(tlhs);
  if (P->keep) {
    P->kept_srhs = std::move(srhs);
    P->kept_t = std::move(trhs);
    P->kept_R = R;
  }
}

// marks nd and every cluster below it
static void mark_subtree(const Node& nd, std::vector<char>* mark) {
  (*mark)[nd.block_id] = 1;
  for (const Node& s : nd.sons) mark_subtree(s, mark);
}

extern "C" {

// Keep (on != 0) x in cluster order and the moments of the following
// oracle_action calls for oracle_action_part.
void oracle_set_keep(void* h, int on) {
  OPlan* P = static_cast<OPlan*>(h);
  P->keep = on != 0;
  if (!P->keep) {
    P->kept_srhs = std::vector<Scalar>();
    P->kept_t = std::vector<Mat>();
    P->kept_R = 0;
  }
}

// Part `part` of `nparts` of one product, for bounded timing samples of the
// CPU baseline without extrapolation.  nparts must be the number of clusters
// of one level L of both trees (a power of two for these binary trees); the
// part is row cluster and column cluster number `part` of level L.  The part
// does exactly the work the full product spends on them: x gathered to
// cluster order for the column cluster's points, the upward pass inside the
// column subtree, every block whose row cluster lies in the row subtree
// (column buckets in the order of the full product), the downward pass
// inside the row subtree.  The work of the levels above L is shared by all
// parts and is done by each of them (moments of the column ancestors, blocks
// of the row ancestors, the downward pass along the path to the part).
// The other column clusters' moments and x values come from the last
// oracle_action with oracle_set_keep on, which must have had the same x: the
// rows of the row subtree then equal that product's rows bit for bit.
// Writes y (n_r x R, natural order) on those rows only and returns their
// first cluster-order row and count in rows[0..1] (-1, -1 if the plan kept
// nothing for this R or nparts is not a level's cluster count).
void oracle_action_part(void* h, int ktype, double l, double c, double sigma2,
                        const double* x, int R, double* y, int part, int nparts,
                        int nthreads, double* work, int64_t* rows) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  OPlan* P = static_cast<OPlan*>(h);
  rows[0] = rows[1] = -1;
  if (P->kept_R != R || P->kept_t.size() != P->ct.by_id.size() || part < 0 || part >= nparts)
    return;
  // the clusters of the first level with nparts clusters (level order)
  auto level_nodes = [nparts](const Tree& t) {
    std::vector<Node*> out;
    for (Node* nd : t.by_id) {
      if (!out.empty() && nd->level != out.back()->level) {
        if ((int)out.size() == nparts) break;
        out.clear();
      }
      out.push_back(nd);
    }
    if ((int)out.size() != nparts) out.clear();
    return out;
  };
  const std::vector<Node*> rl = level_nodes(P->rt), cl = level_nodes(P->ct);
  if ((int)rl.size() != nparts || (int)cl.size() != nparts) return;
  const Node& rs = *rl[part];
  const Node& cs = *cl[part];
  const KernelFn kern = make_kernel(ktype, l, c);
  const int nr = (int)P->rt.root.size, nc = (int)P->ct.root.size;
  const int q = P->ip.q();
  std::vector<Scalar>& srhs = P->kept_srhs;
  std::vector<Mat>& trhs = P->kept_t;
  // x of the column subtree in cluster order; its moments, then those of
  // its ancestors
  for (int r = 0; r < R; ++r)
    for (Index i = cs.begin; i < cs.begin + cs.size; ++i)
      srhs[(size_t)r * nc + i] = x[(size_t)r * nc + P->ct.indices[i]];
  forward(cs, P->ct, srhs.data(), nc, R, &trhs);
  for (const Node* a = cs.dad; a; a = a->dad) {
    Mat& out = trhs[a->block_id];
    out = Mat(q, R);
    for (size_t i = 0; i < a->sons.size(); ++i)
      gemm_acc(a->E[i], trhs[a->sons[i].block_id].a.data(), q, R, out.a.data(), q);
  }
  // blocks whose row cluster is in the row subtree or one of its ancestors
  std::vector<char> mine(P->rt.by_id.size(), 0);
  mark_subtree(rs, &mine);
  for (const Node* a = rs.dad; a; a = a->dad) mine[a->block_id] = 1;
  std::vector<Mat> tlhs(P->rt.by_id.size());
  for (const Node* nd : P->rt.by_id)
    if (mine[nd->block_id]) tlhs[nd->block_id] = Mat(q, R);
  // the part's blocks grouped by row cluster, each group in column-bucket
  // order: every row then accumulates its blocks in the order of the full
  // product.  The groups run in parallel (one OpenMP loop over the part's
  // row clusters: its column buckets are too small to keep the threads
  // busy one bucket at a time), which is exact as long as no two row
  // clusters with dense blocks share points; otherwise the full product's
  // bucket-by-bucket loop is used.
  std::vector<std::vector<const Block*>> byrow(P->rt.by_id.size());
  // rows [row0, row1) of lhs: the subtree's, and those of dense blocks of
  // ancestors (which also cover rows outside the part; they are dropped)
  Index row0 = rs.begin, row1 = rs.begin + rs.size;
  for (auto& b : P->blocks)
    if (mine[b.row->block_id]) {
      byrow[b.row->block_id].push_back(&b);
      if (!b.low_rank) {
        row0 = std::min(row0, b.row->begin);
        row1 = std::max(row1, b.row->begin + b.row->size);
      }
    }
  std::vector<const Node*> groups;
  std::vector<std::pair<Index, Index>> dense_rows;  // (begin, end) of rows with dense blocks
  for (const Node* nd : P->rt.by_id) {
    auto& g = byrow[nd->block_id];
    if (g.empty()) continue;
    std::sort(g.begin(), g.end(), [](const Block* a, const Block* b) {
      return a->col->block_id < b->col->block_id;
    });
    groups.push_back(nd);
    for (const Block* b : g)
      if (!b->low_rank && nd->size) {
        dense_rows.emplace_back(nd->begin, nd->begin + nd->size);
        break;
      }
  }
  std::sort(dense_rows.begin(), dense_rows.end());
  bool disjoint = true;
  for (size_t i = 1; i < dense_rows.size(); ++i)
    disjoint = disjoint && dense_rows[i].first >= dense_rows[i - 1].second;
  const int ldl = (int)(row1 - row0);
  std::vector<Scalar> lhs((size_t)ldl * R, 0.);
  double dense_pairs = 0, lr_pairs = 0;
  if (disjoint) {
#pragma omp parallel for schedule(dynamic) reduction(+ : dense_pairs, lr_pairs)
    for (long gi = 0; gi < (long)groups.size(); ++gi)
      for (const Block* b : byrow[groups[gi]->block_id])
        apply_block(P, kern, *b, srhs.data(), nc, R, trhs, &tlhs, lhs.data(), row0, ldl,
                    &dense_pairs, &lr_pairs);
  } else {
    std::vector<std::vector<const Block*>> sched(P->ct.by_id.size());
    for (const Node* nd : groups)
      for (const Block* b : byrow[nd->block_id]) sched[b->col->block_id].push_back(b);
    for (size_t bj = 0; bj < sched.size(); ++bj) {
      const auto& bucket = sched[bj];
      if (bucket.empty()) continue;
#pragma omp parallel for schedule(dynamic) reduction(+ : dense_pairs, lr_pairs)
      for (long k = 0; k < (long)bucket.size(); ++k)
        apply_block(P, kern, *bucket[k], srhs.data(), nc, R, trhs, &tlhs, lhs.data(), row0, ldl,
                    &dense_pairs, &lr_pairs);
    }
  }
  // downward pass: along the path from the root to the row subtree (dense
  // blocks of ancestors write rows of the subtree only through lhs), then
  // inside it
  std::vector<const Node*> path;
  for (const Node* a = &rs; a; a = a->dad) path.push_back(a);
  for (size_t k = path.size() - 1; k >= 1; --k) {
    const Node& dad = *path[k];
    const Node& son = *path[k - 1];
    const size_t i = (size_t)(&son - dad.sons.data());
    gemmT_acc(dad.E[i], tlhs[dad.block_id].a.data(), q, R, tlhs[son.block_id].a.data(), q);
  }
  backward_part(rs, row0, lhs.data(), ldl, R, tlhs);
  for (int r = 0; r < R; ++r)
    for (Index i = rs.begin; i < rs.begin + rs.size; ++i)
      y[(size_t)r * nr + P->rt.indices[i]] = sigma2 * lhs[(size_t)r * ldl + (i - row0)];
  if (work) {
    work[0] = dense_pairs;
    work[1] = lr_pairs;
  }
  rows[0] = rs.begin;
  rows[1] = rs.size;
}

}  // extern "C"

namespace {
// Lagrange basis of the nodes xi in product form and its derivative:
// l_a(x) = prod_{b != a} (x - xi_b) / (xi_a - xi_b),
// l_a'(x) = sum_{m != a} 1 / (xi_a - xi_m) prod_{b != a, m} (x - xi_b) / (xi_a - xi_b)
void lagrange_product(const std::vector<Scalar>& xi, Scalar x, Scalar* f, Scalar* df) {
  const int n = (int)xi.size();
  for (int a = 0; a < n; ++a) {
    Scalar v = 1, dv = 0;
    for (int b = 0; b < n; ++b)
      if (b != a) v *= (x - xi[b]) / (xi[a] - xi[b]);
    for (int m = 0; m < n; ++m) {
      if (m == a) continue;
      Scalar t = 1. / (xi[a] - xi[m]);
      for (int b = 0; b < n; ++b)
        if (b != a && b != m) t *= (x - xi[b]) / (xi[a] - xi[b]);
      dv += t;
    }
    f[a] = v;
    df[a] = dv;
  }
}

// k'(r) / r of kernels 0..3
Scalar kernel_grad_over_r(int ktype, Scalar l, Scalar r) {
  if (r <= 0) return 0;
  switch (ktype) {
    case 0: return -std::exp(-r / l) / (l * r);
    case 1: {
      const Scalar a = std::sqrt(3.) / l;
      return -a * a * std::exp(-a * r);
    }
    case 2: {
      const Scalar a = std::sqrt(5.) / l;
      return -(a * a / 3.) * (1. + a * r) * std::exp(-a * r);
    }
    case 3: return -std::exp(-0.5 * r * r / (l * l)) / (l * l);
  }
  return std::numeric_limits<Scalar>::quiet_NaN();
}
}  // namespace

extern "C" {

// Gradients of f = sum_r y_r^T K x_r, K = sigma2 H2[k], tree and boxes fixed,
// for one point cloud: values = (f, df/dl, df/dsigma2), dX (n x dim,
// row-major, natural order).  Kernels 0..3.
void oracle_adjoint(void* h, int ktype, double l, double sigma2, const double* x,
                    const double* y, int R, double* values, double* dX, int nthreads) {
  OPlan* P = static_cast<OPlan*>(h);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const int n = (int)P->rt.root.size, dim = (int)P->dim, q = P->ip.q();
  std::vector<Scalar> z((size_t)n * R);
  std::vector<Mat> Ux, Uy;
  action_impl(P, ktype, l, 1., 1., x, R, z.data(), 1, nullptr, &Ux);
  Scalar f1 = 0;
  for (size_t e = 0; e < z.size(); ++e) f1 += y[e] * z[e];
  action_impl(P, ktype + 10, l, 1., 1., x, R, z.data(), 1, nullptr, nullptr);
  Scalar fl = 0;
  for (size_t e = 0; e < z.size(); ++e) fl += y[e] * z[e];
  values[0] = sigma2 * f1;
  values[1] = sigma2 * fl;
  values[2] = f1;
  action_impl(P, ktype, l, 1., 1., y, R, z.data(), 1, nullptr, &Uy);
  std::vector<Scalar> G((size_t)n * dim, 0.);
  const Scalar* X = P->Pr.data();
  const std::vector<Index>& idx = P->rt.indices;
  // near field: both sides of every dense pair
  for (const Block& b : P->blocks) {
    if (b.low_rank) continue;
    for (Index i = 0; i < b.row->size; ++i)
      for (Index j = 0; j < b.col->size; ++j) {
        const Index pi = idx[b.row->begin + i], pj = P->ct.indices[b.col->begin + j];
        Scalar cij = 0;
        for (int r = 0; r < R; ++r) cij += y[(size_t)r * n + pi] * x[(size_t)r * n + pj];
        const Scalar g = kernel_grad_over_r(ktype, l, dist(X + (size_t)pi * dim,
                                                              X + (size_t)pj * dim, dim));
        for (int d = 0; d < dim; ++d) {
          const Scalar diff = X[(size_t)pi * dim + d] - X[(size_t)pj * dim + d];
          G[(size_t)pi * dim + d] += cij * g * diff;
          G[(size_t)pj * dim + d] -= cij * g * diff;
        }
      }
  }
  // far field: gradients of the leaf bases against the leaf expansions
  std::vector<Scalar> f((size_t)dim * (P->ip.deg + 1)), df(f.size());
  const int p1 = (int)P->ip.deg + 1;
  for (Node* nd : P->rt.by_id) {
    if (nd->sons.size()) continue;
    const Mat& ux = Ux[nd->block_id];
    const Mat& uy = Uy[nd->block_id];
    for (Index i = 0; i < nd->size; ++i) {
      const Index pi = idx[nd->begin + i];
      for (int d = 0; d < dim; ++d)
        lagrange_product(P->ip.xi, (X[(size_t)pi * dim + d] - nd->bmin[d]) / nd->bext[d],
                         &f[(size_t)d * p1], &df[(size_t)d * p1]);
      for (int k = 0; k < q; ++k) {
        Scalar hx = 0, hy = 0;
        for (int r = 0; r < R; ++r) {
          hx += ux(k, r) * y[(size_t)r * n + pi];
          hy += uy(k, r) * x[(size_t)r * n + pi];
        }
        for (int d = 0; d < dim; ++d) {
          Scalar gv = df[(size_t)d * p1 + P->ip.idcs[k][d]] / nd->bext[d];
          for (int e = 0; e < dim; ++e)
            if (e != d) gv *= f[(size_t)e * p1 + P->ip.idcs[k][e]];
          G[(size_t)pi * dim + d] += (hx + hy) * gv;
        }
      }
    }
  }
  for (size_t e = 0; e < G.size(); ++e) dX[e] = sigma2 * G[e];
}

// moves the points of a one-cloud plan (dim x n, natural order) keeping the
// tree, boxes, transfer matrices and blocks; the leaf bases are recomputed
void oracle_update_points(void* h, const double* Pnew) {
  OPlan* P = static_cast<OPlan*>(h);
  std::copy(Pnew, Pnew + P->Pr.size(), P->Pr.begin());
  std::copy(Pnew, Pnew + P->Pc.size(), P->Pc.begin());
  for (Tree* t : {&P->rt, &P->ct})
    for (Node* nd : t->by_id)
      if (!nd->sons.size()) nd->V = t->moments(*nd, P->ip);
}

// y = sigma2 * K(Pr, Pc) x  (dense FP64, CovarianceKernel::eval times x)
void oracle_dense_matvec(int ktype, double l, double c, double sigma2, int dim,
                         const double* Pr, int64_t nr, const double* Pc, int64_t nc,
                         const double* x, int R, double* y, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const KernelFn kern = make_kernel(ktype, l, c);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nr; ++i) {
    std::vector<double> acc(R, 0.);
    for (int64_t j = 0; j < nc; ++j) {
      const double k = kern(dist(Pr + i * dim, Pc + j * dim, (Index)dim));
      for (int r = 0; r < R; ++r) acc[r] += k * x[(size_t)r * nc + j];
    }
    for (int r = 0; r < R; ++r) y[(size_t)r * nr + i] = sigma2 * acc[r];
  }
}

double oracle_kernel(int ktype, double l, double c, double r) {
  return make_kernel(ktype, l, c)(r);
}

}  // extern "C"
