// Host-side H2 plan for the matrix-free H2 kernel matvec.
//
// The plan holds everything that depends only on the point clouds, the
// interpolation degree and the admissibility parameter:
//   * two cluster trees (rows, columns) built exactly like FMCA's
//     ClusterTree with CardinalityBisection
//     (FMCA/src/Clustering/ClusterTreeInitializer_ClusterTree.h:24-132,
//      FMCA/src/Clustering/ClusterTreeSplitter.h:60-81),
//     clusters numbered in level order like FMCA's IDDFS iterator
//     (FMCA/src/util/IDDFSForwardIterator.h:37-63);
//   * the Chebyshev tensor-product interpolation tables
//     (FMCA/src/Interpolator/TensorProductInterpolator.h:39-81,
//      FMCA/src/util/MultiIndexSet.h:87-187);
//   * per-cluster 1-D transfer factors: the tensor-product transfer matrix of
//     FMCA (FMCA/src/H2Matrix/compute_cluster_bases_impl.h:37-50) is the
//     Kronecker product of d small (p+1)x(p+1) factors, which is what the GPU
//     applies;
//   * the admissible (far) and inadmissible (near) block lists of
//     H2MatrixBase::computePattern (FMCA/src/H2Matrix/H2MatrixBase.h:160-191)
//     with CompareCluster (FMCA/src/Clustering/Admissibility.h:19-29,95-115),
//     re-organised as row-owned CSR lists for the GPU.
//
// Every floating-point expression that feeds a discrete decision (bounding
// boxes, split dimension, admissibility) is evaluated in the same operation
// order as the reference, and this file must be compiled with
// -ffp-contract=off so that no multiply-add is fused.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace fmca {

// Radial kernels of FMCA's CovarianceKernel (FMCA/src/CovarianceKernel/
// CovarianceKernel.h:56-116).  The numeric codes are part of the C ABI.
enum KernelType : int {
  K_EXPONENTIAL = 0,
  K_MATERN32 = 1,
  K_MATERN52 = 2,
  K_GAUSSIAN = 3,
  K_MATERN72 = 4,
  K_MATERN92 = 5,
  K_INVMULTIQUADRIC = 6,
  K_MULTIQUADRIC = 7,
  K_BIHARMONIC3D = 8,
  K_TRIHARMONIC3D = 9,
  // derivatives dk/dl of the four covariance kernels with respect to the
  // length scale (the far field of H2[dk/dl] is dS/dl at the fixed nodes)
  K_DL_EXPONENTIAL = 10,
  K_DL_MATERN32 = 11,
  K_DL_MATERN52 = 12,
  K_DL_GAUSSIAN = 13,
  // the thin-plate kernels of CovarianceKernel.h:56-59 and 117-118
  K_BIHARMONIC2D = 14,
  K_TPS2D = 15,
  K_NUM_KERNELS = 16
};

// true for the length-scale derivative kernels K_DL_*
inline bool is_dl_kernel(int type) { return type >= K_DL_EXPONENTIAL && type <= K_DL_GAUSSIAN; }

// Parses an FMCA kernel name (case-insensitive, like CovarianceKernel.h:54).
// Returns -1 for names that are not supported.
int kernel_type_from_name(const std::string& name);
const char* kernel_type_name(int type);
// Scalar FP64 evaluation of the radial function k(r) with the reference's
// expression order; used by the host (statistics, tests) only.
double kernel_eval_host(int type, double l, double c, double r);

// Interpolator on [0,1]^d: the Chebyshev tensor-product interpolator
// (kind 0, TensorProductInterpolator.h) or the total-degree interpolator
// (kind 1, TotalDegreeInterpolator.h: DeMarchi nodes, L2-normalised Legendre
// polynomials, dense inverse Vandermonde matrix).
enum { kInterpTensor = 0, kInterpTotalDegree = 1 };
struct Interp {
  int kind = kInterpTensor;
  int dim = 0;
  int deg = 0;
  int q = 0;                 // (deg+1)^dim, or binom(deg+dim, dim)
  std::vector<double> xi;    // tensor: deg+1 univariate nodes
  std::vector<double> w;     // tensor: deg+1 barycentric weights
  std::vector<int> midx;     // q x dim multi-indices, graded-lex order
  std::vector<double> Xi;    // dim x q node coordinates (column-major)
  std::vector<double> invV;  // total degree: q x q inverse of V (row-major),
                             // V(i, k) = polynomial k at node i
  void init(int dim, int deg, int kind = kInterpTensor);
  // 1-D Lagrange factors f[a] = l_a(x), a = 0..deg, with the reference's
  // coincident-node guard (TensorProductInterpolator.h:70-79).
  void lagrange1d(double x, double* f) const;
  // 1-D L2-normalised Legendre polynomials on [0,1], f[a], a = 0..deg
  // (evalPolynomials.h:19-38)
  void legendre1d(double x, double* f) const;
  // total degree: the q polynomial values at u (evalPolynomials.h:50-63)
  void poly(const double* u, double* out) const;
};

// The splits of one tree level done elsewhere (the GPU level sorter of
// h2_tree_gpu.cu): every segment is the index range of one cluster that
// splits, sorted by one coordinate.
struct SortSegment {
  uint32_t begin, size;
  int coord;
};
class LevelSorter {
 public:
  virtual ~LevelSorter() {}
  // Uploads the points (dim x n, natural order) and the identity
  // permutation; false on failure.
  virtual bool start(const double* P, int dim, uint32_t n) = 0;
  // Sorts every segment's range of the permutation by its coordinate
  // (ascending) and returns per segment the coordinates at offsets
  // size / 2 - 1 and size / 2 of the sorted range (split[2 s], split[2 s +
  // 1]). *ties: some segment holds equal coordinates (whose order the
  // reference's std::sort decides); the result is then not used.  false on
  // failure.
  virtual bool sort_level(const std::vector<SortSegment>& segs, std::vector<double>* split,
                          bool* ties) = 0;
  // Copies the permutation back; false on failure.
  virtual bool finish(std::vector<uint32_t>* perm) = 0;
};

class Tree;
// The leaves of the block tree of H2MatrixBase::computePattern
// (H2MatrixBase.h:160-191) built elsewhere (the GPU pattern builder of
// h2_tree_gpu.cu): far (low-rank) and near (dense) (row, column) cluster
// pairs in the order of the reference's depth-first recursion.  false: not
// built; the host recursion runs instead.
class PatternBuilder {
 public:
  virtual ~PatternBuilder() {}
  virtual bool build(const Tree& rows, const Tree& cols, uint32_t qq, double eta,
                     std::vector<int32_t>* far_row, std::vector<int32_t>* far_col,
                     std::vector<int32_t>* near_row, std::vector<int32_t>* near_col) = 0;
};

// Cluster tree in level order.  Cluster c owns cluster-ordered points
// [begin[c], begin[c] + size[c]); perm maps cluster order to natural order
// (ClusterTreeBase::indices()).
class Tree {
 public:
  int dim = 0;
  uint32_t n = 0;
  std::vector<uint32_t> perm;
  std::vector<uint32_t> begin, size;
  std::vector<int32_t> level, parent, son0, nsons;
  std::vector<double> bbmin, bbmax, bbext;  // C x dim, row-major per cluster
  std::vector<int32_t> level_ptr;           // clusters of level l
  int nclusters() const { return (int)begin.size(); }
  int nlevels() const { return (int)level_ptr.size() - 1; }
  // Builds the tree: min_csize is the effective minimum leaf size
  // (H2ClusterTree.h:68-70 passes max(min_cluster_size, q)). The clusters of
  // one level split on up to `threads` host threads (0: one per core, at
  // most 16); the result does not depend on the thread count.
  void build(const double* P, int dim, uint32_t n, uint32_t min_csize, int threads = 0);
  // The same tree with every level's sorts done by `sorter` (one call per
  // level). Returns false, leaving the tree empty, when a sorted range held
  // equal coordinates or the sorter failed: the caller then builds on the
  // host, where std::sort orders equal keys as the reference does.
  bool build_with(LevelSorter* sorter, const double* P, int dim, uint32_t n, uint32_t min_csize);
};

// Row-owned block lists.
struct Pattern {
  // raw block lists as produced by the pattern recursion (row, col ids)
  std::vector<int32_t> far_row, far_col;    // low-rank leaves
  std::vector<int32_t> near_row, near_col;  // dense leaves
  // far field: CSR over row clusters; each entry a column cluster, ascending
  std::vector<int32_t> far_ptr, far_idx;
  // near field: CSR over row leaves (leaf index into Plan::row_leaves);
  // entries are merged half-open intervals of column points (cluster order)
  std::vector<int32_t> near_ptr;
  std::vector<uint32_t> near_ivl;  // pairs (begin, end)
  uint64_t near_pairs = 0;         // sum |tau| |sigma| over dense leaves
};

struct Plan {
  Interp interp;
  Tree rows, cols;
  std::vector<double> points_r, points_c;  // dim x n, natural order
  bool same_tree = false;  // rows and cols built from the same cloud
  double eta = 0.8;
  Pattern pat;
  std::vector<int32_t> row_leaves, col_leaves;  // cluster ids of leaves
  // tensor: per-cluster transfer factors e[c][dd][a][b] (dim x (p+1) x
  // (p+1)): E_c (son c -> its father) = kron over dd of e[c][dd];
  // total degree: dense E_c[k][j] (q x q per cluster, polynomial basis)
  std::vector<double> row_E, col_E;
  // interpolation node coordinates per cluster: C x q x dim
  std::vector<double> row_nodes, col_nodes;

  void build(const double* Pr, uint32_t nr, const double* Pc, uint32_t nc,
             int dim, int deg, double eta, uint32_t min_leaf, bool same,
             int interp_kind = kInterpTensor, LevelSorter* sorter = nullptr,
             PatternBuilder* pattern_builder = nullptr);
  // trees whose sorts ran on the sorter (0, 1 or 2); the others were built
  // on the host
  int trees_sorted_elsewhere = 0;
  // 1 if the pattern builder built the block lists, 0 if the host did
  int pattern_built_elsewhere = 0;
  int build_threads = 0;  // host threads of the tree builds (0: one per core)
  // Block-diagonal plan of independent point clouds: trees, bases and block
  // lists of the parts concatenated (cluster ids, point indices and node
  // indices offset), so one launch per stage covers every cloud.  The parts
  // must share dim and degree.  cloud_offsets receives the first point of
  // every part (count + 1 entries).
  void merge(const std::vector<const Plan*>& parts);
  std::vector<int64_t> cloud_offsets;
  // (m, n, #low-rank blocks, #dense blocks, nz per row, GB)
  // exactly like H2MatrixBase::statistics (H2MatrixBase.h:70-105)
  void statistics(double out[6]) const;
};

// Recomputes the transfer factors of one tree for an interpolator.
void compute_transfer_factors(const Tree& t, const Interp& ip,
                              std::vector<double>* E);
void compute_node_coords(const Tree& t, const Interp& ip,
                         std::vector<double>* nodes);

}  // namespace fmca
