// Plan files: a built plan (trees, permutations, block lists, interpolation
// data) written as a sequence of matrices in the binary layout of FMCA's
// print2bin / bin2Mat (FMCA/src/util/IO.h:532-626): per matrix the element
// size, a row-major flag (always 0), rows and cols as size_t, then the
// column-major data. The first matrix is an int64 header, the second the
// admissibility parameter eta; the interpolator is rebuilt from the header
// (its nodes, weights and inverse Vandermonde matrix are deterministic).
#include "plan_io.h"

#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace fmca {
namespace {

constexpr int64_t kMagic = 0x464d4341;  // "FMCA"
constexpr int64_t kVersion = 1;
constexpr int kHeader = 16;

template <typename T>
void put(std::ofstream& f, const T* data, size_t rows, size_t cols) {
  const size_t head[4] = {sizeof(T), 0, rows, cols};
  f.write(reinterpret_cast<const char*>(head), sizeof(head));
  if (rows * cols) f.write(reinterpret_cast<const char*>(data), rows * cols * sizeof(T));
}

template <typename T>
void put(std::ofstream& f, const std::vector<T>& v) {
  put(f, v.data(), v.size(), 1);
}

template <typename T>
void get(std::ifstream& f, std::vector<T>* v, const char* what) {
  size_t head[4];
  if (!f.read(reinterpret_cast<char*>(head), sizeof(head)))
    throw std::runtime_error(std::string("plan file ends before ") + what);
  if (head[0] != sizeof(T) || head[1] != 0)
    throw std::runtime_error(std::string("plan file: unexpected layout of ") + what);
  const size_t n = head[2] * head[3];
  if (n > ((size_t)1 << 40) / sizeof(T))
    throw std::runtime_error(std::string("plan file: implausible size of ") + what);
  v->resize(n);
  if (n && !f.read(reinterpret_cast<char*>(v->data()), n * sizeof(T)))
    throw std::runtime_error(std::string("plan file ends inside ") + what);
}

void put_tree(std::ofstream& f, const Tree& t) {
  put(f, t.perm);
  put(f, t.begin);
  put(f, t.size);
  put(f, t.level);
  put(f, t.parent);
  put(f, t.son0);
  put(f, t.nsons);
  put(f, t.bbmin);
  put(f, t.bbmax);
  put(f, t.bbext);
  put(f, t.level_ptr);
}

void get_tree(std::ifstream& f, Tree* t, int dim, int64_t n, int64_t C) {
  t->dim = dim;
  t->n = (uint32_t)n;
  get(f, &t->perm, "perm");
  get(f, &t->begin, "begin");
  get(f, &t->size, "size");
  get(f, &t->level, "level");
  get(f, &t->parent, "parent");
  get(f, &t->son0, "son0");
  get(f, &t->nsons, "nsons");
  get(f, &t->bbmin, "bbmin");
  get(f, &t->bbmax, "bbmax");
  get(f, &t->bbext, "bbext");
  get(f, &t->level_ptr, "level_ptr");
  const size_t c = (size_t)C;
  if (t->perm.size() != (size_t)n || t->begin.size() != c || t->size.size() != c ||
      t->level.size() != c || t->parent.size() != c || t->son0.size() != c ||
      t->nsons.size() != c || t->bbmin.size() != c * dim || t->bbmax.size() != c * dim ||
      t->bbext.size() != c * dim || t->level_ptr.empty())
    throw std::runtime_error("plan file: inconsistent cluster tree");
  std::vector<unsigned char> seen((size_t)n, 0);
  for (uint32_t p : t->perm) {
    if (p >= (uint32_t)n) throw std::runtime_error("plan file: permutation out of range");
    if (seen[p]++) throw std::runtime_error("plan file: permutation repeats an index");
  }
  for (size_t i = 0; i < c; ++i)
    if ((uint64_t)t->begin[i] + t->size[i] > (uint64_t)n)
      throw std::runtime_error("plan file: cluster range out of range");
  // level_ptr: nlevels + 1 non-decreasing offsets from 0 to C (a forest of
  // several clouds keeps only the number of levels: every entry 0)
  const int64_t L = (int64_t)t->level_ptr.size() - 1;
  if (L < 1 || t->level_ptr[0] != 0)
    throw std::runtime_error("plan file: bad level offsets");
  bool all_zero = true;
  for (int64_t l = 0; l < L; ++l) {
    if (t->level_ptr[l + 1] < t->level_ptr[l])
      throw std::runtime_error("plan file: level offsets not monotone");
    all_zero = all_zero && t->level_ptr[l + 1] == 0;
  }
  if (!all_zero && t->level_ptr[L] != (int32_t)C)
    throw std::runtime_error("plan file: level offsets do not end at the cluster count");
  // tree links: levels in range, parents before their sons, every son's
  // parent and level consistent with its father
  for (size_t i = 0; i < c; ++i) {
    const int32_t lv = t->level[i], pa = t->parent[i], s0 = t->son0[i], ns = t->nsons[i];
    if (lv < 0 || lv >= L) throw std::runtime_error("plan file: cluster level out of range");
    if (pa < -1 || pa >= (int64_t)C || pa == (int32_t)i)
      throw std::runtime_error("plan file: parent out of range");
    if (ns < 0) throw std::runtime_error("plan file: negative son count");
    if (ns > 0) {
      if (s0 <= (int32_t)i || (int64_t)s0 + ns > C)
        throw std::runtime_error("plan file: sons out of range");
      for (int32_t s = s0; s < s0 + ns; ++s)
        if (t->parent[s] != (int32_t)i || t->level[s] != lv + 1)
          throw std::runtime_error("plan file: inconsistent parent links");
    }
  }
}

// offsets of a CSR list: first 0, non-decreasing
bool csr_ok(const std::vector<int32_t>& ptr) {
  if (ptr.empty() || ptr[0] != 0) return false;
  for (size_t i = 1; i < ptr.size(); ++i)
    if (ptr[i] < ptr[i - 1]) return false;
  return true;
}

}  // namespace

void save_plan(const Plan& P, int64_t min_leaf, const std::string& path) {
  std::ofstream f(path, std::ios::out | std::ios::binary | std::ios::trunc);
  if (!f) throw std::runtime_error("cannot open " + path + " for writing");
  int64_t h[kHeader] = {kMagic,
                        kVersion,
                        P.interp.dim,
                        P.interp.deg,
                        P.interp.kind,
                        P.same_tree ? 1 : 0,
                        min_leaf,
                        (int64_t)P.rows.n,
                        (int64_t)P.cols.n,
                        P.rows.nclusters(),
                        P.cols.nclusters(),
                        (int64_t)P.pat.near_pairs,
                        0,
                        0,
                        0,
                        0};
  put(f, h, kHeader, 1);
  put(f, &P.eta, 1, 1);
  put(f, P.points_r.data(), (size_t)P.interp.dim, P.points_r.size() / P.interp.dim);
  put(f, P.points_c.data(), (size_t)P.interp.dim, P.points_c.size() / P.interp.dim);
  put_tree(f, P.rows);
  put_tree(f, P.cols);
  const Pattern& pt = P.pat;
  put(f, pt.far_row);
  put(f, pt.far_col);
  put(f, pt.near_row);
  put(f, pt.near_col);
  put(f, pt.far_ptr);
  put(f, pt.far_idx);
  put(f, pt.near_ptr);
  put(f, pt.near_ivl);
  put(f, P.row_leaves);
  put(f, P.col_leaves);
  put(f, P.row_E);
  put(f, P.col_E);
  put(f, P.row_nodes);
  put(f, P.col_nodes);
  put(f, P.cloud_offsets);
  f.flush();
  if (!f) throw std::runtime_error("write to " + path + " failed");
}

void load_plan(const std::string& path, Plan* P, int64_t* min_leaf) {
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::vector<int64_t> h;
  get(f, &h, "header");
  if (h.size() != (size_t)kHeader || h[0] != kMagic)
    throw std::runtime_error(path + " is not a plan file");
  if (h[1] != kVersion) throw std::runtime_error("unsupported plan file version");
  const int dim = (int)h[2], deg = (int)h[3], kind = (int)h[4];
  if (dim < 1 || dim > 64 || deg < 0 || deg > 16 ||
      (kind != kInterpTensor && kind != kInterpTotalDegree) || h[7] < 1 || h[8] < 1 ||
      h[9] < 1 || h[10] < 1)
    throw std::runtime_error("plan file: bad header");
  *P = Plan();
  P->interp.init(dim, deg, kind);
  P->same_tree = h[5] != 0;
  *min_leaf = h[6];
  std::vector<double> eta;
  get(f, &eta, "eta");
  if (eta.size() != 1) throw std::runtime_error("plan file: bad eta");
  P->eta = eta[0];
  get(f, &P->points_r, "row points");
  get(f, &P->points_c, "column points");
  if (P->points_r.size() != (size_t)dim * h[7] || P->points_c.size() != (size_t)dim * h[8])
    throw std::runtime_error("plan file: inconsistent points");
  get_tree(f, &P->rows, dim, h[7], h[9]);
  get_tree(f, &P->cols, dim, h[8], h[10]);
  Pattern& pt = P->pat;
  get(f, &pt.far_row, "far rows");
  get(f, &pt.far_col, "far cols");
  get(f, &pt.near_row, "near rows");
  get(f, &pt.near_col, "near cols");
  get(f, &pt.far_ptr, "far CSR");
  get(f, &pt.far_idx, "far CSR");
  get(f, &pt.near_ptr, "near CSR");
  get(f, &pt.near_ivl, "near intervals");
  pt.near_pairs = (uint64_t)h[11];
  get(f, &P->row_leaves, "row leaves");
  get(f, &P->col_leaves, "column leaves");
  get(f, &P->row_E, "row transfers");
  get(f, &P->col_E, "column transfers");
  get(f, &P->row_nodes, "row nodes");
  get(f, &P->col_nodes, "column nodes");
  get(f, &P->cloud_offsets, "cloud offsets");
  // the block lists index clusters and leaves of the trees just read
  const int64_t Cr = h[9], Cc = h[10];
  auto in = [](const std::vector<int32_t>& v, int64_t lim) {
    for (int32_t x : v)
      if (x < 0 || x >= lim) return false;
    return true;
  };
  if (pt.far_row.size() != pt.far_col.size() || pt.near_row.size() != pt.near_col.size() ||
      !in(pt.far_row, Cr) || !in(pt.far_col, Cc) || !in(pt.near_row, Cr) ||
      !in(pt.near_col, Cc) || !in(pt.far_idx, Cc) || !in(P->row_leaves, Cr) ||
      !in(P->col_leaves, Cc) || pt.far_ptr.size() != (size_t)Cr + 1 ||
      pt.near_ptr.size() != P->row_leaves.size() + 1 ||
      P->row_nodes.size() != (size_t)Cr * P->interp.q * dim ||
      P->col_nodes.size() != (size_t)Cc * P->interp.q * dim)
    throw std::runtime_error("plan file: inconsistent block lists");
  if (!csr_ok(pt.far_ptr) || !csr_ok(pt.near_ptr) ||
      pt.far_ptr.back() != (int32_t)pt.far_idx.size() ||
      (size_t)pt.near_ptr.back() * 2 != pt.near_ivl.size())
    throw std::runtime_error("plan file: inconsistent CSR lists");
  for (size_t i = 0; i < pt.near_ivl.size(); i += 2)
    if (pt.near_ivl[i] > pt.near_ivl[i + 1] || pt.near_ivl[i + 1] > (uint32_t)h[8])
      throw std::runtime_error("plan file: interval out of range");
  for (int32_t c : P->row_leaves)
    if (P->rows.nsons[c] != 0) throw std::runtime_error("plan file: row leaf with sons");
  for (int32_t c : P->col_leaves)
    if (P->cols.nsons[c] != 0) throw std::runtime_error("plan file: column leaf with sons");
  // transfer data: d Kronecker factors of (p + 1)^2 (tensor) or a dense
  // q x q matrix (total degree) per cluster
  const size_t p1 = (size_t)deg + 1, q = (size_t)P->interp.q;
  const size_t per = kind == kInterpTensor ? (size_t)dim * p1 * p1 : q * q;
  if (P->row_E.size() != (size_t)Cr * per || P->col_E.size() != (size_t)Cc * per)
    throw std::runtime_error("plan file: inconsistent transfer data");
  // cloud offsets: none (one cloud) or count + 1 non-decreasing row offsets
  // from 0 to the row count
  const std::vector<int64_t>& co = P->cloud_offsets;
  if (!co.empty()) {
    bool ok = co.size() >= 2 && co[0] == 0 && co.back() == h[7];
    for (size_t i = 1; ok && i < co.size(); ++i) ok = co[i] >= co[i - 1];
    if (!ok) throw std::runtime_error("plan file: inconsistent cloud offsets");
  }
}

}  // namespace fmca
