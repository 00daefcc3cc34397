// extern "C" boundary of fmca_gb300 (declared in include/fmca_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fmca_gb300.h"
#include "c_api_internal.h"
#include "plan_io.h"
#include "near_pack.h"
#include "h2_gpu.h"
#include "h2_plan.h"

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace fmca {
namespace capi {
fmca_status fail(fmca_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}
}  // namespace capi
}  // namespace fmca

namespace {
using fmca::capi::fail;
fmca_status ok() { return FMCA_OK; }

fmca_status check_kernel(const fmca_kernel_desc* k) {
  if (!k) return fail(FMCA_ERR_INVALID_ARGUMENT, "kernel descriptor is NULL");
  if (k->type < 0 || k->type >= fmca::K_NUM_KERNELS)
    return fail(FMCA_ERR_INVALID_ARGUMENT,
                "unknown kernel type " + std::to_string(k->type));
  if (!(k->l > 0) || !std::isfinite(k->l))
    return fail(FMCA_ERR_INVALID_ARGUMENT, "kernel length scale must be > 0");
  if (!std::isfinite(k->sigma2) || !std::isfinite(k->c))
    return fail(FMCA_ERR_INVALID_ARGUMENT, "kernel parameters must be finite");
  return FMCA_OK;
}

fmca_status check_gpu_plan(const fmca_plan* p, int precision) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  if (precision != FMCA_PREC_FP64 && precision != FMCA_PREC_MIXED &&
      precision != FMCA_PREC_FP32)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "unknown precision mode");
  if (p->plan.interp.dim > 3)
    return fail(FMCA_ERR_UNSUPPORTED, "the GPU path supports dim <= 3");
  if (p->plan.interp.kind == fmca::kInterpTensor && p->plan.interp.deg > 7)
    return fail(FMCA_ERR_UNSUPPORTED, "the GPU path supports tensor-product degree <= 7");
  if (p->plan.interp.kind == fmca::kInterpTotalDegree &&
      (p->plan.interp.deg > 15 || p->plan.interp.q > 120))
    return fail(FMCA_ERR_UNSUPPORTED,
                "the GPU path supports total degree <= 15 with at most 120 nodes");
  return FMCA_OK;
}
}  // namespace

namespace fmca {
namespace capi {
gpu::KernelDesc to_desc(const fmca_kernel_desc* k) {
  gpu::KernelDesc d;
  d.type = k->type;
  d.l = k->l;
  d.c = k->c;
  d.nu = k->nu;
  d.sigma2 = k->sigma2;
  return d;
}

gpu::CallOpts call_opts(const fmca_plan* p) {
  gpu::CallOpts o;
  o.profile = p->profile.load();
  o.wait_ns = p->wait_ns.load();
  o.stall = p->stall.load();
  o.autotune = p->autotune.load();
  return o;
}

fmca_status check_matvec_args(const fmca_plan* p, const fmca_kernel_desc* kernel,
                              int precision, int dtype, int order, int nrhs,
                              const void* x, const void* y) {
  fmca_status s = check_gpu_plan(p, precision);
  if (s != FMCA_OK) return s;
  s = check_kernel(kernel);
  if (s != FMCA_OK) return s;
  if (dtype != FMCA_DTYPE_F64 && dtype != FMCA_DTYPE_F32)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "unknown dtype");
  if (order != FMCA_ORDER_NATURAL && order != FMCA_ORDER_CLUSTER)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "unknown order");
  if (nrhs < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "nrhs must be >= 1");
  if (!x || !y) return fail(FMCA_ERR_INVALID_ARGUMENT, "x or y is NULL");
  return FMCA_OK;
}
}  // namespace capi
}  // namespace fmca

namespace {
using fmca::capi::to_desc;
}  // namespace

extern "C" {

const char* fmca_last_error(void) { return g_last_error.c_str(); }
const char* fmca_version(void) { return "fmca_gb300 0.1.0"; }

fmca_status fmca_kernel_type_from_name(const char* name, int* type) {
  if (!name || !type) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  const int t = fmca::kernel_type_from_name(name);
  if (t < 0)
    return fail(FMCA_ERR_UNSUPPORTED, std::string("kernel not implemented: ") + name);
  *type = t;
  return ok();
}

fmca_status fmca_plan_create(const double* P_rows, int dim, int64_t n_rows,
                             const double* P_cols, int64_t n_cols, int degree,
                             double eta, int64_t min_leaf, fmca_plan** out) {
  return fmca_plan_create_ex(P_rows, dim, n_rows, P_cols, n_cols,
                             FMCA_INTERP_TENSOR_PRODUCT, degree, eta, min_leaf, out);
}

namespace {
// fmca_plan_create_ex, with the trees' level sorts on `sorter` if given
fmca_status create_plan(const double* P_rows, int dim, int64_t n_rows, const double* P_cols,
                        int64_t n_cols, int interpolator, int degree, double eta,
                        int64_t min_leaf, fmca::LevelSorter* sorter,
                        fmca::PatternBuilder* pattern_builder, int* sorted_elsewhere,
                        int* pattern_elsewhere, fmca_plan** out) {
  if (!out) return fail(FMCA_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!P_rows) return fail(FMCA_ERR_INVALID_ARGUMENT, "P_rows is NULL");
  if (dim < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "dim must be >= 1");
  if (n_rows < 1 || n_rows > (int64_t)0xFFFFFFFEll)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "n_rows out of range");
  const bool same = (P_cols == nullptr || P_cols == P_rows);
  if (same) n_cols = n_rows;
  if (n_cols < 1 || n_cols > (int64_t)0xFFFFFFFEll)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "n_cols out of range");
  if (degree < 0 || degree > 16)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "degree out of range");
  if (interpolator != FMCA_INTERP_TENSOR_PRODUCT && interpolator != FMCA_INTERP_TOTAL_DEGREE)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "unknown interpolator");
  // the total-degree nodes come from Halton sequences in the first three
  // prime bases; the GPU passes take at most 16 polynomial factors per
  // dimension and dense transfer matrices of at most 120 x 120
  if (interpolator == FMCA_INTERP_TOTAL_DEGREE) {
    int64_t q = 1;
    for (int i = 1; i <= dim && dim <= 3; ++i) q = q * (degree + i) / i;  // binom(degree + dim, dim)
    if (dim > 3 || degree > 15 || q > 120)
      return fail(FMCA_ERR_UNSUPPORTED,
                  "total-degree interpolation needs dim <= 3, degree <= 15 and at most 120 "
                  "nodes (degree <= 7 in 3-D, <= 14 in 2-D)");
  }
  if (!(eta >= 0) || !std::isfinite(eta))
    return fail(FMCA_ERR_INVALID_ARGUMENT, "eta must be finite and >= 0");
  if (min_leaf < 0 || min_leaf > (int64_t)0x7FFFFFFF)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "min_leaf out of range");
  for (int64_t i = 0; i < (int64_t)dim * n_rows; ++i)
    if (!std::isfinite(P_rows[i]))
      return fail(FMCA_ERR_INVALID_ARGUMENT, "P_rows holds a non-finite value");
  if (!same)
    for (int64_t i = 0; i < (int64_t)dim * n_cols; ++i)
      if (!std::isfinite(P_cols[i]))
        return fail(FMCA_ERR_INVALID_ARGUMENT, "P_cols holds a non-finite value");
  try {
    fmca_plan* p = new fmca_plan();
    p->min_leaf = min_leaf;
    p->plan.build(P_rows, (uint32_t)n_rows, same ? P_rows : P_cols,
                  (uint32_t)n_cols, dim, degree, eta, (uint32_t)min_leaf, same,
                  interpolator == FMCA_INTERP_TOTAL_DEGREE ? fmca::kInterpTotalDegree
                                                           : fmca::kInterpTensor,
                  sorter, pattern_builder);
    if (sorted_elsewhere) *sorted_elsewhere = p->plan.trees_sorted_elsewhere;
    if (pattern_elsewhere) *pattern_elsewhere = p->plan.pattern_built_elsewhere;
    *out = p;
  } catch (const std::bad_alloc&) {
    return fail(FMCA_ERR_OUT_OF_MEMORY, "host allocation failed while building the plan");
  } catch (const std::exception& e) {
    return fail(FMCA_ERR_INTERNAL, e.what());
  }
  return ok();
}
}  // namespace

fmca_status fmca_plan_create_ex(const double* P_rows, int dim, int64_t n_rows,
                                const double* P_cols, int64_t n_cols, int interpolator,
                                int degree, double eta, int64_t min_leaf, fmca_plan** out) {
  return create_plan(P_rows, dim, n_rows, P_cols, n_cols, interpolator, degree, eta, min_leaf,
                     nullptr, nullptr, nullptr, nullptr, out);
}

fmca_status fmca_plan_create_gpu(const double* P_rows, int dim, int64_t n_rows,
                                 const double* P_cols, int64_t n_cols, int interpolator,
                                 int degree, double eta, int64_t min_leaf, int* gpu_parts,
                                 fmca_plan** out) {
  if (gpu_parts) gpu_parts[0] = gpu_parts[1] = 0;
  std::unique_ptr<fmca::LevelSorter> sorter = fmca::gpu::make_gpu_level_sorter();
  std::unique_ptr<fmca::PatternBuilder> pb = fmca::gpu::make_gpu_pattern_builder();
  int trees = 0, pattern = 0;
  const fmca_status s = create_plan(P_rows, dim, n_rows, P_cols, n_cols, interpolator, degree,
                                    eta, min_leaf, sorter.get(), pb.get(), &trees, &pattern, out);
  if (gpu_parts) {
    gpu_parts[0] = trees;
    gpu_parts[1] = pattern;
  }
  return s;
}

fmca_status fmca_plan_create_batched(const double* const* P, const int64_t* n_points,
                                     int count, int dim, int degree, double eta,
                                     int64_t min_leaf, fmca_plan** out) {
  if (!out) return fail(FMCA_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!P || !n_points || count < 1)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "need at least one point cloud");
  if (dim < 1 || degree < 0 || degree > 16 || !(eta >= 0) || !std::isfinite(eta) ||
      min_leaf < 0 || min_leaf > (int64_t)0x7FFFFFFF)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "bad dim, degree, eta or min_leaf");
  int64_t total = 0;
  for (int i = 0; i < count; ++i) {
    if (!P[i] || n_points[i] < 1)
      return fail(FMCA_ERR_INVALID_ARGUMENT, "empty point cloud " + std::to_string(i));
    total += n_points[i];
    for (int64_t e = 0; e < (int64_t)dim * n_points[i]; ++e)
      if (!std::isfinite(P[i][e]))
        return fail(FMCA_ERR_INVALID_ARGUMENT,
                    "point cloud " + std::to_string(i) + " holds a non-finite value");
  }
  if (total > (int64_t)0xFFFFFFFEll)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "too many points in total");
  try {
    std::vector<fmca::Plan> parts(count);
    std::atomic<int> next(0);
    const int nth = std::max(1, std::min<int>(count, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    // the cores not taken by whole clouds go to each cloud's tree build
    const int per = std::max(1, (int)std::thread::hardware_concurrency() / nth);
    std::vector<std::exception_ptr> errs(nth);
    for (int t = 0; t < nth; ++t)
      pool.emplace_back([&, t]() {
        try {
          for (int i = next++; i < count; i = next++) {
            parts[i].build_threads = per;
            parts[i].build(P[i], (uint32_t)n_points[i], P[i], (uint32_t)n_points[i], dim,
                           degree, eta, (uint32_t)min_leaf, true);
          }
        } catch (...) {
          errs[t] = std::current_exception();
          next = count;
        }
      });
    for (auto& th : pool) th.join();
    for (auto& e : errs)
      if (e) std::rethrow_exception(e);
    std::vector<const fmca::Plan*> ptrs;
    for (auto& p : parts) ptrs.push_back(&p);
    fmca_plan* p = new fmca_plan();
    p->min_leaf = min_leaf;
    p->plan.merge(ptrs);
    *out = p;
  } catch (const std::bad_alloc&) {
    return fail(FMCA_ERR_OUT_OF_MEMORY, "host allocation failed while building the plan");
  } catch (const std::exception& e) {
    return fail(FMCA_ERR_INTERNAL, e.what());
  }
  return ok();
}

fmca_status fmca_plan_destroy(fmca_plan* plan) {
  if (!plan) return ok();
  fmca::gpu::destroy(plan->dev);
  if (plan->hx) cudaFree(plan->hx);
  if (plan->hy) cudaFree(plan->hy);
  delete plan;
  return ok();
}

fmca_status fmca_plan_cloud_offsets(const fmca_plan* p, int64_t* offsets, int* count) {
  if (!p || !count) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  const std::vector<int64_t>& co = p->plan.cloud_offsets;
  if (co.size() >= 2) {
    *count = (int)co.size() - 1;
    if (offsets) std::copy(co.begin(), co.end(), offsets);
  } else {
    *count = 1;
    if (offsets) {
      offsets[0] = 0;
      offsets[1] = (int64_t)p->plan.rows.n;
    }
  }
  return ok();
}

fmca_status fmca_plan_save(const fmca_plan* p, const char* path) {
  if (!p || !path) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  try {
    fmca::save_plan(p->plan, p->min_leaf, path);
  } catch (const std::bad_alloc&) {
    return fail(FMCA_ERR_OUT_OF_MEMORY, "host allocation failed while saving the plan");
  } catch (const std::exception& e) {
    return fail(FMCA_ERR_INVALID_ARGUMENT, e.what());
  }
  return ok();
}

fmca_status fmca_plan_load(const char* path, fmca_plan** out) {
  if (!out) return fail(FMCA_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!path) return fail(FMCA_ERR_INVALID_ARGUMENT, "path is NULL");
  fmca_plan* p = new (std::nothrow) fmca_plan();
  if (!p) return fail(FMCA_ERR_OUT_OF_MEMORY, "host allocation failed");
  try {
    fmca::load_plan(path, &p->plan, &p->min_leaf);
  } catch (const std::bad_alloc&) {
    delete p;
    return fail(FMCA_ERR_OUT_OF_MEMORY, "host allocation failed while loading the plan");
  } catch (const std::exception& e) {
    delete p;
    return fail(FMCA_ERR_INVALID_ARGUMENT, e.what());
  }
  *out = p;
  return ok();
}

fmca_status fmca_plan_interpolator(const fmca_plan* p, double* nodes, double* invV) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  const fmca::Interp& ip = p->plan.interp;
  if (nodes) std::copy(ip.Xi.begin(), ip.Xi.end(), nodes);
  if (invV && ip.kind == fmca::kInterpTotalDegree)
    for (int i = 0; i < ip.q; ++i)
      for (int j = 0; j < ip.q; ++j) invV[(size_t)j * ip.q + i] = ip.invV[(size_t)i * ip.q + j];
  return ok();
}

fmca_status fmca_plan_info(const fmca_plan* p, int64_t out[FMCA_INFO_COUNT]) {
  if (!p || !out) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  for (int i = 0; i < FMCA_INFO_COUNT; ++i) out[i] = 0;
  const fmca::Plan& P = p->plan;
  out[FMCA_INFO_N_ROWS] = P.rows.n;
  out[FMCA_INFO_N_COLS] = P.cols.n;
  out[FMCA_INFO_DIM] = P.interp.dim;
  out[FMCA_INFO_DEGREE] = P.interp.deg;
  out[FMCA_INFO_Q] = P.interp.q;
  out[FMCA_INFO_INTERPOLATOR] = P.interp.kind == fmca::kInterpTotalDegree
                                    ? FMCA_INTERP_TOTAL_DEGREE
                                    : FMCA_INTERP_TENSOR_PRODUCT;
  out[FMCA_INFO_ROW_CLUSTERS] = P.rows.nclusters();
  out[FMCA_INFO_COL_CLUSTERS] = P.cols.nclusters();
  out[FMCA_INFO_FAR_BLOCKS] = (int64_t)P.pat.far_row.size();
  out[FMCA_INFO_NEAR_BLOCKS] = (int64_t)P.pat.near_row.size();
  out[FMCA_INFO_NEAR_PAIRS] = (int64_t)P.pat.near_pairs;
  out[FMCA_INFO_ROW_LEVELS] = P.rows.nlevels();
  out[FMCA_INFO_COL_LEVELS] = P.cols.nlevels();
  out[FMCA_INFO_ROW_LEAVES] = (int64_t)P.row_leaves.size();
  out[FMCA_INFO_COL_LEAVES] = (int64_t)P.col_leaves.size();
  out[FMCA_INFO_MIN_LEAF] =
      p->min_leaf > P.interp.q ? p->min_leaf : (int64_t)P.interp.q;
  return ok();
}

fmca_status fmca_plan_statistics(const fmca_plan* p, double out[6]) {
  if (!p || !out) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  p->plan.statistics(out);
  return ok();
}

fmca_status fmca_plan_permutation(const fmca_plan* p, int side, uint32_t* perm) {
  if (!p || !perm) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (side != 0 && side != 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "side must be 0 or 1");
  const fmca::Tree& t = side == 0 ? p->plan.rows : p->plan.cols;
  std::memcpy(perm, t.perm.data(), sizeof(uint32_t) * t.n);
  return ok();
}

fmca_status fmca_plan_clusters(const fmca_plan* p, int side, int32_t* meta,
                               double* bb) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  if (side != 0 && side != 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "side must be 0 or 1");
  const fmca::Tree& t = side == 0 ? p->plan.rows : p->plan.cols;
  const int C = t.nclusters(), dim = t.dim;
  for (int c = 0; c < C; ++c) {
    if (meta) {
      meta[4 * c + 0] = (int32_t)t.begin[c];
      meta[4 * c + 1] = (int32_t)t.size[c];
      meta[4 * c + 2] = t.level[c];
      meta[4 * c + 3] = t.parent[c];
    }
    if (bb)
      for (int d = 0; d < dim; ++d) {
        bb[(size_t)c * 3 * dim + d] = t.bbmin[(size_t)c * dim + d];
        bb[(size_t)c * 3 * dim + dim + d] = t.bbmax[(size_t)c * dim + d];
        bb[(size_t)c * 3 * dim + 2 * dim + d] = t.bbext[(size_t)c * dim + d];
      }
  }
  return ok();
}

fmca_status fmca_plan_blocks(const fmca_plan* p, int kind, int32_t* rows,
                             int32_t* cols) {
  if (!p || !rows || !cols) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (kind != 0 && kind != 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "kind must be 0 or 1");
  const auto& r = kind == 0 ? p->plan.pat.far_row : p->plan.pat.near_row;
  const auto& c = kind == 0 ? p->plan.pat.far_col : p->plan.pat.near_col;
  std::memcpy(rows, r.data(), sizeof(int32_t) * r.size());
  std::memcpy(cols, c.data(), sizeof(int32_t) * c.size());
  return ok();
}

fmca_status fmca_plan_near_packed(const fmca_plan* p, int64_t* ngroups, int64_t* nintervals,
                                  uint32_t* groups, uint32_t* intervals) {
  if (!p || !ngroups || !nintervals) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  try {
    fmca::PackedNear pk;
    fmca::build_near_packed(p->plan, 128, &pk);
    const int64_t ng = (int64_t)pk.ngroups(), ni = (int64_t)pk.imask.size();
    if (groups && intervals) {
      if (*ngroups < ng || *nintervals < ni)
        return fail(FMCA_ERR_INVALID_ARGUMENT, "arrays smaller than the counts");
      for (int64_t g = 0; g < ng; ++g) {
        groups[5 * g + 0] = pk.tbegin[g];
        groups[5 * g + 1] = pk.tcount[g];
        groups[5 * g + 2] = (uint32_t)pk.ivl_begin[g];
        groups[5 * g + 3] = (uint32_t)pk.ivl_end[g];
        groups[5 * g + 4] = pk.split[g];
      }
      for (int64_t i = 0; i < ni; ++i) {
        intervals[3 * i + 0] = pk.ivl[2 * i];
        intervals[3 * i + 1] = pk.ivl[2 * i + 1];
        intervals[3 * i + 2] = pk.imask[i];
      }
    }
    *ngroups = ng;
    *nintervals = ni;
  } catch (const std::exception& e) {
    return fail(FMCA_ERR_INTERNAL, e.what());
  }
  return ok();
}

fmca_status fmca_matvec_workspace_size(const fmca_plan* p, int precision,
                                       int nrhs, size_t* bytes) {
  fmca_status s = check_gpu_plan(p, precision);
  if (s != FMCA_OK) return s;
  if (!bytes || nrhs < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "bad nrhs or NULL bytes");
  *bytes = fmca::gpu::workspace_bytes(p->plan, precision, nrhs);
  return ok();
}

fmca_status fmca_matvec(fmca_plan* p, const fmca_kernel_desc* kernel,
                        int precision, int dtype, int order, int nrhs,
                        const void* x, int64_t x_stride_i, int64_t x_stride_r,
                        void* y, int64_t y_stride_i, int64_t y_stride_r,
                        void* workspace, size_t workspace_bytes, void* stream) {
  fmca_status s = check_gpu_plan(p, precision);
  if (s != FMCA_OK) return s;
  s = check_kernel(kernel);
  if (s != FMCA_OK) return s;
  if (dtype != FMCA_DTYPE_F64 && dtype != FMCA_DTYPE_F32)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "unknown dtype");
  if (order != FMCA_ORDER_NATURAL && order != FMCA_ORDER_CLUSTER)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "unknown order");
  if (nrhs < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "nrhs must be >= 1");
  if (!x || !y) return fail(FMCA_ERR_INVALID_ARGUMENT, "x or y is NULL");
  std::string err;
  int st = fmca::gpu::upload(p->plan, precision, &p->dev, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  st = fmca::gpu::matvec(p->plan, p->dev, to_desc(kernel), precision, dtype, order,
                         nrhs, x, x_stride_i, x_stride_r, y, y_stride_i, y_stride_r,
                         workspace, workspace_bytes, (cudaStream_t)stream, &err,
                         fmca::capi::call_opts(p));
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

fmca_status fmca_plan_assembled_size(const fmca_plan* p, int precision, size_t* bytes) {
  fmca_status s = check_gpu_plan(p, precision);
  if (s != FMCA_OK) return s;
  if (!bytes) return fail(FMCA_ERR_INVALID_ARGUMENT, "bytes is NULL");
  *bytes = fmca::gpu::assembled_bytes(p->plan, precision);
  return ok();
}

fmca_status fmca_plan_assemble(fmca_plan* p, const fmca_kernel_desc* kernel, int precision,
                               void* stream) {
  fmca_status s = check_gpu_plan(p, precision);
  if (s != FMCA_OK) return s;
  s = check_kernel(kernel);
  if (s != FMCA_OK) return s;
  std::string err;
  int st = fmca::gpu::upload(p->plan, precision, &p->dev, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  st = fmca::gpu::assemble(p->plan, p->dev, to_desc(kernel), precision, (cudaStream_t)stream,
                           &err, fmca::capi::call_opts(p));
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

fmca_status fmca_matvec_assembled(fmca_plan* p, int precision, int dtype, int order, int nrhs,
                                  const void* x, int64_t x_stride_i, int64_t x_stride_r,
                                  void* y, int64_t y_stride_i, int64_t y_stride_r,
                                  void* workspace, size_t workspace_bytes, void* stream) {
  fmca_status s = check_gpu_plan(p, precision);
  if (s != FMCA_OK) return s;
  if (dtype != FMCA_DTYPE_F64 && dtype != FMCA_DTYPE_F32)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "unknown dtype");
  if (order != FMCA_ORDER_NATURAL && order != FMCA_ORDER_CLUSTER)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "unknown order");
  if (nrhs < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "nrhs must be >= 1");
  if (!x || !y) return fail(FMCA_ERR_INVALID_ARGUMENT, "x or y is NULL");
  const int ap = p->dev ? fmca::gpu::assembled_precision(p->dev) : -1;
  if (ap < 0)
    return fail(FMCA_ERR_INVALID_ARGUMENT,
                "the plan holds no assembled blocks (fmca_plan_assemble)");
  if ((ap == FMCA_PREC_FP64) != (precision == FMCA_PREC_FP64))
    return fail(FMCA_ERR_INVALID_ARGUMENT,
                "the plan's blocks were assembled in another precision (FP64 blocks serve "
                "FMCA_PREC_FP64, FP32 blocks FMCA_PREC_FP32 and FMCA_PREC_MIXED)");
  std::string err;
  int st = fmca::gpu::upload(p->plan, precision, &p->dev, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  st = fmca::gpu::matvec_assembled(p->plan, p->dev, precision, dtype, order, nrhs, x,
                                   x_stride_i, x_stride_r, y, y_stride_i, y_stride_r,
                                   workspace, workspace_bytes, (cudaStream_t)stream, &err,
                                   fmca::capi::call_opts(p));
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

fmca_status fmca_plan_release_assembled(fmca_plan* p) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  fmca::gpu::release_assembled(p->dev);
  return ok();
}

fmca_status fmca_matvec_host(fmca_plan* p, const fmca_kernel_desc* kernel,
                             int precision, int order, int nrhs, const double* x,
                             double* y) {
  fmca_status s = check_gpu_plan(p, precision);
  if (s != FMCA_OK) return s;
  if (!x || !y || nrhs < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "bad x, y or nrhs");
  const size_t bx = sizeof(double) * (size_t)p->plan.cols.n * nrhs;
  const size_t by = sizeof(double) * (size_t)p->plan.rows.n * nrhs;
  cudaError_t e;
  if (p->hx_bytes < bx) {
    if (p->hx) cudaFree(p->hx);
    p->hx = nullptr;
    p->hx_bytes = 0;
    if ((e = cudaMalloc(&p->hx, bx)) != cudaSuccess)
      return fail(FMCA_ERR_OUT_OF_MEMORY, cudaGetErrorString(e));
    p->hx_bytes = bx;
  }
  if (p->hy_bytes < by) {
    if (p->hy) cudaFree(p->hy);
    p->hy = nullptr;
    p->hy_bytes = 0;
    if ((e = cudaMalloc(&p->hy, by)) != cudaSuccess)
      return fail(FMCA_ERR_OUT_OF_MEMORY, cudaGetErrorString(e));
    p->hy_bytes = by;
  }
  if ((e = cudaMemcpy(p->hx, x, bx, cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(FMCA_ERR_CUDA, cudaGetErrorString(e));
  s = fmca_matvec(p, kernel, precision, FMCA_DTYPE_F64, order, nrhs, p->hx, 1,
                  (int64_t)p->plan.cols.n, p->hy, 1, (int64_t)p->plan.rows.n, nullptr,
                  0, nullptr);
  if (s != FMCA_OK) return s;
  if ((e = cudaMemcpy(y, p->hy, by, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return fail(FMCA_ERR_CUDA, cudaGetErrorString(e));
  return fmca_plan_check_device_error(p);
}

fmca_status fmca_plan_check_device_error(fmca_plan* p) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  std::string err;
  int st = fmca::gpu::check_device_error(p->dev, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

fmca_status fmca_matvec_adjoint_workspace_size(const fmca_plan* p, int precision, int nrhs,
                                               size_t* bytes) {
  fmca_status s = check_gpu_plan(p, precision);
  if (s != FMCA_OK) return s;
  if (!bytes || nrhs < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "bad nrhs or NULL bytes");
  if (p->plan.interp.kind != fmca::kInterpTensor)
    return fail(FMCA_ERR_UNSUPPORTED, "the adjoint needs a tensor-product plan");
  *bytes = fmca::gpu::adjoint_workspace_bytes(p->plan, precision, nrhs);
  return ok();
}

fmca_status fmca_matvec_adjoint(fmca_plan* p, const fmca_kernel_desc* kernel, int precision,
                                int dtype, int nrhs, const void* x, int64_t x_stride_i,
                                int64_t x_stride_r, const void* y, int64_t y_stride_i,
                                int64_t y_stride_r, double* values, void* dX,
                                int64_t dX_stride_i, int64_t dX_stride_d, void* Kx, void* Ky,
                                void* workspace, size_t workspace_bytes, void* stream) {
  fmca_status s =
      fmca::capi::check_matvec_args(p, kernel, precision, dtype, FMCA_ORDER_NATURAL, nrhs,
                                    x, y);
  if (s != FMCA_OK) return s;
  if (p->plan.interp.kind != fmca::kInterpTensor)
    return fail(FMCA_ERR_UNSUPPORTED, "the adjoint needs a tensor-product plan");
  std::string err;
  int st = fmca::gpu::upload(p->plan, precision, &p->dev, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  st = fmca::gpu::adjoint(p->plan, p->dev, to_desc(kernel), precision, dtype, nrhs, x,
                          x_stride_i, x_stride_r, y, y_stride_i, y_stride_r, values, dX,
                          dX_stride_i, dX_stride_d, Kx, Ky, workspace, workspace_bytes,
                          (cudaStream_t)stream, &err, fmca::capi::call_opts(p));
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

fmca_status fmca_plan_update_points(fmca_plan* p, const double* P_rows, const double* P_cols) {
  if (!p || !P_rows) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  fmca::Plan& P = p->plan;
  const size_t dim = P.interp.dim;
  const bool same = P.same_tree && (P_cols == nullptr || P_cols == P_rows);
  if (!same && !P_cols)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "P_cols is required for two point clouds");
  for (size_t i = 0; i < dim * P.rows.n; ++i)
    if (!std::isfinite(P_rows[i]))
      return fail(FMCA_ERR_INVALID_ARGUMENT, "P_rows holds a non-finite value");
  if (!same)
    for (size_t i = 0; i < dim * P.cols.n; ++i)
      if (!std::isfinite(P_cols[i]))
        return fail(FMCA_ERR_INVALID_ARGUMENT, "P_cols holds a non-finite value");
  P.points_r.assign(P_rows, P_rows + dim * P.rows.n);
  if (same)
    P.points_c = P.points_r;
  else
    P.points_c.assign(P_cols, P_cols + dim * P.cols.n);
  std::string err;
  int st = fmca::gpu::update_points(P, p->dev, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

}  // extern "C"

struct fmca_graph {
  cudaGraphExec_t exec = nullptr;
  void* own_ws = nullptr;
  int device = -1;
};

extern "C" {

fmca_status fmca_matvec_graph_create(fmca_plan* p, const fmca_kernel_desc* kernel,
                                     int precision, int dtype, int order, int nrhs,
                                     const void* x, int64_t x_stride_i, int64_t x_stride_r,
                                     void* y, int64_t y_stride_i, int64_t y_stride_r,
                                     void* workspace, size_t workspace_bytes,
                                     fmca_graph** out) {
  if (!out) return fail(FMCA_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  fmca_status s =
      fmca::capi::check_matvec_args(p, kernel, precision, dtype, order, nrhs, x, y);
  if (s != FMCA_OK) return s;
  fmca_graph* g = new fmca_graph();
  cudaGetDevice(&g->device);
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaError_t e;
  auto cleanup = [&](fmca_status code, const std::string& msg) {
    if (graph) cudaGraphDestroy(graph);
    if (st) cudaStreamDestroy(st);
    if (g->own_ws) cudaFree(g->own_ws);
    delete g;
    return fail(code, msg);
  };
  if (!workspace) {
    workspace_bytes = fmca::gpu::workspace_bytes(p->plan, precision, nrhs);
    if ((e = cudaMalloc(&g->own_ws, workspace_bytes)) != cudaSuccess)
      return cleanup(FMCA_ERR_OUT_OF_MEMORY, cudaGetErrorString(e));
    workspace = g->own_ws;
  }
  if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess)
    return cleanup(FMCA_ERR_CUDA, cudaGetErrorString(e));
  // one ordinary run first: uploads the plan and sets kernel attributes
  s = fmca_matvec(p, kernel, precision, dtype, order, nrhs, x, x_stride_i, x_stride_r, y,
                  y_stride_i, y_stride_r, workspace, workspace_bytes, st);
  if (s != FMCA_OK) return cleanup(s, fmca_last_error());
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess)
    return cleanup(FMCA_ERR_CUDA, cudaGetErrorString(e));
  const bool prof = p->profile.exchange(false);
  if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
    p->profile = prof;
    return cleanup(FMCA_ERR_CUDA, cudaGetErrorString(e));
  }
  s = fmca_matvec(p, kernel, precision, dtype, order, nrhs, x, x_stride_i, x_stride_r, y,
                  y_stride_i, y_stride_r, workspace, workspace_bytes, st);
  e = cudaStreamEndCapture(st, &graph);
  p->profile = prof;
  if (s != FMCA_OK) return cleanup(s, fmca_last_error());
  if (e != cudaSuccess) return cleanup(FMCA_ERR_CUDA, cudaGetErrorString(e));
  if ((e = cudaGraphInstantiate(&g->exec, graph, 0)) != cudaSuccess)
    return cleanup(FMCA_ERR_CUDA, cudaGetErrorString(e));
  cudaGraphDestroy(graph);
  cudaStreamDestroy(st);
  *out = g;
  return ok();
}

fmca_status fmca_graph_launch(fmca_graph* g, void* stream) {
  if (!g || !g->exec) return fail(FMCA_ERR_INVALID_ARGUMENT, "graph is NULL");
  cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(FMCA_ERR_CUDA, cudaGetErrorString(e));
  return ok();
}

fmca_status fmca_graph_destroy(fmca_graph* g) {
  if (!g) return ok();
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->own_ws) cudaFree(g->own_ws);
  delete g;
  return ok();
}

fmca_status fmca_plan_set_profiling(fmca_plan* p, int enable) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  p->profile = enable != 0;
  return ok();
}

fmca_status fmca_plan_set_wait_limit(fmca_plan* p, uint64_t ns) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  p->wait_ns = ns;
  return ok();
}

fmca_status fmca_plan_set_autotune(fmca_plan* p, int enable) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  p->autotune = enable != 0;
  return ok();
}

fmca_status fmca_plan_tuned_config(fmca_plan* p, int precision, int kernel_type, int nrhs,
                                   int32_t out[FMCA_TUNE_COUNT]) {
  if (!p || !out) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (nrhs < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "nrhs must be >= 1");
  fmca::gpu::tuned_config(p->dev, precision, kernel_type, nrhs, out);
  return ok();
}

fmca_status fmca_plan_set_tuned_config(fmca_plan* p, int precision, int kernel_type, int nrhs,
                                       const int32_t cfg[FMCA_TUNE_COUNT]) {
  if (!p || !cfg) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  if (nrhs < 1) return fail(FMCA_ERR_INVALID_ARGUMENT, "nrhs must be >= 1");
  if (!fmca::gpu::resident(p->dev, precision))
    return fail(FMCA_ERR_INVALID_ARGUMENT,
                "the plan is not resident on the current device for this precision");
  std::string err;
  const int st = fmca::gpu::set_tuned_config(p->dev, precision, kernel_type, nrhs, cfg, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

fmca_status fmca_plan_set_stalled_wait(fmca_plan* p, int on) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  p->stall = on != 0;
  return ok();
}

fmca_status fmca_plan_device_bytes(const fmca_plan* p, size_t* bytes) {
  if (!p || !bytes) return fail(FMCA_ERR_INVALID_ARGUMENT, "NULL argument");
  *bytes = fmca::gpu::device_bytes(p->dev) + p->hx_bytes + p->hy_bytes;
  return ok();
}

fmca_status fmca_plan_profile(fmca_plan* p, double* stage_ms, int64_t* launches) {
  if (!p) return fail(FMCA_ERR_INVALID_ARGUMENT, "plan is NULL");
  double tmp[FMCA_STAGE_COUNT];
  std::string err;
  int st = fmca::gpu::profile(p->dev, stage_ms ? stage_ms : tmp, launches, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

fmca_status fmca_kernel_eval(const fmca_kernel_desc* kernel, int dim,
                             const double* PR, int64_t n_r, const double* PC,
                             int64_t n_c, double* out) {
  fmca_status s = check_kernel(kernel);
  if (s != FMCA_OK) return s;
  if (!PR || !PC || !out || dim < 1 || n_r < 1 || n_c < 1)
    return fail(FMCA_ERR_INVALID_ARGUMENT, "bad arguments");
  std::string err;
  int st = fmca::gpu::dense_eval(to_desc(kernel), dim, PR, n_r, PC, n_c, out, &err);
  if (st != FMCA_OK) return fail((fmca_status)st, err);
  return ok();
}

}  // extern "C"
