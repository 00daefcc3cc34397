/*
 * fmca_gb300 — C ABI of the GB300 H2-matrix kernel matvec.
 *
 * This is the drop-in boundary for FMCA's matrix-free H2 product.  Every
 * entry point takes plain pointers and sizes, returns an fmca_status and
 * never aborts; a message for the last failure of the calling thread is
 * available from fmca_last_error().
 *
 * Reference interfaces replaced (paths inside muchip/fmca):
 *   fmca_plan_create      H2ClusterTree(mom, min_csize, P) for rows and
 *                         columns + H2Matrix::computePattern(rct, cct, eta):
 *                         FMCA/src/H2Matrix/H2ClusterTree.h:60-74,
 *                         FMCA/src/H2Matrix/H2MatrixBase.h:160-191;
 *                         the Python constructor pyH2Matrix(ker, Pr, Pc, p,
 *                         eta): py/FMCA.cpp:210-220.
 *   fmca_plan_statistics  H2MatrixBase::statistics(): H2MatrixBase.h:70-105,
 *                         py/FMCA.cpp:222.
 *   fmca_plan_permutation ClusterTreeBase::indices(), pyH2Matrix::rindices /
 *                         cindices: FMCA/src/Clustering/ClusterTreeBase.h:63-65,
 *                         py/FMCA.cpp:224-229.
 *   fmca_plan_clusters    per-cluster bounding boxes and index ranges of the
 *                         two trees (ClusterTreeBase::bb/indices_begin/
 *                         block_size): ClusterTreeBase.h:61-71.
 *   fmca_plan_blocks      the leaves of the block tree built by
 *                         computePattern (low-rank / dense): H2MatrixBase.h:
 *                         160-191.
 *   fmca_matvec           H2MatrixBase::action(mat_eval, rhs) with the
 *                         (unsymmetric)NystromEvaluator + CovarianceKernel:
 *                         H2MatrixBase.h:113-152, NystromEvaluator.h:40-71,
 *                         unsymmetricNystromEvaluator.h:42-73,
 *                         CovarianceKernel.h:50-151; in natural order it is
 *                         pyH2Matrix::action: py/FMCA.cpp:230-240.
 *   fmca_matvec_host      the same as fmca_matvec with host buffers (the
 *                         call made by the Python binding's .action).
 *   fmca_kernel_eval      CovarianceKernel::eval(PR, PC): CovarianceKernel.h:
 *                         145-151 (FP64, host buffers, GPU evaluation).
 */
#ifndef FMCA_GB300_H_
#define FMCA_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  FMCA_OK = 0,
  FMCA_ERR_INVALID_ARGUMENT = 1,
  FMCA_ERR_UNSUPPORTED = 2,
  FMCA_ERR_CUDA = 3,
  FMCA_ERR_OUT_OF_MEMORY = 4,
  FMCA_ERR_TIMEOUT = 5,
  FMCA_ERR_INTERNAL = 6
} fmca_status;

/* Kernel codes; names as accepted by FMCA's CovarianceKernel. */
enum {
  FMCA_KERNEL_EXPONENTIAL = 0,
  FMCA_KERNEL_MATERN32 = 1,
  FMCA_KERNEL_MATERN52 = 2,
  FMCA_KERNEL_GAUSSIAN = 3,
  FMCA_KERNEL_MATERN72 = 4,
  FMCA_KERNEL_MATERN92 = 5,
  FMCA_KERNEL_INVMULTIQUADRIC = 6,
  FMCA_KERNEL_MULTIQUADRIC = 7,
  FMCA_KERNEL_BIHARMONIC3D = 8,
  FMCA_KERNEL_TRIHARMONIC3D = 9,
  /* dk/dl of EXPONENTIAL, MATERN32, MATERN52, GAUSSIAN (names "DL_..."):
     fmca_matvec with these gives sigma2 * H2[dk/dl] x, the derivative of the
     H2 product with respect to the length scale at fixed nodes */
  FMCA_KERNEL_DL_EXPONENTIAL = 10,
  FMCA_KERNEL_DL_MATERN32 = 11,
  FMCA_KERNEL_DL_MATERN52 = 12,
  FMCA_KERNEL_DL_GAUSSIAN = 13,
  /* (r/l)^2 log(r/l), 0 below r = DBL_EPSILON (CovarianceKernel.h:56-59) */
  FMCA_KERNEL_BIHARMONIC2D = 14,
  /* r^2 log(r), 0 at r = 0; l is not used (CovarianceKernel.h:117-118) */
  FMCA_KERNEL_TPS2D = 15
};

/* Arithmetic of the matvec. */
enum {
  /* every stage in FP64 on CUDA cores: the plain FP64 GPU H2 product */
  FMCA_PREC_FP64 = 0,
  /* kernel values in FP32; near-field and far-field contractions on the
     tensor cores with FP16 hi/lo split operands (three products, about 22
     significant bits) and FP32 accumulation; transfers, leaf moments and the
     leaf gather in FP32; final near + far combination in FP64.  Kernels that
     are not bounded by 1 (MULTIQUADRIC, INVMULTIQUADRIC, BIHARMONIC2D/3D,
     TRIHARMONIC3D, TPS2D) use FMCA_PREC_FP32, and so do fewer than 17 right-hand
     sides unless the autotuner (fmca_plan_set_autotune) measured the
     tensor-core path, with the columns padded to 32, faster. */
  FMCA_PREC_MIXED = 1,
  /* every stage in FP32 on CUDA cores with FP32 accumulation, final
     combination in FP64 */
  FMCA_PREC_FP32 = 2
};

enum { FMCA_DTYPE_F64 = 0, FMCA_DTYPE_F32 = 1 };
/* FMCA_ORDER_NATURAL: x and y are indexed like the input point clouds
   (pyH2Matrix::action).  FMCA_ORDER_CLUSTER: both are in cluster order
   (H2MatrixBase::action). */
enum { FMCA_ORDER_NATURAL = 0, FMCA_ORDER_CLUSTER = 1 };

typedef struct {
  int type;      /* FMCA_KERNEL_* */
  double l;      /* length scale (CovarianceKernel l) */
  double c;      /* shift of the (inverse) multiquadric (CovarianceKernel c) */
  double nu;     /* accepted for signature parity; unused */
  double sigma2; /* variance: K = sigma2 * k(r); 1.0 reproduces FMCA */
} fmca_kernel_desc;

typedef struct fmca_plan fmca_plan;

/* Plan information, indices of fmca_plan_info's output array. */
enum {
  FMCA_INFO_N_ROWS = 0,
  FMCA_INFO_N_COLS = 1,
  FMCA_INFO_DIM = 2,
  FMCA_INFO_DEGREE = 3,
  FMCA_INFO_Q = 4,
  FMCA_INFO_ROW_CLUSTERS = 5,
  FMCA_INFO_COL_CLUSTERS = 6,
  FMCA_INFO_FAR_BLOCKS = 7,
  FMCA_INFO_NEAR_BLOCKS = 8,
  FMCA_INFO_NEAR_PAIRS = 9,
  FMCA_INFO_ROW_LEVELS = 10,
  FMCA_INFO_COL_LEVELS = 11,
  FMCA_INFO_ROW_LEAVES = 12,
  FMCA_INFO_COL_LEAVES = 13,
  FMCA_INFO_MIN_LEAF = 14,
  FMCA_INFO_INTERPOLATOR = 15, /* FMCA_INTERP_* */
  FMCA_INFO_COUNT = 16
};

/* Message of the last failure on this thread (empty if none). */
const char* fmca_last_error(void);
/* Library version string. */
const char* fmca_version(void);

/* Maps an FMCA kernel name ("MATERN32", case-insensitive) to its code. */
fmca_status fmca_kernel_type_from_name(const char* name, int* type);

/* Builds the plan on the host.  P_rows: dim x n_rows, column-major FP64
   (one point per column, like FMCA's Matrix P).  P_cols may be NULL or equal
   to P_rows for the symmetric case.  degree: interpolation degree p.
   min_leaf: minimum leaf size (the effective value is max(min_leaf,
   (p+1)^dim) like H2ClusterTree::init).  Device data is uploaded lazily on
   the first matvec to the current CUDA device. */
fmca_status fmca_plan_create(const double* P_rows, int dim, int64_t n_rows,
                             const double* P_cols, int64_t n_cols, int degree,
                             double eta, int64_t min_leaf, fmca_plan** out);
fmca_status fmca_plan_destroy(fmca_plan* plan);

/* Interpolators of fmca_plan_create_ex. */
enum { FMCA_INTERP_TENSOR_PRODUCT = 0, FMCA_INTERP_TOTAL_DEGREE = 1 };

/* fmca_plan_create with a choice of interpolator.  Replaces the Interpolator
   parameter of NystromMoments<Interpolator> (FMCA/src/Moments/
   NystromMoments.h:15-31): FMCA_INTERP_TENSOR_PRODUCT is
   TensorProductInterpolator (q = (p+1)^dim, what fmca_plan_create builds);
   FMCA_INTERP_TOTAL_DEGREE is TotalDegreeInterpolator
   (FMCA/src/Interpolator/TotalDegreeInterpolator.h:26-47: q = binom(p+dim,
   dim) DeMarchi nodes, Legendre polynomials, coupling invV K invV^T), the
   interpolator the reference's Python module instantiates
   (py/FMCA.cpp:37-40).  Total degree: dim <= 3, degree <= 15 and at most
   120 nodes (degree <= 7 in 3-D, <= 14 in 2-D); the adjoint and batched
   plans are tensor-product only (FMCA_ERR_UNSUPPORTED). */
fmca_status fmca_plan_create_ex(const double* P_rows, int dim, int64_t n_rows,
                                const double* P_cols, int64_t n_cols, int interpolator,
                                int degree, double eta, int64_t min_leaf, fmca_plan** out);

/* fmca_plan_create_ex with the plan's structure built on the GPU (current
   device), giving the identical plan:
   - cluster trees: every level of a tree is one segmented radix sort of the
     index ranges of the clusters that split, in place of the reference's
     std::sort per cluster (ClusterTreeSplitter.h:60-81 called by
     ClusterTreeInitializer_ClusterTree.h:56-86).  Where a sorted range holds
     equal coordinates, whose order the reference's std::sort decides, that
     tree is built on the host instead;
   - block pattern: the block tree of computePattern (H2MatrixBase.h:
     160-191) level by level, the same admissibility decisions in the same
     FP64 operation order, the leaves sorted into the reference's
     depth-first order.
   gpu_parts (may be NULL) receives two ints: the number of trees sorted on
   the GPU (0, 1, or 2 for two point clouds) and 1 if the block lists were
   built there.  Bounding boxes, interpolation data and the derived GPU
   lists are built on the host as for fmca_plan_create_ex.  Synchronous;
   uses its own stream and frees its device memory before returning. */
fmca_status fmca_plan_create_gpu(const double* P_rows, int dim, int64_t n_rows,
                                 const double* P_cols, int64_t n_cols, int interpolator,
                                 int degree, double eta, int64_t min_leaf, int* gpu_parts,
                                 fmca_plan** out);

/* One plan for many independent point clouds (batching): cloud i has
   n_points[i] points P[i] (dim x n_i, column-major FP64); every cloud gets
   its own tree and block lists exactly as fmca_plan_create would build them
   (for P_cols = NULL), and the plan is their block-diagonal union.  A matvec
   on it takes the clouds' right-hand sides concatenated in cloud order
   (sum n_i rows) and runs every stage for all clouds in one launch.  No
   counterpart in the reference (one H2Matrix per cloud there). */
fmca_status fmca_plan_create_batched(const double* const* P, const int64_t* n_points,
                                     int count, int dim, int degree, double eta,
                                     int64_t min_leaf, fmca_plan** out);

/* A matvec recorded once into a CUDA graph and replayed with one launch.
   The graph binds the given x, y and workspace pointers (workspace NULL: the
   graph allocates its own).  The plan must outlive the graph. */
typedef struct fmca_graph fmca_graph;
fmca_status fmca_matvec_graph_create(fmca_plan* plan, const fmca_kernel_desc* kernel,
                                     int precision, int dtype, int order, int nrhs,
                                     const void* x, int64_t x_stride_i,
                                     int64_t x_stride_r, void* y, int64_t y_stride_i,
                                     int64_t y_stride_r, void* workspace,
                                     size_t workspace_bytes, fmca_graph** out);
fmca_status fmca_graph_launch(fmca_graph* graph, void* stream);
fmca_status fmca_graph_destroy(fmca_graph* graph);
fmca_status fmca_plan_info(const fmca_plan* plan, int64_t out[FMCA_INFO_COUNT]);
/* (rows, cols, #low-rank blocks, #dense blocks, nz per row, storage GB) */
fmca_status fmca_plan_statistics(const fmca_plan* plan, double out[6]);
/* side 0: rows, 1: columns.  perm[i] = natural index of cluster-order i. */
fmca_status fmca_plan_permutation(const fmca_plan* plan, int side,
                                  uint32_t* perm);
/* Per cluster in level order: meta[4c+0..3] = (begin, size, level, parent),
   bb[3*dim*c + ...] = (min[dim], max[dim], extent[dim]).  Either pointer may
   be NULL. */
fmca_status fmca_plan_clusters(const fmca_plan* plan, int side, int32_t* meta,
                               double* bb);
/* The interpolator of the plan: nodes (dim x q, column-major, on [0,1]^dim
   in the plan's node order: TensorProductInterpolator::Xi or the DeMarchi
   points of TotalDegreeInterpolator::Xi) and, for total degree, invV (q x q,
   column-major; TotalDegreeInterpolator::invV).  Either pointer may be NULL;
   invV is left untouched for a tensor-product plan. */
fmca_status fmca_plan_interpolator(const fmca_plan* plan, double* nodes, double* invV);
/* Clouds of a plan: *count receives their number (1 for a plan of one
   point cloud) and, when offsets is not NULL, offsets[0 .. count] the first
   row of every cloud followed by the total row count, in the order the
   clouds were given to fmca_plan_create_batched. */
fmca_status fmca_plan_cloud_offsets(const fmca_plan* plan, int64_t* offsets, int* count);
/* Plan files.  fmca_plan_save writes the host plan (points, both cluster
   trees, block lists, transfer and node data) as a sequence of matrices in
   the binary layout of FMCA's print2bin / bin2Mat (FMCA/src/util/IO.h:
   532-626: element size, row-major flag, rows and cols as size_t, then the
   column-major data); fmca_plan_load reads it back into a new plan that
   behaves exactly like the saved one, without rebuilding the trees or the
   block pattern.  Device data is not stored: it is uploaded on the first
   matvec as for a new plan.  Malformed files give FMCA_ERR_INVALID_ARGUMENT. */
fmca_status fmca_plan_save(const fmca_plan* plan, const char* path);
fmca_status fmca_plan_load(const char* path, fmca_plan** out);
/* kind 0: low-rank (far) blocks, 1: dense (near) blocks; row/col cluster ids
   in the order the pattern recursion produced them. */
fmca_status fmca_plan_blocks(const fmca_plan* plan, int kind, int32_t* rows,
                             int32_t* cols);
/* The packed near groups of the tensor-core kernel sum with one target half
   (an autotuner choice, FMCA_TUNE_NEAR_PACK): the rows of up to two
   consecutive row leaves per group of up to 128 targets, over the union of
   the leaves' source intervals.  Pass NULL groups and intervals for the
   counts (both 0 where the plan has no packed groups: they would not save a
   tenth of the groups of one leaf each); then groups receives ngroups x 5
   values (first target, targets, first interval, end interval, targets of
   the group's first leaf) in launch order, and intervals nintervals x 3
   (first source, end source, leaves served: bit 0 the group's first leaf,
   bit 1 its second), targets and sources in cluster order.  The groups
   cover the dense blocks of H2MatrixBase.h:143-146 (every pair of a row
   leaf and a point of its dense blocks) once. */
fmca_status fmca_plan_near_packed(const fmca_plan* plan, int64_t* ngroups, int64_t* nintervals,
                                  uint32_t* groups, uint32_t* intervals);

/* Device memory the plan holds now, in bytes: its uploaded data (lists,
   points, nodes, transfers), the workspace it owns (allocated or grown by
   matvecs called without a workspace) and the staging buffers of
   fmca_matvec_host.  0 before the first matvec.  No reference counterpart
   (H2MatrixBase::statistics, H2MatrixBase.h:70-105, reports the storage of
   an assembled matrix, not device memory). */
fmca_status fmca_plan_device_bytes(const fmca_plan* plan, size_t* bytes);

/* Bytes of device workspace fmca_matvec needs for nrhs right-hand sides. */
fmca_status fmca_matvec_workspace_size(const fmca_plan* plan, int precision,
                                       int nrhs, size_t* bytes);

/* y = K_H2 x on the GPU.  x: n_cols x nrhs, y: n_rows x nrhs, both device
   pointers of dtype; element (i, r) lives at ptr[i*stride_i + r*stride_r]
   (column-major FMCA layout: stride_i = 1, stride_r = n).  workspace: device
   memory of fmca_matvec_workspace_size bytes, or NULL to use a buffer owned
   by the plan.  stream: a cudaStream_t (NULL = legacy default stream).  The
   call is asynchronous; device-side failures (timeouts of bounded waits) are
   reported by fmca_plan_check_device_error after a synchronisation. */
fmca_status fmca_matvec(fmca_plan* plan, const fmca_kernel_desc* kernel,
                        int precision, int dtype, int order, int nrhs,
                        const void* x, int64_t x_stride_i, int64_t x_stride_r,
                        void* y, int64_t y_stride_i, int64_t y_stride_r,
                        void* workspace, size_t workspace_bytes, void* stream);

/* The same product as fmca_matvec, for callers that cannot allocate device
   memory when they run it: for instance a plugin inside an application that
   owns all GPU memory through its own allocator or budget, or a latency-bound
   loop that cannot afford cudaMalloc / cudaFree (both can synchronise the
   device).  This entry point allocates nothing: its scratch is a fixed
   64 MiB device array built into the library (held on every GPU that loads
   it until the process exits), and the caller passes x and y as for
   fmca_matvec.  Has no counterpart in the reference.
   - Plans whose scratch for this precision and nrhs exceeds 64 MiB (see
     fmca_matvec_workspace_size) are rejected with FMCA_ERR_UNSUPPORTED.
   - The plan must already be resident on the current device for this
     precision (it becomes resident, allocating once, on its first
     fmca_matvec / fmca_matvec_host call there); otherwise
     FMCA_ERR_INVALID_ARGUMENT.
   - The first call on each device looks up the array's device address; make
     that first call before any stream capture.
   - All calls share the one array: calls whose GPU work overlaps (other
     streams, other threads) race and give wrong results. */
fmca_status fmca_matvec_static_scratch(fmca_plan* plan,
                                       const fmca_kernel_desc* kernel,
                                       int precision, int dtype, int order,
                                       int nrhs, const void* x,
                                       int64_t x_stride_i, int64_t x_stride_r,
                                       void* y, int64_t y_stride_i,
                                       int64_t y_stride_r, void* stream);

/* The same product with FP64 column-major host buffers (ld = n); copies in
   and out and synchronises. */
fmca_status fmca_matvec_host(fmca_plan* plan, const fmca_kernel_desc* kernel,
                             int precision, int order, int nrhs,
                             const double* x, double* y);

/* Assembled H2 matrix: the far-field coupling blocks S (kernel at the
   interpolation nodes, q x q per admissible block) and the dense near-field
   blocks evaluated once and kept in device memory, traded for the kernel
   evaluations of every later product (repeated products with one kernel:
   iterative solvers, trace estimation, the FP64 residual of a mixed solve).

   fmca_plan_assembled_size: device bytes the stored blocks take for this
   precision (FP64 values for FMCA_PREC_FP64, FP32 values for FMCA_PREC_FP32
   and FMCA_PREC_MIXED), counted on the host; no device is needed.
   Replaces nothing in the reference (its H2MatrixBase::statistics,
   H2MatrixBase.h:70-105, estimates the storage of an assembled FP64 matrix).

   fmca_plan_assemble: H2MatrixBase::computeH2Matrix (H2MatrixBase.h:222-255;
   the H2Matrix(CT, mat_eval, eta) constructor, H2Matrix.h:53-66): evaluates
   and stores every block for this kernel on the current device, replacing
   blocks stored earlier.  The kernel evaluations run asynchronously on
   stream; the allocation and the block offsets are synchronous.
   FMCA_ERR_OUT_OF_MEMORY leaves the plan without stored blocks.

   fmca_matvec_assembled: H2MatrixBase::operator* (H2MatrixBase.h:107-109,
   matrix_vector_product_impl.h:17-98): y = K_H2 x from the stored blocks,
   with the upward and downward passes of fmca_matvec.  The kernel is the
   one the blocks were assembled with; precision must be FMCA_PREC_FP64 for
   FP64 blocks and FMCA_PREC_FP32 or FMCA_PREC_MIXED for FP32 blocks (the
   stored blocks are contracted on the FP32 CUDA cores), otherwise
   FMCA_ERR_INVALID_ARGUMENT, as without stored blocks.  Arguments, workspace
   (fmca_matvec_workspace_size of the same precision suffices) and stream as
   for fmca_matvec.

   fmca_plan_release_assembled: frees the stored blocks (no-op without). */
fmca_status fmca_plan_assembled_size(const fmca_plan* plan, int precision,
                                     size_t* bytes);
fmca_status fmca_plan_assemble(fmca_plan* plan, const fmca_kernel_desc* kernel,
                               int precision, void* stream);
fmca_status fmca_matvec_assembled(fmca_plan* plan, int precision, int dtype,
                                  int order, int nrhs, const void* x,
                                  int64_t x_stride_i, int64_t x_stride_r,
                                  void* y, int64_t y_stride_i,
                                  int64_t y_stride_r, void* workspace,
                                  size_t workspace_bytes, void* stream);
fmca_status fmca_plan_release_assembled(fmca_plan* plan);

/* Adjoint of the H2 product (no counterpart in the reference, which has no
   derivatives).  For f = sum_r y_r^T K x_r with K = sigma2 * H2[k] (cluster
   tree, boxes and interpolation nodes held fixed), it computes on the device:
     values[0..2] = f, df/dl, df/dsigma2   (FP64; NaN for df/dl of kernels
                                            without a DL_ counterpart)
     dX           = df/dX, n x dim in natural order (strides), dtype of x;
                    needs one point cloud (P_cols NULL) and one of
                    EXPONENTIAL, MATERN32, MATERN52, GAUSSIAN
     Kx           = K x  (n_rows x nrhs, strides of y), optional
     Ky           = K y  (n_cols x nrhs, strides of x; one point cloud)
   Any output pointer may be NULL.  x: n_cols x nrhs, y: n_rows x nrhs, both
   device buffers of dtype.  workspace: fmca_matvec_adjoint_workspace_size
   bytes or NULL (plan-owned).  Asynchronous on stream. */
fmca_status fmca_matvec_adjoint_workspace_size(const fmca_plan* plan,
                                               int precision, int nrhs,
                                               size_t* bytes);
fmca_status fmca_matvec_adjoint(fmca_plan* plan, const fmca_kernel_desc* kernel,
                                int precision, int dtype, int nrhs,
                                const void* x, int64_t x_stride_i,
                                int64_t x_stride_r, const void* y,
                                int64_t y_stride_i, int64_t y_stride_r,
                                double* values, void* dX, int64_t dX_stride_i,
                                int64_t dX_stride_d, void* Kx, void* Ky,
                                void* workspace, size_t workspace_bytes,
                                void* stream);
/* Replaces the point coordinates (dim x n, column-major FP64, host) while
   keeping the cluster tree, boxes, interpolation nodes and block lists: the
   H2 matrix of moved points with a frozen structure, as differentiated by
   fmca_matvec_adjoint.  P_cols may be NULL for one point cloud.  Synchronous.
   No counterpart in the reference (which rebuilds the tree). */
fmca_status fmca_plan_update_points(fmca_plan* plan, const double* P_rows,
                                    const double* P_cols);

/* Returns FMCA_ERR_TIMEOUT if a kernel of this plan gave up a bounded wait
   since the last call, and clears the flag.  Synchronises the device. */
fmca_status fmca_plan_check_device_error(fmca_plan* plan);

/* Limit, in ns, of every bounded wait inside the kernel sums (near and far
   field) of this plan's following matvecs and adjoints; 0 restores the
   default of 2 s.  A kernel whose wait runs out raises the plan's device
   error flag (FMCA_ERR_TIMEOUT from fmca_plan_check_device_error), drains
   its own copies and tensor-core products under a fixed limit, frees its
   tensor memory and returns; the results of that call are undefined and
   the GPU context stays usable.  No counterpart in the reference (which has no GPU waits). */
fmca_status fmca_plan_set_wait_limit(fmca_plan* plan, uint64_t ns);
/* Test hook for the timeout path (no reference counterpart): while on,
   the first wait of every kernel-sum CTA of this plan's matvecs is on a
   barrier that nothing completes, so it runs out after the wait limit and
   the call ends with FMCA_ERR_TIMEOUT as described above, without a GPU
   fault.  Off by default; results of calls made while it is on are
   undefined. */
fmca_status fmca_plan_set_stalled_wait(fmca_plan* plan, int on);

/* Autotuner (no counterpart in the reference, whose column-bucket loop,
   H2MatrixBase.h:127-148, has no launch shapes to choose).  While enabled,
   the first mixed-precision matvec of each (precision, kernel type, nrhs)
   key on this plan measures the launch shapes below with CUDA events on the
   caller's stream and keeps the fastest for every later call of that key:
     - nrhs <= 16: FP32 CUDA-core kernel sums, or tensor-core kernel sums
       with the right-hand sides padded to 32 columns;
     - the near-field kernel sum's copy-ring stages (4..7) and tiles per
       accumulation unit (1..3), with target groups of two halves of 128 or
       of one (small leaves), launched with one CTA per group or as a
       persistent grid of one CTA per SM that runs the groups in turn;
     - the far field on sibling-paired tensor grids or on interpolation
       nodes (3-D plans of degree 4), with its stages, units and launch
       form;
     - the transfer passes' level thresholds for 8 warps per cluster and
       for splitting the right-hand sides into slices of 8.
   That first call takes longer (about 20 kernel-sum runs) and gives the
   same result as a call with the chosen shapes.  Calls made inside a CUDA
   stream capture, adjoints and FP64 / FP32 matvecs do not tune (they use the
   tuned shapes of their key if there are any, else the defaults).  Off by
   default. */
fmca_status fmca_plan_set_autotune(fmca_plan* plan, int enable);
/* Indices of fmca_plan_tuned_config's output. */
enum {
  FMCA_TUNE_TUNED = 0,            /* 1: chosen by the autotuner, 0: defaults */
  FMCA_TUNE_NEAR_STAGES = 1,      /* near field: copy-ring stages */
  FMCA_TUNE_NEAR_UNIT = 2,        /* near field: tiles per accumulation unit */
  FMCA_TUNE_FAR_PAIRS = 3,        /* 1: paired tensor grids, 0: nodes */
  FMCA_TUNE_FAR_GRID_STAGES = 4,  /* far field on paired grids: stages */
  FMCA_TUNE_FAR_GRID_UNIT = 5,    /*   and tiles per unit */
  FMCA_TUNE_FAR_NODE_STAGES = 6,  /* far field on nodes: stages */
  FMCA_TUNE_FAR_NODE_UNIT = 7,    /*   and tiles per unit */
  FMCA_TUNE_WIDE_BELOW = 8,       /* transfer levels with fewer clusters: 8 warps each */
  FMCA_TUNE_SLICE_BELOW = 9,      /* transfer levels with fewer clusters: RHS slices of 8 */
  FMCA_TUNE_SMALL_R_TENSOR = 10,  /* nrhs <= 16: 1 tensor cores, 0 CUDA cores */
  FMCA_TUNE_NEAR_HALVES = 11,     /* near field: groups of 2 x 128 or 1 x 128 targets */
  FMCA_TUNE_NEAR_PERSIST = 12,    /* near field: 1 one CTA per SM running groups in turn */
  FMCA_TUNE_FAR_PERSIST = 13,     /* far field: the same */
  FMCA_TUNE_US = 14,              /* time the tuning took, microseconds */
  FMCA_TUNE_TUNINGS = 15,         /* tuning runs on this plan so far */
  FMCA_TUNE_FAR_KRON = 16,        /* GAUSSIAN on tensor-product nodes, mixed precision:
                                     1 far field as Kronecker products, 0 kernel sums */
  FMCA_TUNE_NEAR_PACK = 17,       /* near field with 1 x 128 targets, one CTA per group:
                                     1 rows of up to two leaves per group, 0 one leaf */
  FMCA_TUNE_COUNT = 18
};
/* The launch shapes a matvec of this key uses now: the tuned ones, or the
   defaults (FMCA_TUNE_TUNED = 0). */
fmca_status fmca_plan_tuned_config(fmca_plan* plan, int precision, int kernel_type, int nrhs,
                                   int32_t out[FMCA_TUNE_COUNT]);
/* Sets the launch shapes of a key as if the autotuner had chosen them
   (entries FMCA_TUNE_NEAR_STAGES .. FMCA_TUNE_FAR_PERSIST, FMCA_TUNE_FAR_KRON
   and FMCA_TUNE_NEAR_PACK of cfg; the others are ignored): for reusing
   shapes tuned earlier, for instance in another
   process on the same plan.  The plan must be resident on the current
   device (after one matvec).  Out-of-range shapes give
   FMCA_ERR_INVALID_ARGUMENT. */
fmca_status fmca_plan_set_tuned_config(fmca_plan* plan, int precision, int kernel_type,
                                       int nrhs, const int32_t cfg[FMCA_TUNE_COUNT]);

/* Stages of one matvec, indices of fmca_plan_profile's output. */
enum {
  FMCA_STAGE_GATHER = 0,     /* natural -> cluster order */
  FMCA_STAGE_LEAFMOM = 1,    /* leaf moments (upward pass, leaves) */
  FMCA_STAGE_M2M = 2,        /* transfers, upward pass */
  FMCA_STAGE_FAR = 3,        /* far-field coupling */
  FMCA_STAGE_L2L = 4,        /* transfers, downward pass */
  FMCA_STAGE_LEAFGATHER = 5, /* leaf gather (downward pass, leaves) */
  FMCA_STAGE_NEAR = 6,       /* near field */
  FMCA_STAGE_SCATTER = 7,    /* combination and cluster -> natural order */
  FMCA_STAGE_COUNT = 8
};

/* Enables CUDA-event timing of the stages of the following matvecs on this
   plan (adds one event record per stage; off by default).  No reference
   counterpart: the reference times phases with Tictoc
   (FMCA/src/util/Tictoc.h:22-42) around whole calls only. */
fmca_status fmca_plan_set_profiling(fmca_plan* plan, int enable);
/* Stage times in ms of the last matvec on this plan (waits for its events)
   and the number of kernels it launched.  stage_ms has FMCA_STAGE_COUNT
   entries; either pointer may be NULL. */
fmca_status fmca_plan_profile(fmca_plan* plan, double* stage_ms,
                              int64_t* launches);

/* Dense kernel matrix K(PR, PC) (n_r x n_c, column-major FP64 host buffers),
   evaluated on the GPU in FP64; like CovarianceKernel::eval. */
fmca_status fmca_kernel_eval(const fmca_kernel_desc* kernel, int dim,
                             const double* PR, int64_t n_r, const double* PC,
                             int64_t n_c, double* out);

#ifdef __cplusplus
}
#endif
#endif /* FMCA_GB300_H_ */
