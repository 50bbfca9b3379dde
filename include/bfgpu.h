/*
 * bfgpu.h -- C ABI of the GB300 far-field butterfly library (libbfgpu.so).
 *
 * The library replaces the far-field hot path of ButterflyFactorizations.jl:
 * the butterfly matvec (forward, adjoint, transpose; one or many right-hand
 * sides) and the kernel sampling + partial-RRQR skeletonisation that builds the
 * factors.  Every entry point below names the reference interface it stands in
 * for (paths relative to the ButterflyFactorizations.jl repository).
 *
 * Conventions
 *   - Plain pointers and sizes only; no exceptions cross the ABI.  Every call
 *     returns a status code (BF_OK on success); bf_last_error() returns a
 *     thread-local description of the last failure.
 *   - Indices are 0-based (the Julia binding subtracts 1).
 *   - Complex numbers are interleaved (re, im) doubles, i.e. Julia ComplexF64.
 *   - Matrices of right-hand sides are column-major with a leading dimension.
 *   - An operator handle owns its device memory and its CUDA stream.  Calls on
 *     one handle must be serialised by the caller (the reference operator is
 *     likewise not re-entrant, src/Matrixassembly/matrixstructs.jl:20-21);
 *     distinct handles are independent.
 *   - There is no CPU fallback: without a usable CUDA device every compute
 *     entry point returns BF_ECUDA.
 */
#ifndef BFGPU_H
#define BFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define BF_API __attribute__((visibility("default")))
#else
#define BF_API
#endif

/* ---- status codes (no reference counterpart: Julia raises exceptions) ---- */
enum {
  BF_OK = 0,
  BF_EINVAL = 1,    /* invalid argument or malformed factor description */
  BF_ENOMEM = 2,    /* device or host allocation failed                  */
  BF_ECUDA = 3,     /* CUDA runtime / launch error, or no device          */
  BF_ETIMEOUT = 4,  /* a bounded device-side wait gave up                 */
  BF_ENOTSUP = 5,   /* feature not supported for this operator            */
  BF_ESTATE = 6     /* call not valid in the handle's current state       */
};

/* ---- operation selector for matvecs ---- */
enum {
  BF_OP_N = 0, /* y = beta*y + alpha*A*x            (matrixvector.jl:8-65)        */
  BF_OP_C = 1, /* y = beta*y + alpha*A'*x (adjoint) (matrix_adj_tr.jl:8-25)       */
  BF_OP_T = 2  /* y = beta*y + alpha*transpose(A)*x (matrix_adj_tr.jl:28-40)      */
};

/* ---- pointer-location flags for matvecs ---- */
enum {
  BF_PTR_HOST = 0,  /* x, y are host pointers: copies happen inside the call */
  BF_PTR_DEVICE = 1 /* x, y are device pointers: the call is stream-ordered  */
};

typedef struct bf_context* bf_ctx_t;
typedef struct bf_tree* bf_tree_t;
typedef struct bf_operator* bf_op_t;
typedef struct bf_batch* bf_batch_t;

BF_API int bf_version(void);
BF_API const char* bf_status_string(int status);
BF_API const char* bf_last_error(void);

/* Create / destroy a device context (one CUDA device). */
BF_API int bf_ctx_create(int device, bf_ctx_t* out);
BF_API int bf_ctx_destroy(bf_ctx_t ctx);

/* ------------------------------------------------------------------------
 * Cluster trees (caller-side utility).
 * A 2^3 tree on the bounding cube of the points: a node is a leaf when it
 * holds <= max_points points (max_points > 0), or sits at depth max_depth
 * (max_depth >= 0, root depth 0), or holds one point.  Stands in for the
 * H2Trees.TwoNTree the reference clusters with (ext/BFH2Trees/BFH2Trees.jl),
 * exposing the tree contract of src/treeinterface.jl:39-164 as arrays.
 * values(node) = perm[begin[node] .. end[node]-1].
 * ------------------------------------------------------------------------ */
BF_API int bf_tree_build(const double* xyz, int64_t n_points, int32_t max_points,
                         int32_t max_depth, bf_tree_t* out);
BF_API int bf_tree_from_arrays(int64_t n_nodes, int64_t n_points, const double* center,
                               const double* halfsize, const int32_t* parent,
                               const int32_t* first_child, const int32_t* n_child,
                               const int64_t* begin, const int64_t* end, const int64_t* perm,
                               bf_tree_t* out);
BF_API int bf_tree_size(bf_tree_t tree, int64_t* n_nodes, int64_t* n_points, int32_t* depth);
BF_API int bf_tree_export(bf_tree_t tree, double* center, double* halfsize, int32_t* level,
                          int32_t* parent, int32_t* first_child, int32_t* n_child,
                          int64_t* begin, int64_t* end, int64_t* perm);
BF_API int bf_tree_destroy(bf_tree_t tree);

/* Near/far interaction lists: src/Matrixassembly/intlists.jl:30-217 with the
 * AABB isFarFunctor(alpha) of ext/BFH2Trees/h2admissible.jl:11-45; options as
 * the reference's nearandfar (minbflvl, leafcomp, leafimbalance, and
 * unbalancedints: only the larger node of a pair splits, intlists.jl:121-149).
 * Call with capacity 0 to query *n_far; pairs are written as
 * (far_obs[i], far_src[i]) in the reference's depth-first order. */
BF_API int bf_nearandfar(bf_tree_t obs_tree, bf_tree_t src_tree, double alpha,
                         int32_t minbflvl, int32_t leafcomp, int32_t leafimbalance,
                         int32_t unbalancedints, int64_t* far_obs, int64_t* far_src, int64_t capacity,
                         int64_t* n_far, int64_t* n_near);

/* The same tree and interaction lists, built on the GPU (the reference builds
 * its trees in H2Trees, ext/BFH2Trees/bisection_tree.jl:27-145, and its lists
 * in intlists.jl:30-217, on the host).  bf_tree_build_gpu returns a tree
 * identical, node for node and point for point, to bf_tree_build's: the device
 * partitions the points level by level, the host numbers the nodes.
 * bf_nearandfar_gpu returns the far and near pairs of bf_nearandfar /
 * bf_near_pairs in the same depth-first order (level-synchronous traversal on
 * the device, outputs placed by their depth-first keys); capacities 0 query
 * *n_far / *n_near.  Traversals deeper than 21 levels return BF_ENOTSUP. */
BF_API int bf_tree_build_gpu(bf_ctx_t ctx, const double* xyz, int64_t n_points,
                             int32_t max_points, int32_t max_depth, bf_tree_t* out);
BF_API int bf_nearandfar_gpu(bf_ctx_t ctx, bf_tree_t obs_tree, bf_tree_t src_tree, double alpha,
                             int32_t minbflvl, int32_t leafcomp, int32_t leafimbalance,
                             int32_t unbalancedints, int64_t* far_obs, int64_t* far_src, int64_t far_capacity,
                             int64_t* near_obs, int64_t* near_src, int64_t near_capacity,
                             int64_t* n_far, int64_t* n_near);

/* Near pairs of the same traversal (the nearints of intlists.jl:30-217):
 * (near_obs[i], near_src[i]) in depth-first order; capacity 0 queries *n_near. */
BF_API int bf_near_pairs(bf_tree_t obs_tree, bf_tree_t src_tree, double alpha,
                         int32_t minbflvl, int32_t leafcomp, int32_t leafimbalance,
                         int32_t unbalancedints, int64_t* near_obs, int64_t* near_src, int64_t capacity,
                         int64_t* n_near);

/* ------------------------------------------------------------------------
 * Construction on the GPU.
 * Replaces assemble_BF (src/ButterflyFactorization/bfassembly.jl:48-200),
 * called once per far pair by PetrovGalerkinBF
 * (src/Matrixassembly/petrovgalerkinbf.jl:129-151), with the PartialQR
 * compressor (src/ButterflyFactorization/compressors.jl:81-165) and the
 * ButterflyRankEstimator (src/ButterflyFactorization/rankestimation.jl:93-98).
 * All far pairs of one operator are built level by level in batched launches
 * on the point Helmholtz kernel G(r) = exp(-i k r) / (4 pi r).
 * ------------------------------------------------------------------------ */
typedef struct {
  double c_tau;          /* rank-estimator constant Ctau (reference default 4.0;
                            PetrovGalerkinBF with isFar uses 2.9592)              */
  int32_t min_samples;   /* lower bound on sampled rows (reference: 10)           */
  int32_t adaptive;      /* 1 = double the sample while r > floor(0.8 rows)      */
  uint64_t seed;         /* keys the observer-row sampling                        */
  int32_t rank_mode;     /* 0 = oversampling estimator; 1 = learned surrogate      */
  int32_t keep_mixed;    /* 1 = also keep complex-FP32 factors for bf_matvec_mixed */
  const float* surrogate_weights; /* MLP weights when rank_mode == 1 (else NULL)   */
  int64_t surrogate_nweights;
  double surrogate_margin; /* log-rank safety margin of surrogate-seeded sample
                              counts: rows = ceil(exp(pred + margin) / 0.8) + 2 */
  int32_t factor_storage;  /* BF_STORE_C32 (default): complex FP32 entries, 8 B,
                              exact for the build's FP32 values; BF_STORE_FF:
                              float-float entries, 16 B, the FP64-width layout
                              that ComplexF64 factors (the reference's acctype,
                              bfassembly.jl:61) import into                     */
  int32_t estimator;     /* rank estimator of the sample counts:
                            BF_EST_BUTTERFLY (default): ButterflyRankEstimator(c_tau),
                            max(ceil(c_tau log(1/eps)), 10), rankestimation.jl:93-98;
                            BF_EST_GEOMETRIC: GeometricRankEstimator(geo_c, geo_ceps;
                            Rmin=geo_rmin), max(ceil(C (k a_s a_o / d)^2 + Ceps log(1/eps)),
                            Rmin) with the node radii a and the center distance d
                            (rankestimation.jl:13-25, ext/BFH2Trees/h2rankest.jl:8-38)   */
  int32_t geo_rmin;      /* default 3                                              */
  double geo_c;          /* default 1.5                                            */
  double geo_ceps;       /* default 1.5                                            */
} bf_build_opts;

enum { BF_EST_BUTTERFLY = 0, BF_EST_GEOMETRIC = 1 };

/* ---- factor storage of GPU-built operators (bf_build_opts.factor_storage) ---- */
enum {
  BF_STORE_C32 = 0,
  BF_STORE_FF = 1
};

BF_API void bf_build_opts_default(bf_build_opts* opts);

BF_API int bf_build(bf_ctx_t ctx, const double* obs_xyz, int64_t n_obs, const double* src_xyz,
                    int64_t n_src, bf_tree_t obs_tree, bf_tree_t src_tree,
                    const int64_t* far_obs, const int64_t* far_src, int64_t n_far, double k,
                    double tol, const bf_build_opts* opts, bf_op_t* out);

/* Near field of the operator: the near blocks K(values(o), values(s)) of the
 * given near pairs (PetrovGalerkinBF's BlockSparseMatrix,
 * src/Matrixassembly/petrovgalerkinbf.jl:57-119), evaluated on the GPU in FP64
 * for the point Helmholtz kernel (the singular self-term r = 0 is left out:
 * those entries are zero) and stored as float-float entries, once per
 * direction.  Afterwards bf_matvec and bf_matvec_noalloc apply near + far in
 * one device pass (src/matrixalgebra/matrixvector.jl:28-33), forward, adjoint
 * and transpose.  The point sets and trees are the ones the far field was
 * built with. */
BF_API int bf_op_add_near(bf_op_t op, const double* obs_xyz, int64_t n_obs,
                          const double* src_xyz, int64_t n_src, bf_tree_t obs_tree,
                          bf_tree_t src_tree, const int64_t* near_obs, const int64_t* near_src,
                          int64_t n_near, double k);

/* One compression of the GPU build, for parity tests: one call of the
 * PartialQR compressor (src/ButterflyFactorization/compressors.jl:81-165,
 * without the adaptive re-sampling of :134-151) on the device launches
 * bf_build uses.  Rows: n_rows observer points sampled from obs_index (n_obs
 * points) by the keyed bijection that stands in for the reference's
 * randperm (compressors.jl:101), written to rows_out[n_rows] (optional).
 * Z_out (optional, complex64 n_rows x n_src, column-major): the sampled
 * kernel block G(obs[rows[i]], src[src_index[j]]).  Then the pivoted QR with
 * rtol eps (compressors.jl:128-131): *rank_out; perm_out[n_src] the column
 * pivot order (positions into src_index); skeleton_out[rank] =
 * src_index[perm[0..rank)] (compressors.jl:162); T_out (complex64, rank x
 * n_src, column-major, capacity min(n_rows, n_src) * n_src) the
 * interpolation matrix R11^-1 Q1^H Z (compressors.jl:155-160).  Host
 * pointers; synchronous. */
BF_API int bf_compress_block(bf_ctx_t ctx, const double* obs_xyz, int64_t n_obs_pts,
                             const double* src_xyz, int64_t n_src_pts, const int64_t* obs_index,
                             int32_t n_obs, const int64_t* src_index, int32_t n_src,
                             int32_t n_rows, uint64_t key, double k, double eps,
                             int32_t* rows_out, float* Z_out, int32_t* rank_out,
                             int32_t* perm_out, int32_t* skeleton_out, float* T_out);

/* ------------------------------------------------------------------------
 * Learned rank surrogate (no reference counterpart; it replaces the fixed
 * ButterflyRankEstimator sample count, rankestimation.jl:93-98, whose
 * under-estimates cost the adaptive re-sampling of compressors.jl:134-151).
 * A 4 -> 64 -> 64 -> 1 MLP (tanh-form GELU; FP32 master weights rounded to
 * BF16 in every evaluation, FP32 accumulation) maps the features of a
 * compression (columns 14..17 of a rank record) to log(rank).  Weight vector:
 * bf_surrogate_nweights() floats (normalisation mu[4], sigma[4], W1[64][4],
 * b1[64], W2[64][64], b2[64], w3[64], b3).  All buffers are host memory. */
typedef struct {
  int32_t epochs;  /* passes over the records                          */
  int32_t batch;   /* samples per Adam step                            */
  float lr;        /* Adam step size                                   */
  float beta1, beta2, eps;
  uint64_t seed;   /* shuffling seed                                   */
} bf_train_opts;

BF_API void bf_train_opts_default(bf_train_opts* opts);
BF_API int bf_surrogate_nweights(void);
/* normalisation from the features (n x 4), Glorot-uniform layers from seed */
BF_API int bf_surrogate_init(const float* features, int64_t n, uint64_t seed, float* weights);
/* mean 0.5 (y - target)^2 over the n samples and its gradient (GPU kernels) */
BF_API int bf_surrogate_grad(bf_ctx_t ctx, const float* weights, const float* features,
                             const float* targets, int64_t n, float* grad, float* loss);
/* Adam training on the GPU; weights in: initial, out: trained; optional
 * loss_per_epoch[epochs] (mean batch loss of each epoch) */
BF_API int bf_surrogate_train(bf_ctx_t ctx, const float* features, const float* targets,
                              int64_t n, const bf_train_opts* opts, float* weights,
                              float* loss_per_epoch);
/* predicted log(rank) of n feature rows (GPU kernel) */
BF_API int bf_surrogate_predict(bf_ctx_t ctx, const float* weights, const float* features,
                                int64_t n, float* out);

/* ------------------------------------------------------------------------
 * Import of factors built elsewhere (the parity path): a set of
 * ButterflyFactorization objects (src/ButterflyFactorization/bfstructs.jl:21-146)
 * described block by block.  stage = 0 for Q blocks, l (1-based) for blocks of
 * R level l, -1 for P blocks.  Keys are the reference routing keys
 * (obs_out, src_out, obs_in, src_in).  Block data are ComplexF64, column-major
 * rows x cols, starting at data + 2*data_off[b].  identity[b] != 0 marks a
 * UniformScaling block (rows/cols/data ignored).  The node->values maps of the
 * observer (test) and source (trial) trees are CSR arrays: values(node) =
 * idx[ptr[node] .. ptr[node+1]-1] (0-based point indices).
 * ------------------------------------------------------------------------ */
typedef struct {
  int64_t n_rows, n_cols;
  int64_t n_blocks;
  const int32_t* bf;
  const int32_t* stage;
  const int64_t* obs_out;
  const int64_t* src_out;
  const int64_t* obs_in;
  const int64_t* src_in;
  const int32_t* rows;
  const int32_t* cols;
  const int8_t* identity;
  const int64_t* data_off;
  const double* data;
  int64_t n_obs_nodes;
  const int64_t* obs_ptr;
  const int64_t* obs_idx;
  int64_t n_src_nodes;
  const int64_t* src_ptr;
  const int64_t* src_idx;
} bf_factor_desc;

BF_API int bf_import_factors(bf_ctx_t ctx, const bf_factor_desc* desc, bf_op_t* out);

/* ------------------------------------------------------------------------
 * Matvec, FP64-accurate: Y = beta*Y + alpha*op(A)*X over all far blocks.
 * Replaces mul!(y, A::PetrovGalerkinBF, x, alpha, beta) far part
 * (src/matrixalgebra/matrixvector.jl:8-65), the per-block flat mul!
 * (src/Butterflyalgebra/bfvector.jl:200-296) and the multi-RHS column loop
 * (src/Butterflyalgebra/bfmatrix.jl:10-75).  adjoint/transpose reuse the
 * forward factors (no copy; cf. src/Butterflyalgebra/bfadjtr.jl:43-67).
 * x, y: complex (re,im) doubles; alpha, beta: complex scalars as double[2].
 * stream: a cudaStream_t, or NULL for the handle's own stream.
 * Forward calls with nrhs >= 8 on an operator without a near field run whole
 * chunks of 8 columns through a one-operator batch (each factor entry loaded
 * serves up to 4 columns); its buffers (8 workspaces, 8 columns of x and y)
 * are allocated at the first such call and kept with the handle.  If they do
 * not fit, the columns run one by one.
 * ------------------------------------------------------------------------ */
BF_API int bf_matvec(bf_op_t op, int trans, int64_t nrhs, const double* x, int64_t ldx,
                     double* y, int64_t ldy, const double* alpha, const double* beta,
                     int ptr_mode, void* stream);

/* Errors of asynchronous matvecs (no reference counterpart: a Julia mul!
 * raises at the call).  A device-pointer bf_matvec or bf_matvec_noalloc
 * returns before its kernels have run; when one of its bounded device-side
 * waits gives up (BF_ETIMEOUT, the output is then invalid), the library notes
 * it in host memory.  bf_op_check synchronises `stream` (NULL: the handle's
 * own stream) and returns BF_ETIMEOUT if such a timeout happened since the
 * last check, else BF_OK; the next matvec call on the handle also reports it
 * (and then does no work).  Host-pointer calls report their own timeout. */
BF_API int bf_op_check(bf_op_t op, void* stream);

/* Test hook of the timeout path (no reference counterpart): the number of
 * polls a bounded wait of this operator's plain-path bulk-copy kernel makes
 * before it gives up.  polls < 0 restores the default (about one second of
 * polling); 0 makes every such wait give up at once. */
BF_API int bf_op_set_wait_limit(bf_op_t op, int64_t polls);

/* Allocation-free FP64-accurate matvec on device pointers.  No counterpart in
 * the reference (the Julia package always allocates through its workspaces).
 * For callers that cannot allocate device memory when they apply the
 * operator: a callback running while the caller's memory pool is locked or
 * exhausted (a solver inside an application that owns all device memory), a
 * real-time loop with a fixed allocation budget.  Same arguments as bf_matvec
 * with ptr_mode = BF_PTR_DEVICE.  The level workspace is one file-scope
 * device array of 16 MiB (1,048,576 complex entries) that every GPU loading
 * the library holds until the process exits; operators whose workspace
 * (bf_op_stats.workspace_entries) is larger are rejected with BF_EINVAL.
 * The first call on a device looks up the array's device address (and the
 * driver may load kernel code), so make that first call before any stream
 * capture.  All calls share the array and it keeps the last call's
 * contents: calls that overlap on the GPU (for example, issued on two
 * streams) race with each other; serialise them.  The call is asynchronous:
 * a device-side timeout is reported by bf_op_check or the next call. */
BF_API int bf_matvec_noalloc(bf_op_t op, int trans, int64_t nrhs, const double* x, int64_t ldx,
                             double* y, int64_t ldy, const double* alpha, const double* beta,
                             void* stream);

/* Many-RHS mixed precision (the column loop of src/Butterflyalgebra/
 * bfmatrix.jl:10-75 as one dense contraction per level): factors rounded to
 * complex FP32 and split into BF16 hi/lo, contracted against 128 right-hand
 * sides at a time in three tensor-core passes with FP32 accumulation.  Same
 * arguments and semantics as bf_matvec (y <- alpha*op(A)*x + beta*y); relative
 * error ~1e-5 instead of ~1e-14.  The first call packs the BF16 factors and
 * allocates a workspace of 1 KB per level slot. */
BF_API int bf_matvec_mixed(bf_op_t op, int trans, int64_t nrhs, const double* x, int64_t ldx,
                           double* y, int64_t ldy, const double* alpha, const double* beta,
                           int ptr_mode, void* stream);

/* size(A) (src/matrixalgebra/dims.jl:13-20). */
BF_API int bf_op_size(bf_op_t op, int64_t* n_rows, int64_t* n_cols);

typedef struct {
  int64_t n_bf;              /* far blocks (butterflies)                        */
  int64_t n_stages;          /* launches of the level sequence (Q, R..., P)     */
  int64_t n_tasks;           /* dense + copy tasks over all stages              */
  int64_t factor_entries;    /* stored complex entries (incl. stacking zeros)   */
  int64_t factor_bytes;      /* bytes of the FP64-accurate factor array         */
  int64_t workspace_entries; /* complex entries of the level vectors            */
  int64_t map_entries;       /* int32 row/column routing entries                */
  int64_t alg_bytes_fwd;     /* algorithmic bytes of one 1-RHS matvec           */
  int64_t max_rank;          /* largest block row count                         */
  double build_seconds;      /* wall time of bf_build (0 for imports)           */
  int64_t compressions;      /* partial-QR compressions performed               */
  int64_t retries;           /* adaptive re-samplings                           */
  int64_t kernel_entries;    /* Helmholtz entries evaluated during the build    */
  double build_compress_seconds; /* of build_seconds: compression rounds (task
                                    arrays, GPU sampling + QR + solve, waits)     */
  double build_pack_seconds;     /* of build_seconds: level/task packing (host)   */
  double build_upload_seconds;   /* of build_seconds: factor repack + upload      */
  int64_t surrogate_fallbacks;   /* surrogate-seeded compressions that fell back
                                    to the oversampling estimator                 */
  int64_t near_pairs;            /* near-field blocks (0: far field only)           */
  int64_t near_entries;          /* stored near-field entries, both directions      */
  int64_t near_bytes_fwd;        /* algorithmic bytes of one forward near product   */
} bf_op_stats;

BF_API int bf_op_stats_get(bf_op_t op, bf_op_stats* stats);

/* Copy back the factors of far blocks bf_begin <= bf < bf_end as the
 * reference block list (same layout as bf_factor_desc; data_off counts complex
 * entries from the first exported block).  Call with data == NULL to query
 * n_blocks and n_data.  as_float32 != 0 writes complex64 (pairs of float) into
 * data, which is exact for factors built by bf_build. */
BF_API int bf_op_export_blocks(bf_op_t op, int64_t bf_begin, int64_t bf_end, int64_t* n_blocks,
                               int64_t* n_data, int32_t* bf, int32_t* stage, int64_t* obs_out,
                               int64_t* src_out, int64_t* obs_in, int64_t* src_in,
                               int32_t* rows, int32_t* cols, int8_t* identity, int64_t* data_off,
                               void* data, int32_t as_float32);

/* Rank records of the build, one per compression (the richer form of the
 * reference RankLogger, src/ButterflyFactorization/bfstructs.jl:220-232 and
 * compressors.jl:153): BF_RANK_REC_LEN values per record in
 * rec[BF_RANK_REC_LEN*i ...]:
 * bf, stage, obs_node, src_node, n_obs, n_cols, rows_initial, rows_final,
 * retries, rank, radius_obs, radius_src, center_distance, k, then the four
 * rank-surrogate features: level, k * box diameter, separation / diameter,
 * log(1 + min(observer points, compressed columns)).
 * Call with rec == NULL to query *n_rec. */
#define BF_RANK_REC_LEN 18
BF_API int bf_op_rank_log(bf_op_t op, int64_t* n_rec, double* rec);

/* Device time of each level launch of one matvec (CUDA events on the handle's
 * stream, mean over nrep passes) and the algorithmic bytes each launch moves
 * (factor entries + vector entries read and written, 16 B per complex
 * entry).  Arrays have n_stages entries (bf_op_stats.n_stages). */
BF_API int bf_op_profile(bf_op_t op, int trans, int32_t nrep, double* ms_per_stage,
                         int64_t* bytes_per_stage, int64_t* kernels_per_matvec);

/* Per-level device time of the mixed path for one chunk of 128 right-hand
 * sides, with the bytes each level moves (BF16 factor blocks + FP32 slots read
 * and written) and its useful flops (8 per complex multiply-add and RHS).
 * No reference counterpart (measurement hook). */
BF_API int bf_op_profile_mixed(bf_op_t op, int trans, int32_t nrep, double* ms_per_stage,
                               int64_t* bytes_per_stage, double* flops_per_stage,
                               int64_t* kernels_per_chunk);

/* Memory of the mixed path: BF16 factor bytes, workspace bytes, work units
 * (both directions).  Packs the mixed factors if not done yet. */
BF_API int bf_op_mixed_info(bf_op_t op, int64_t* factor_bytes, int64_t* workspace_bytes,
                            int64_t* work_units);

/* Shapes of the packed level tasks (stage index, kind 0 = dense / 1 = copy,
 * rows M, columns n), in launch order.  Call with stage == NULL to query
 * *n_tasks.  Used by the tile autotuner and by diagnostics. */
BF_API int bf_op_task_shapes(bf_op_t op, int64_t* n_tasks, int32_t* stage, int32_t* kind,
                             int32_t* M, int32_t* n);

/* Butterfly recompression: recompress_BF(BF, tau) of every far block
 * (src/Butterflyalgebra/algrecomp.jl:19-148): the right pass (R levels from the
 * last to the second, blocks sharing a column space stacked and compressed by
 * pivoted QR at rtol tau, the transfer matrix moved into the previous level)
 * and the left pass (the same on the adjoint).  The stacks of a level are
 * compressed in one batched launch of the build's pivoted-QR kernel (FP32
 * Householder, FP64 norms and pivots); Q = A[:, p[1:r]] R11^-1 replaces the
 * blocks and R[:, invperm(p)] moves into the neighbouring level.  Groups
 * holding identity blocks are left as they are.  Arithmetic is FP32 (tau
 * below about 1e-6 gains nothing).  Returns a new operator with the storage
 * of the input (float-float entries with zero low parts when the input was
 * float-float); the input is unchanged.  Operators with a near field are
 * refused (BF_ENOTSUP). */
BF_API int bf_op_recompress(bf_op_t op, double tau, bf_op_t* out);

/* Materialised adjoint (trans = BF_OP_C) or transpose (BF_OP_T): a new
 * operator whose forward matvec is op(A) x, as the reference's adjoint(BF) /
 * transpose(BF) (src/Butterflyalgebra/bfadjtr.jl:13-67) build one: blocks
 * conjugate-transposed (transposed) with swapped routing keys, R levels
 * reversed, Q and P exchanged, the trees swapped.  The factor storage is kept.
 * bf_matvec's BF_OP_C / BF_OP_T views need no copy; the copy runs at the
 * forward kernels' speed for twice the factor memory.  Operators with a near
 * field are refused (BF_ENOTSUP). */
BF_API int bf_op_adjoint_copy(bf_op_t op, int trans, bf_op_t* out);

/* Persisted operators (no reference counterpart: the reference keeps its
 * factors in memory only and rebuilds them with every assemble_BF,
 * src/ButterflyFactorization/bfassembly.jl:48-200).  bf_op_save writes the
 * operator in its packed, device-ready form (level tasks, routing maps,
 * launch lists, leaf orders, the factor array in its storage, the block list
 * for bf_op_export_blocks, statistics and rank records) with a format version,
 * a byte-order mark and 64-bit hashes.  bf_op_load reads such a file onto the
 * device of ctx without rebuilding: it rejects a wrong magic or truncated /
 * corrupted file with BF_EINVAL and another format version or byte order with
 * BF_ENOTSUP, and checks every offset a kernel will follow before upload. */
BF_API int bf_op_save(bf_op_t op, const char* path);
BF_API int bf_op_load(bf_ctx_t ctx, const char* path, bf_op_t* out);

BF_API int bf_op_destroy(bf_op_t op);

/* ------------------------------------------------------------------------
 * Batches: many independent operators, each with its own number of right-hand
 * sides and its own direction, applied by one launch sequence (no reference
 * counterpart: the reference runs each mul! and each column separately,
 * bfmatrix.jl:10-75, and materialises every adjoint, bfadjtr.jl:43-67).
 * FP64-accurate, y_i = op_i(A_i) x_i for every operator i and column, with
 * op_i = BF_OP_N, BF_OP_C (adjoint, matrix_adj_tr.jl:8-25) or BF_OP_T
 * (transpose, matrix_adj_tr.jl:28-40).  The level sequences are merged (one
 * persistent launch per level and task class for all operators; adjoints walk
 * their levels backwards) and captured once as a CUDA graph; right-hand sides
 * run in chunks of rhs_chunk (default 8), and the forward routines apply every
 * factor entry they load to up to four right-hand sides of a chunk.  All
 * operators must have the same factor storage (all complex FP32, or all
 * float-float).  The operators must outlive the batch. */
BF_API int bf_batch_create_op(bf_ctx_t ctx, bf_op_t const* ops, const int32_t* trans,
                              const int32_t* nrhs, int32_t n_ops, int32_t rhs_chunk,
                              bf_batch_t* out);
/* bf_batch_create_op with every operator forward (trans == NULL). */
BF_API int bf_batch_create(bf_ctx_t ctx, bf_op_t const* ops, const int32_t* nrhs,
                           int32_t n_ops, int32_t rhs_chunk, bf_batch_t* out);
/* Device buffers of operator i: x (n_in x nrhs) and y (n_out x nrhs), complex
 * double, column-major, leading dimension = size (n_in = columns of op_i(A_i),
 * n_out = its rows).  bf_batch_run reads every x buffer and writes every y. */
BF_API int bf_batch_buffers(bf_batch_t b, int32_t op, double** x_dev, double** y_dev);
/* one graph launch on stream (NULL: the batch's own stream, synchronised) */
BF_API int bf_batch_run(bf_batch_t b, void* stream);
/* copies x[i] (ldx[i] >= n_in_i; NULL ldx: packed) in, runs, copies y[i] out;
 * ptr_mode BF_PTR_HOST or BF_PTR_DEVICE */
BF_API int bf_batch_matvec(bf_batch_t b, const double* const* x, const int64_t* ldx,
                           double* const* y, const int64_t* ldy, int ptr_mode, void* stream);
/* Autotuner: times nrep graph replays for every candidate of (right-hand sides
 * per factor load in the forward routines: 1 or 4; item order: longest first
 * or operator/task order; 2, 4 or 6 persistent CTAs per SM), keeps the
 * fastest.  best_cfg[3] = {nr_max, order, ctas_per_sm}. */
BF_API int bf_batch_autotune(bf_batch_t b, int32_t nrep, double* best_ms, int32_t* best_cfg);
BF_API int bf_batch_info(bf_batch_t b, int64_t* graph_nodes, int64_t* work_items,
                         int64_t* workspace_bytes, int32_t* rhs_chunks);
BF_API int bf_batch_destroy(bf_batch_t b);

#ifdef __cplusplus
}
#endif

#endif /* BFGPU_H */
