/*
 * bioshell_crmsd.h -- C ABI of the GB300-native all-vs-all crmsd engine.
 *
 * This is the drop-in boundary for the crmsd path of bioshell-pdb.  The
 * reference (BioShell 4.0.0-dev, Rust) has no crmsd routine yet -- the only
 * trace is the dependency comment at bioshell-pdb/Cargo.toml:27 -- so the
 * entry points below are the ones the crate's calc module would bind through
 * an `extern "C"` block built from build.rs.  Each declaration names the
 * reference interface it serves:
 *
 *   crmsd of one pair            -> bioshell-pdb/src/calc/mod.rs:1-10 (new fn
 *                                   beside SubstructureAxis::from_3d_points,
 *                                   calc/substructures.rs:17, same
 *                                   `&[T: HasCartesians]` inputs,
 *                                   bioshell-core/src/has_cartesians.rs:6-8)
 *   all-vs-all distance matrix   -> fills the matrix that
 *                                   HierarchicalClusteringMatrix::new builds
 *                                   from n(n-1)/2 closure calls
 *                                   (bioshell-clustering/src/hierarchical/
 *                                   clustering_matrix.rs:11-22)
 *   batched all-vs-all           -> one such matrix per decoy set, for the
 *                                   per-set clustering loop of a caller
 *                                   (OPTICS over each set, optics.rs:51-58)
 *
 * Conventions
 *   - Coordinates are f64 AoS xyz triples, `[n][L][3]`, the layout of
 *     bioshell_core::Vec3 (bioshell-core/src/vec3.rs:44-51); every atom has
 *     the same weight and each structure is centred on its arithmetic mean.
 *   - Pointers may be host memory (pageable or pinned) or device memory of
 *     the context's GPU; the library detects which.
 *   - The caller owns inputs and outputs; the context owns device workspaces.
 *   - Every call returns a bs_status; 0 is success.  No C++ exception and no
 *     abort crosses this boundary.  bs_last_error() describes the last
 *     failure of a context.
 *   - A context is used by one host thread at a time.  All work runs on the
 *     context's CUDA stream; calls return after their results are in `out`.
 *   - No CPU fallback exists: without a usable sm_103 GPU every compute call
 *     fails with BS_ERR_NO_DEVICE.
 */
#ifndef BIOSHELL_CRMSD_H
#define BIOSHELL_CRMSD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BS_API __attribute__((visibility("default")))

#define BS_ABI_VERSION 3
#define BS_OPTS_VERSION 1

typedef int32_t bs_status;
enum {
  BS_OK = 0,
  BS_ERR_INVALID_ARG = 1,  /* null pointer, n < 0, L < 1, bad option value  */
  BS_ERR_CUDA = 2,         /* a CUDA runtime/driver call failed              */
  BS_ERR_OOM = 3,          /* device or pinned allocation failed             */
  BS_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up             */
  BS_ERR_UNSUPPORTED = 5,  /* shape outside what this path supports          */
  BS_ERR_NONFINITE = 6,    /* NaN or Inf in the input coordinates            */
  BS_ERR_BUDGET = 7,       /* request exceeds the context's HBM budget       */
  BS_ERR_NO_DEVICE = 8,    /* no usable GPU (or not an sm_103 device)        */
  BS_ERR_INTERNAL = 9,     /* invariant violated inside the library          */
  BS_ERR_CANCELLED = 10    /* the request was cancelled before it ran        */
};

typedef struct bs_ctx bs_ctx;

/* Arithmetic of the all-vs-all fill. */
enum {
  /* FP64 centring, FP64 CUDA-core covariance, FP64 QCP: the plain method. */
  BS_PRECISION_PLAIN64 = 0,
  /* Exact fixed-point digits on tcgen05 tensor cores + FP32/integer QCP with
   * an exact Rayleigh-quotient cancellation step; pairs whose error bound is
   * not below the tolerance are recomputed with exact integer covariances. */
  BS_PRECISION_MIXED = 1
};

/* Layout of the result buffer. */
enum {
  BS_LAYOUT_TRIANGLE = 0, /* n(n-1)/2 values, row-major upper triangle:
                             index(i,j) = i*n - i*(i+1)/2 + (j-i-1), i<j   */
  BS_LAYOUT_SQUARE = 1    /* n*n values, symmetric, zero diagonal          */
};

/* Element type of the result buffer. */
enum { BS_OUT_F64 = 0, BS_OUT_F32 = 1 };

typedef struct {
  uint32_t version;   /* must be BS_OPTS_VERSION (bs_opts_init sets it)   */
  int32_t precision;  /* BS_PRECISION_*                                    */
  int32_t layout;     /* BS_LAYOUT_*                                       */
  int32_t out_type;   /* BS_OUT_*                                          */
  double tolerance;   /* mixed path: certified per-pair |dRMSD| bound in
                         Angstrom against exact arithmetic on the input
                         coordinates (grid quantisation + fast-path
                         arithmetic); pairs whose fast-path bound does not
                         meet it are recomputed exactly.  <= 0 selects the
                         default, 1e-4                                    */
  int32_t flags;      /* BS_FLAG_* bits                                    */
  int32_t flag_queue; /* mixed path: capacity of the queue of pairs to
                         recompute exactly; <= 0 selects the default,
                         min(2^24, pairs).  Pairs flagged beyond it are
                         found by a scan of the result for their sentinel  */
  int32_t row_begin;  /* bs_all_vs_all, mixed path, packed triangle: only
                         the pairs (i, j) with row_begin <= i < row_end are
                         computed and written; the rest of `out` (which
                         keeps its full n(n-1)/2 size) is left untouched.
                         row_begin a multiple of 40; row_end a multiple of
                         40 or n; both 0 = every row.  The partition of one
                         all-vs-all over several GPUs (bs_partition_rows)  */
  int32_t row_end;
  int32_t reserved[4];
} bs_opts;

/* bs_opts.flags */
enum {
  /* Launch the mixed-path kernels one by one instead of replaying a CUDA
   * graph captured for the call's shape (a graph is captured the first time
   * a shape is seen and replayed for every later call of that shape). */
  BS_FLAG_NO_GRAPH = 1,
  /* Mixed path: pick each structure set's tile shape (40 x 20 structures,
   * or 40 x 10, which wastes fewer pair slots on small sets but costs twice
   * the tensor-core instructions per pair) by timing both on a synthetic set
   * of the same chain-length and size class the first time the class is
   * seen on the context; the choice is cached for later calls. */
  BS_FLAG_AUTOTUNE = 2
};

/* Per-call counters of the last compute call on a context. */
typedef struct {
  int64_t pairs;           /* pairs written                                  */
  int64_t pairs_refined;   /* mixed path: pairs recomputed exactly           */
  double ms_total;         /* device time of the whole call (CUDA events)    */
  double ms_h2d;           /* host -> device copy of the coordinates         */
  double ms_prep;          /* centring / quantisation pass                   */
  double ms_main;          /* covariance + QCP kernel                        */
  double ms_refine;        /* exact recomputation of flagged pairs           */
  double ms_d2h;           /* device -> host copy of the result              */
  int32_t scale_exp;       /* mixed path: coordinate grid is 2^scale_exp A
                              (of the first structure set)                   */
  int32_t main_launches;   /* kernels launched by the call                   */
  int32_t jobs;            /* structure sets (or query blocks) in the call   */
  int32_t graph;           /* 0 direct launches, 1 graph captured and run,
                              2 captured graph replayed                      */
  double quant_bound;      /* mixed path: worst RMSD change from the grid    */
  int64_t bytes_h2d;
  int64_t bytes_d2h;
  int32_t narrow_jobs;     /* structure sets run with 40 x 10 tiles          */
  int32_t tuned_classes;   /* shape classes the autotuner timed in this call */
  int64_t pairs_plain;     /* mixed path: pairs of structure sets that no
                              coordinate grid fits (chains beyond ~3,000
                              atoms, coordinates beyond +-32768 A), computed
                              on the plain FP64 GPU path instead            */
} bs_metrics;

/* ---- version / errors -------------------------------------------------- */
BS_API int32_t bs_abi_version(void);
BS_API const char *bs_status_string(bs_status s);
/* Last error message of `ctx` (never NULL; "" when none). */
BS_API const char *bs_last_error(const bs_ctx *ctx);

/* ---- context ----------------------------------------------------------- */
/* Creates a context on CUDA device `device`.  `hbm_budget_bytes` caps the
 * device workspace the context may hold (0 = 90% of free memory). */
BS_API bs_status bs_ctx_create(bs_ctx **out, int32_t device, size_t hbm_budget_bytes);
BS_API void bs_ctx_destroy(bs_ctx *ctx);
BS_API void bs_opts_init(bs_opts *opts);
BS_API bs_status bs_get_metrics(const bs_ctx *ctx, bs_metrics *out);
/* Releases cached device workspaces (they regrow on demand). */
BS_API bs_status bs_ctx_trim(bs_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), so callers can order or time
 * their own work against the engine's. */
BS_API void *bs_ctx_stream(const bs_ctx *ctx);

/* ---- crmsd ------------------------------------------------------------- */
/* crmsd of one pair of index-matched point sets a[L][3], b[L][3]
 * (new bioshell_pdb::calc::crmsd; runs on the GPU as a batch of one). */
BS_API bs_status bs_crmsd(bs_ctx *ctx, const double *a, const double *b, int32_t L, double *out_rmsd);

/* ---- superposition ---------------------------------------------------- */
/* The optimal superposition of b onto a as a rototranslation: the proper
 * rotation rot[9] (3x3, row-major) and translation trans[3] with
 * rot * b_k + trans ~ a_k in the least-squares sense -- the rotation and
 * translation a bioshell_pdb::calc::Rototranslation carries
 * (transformation.rs:22-37; applied as R v + t by apply_mut, :171-174).
 * rmsd (may be NULL) receives the RMSD of that superposition, which is the
 * crmsd of the pair.  FP64 on the raw coordinates (QCP key matrix, Jacobi
 * eigenvector); pointers may be host or device memory. */
BS_API bs_status bs_superpose(bs_ctx *ctx, const double *a, const double *b, int32_t L, double *rot,
                              double *trans, double *rmsd);

/* The same for an explicit pair list of xyz[n][L][3]: pair t superposes
 * structure jj[t] onto structure ii[t]; rot[t][9], trans[t][3], rmsd[t]
 * (rmsd may be NULL).  Out-of-range indices return BS_ERR_INVALID_ARG,
 * non-finite coordinates BS_ERR_NONFINITE. */
BS_API bs_status bs_superpose_pairs(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const int64_t *ii,
                                    const int64_t *jj, int64_t npairs, double *rot, double *trans, double *rmsd);

/* All-vs-all crmsd of n structures xyz[n][L][3] into `out` (layout and
 * element type from `opts`, NULL = defaults: mixed precision, packed f64
 * triangle).  Replaces the n(n-1)/2 distance-closure calls of
 * HierarchicalClusteringMatrix::new (clustering_matrix.rs:11-22).
 * Chains of up to 16,384 atoms.  On the mixed path a structure set that no
 * coordinate grid fits (chains beyond ~3,000 atoms, or coordinates beyond
 * +-32768 A) is computed on the plain FP64 GPU path instead
 * (bs_metrics.pairs_plain); with a row range it returns BS_ERR_UNSUPPORTED. */
BS_API bs_status bs_all_vs_all(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const bs_opts *opts,
                               void *out);

/* Row ranges that split the n(n-1)/2 pairs of one all-vs-all into `parts`
 * ranges of nearly equal pair counts (bounds[0] = 0 <= bounds[1] <= ... <=
 * bounds[parts] = n, inner bounds multiples of 40 or n): part p is the row range
 * [bounds[p], bounds[p+1]) of bs_opts.row_begin/row_end, e.g. one per GPU,
 * each with its own context and no exchange between them (the pairs are
 * independent).  Host only. */
BS_API bs_status bs_partition_rows(int64_t n, int32_t parts, int64_t *bounds);

/* One structure set of a batched call. */
typedef struct {
  const double *xyz; /* [n][L][3] f64 AoS, host or device memory            */
  int64_t n;         /* structures in the set (>= 0)                         */
  int32_t L;         /* atoms per structure (>= 1)                           */
  int32_t reserved;
  void *out;         /* the set's result: layout and element type of opts   */
} bs_set_desc;

/* All-vs-all crmsd of every set in `sets` (sizes and chain lengths may
 * differ), each into its own `out`.  On the mixed path all sets run in one
 * persistent tensor-core launch (one call sequence, replayed as a CUDA
 * graph for repeated shapes); each set gets its own coordinate grid and
 * error budget, so a set's result does not depend on the other sets in the
 * call.  The plain path runs the sets one after another. */
BS_API bs_status bs_batched(bs_ctx *ctx, const bs_set_desc *sets, int32_t nsets, const bs_opts *opts);

/* eps-neighbour lists of n structures (the input of OPTICS,
 * optics.rs:51-148, through NeighborsOf, points_set.rs:29-39) without the
 * dense matrix: the all-vs-all runs on the mixed path and keeps, for every
 * structure i, the structures j != i with crmsd(i, j) <= eps, ordered by
 * (crmsd, j) -- the f32 values the dense f32 matrix would hold.  The lists
 * stay on the context; *nnz receives their total length, and
 * bs_neighbors_get copies them out (CSR: row_ptr[n + 1] int64, col[nnz]
 * int32, dist[nnz] f32; host or device memory).  Mixed precision only. */
BS_API bs_status bs_neighbors(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, double eps, const bs_opts *opts,
                              int64_t *nnz);
BS_API bs_status bs_neighbors_get(bs_ctx *ctx, int64_t *row_ptr, int32_t *col, float *dist);
/* The autotuner's cache of a context: the tile shape of the class of sets
 * with chain length L and size n (narrow = 1: 40 x 10 tiles, 0: 40 x 20).
 * bs_tune_get returns -1 for a class not timed yet; bs_tune_set fixes a
 * class's choice (it is then not timed). */
BS_API bs_status bs_tune_get(bs_ctx *ctx, int32_t L, int64_t n, int32_t *narrow);
BS_API bs_status bs_tune_set(bs_ctx *ctx, int32_t L, int64_t n, int32_t narrow);
/* The cache as a list, to persist it: up to `cap` classes, each as
 * (L_class, n_class, narrow) with L_class atoms and n_class structures a
 * representative of the class (bs_tune_set(ctx, L_class, n_class, narrow)
 * restores it); *count is the number of classes cached, *num_sms the
 * context's SM count (a cache applies to GPUs of that size). */
BS_API bs_status bs_tune_list(bs_ctx *ctx, int32_t *L_class, int64_t *n_class, int32_t *narrow, int32_t cap,
                              int32_t *count, int32_t *num_sms);

/* crmsd of an explicit pair list: out[t] = crmsd(xyz[ii[t]], xyz[jj[t]]),
 * f64.  Used for sampled checks and for sparse consumers. */
BS_API bs_status bs_pairs(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const int64_t *ii,
                          const int64_t *jj, int64_t npairs, const bs_opts *opts, double *out);

/* All-vs-all crmsd without any device allocation (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc: code running inside
 * another framework's memory pool, plugins that may only use the buffers they
 * are given, or processes whose device footprint must stay fixed.  `xyz`
 * ([n][L][3] f64) and `out` (packed f64 upper triangle, n(n-1)/2 values) must
 * be device memory of the current device; the work runs on `stream` (a
 * cudaStream_t; NULL = the legacy default stream) with the mixed-precision
 * method of bs_all_vs_all and its default tolerance, and the call returns
 * when `out` is complete.
 *   - Limits: n <= 512 structures, L <= 512 atoms; larger sizes return
 *     BS_ERR_UNSUPPORTED without touching the GPU.
 *   - Scratch lives in static device arrays of the library (about 7.4 MB,
 *     held by every GPU that loads the library until the process exits).
 *   - The call cannot be captured into a CUDA graph: it copies its tables
 *     from host memory, reads its counters back and synchronises `stream`.
 *     On a stream that is being captured it returns BS_ERR_UNSUPPORTED
 *     before any other CUDA call, and the capture stays valid.
 *   - All calls share the scratch: each call clears what must start at zero,
 *     but calls whose work overlaps on the GPU (e.g. on two streams at once)
 *     race and must not be issued. */
BS_API bs_status bs_all_vs_all_static(const double *xyz, int64_t n, int32_t L, double *out, void *stream);

/* ---- serving ------------------------------------------------------------
 * A request loop over a device-resident structure library (the
 * CrmsdServer::{new, submit, wait} handle a maintainer would add beside the
 * all-vs-all call; no counterpart exists in the reference).  The library is
 * bucketed by chain length; a query is a batch of structures of one
 * bucket's length and gets, for every query structure, the top_k library
 * structures of that bucket nearest by crmsd.  Mixed-in clustering jobs run
 * an all-vs-all plus OPTICS (optics.rs:51-148) on their own structures.
 *
 * Batching is continuous: a scheduler thread launches whatever is queued for
 * a bucket as one batch as soon as one of max_inflight device slots is free
 * and the batch's device memory fits the server's budget, so requests that
 * arrive while others are on the GPU are admitted as slots and memory free
 * up, and their work overlaps on the device.  Every query's result depends
 * only on the query and the library: the same alone or in any mix.
 * submit, poll, wait and stats may be called from any thread.
 * Creation sizes every slot's device and pinned buffers for a full batch of
 * each bucket (mixed precision, where the budget holds it), so buffers do not
 * grow while requests wait.  With the environment variable BS_SERVER_TRACE
 * naming a file, a server appends a per-batch and per-request timing trace
 * to it when destroyed. */
typedef struct bs_server bs_server;

typedef struct {
  int32_t nbuckets;
  const int32_t *bucket_L;           /* atoms per structure of each bucket    */
  const int64_t *bucket_n;           /* structures in each bucket             */
  const double *const *bucket_xyz;   /* [n][L][3] f64 per bucket (host/device) */
  int32_t top_k;                     /* hits per query structure, 1..64      */
  int32_t max_inflight;              /* batches on the device at once (0 = 4) */
  size_t hbm_budget;                 /* device bytes for in-flight work
                                        (0 = half the free memory after the
                                        library is resident)                 */
  int32_t precision;                 /* BS_PRECISION_MIXED or _PLAIN64       */
  int32_t max_batch_rows;            /* query structures per batch (0 = 4096) */
  double tolerance;                  /* as bs_opts.tolerance (<= 0: 1e-4)    */
  int32_t index_min;                 /* mixed precision: buckets of at least
                                        this many structures get a library
                                        index that prunes the screen (their
                                        results are unchanged); 0 = 16384,
                                        < 0 = never                         */
  int32_t reserved[5];
} bs_server_config;

typedef struct {
  int64_t queries_done;     /* query requests completed                      */
  int64_t clusters_done;    /* clustering jobs completed                     */
  int64_t pairs;            /* crmsd values computed by completed requests   */
  int64_t batches;          /* device batches launched                       */
  int64_t plain_fallbacks;  /* queries outside their bucket's grid, served
                               by the plain FP64 path                        */
  int64_t pending;          /* requests submitted and not yet completed      */
  double p50_ms;            /* query latency, submit -> results ready        */
  double p99_ms;
  double max_ms;
  double mean_ms;
  double cluster_p50_ms;    /* clustering-job latency                        */
  double cluster_p99_ms;
  double pairs_per_s;       /* pairs / wall time since the last reset        */
  double mean_batch_rows;   /* query structures per batch                    */
  double seconds;           /* wall time since the last reset                */
  int64_t pairs_screened;   /* (query, library) pairs the screens of launched
                               batches covered, in tiles of 40 x 20; below
                               the requests' pairs when library indexes
                               prune                                         */
} bs_server_stats;

BS_API bs_status bs_server_create(bs_server **out, int32_t device, const bs_server_config *cfg);
/* Stops the scheduler after the requests in flight and frees everything. */
BS_API void bs_server_destroy(bs_server *s);
BS_API const char *bs_server_last_error(const bs_server *s);
/* Queues q structures xyz[q][L][3] (copied before the call returns); L must
 * be one of the bucket lengths. */
BS_API bs_status bs_server_submit(bs_server *s, const double *xyz, int32_t q, int32_t L, int64_t *ticket);
/* Queues an all-vs-all + OPTICS clustering job over n structures. */
BS_API bs_status bs_server_submit_cluster(bs_server *s, const double *xyz, int64_t n, int32_t L, double eps,
                                          int32_t min_points, int64_t *ticket);
/* done = 1 once the request's results are ready. */
BS_API bs_status bs_server_poll(bs_server *s, int64_t ticket, int32_t *done);
/* Waits (at most timeout_s seconds; <= 0: no limit) and returns a query's
 * results: hit_index[q][top_k] (library index within the bucket, -1 where
 * the bucket has fewer structures) and hit_rmsd[q][top_k], ascending.  The
 * ticket is released.  BS_ERR_TIMEOUT if not ready in time. */
BS_API bs_status bs_server_wait(bs_server *s, int64_t ticket, int64_t *hit_index, double *hit_rmsd,
                                double timeout_s);
/* The same for a clustering job: OPTICS cluster index of every structure. */
BS_API bs_status bs_server_wait_cluster(bs_server *s, int64_t ticket, int64_t *cluster_of, double timeout_s);
BS_API bs_status bs_server_get_stats(bs_server *s, bs_server_stats *out);
/* Cancels a request that is still queued: *cancelled = 1 and its wait
 * returns BS_ERR_CANCELLED.  A request already handed to the GPU (or done)
 * is not stopped: *cancelled = 0 and its wait returns its result. */
BS_API bs_status bs_server_cancel(bs_server *s, int64_t ticket, int32_t *cancelled);
/* Clears the latency record and restarts the wall clock of the stats. */
BS_API bs_status bs_server_reset_stats(bs_server *s);

/* ---- clustering of a crmsd matrix --------------------------------------- */
/* Merge rules of bioshell-clustering/src/hierarchical/strategies/mod.rs. */
enum {
  BS_LINK_SINGLE = 0,
  BS_LINK_COMPLETE = 1,
  BS_LINK_AVERAGE = 2,
  BS_LINK_MEDIAN = 3,
  BS_LINK_CENTROID = 4,
  BS_LINK_WARD = 5
};

/* Hierarchical agglomerative clustering of the n items of a packed-triangle
 * crmsd matrix (`tri` as written by bs_all_vs_all, element type out_type),
 * with the semantics of hierarchical_clustering
 * (bioshell-clustering/src/hierarchical/hierarchical.rs:22-80): f32
 * distances, first-minimum tie-breaking, the reference's size bookkeeping.
 * Writes the n-1 merges in order: merges[s] = {left id, right id, new id,
 * size}, merge_dist[s] = merging distance; leaves are 0..n-1 and merged
 * clusters n, n+1, ... (the root is 2n-2).  Runs on the host. */
BS_API bs_status bs_hierarchical(const void *tri, int64_t n, int32_t out_type, int32_t rule, int64_t *merges,
                                 float *merge_dist);
/* The same on the GPU of `ctx`: the whole merge loop in one cooperative
 * launch over a device-resident n x n f32 matrix (n^2 x 4 bytes of the
 * context's budget), with the same merges and merge distances as
 * bs_hierarchical bit for bit.  tri may be host or device memory; merges
 * and merge_dist receive the results (host or device memory). */
BS_API bs_status bs_hierarchical_gpu(bs_ctx *ctx, const void *tri, int64_t n, int32_t out_type, int32_t rule,
                                     int64_t *merges, float *merge_dist);
/* Cluster label of every item at a distance cutoff, as retrieve_clusters
 * (hierarchical.rs:136-169) splits the tree; labels number the clusters in
 * the order that function returns them. */
BS_API bs_status bs_cut_tree(const int64_t *merges, const float *merge_dist, int64_t n, float cutoff,
                             int64_t *labels);
/* OPTICS (bioshell-clustering/src/optics.rs:51-148) over the matrix:
 * clustering order, reachability in that order, and the cluster index of
 * every item (clusters split where reachability is undefined = 10 eps). */
BS_API bs_status bs_optics(const void *tri, int64_t n, int32_t out_type, double eps, int32_t min_points,
                           int64_t *order, double *reach, int64_t *cluster_of);
/* The same over sparse neighbour lists (CSR: the neighbours of item i are
 * col[row_ptr[i] .. row_ptr[i+1]) at distances dist[...], as bs_neighbors
 * returns them: every j != i with d(i, j) <= eps, ordered by (d, j)).  The
 * point itself is added at distance 0 as CartesianPoints::neighbors_of
 * includes it (points_set.rs:150-169); results equal bs_optics on the dense
 * f32 matrix holding the same values. */
BS_API bs_status bs_optics_neighbors(const int64_t *row_ptr, const int32_t *col, const float *dist, int64_t n,
                                     double eps, int32_t min_points, int64_t *order, double *reach,
                                     int64_t *cluster_of);

/* ---- data formats on either side of the path (host) --------------------- */
/* Message of the last failed call below on this thread (never NULL). */
BS_API const char *bs_io_last_error(void);
/* Multi-model ingestion: the coordinates of every model of a PDB or mmCIF
 * file (format 0 = detect from the first line, 1 = PDB, 2 = mmCIF) as
 * bioshell-pdb keeps them in Structure::model_coordinates (structure.rs:100),
 * read in one pass instead of a set_model per model: PDB ATOM/HETATM records
 * with models split at ENDMDL (load_pdb.rs:52-115, Vec3::from_pdb_line,
 * vec3.rs:241-246); mmCIF _atom_site rows with models in order of first
 * appearance of pdbx_PDB_model_num (pdb_atom.rs:130-170).  selection 0 keeps
 * every atom, 1 the atoms named " CA " (IsCA, pdb_atom_filters.rs:388-413;
 * mmCIF names formatted as format_atom_name does, pdb_atom.rs:306-331).
 * Every model must hold the same atoms.  *n_models x *n_atoms coordinates
 * are then copied by bs_models_copy into xyz[n][L][3] (host or device
 * memory, e.g. a bs_host_alloc buffer that feeds bs_all_vs_all). */
typedef struct bs_models bs_models;
BS_API bs_status bs_models_read(const char *path, int32_t format, int32_t selection, bs_models **out, int64_t *n_models,
                                int32_t *n_atoms);
BS_API bs_status bs_models_copy(const bs_models *m, double *xyz);
BS_API void bs_models_free(bs_models *m);
/* Distance-matrix TSV, the input of the clust tool (clust.rs:102-105,
 * tests/test_files/d5.tsv): "label<TAB>label<TAB>value" lines.
 * bs_tsv_write writes the n(n-1)/2 pairs of a packed triangle (host or
 * device memory, element type out_type) in row order, labels[i] (NULL: the
 * index) and `decimals` digits after the point (<= 0: 6), rounded as
 * printf("%.*f") rounds; device triangles are streamed through pinned
 * buffers while all host threads format.  bs_tsv_read numbers the labels in
 * order of first appearance (row, then column label); pair {i, j} takes the
 * value of line (i, j), else of line (j, i) when `symmetric`, else
 * default_value; bs_tsv_matrix copies the f32 packed triangle out. */
typedef struct bs_tsv bs_tsv;
BS_API bs_status bs_tsv_write(const char *path, const void *tri, int64_t n, int32_t out_type, const char *const *labels,
                              int32_t decimals);
BS_API bs_status bs_tsv_read(const char *path, double default_value, int32_t symmetric, bs_tsv **out, int64_t *n);
BS_API bs_status bs_tsv_matrix(const bs_tsv *t, float *tri);
BS_API const char *bs_tsv_label(const bs_tsv *t, int64_t i);
BS_API void bs_tsv_free(bs_tsv *t);
/* ---- pinned host memory ------------------------------------------------- */
/* Page-locked host buffers for fast host<->device staging (cudaHostAlloc);
 * free with bs_host_free.  Pageable memory is accepted everywhere too. */
BS_API bs_status bs_host_alloc(size_t bytes, void **out);
BS_API bs_status bs_host_free(void *p);

/* ---- test hooks (no reference counterpart) ------------------------------
 * These run the engine's fixed-point epilogue arithmetic on the HOST, so the
 * CPU test-suite can check the exact-digit algebra without a GPU.  They are
 * never used by the compute entry points above. */

/* The row bands of the banded read-back for one set of n structures asked
 * for in `bands` bands: writes the packed-triangle index at which each band
 * ends (the last is n(n-1)/2) and their count (at most cap).  Host only. */
BS_API bs_status bs_selftest_bands(int64_t n, int32_t bands, int64_t *elem_end, int32_t cap, int32_t *count);
/* Digits of one structure's centred coordinates at grid 2^scale_exp:
 * digits[3][3][L] (digit-major, then coordinate, then atom) as stored, i.e.
 * e0, e1 and e2 = 16 d2 with n = 2^14 e0 + 2^5 e1 + d2, plus the exact
 * squared norm of n (int64) and the RMS quantisation residual (Angstrom). */
BS_API bs_status bs_selftest_digits(const double *xyz, int32_t L, int32_t scale_exp, int32_t *digits,
                                    int64_t *g_exact, double *qres);
/* The mixed-path epilogue for one pair from its level sums levels[4][9]
 * (levels 0-2 exact integers, level 3 = S3 + S4/512, stored as float), exact
 * squared norms, quantisation residuals, the level-3 rounding bound d34
 * (error of E, units 2^(2 scale_exp)) and the total tolerance; returns rmsd
 * and whether the pair would be recomputed (flag = 1). */
BS_API bs_status bs_selftest_epilogue(const float *levels, int64_t ga, int64_t gb, double qa, double qb,
                                      double d34, int32_t scale_exp, int32_t L, double tolerance, double *rmsd,
                                      int32_t *flag);
/* The serving screen's bracket for one pair: m9 = S0 + S1/512 + S11/2^18
 * (S11 = sum e1 e1: the covariance of the structures with digit 2 dropped,
 * t = n - e2/16, in units of 2^28 grid products), gsum = the sum of the two
 * truncated structures' squared norms (grid units), de = a bound on the
 * rounding of S11 as an error of E (grid units; 0 when exact), dr = the sum
 * of their RMS distances from the full structures (Angstrom); returns
 * lo <= crmsd(n_a, n_b) <= hi (Angstrom) before their rounding to half
 * precision. */
BS_API bs_status bs_selftest_screen(const float *m9, double gsum, double de, double dr, int32_t scale_exp, int32_t L,
                                    float *lo, float *hi);
/* The exact recomputation from integer coordinates n_a[3][L], n_b[3][L]. */
BS_API bs_status bs_selftest_exact(const int32_t *na, const int32_t *nb, int32_t L, int32_t scale_exp,
                                   double *rmsd);
/* The superposition math of bs_superpose on the host (sequential sums):
 * rot[9], trans[3] with rot b_k + trans ~ a_k, and its RMSD. */
BS_API bs_status bs_selftest_superpose(const double *a, const double *b, int32_t L, double *rot, double *trans,
                                       double *rmsd);

/* GPU diagnostics of the mixed path.  bs_debug_tile_levels returns the raw
 * tensor-core level sums of the first two tiles (structures 0..39 against
 * 0..19 and 20..39) as levels[4][128][128] (level, row, column; rows and
 * columns in the digit-matrix order of the engine: structure s, coordinate c
 * at 32*(s/10) + 3*(s%10) + c, plus 1 when s%10 >= 5).  bs_debug_pair_levels
 * returns, for each listed pair, the level sums computed with integer
 * CUDA-core arithmetic (levels[npairs][4][9]) and that path's crmsd. */
BS_API bs_status bs_debug_tile_levels(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, float *levels);
BS_API bs_status bs_debug_pair_levels(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const int64_t *ii,
                                      const int64_t *jj, int64_t npairs, float *levels, double *rmsd);

/* Failure-injection hooks for tests (no counterpart in the reference; the
 * reference reports failures only through Result values,
 * bioshell-pdb/src/pdb_parsing_error.rs:7).  Both act on the host or through
 * a kernel argument: nothing here faults or stalls a GPU.
 *   bs_debug_set_wait_limit: the bound, in nanoseconds, on each grid-barrier
 *     wait of this context's GPU hierarchical clustering and on each
 *     pipeline (mbarrier) wait of the copy and MMA threads of its all-vs-all
 *     tensor-core kernel (0 restores the defaults, 2 s and 4 s).  A wait that runs out makes every
 *     block of the launch stop (the tensor-core kernel first lets its copies
 *     and MMAs in flight complete and frees its tensor memory) and the call
 *     return BS_ERR_TIMEOUT; the context stays usable.
 *   bs_debug_fail_alloc: the `after`-th device workspace allocation of this
 *     context from now on (0: the next one) fails as if the GPU were out of
 *     memory (BS_ERR_OOM, nothing allocated); -1 disarms the hook. */
BS_API bs_status bs_debug_set_wait_limit(bs_ctx *ctx, int64_t ns);
BS_API bs_status bs_debug_fail_alloc(bs_ctx *ctx, int64_t after);

/* Measured FP64 FMA rate of GPU `device` in FLOP/s (2 per fused multiply-add):
 * eight independent chains of fma per thread on 8 blocks of 256 threads per
 * SM, the best of three ~0.1 s launches.  The denominator of the plain FP64
 * path's roofline fraction; a diagnostic with no counterpart in the
 * reference. */
BS_API bs_status bs_diag_fp64_peak(int32_t device, double *flops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* BIOSHELL_CRMSD_H */
