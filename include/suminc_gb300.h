/*
 * suminc_gb300.h -- C ABI of the GB300 delta-accumulative incremental
 * PageRank / SSSP workers over a (summarized) graph.
 *
 * Conventions
 *   - Every entry point returns an sg_status; no C++ exception crosses it.
 *   - Host pointers are caller-owned and copied (or written) before return.
 *   - Device memory is owned by the context; one CUDA stream per context,
 *     created at the device's highest stream priority.  The summary repair
 *     after a batch also runs its shortcut solves on a second stream of the
 *     lowest priority, ordered against the context's stream by events; both
 *     have finished when the call returns.
 *   - A context must not be used by two host threads at once; distinct
 *     contexts are independent.
 *   - Vertex ids are dense 0..n-1 ("vid = rank of oid" as in the reference's
 *     vertex map, grape/vertex_map/global_vertex_map.h:145-166).
 *
 * Each declaration names the reference interface it replaces (paths relative
 * to the SumInc repository).
 */
#ifndef SUMINC_GB300_H_
#define SUMINC_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sg_ctx sg_ctx;

typedef enum sg_status {
  SG_OK = 0,
  SG_ERR_INVALID = 1,       /* bad argument, null handle, vertex id >= n   */
  SG_ERR_CUDA = 2,          /* CUDA runtime error, see sg_last_error()      */
  SG_ERR_OOM = 3,           /* device or host allocation failed             */
  SG_ERR_STATE = 4,         /* call out of order (IncEval before PEval ...) */
  SG_ERR_NOT_CONVERGED = 5, /* round cap reached before the residual test   */
  SG_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up           */
  SG_ERR_UNSUPPORTED = 7,
  SG_ERR_TOO_LARGE = 8      /* input exceeds a fixed capacity (see below)   */
} sg_status;

/* One line of the reference's update file: "a u v [w]" or "d u v"
 * (grape/fragment/inc_fragment_builder.h:38-70).  A weight change is a
 * delete followed by an add of the same pair, as in the reference. */
typedef enum sg_update_op { SG_UPD_ADD = 0, SG_UPD_DEL = 1 } sg_update_op;

typedef struct sg_update {
  uint32_t src;
  uint32_t dst;
  float weight; /* ignored for unweighted graphs */
  uint32_t op;  /* sg_update_op */
} sg_update;

/* Runtime options; the fields mirror the reference's gflags
 * (examples/analytical_apps/flags.cc:28-70). */
/* sg_options.message_type */
enum { SG_MSG_PUSH = 0, SG_MSG_PULL = 1 };

typedef struct sg_options {
  double damping;             /* PageRankIngress::d (pagerank_ingress.h:23) */
  double termcheck_threshold; /* FLAGS_termcheck_threshold: stop when the L1
                                 residual sum|delta| falls below it          */
  int32_t max_rounds;         /* per PEval / IncEval round cap (FLAGS_pr_mr) */
  int32_t compress;           /* FLAGS_compress: run on the summarized graph */
  int32_t max_node_num;       /* FLAGS_max_node_num (cluster size cap)       */
  int32_t min_node_num;       /* FLAGS_min_node_num (smallest cluster kept)  */
  int32_t mirror_k;           /* FLAGS_mirror_k (mirror creation threshold)  */
  int32_t profile;            /* bitmask of kernel classes to time with CUDA
                                 events (0xFF = all); resolved per call      */
  double compress_threshold;  /* FLAGS_compress_threshold (benefit bound)    */
  double sssp_delta;          /* delta-stepping bucket width, 0 = automatic  */
  double slack;               /* extra adjacency capacity per vertex (0.125) */
  double adjoint_rel_tol;     /* adjoint stop: residual < tol * sum|dL/dx|   */
  int32_t pull_hubs;          /* push values of the highest out-degree vertices
                                 each pull CTA keeps in shared memory: 0 =
                                 automatic (up to 12,288), -1 = none (and the
                                 pull in vertex-id order instead of degree
                                 rank order), k > 0 = at most min(k, 16,384) */
  int32_t message_type;       /* FLAGS_message_type for PageRank: 0 = push
                                 (SumSyncIterWorker / IngressSyncIterWorker),
                                 1 = pull (SumSyncIterWorkerPull: synchronous
                                 in-neighbour rounds, Σ|x - x_prev| stop
                                 test, 200-step cap; with compress = 1 the
                                 summary must have no mirrors)              */
  int32_t reserved[6];
} sg_options;

/* Counters of the last PEval / IncEval / batch call. */
typedef struct sg_stats {
  int32_t rounds;           /* propagation rounds executed                  */
  int32_t converged;        /* 1 when the residual test passed              */
  double residual;          /* last L1 residual (PageRank) or 0             */
  uint64_t edges_relaxed;   /* edge relaxations performed (GTEPS numerator) */
  uint64_t vertex_visits;   /* active-vertex visits                          */
  uint64_t shortcut_edges;  /* shortcut (entry->exit) relaxations            */
  uint64_t improvements;    /* SSSP distance improvements                    */
  double elapsed_ms;        /* device time of the call (CUDA events)        */
  double kernel_ms[8];      /* per-kernel-class device time (profile = 1)   */
  uint64_t kernel_launches[8];
  uint64_t live_edges;      /* current edge count                            */
  uint64_t reset_vertices;  /* SSSP IncEval: vertices reset by deletions     */
  uint64_t launches_total;  /* kernels launched by the library since reset   */
  uint64_t edges_pull;      /* relaxations done by dense pull rounds         */
  uint64_t edges_push;      /* relaxations by push rounds (0: every PageRank
                               round is a dense pull)                       */
  uint64_t repacks;         /* adjacency pool repacks since sg_reset_stats
                               (a direction whose free tail could not hold a
                               batch's worst case was rewritten)            */
} sg_stats;

/* kernel classes reported in sg_stats.kernel_ms / kernel_launches */
enum {
  SG_K_PR_PULL = 0,   /* dense pull round (edge-balanced gather)     */
  SG_K_SUM_LOCAL = 1, /* summary: cluster-local precompute           */
  SG_K_PR_VERTEX = 2, /* vertex update / residual / frontier build   */
  SG_K_APPLY = 3,     /* delta-graph applier                         */
  SG_K_SSSP = 4,      /* delta-stepping persistent kernel            */
  SG_K_SUMMARY = 5,   /* summarized rounds / shortcut precompute     */
  SG_K_BATCH = 6,     /* batched queries                              */
  SG_K_ADJOINT = 7    /* transposed delta iteration + gradients      */
};

/* ---------------------------------------------------------------- context */

/* Fills *opt with the reference's defaults (d = 0.85, threshold 1e-6 as the
 * SumInc run scripts pass it, max_node_num 150, min_node_num 8, mirror_k 4,
 * compress_threshold 1). */
sg_status sg_options_default(sg_options* opt);

/* Creates a context on CUDA device `device`.  Replaces the implicit global
 * state of the reference's CUDA shim (cudaCode/my_worker.cu:66-122,
 * tjn::init storing raw pointers in __device__ globals). */
sg_status sg_ctx_create(int device, const sg_options* opt, sg_ctx** out);
sg_status sg_ctx_destroy(sg_ctx* ctx);

/* Message of the last failing call on this context (never NULL). */
const char* sg_last_error(const sg_ctx* ctx);

/* Runs subsequent work of this context on `stream` (a cudaStream_t); its
 * priority is the caller's.  The summary repair's solve stream still waits
 * for the work queued on it and is waited for by it, through events. */
sg_status sg_ctx_set_stream(sg_ctx* ctx, void* stream);
sg_status sg_get_stats(const sg_ctx* ctx, sg_stats* out);

/* Clears the counters of sg_get_stats (kernel times, launches). */
sg_status sg_reset_stats(sg_ctx* ctx);

/* Device-side timing on the context's stream: record event `slot` (0..7),
 * then read the milliseconds between two recorded slots. */
sg_status sg_ctx_record_event(sg_ctx* ctx, int slot);
sg_status sg_ctx_elapsed_ms(sg_ctx* ctx, int a, int b, double* ms);
sg_status sg_ctx_synchronize(sg_ctx* ctx);

/* Changes sg_options.profile (kernel classes timed with CUDA events). */
sg_status sg_ctx_set_profile(sg_ctx* ctx, int32_t mask);

/* ------------------------------------------------------------------ graph */

/* Loads a directed graph from a host CSR: row_ptr[n+1], col[m], optional
 * weights w[m] (NULL for PageRank's EmptyType edges).  Builds the device
 * out-CSR and in-CSR with per-vertex slack for in-place updates.  Replaces
 * LoadGraph + ImmutableEdgecutFragment::Init
 * (grape/fragment/loader.h, immutable_edgecut_fragment.h:129-377). */
sg_status sg_graph_load_csr(sg_ctx* ctx, uint32_t n, const uint64_t* row_ptr,
                            const uint32_t* col, const float* w);

/* Generates a seeded R-MAT graph on the device: 2^scale vertices, exactly
 * `edges` distinct directed edges, self loops dropped, probabilities a,b,c
 * (d = 1-a-b-c).  weight_kind: 0 none, 1 integer U[wlo,whi], 2 float
 * U[wlo,whi].  Same edges as sg_util_rmat_host() for the same arguments. */
sg_status sg_graph_generate_rmat(sg_ctx* ctx, int scale, uint64_t edges,
                                 double a, double b, double c, uint64_t seed,
                                 int weight_kind, double wlo, double whi);

sg_status sg_graph_num_vertices(const sg_ctx* ctx, uint32_t* n);
sg_status sg_graph_num_edges(const sg_ctx* ctx, uint64_t* m);

/* Copies the current graph to host as a packed CSR with rows sorted by
 * destination: row_ptr[n+1], col[m], w[m] (w may be NULL). */
sg_status sg_graph_download_csr(sg_ctx* ctx, uint64_t* row_ptr, uint32_t* col,
                                float* w);

/* Applies one update batch in place on the device (delete, replace, insert;
 * per-vertex segments compacted, overflowing segments relocated), and
 * amends every live application state: PageRank retracts / re-issues the
 * values of vertices whose out-adjacency changed, SSSP resets the
 * dependants of deleted tree edges.  Replaces IncFragmentBuilder::Init/Build
 * (inc_fragment_builder.h:29-133) with AmendValue(-1/+1)
 * (sum_sync_iter_worker.h:139-180, :214-345) and the reset part of
 * SumSyncTraversalWorker::deltaCompute (sum_sync_traversal_worker.h:113-261).
 * Semantics follow the reference: an add of an existing pair replaces it,
 * duplicate adds keep the first, deletes of absent edges are ignored. */
sg_status sg_apply_updates(sg_ctx* ctx, uint64_t count, const sg_update* upd);

/* Same as sg_apply_updates with the batch already in device memory. */
sg_status sg_apply_updates_device(sg_ctx* ctx, uint64_t count, const sg_update* dptr);

/* ------------------------------------------------------------- PageRank */

/* Batch evaluation (PEval) of delta-accumulative PageRank from
 * init_v = 0, init_c = (1-d)/N (pagerank_ingress.h:27-32) to an L1 residual
 * below termcheck_threshold.  Replaces the batch stage of
 * SumSyncIterWorker::Query (sum_sync_iter_worker.h:788-1506) and, for the
 * uncompressed graph, IngressSyncIterWorker::Query
 * (ingress_sync_iter_worker.h:209-370).  out: host float[n] or NULL. */
sg_status sg_pr_peval(sg_ctx* ctx, float* out);

/* Incremental evaluation after sg_apply_updates: iterates the amended
 * deltas to convergence (sum_sync_iter_worker.h:1507-1695). */
sg_status sg_pr_inceval(sg_ctx* ctx, float* out);

/* Current PageRank values (host float[n]). */
sg_status sg_pr_values(sg_ctx* ctx, float* out);

/* Residual deltas (host float[n]). */
sg_status sg_pr_deltas(sg_ctx* ctx, float* out);

/* Device pointer to the values (valid until the next call on ctx). */
sg_status sg_pr_values_device(sg_ctx* ctx, const float** dptr);

/* ------------------------------------------------------ summarized graph */

/* Counters of the summarized graph (the quantities the reference logs while
 * building it: CompressorBase::statistic, compressor_base.h:431-519, and
 * sketch2csr_mirror, :4636-4880). */
typedef struct sg_summary_info {
  uint64_t clusters;          /* kept clusters (supernode_ids)               */
  uint64_t supernodes;        /* one per entry vertex and in-mirror          */
  uint64_t cluster_members;   /* members incl. absorbed vertices             */
  uint64_t sources;           /* entry vertices                               */
  uint64_t bound_nodes;       /* exit vertices                                */
  uint64_t bound_index;       /* shortcut weights entry -> exit / out-mirror */
  uint64_t inner_index;       /* residual shortcuts (inner_delta)             */
  uint64_t inner_value_index; /* value shortcuts (inner_value)                */
  uint64_t all_rows;          /* vertices + mirror rows                       */
  uint64_t absorbed;          /* unclustered mirror candidates absorbed       */
  uint64_t in_mirrors;
  uint64_t out_mirrors;
  uint64_t sync_edges;        /* master <-> mirror edges                      */
  uint64_t boundary_edges;    /* ib_e: exit -> outside, unclustered edges     */
  uint64_t shortcut_edges;    /* is_e: entry -> exit shortcuts                */
  uint64_t node_type_count[7];/* NodeType 0..6 (grape/types.h:70-78)          */
} sg_summary_info;

/* Builds the summarized graph from a clustering (the cluster file records
 * of compress_by_cluster, compressor_base.h:3160-3250): cluster i =
 * members[cluster_ptr[i] .. cluster_ptr[i+1]).  Applies the reference's
 * benefit filter and mirror choice (get_init_supernode_by_clusters, :3253),
 * absorbs unclustered mirror candidates (final_build_supernode, :3616),
 * marks exits (judge_out_bound_node, :3924), builds cluster subgraphs
 * (:3786), computes every supernode's shortcuts on the device
 * (build_iter_index_mirror, iter_compressor.h:318-491), node types (:4144)
 * and the sketch CSRs (:4636).  With options.compress = 1, PEval and IncEval
 * then run the summarized rounds (sum_sync_iter_worker.h:949-1492) before
 * the plain ones. */
sg_status sg_summary_build(sg_ctx* ctx, uint32_t n_clusters, const uint32_t* cluster_ptr,
                           const uint32_t* members);
sg_status sg_summary_info_get(sg_ctx* ctx, sg_summary_info* out);

/* Diagnostic check of the incremental summary repair.  After each batch the
 * device repairs the summary's PageRank tables itself (entry changes,
 * exits, the touched supernodes' shortcuts, node types, the is / ib CSRs and
 * the correction lists: the inc_run of iter_compressor.h:796-896 and
 * compressor_base.h:5634-5924); the host restatement of the same repair runs
 * on demand.  This brings the host copy up to date and compares the two:
 * per row, as sets of targets, weights within a relative 1e-4. */
typedef struct sg_summary_check {
  uint64_t rows;       /* rows compared (vertices + mirror rows)                */
  uint64_t type_diff;  /* vertices whose node type differs                      */
  uint64_t list_diff;  /* entry / exit / single lists that differ (0..3)        */
  uint64_t ib_diff;    /* boundary rows that differ                             */
  uint64_t is_diff;    /* shortcut rows (bound_delta) that differ               */
  uint64_t corr_diff;  /* supernode correction lists (inner_value / inner_delta) */
  double max_rel;      /* largest relative weight difference of matched entries */
} sg_summary_check;
sg_status sg_summary_check_tables(sg_ctx* ctx, sg_summary_check* out);

/* ----------------------------------------------------------------- SSSP */

/* Batch SSSP from `source` with FP64 distances over the edge weights
 * (delta-stepping).  Unreachable vertices read +inf.  Replaces the batch
 * stage of SumSyncTraversalWorker::Query (sum_sync_traversal_worker.h:543,
 * :1037-1420) with SSSPIngress (sssp_ingress.h:25-265, weighted branch).
 * out: host double[n] or NULL. */
sg_status sg_sssp_peval(sg_ctx* ctx, uint32_t source, double* out);

/* Incremental SSSP after sg_apply_updates: re-seeds the reset vertices from
 * their in-neighbours and relaxes from every improved vertex
 * (sum_sync_traversal_worker.h:262-352, :1424-1690).  With compress = 1 and
 * a summarized PEval before it, the relaxation runs over the summary
 * (boundary edges and repaired shortcuts), followed by the correction of
 * the inner members. */
sg_status sg_sssp_inceval(sg_ctx* ctx, double* out);

sg_status sg_sssp_distances(sg_ctx* ctx, double* out);

/* Shortest-path tree parents (host uint32[n]; UINT32_MAX for the source and
 * unreachable vertices) -- the DependencyData::parent_gid the reference
 * keeps (grape/utils/dependency_data.h:12-33). */
sg_status sg_sssp_parents(sg_ctx* ctx, uint32_t* out);

/* Failure detection of the device-side waits (no counterpart in the
 * reference, which has none).  Every wait in the persistent kernels (the
 * grid barrier of SSSP, its reset BFS and the batched kernel) spins a
 * bounded number of times, then records an error word and returns, and the
 * host call reports SG_ERR_TIMEOUT with the context still usable.  This
 * entry point runs that barrier with four CTAs: skip_one_block = 0 lets all
 * arrive (SG_OK); 1 keeps one away, so the wait runs out after about 10 ms
 * (SG_ERR_TIMEOUT). */
sg_status sg_debug_barrier_probe(sg_ctx* ctx, int32_t skip_one_block);

/* ------------------------------------------- personalized PageRank, batches */

/* Personalized PageRank of one query on the plain graph: teleport mass
 * (1-d) spread uniformly over the seeds (the PPR app's seed set,
 * examples/analytical_apps/ppr/ppr.h:24-31), x = 0 at start, the Ingress
 * delta rounds of sg_pr_peval to the same residual test.  out: host
 * float[n] or NULL.  Seeds should be distinct (a repeated seed gets its
 * share once per occurrence).  Leaves no IncEval state behind. */
sg_status sg_ppr(sg_ctx* ctx, uint32_t n_seeds, const uint32_t* seeds, float* out);

/* A batch of independent queries evaluated by one persistent kernel (no
 * counterpart in the reference, which answers one query per run):
 *   PPR  query q teleports to seeds[seed_ptr[q] .. seed_ptr[q+1]), each
 *        query as sg_ppr; at most 256 queries;
 *   SSSP one distance vector per source, as sg_sssp_peval; at most 64
 *        sources; needs a weighted graph. */
typedef struct {
  uint32_t ppr_queries;
  const uint32_t* ppr_seed_ptr;  /* [ppr_queries + 1], seed_ptr[0] = 0   */
  const uint32_t* ppr_seeds;     /* vertex ids                           */
  uint32_t sssp_sources;
  const uint32_t* sources;       /* [sssp_sources] vertex ids            */
} sg_batch_spec;

typedef struct {
  uint32_t ppr_queries, sssp_sources;
  uint32_t chunk_quads;      /* schedule: quads per PPR work chunk        */
  uint32_t blocks_per_sm;    /* schedule: persistent CTAs per SM          */
  double sssp_bucket;        /* schedule: delta-stepping bucket width     */
  int32_t graph_launch;      /* 1 when the run replayed a CUDA graph      */
  double tune_ms;            /* host time of the last autotune            */
  uint32_t iterations;       /* persistent-kernel iterations              */
  uint32_t ppr_pulls, sssp_steps, sssp_scans;
  uint32_t ppr_not_converged;/* queries that hit the round cap            */
  uint64_t ppr_edge_visits;  /* sum over pulls of edges x queries pulled  */
  uint64_t sssp_relaxations; /* (edge, source) pairs relaxed              */
  uint64_t sssp_improvements;
  double elapsed_ms;         /* device time of the launch sequence        */
} sg_batch_info;

/* Runs the batch.  The first batch of a given shape on a graph picks the
 * schedule by timing candidates (chunk size x CTAs per SM for PPR, bucket
 * width for SSSP) and captures the launch sequence in a CUDA graph; later
 * batches of that shape replay it.  Outputs (host, or NULL to keep them on
 * the device): ppr_out float[ppr_queries][n], sssp_out double[sources][n]
 * (+inf for unreachable). */
sg_status sg_batch_run(sg_ctx* ctx, const sg_batch_spec* spec, float* ppr_out,
                       double* sssp_out);
/* As sg_batch_run, re-running the autotuner first. */
sg_status sg_batch_tune_run(sg_ctx* ctx, const sg_batch_spec* spec,
                            float* ppr_out, double* sssp_out);
sg_status sg_batch_info_get(sg_ctx* ctx, sg_batch_info* out);
/* Per PPR query of the last batch: rounds (counted as sg_pr_peval counts
 * them) and final residual; arrays of ppr_queries entries, either NULL. */
sg_status sg_batch_query_stats(sg_ctx* ctx, int32_t* rounds, double* residual);
/* Device pointers to the last batch's outputs (layouts as above); valid
 * until the next batch or sg_ctx_destroy. */
sg_status sg_batch_outputs_device(sg_ctx* ctx, const float** ppr,
                                  const double** sssp);

/* ------------------------------------------ weighted PageRank and adjoint */

/* PageRank with edge weights (no counterpart in the reference, whose
 * PageRank divides by the out-degree): x = (1-d) t + d M x with
 * M[v][u] = w_uv as loaded (column-normalised weights make M column-
 * stochastic), teleport t (host float[n], or NULL for uniform 1/n); the
 * Ingress delta rounds of sg_pr_peval with the weights applied in the
 * gather, to the same residual test.  x_out: host float[n] or NULL. */
sg_status sg_pr_weighted(sg_ctx* ctx, const float* tele, float* x_out);

/* Column-normalises the weights: every edge weight w_uv is divided by the
 * sum of u's out-edge weights (rows with weight sum 0 are left alone). */
sg_status sg_graph_normalize_weights(sg_ctx* ctx);

/* Adjoint of the last sg_pr_weighted on the current graph: given
 * dl_dx = dL/dx (host float[n]) solves lambda = dl_dx + d M^T lambda by the
 * transposed delta iteration (pulls along out-edges) to a residual below
 * opt.adjoint_rel_tol * sum|dl_dx|, then
 *   dl_dw[e]  = d * lambda[v] * x[u] for the e-th edge (u, v) in the order
 *               of sg_graph_download_csr (host float[m] or NULL),
 *   dl_dtele  = (1-d) * lambda (host float[n] or NULL). */
sg_status sg_pr_adjoint(sg_ctx* ctx, const float* dl_dx, float* dl_dw, float* dl_dtele);
/* As sg_pr_adjoint with dl_dx already in device memory. */
sg_status sg_pr_adjoint_device(sg_ctx* ctx, const float* d_dl_dx, float* dl_dw,
                               float* dl_dtele);

typedef struct {
  int32_t forward_rounds, adjoint_rounds;
  double forward_ms, adjoint_ms;      /* device time; adjoint incl. gradients */
  double forward_residual, adjoint_residual;
  uint64_t forward_edges, adjoint_edges, gradient_edges;
} sg_adjoint_info;
sg_status sg_adjoint_info_get(sg_ctx* ctx, sg_adjoint_info* out);
/* The forward values x and the adjoint lambda (each host float[n] or NULL). */
sg_status sg_adjoint_values(sg_ctx* ctx, float* x, float* lambda);

/* ------------------------------------------------- allocation-free PEval */

/* Largest vertex count sg_pr_peval_noalloc accepts. */
#define SG_PR_NOALLOC_MAX_VERTICES (1u << 22)

/* PageRank PEval that allocates nothing -- no counterpart in the reference.
 * For callers that cannot call cudaMalloc: a process whose device memory is
 * owned by another framework's pool, or latency-bound loops that must not
 * hit cudaMalloc's implicit synchronisation.  The caller passes a packed CSR (d_row_ptr[n+1],
 * d_col[m]) and the outputs (d_values[n], d_deltas[n]) in device memory of
 * the current device, and a stream (NULL = default stream); the result is
 * the delta-accumulative PageRank of sg_pr_peval (L1 residual below
 * `threshold`).  Scratch (one float per vertex and a few control words) is a
 * fixed file-scope device array of SG_PR_NOALLOC_MAX_VERTICES entries that
 * every GPU loading the library keeps until the process exits; n above that
 * returns SG_ERR_TOO_LARGE.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current.
 * Every call shares the array: calls whose work overlaps on the GPU race
 * and must be serialised by the caller.  Each round ends by reading two
 * control words back to the host, which synchronises `stream` once per
 * round, so no call can run under stream capture or inside a CUDA graph.
 * A CUDA error still pending from the
 * caller's own work makes the call return SG_ERR_CUDA before it launches
 * anything, and that error is left for the caller to collect.  Returns
 * SG_ERR_NOT_CONVERGED when max_rounds is reached. */
sg_status sg_pr_peval_noalloc(uint32_t n, uint64_t m, const uint64_t* d_row_ptr,
                              const uint32_t* d_col, double damping,
                              double threshold, int32_t max_rounds, void* stream,
                              float* d_values, float* d_deltas,
                              int32_t* rounds_out, double* residual_out);

/* ------------------------------------------------ the reference's files */

/* Loads a graph from the reference's text files: efile lines "u v" or
 * "u v w" (oids; w read when weighted != 0), vfile one oid per line (NULL:
 * the oids seen in efile).  Vertex ids are the ranks of the distinct oids
 * (oids 0..N-1 keep their value), as the reference's vertex map
 * (grape/vertex_map/global_vertex_map.h:145-166); a repeated (u, v) keeps
 * its first line. */
sg_status sg_graph_load_files(sg_ctx* ctx, const char* efile, const char* vfile,
                              int weighted);
/* oid of every vertex id (host uint64_t[n]). */
sg_status sg_graph_vertex_oids(sg_ctx* ctx, uint64_t* oids);
/* Names the vertices of a graph loaded from arrays: oids[v] for v < n,
 * strictly increasing (the vertex map's order); the update and cluster
 * files are then read in these oids. */
sg_status sg_graph_set_vertex_oids(sg_ctx* ctx, const uint64_t* oids);
/* Applies an update file ("a u v [w]" / "d u v" lines, oids;
 * grape/fragment/inc_fragment_builder.h:38-70) as one batch. */
sg_status sg_apply_update_file(sg_ctx* ctx, const char* path);
/* Saves / loads the summary's cluster state in the reference's serialized
 * layout (serialize_cluster / de_serialize_cluster, compressor_base.h:
 * 2987-3158): the supernode candidates and mirrors chosen from the
 * clustering, so a later run on the same graph skips that step.  Loading
 * rebuilds everything after it (exits, subgraphs, shortcuts, sketch). */
sg_status sg_summary_save(sg_ctx* ctx, const char* path);
sg_status sg_summary_load(sg_ctx* ctx, const char* path);
/* sg_summary_build from a cluster file (records "size oid_1 ... oid_size",
 * the <efile>.c_<max_node_num> file of compressor_base.h:3174-3243). */
sg_status sg_summary_build_file(sg_ctx* ctx, const char* path);

/* ------------------------------------------------------ host utilities
 * (no GPU needed; used to make inputs identical on every side) */

/* Host twin of sg_graph_generate_rmat: writes row_ptr[2^scale+1], col[edges]
 * and, when w != NULL and weight_kind != 0, w[edges]. */
sg_status sg_util_rmat_host(int scale, uint64_t edges, double a, double b,
                            double c, uint64_t seed, int weight_kind,
                            double wlo, double whi, uint64_t* row_ptr,
                            uint32_t* col, float* w);

typedef struct sg_hostgraph sg_hostgraph;

/* A host adjacency mirror used to draw update batches that are valid for the
 * current graph (inserts of absent pairs, deletes of present edges). */
sg_status sg_hostgraph_create(uint32_t n, const uint64_t* row_ptr,
                              const uint32_t* col, const float* w,
                              sg_hostgraph** out);
sg_status sg_hostgraph_destroy(sg_hostgraph* g);

/* Draws a batch of n_ins inserts of uniform absent (u,v) pairs, n_del
 * deletes of uniformly chosen present edges and n_rew weight changes
 * (emitted as a delete plus an add), applies it to the mirror and writes
 * n_ins + n_del + 2*n_rew records to out.  New weights are integers
 * U[wlo,whi] when integer_weights, else float U[wlo,whi]. */
sg_status sg_hostgraph_gen_updates(sg_hostgraph* g, uint64_t n_ins,
                                   uint64_t n_del, uint64_t n_rew,
                                   uint64_t seed, int integer_weights,
                                   double wlo, double whi, sg_update* out);

/* The in-repo greedy clustering used to produce the cluster file of the
 * summarized graph: restates the reference's flag-default builder
 * parallel_find_multi_source_supernode_2_sort_sample with one compress
 * thread (grape/fragment/compressor_base.h:367-419, :1448-1875), drawing its
 * candidate samples from a generator seeded by `seed` instead of
 * std::random_device.  Output: cluster i = members[cluster_ptr[i] ..
 * cluster_ptr[i+1]) (sorted); the caller provides cluster_ptr[n+1] and
 * members[n]. */
sg_status sg_util_greedy_clusters(uint32_t n, const uint64_t* row_ptr,
                                  const uint32_t* col, int max_node_num,
                                  int min_node_num, uint64_t seed,
                                  uint32_t* cluster_ptr, uint32_t* members,
                                  uint32_t* n_clusters);

/* Packed copy of the mirror (rows sorted). */
/* The summary's cluster state for a clustering, in the reference's
 * serialized layout (as sg_summary_save writes it), computed on the host.
 * out: buffer of *size bytes or NULL (then only *size is set). */
sg_status sg_util_summary_serialize(uint32_t n, const uint64_t* row_ptr,
                                    const uint32_t* col, uint32_t n_clusters,
                                    const uint32_t* cluster_ptr,
                                    const uint32_t* members, int min_node_num,
                                    int mirror_k, double compress_threshold,
                                    uint8_t* out, uint64_t* size);
sg_status sg_hostgraph_num_edges(const sg_hostgraph* g, uint64_t* m);
sg_status sg_hostgraph_csr(const sg_hostgraph* g, uint64_t* row_ptr,
                           uint32_t* col, float* w);

#ifdef __cplusplus
}
#endif

#endif /* SUMINC_GB300_H_ */
