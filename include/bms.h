/*
 * bms.h — C ABI of the GB300 batched subgraph-isomorphism engine (libbms.so).
 *
 * The entry points mirror the reference library's hot path, stage by stage
 * (AnySparse/BMS2, namespace `sigmo`, header-only SYCL C++20).  The reference
 * has no FFI of its own: its boundary is a set of C++ templates called from the
 * driver's main() (library/src/BMS2.cpp:7-393).  Each function below names the
 * reference interface it replaces.  Conventions:
 *   - every call returns an int status: BMS_OK (0) or a negative BMS_E* code;
 *     no C++ exception crosses this boundary; bms_last_error() gives a message;
 *   - one context per host thread (contexts are independent, a context is not
 *     re-entrant — the reference is single-threaded with one sycl::queue);
 *   - input arrays are borrowed for the duration of the call and copied;
 *   - node ids are global within a batch, as in DeviceBatchedCSRGraph
 *     (library/include/graph.hpp:58-66).
 */
#ifndef BMS_H
#define BMS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BMS_ABI_VERSION 2

/* Limits of this implementation.  The reference itself is defined for data
 * graphs of at most 64 nodes and queries of at most 30 nodes (64-bit bitsets,
 * utils.hpp:90-120, signature.hpp:614; MAX_QUERY_NODES, isomorphism.hpp:248). */
#define BMS_MAX_DATA_NODES 128u
#define BMS_MAX_QUERY_NODES 64u
#define BMS_MAX_REFINE_STEPS 8
#define BMS_WILDCARD_LABEL 255u       /* types.hpp:18 */
#define BMS_NULL_NODE 0xFFFFFFFFu     /* types.hpp:22 */

typedef enum {
  BMS_OK = 0,
  BMS_EINVAL = -1,       /* bad argument or malformed input (graph.hpp:200 throws) */
  BMS_ENOMEM = -2,       /* device or host allocation failed */
  BMS_ECUDA = -3,        /* a CUDA runtime call failed */
  BMS_EIO = -4,          /* file could not be opened or read */
  BMS_ESTATE = -5,       /* call out of order (e.g. join before map) */
  BMS_EUNSUPPORTED = -6, /* input exceeds BMS_MAX_* limits */
  BMS_ETIMEDOUT = -7,    /* a bounded host wait expired */
  BMS_EINCOMPLETE = -8,  /* some pairs hit the expansion budget (see status) */
  BMS_ENODEV = -9        /* no usable CUDA device */
} bms_status;

typedef enum { BMS_QUERY = 0, BMS_DATA = 1 } bms_kind;
/* join mode: find-first reports min(count,1) per pair (isomorphism.hpp:298,
 * default of the reference driver); count-all is the driver's --find-all. */
typedef enum { BMS_FIND_FIRST = 0, BMS_COUNT_ALL = 1 } bms_mode;
/* search order: GMCR = query-index order 0..n-1, the only order of the
 * reference (isomorphism.hpp:414-448); LEARNED = cost-model order; GIVEN =
 * the orders last set with bms_set_query_order. */
typedef enum { BMS_ORDER_GMCR = 0, BMS_ORDER_LEARNED = 1, BMS_ORDER_GIVEN = 2 } bms_order;
/* join semantics.  EXACT counts every injective, induced, label-preserving
 * embedding inside the candidate sets.  REFERENCE_DFS restates the reference
 * DFS literally, including the visited bit it never clears when a frame
 * advances (isomorphism.hpp:414-448), with mapping[] reset to NULL per root;
 * it requires BMS_ORDER_GMCR. */
typedef enum { BMS_SEM_EXACT = 0, BMS_SEM_REFERENCE_DFS = 1 } bms_semantics;

/* per-pair status codes (bms_get_pair_status) */
#define BMS_PAIR_DONE 0u
#define BMS_PAIR_INCOMPLETE 1u /* the expansion budget ran out */

/* ------------------------------------------------------------------ errors */
/* Last error message of `ctx`, or of the calling thread when ctx is NULL. */
const char* bms_last_error(const void* ctx);
const char* bms_status_name(int status);
int bms_abi_version(void);

/* ------------------------------------------------------- host graph batches */
/* A host-side batched CSR, the reference's std::vector<CSRGraph> flattened
 * the way createDeviceCSRGraph flattens it (graph.hpp:251-310). */
typedef struct bms_graphs bms_graphs;
typedef struct {
  uint32_t n_graphs;
  uint32_t max_nodes;             /* largest graph */
  uint64_t n_nodes;
  uint64_t n_entries;             /* CSR entries (two per undirected edge) */
  const uint32_t* graph_offsets;  /* [n_graphs + 1] */
  const uint32_t* row_offsets;    /* [n_nodes + 1], global */
  const uint32_t* column_indices; /* [n_entries], global node ids */
  const uint8_t* node_labels;     /* [n_nodes] */
  const uint8_t* edge_labels;     /* [n_entries] */
} bms_graphs_view;

/* io::loadCSRGraphsFromFile (io.hpp:43-52) + IntermediateGraph(line) and
 * toCSRGraph() (graph.hpp:147-243): one graph per line,
 * "n#N l#L {id label}xN e#E {u v [elabel]}xE".  Empty lines are skipped;
 * a malformed line fails with BMS_EINVAL unless skip_invalid is set, in which
 * case it is dropped (the batch driver's behaviour, BMS2_batch.cpp:121-124).
 * max_graphs = 0 means no limit (--max-data-graphs / --max-query-graphs). */
int bms_graphs_parse_file(const char* path, uint32_t max_graphs, int skip_invalid, bms_graphs** out);
int bms_graphs_parse_text(const char* text, size_t len, uint32_t max_graphs, int skip_invalid, bms_graphs** out);
/* Wrap caller CSR arrays (copied).  edge_labels may be NULL (all zero). */
int bms_graphs_from_csr(uint32_t n_graphs, const uint32_t* graph_offsets, const uint32_t* row_offsets,
                        const uint32_t* column_indices, const uint8_t* node_labels, const uint8_t* edge_labels,
                        bms_graphs** out);
int bms_graphs_view_of(const bms_graphs* g, bms_graphs_view* out);
/* Write in the reference text format (generate_data.py:74-92 layout). */
int bms_graphs_write_file(const bms_graphs* g, const char* path);
/* Keep graphs whose node count is in [min_nodes, max_nodes] (--query-filter,
 * BMS2.cpp:27-34). */
int bms_graphs_filter_size(const bms_graphs* g, uint32_t min_nodes, uint32_t max_nodes, bms_graphs** out);
void bms_graphs_free(bms_graphs* g);
/* Page-lock a host batch (no reference counterpart) so that its uploads, and
 * every slice bms_run_batches takes from it, copy by asynchronous DMA instead
 * of through staging buffers.  Undone by bms_graphs_unpin or bms_graphs_free.
 * Pinning a pinned batch does nothing. */
int bms_graphs_pin(bms_graphs* g);
int bms_graphs_unpin(bms_graphs* g);

/* ------------------------------------------- seeded synthetic molecular data */
/* Not part of the reference (its datasets are converted from SMARTS with rdkit,
 * generate_data.py).  Labels use the reference converter's ids
 * (generate_data.py:8): N=0 Cl=1 Br=3 O=7 C=8 S=9 F=10. */
typedef enum { BMS_SIZE_UNIFORM = 0, BMS_SIZE_NORMAL = 1, BMS_SIZE_LOGNORMAL = 2 } bms_size_dist;
typedef struct {
  uint32_t n_graphs;
  uint32_t size_dist;   /* bms_size_dist */
  double p0, p1;        /* uniform: unused; normal: mean, sd; lognormal: median, sigma */
  uint32_t min_nodes, max_nodes;
  uint32_t min_rings, max_rings;
} bms_mol_params;
int bms_synth_molecules(const bms_mol_params* p, uint64_t seed, bms_graphs** out);

typedef struct {
  uint32_t n_queries;
  uint32_t min_nodes, max_nodes;
  double frac_carbon;      /* pure-carbon chains and rings */
  double frac_adversarial; /* fused carbon rings, long chains, halogen stars */
} bms_query_params;
/* Queries are connected induced subgraphs of random graphs of `source`,
 * numbered in random depth-first discovery order. */
int bms_synth_queries(const bms_query_params* p, const bms_graphs* source, uint64_t seed, bms_graphs** out);

/* ------------------------------------------------------------------ shards */
/* Owner rank of every data graph for `world` GPUs: the reference MPI driver's
 * longest-processing-time balancing (BMS2_mpi.cpp:78-157): cost = nodes^2 +
 * edges, graphs by decreasing cost (stable), each to the least-loaded rank (the
 * lowest on ties).  owners[n_graphs]; loads[world] (nullable) receives each
 * rank's summed cost.  Host only. */
int bms_shard_lpt(uint32_t n_graphs, const uint32_t* graph_offsets, const uint32_t* row_offsets, uint32_t world,
                  uint32_t* owners, double* loads);

/* --------------------------------------------------------------- contexts */
typedef struct bms_ctx bms_ctx;
int bms_create(int device, bms_ctx** out);
void bms_destroy(bms_ctx* ctx);
/* Run all work of ctx on `stream` (a cudaStream_t; NULL restores the
 * context's own stream). */
int bms_set_stream(bms_ctx* ctx, void* stream);
/* Per (pair, root) expansion budget of the join; 0 = unlimited (default). */
int bms_set_expansion_budget(bms_ctx* ctx, uint64_t budget);
/* Log per-query-vertex expansions in bms_run (count-all, GMCR or given order,
 * EXACT semantics only) for bms_vertex_expansions; off by default. */
int bms_set_logging(bms_ctx* ctx, int vertex_expansions);

/* Engine options (no reference counterpart). */
typedef enum {
  BMS_OPT_FILTER_KERNEL = 1, /* fused filter: BMS_FILTER_SLICED (default) or BMS_FILTER_BALLOT */
  BMS_OPT_JOIN_STEPS = 2,    /* DFS steps a warp runs between refills (default 32) */
  BMS_OPT_SPLIT_BUDGET = 3,  /* expansions after which a join search hands its unexplored subtrees
                                to the next round (default 1024; 0 = never split) */
  BMS_OPT_SUBTREE_CAP = 4,   /* entries of each of the two subtree buffers (88 B each); 0 = one per
                                record, at least 65,536 and at most 4,194,304 (default) */
  BMS_OPT_CUDA_GRAPH = 5,    /* 1 (default): bms_run captures its device work as a CUDA graph on the
                                second run with unchanged inputs and settings, and replays it after;
                                0: every run launches its kernels one by one */
  BMS_OPT_USE_CS = 6,        /* 1: the clustered join of the reference driver's --use-cs
                                (BMS2.cpp:218-296) replaces the join of bms_join, bms_run and the batch
                                drivers; 0 (default): the plain join.  See below. */
  BMS_OPT_RESIDENT_SIGNATURES = 7 /* 1: bms_run_resident computes the data-side signatures of the whole
                                resident batch once (for its refine_steps) and every later window and
                                call reuses them; 0 (default): each window computes its own.  For
                                serving many small query batches over the same resident data. */
} bms_option;
/* Clustered join.  The loaded queries are one cluster in the layout of the
 * reference's cluster files (generate_cs.py:338-362, 555-577): query 0 is the
 * prototype P and every member lists P's nodes first, in P's order.  Step 1
 * (join::joinPartialCandidates2, isomorphism.hpp:1021-1178) finds every match of
 * P's nodes in every data graph over P's own candidate rows; step 2
 * (join::joinWithPartialMatches, isomorphism.hpp:756-977) extends each match with
 * every query of its data graph's GMCR row: a query smaller than P adds 0, one of
 * P's size adds 1, a larger one adds its completions from node |V(P)| on over
 * its own candidate rows.  Requires BMS_ORDER_GMCR; both semantics and both
 * modes apply (REFERENCE_DFS restates both reference DFS loops literally).  With
 * an empty query 0 the plain join runs, as in the reference driver.  The label
 * screen of the fused filter is off in this mode (every GMCR pair gets its
 * candidate rows), the expansion budget and the join schedule do not apply, and
 * bms_stats.n_partial_matches reports step 1's matches. */
#define BMS_FILTER_SLICED 0 /* clause masks per data graph in shared memory, one thread per query */
#define BMS_FILTER_BALLOT 1 /* one lane per data node, candidate rows formed by warp ballots */
int bms_set_option(bms_ctx* ctx, int option, int64_t value);

/* createDeviceCSRGraph (graph.hpp:251-310): upload a batch as the query or the
 * data side.  The CSR must be symmetric with column ids inside each graph; the
 * check runs on the device and is reported by the next stage call.  Edge labels
 * are accepted but not copied: matching never reads them (as in the reference).
 * Arrays in page-locked memory are copied asynchronously: keep them unchanged
 * until the next stage call, run or read-back on the context returns. */
int bms_load_graphs(bms_ctx* ctx, int kind, const bms_graphs* g);
int bms_load_csr(bms_ctx* ctx, int kind, uint32_t n_graphs, const uint32_t* graph_offsets,
                 const uint32_t* row_offsets, const uint32_t* column_indices, const uint8_t* node_labels,
                 const uint8_t* edge_labels);

/* ------------------------------------------------------- staged pipeline */
/* Signature<>::generate{Data,Query}Signatures (signature.hpp:56-73,124-151),
 * PathSignature (:455-519), CycleSignature (:574-719) and the distance-shell
 * refinement refine{Data,Query}Signatures(k) for k = 1..refine_steps
 * (:335-389), for both sides. */
int bms_signatures(bms_ctx* ctx, int refine_steps);
/* filter::filterCandidates (isomorphism.hpp:30-104): dense query-major
 * candidate bitset, uint32 words, ceil(data_nodes/32) words per query node
 * (candidates.hpp:10-24). */
int bms_filter(bms_ctx* ctx);
/* filter::refineCandidates (isomorphism.hpp:106-203) with shell step k. */
int bms_refine(bms_ctx* ctx, int step);
/* mapping::GMCR::generateGMCR (gmcr.hpp:35-144).  Query ids within a data
 * graph's row are ascending.  *n_pairs receives the number of valid pairs. */
int bms_map(bms_ctx* ctx, uint64_t* n_pairs);
/* join::joinCandidates (isomorphism.hpp:291-472) over the mapped pairs.
 * *total receives the sum of per-pair counts (the driver's "# Matches"). */
int bms_join(bms_ctx* ctx, int mode, int order, int semantics, uint64_t* total);

/* ------------------------------------------------------- fused pipeline */
/* Signatures, filter, refine 1..refine_steps, mapping and join in one pass
 * that never materialises the dense candidate matrix.  Results are identical
 * to the staged pipeline's.  The persistent join and the filter run as CUDA
 * kernels on the context's stream. */
int bms_run(bms_ctx* ctx, int refine_steps, int mode, int order, int semantics, uint64_t* total);
/* The batch driver (BMS2_batch.cpp:101-305): the loaded queries against a host
 * batch of data graphs taken batch_graphs graphs at a time (0 = the
 * reference's 100,000).  Each slice is uploaded as the data side (its global
 * ids rebased on the device) and run through bms_run; *total receives the sum
 * over the slices and per_query (optional, [n_query_graphs]) each query's
 * matches (find-first: its data graphs with a match).  Afterwards the context
 * holds the last slice as its data side and that slice's per-pair results;
 * bms_get_stats then reports stage times, launches, matches and expansions
 * summed over the slices (graph, node and valid-pair counts: the last slice). */
int bms_run_batches(bms_ctx* ctx, const bms_graphs* data, uint32_t batch_graphs, int refine_steps, int mode,
                    int order, int semantics, uint64_t* total, uint64_t* per_query);
/* Device-resident data (no reference counterpart; its batch driver re-reads
 * the file each time): bms_load_resident uploads a data batch once and keeps
 * it in HBM; bms_run_resident runs the loaded queries over it in windows of
 * window_graphs graphs (0 = 100,000), each window a view of the resident
 * buffers (nothing copied), with the totals, per-query matches and statistics
 * of bms_run_batches.  Afterwards the data side is the last window.  A later
 * bms_load_graphs / bms_load_csr of the data side replaces the views. */
int bms_load_resident(bms_ctx* ctx, const bms_graphs* data);
int bms_run_resident(bms_ctx* ctx, uint32_t window_graphs, int refine_steps, int mode, int order, int semantics,
                     uint64_t* total, uint64_t* per_query);

/* ------------------------------------------------------------- results */
typedef struct {
  uint32_t n_query_graphs, n_data_graphs;
  uint64_t n_query_nodes, n_data_nodes;
  uint64_t n_pairs;          /* query graphs x data graphs */
  uint64_t n_valid_pairs;    /* GMCR tasks */
  uint64_t n_incomplete;     /* pairs that hit the expansion budget */
  uint64_t total_matches;
  uint64_t expansions;       /* successful assignments in the join, roots included */
  uint32_t refine_steps;
  uint32_t last_mode, last_order, last_semantics;
  /* device time of the last stage calls, milliseconds (CUDA events) */
  float ms_signatures, ms_filter, ms_refine, ms_map, ms_order, ms_join, ms_total;
  uint64_t kernel_launches;  /* CUDA kernels launched by the last pipeline call */
  uint64_t n_partial_matches; /* clustered join: prototype matches over all data graphs */
} bms_stats;
int bms_get_stats(bms_ctx* ctx, bms_stats* out);

/* GMCR as the reference stores it (gmcr.hpp:220-224): data_graph_offsets
 * [n_data_graphs+1] and query_graph_indices [n_valid_pairs]. */
int bms_get_gmcr(bms_ctx* ctx, uint32_t* data_graph_offsets, uint32_t* query_graph_indices, uint64_t cap);
/* GMCR data_graph_offsets from per-data-graph pair counts, on the device, with
 * no device allocation: counts[n] and offsets[n + 1] are device pointers owned
 * by the caller; offsets[i] = counts[0] + ... + counts[i-1] and offsets[n] is
 * the total.  No counterpart in the reference.  It serves callers that must not
 * allocate device memory while they run — applications whose device memory is
 * held by their own pool allocator, and latency-sensitive pipelines that cannot
 * take the device-wide synchronisation of cudaMalloc/cudaFree — by keeping the
 * scan's scratch in a fixed 256 KiB array that every GPU loading libbms holds
 * until the process exits.  Limit: n <= 100,000,000 (BMS_EUNSUPPORTED above).
 * The first call on a device looks up that array's device address (a one-time
 * set-up per device and current context: a caller that makes another context
 * current on the device gets a fresh lookup); make that first call before any
 * stream capture.  cudaDeviceReset ends the context the address belongs to, as
 * it ends every other libbms device buffer: use no libbms state of that device
 * afterwards in the same process.  All calls share the
 * one array, so calls that overlap on the GPU (other streams, other threads)
 * race: order them.  The work is queued on `stream` (a cudaStream_t, NULL for
 * the default stream); the call does not wait for it. */
int bms_gmcr_offsets_static(const uint32_t* counts, uint32_t* offsets, uint64_t n, void* stream);
/* Per-pair counts in GMCR order (find-first: 0/1). */
/* Embeddings of GMCR pair `pair` after a count-all EXACT run (no reference
 * counterpart: the reference only counts).  Every injective induced embedding
 * the join counted, as n bytes each (n = the query's size): out[k * n + u] =
 * local data node mapped to query vertex u; sorted lexicographically, so the
 * output does not depend on the search order.  Writes min(found,
 * max_embeddings) embeddings; *n_embeddings receives how many exist. */
int bms_get_embeddings(bms_ctx* ctx, uint64_t pair, uint8_t* out, uint64_t max_embeddings, uint64_t* n_embeddings);
int bms_get_pair_counts(bms_ctx* ctx, uint64_t* counts, uint64_t cap);
/* Per-pair expansion counts in GMCR order. */
int bms_get_pair_expansions(bms_ctx* ctx, uint64_t* expansions, uint64_t cap);
int bms_get_pair_status(bms_ctx* ctx, uint8_t* status, uint64_t cap);
/* Candidates::getHostCandidates (candidates.hpp:181-186): the dense matrix,
 * n_query_nodes x ceil(n_data_nodes/32) uint32 words (staged pipeline only). */
int bms_get_candidates(bms_ctx* ctx, uint32_t* words, uint64_t cap);
/* Node signatures of one side.  Any pointer may be NULL.  label_gen[n],
 * path[4n], cycle[4n] (5-same, 5-diff, 6-same, 6-diff), shells[steps*n]
 * step-major. */
int bms_get_signatures(bms_ctx* ctx, int kind, uint64_t* label_gen, uint64_t* path, uint16_t* cycle,
                       uint64_t* shells);

/* ------------------------------------------------------ learned ordering */
/* 12 features per query vertex (see bms_feature_names), computed from the
 * loaded queries and the mapped pairs.  Requires bms_map or bms_run. */
#define BMS_NUM_FEATURES 12
#define BMS_MLP_HIDDEN 64
#define BMS_MLP_PARAMS (64 * 12 + 64 + 64 * 64 + 64 + 64 + 1)
const char* bms_feature_name(int i);
int bms_query_features(bms_ctx* ctx, float* features /* [n_query_nodes*12] */);
/* Per query vertex: total successful assignments at that vertex over all
 * mapped pairs in the last plain-order (BMS_ORDER_GMCR, BMS_SEM_EXACT) join. */
int bms_vertex_expansions(bms_ctx* ctx, uint64_t* expansions /* [n_query_nodes] */);
/* Train the cost model on the GPU with the library's own forward/backward and
 * Adam kernels: BF16 weights, FP32 accumulation, MSE loss.  x [n*12], y [n].
 * *final_loss (nullable) receives the last epoch's mean loss. */
int bms_model_train(bms_ctx* ctx, const float* x, const float* y, uint32_t n, uint32_t epochs, uint32_t batch,
                    float lr, uint64_t seed, float* final_loss);
/* One forward+backward on the GPU (for gradient checks): params in the
 * BMS_MLP_PARAMS layout W1[64x12] b1 W2[64x64] b2 w3 b3; outputs y[n] and
 * grad[BMS_MLP_PARAMS]. */
int bms_model_grad(bms_ctx* ctx, const float* params, const float* x, const float* y_target, uint32_t n,
                   float* y_out, float* grad, float* loss);
int bms_model_get(bms_ctx* ctx, float* params);
int bms_model_set(bms_ctx* ctx, const float* params);
int bms_model_save(bms_ctx* ctx, const char* path);
int bms_model_load(bms_ctx* ctx, const char* path);
/* Predicted log2 expansion cost per query vertex and the resulting per-query
 * order (order[n_query_nodes], local vertex ids, query by query). */
int bms_model_predict(bms_ctx* ctx, float* cost, uint8_t* order);
/* Explicit search orders for BMS_ORDER_GIVEN (no reference counterpart; the
 * reference searches in query-index order only): order[n_query_nodes], query
 * by query, order[qoff + t] = the local vertex searched at depth t; each
 * query's slice must be a permutation of 0..n-1.  Kept until the query side is
 * loaded again.  Like the learned order it only permutes the search (EXACT
 * semantics; counts are unchanged); the cost model's training logs the
 * expansions of candidate orders with it (bms_set_logging works for GMCR and
 * GIVEN orders). */
int bms_set_query_order(bms_ctx* ctx, const uint8_t* order, uint64_t n_query_nodes);

/* ------------------------------------------------------------ scheduling */
/* Schedule of the persistent join, one row per size bucket.  Bucket b holds
 * the (query, data graph) pairs whose data graph has at most max_data_nodes[b]
 * nodes (32, 64, 128; bucket 3 is unused); its search sets hold that many
 * bits, in machine words of word_bits[b] bits (32 or 64; bucket 0 always 32).
 * Per bucket: task granularity (split_depth 0 = one task per pair, 1 = one per
 * (pair, root)), lanes_per_pair (per-pair tasks: 1, 2, 4, 8, 16 or 32 lanes
 * share a pair, lane g of the group searching the roots of rank g modulo the
 * group size — 32 is one warp per pair, the reference's sub-group per task,
 * isomorphism.hpp:401), launch shape, DFS steps a warp runs between refills,
 * how many idle lanes trigger a refill, and the expansions after which a
 * search hands its unexplored subtrees to the next round (0 = never).
 * bms_autotune times candidate schedules of every bucket on the loaded
 * workload (each bucket's kernels timed on their own) and installs the
 * fastest; ms[b] is the bucket's join time under the chosen row.
 * BMS_OPT_JOIN_STEPS and BMS_OPT_SPLIT_BUDGET set their column for every bucket. */
#define BMS_SCHED_BUCKETS 4
typedef struct {
  uint32_t max_data_nodes[BMS_SCHED_BUCKETS]; /* read-only */
  uint32_t word_bits[BMS_SCHED_BUCKETS];      /* 32 or 64 (bucket 0: 32) */
  uint32_t split_depth[BMS_SCHED_BUCKETS];
  uint32_t blocks_per_sm[BMS_SCHED_BUCKETS];
  uint32_t warps_per_block[BMS_SCHED_BUCKETS]; /* 1..8 */
  uint32_t steps[BMS_SCHED_BUCKETS];
  uint32_t refill[BMS_SCHED_BUCKETS];          /* idle lanes of a warp that trigger a refill, 1..32 */
  uint32_t split_budget[BMS_SCHED_BUCKETS];
  uint32_t lanes_per_pair[BMS_SCHED_BUCKETS];  /* 1, 2, 4, 8, 16, 32 */
  float ms[BMS_SCHED_BUCKETS];
} bms_schedule;
int bms_get_schedule(bms_ctx* ctx, bms_schedule* out);
int bms_set_schedule(bms_ctx* ctx, const bms_schedule* s);
int bms_autotune(bms_ctx* ctx, int refine_steps, int mode, int order, bms_schedule* out);

#ifdef __cplusplus
}
#endif
#endif /* BMS_H */
