// Internal interfaces between the host runtime (api.cpp) and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace bms {

constexpr uint32_t kMaxDataNodes = 128;  // two 64-bit words per bitset row
constexpr uint32_t kMaxQueryNodes = 64;
constexpr int kMaxSteps = 8;
constexpr uint8_t kWildcard = 255;

// validation bits raised by the signature kernel
constexpr uint32_t kErrColumn = 1u;     // a column id outside its graph
constexpr uint32_t kErrAsym = 2u;       // adjacency is not symmetric (as a set)
constexpr uint32_t kErrTooLarge = 4u;   // graph exceeds the side's node limit
constexpr uint32_t kErrOverflow = 8u;   // an output buffer was too small
constexpr uint32_t kErrBudget = 16u;    // some task hit its expansion budget
constexpr uint32_t kErrRows = 32u;      // row offsets decrease or exceed the entry count

// A batched CSR on the device (DeviceBatchedCSRGraph, graph.hpp:58-66).
struct DGraphs {
  const uint32_t* goff;
  const uint32_t* rowp;
  const uint32_t* col;
  const uint8_t* lab;
  uint32_t G;
  uint64_t N;
  uint64_t E;  // CSR entries; row offsets beyond it are rejected
};

// Signatures of one side.  Each node has a 128-byte filter record, one cache
// line, holding everything the filter and refine stages compare:
//   w0  label | degree << 32        w1  cycle: 4 x uint16 (5-same, 5-diff, 6-same, 6-diff)
//   w2..w5  256-bit path filter     w6..w13  distance shells 1..8 (16 nibbles each)
//   w14 label signature (neighbour label counts)   w15 zero
// adj holds two 64-bit words per node: the set of local ids in the node's CSR
// row; adjin the set of local ids whose rows contain the node (equal to adj
// when the graph is symmetric).
constexpr int kRecWords = 16;
struct DSigs {
  uint64_t* frec;       // [N*16]
  uint64_t* adj;        // [N*2]
  uint64_t* adjin;      // [N*2]
  uint64_t* ghist;      // [G]   per-graph nibble histogram of labels < 16
  uint32_t* glabset;    // [G]   bit l: some node has label l (< 16)
  uint32_t* maxin;      // [2]   largest in-degree (distinct in-neighbours) of the side; the signatures
                        //       kernel's graph counter
  int R;
};

// One mapped (query, data graph) pair whose join is still to run.
struct PairRec {
  uint32_t q;
  uint32_t d;
  uint32_t gpos;   // position in GMCR order
  uint32_t c_row;  // first candidate row in the arena (rows of 2 x uint64)
};

// A join task: a pair and the local id of the root (first vertex of the order).
struct Task {
  uint32_t pair;
  uint32_t root;
};

// The join runs in rounds.  A search that passes the round's expansion budget
// writes every unexplored subtree it holds — the mapped prefix of its path and
// the candidates left at that depth — as one SubTask and stops; the next round
// runs those subtrees in parallel.  The last round has no budget.
constexpr int kJoinRounds = 6;
constexpr uint32_t kNoRecord = 0xFFFFFFFFu;  // a SubTask slot that holds nothing
struct SubTask {
  uint32_t rec;                   // record (pair) index, or kNoRecord
  uint32_t depth;                 // depth of the candidates; f[0..depth) is the prefix
  uint64_t cand[2];               // candidates left at that depth
  uint8_t f[kMaxQueryNodes];      // data node mapped at each depth of the prefix
};

// Per-query search order: perm[q*64 + t] is the vertex at depth t; dadj[q*64 + t]
// has bit i (i < t) set iff the vertex at depth i is in the CSR row of the
// vertex at depth t (the reference's query_adj_masks, isomorphism.hpp:383-390).
struct DOrder {
  uint8_t* perm;
  uint64_t* dadj;
};

// Device counters of one run, zeroed at its start.  The pipeline reads its
// sizes from here, so no stage waits for the host between launches.
struct Counters {
  unsigned long long recs;        // PairRecs written
  unsigned long long rows;        // candidate rows allocated in the arena
  unsigned long long tasks;       // join tasks emitted
  unsigned int work[4];           // pair-filter work heads, one per size class
  unsigned long long total;       // sum of per-pair counts
  unsigned long long expansions;  // sum of per-pair expansions
  unsigned long long incomplete;  // pairs that hit the expansion budget
  unsigned long long recs_wide;   // records [0, recs_wide) come from data graphs of > 64 nodes
  unsigned long long recs_mid;    // records [recs_wide, recs_mid) come from graphs of 33..64 nodes
  // join: work-stealing head per round and record class, subtrees per round
  unsigned long long join_head[kJoinRounds][3];
  unsigned long long sub_n[kJoinRounds + 1];
  // clustered join: prototype matches and the roots and pushes that found them,
  // data graphs taken
  unsigned long long partials;
  unsigned long long partial_exps;
  unsigned int cs_head;
  unsigned int cs_ghead;          // clustered join (EXACT): data graphs taken by the enumeration
  unsigned long long cs_n[3];     // clustered entries written per class
};

// Clustered join (the reference driver's --use-cs), REFERENCE_DFS semantics:
// query 0 is the prototype, `end` its node count.  One warp per data graph
// enumerates the prototype's matches from its candidate rows, then extends
// each with every query of the graph's GMCR row.  (EXACT runs in the join
// kernels: JoinArgs.cs_end.)
struct CsArgs {
  DGraphs q, d;
  DSigs qs, ds;
  DOrder o;                    // the plain order (position = query vertex)
  const PairRec* recs;
  const uint64_t* arena;
  const uint32_t* gmcr_off;    // [D + 1]
  const uint4* pos_desc;       // per GMCR position {record (kNoRecord: none), first row, query nodes, query}
  uint64_t rec_cap;            // entries of pos_desc (positions beyond: a run that overflowed)
  const uint32_t* dperm;       // data graphs in work order
  const uint32_t* dense;       // staged pipeline: dense candidate matrix (rows of a one-node prototype)
  uint64_t W;                  // its words per row
  uint32_t end;
  Counters* ctr;
  unsigned long long* pair_count;
  unsigned long long* pair_exp;
  uint32_t* pair_flag;
};

// ----------------------------------------------------------------- launchers
// All return cudaSuccess or the launch error.
int sm_count();
// kernels launched by this host thread (every launcher counts its launches)
extern thread_local unsigned long long g_launches;
inline void note_launch() { ++g_launches; }

cudaError_t launch_signatures(const DGraphs& g, DSigs s, uint32_t max_nodes, uint32_t* err, cudaStream_t st);

// Staged (reference-shaped) stages on the dense query-major candidate matrix.
cudaError_t launch_filter_dense(const DGraphs& q, const DSigs& qs, const DGraphs& d, const DSigs& ds, uint32_t* cand,
                                uint64_t W, cudaStream_t st);
cudaError_t launch_refine_dense(const DSigs& qs, uint64_t Qn, const DSigs& ds, uint64_t Dn, int step, uint32_t* cand,
                                uint64_t W, cudaStream_t st);
// GMCR validity from the dense matrix: valid bits [D][QW] and per-data-graph counts.
cudaError_t launch_gmcr_dense(const DGraphs& q, const DGraphs& d, const uint32_t* cand, uint64_t W, uint32_t* valid,
                              uint32_t QW, uint32_t* vcounts, cudaStream_t st);
// Staged path: number of query nodes of every GMCR pair, then one PairRec per
// pair with its candidate rows gathered from the dense matrix.
cudaError_t launch_pair_nodes(const DGraphs& q, const uint32_t* qidx, uint64_t T, uint32_t* nodes, cudaStream_t st);
cudaError_t launch_gather_pairs(const DGraphs& q, const DGraphs& d, const uint32_t* cand, uint64_t W,
                                const uint32_t* offsets, const uint32_t* qidx, const uint32_t* row_off, PairRec* recs,
                                uint64_t* arena, cudaStream_t st);
cudaError_t launch_set_counter(unsigned long long* dst, unsigned long long value, cudaStream_t st);

// Label totals over all data nodes (labels 0..255).
cudaError_t launch_label_count(const DGraphs& d, unsigned long long* counts, cudaStream_t st);
// Per query: vertex order of the validity test (rarest label first, then
// highest degree) and, per vertex, an earlier vertex with an identical filter
// record (0xFF if none).
cudaError_t launch_query_prep(const DGraphs& q, const DSigs& qs, const unsigned long long* label_count,
                              uint8_t* filter_order, uint8_t* dup, cudaStream_t st);

// Distance shells projected onto the labels that occur in the queries (a label
// absent from every query has a zero query nibble, which any data nibble
// satisfies): shell k keeps the K nibbles at positions pos[0..K-1]; with K <= 8
// two projected shells share one 64-bit word, else one shell per word.
struct ShellPack {
  uint32_t K;
  uint32_t PW;         // packed words per node
  uint8_t pos[16];
};
cudaError_t launch_pack_query_shells(const DGraphs& q, const DSigs& qs, ShellPack sp, uint64_t* qpack,
                                     cudaStream_t st);

// Fused filter + refine + GMCR validity for every (query, data graph) pair.
struct PairFilterArgs {
  DGraphs q, d;
  DSigs qs, ds;
  const uint8_t* filter_order;  // [Q*64]
  const uint8_t* dup;           // [Q*64] vertex with an identical record, earlier in the order, or 0xFF
  const uint64_t* qpack;        // [Qn*8] packed query shells
  ShellPack sp;
  const uint32_t* dperm;        // data graph ids grouped by size class
  uint32_t class_begin, class_end;
  int class_id;
  uint32_t* valid;              // [D][QW] GMCR validity bits
  uint32_t QW;
  uint32_t* vcounts;            // [D] valid pairs per data graph
  PairRec* recs;                // appended join-eligible pairs
  uint64_t rec_cap;
  uint64_t* arena;              // candidate rows, 2 words each
  uint64_t row_cap;
  Counters* ctr;
  uint32_t* err;
  int skip_by_labels;           // skip pairs whose label multiset cannot embed (EXACT only)
  unsigned int* cand_sum;       // nullable: per query node, sum of candidate-set sizes over records
};
cudaError_t launch_pair_filter(const PairFilterArgs& a, int rounds, cudaStream_t st);

// Bit-sliced fused filter (k_sliced.cu): per query node a clause program (mask
// ids), per data graph a shared-memory table of the used clause masks.
struct SlicedArgs {
  DGraphs q, d;
  DSigs qs, ds;
  const uint8_t* filter_order;  // [Q*64]
  const uint8_t* dup;           // [Q*64]
  const uint32_t* qorder;       // [Q] query ids by decreasing node count
  const uint2* desc;            // [Q*64] per (query, level): program groups, vertex, dup source, slow flags
  const uint4* screen;          // [Q] screen records in screening order (launch_screen)
  const uint32_t* prog_off;     // [Qn+1]
  const uint16_t* prog;         // compact mask indices
  const uint8_t* slow;          // [Qn] clauses outside the table
  const uint16_t* used_ids;     // compact index -> clause id
  const uint32_t* used_bits;    // [kClauseIds/32 + 1] bit id: some query uses clause id
  const uint16_t* remap;        // clause id -> compact index (used ids only)
  const uint32_t* n_used;       // number of used clauses (device)
  uint32_t n_used_cap;          // bound used to size shared memory
  ShellPack sp;
  const uint32_t* dperm;
  uint32_t class_begin, class_end;
  int class_id;
  uint32_t* valid;
  uint32_t QW;
  uint32_t* vcounts;
  PairRec* recs;
  uint64_t rec_cap;
  uint64_t* arena;
  uint64_t row_cap;
  Counters* ctr;
  uint32_t* err;
  int skip_by_labels;
};
constexpr uint32_t kClauseIds = 320 + kMaxSteps * 16 * 15;
cudaError_t launch_query_programs(const DGraphs& q, const DSigs& qs, ShellPack sp, uint32_t* len, uint32_t* prog_off,
                                  uint32_t* scan_scratch, uint32_t* used, uint16_t* remap, uint16_t* used_ids,
                                  uint32_t* n_used, uint16_t* prog, uint8_t* slow, uint64_t prog_cap,
                                  uint32_t* prog_total_host, cudaStream_t st);
size_t sliced_smem_bytes(const SlicedArgs& a, int words);
// Screen records of the sliced filter: query, size, label set and histogram in
// screening order (after the query signatures).
cudaError_t launch_screen(const DGraphs& q, const DSigs& qs, const uint32_t* qorder, uint4* screen, cudaStream_t st);
// Per (query, level) descriptors of the sliced filter (after query_prep and the programs).
cudaError_t launch_level_desc(const DGraphs& q, const uint8_t* filter_order, const uint8_t* dup,
                              const uint32_t* prog_off, const uint8_t* slow, uint2* desc, cudaStream_t st);
// words: 64-bit words per node mask (1: graphs of 33..64 nodes, 2: 65..128),
// or 0 for 32-bit masks (graphs of <= 32 nodes).
cudaError_t launch_sliced_filter(const SlicedArgs& a, int words, size_t smem, cudaStream_t st);

// exclusive scan of n uint32 values into out[0..n] (out[n] = total); scratch
// must hold scan_scratch_words(n) words.
size_t scan_scratch_words(uint64_t n);
cudaError_t launch_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* scratch, cudaStream_t st);
// Data graphs grouped by size class into dperm: 65..128 nodes first, then
// 33..64, then <= 32, each class in batch order.  scratch holds
// class_scratch_words(G) words.
uint64_t class_scratch_words(uint32_t G);
cudaError_t launch_size_classes(const uint32_t* goff, uint32_t G, uint32_t* scratch, uint32_t* dperm, cudaStream_t st);

// GMCR query indices from the valid bits and offsets.
cudaError_t launch_gmcr_indices(const uint32_t* valid, uint32_t QW, uint32_t Q, uint32_t D, const uint32_t* offsets,
                                uint32_t* qidx, cudaStream_t st);
// Fill in PairRec::gpos of records produced by the fused filter.
cudaError_t launch_pair_positions(PairRec* recs, const Counters* ctr, uint64_t rec_cap, const uint32_t* valid,
                                  uint32_t QW, const uint32_t* offsets, cudaStream_t st);

// Plain (query-index) order; depth adjacency of any order whose perm is set.
cudaError_t launch_plain_order(const DGraphs& q, DOrder o, cudaStream_t st);
cudaError_t launch_order_adjacency(const DGraphs& q, const DSigs& qs, DOrder o, cudaStream_t st);

// One task per root of every record under the order (atomic append).
cudaError_t launch_task_emit(const PairRec* recs, uint64_t rec_cap, const DGraphs& q, DOrder o, const uint64_t* arena,
                             Task* tasks, uint64_t task_cap, Counters* ctr, uint32_t* err, cudaStream_t st);

struct JoinArgs {
  DGraphs q, d;
  DSigs ds;  // adjacency rows of the data side
  DOrder o;
  const PairRec* recs;
  uint64_t rec_cap;
  const uint64_t* arena;
  const Task* tasks;               // (pair, root) tasks when per_pair == 0
  uint64_t task_cap;
  int per_pair;                    // 1: one task per record (all its roots)
  Counters* ctr;
  unsigned long long* pair_count;  // per record
  unsigned long long* pair_exp;    // per record
  uint32_t* pair_flag;             // per record: bit0 found (find-first), bit1 incomplete
  unsigned long long* vertex_exp;  // nullable: per query node expansions (plain-order logging)
  uint64_t budget;                 // 0 = unlimited
  int find_first;
  int literal;                     // REFERENCE_DFS semantics
  int steps;                       // DFS steps between refills
  uint32_t refill;                 // idle lanes of a warp that trigger a refill (1..32)
  SubTask* sub[2];                 // subtrees: round r reads sub[r & 1], writes sub[(r + 1) & 1]
  uint64_t sub_cap;                // entries of each subtree buffer
  uint32_t split_budget;           // expansions before a search splits (0: never)
  uint32_t lanes_log2;             // per-record tasks: 2^lanes_log2 lanes per record (root ranks g mod 2^lanes_log2)
  int round;                       // set by launch_join
  // Clustered join (EXACT): with cs_end > 0, round 0 first writes every
  // prototype match as entries (match, first member, data graph) per size
  // class, then the class kernels start each entry's members like subtrees
  // with the match as prefix.
  uint32_t cs_end;                 // prototype size (query 0), 0: plain join
  const uint32_t* gmcr_off;        // [D + 1]
  const uint4* pos_desc;           // per GMCR position {record (kNoRecord: none), first row, query nodes, query}
  const uint32_t* dperm;           // data graphs, largest class first
  DSigs qs;                        // query signatures (a one-node prototype's row)
  const uint32_t* dense;           // staged pipeline: dense candidate matrix, else null
  uint64_t dense_w;                // its words per row
  uint8_t* cs_ent[3];              // entries of each class: CsEntry header + the match's bytes
  uint64_t cs_cap;                 // entries each array holds
  uint32_t cs_stride;              // bytes per entry
  uint32_t* err;                   // overflow flag (kErrOverflow)
};
// Clustered entry: data graph, first member (index into the graph's GMCR row);
// the match's end bytes follow (padded to 8).
struct CsEntry {
  uint32_t d;
  uint32_t j0;
};
constexpr uint32_t kCsMembers = 32;  // members of the graph's GMCR row per entry
// Launch shape and task settings of one record class (size bucket) of the join.
struct ClassLaunch {
  int blocks, threads;
  int per_pair;           // 1: one task per record (or per lane of its group); 0: (pair, root) tasks
  int steps;              // DFS steps between refills
  uint32_t refill;        // idle lanes that trigger a refill
  uint32_t split_budget;  // 0: never split
  uint32_t lanes_log2;    // per-record tasks: 2^lanes_log2 lanes share a record's roots
  int word_bits;          // machine word of the search sets: 32 or 64
};
// All rounds of the join; the per-class fields of `a` come from cl[class].
// With timers, events [round][class][0/1] bracket each class's launches.
// Streams on which a round's three class kernels run side by side (the tail
// of one class fills with the blocks of the others); without them, or with
// timers, the classes run one after the other on `st`.
struct JoinStreams {
  cudaStream_t side[2];
  cudaEvent_t fork, done[2];
};
cudaError_t launch_join(const JoinArgs& a, const ClassLaunch cl[3], cudaStream_t st,
                        cudaEvent_t (*timers)[3][2] = nullptr, const JoinStreams* js = nullptr);

// Embeddings of one record (EXACT semantics): every mapping by query vertex.
struct EmbedArgs {
  DGraphs q, d;
  DSigs ds;
  DOrder o;
  const PairRec* recs;
  uint64_t rec;                // the record
  const uint64_t* arena;
  uint8_t* out;                // [cap * n]
  uint64_t cap;
  unsigned long long* count;   // embeddings found (may exceed cap)
};
// out = the index of the record at GMCR position gpos (unchanged if none)
// Descriptor of every GMCR position: {record, its first candidate row, query
// nodes, query}; positions without a record read kNoRecord.
cudaError_t launch_pos_desc(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, const DGraphs& q, uint4* desc,
                               cudaStream_t st);
cudaError_t launch_cs_join(const CsArgs& a, bool find_first, cudaStream_t st);  // REFERENCE_DFS
cudaError_t launch_find_record(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, uint32_t gpos,
                               unsigned long long* out, cudaStream_t st);
cudaError_t launch_embed(const EmbedArgs& a, cudaStream_t st);

// Totals over the records (count, expansions, incomplete pairs) into ctr.
cudaError_t launch_totals(const Counters* ctr_in, uint64_t rec_cap, const unsigned long long* pair_count,
                          const unsigned long long* pair_exp, const uint32_t* pair_flag, int find_first, Counters* ctr,
                          cudaStream_t st);
// Per-record results into GMCR order (arrays of T entries, zero-filled first).
// Batch slices: subtract the slice's first entry / node id from its row offsets
// and column ids.
cudaError_t launch_rebase(uint32_t* rowp, uint64_t n_rowp, uint32_t entry_base, uint32_t* col, uint64_t n_col,
                          uint32_t node_base, cudaStream_t st);
// per_query[q] += matches of the records with query q (find-first: 1 per record with a match).
cudaError_t launch_query_totals(const PairRec* recs, const Counters* ctr, uint64_t rec_cap,
                                const unsigned long long* pair_count, int find_first, uint32_t Q,
                                unsigned long long* per_query, cudaStream_t st);
cudaError_t launch_scatter(const PairRec* recs, const Counters* ctr, uint64_t rec_cap,
                           const unsigned long long* pair_count, const unsigned long long* pair_exp,
                           const uint32_t* pair_flag, int find_first, uint64_t* counts, uint64_t* exps,
                           uint8_t* status, cudaStream_t st);

// ------------------------------------------------------------- learned order
constexpr int kFeatures = 12;
constexpr int kHidden = 64;
constexpr int kParams = kHidden * kFeatures + kHidden + kHidden * kHidden + kHidden + kHidden + 1;
struct DFeatureArgs {
  DGraphs q;
  DSigs qs;
  const unsigned long long* label_count;  // [256] data nodes per label
  uint64_t data_nodes;
  const unsigned int* cand_sum;           // [Qn] sum over records of candidate-set sizes
  const unsigned int* recs_per_query;     // [Q]
  float* features;                        // [Qn * 12]
};
// Per query: number of records; per query node: sum of candidate-set sizes.
cudaError_t launch_record_stats(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, const DGraphs& q,
                                const uint64_t* arena, unsigned int* per_query, unsigned int* cand_sum,
                                cudaStream_t st);
cudaError_t launch_features(const DFeatureArgs& a, cudaStream_t st);
// Inference: cost per query node, then a per-query greedy connected order.
cudaError_t launch_mlp_predict(const float* features, uint64_t n, const uint16_t* wbf16, float* cost, cudaStream_t st);
cudaError_t launch_learned_order(const DGraphs& q, const DSigs& qs, const float* cost, DOrder o, cudaStream_t st);
// Training: forward + backward per 32-sample block into partial gradients,
// then a fixed-order reduction (deterministic).  n_total scales the MSE.
int mlp_grad_blocks(uint32_t n);
cudaError_t launch_mlp_grad(const float* x, const float* y, uint32_t n, uint32_t n_total, const uint16_t* wbf16,
                            float* grad_partial, float* pred, float* loss_partial, cudaStream_t st);
cudaError_t launch_mlp_reduce(const float* grad_partial, int blocks, float* grad, const float* loss_partial, float* loss,
                              uint32_t n, cudaStream_t st);
cudaError_t launch_adam(float* master, uint16_t* wbf16, const float* grad, float* m, float* v, float lr, float b1,
                        float b2, float eps, int step, cudaStream_t st);
cudaError_t launch_to_bf16(const float* master, uint16_t* wbf16, int n, cudaStream_t st);

}  // namespace bms
