// Context of libbms shared by the API translation units (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/bms.h"
#include "graphs.h"
#include "internal.h"

namespace bms {

// Counts device (re)allocations and frees of every DevBuf: a captured pipeline
// graph holds raw device pointers and stays valid only within one epoch.
extern std::atomic<unsigned long long> g_alloc_epoch;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  bool owned = true;  // false: a view into another buffer (never freed here)
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p && owned) cudaFree(p);
    if (p) ++g_alloc_epoch;
    p = nullptr;
    bytes = 0;
    owned = true;
  }
  // Make this buffer a view of `bytes` bytes at `q` (owned elsewhere).
  void alias(void* q, size_t b) {
    release();
    p = q;
    bytes = b;
    owned = false;
    ++g_alloc_epoch;
  }
  cudaError_t ensure(size_t b) {
    if (b <= bytes && p) return cudaSuccess;  // an owned buffer or a view that is large enough
    release();
    if (b == 0) b = 16;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    else p = nullptr;
    ++g_alloc_epoch;
    return e;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct Side {
  bool loaded = false;
  uint32_t G = 0;
  uint64_t N = 0, E = 0;
  uint32_t max_nodes = 0;
  std::vector<uint32_t> h_goff;
  std::vector<uint32_t> h_size_order;  // query side: graph ids by decreasing node count
  DevBuf goff, rowp, col, lab, size_order;  // edge labels stay on the host: matching never reads them
  DevBuf frec, adj, adjin, ghist, glabset, maxin;
  int sig_steps = -1;
  bool asymmetric = false;
  uint32_t labels_lt16 = 0;  // bit l: some node carries label l < 16
  DGraphs dg() const { return DGraphs{goff.as<uint32_t>(), rowp.as<uint32_t>(), col.as<uint32_t>(), lab.as<uint8_t>(), G, N, E}; }
  DSigs ds() const {
    return DSigs{frec.as<uint64_t>(), adj.as<uint64_t>(), adjin.as<uint64_t>(), ghist.as<uint64_t>(),
                 glabset.as<uint32_t>(), maxin.as<uint32_t>(), sig_steps < 0 ? 0 : sig_steps};
  }
};

enum Ev { EV_START, EV_SIG, EV_FILTER, EV_MAP, EV_ORDER, EV_JOIN, EV_END, EV_COUNT };

// Everything that decides what bms_run enqueues.  A captured graph of the
// pipeline is replayed only while the key is unchanged (compared bytewise;
// built from a zeroed object so padding compares equal).
struct PlanKey {
  unsigned long long load_gen, epoch;
  int R, mode, order, sem, filter_kernel, model_set, use_cs;
  unsigned long long given_gen;
  uint64_t sub_cap_opt, budget, rec_cap, row_cap, task_cap, sub_cap, cs_cap;
  bms_schedule sched;
};

}  // namespace bms

using bms::Counters;
using bms::DevBuf;
using bms::Side;
using bms::EV_COUNT;
using bms::PlanKey;

struct bms_ctx {
  int device = 0;
  cudaStream_t own = nullptr, st = nullptr;
  std::string err;
  Side q, d;
  DevBuf errflag;  // [0] data side, [1] query side, [2] run
  uint32_t* h_err = nullptr;
  DevBuf ctr;
  Counters* h_ctr = nullptr;
  uint32_t* h_T = nullptr;
  // staged dense matrix
  DevBuf cand;
  uint64_t W = 0;
  bool have_cand = false;
  // mapping
  DevBuf valid, vcounts, gmcr_off, qidx, scan_scratch, row_off, pair_nodes;
  uint32_t QW = 0;
  bool mapped = false, have_qidx = false;
  uint64_t T = 0;
  // records and join
  DevBuf recs, arena, tasks, pair_count, pair_exp, pair_flag;
  DevBuf sub[2];  // join subtrees, ping-pong between rounds
  Side dres;         // resident data batch (bms_load_resident); the data side views windows of it
  DevBuf per_query;  // bms_run_batches: per-query totals
  DevBuf level_desc;  // sliced filter: per (query, level) descriptors
  DevBuf screen;      // sliced filter: per-query screen records
  DevBuf embed_out, embed_tmp;  // bms_get_embeddings
  DevBuf pos_desc;              // clustered join: descriptor of each GMCR position
  DevBuf cs_ent[3];             // clustered join (EXACT): entries per size class
  uint64_t cs_cap = 0;          // entries each of cs_ent holds (grown on overflow)
  bool use_cs = false;          // BMS_OPT_USE_CS
  bool last_cs = false;         // the last join was the clustered join
  uint64_t sub_cap = 0;
  uint64_t sub_cap_opt = 0;  // BMS_OPT_SUBTREE_CAP (0: automatic)
  uint64_t rec_cap = 0, row_cap = 0, task_cap = 0;
  DevBuf dperm;
  DevBuf class_scratch;  // tile counts and scans of the size-class partition
  uint32_t class_begin[3] = {0, 0, 0}, class_end[3] = {0, 0, 0};
  DevBuf filter_order, filter_dup, qpack, prog_len, prog_off, prog, prog_slow, prog_used, prog_remap, prog_ids, prog_nused, label_count, perm, dadj, vertex_exp, cand_sum, recs_per_query, features, cost;
  bool have_results = false, have_vexp = false;
  int last_mode = 0, last_order = 0, last_sem = 0;
  DevBuf tmp;
  // cost model
  DevBuf model_master, model_bf16, adam_m, adam_v, grad, grad_partial, loss_buf, train_x, train_y, pred;
  bool model_set = false;
  // BMS_ORDER_GIVEN: per-query orders in the perm layout ([Q][64] bytes)
  DevBuf given_perm;
  bool given_set = false;
  unsigned long long given_gen = 0;
  bool log_vertices = false;
  int filter_kernel = 0;  // BMS_FILTER_SLICED or BMS_FILTER_BALLOT
  uint64_t budget = 0;
  bms_schedule sched{};
  cudaEvent_t class_ev[bms::kJoinRounds][3][2] = {};  // per-class join timers of the autotuner
  bms::JoinStreams join_streams{};  // side streams of the join's class kernels (created on first use)
  bool join_streams_failed = false;
  // BMS_OPT_RESIDENT_SIGNATURES: data-side signatures of the resident batch,
  // computed once for dres_sig_R refine steps (-1: none), with their error bits
  bool resident_sigs = false;
  int dres_sig_R = -1;
  DevBuf dres_err;
  bool d_sig_cached = false;  // the data side is a window whose signatures are cached
  // CUDA graph of the fused pipeline (BMS_OPT_CUDA_GRAPH)
  bool use_graph = true;
  unsigned long long load_gen = 0;  // bumped by every upload
  PlanKey plan_key{};
  bool plan_warm = false;           // an eager run with plan_key completed
  bool capture_failed = false;      // capturing plan_key failed: run it eagerly
  cudaGraph_t plan_graph = nullptr;
  cudaGraphExec_t plan_exec = nullptr;
  unsigned long long plan_launches = 0;  // kernels in the graph
  cudaEvent_t ev[EV_COUNT] = {};
  bms_stats stats{};
};


namespace bms {
int fail(bms_ctx* c, int code, const std::string& msg);
int fail_cuda(bms_ctx* c, cudaError_t e, const char* what);
// learned order of every query from the current records (needs a model);
// fills c->perm (the caller derives the depth adjacency)
int learned_order(bms_ctx* c);
// per-vertex features of the current records into c->features
int compute_features(bms_ctx* c);
// re-run the join over the tasks of the last run with a given launch shape
// The join alone over the current records with schedule `sched` (EXACT
// semantics): total and per-class milliseconds.
int rejoin_timed(bms_ctx* c, const bms_schedule& sched, float* ms, float class_ms[3]);
// Buckets 0..2 = data graphs of <= 32, <= 64, <= 128 nodes; defaults.
bms_schedule default_schedule();
}  // namespace bms

#define CK(call)                                                   \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return bms::fail_cuda(c, e_, #call);    \
  } while (0)

#define GUARD(c)                                                        \
  if (!(c)) return bms::fail(nullptr, BMS_EINVAL, "null context");      \
  if (cudaSetDevice((c)->device) != cudaSuccess) return bms::fail(c, BMS_ECUDA, "cudaSetDevice failed");
