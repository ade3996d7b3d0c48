// C ABI of libbms: contexts, uploads, the staged and fused pipelines, results.
// Every entry point catches everything: no exception crosses the boundary.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/bms.h"
#include "graphs.h"
#include "internal.h"

using namespace bms;

#include "ctx.h"

namespace bms {

std::atomic<unsigned long long> g_alloc_epoch{0};

bms_schedule default_schedule() {
  bms_schedule s;
  std::memset(&s, 0, sizeof s);
  const uint32_t nodes[3] = {32, 64, 128};
  for (int i = 0; i < 3; ++i) {
    s.max_data_nodes[i] = nodes[i];
    s.word_bits[i] = 32;  // measured faster than 64-bit words on every bucket
    s.lanes_per_pair[i] = 1;
    s.split_depth[i] = 0;
    s.blocks_per_sm[i] = 3;
    s.warps_per_block[i] = 8;
    s.steps[i] = 32;
    s.refill[i] = 4;
    s.split_budget[i] = 1024;
  }
  return s;
}

int fail(bms_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  bms::set_thread_error(msg);
  return code;
}
int fail_cuda(bms_ctx* c, cudaError_t e, const char* what) {
  cudaGetLastError();
  return fail(c, e == cudaErrorMemoryAllocation ? BMS_ENOMEM : BMS_ECUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace bms

namespace {

// Timing events are recorded as external event nodes while the stream is being
// captured into the pipeline graph, plainly otherwise (the external flag is
// only valid during a capture).
cudaError_t record_event(bms_ctx* c, Ev e) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const cudaError_t r = cudaStreamIsCapturing(c->st, &cs);
  if (r != cudaSuccess) return r;
  return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(c->ev[e], c->st, cudaEventRecordExternal)
                                             : cudaEventRecord(c->ev[e], c->st);
}

void drop_plan(bms_ctx* c);

int check_side_errors(bms_ctx* c, const char* side, uint32_t e) {
  if (e & kErrRows) return fail(c, BMS_EINVAL, std::string(side) + ": row offsets decrease or exceed the entry count");
  if (e & kErrColumn) return fail(c, BMS_EINVAL, std::string(side) + ": a column id lies outside its graph");
  if (e & kErrTooLarge) return fail(c, BMS_EUNSUPPORTED, std::string(side) + ": a graph exceeds the node limit");
  return BMS_OK;
}

// Upload a batch.  With `slice` the view is a window of a larger batch: its
// offsets and column ids are global, graph_offsets[0] and row_offsets[0] give
// the window's first node and entry, and the ids are rebased on the device.
// Drop the buffers of a side that are views of the resident batch.
void release_views(Side& s) {
  for (DevBuf* b : {&s.goff, &s.rowp, &s.col, &s.lab, &s.frec, &s.adj, &s.adjin, &s.ghist, &s.glabset,
                    &s.maxin, &s.size_order})
    if (!b->owned) b->release();
}

int upload(bms_ctx* c, Side& s, const bms_graphs_view& v, uint32_t limit, const char* name, bool slice = false) {
  if (v.n_graphs && !v.graph_offsets) return fail(c, BMS_EINVAL, "graph_offsets is null");
  release_views(s);
  const uint32_t G = v.n_graphs;
  const uint32_t node_base = slice && G ? v.graph_offsets[0] : 0;
  if (G && v.graph_offsets[0] != node_base) return fail(c, BMS_EINVAL, "graph_offsets[0] must be 0");
  if (G && v.graph_offsets[G] < node_base) return fail(c, BMS_EINVAL, "graph_offsets must be non-decreasing");
  const uint64_t N = G ? v.graph_offsets[G] - node_base : 0;
  if (N && (!v.row_offsets || !v.node_labels)) return fail(c, BMS_EINVAL, "row_offsets or node_labels is null");
  const uint32_t entry_base = slice && N ? v.row_offsets[0] : 0;
  // checked before anything is sized or copied: a last offset below the first
  // would wrap the entry count and over-read the caller's column array
  if (N && v.row_offsets[N] < entry_base) return fail(c, BMS_EINVAL, "row_offsets must be non-decreasing");
  const uint64_t E = N ? uint64_t(v.row_offsets[N]) - entry_base : 0;
  if (N && v.row_offsets[0] != entry_base) return fail(c, BMS_EINVAL, "row_offsets[0] must be 0");
  if (E && !v.column_indices) return fail(c, BMS_EINVAL, "column_indices is null");
  s.loaded = false;
  s.sig_steps = -1;
  if (&s == &c->d) c->d_sig_cached = false;  // an upload replaces a resident window
  ++c->load_gen;
  // the large arrays first: their copies run while the host checks the offsets
  // (a batch that fails the checks leaves the side unloaded)
  CK(s.goff.ensure(sizeof(uint32_t) * (G + 1)));
  CK(s.rowp.ensure(sizeof(uint32_t) * (N + 1)));
  CK(s.col.ensure(sizeof(uint32_t) * (E ? E : 1)));
  CK(s.lab.ensure(N ? N : 1));
  if (E) {
    CK(cudaMemcpyAsync(s.col.p, v.column_indices, sizeof(uint32_t) * E, cudaMemcpyHostToDevice, c->st));
    // edge labels are never read by matching (the reference ignores them too,
    // isomorphism.hpp:30-472): they are accepted but not copied to the device
  }
  if (N) {
    CK(cudaMemcpyAsync(s.rowp.p, v.row_offsets, sizeof(uint32_t) * (N + 1), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(s.lab.p, v.node_labels, N, cudaMemcpyHostToDevice, c->st));
  } else {
    CK(cudaMemsetAsync(s.rowp.p, 0, sizeof(uint32_t), c->st));
  }
  uint32_t mx = 0, dec = 0;  // one branch-free pass
  for (uint32_t i = 0; i < G; ++i) {
    const uint32_t a = v.graph_offsets[i], b = v.graph_offsets[i + 1];
    dec |= uint32_t(b < a);
    mx = std::max(mx, b - a);
  }
  if (dec || mx > limit) {
    cudaStreamSynchronize(c->st);  // the caller's arrays are free again once this returns
    if (dec) return fail(c, BMS_EINVAL, "graph_offsets must be non-decreasing");
    return fail(c, BMS_EUNSUPPORTED,
                std::string(name) + " graph with " + std::to_string(mx) + " nodes exceeds the limit of " + std::to_string(limit));
  }
  s.G = G;
  s.N = N;
  s.E = E;
  s.max_nodes = mx;
  s.h_goff.assign(v.graph_offsets, v.graph_offsets + G + 1);
  if (node_base)
    for (auto& x : s.h_goff) x -= node_base;
  if (&s == &c->q) c->given_set = false;  // explicit orders belong to the queries they were set for
  s.labels_lt16 = 0;  // the query side's label set packs the shell clauses
  if (&s == &c->q)
    for (uint64_t i = 0; i < N; ++i)
      if (v.node_labels[i] < 16) s.labels_lt16 |= 1u << v.node_labels[i];
  if (!G) s.h_goff.assign(1, 0);
  // offsets that need no rebasing go straight from the caller's array (no
  // staging pass when it is page-locked, like the other arrays)
  CK(cudaMemcpyAsync(s.goff.p, G && !node_base ? v.graph_offsets : s.h_goff.data(), sizeof(uint32_t) * (G + 1),
                     cudaMemcpyHostToDevice, c->st));
  if (&s == &c->q) {  // the fused filter screens queries longest first
    s.h_size_order.resize(G);
    for (uint32_t i = 0; i < G; ++i) s.h_size_order[i] = i;
    std::stable_sort(s.h_size_order.begin(), s.h_size_order.end(), [&](uint32_t x, uint32_t y) {
      return s.h_goff[x + 1] - s.h_goff[x] > s.h_goff[y + 1] - s.h_goff[y];
    });
    CK(s.size_order.ensure(sizeof(uint32_t) * (G ? G : 1)));
    if (G)
      CK(cudaMemcpyAsync(s.size_order.p, s.h_size_order.data(), sizeof(uint32_t) * G, cudaMemcpyHostToDevice, c->st));
  }
  if (N) CK(launch_rebase(s.rowp.as<uint32_t>(), N + 1, entry_base, s.col.as<uint32_t>(), E, node_base, c->st));
  CK(s.frec.ensure(sizeof(uint64_t) * kRecWords * (N ? N : 1)));
  CK(s.adj.ensure(sizeof(uint64_t) * 2 * (N ? N : 1)));
  CK(s.adjin.ensure(sizeof(uint64_t) * 2 * (N ? N : 1)));
  CK(s.ghist.ensure(sizeof(uint64_t) * (G ? G : 1)));
  CK(s.glabset.ensure(sizeof(uint32_t) * (G ? G : 1)));
  CK(s.maxin.ensure(2 * sizeof(uint32_t)));  // in-degree bound, graph counter of the signatures kernel
  s.loaded = true;
  return BMS_OK;
}

void invalidate_downstream(bms_ctx* c) {
  c->have_cand = false;
  c->mapped = false;
  c->have_qidx = false;
  c->have_results = false;
  c->have_vexp = false;
}

// Data graphs grouped by size class, largest class first (it carries the most
// work): 65..128 nodes, 33..64, then <= 32 (empty graphs included), each class
// in batch order.  The host counts the classes (the launches need their
// bounds); the permutation itself is built on the device.
int build_classes(bms_ctx* c) {
  const uint32_t G = c->d.G;
  const uint32_t* go = c->d.h_goff.data();
  uint32_t gt32 = 0, gt64 = 0;
  for (uint32_t g = 0; g < G; ++g) {
    const uint32_t m = go[g + 1] - go[g];
    gt32 += uint32_t(m > 32);
    gt64 += uint32_t(m > 64);
  }
  const uint32_t count[3] = {G - gt32, gt32 - gt64, gt64};
  c->class_begin[2] = 0;
  c->class_begin[1] = count[2];
  c->class_begin[0] = count[2] + count[1];
  for (int k = 0; k < 3; ++k) c->class_end[k] = c->class_begin[k] + count[k];
  CK(c->dperm.ensure(sizeof(uint32_t) * (G ? G : 1)));
  if (!G) return BMS_OK;
  CK(c->class_scratch.ensure(sizeof(uint32_t) * class_scratch_words(G)));
  CK(launch_size_classes(c->d.dg().goff, G, c->class_scratch.as<uint32_t>(), c->dperm.as<uint32_t>(), c->st));
  return BMS_OK;
}

int run_signatures(bms_ctx* c, int R) {
  CK(cudaMemsetAsync(c->errflag.p, 0, 4 * sizeof(uint32_t), c->st));
  Side* sides[2] = {&c->d, &c->q};
  for (int i = 0; i < 2; ++i) {
    Side& s = *sides[i];
    s.sig_steps = R;
    if (i == 0 && c->d_sig_cached && c->dres_sig_R == R) {  // computed once for the resident batch
      CK(cudaMemcpyAsync(c->errflag.p, c->dres_err.p, sizeof(uint32_t), cudaMemcpyDeviceToDevice, c->st));
      continue;
    }
    CK(cudaMemsetAsync(s.maxin.p, 0, 2 * sizeof(uint32_t), c->st));
    CK(launch_signatures(s.dg(), s.ds(), i == 0 ? kMaxDataNodes : kMaxQueryNodes, c->errflag.as<uint32_t>() + i, c->st));
  }
  return BMS_OK;
}

int read_side_errors(bms_ctx* c) {
  CK(cudaMemcpyAsync(c->h_err, c->errflag.p, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->d.asymmetric = (c->h_err[0] & kErrAsym) != 0;
  c->q.asymmetric = (c->h_err[1] & kErrAsym) != 0;
  int r = check_side_errors(c, "data", c->h_err[0]);
  if (r) {
    c->d.sig_steps = -1;
    return r;
  }
  r = check_side_errors(c, "query", c->h_err[1]);
  if (r) {
    c->q.sig_steps = -1;
    return r;
  }
  return BMS_OK;
}

int ensure_join_buffers(bms_ctx* c) {
  CK(c->recs.ensure(sizeof(PairRec) * (c->rec_cap ? c->rec_cap : 1)));
  CK(c->arena.ensure(sizeof(uint64_t) * 2 * (c->row_cap ? c->row_cap : 1)));
  CK(c->tasks.ensure(sizeof(Task) * (c->task_cap ? c->task_cap : 1)));
  CK(c->pair_count.ensure(sizeof(unsigned long long) * (c->rec_cap ? c->rec_cap : 1)));
  CK(c->pair_exp.ensure(sizeof(unsigned long long) * (c->rec_cap ? c->rec_cap : 1)));
  CK(c->pair_flag.ensure(sizeof(uint32_t) * (c->rec_cap ? c->rec_cap : 1)));
  // subtree buffers: one entry per record up to 4M entries (352 MiB each); a
  // search that finds no room keeps its work instead of splitting
  c->sub_cap = c->sub_cap_opt ? c->sub_cap_opt : std::min<uint64_t>(std::max<uint64_t>(c->rec_cap, 1 << 16), 1 << 22);
  for (auto& b : c->sub) CK(b.ensure(sizeof(SubTask) * c->sub_cap));
  return BMS_OK;
}

DOrder order_of(bms_ctx* c) { return DOrder{c->perm.as<uint8_t>(), c->dadj.as<uint64_t>()}; }

// One task per pair, or per (pair, root) where the schedule splits pairs; the
// literal reference DFS restarts its visited set per root, so it always splits.
bool needs_tasks(const bms_schedule& s, int sem) {
  if (sem == BMS_SEM_REFERENCE_DFS) return true;
  for (int k = 0; k < 3; ++k)
    if (s.split_depth[k] >= 1) return true;
  return false;
}

void class_launches(const bms_schedule& s, int sem, ClassLaunch cl[3]) {
  for (int k = 0; k < 3; ++k) {
    cl[k].blocks = sm_count() * int(s.blocks_per_sm[k] ? s.blocks_per_sm[k] : 3);
    cl[k].threads = 32 * int(s.warps_per_block[k] ? s.warps_per_block[k] : 8);
    cl[k].per_pair = (sem == BMS_SEM_REFERENCE_DFS || s.split_depth[k] >= 1) ? 0 : 1;
    cl[k].steps = int(s.steps[k] ? s.steps[k] : 32);
    cl[k].refill = s.refill[k] ? (s.refill[k] > 32 ? 32u : s.refill[k]) : 4u;
    cl[k].split_budget = s.split_budget[k];
    uint32_t lg = 0;
    while (lg < 5 && (1u << (lg + 1)) <= s.lanes_per_pair[k]) ++lg;
    cl[k].lanes_log2 = lg;
    cl[k].word_bits = k == 0 || s.word_bits[k] == 32 ? 32 : 64;
  }
}

// The join arguments shared by every record class (the per-class ones come
// from class_launches).
JoinArgs join_args(bms_ctx* c, int mode, int sem, bool log_vertices) {
  JoinArgs ja{};
  ja.q = c->q.dg();
  ja.d = c->d.dg();
  ja.ds = c->d.ds();
  ja.o = order_of(c);
  ja.recs = c->recs.as<PairRec>();
  ja.arena = c->arena.as<uint64_t>();
  ja.rec_cap = c->rec_cap;
  ja.tasks = c->tasks.as<Task>();
  ja.task_cap = c->task_cap;
  ja.ctr = c->ctr.as<Counters>();
  ja.pair_count = c->pair_count.as<unsigned long long>();
  ja.pair_exp = c->pair_exp.as<unsigned long long>();
  ja.pair_flag = c->pair_flag.as<uint32_t>();
  ja.vertex_exp = log_vertices ? c->vertex_exp.as<unsigned long long>() : nullptr;
  ja.budget = c->budget;
  ja.find_first = mode == BMS_FIND_FIRST;
  ja.literal = sem == BMS_SEM_REFERENCE_DFS;
  ja.sub[0] = c->sub[0].as<SubTask>();
  ja.sub[1] = c->sub[1].as<SubTask>();
  ja.sub_cap = c->sub_cap;
  return ja;
}

// Side streams and fork/join events of the join (created once per context; a
// creation failure leaves the classes on the main stream).
const JoinStreams* join_streams(bms_ctx* c) {
  JoinStreams& js = c->join_streams;
  if (c->join_streams_failed) return nullptr;
  if (!js.fork) {
    bool ok = true;
    for (auto& s : js.side) ok = ok && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess;
    for (auto& e : js.done) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&js.fork, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      c->join_streams_failed = true;  // the objects created so far are released by bms_destroy
      return nullptr;
    }
  }
  return &js;
}

// The clustered join applies when it is switched on and query 0 has nodes
// (the reference driver keeps the plain join for a depth of 0, BMS2.cpp:233).
bool cs_active(const bms_ctx* c) {
  return c->use_cs && c->q.G > 0 && c->q.h_goff.size() > 1 && c->q.h_goff[1] > c->q.h_goff[0];
}

// Clustered join over the records in place: GMCR position -> record, then
// EXACT: round 0 of the join kernels takes data graphs (prototype matches
// extended by the join's own steps, long searches split into later rounds);
// REFERENCE_DFS: one warp per data graph restating both reference loops
// (k_cs.cu).  `dense`: the staged pipeline's matrix.
int cs_join(bms_ctx* c, int mode, int sem, const uint32_t* dense) {
  CK(c->pos_desc.ensure(sizeof(uint4) * (c->rec_cap ? c->rec_cap : 1)));
  Counters* ctr = c->ctr.as<Counters>();
  CK(launch_pos_desc(c->recs.as<PairRec>(), ctr, c->rec_cap, c->q.dg(), c->pos_desc.as<uint4>(), c->st));
  const uint32_t end = c->q.h_goff[1] - c->q.h_goff[0];
  if (sem == BMS_SEM_EXACT) {
    JoinArgs ja = join_args(c, mode, sem, false);
    ja.cs_end = end;
    ja.gmcr_off = c->gmcr_off.as<uint32_t>();
    ja.pos_desc = c->pos_desc.as<uint4>();
    ja.dperm = c->dperm.as<uint32_t>();
    ja.qs = c->q.ds();
    ja.dense = dense;
    ja.dense_w = c->W;
    // entries: header + the match's bytes padded to 8, one array per class
    ja.cs_stride = uint32_t(sizeof(CsEntry)) + ((end + 7u) & ~7u);
    if (c->cs_cap == 0) c->cs_cap = std::max<uint64_t>(1 << 16, c->rec_cap);
    ja.cs_cap = c->cs_cap;
    for (int k = 0; k < 3; ++k) {
      CK(c->cs_ent[k].ensure(uint64_t(ja.cs_stride) * c->cs_cap));
      ja.cs_ent[k] = c->cs_ent[k].as<uint8_t>();
    }
    ja.err = c->errflag.as<uint32_t>() + 2;
    ClassLaunch cl[3];
    class_launches(c->sched, sem, cl);
    CK(launch_join(ja, cl, c->st, nullptr, join_streams(c)));
    return BMS_OK;
  }
  CsArgs a{};
  a.q = c->q.dg();
  a.d = c->d.dg();
  a.qs = c->q.ds();
  a.ds = c->d.ds();
  a.o = order_of(c);
  a.recs = c->recs.as<PairRec>();
  a.arena = c->arena.as<uint64_t>();
  a.gmcr_off = c->gmcr_off.as<uint32_t>();
  a.pos_desc = c->pos_desc.as<uint4>();
  a.rec_cap = c->rec_cap;
  a.dperm = c->dperm.as<uint32_t>();
  a.dense = dense;
  a.W = c->W;
  a.end = end;
  a.ctr = ctr;
  a.pair_count = c->pair_count.as<unsigned long long>();
  a.pair_exp = c->pair_exp.as<unsigned long long>();
  a.pair_flag = c->pair_flag.as<uint32_t>();
  CK(launch_cs_join(a, mode == BMS_FIND_FIRST, c->st));
  return BMS_OK;
}

// Order, tasks, join and totals over the records already in place.  `dense`
// (staged pipeline) is the candidate matrix the records were gathered from.
int join_records(bms_ctx* c, int mode, int order, int sem, bool log_vertices, const uint32_t* dense) {
  const uint64_t Qslots = uint64_t(c->q.G ? c->q.G : 1) * kMaxQueryNodes;
  CK(c->perm.ensure(Qslots));
  CK(c->dadj.ensure(sizeof(uint64_t) * Qslots));
  if (order == BMS_ORDER_LEARNED) {
    int r = learned_order(c);
    if (r) return r;
  } else if (order == BMS_ORDER_GIVEN) {
    CK(cudaMemcpyAsync(c->perm.p, c->given_perm.p, Qslots, cudaMemcpyDeviceToDevice, c->st));
  } else {
    CK(launch_plain_order(c->q.dg(), order_of(c), c->st));
  }
  CK(launch_order_adjacency(c->q.dg(), c->q.ds(), order_of(c), c->st));
  CK(record_event(c, EV_ORDER));
  CK(cudaMemsetAsync(c->pair_count.p, 0, sizeof(unsigned long long) * c->rec_cap, c->st));
  CK(cudaMemsetAsync(c->pair_exp.p, 0, sizeof(unsigned long long) * c->rec_cap, c->st));
  CK(cudaMemsetAsync(c->pair_flag.p, 0, sizeof(uint32_t) * c->rec_cap, c->st));
  Counters* ctr = c->ctr.as<Counters>();
  c->last_cs = cs_active(c);
  if (c->last_cs) {
    const int r = cs_join(c, mode, sem, dense);
    if (r) return r;
    CK(record_event(c, EV_JOIN));
    CK(launch_totals(ctr, c->rec_cap, c->pair_count.as<unsigned long long>(), c->pair_exp.as<unsigned long long>(),
                     c->pair_flag.as<uint32_t>(), mode == BMS_FIND_FIRST, ctr, c->st));
    c->last_mode = mode;
    c->last_order = order;
    c->last_sem = sem;
    return BMS_OK;
  }
  if (needs_tasks(c->sched, sem))
    CK(launch_task_emit(c->recs.as<PairRec>(), c->rec_cap, c->q.dg(), order_of(c), c->arena.as<uint64_t>(),
                        c->tasks.as<Task>(), c->task_cap, ctr, c->errflag.as<uint32_t>() + 2, c->st));
  if (log_vertices) {
    CK(c->vertex_exp.ensure(sizeof(unsigned long long) * (c->q.N ? c->q.N : 1)));
    CK(cudaMemsetAsync(c->vertex_exp.p, 0, sizeof(unsigned long long) * (c->q.N ? c->q.N : 1), c->st));
  }
  const JoinArgs ja = join_args(c, mode, sem, log_vertices);
  ClassLaunch cl[3];
  class_launches(c->sched, sem, cl);
  CK(launch_join(ja, cl, c->st, nullptr, join_streams(c)));
  CK(record_event(c, EV_JOIN));
  CK(launch_totals(ctr, c->rec_cap, ja.pair_count, ja.pair_exp, ja.pair_flag, ja.find_first, ctr, c->st));
  c->last_mode = mode;
  c->last_order = order;
  c->last_sem = sem;
  return BMS_OK;
}

int finish_run(bms_ctx* c, uint64_t* total) {
  CK(record_event(c, EV_END));
  CK(cudaMemcpyAsync(c->h_ctr, c->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(c->h_err, c->errflag.p, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(c->h_T, c->gmcr_off.as<uint32_t>() + c->d.G, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return BMS_OK;
  (void)total;
}

float elapsed(bms_ctx* c, Ev a, Ev b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]) != cudaSuccess) {
    cudaGetLastError();
    return 0.f;
  }
  return ms;
}

int validate_modes(bms_ctx* c, int mode, int order, int sem) {
  if (mode != BMS_FIND_FIRST && mode != BMS_COUNT_ALL) return fail(c, BMS_EINVAL, "invalid mode");
  if (order != BMS_ORDER_GMCR && order != BMS_ORDER_LEARNED && order != BMS_ORDER_GIVEN)
    return fail(c, BMS_EINVAL, "invalid order");
  if (order == BMS_ORDER_GIVEN && !c->given_set)
    return fail(c, BMS_ESTATE, "BMS_ORDER_GIVEN: set the orders of the loaded queries with bms_set_query_order");
  if (sem != BMS_SEM_EXACT && sem != BMS_SEM_REFERENCE_DFS) return fail(c, BMS_EINVAL, "invalid semantics");
  if (sem == BMS_SEM_REFERENCE_DFS && order != BMS_ORDER_GMCR)
    return fail(c, BMS_EINVAL, "REFERENCE_DFS semantics require the GMCR order");
  if (c->use_cs && order != BMS_ORDER_GMCR)
    return fail(c, BMS_EINVAL, "the clustered join extends the prototype's nodes first: it requires the GMCR order");
  if (order != BMS_ORDER_GMCR && (c->q.asymmetric || c->d.asymmetric))
    return fail(c, BMS_EINVAL, "a search order other than the GMCR order requires symmetric adjacency");
  return BMS_OK;
}

int run_fused(bms_ctx* c, int R, int mode, int order, int sem, uint64_t* total, bool log_vertices, int attempt);

int run_ballot_filter(bms_ctx* c, const ShellPack& sp, int sem) {
  PairFilterArgs pa{};
  pa.qpack = c->qpack.as<uint64_t>();
  pa.sp = sp;
  pa.q = c->q.dg();
  pa.d = c->d.dg();
  pa.qs = c->q.ds();
  pa.ds = c->d.ds();
  pa.filter_order = c->filter_order.as<uint8_t>();
  pa.dup = c->filter_dup.as<uint8_t>();
  pa.dperm = c->dperm.as<uint32_t>();
  pa.valid = c->valid.as<uint32_t>();
  pa.QW = c->QW;
  pa.vcounts = c->vcounts.as<uint32_t>();
  pa.recs = c->recs.as<PairRec>();
  pa.rec_cap = c->rec_cap;
  pa.arena = c->arena.as<uint64_t>();
  pa.row_cap = c->row_cap;
  pa.ctr = c->ctr.as<Counters>();
  pa.err = c->errflag.as<uint32_t>() + 2;
  pa.skip_by_labels = sem == BMS_SEM_EXACT && !c->use_cs;
  pa.cand_sum = nullptr;
  const int rounds[3] = {1, 2, 4};
  for (int k = 2; k >= 0; --k) {
    pa.class_begin = c->class_begin[k];
    pa.class_end = c->class_end[k];
    pa.class_id = k;
    CK(launch_pair_filter(pa, rounds[k], c->st));
    // record class boundaries: > 64 nodes, then 33..64 nodes, then the rest
    if (k > 0)
      CK(cudaMemcpyAsync(k == 2 ? &pa.ctr->recs_wide : &pa.ctr->recs_mid, &pa.ctr->recs, sizeof(unsigned long long),
                         cudaMemcpyDeviceToDevice, c->st));
  }
  return BMS_OK;
}

// Clause programs of the queries, then the sliced filter: data graphs of more
// than 64 nodes first (two-word masks), then 33..64 nodes, then the rest (one
// word); the record counter after each launch marks the class boundary.
int run_sliced_filter(bms_ctx* c, const ShellPack& sp, int R, int sem) {
  const uint64_t Qn = c->q.N ? c->q.N : 1;
  const uint64_t per_node = 6 + uint64_t(R) * 16 + 256 + 8;  // clauses, padded to groups of 8
  CK(c->prog_len.ensure(sizeof(uint32_t) * Qn));
  CK(c->prog_off.ensure(sizeof(uint32_t) * (Qn + 1)));
  CK(c->prog.ensure(sizeof(uint16_t) * Qn * per_node));
  CK(c->prog_slow.ensure(Qn));
  CK(c->prog_used.ensure(sizeof(uint32_t) * (kClauseIds / 32 + 1)));
  CK(c->prog_remap.ensure(sizeof(uint16_t) * kClauseIds));
  CK(c->prog_ids.ensure(sizeof(uint16_t) * kClauseIds));
  CK(c->prog_nused.ensure(sizeof(uint32_t)));
  CK(c->tmp.ensure(sizeof(uint32_t) * scan_scratch_words(Qn)));
  CK(launch_query_programs(c->q.dg(), c->q.ds(), sp, c->prog_len.as<uint32_t>(), c->prog_off.as<uint32_t>(),
                           c->tmp.as<uint32_t>(), c->prog_used.as<uint32_t>(), c->prog_remap.as<uint16_t>(),
                           c->prog_ids.as<uint16_t>(), c->prog_nused.as<uint32_t>(), c->prog.as<uint16_t>(),
                           c->prog_slow.as<uint8_t>(), Qn * per_node, nullptr, c->st));
  CK(c->level_desc.ensure(sizeof(uint2) * uint64_t(c->q.G ? c->q.G : 1) * kMaxQueryNodes));
  CK(c->screen.ensure(sizeof(uint4) * (c->q.G ? c->q.G : 1)));
  CK(launch_screen(c->q.dg(), c->q.ds(), c->q.size_order.as<uint32_t>(), c->screen.as<uint4>(), c->st));
  CK(launch_level_desc(c->q.dg(), c->filter_order.as<uint8_t>(), c->filter_dup.as<uint8_t>(),
                       c->prog_off.as<uint32_t>(), c->prog_slow.as<uint8_t>(), c->level_desc.as<uint2>(), c->st));
  SlicedArgs a{};
  a.q = c->q.dg();
  a.d = c->d.dg();
  a.qs = c->q.ds();
  a.ds = c->d.ds();
  a.filter_order = c->filter_order.as<uint8_t>();
  a.dup = c->filter_dup.as<uint8_t>();
  a.qorder = c->q.size_order.as<uint32_t>();
  a.desc = c->level_desc.as<uint2>();
  a.screen = c->screen.as<uint4>();
  a.prog_off = c->prog_off.as<uint32_t>();
  a.prog = c->prog.as<uint16_t>();
  a.slow = c->prog_slow.as<uint8_t>();
  a.used_ids = c->prog_ids.as<uint16_t>();
  a.used_bits = c->prog_used.as<uint32_t>();
  a.remap = c->prog_remap.as<uint16_t>();
  a.n_used = c->prog_nused.as<uint32_t>();
  uint32_t cap = 16 + 16 + 32 + 256 + uint32_t(R) * sp.K * 15;
  a.n_used_cap = (cap < kClauseIds ? cap : kClauseIds) + 1;  // + the all-ones padding mask
  a.sp = sp;
  a.dperm = c->dperm.as<uint32_t>();
  a.valid = c->valid.as<uint32_t>();
  a.QW = c->QW;
  a.vcounts = c->vcounts.as<uint32_t>();
  a.recs = c->recs.as<PairRec>();
  a.rec_cap = c->rec_cap;
  a.arena = c->arena.as<uint64_t>();
  a.row_cap = c->row_cap;
  a.ctr = c->ctr.as<Counters>();
  a.err = c->errflag.as<uint32_t>() + 2;
  a.skip_by_labels = sem == BMS_SEM_EXACT && !c->use_cs;
  // two-word graphs (> 64 nodes)
  a.class_begin = c->class_begin[2];
  a.class_end = c->class_end[2];
  a.class_id = 2;
  size_t smem = sliced_smem_bytes(a, 2);
  if (smem > (220u << 10)) return fail(c, BMS_EUNSUPPORTED, "too many queries for the sliced filter's shared memory");
  CK(launch_sliced_filter(a, 2, smem, c->st));
  CK(cudaMemcpyAsync(&a.ctr->recs_wide, &a.ctr->recs, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, c->st));
  // one-word graphs: 33..64 nodes in 64-bit masks, <= 32 nodes in 32-bit masks
  for (int k = 1; k >= 0; --k) {
    a.class_begin = c->class_begin[k];
    a.class_end = c->class_end[k];
    a.class_id = k;
    CK(launch_sliced_filter(a, k, sliced_smem_bytes(a, k), c->st));
    if (k == 1)
      CK(cudaMemcpyAsync(&a.ctr->recs_mid, &a.ctr->recs, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, c->st));
  }
  return BMS_OK;
}

}  // namespace

extern "C" {

const char* bms_last_error(const void* ctx) {
  if (!ctx) return bms::thread_error();
  return static_cast<const bms_ctx*>(ctx)->err.c_str();
}

int bms_create(int device, bms_ctx** out) {
  if (!out) return fail(nullptr, BMS_EINVAL, "out is null");
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return fail(nullptr, BMS_ENODEV, "no CUDA device");
  }
  if (device < 0 || device >= n) return fail(nullptr, BMS_ENODEV, "device index out of range");
  bms_ctx* c = new (std::nothrow) bms_ctx();
  if (!c) return fail(nullptr, BMS_ENOMEM, "out of host memory");
  c->device = device;
  auto bad = [&](cudaError_t e, const char* w) {
    int r = fail_cuda(c, e, w);
    bms_destroy(c);
    return r;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return bad(e, "cudaSetDevice");
  e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bad(e, "cudaStreamCreate");
  c->st = c->own;
  for (int i = 0; i < EV_COUNT; ++i) {
    e = cudaEventCreate(&c->ev[i]);
    if (e != cudaSuccess) return bad(e, "cudaEventCreate");
  }
  if ((e = c->errflag.ensure(4 * sizeof(uint32_t))) != cudaSuccess) return bad(e, "alloc");
  if ((e = c->ctr.ensure(sizeof(Counters))) != cudaSuccess) return bad(e, "alloc");
  if ((e = cudaMallocHost(&c->h_err, 4 * sizeof(uint32_t))) != cudaSuccess) return bad(e, "cudaMallocHost");
  if ((e = cudaMallocHost(&c->h_ctr, sizeof(Counters))) != cudaSuccess) return bad(e, "cudaMallocHost");
  if ((e = cudaMallocHost(&c->h_T, sizeof(uint32_t))) != cudaSuccess) return bad(e, "cudaMallocHost");
  std::memset(c->h_ctr, 0, sizeof(Counters));
  *c->h_T = 0;
  c->sched = default_schedule();
  *out = c;
  return BMS_OK;
}

void bms_destroy(bms_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  drop_plan(c);
  for (auto& r : c->class_ev)
    for (auto& k : r)
      for (auto& e : k)
        if (e) cudaEventDestroy(e);
  for (int i = 0; i < EV_COUNT; ++i)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  for (cudaStream_t s : c->join_streams.side)
    if (s) cudaStreamDestroy(s);
  if (c->join_streams.fork) cudaEventDestroy(c->join_streams.fork);
  for (cudaEvent_t e : c->join_streams.done)
    if (e) cudaEventDestroy(e);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->h_ctr) cudaFreeHost(c->h_ctr);
  if (c->h_T) cudaFreeHost(c->h_T);
  cudaStream_t own = c->own;
  delete c;  // DevBuf destructors free device memory
  if (own) cudaStreamDestroy(own);
  cudaGetLastError();
}

int bms_set_stream(bms_ctx* c, void* stream) {
  GUARD(c);
  CK(cudaStreamSynchronize(c->st));
  c->st = stream ? static_cast<cudaStream_t>(stream) : c->own;
  return BMS_OK;
}

int bms_set_expansion_budget(bms_ctx* c, uint64_t budget) {
  GUARD(c);
  c->budget = budget;
  return BMS_OK;
}

int bms_set_option(bms_ctx* c, int option, int64_t value) {
  GUARD(c);
  switch (option) {
    case BMS_OPT_FILTER_KERNEL:
      if (value != BMS_FILTER_SLICED && value != BMS_FILTER_BALLOT) return fail(c, BMS_EINVAL, "unknown filter kernel");
      c->filter_kernel = int(value);
      return BMS_OK;
    case BMS_OPT_JOIN_STEPS:
      if (value < 1 || value > 4096) return fail(c, BMS_EINVAL, "join steps must be in [1, 4096]");
      for (int i = 0; i < 3; ++i) c->sched.steps[i] = uint32_t(value);
      return BMS_OK;
    case BMS_OPT_SPLIT_BUDGET:
      if (value < 0 || value > (int64_t(1) << 31)) return fail(c, BMS_EINVAL, "split budget must be in [0, 2^31]");
      for (int i = 0; i < 3; ++i) c->sched.split_budget[i] = uint32_t(value);
      return BMS_OK;
    case BMS_OPT_CUDA_GRAPH:
      c->use_graph = value != 0;
      if (!c->use_graph) drop_plan(c);
      return BMS_OK;
    case BMS_OPT_SUBTREE_CAP:
      if (value < 0 || value > (int64_t(1) << 28)) return fail(c, BMS_EINVAL, "subtree capacity must be in [0, 2^28]");
      c->sub_cap_opt = uint64_t(value);
      return BMS_OK;
    case BMS_OPT_USE_CS:
      if (value != 0 && value != 1) return fail(c, BMS_EINVAL, "clustered join is 0 (off) or 1 (on)");
      c->use_cs = value != 0;
      return BMS_OK;
    case BMS_OPT_RESIDENT_SIGNATURES:
      if (value != 0 && value != 1) return fail(c, BMS_EINVAL, "resident signatures is 0 (off) or 1 (on)");
      c->resident_sigs = value != 0;
      return BMS_OK;
    default:
      return fail(c, BMS_EINVAL, "unknown option");
  }
}

int bms_set_query_order(bms_ctx* c, const uint8_t* order, uint64_t n) {
  GUARD(c);
  if (!c->q.loaded) return fail(c, BMS_ESTATE, "load the query graphs first");
  if (n != c->q.N || (n && !order)) return fail(c, BMS_EINVAL, "the order must hold one entry per query node");
  const uint32_t Q = c->q.G;
  std::vector<uint8_t> perm(uint64_t(Q ? Q : 1) * kMaxQueryNodes, 0);
  for (uint32_t g = 0; g < Q; ++g) {
    const uint32_t qoff = c->q.h_goff[g], m = c->q.h_goff[g + 1] - qoff;
    uint64_t seen = 0;
    for (uint32_t t = 0; t < m; ++t) {
      const uint32_t u = order[qoff + t];
      if (u >= m || ((seen >> u) & 1ull))
        return fail(c, BMS_EINVAL, "query " + std::to_string(g) + ": the order is not a permutation of its vertices");
      seen |= 1ull << u;
      perm[uint64_t(g) * kMaxQueryNodes + t] = uint8_t(u);
    }
  }
  CK(c->given_perm.ensure(perm.size()));
  CK(cudaMemcpyAsync(c->given_perm.p, perm.data(), perm.size(), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->given_set = true;
  ++c->given_gen;
  return BMS_OK;
}

int bms_set_logging(bms_ctx* c, int vertex_expansions) {
  GUARD(c);
  c->log_vertices = vertex_expansions != 0;
  return BMS_OK;
}

int bms_load_graphs(bms_ctx* c, int kind, const bms_graphs* g) {
  GUARD(c);
  if (!g) return fail(c, BMS_EINVAL, "graphs is null");
  bms_graphs_view v;
  bms_graphs_view_of(g, &v);
  if (kind != BMS_QUERY && kind != BMS_DATA) return fail(c, BMS_EINVAL, "invalid kind");
  invalidate_downstream(c);
  Side& s = kind == BMS_QUERY ? c->q : c->d;
  int r = upload(c, s, v, kind == BMS_QUERY ? kMaxQueryNodes : kMaxDataNodes, kind == BMS_QUERY ? "query" : "data");
  if (r) return r;
  if (kind == BMS_DATA) return build_classes(c);
  return BMS_OK;
}

int bms_load_csr(bms_ctx* c, int kind, uint32_t n_graphs, const uint32_t* goff, const uint32_t* rowp,
                 const uint32_t* col, const uint8_t* lab, const uint8_t* elab) {
  GUARD(c);
  if (kind != BMS_QUERY && kind != BMS_DATA) return fail(c, BMS_EINVAL, "invalid kind");
  if (!goff) return fail(c, BMS_EINVAL, "graph_offsets is null");
  bms_graphs_view v{};
  v.n_graphs = n_graphs;
  v.graph_offsets = goff;
  v.row_offsets = rowp;
  v.column_indices = col;
  v.node_labels = lab;
  v.edge_labels = elab;
  invalidate_downstream(c);
  Side& s = kind == BMS_QUERY ? c->q : c->d;
  int r = upload(c, s, v, kind == BMS_QUERY ? kMaxQueryNodes : kMaxDataNodes, kind == BMS_QUERY ? "query" : "data");
  if (r) return r;
  if (kind == BMS_DATA) return build_classes(c);
  return BMS_OK;
}

int bms_signatures(bms_ctx* c, int R) {
  GUARD(c);
  if (!c->q.loaded || !c->d.loaded) return fail(c, BMS_ESTATE, "load query and data graphs first");
  if (R < 0 || R > BMS_MAX_REFINE_STEPS) return fail(c, BMS_EINVAL, "refine_steps must be in [0, 8]");
  // signatures are a pure function of the loaded graphs: steps 1..k do not
  // change when more steps are requested, so an existing candidate matrix
  // stays valid (uploads invalidate it)
  CK(record_event(c, EV_START));
  int r = run_signatures(c, R);
  if (r) return r;
  CK(record_event(c, EV_SIG));
  r = read_side_errors(c);
  if (r) return r;
  c->stats.ms_signatures = elapsed(c, EV_START, EV_SIG);
  c->stats.refine_steps = uint32_t(R);
  return BMS_OK;
}

int bms_filter(bms_ctx* c) {
  GUARD(c);
  if (c->q.sig_steps < 0 || c->d.sig_steps < 0) return fail(c, BMS_ESTATE, "compute signatures first");
  c->W = (c->d.N + 31) / 32;
  const uint64_t words = c->q.N * c->W;
  CK(c->cand.ensure(sizeof(uint32_t) * (words ? words : 1)));
  if (words) CK(cudaMemsetAsync(c->cand.p, 0, sizeof(uint32_t) * words, c->st));
  CK(record_event(c, EV_SIG));
  CK(launch_filter_dense(c->q.dg(), c->q.ds(), c->d.dg(), c->d.ds(), c->cand.as<uint32_t>(), c->W, c->st));
  CK(record_event(c, EV_FILTER));
  CK(cudaStreamSynchronize(c->st));
  c->stats.ms_filter = elapsed(c, EV_SIG, EV_FILTER);
  c->have_cand = true;
  c->mapped = c->have_qidx = c->have_results = false;
  return BMS_OK;
}

int bms_refine(bms_ctx* c, int step) {
  GUARD(c);
  if (!c->have_cand) return fail(c, BMS_ESTATE, "run bms_filter first");
  if (step < 1 || step > c->q.sig_steps || step > c->d.sig_steps)
    return fail(c, BMS_EINVAL, "step must be in [1, refine_steps of bms_signatures]");
  CK(record_event(c, EV_SIG));
  CK(launch_refine_dense(c->q.ds(), c->q.N, c->d.ds(), c->d.N, step, c->cand.as<uint32_t>(), c->W, c->st));
  CK(record_event(c, EV_FILTER));
  CK(cudaStreamSynchronize(c->st));
  c->stats.ms_refine = elapsed(c, EV_SIG, EV_FILTER);
  c->mapped = c->have_qidx = c->have_results = false;
  return BMS_OK;
}

int bms_map(bms_ctx* c, uint64_t* n_pairs) {
  GUARD(c);
  if (!c->have_cand) return fail(c, BMS_ESTATE, "run bms_filter first");
  const uint32_t D = c->d.G;
  c->QW = (c->q.G + 31) / 32;
  CK(c->valid.ensure(sizeof(uint32_t) * (uint64_t(D) * c->QW + 1)));
  CK(c->vcounts.ensure(sizeof(uint32_t) * (D + 1)));
  CK(c->gmcr_off.ensure(sizeof(uint32_t) * (D + 1)));
  CK(c->scan_scratch.ensure(sizeof(uint32_t) * scan_scratch_words(D)));
  CK(record_event(c, EV_FILTER));
  CK(launch_gmcr_dense(c->q.dg(), c->d.dg(), c->cand.as<uint32_t>(), c->W, c->valid.as<uint32_t>(), c->QW,
                       c->vcounts.as<uint32_t>(), c->st));
  CK(launch_scan_u32(c->vcounts.as<uint32_t>(), c->gmcr_off.as<uint32_t>(), D, c->scan_scratch.as<uint32_t>(), c->st));
  CK(cudaMemcpyAsync(c->h_T, c->gmcr_off.as<uint32_t>() + D, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->T = *c->h_T;
  CK(c->qidx.ensure(sizeof(uint32_t) * (c->T ? c->T : 1)));
  CK(launch_gmcr_indices(c->valid.as<uint32_t>(), c->QW, c->q.G, D, c->gmcr_off.as<uint32_t>(), c->qidx.as<uint32_t>(), c->st));
  CK(record_event(c, EV_MAP));
  CK(cudaStreamSynchronize(c->st));
  c->stats.ms_map = elapsed(c, EV_FILTER, EV_MAP);
  c->mapped = true;
  c->have_qidx = true;
  c->have_results = false;
  c->stats.n_valid_pairs = c->T;
  if (n_pairs) *n_pairs = c->T;
  return BMS_OK;
}

int bms_join(bms_ctx* c, int mode, int order, int sem, uint64_t* total) {
  GUARD(c);
  if (!c->mapped) return fail(c, BMS_ESTATE, "run bms_map first");
  int r = validate_modes(c, mode, order, sem);
  if (r) return r;
  const uint64_t T = c->T;
  // one record per GMCR pair, candidate rows gathered from the dense matrix
  CK(c->pair_nodes.ensure(sizeof(uint32_t) * (T + 1)));
  CK(c->row_off.ensure(sizeof(uint32_t) * (T + 1)));
  CK(c->tmp.ensure(sizeof(uint32_t) * scan_scratch_words(T)));
  CK(launch_pair_nodes(c->q.dg(), c->qidx.as<uint32_t>(), T, c->pair_nodes.as<uint32_t>(), c->st));
  CK(launch_scan_u32(c->pair_nodes.as<uint32_t>(), c->row_off.as<uint32_t>(), T, c->tmp.as<uint32_t>(), c->st));
  uint32_t rows = 0;
  CK(cudaMemcpyAsync(c->h_T, c->row_off.as<uint32_t>() + T, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  rows = *c->h_T;
  c->rec_cap = std::max<uint64_t>(T, 1);
  c->row_cap = std::max<uint64_t>(rows, 1);
  c->task_cap = std::max<uint64_t>(uint64_t(rows) * 2, 1024);
  // tasks <= roots <= 128 per record; grown below if the first attempt overflows
  for (int attempt = 0; attempt < 2; ++attempt) {
    r = ensure_join_buffers(c);
    if (r) return r;
    CK(cudaMemsetAsync(c->ctr.p, 0, sizeof(Counters), c->st));
    CK(cudaMemsetAsync(c->errflag.as<uint32_t>() + 2, 0, sizeof(uint32_t), c->st));
    CK(record_event(c, EV_MAP));
    CK(launch_gather_pairs(c->q.dg(), c->d.dg(), c->cand.as<uint32_t>(), c->W, c->gmcr_off.as<uint32_t>(),
                           c->qidx.as<uint32_t>(), c->row_off.as<uint32_t>(), c->recs.as<PairRec>(),
                           c->arena.as<uint64_t>(), c->st));
    CK(launch_set_counter(&c->ctr.as<Counters>()->recs, T, c->st));
    CK(launch_set_counter(&c->ctr.as<Counters>()->recs_wide, T, c->st));  // GMCR order mixes sizes
    CK(launch_set_counter(&c->ctr.as<Counters>()->recs_mid, T, c->st));
    r = join_records(c, mode, order, sem,
                     mode == BMS_COUNT_ALL && order != BMS_ORDER_LEARNED && sem == BMS_SEM_EXACT && !cs_active(c),
                     c->cand.as<uint32_t>());
    if (r) return r;
    CK(cudaMemcpyAsync(c->h_T, c->gmcr_off.as<uint32_t>() + c->d.G, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
    r = finish_run(c, total);
    if (r) return r;
    if (!(c->h_err[2] & kErrOverflow)) break;
    c->task_cap = std::max<uint64_t>(c->h_ctr->tasks + 1, c->task_cap * 2);
    for (unsigned long long n : c->h_ctr->cs_n)
      if (c->cs_cap && n > c->cs_cap) c->cs_cap = std::max<uint64_t>(c->cs_cap, n + n / 8 + 1024);
  }
  if (c->h_err[2] & kErrOverflow) return fail(c, BMS_ENOMEM, "join task buffer overflow");
  c->have_results = true;
  c->have_vexp = mode == BMS_COUNT_ALL && order != BMS_ORDER_LEARNED && sem == BMS_SEM_EXACT && !c->last_cs;
  c->stats.ms_order = elapsed(c, EV_MAP, EV_ORDER);
  c->stats.ms_join = elapsed(c, EV_ORDER, EV_JOIN);
  c->stats.total_matches = c->h_ctr->total;
  c->stats.expansions = c->h_ctr->expansions;
  c->stats.n_incomplete = c->h_ctr->incomplete;
  c->stats.n_partial_matches = c->h_ctr->partials;
  if (total) *total = c->h_ctr->total;
  return c->h_ctr->incomplete ? fail(c, BMS_EINCOMPLETE, "some pairs hit the expansion budget") : BMS_OK;
}

int bms_run(bms_ctx* c, int R, int mode, int order, int sem, uint64_t* total) {
  GUARD(c);
  try {
    const bool log = c->log_vertices && mode == BMS_COUNT_ALL && order != BMS_ORDER_LEARNED && sem == BMS_SEM_EXACT;
    return run_fused(c, R, mode, order, sem, total, log, 0);
  } catch (...) {
    return fail(c, BMS_ENOMEM, "host exception in bms_run");
  }
}

int bms_get_embeddings(bms_ctx* c, uint64_t pair, uint8_t* out, uint64_t max_embeddings, uint64_t* n_embeddings) {
  GUARD(c);
  if (!n_embeddings || (max_embeddings && !out)) return fail(c, BMS_EINVAL, "out or n_embeddings is null");
  if (!c->have_results) return fail(c, BMS_ESTATE, "run the pipeline first");
  if (c->last_sem != BMS_SEM_EXACT || c->last_mode != BMS_COUNT_ALL)
    return fail(c, BMS_ESTATE, "embeddings are defined for count-all runs with EXACT semantics");
  if (c->last_cs) return fail(c, BMS_ESTATE, "embeddings follow the plain join; switch the clustered join off");
  if (pair >= c->T) return fail(c, BMS_EINVAL, "pair index beyond the GMCR");
  // the pair's record (pairs the join skips have none and no embedding)
  CK(c->embed_tmp.ensure(2 * sizeof(unsigned long long)));
  unsigned long long* dev = c->embed_tmp.as<unsigned long long>();
  CK(cudaMemsetAsync(dev, 0xFF, sizeof(unsigned long long), c->st));
  CK(cudaMemsetAsync(dev + 1, 0, sizeof(unsigned long long), c->st));
  CK(launch_find_record(c->recs.as<PairRec>(), c->ctr.as<Counters>(), c->rec_cap, uint32_t(pair), dev, c->st));
  unsigned long long h[2] = {0, 0};
  CK(cudaMemcpyAsync(h, dev, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  *n_embeddings = 0;
  if (h[0] == ~0ull) return BMS_OK;
  const uint64_t rec = h[0];
  CK(cudaMemcpy(&h[1], c->pair_count.as<unsigned long long>() + rec, sizeof(unsigned long long),
                cudaMemcpyDeviceToHost));
  const uint64_t total = h[1];
  PairRec pr;
  CK(cudaMemcpy(&pr, c->recs.as<PairRec>() + rec, sizeof(PairRec), cudaMemcpyDeviceToHost));
  const uint32_t n = c->q.h_goff[pr.q + 1] - c->q.h_goff[pr.q];
  if (total * n > (uint64_t(1) << 32)) return fail(c, BMS_EUNSUPPORTED, "more than 4 GiB of embeddings for one pair");
  if (total) {
    CK(c->embed_out.ensure(total * n));
    EmbedArgs a{};
    a.q = c->q.dg();
    a.d = c->d.dg();
    a.ds = c->d.ds();
    a.o = order_of(c);
    a.recs = c->recs.as<PairRec>();
    a.rec = rec;
    a.arena = c->arena.as<uint64_t>();
    a.out = c->embed_out.as<uint8_t>();
    a.cap = total;
    a.count = dev + 1;
    CK(launch_embed(a, c->st));
    CK(cudaMemcpyAsync(&h[1], dev + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
    std::vector<uint8_t> all(total * n);
    CK(cudaMemcpyAsync(all.data(), c->embed_out.p, total * n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (h[1] != total) return fail(c, BMS_ECUDA, "embedding enumeration disagrees with the pair count");
    std::vector<uint64_t> idx(total);
    for (uint64_t k = 0; k < total; ++k) idx[k] = k;
    std::sort(idx.begin(), idx.end(), [&](uint64_t x, uint64_t y) {
      return std::memcmp(&all[x * n], &all[y * n], n) < 0;
    });
    for (uint64_t k = 0; k < std::min<uint64_t>(total, max_embeddings); ++k)
      std::memcpy(out + k * n, &all[idx[k] * n], n);
  }
  *n_embeddings = total;
  return BMS_OK;
}

int bms_load_resident(bms_ctx* c, const bms_graphs* data) {
  GUARD(c);
  if (!data) return fail(c, BMS_EINVAL, "data is null");
  invalidate_downstream(c);
  release_views(c->d);  // views of the previous resident batch
  c->d.loaded = false;
  c->d_sig_cached = false;
  c->dres_sig_R = -1;
  bms_graphs_view v;
  bms_graphs_view_of(data, &v);
  return upload(c, c->dres, v, kMaxDataNodes, "data");
}

namespace {
// The data side becomes a view of resident graphs [g0, g1): graph offsets from
// g0 on (global node ids), every node- and entry-indexed buffer shared, the
// per-graph arrays from g0 on.  Nothing is copied.
void view_window(bms_ctx* c, uint32_t g0, uint32_t g1) {
  Side& r = c->dres;
  Side& d = c->d;
  d.G = g1 - g0;
  d.N = r.N;
  d.E = r.E;
  d.max_nodes = r.max_nodes;
  d.h_goff.assign(r.h_goff.begin() + g0, r.h_goff.begin() + g1 + 1);
  d.goff.alias(r.goff.as<uint32_t>() + g0, sizeof(uint32_t) * (d.G + 1));
  d.rowp.alias(r.rowp.p, r.rowp.bytes);
  d.col.alias(r.col.p, r.col.bytes);
  d.lab.alias(r.lab.p, r.lab.bytes);
  d.frec.alias(r.frec.p, r.frec.bytes);
  d.adj.alias(r.adj.p, r.adj.bytes);
  d.adjin.alias(r.adjin.p, r.adjin.bytes);
  d.ghist.alias(r.ghist.as<uint64_t>() + g0, sizeof(uint64_t) * (d.G ? d.G : 1));
  d.glabset.alias(r.glabset.as<uint32_t>() + g0, sizeof(uint32_t) * (d.G ? d.G : 1));
  d.maxin.alias(r.maxin.p, r.maxin.bytes);
  d.sig_steps = -1;
  d.asymmetric = false;
  d.labels_lt16 = 0;
  d.loaded = true;
  ++c->load_gen;
}
}  // namespace

int bms_run_resident(bms_ctx* c, uint32_t window_graphs, int R, int mode, int order, int sem, uint64_t* total,
                     uint64_t* per_query) {
  GUARD(c);
  if (!c->dres.loaded) return fail(c, BMS_ESTATE, "load a resident data batch first");
  if (!c->q.loaded) return fail(c, BMS_ESTATE, "load the query graphs first");
  if (window_graphs == 0) window_graphs = 100000;
  try {
    const uint32_t G = c->dres.G, Q = c->q.G;
    if (per_query) {
      CK(c->per_query.ensure(sizeof(unsigned long long) * (Q ? Q : 1)));
      CK(cudaMemsetAsync(c->per_query.p, 0, sizeof(unsigned long long) * (Q ? Q : 1), c->st));
    }
    if (R < 0 || R > BMS_MAX_REFINE_STEPS) return fail(c, BMS_EINVAL, "refine_steps must be in [0, 8]");
    float ms_resident_sigs = 0.f;
    if (!c->resident_sigs) {
      c->dres_sig_R = -1;  // windows write the shared arrays and their own in-degree bound
    } else if (c->dres_sig_R != R) {
      // every node of the resident batch once, with the batch's in-degree bound and error bits
      Side& r = c->dres;
      CK(c->dres_err.ensure(sizeof(uint32_t)));
      CK(cudaMemsetAsync(c->errflag.p, 0, 4 * sizeof(uint32_t), c->st));
      CK(cudaMemsetAsync(r.maxin.p, 0, 2 * sizeof(uint32_t), c->st));
      r.sig_steps = R;
      CK(record_event(c, EV_START));
      CK(launch_signatures(r.dg(), r.ds(), kMaxDataNodes, c->errflag.as<uint32_t>(), c->st));
      CK(record_event(c, EV_SIG));
      CK(cudaMemcpyAsync(c->dres_err.p, c->errflag.p, sizeof(uint32_t), cudaMemcpyDeviceToDevice, c->st));
      CK(cudaMemcpyAsync(c->h_err, c->errflag.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      ms_resident_sigs = elapsed(c, EV_START, EV_SIG);
      int r2 = check_side_errors(c, "data", c->h_err[0]);
      if (r2) return r2;
      c->dres_sig_R = R;
    }
    uint64_t sum = 0;
    int incomplete = 0;
    bms_stats acc{};
    acc.ms_signatures = ms_resident_sigs;
    uint32_t g0 = 0;
    do {
      const uint32_t g1 = std::min<uint64_t>(G, uint64_t(g0) + window_graphs);
      invalidate_downstream(c);
      view_window(c, g0, g1);
      c->d_sig_cached = c->resident_sigs && c->dres_sig_R == R;
      int r = build_classes(c);
      if (r) return r;
      uint64_t t = 0;
      r = run_fused(c, R, mode, order, sem, &t, false, 0);
      if (r == BMS_EINCOMPLETE) incomplete = 1;
      else if (r) return r;
      sum += t;
      acc.total_matches += c->stats.total_matches;
      acc.expansions += c->stats.expansions;
      acc.n_incomplete += c->stats.n_incomplete;
      acc.kernel_launches += c->stats.kernel_launches;
      acc.ms_signatures += c->stats.ms_signatures;
      acc.ms_filter += c->stats.ms_filter;
      acc.ms_map += c->stats.ms_map;
      acc.ms_order += c->stats.ms_order;
      acc.ms_join += c->stats.ms_join;
      acc.ms_total += c->stats.ms_total;
      if (per_query)
        CK(launch_query_totals(c->recs.as<PairRec>(), c->ctr.as<Counters>(), c->rec_cap,
                               c->pair_count.as<unsigned long long>(), mode == BMS_FIND_FIRST, Q,
                               c->per_query.as<unsigned long long>(), c->st));
      g0 = g1;
    } while (g0 < G);
    if (per_query && Q) {
      CK(cudaMemcpyAsync(per_query, c->per_query.p, sizeof(uint64_t) * Q, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
    }
    c->stats.total_matches = acc.total_matches;
    c->stats.expansions = acc.expansions;
    c->stats.n_incomplete = acc.n_incomplete;
    c->stats.kernel_launches = acc.kernel_launches;
    c->stats.ms_signatures = acc.ms_signatures;
    c->stats.ms_filter = acc.ms_filter;
    c->stats.ms_map = acc.ms_map;
    c->stats.ms_order = acc.ms_order;
    c->stats.ms_join = acc.ms_join;
    c->stats.ms_total = acc.ms_total;
    if (total) *total = sum;
    return incomplete ? fail(c, BMS_EINCOMPLETE, "some pairs hit the expansion budget") : BMS_OK;
  } catch (...) {
    return fail(c, BMS_ENOMEM, "host exception in bms_run_resident");
  }
}

static void release_graph_pins(bms_graphs* g) {
  for (void* p : g->pinned) cudaHostUnregister(p);
  g->pinned.clear();
  g->release_pins = nullptr;
}

int bms_graphs_pin(bms_graphs* g) {
  if (!g) {
    set_thread_error("graphs is null");
    return BMS_EINVAL;
  }
  if (!g->pinned.empty()) return BMS_OK;
  g->release_pins = release_graph_pins;
  auto reg = [&](void* p, size_t bytes) -> cudaError_t {
    if (!bytes) return cudaSuccess;
    const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
    if (e == cudaSuccess) g->pinned.push_back(p);
    return e;
  };
  cudaError_t e = reg(g->goff.data(), g->goff.size() * sizeof(uint32_t));
  if (e == cudaSuccess) e = reg(g->rowp.data(), g->rowp.size() * sizeof(uint32_t));
  if (e == cudaSuccess) e = reg(g->col.data(), g->col.size() * sizeof(uint32_t));
  if (e == cudaSuccess) e = reg(g->lab.data(), g->lab.size());  // edge labels are never copied
  if (e != cudaSuccess) {
    cudaGetLastError();
    release_graph_pins(g);
    set_thread_error(std::string("cudaHostRegister: ") + cudaGetErrorString(e));
    return BMS_ECUDA;
  }
  return BMS_OK;
}

int bms_graphs_unpin(bms_graphs* g) {
  if (!g) {
    set_thread_error("graphs is null");
    return BMS_EINVAL;
  }
  release_graph_pins(g);
  return BMS_OK;
}

int bms_run_batches(bms_ctx* c, const bms_graphs* data, uint32_t batch_graphs, int R, int mode, int order, int sem,
                    uint64_t* total, uint64_t* per_query) {
  GUARD(c);
  if (!data) return fail(c, BMS_EINVAL, "data is null");
  if (!c->q.loaded) return fail(c, BMS_ESTATE, "load the query graphs first");
  if (batch_graphs == 0) batch_graphs = 100000;  // BMS2_batch.cpp:12
  try {
    const uint32_t G = data->n_graphs(), Q = c->q.G;
    if (per_query) {
      CK(c->per_query.ensure(sizeof(unsigned long long) * (Q ? Q : 1)));
      CK(cudaMemsetAsync(c->per_query.p, 0, sizeof(unsigned long long) * (Q ? Q : 1), c->st));
    }
    uint64_t sum = 0;
    int incomplete = 0;
    bms_stats acc{};
    uint32_t g0 = 0;
    do {
      const uint32_t g1 = std::min<uint64_t>(G, uint64_t(g0) + batch_graphs);
      const uint32_t n0 = data->goff[g0];
      bms_graphs_view v{};
      v.n_graphs = g1 - g0;
      v.graph_offsets = data->goff.data() + g0;
      v.row_offsets = data->rowp.data() + n0;
      v.column_indices = data->col.data() + (data->col.empty() ? 0 : data->rowp[n0]);
      v.node_labels = data->lab.data() + n0;
      v.edge_labels = data->elab.data() + (data->elab.empty() ? 0 : data->rowp[n0]);
      invalidate_downstream(c);
      int r = upload(c, c->d, v, kMaxDataNodes, "data", true);
      if (r) return r;
      r = build_classes(c);
      if (r) return r;
      uint64_t t = 0;
      r = run_fused(c, R, mode, order, sem, &t, false, 0);
      if (r == BMS_EINCOMPLETE) incomplete = 1;
      else if (r) return r;
      sum += t;
      acc.total_matches += c->stats.total_matches;
      acc.expansions += c->stats.expansions;
      acc.n_incomplete += c->stats.n_incomplete;
      acc.kernel_launches += c->stats.kernel_launches;
      acc.ms_signatures += c->stats.ms_signatures;
      acc.ms_filter += c->stats.ms_filter;
      acc.ms_map += c->stats.ms_map;
      acc.ms_order += c->stats.ms_order;
      acc.ms_join += c->stats.ms_join;
      acc.ms_total += c->stats.ms_total;
      if (per_query)
        CK(launch_query_totals(c->recs.as<PairRec>(), c->ctr.as<Counters>(), c->rec_cap,
                               c->pair_count.as<unsigned long long>(), mode == BMS_FIND_FIRST, Q,
                               c->per_query.as<unsigned long long>(), c->st));
      g0 = g1;
    } while (g0 < G);
    if (per_query && Q) {
      CK(cudaMemcpyAsync(per_query, c->per_query.p, sizeof(uint64_t) * Q, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
    }
    // stage times and counters over all slices (graph, node and valid-pair
    // counts stay the last slice's: they size its per-pair results)
    c->stats.total_matches = acc.total_matches;
    c->stats.expansions = acc.expansions;
    c->stats.n_incomplete = acc.n_incomplete;
    c->stats.kernel_launches = acc.kernel_launches;
    c->stats.ms_signatures = acc.ms_signatures;
    c->stats.ms_filter = acc.ms_filter;
    c->stats.ms_map = acc.ms_map;
    c->stats.ms_order = acc.ms_order;
    c->stats.ms_join = acc.ms_join;
    c->stats.ms_total = acc.ms_total;
    if (total) *total = sum;
    return incomplete ? fail(c, BMS_EINCOMPLETE, "some pairs hit the expansion budget") : BMS_OK;
  } catch (...) {
    return fail(c, BMS_ENOMEM, "host exception in bms_run_batches");
  }
}

}  // extern "C"

namespace {

// Device work of one fused run: signatures -> filter -> GMCR -> order -> join
// -> totals.  No host synchronisation, so it can be captured as a CUDA graph.
int enqueue_fused(bms_ctx* c, int R, int mode, int order, int sem, bool log_vertices) {
  const uint32_t D = c->d.G;
  if (order == BMS_ORDER_LEARNED)
    CK(cudaMemsetAsync(c->cand_sum.p, 0, sizeof(unsigned int) * (c->q.N ? c->q.N : 1), c->st));
  CK(cudaMemsetAsync(c->ctr.p, 0, sizeof(Counters), c->st));
  CK(record_event(c, EV_START));
  int r = run_signatures(c, R);
  if (r) return r;
  CK(launch_label_count(c->d.dg(), c->label_count.as<unsigned long long>(), c->st));
  CK(launch_query_prep(c->q.dg(), c->q.ds(), c->label_count.as<unsigned long long>(), c->filter_order.as<uint8_t>(),
                       c->filter_dup.as<uint8_t>(), c->st));
  ShellPack sp{};
  for (uint32_t l = 0; l < 16; ++l)
    if ((c->q.labels_lt16 >> l) & 1u) sp.pos[sp.K++] = uint8_t(l);
  sp.PW = sp.K == 0 ? 0u : (sp.K <= 8 ? uint32_t(R + 1) / 2 : uint32_t(R));
  CK(c->qpack.ensure(sizeof(uint64_t) * 8 * (c->q.N ? c->q.N : 1)));
  CK(launch_pack_query_shells(c->q.dg(), c->q.ds(), sp, c->qpack.as<uint64_t>(), c->st));
  CK(record_event(c, EV_SIG));
  r = c->filter_kernel == BMS_FILTER_BALLOT ? run_ballot_filter(c, sp, sem) : run_sliced_filter(c, sp, R, sem);
  if (r) return r;
  CK(record_event(c, EV_FILTER));
  CK(launch_scan_u32(c->vcounts.as<uint32_t>(), c->gmcr_off.as<uint32_t>(), D, c->scan_scratch.as<uint32_t>(), c->st));
  CK(launch_pair_positions(c->recs.as<PairRec>(), c->ctr.as<Counters>(), c->rec_cap, c->valid.as<uint32_t>(), c->QW,
                           c->gmcr_off.as<uint32_t>(), c->st));
  CK(record_event(c, EV_MAP));
  return join_records(c, mode, order, sem, log_vertices && !cs_active(c), nullptr);
}

PlanKey plan_key(const bms_ctx* c, int R, int mode, int order, int sem) {
  PlanKey k;
  std::memset(&k, 0, sizeof k);
  k.load_gen = c->load_gen;
  k.epoch = g_alloc_epoch.load();
  k.R = R;
  k.mode = mode;
  k.order = order;
  k.sem = sem;
  k.filter_kernel = c->filter_kernel;
  k.model_set = c->model_set ? 1 : 0;
  k.use_cs = c->use_cs ? 1 : 0;
  k.given_gen = order == BMS_ORDER_GIVEN ? c->given_gen : 0;
  k.sub_cap_opt = c->sub_cap_opt;
  k.budget = c->budget;
  k.rec_cap = c->rec_cap;
  k.row_cap = c->row_cap;
  k.task_cap = c->task_cap;
  k.cs_cap = c->cs_cap;
  k.sub_cap = c->sub_cap;
  k.sched = c->sched;
  return k;
}

bool same_key(const PlanKey& a, const PlanKey& b) { return std::memcmp(&a, &b, sizeof(PlanKey)) == 0; }

void drop_plan(bms_ctx* c) {
  if (c->plan_exec) cudaGraphExecDestroy(c->plan_exec);
  if (c->plan_graph) cudaGraphDestroy(c->plan_graph);
  c->plan_exec = nullptr;
  c->plan_graph = nullptr;
  c->plan_warm = false;
}

// Capture enqueue_fused into a graph and instantiate it; false (and no plan)
// if anything in the capture failed.
bool capture_plan(bms_ctx* c, int R, int mode, int order, int sem, const PlanKey& key) {
  drop_plan(c);
  if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const unsigned long long l0 = g_launches;
  const int r = enqueue_fused(c, R, mode, order, sem, false);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(c->st, &g);
  const unsigned long long launches = g_launches - l0;
  if (r != BMS_OK || e != cudaSuccess || !g || !same_key(key, plan_key(c, R, mode, order, sem))) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    c->plan_key = key;
    c->capture_failed = true;  // run eagerly until the key changes
    return false;
  }
  cudaGraphExec_t x = nullptr;
  if (cudaGraphInstantiate(&x, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    c->plan_key = key;
    c->capture_failed = true;
    return false;
  }
  c->plan_graph = g;
  c->plan_exec = x;
  c->plan_launches = launches;
  c->plan_key = key;
  c->plan_warm = true;
  return true;
}

int complete_fused(bms_ctx* c, int R, int mode, int order, int sem, uint64_t* total, bool log_vertices, int attempt,
                   unsigned long long launches);

int run_fused(bms_ctx* c, int R, int mode, int order, int sem, uint64_t* total, bool log_vertices, int attempt) {
  if (!c->q.loaded || !c->d.loaded) return fail(c, BMS_ESTATE, "load query and data graphs first");
  const unsigned long long launches0 = g_launches;
  if (R < 0 || R > BMS_MAX_REFINE_STEPS) return fail(c, BMS_EINVAL, "refine_steps must be in [0, 8]");
  int r = validate_modes(c, mode, order, sem);
  if (r) return r;
  invalidate_downstream(c);
  const uint32_t D = c->d.G, Q = c->q.G;
  c->QW = (Q + 31) / 32;
  CK(c->valid.ensure(sizeof(uint32_t) * (uint64_t(D) * c->QW + 1)));
  CK(c->vcounts.ensure(sizeof(uint32_t) * (D + 1)));
  CK(c->gmcr_off.ensure(sizeof(uint32_t) * (D + 1)));
  CK(c->scan_scratch.ensure(sizeof(uint32_t) * scan_scratch_words(D)));
  CK(c->filter_order.ensure(uint64_t(Q ? Q : 1) * kMaxQueryNodes));
  CK(c->filter_dup.ensure(uint64_t(Q ? Q : 1) * kMaxQueryNodes));
  CK(c->label_count.ensure(256 * sizeof(unsigned long long)));
  if (c->rec_cap == 0) {
    c->rec_cap = std::max<uint64_t>(1 << 16, std::min<uint64_t>(uint64_t(Q) * D, uint64_t(1) << 22));
    c->row_cap = c->rec_cap * 24;
    c->task_cap = c->rec_cap * 8;
  }
  r = ensure_join_buffers(c);
  if (r) return r;
  if (order == BMS_ORDER_LEARNED) CK(c->cand_sum.ensure(sizeof(unsigned int) * (c->q.N ? c->q.N : 1)));
  // CUDA graph: the first run with a given key runs eagerly (and settles every
  // allocation), the second captures the pipeline, later ones replay it.
  bool graphable = c->use_graph && attempt == 0 && !log_vertices;
  if (graphable) {
    const PlanKey key = plan_key(c, R, mode, order, sem);
    if (c->capture_failed) {
      if (same_key(key, c->plan_key)) graphable = false;
      else c->capture_failed = false;
    }
  }
  if (graphable) {
    const PlanKey key = plan_key(c, R, mode, order, sem);
    if (c->plan_warm && same_key(key, c->plan_key) && (c->plan_exec || capture_plan(c, R, mode, order, sem, key))) {
      CK(cudaGraphLaunch(c->plan_exec, c->st));
      return complete_fused(c, R, mode, order, sem, total, false, attempt, c->plan_launches);
    }
    drop_plan(c);
  }
  r = enqueue_fused(c, R, mode, order, sem, log_vertices);
  if (r) return r;
  r = complete_fused(c, R, mode, order, sem, total, log_vertices, attempt, g_launches - launches0);
  if (graphable && (r == BMS_OK || r == BMS_EINCOMPLETE) && !c->plan_exec && !c->capture_failed) {
    c->plan_key = plan_key(c, R, mode, order, sem);
    c->plan_warm = true;
  }
  return r;
}

// Read the run's counters back (the one host synchronisation), check errors,
// grow the buffers and rerun on overflow, fill the stats.
int complete_fused(bms_ctx* c, int R, int mode, int order, int sem, uint64_t* total, bool log_vertices, int attempt,
                   unsigned long long launches) {
  int r = finish_run(c, total);
  if (r) return r;
  r = check_side_errors(c, "data", c->h_err[0]);
  if (r) {
    c->d.sig_steps = -1;
    return r;
  }
  r = check_side_errors(c, "query", c->h_err[1]);
  if (r) {
    c->q.sig_steps = -1;
    return r;
  }
  c->d.asymmetric = (c->h_err[0] & kErrAsym) != 0;
  c->q.asymmetric = (c->h_err[1] & kErrAsym) != 0;
  if (order != BMS_ORDER_GMCR && (c->d.asymmetric || c->q.asymmetric))
    return fail(c, BMS_EINVAL, "a search order other than the GMCR order requires symmetric adjacency");
  if (c->h_err[2] & kErrOverflow) {
    drop_plan(c);
    if (attempt >= 2) return fail(c, BMS_ENOMEM, "result buffers overflow");
    const Counters& h = *c->h_ctr;
    c->rec_cap = std::max<uint64_t>(c->rec_cap, h.recs + h.recs / 8 + 1024);
    c->row_cap = std::max<uint64_t>(c->row_cap, h.rows + h.rows / 8 + 16384);
    c->task_cap = std::max<uint64_t>(c->task_cap, h.tasks + h.tasks / 8 + 16384);
    bool cs_over = false;  // the clustered entries explain the overflow
    for (unsigned long long n : h.cs_n)
      if (c->cs_cap && n > c->cs_cap) {
        cs_over = true;
        c->cs_cap = std::max<uint64_t>(c->cs_cap, n + n / 8 + 1024);
      }
    if (!cs_over && h.recs <= c->rec_cap && h.rows <= c->row_cap && h.tasks < c->task_cap / 2) c->task_cap *= 2;
    return run_fused(c, R, mode, order, sem, total, log_vertices, attempt + 1);
  }
  c->T = *c->h_T;
  c->mapped = true;
  c->have_qidx = false;
  c->have_results = true;
  c->have_vexp = log_vertices && !c->last_cs;
  c->stats.refine_steps = uint32_t(R);
  c->stats.ms_signatures = elapsed(c, EV_START, EV_SIG);
  c->stats.ms_filter = elapsed(c, EV_SIG, EV_FILTER);
  c->stats.ms_refine = 0.f;
  c->stats.ms_map = elapsed(c, EV_FILTER, EV_MAP);
  c->stats.kernel_launches = launches;
  c->stats.ms_order = elapsed(c, EV_MAP, EV_ORDER);
  c->stats.ms_join = elapsed(c, EV_ORDER, EV_JOIN);
  c->stats.ms_total = elapsed(c, EV_START, EV_END);
  c->stats.n_valid_pairs = c->T;
  c->stats.total_matches = c->h_ctr->total;
  c->stats.expansions = c->h_ctr->expansions;
  c->stats.n_incomplete = c->h_ctr->incomplete;
  c->stats.n_partial_matches = c->h_ctr->partials;
  if (total) *total = c->h_ctr->total;
  return c->h_ctr->incomplete ? fail(c, BMS_EINCOMPLETE, "some pairs hit the expansion budget") : BMS_OK;
}

}  // namespace

int bms::rejoin_timed(bms_ctx* c, const bms_schedule& sched, float* ms, float class_ms[3]) {
  if (!c->have_results) return fail(c, BMS_ESTATE, "run the pipeline first");
  if (c->last_sem == BMS_SEM_REFERENCE_DFS) return fail(c, BMS_ESTATE, "timing runs use EXACT semantics");
  if (c->last_cs) return fail(c, BMS_ESTATE, "timing runs time the plain join; switch the clustered join off");
  Counters* ctr = c->ctr.as<Counters>();
  static_assert(offsetof(Counters, sub_n) == offsetof(Counters, join_head) + sizeof(Counters::join_head),
                "join heads and subtree counts are cleared together");
  if (!c->class_ev[0][0][0])
    for (auto& r : c->class_ev)
      for (auto& k : r)
        for (auto& e : k) CK(cudaEventCreate(&e));
  ClassLaunch cl[3];
  class_launches(sched, c->last_sem, cl);
  const bool tasks = needs_tasks(sched, c->last_sem);
  // a (pair, root) schedule may need a larger task buffer than the last run
  // had: grow it and time again, as a pipeline run would
  for (int attempt = 0; attempt < 2; ++attempt) {
    CK(cudaMemsetAsync(&ctr->join_head, 0, sizeof(ctr->join_head) + sizeof(ctr->sub_n), c->st));
    CK(cudaMemsetAsync(c->errflag.as<uint32_t>() + 2, 0, sizeof(uint32_t), c->st));
    CK(cudaMemsetAsync(c->pair_count.p, 0, sizeof(unsigned long long) * c->rec_cap, c->st));
    CK(cudaMemsetAsync(c->pair_exp.p, 0, sizeof(unsigned long long) * c->rec_cap, c->st));
    CK(cudaMemsetAsync(c->pair_flag.p, 0, sizeof(uint32_t) * c->rec_cap, c->st));
    CK(record_event(c, EV_ORDER));
    if (tasks) {
      CK(cudaMemsetAsync(&ctr->tasks, 0, sizeof(ctr->tasks), c->st));
      CK(launch_task_emit(c->recs.as<PairRec>(), c->rec_cap, c->q.dg(), order_of(c), c->arena.as<uint64_t>(),
                          c->tasks.as<Task>(), c->task_cap, ctr, c->errflag.as<uint32_t>() + 2, c->st));
    }
    const JoinArgs ja = join_args(c, c->last_mode, c->last_sem, false);
    CK(launch_join(ja, cl, c->st, c->class_ev));
    CK(record_event(c, EV_JOIN));
    CK(cudaMemcpyAsync(c->h_err + 2, c->errflag.as<uint32_t>() + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(&c->h_ctr->tasks, &ctr->tasks, sizeof(ctr->tasks), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (!(c->h_err[2] & kErrOverflow)) break;
    if (attempt == 1) return fail(c, BMS_ENOMEM, "join task buffer overflow while timing");
    c->task_cap = std::max<uint64_t>(c->task_cap, c->h_ctr->tasks + c->h_ctr->tasks / 8 + 16384);
    CK(c->tasks.ensure(sizeof(Task) * c->task_cap));
  }
  *ms = elapsed(c, EV_ORDER, EV_JOIN);
  bool splits = false;
  for (int k = 0; k < 3; ++k) splits = splits || cl[k].split_budget != 0;
  for (int k = 0; k < 3; ++k) {
    class_ms[k] = 0.f;
    for (int r = 0; r < (splits ? kJoinRounds : 1); ++r) {
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, c->class_ev[r][k][0], c->class_ev[r][k][1]));
      class_ms[k] += t;
    }
  }
  return BMS_OK;  // the timed join recomputed the same per-record counts
}

namespace {

int scatter_results(bms_ctx* c, uint64_t* counts, uint64_t* exps, uint8_t* status) {
  CK(launch_scatter(c->recs.as<PairRec>(), c->ctr.as<Counters>(), c->rec_cap, c->pair_count.as<unsigned long long>(),
                    c->pair_exp.as<unsigned long long>(), c->pair_flag.as<uint32_t>(), c->last_mode == BMS_FIND_FIRST,
                    counts, exps, status, c->st));
  return BMS_OK;
}

int ensure_qidx(bms_ctx* c) {
  if (c->have_qidx) return BMS_OK;
  CK(c->qidx.ensure(sizeof(uint32_t) * (c->T ? c->T : 1)));
  CK(launch_gmcr_indices(c->valid.as<uint32_t>(), c->QW, c->q.G, c->d.G, c->gmcr_off.as<uint32_t>(),
                         c->qidx.as<uint32_t>(), c->st));
  c->have_qidx = true;
  return BMS_OK;
}

}  // namespace

extern "C" {

int bms_get_stats(bms_ctx* c, bms_stats* out) {
  GUARD(c);
  if (!out) return fail(c, BMS_EINVAL, "out is null");
  c->stats.n_query_graphs = c->q.G;
  c->stats.n_data_graphs = c->d.G;
  c->stats.n_query_nodes = c->q.N;
  c->stats.n_data_nodes = c->d.N;
  c->stats.n_pairs = uint64_t(c->q.G) * c->d.G;
  c->stats.last_mode = uint32_t(c->last_mode);
  c->stats.last_order = uint32_t(c->last_order);
  c->stats.last_semantics = uint32_t(c->last_sem);
  *out = c->stats;
  return BMS_OK;
}

int bms_get_gmcr(bms_ctx* c, uint32_t* offsets, uint32_t* qidx, uint64_t cap) {
  GUARD(c);
  if (!c->mapped) return fail(c, BMS_ESTATE, "no mapping: run bms_map or bms_run");
  if (offsets)
    CK(cudaMemcpyAsync(offsets, c->gmcr_off.p, sizeof(uint32_t) * (c->d.G + 1), cudaMemcpyDeviceToHost, c->st));
  if (qidx) {
    if (cap < c->T) return fail(c, BMS_EINVAL, "capacity below the number of mapped pairs");
    int r = ensure_qidx(c);
    if (r) return r;
    if (c->T) CK(cudaMemcpyAsync(qidx, c->qidx.p, sizeof(uint32_t) * c->T, cudaMemcpyDeviceToHost, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  return BMS_OK;
}

static int get_pair_array(bms_ctx* c, int which, void* out, uint64_t cap) {
  if (!c->have_results) return fail(c, BMS_ESTATE, "no join results");
  if (!out) return fail(c, BMS_EINVAL, "out is null");
  if (cap < c->T) return fail(c, BMS_EINVAL, "capacity below the number of mapped pairs");
  const size_t elem = which == 2 ? 1 : 8;
  CK(c->tmp.ensure(elem * (c->T ? c->T : 1)));
  if (c->T) CK(cudaMemsetAsync(c->tmp.p, 0, elem * c->T, c->st));
  int r = scatter_results(c, which == 0 ? c->tmp.as<uint64_t>() : nullptr, which == 1 ? c->tmp.as<uint64_t>() : nullptr,
                          which == 2 ? c->tmp.as<uint8_t>() : nullptr);
  if (r) return r;
  if (c->T) CK(cudaMemcpyAsync(out, c->tmp.p, elem * c->T, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return BMS_OK;
}

int bms_get_pair_counts(bms_ctx* c, uint64_t* counts, uint64_t cap) {
  GUARD(c);
  return get_pair_array(c, 0, counts, cap);
}
int bms_get_pair_expansions(bms_ctx* c, uint64_t* e, uint64_t cap) {
  GUARD(c);
  return get_pair_array(c, 1, e, cap);
}
int bms_get_pair_status(bms_ctx* c, uint8_t* s, uint64_t cap) {
  GUARD(c);
  return get_pair_array(c, 2, s, cap);
}

int bms_get_candidates(bms_ctx* c, uint32_t* words, uint64_t cap) {
  GUARD(c);
  if (!c->have_cand) return fail(c, BMS_ESTATE, "no dense candidate matrix: run bms_filter");
  const uint64_t n = c->q.N * c->W;
  if (!words || cap < n) return fail(c, BMS_EINVAL, "capacity below n_query_nodes * ceil(n_data_nodes/32)");
  if (n) CK(cudaMemcpyAsync(words, c->cand.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return BMS_OK;
}

int bms_get_signatures(bms_ctx* c, int kind, uint64_t* label_gen, uint64_t* path, uint16_t* cycle, uint64_t* shells) {
  GUARD(c);
  if (kind != BMS_QUERY && kind != BMS_DATA) return fail(c, BMS_EINVAL, "invalid kind");
  Side& s = kind == BMS_QUERY ? c->q : c->d;
  if (s.sig_steps < 0) return fail(c, BMS_ESTATE, "no signatures: run bms_signatures or bms_run");
  std::vector<uint64_t> rec;
  try {
    rec.resize(s.N * kRecWords);
  } catch (const std::bad_alloc&) {
    return fail(c, BMS_ENOMEM, "out of host memory");
  }
  if (s.N) CK(cudaMemcpyAsync(rec.data(), s.frec.p, sizeof(uint64_t) * kRecWords * s.N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  const int R = s.sig_steps;
  for (uint64_t v = 0; v < s.N; ++v) {
    const uint64_t* r = rec.data() + kRecWords * v;
    if (label_gen) label_gen[v] = r[14];
    if (path)
      for (int i = 0; i < 4; ++i) path[4 * v + i] = r[2 + i];
    if (cycle)
      for (int i = 0; i < 4; ++i) cycle[4 * v + i] = uint16_t(r[1] >> (16 * i));
    if (shells)
      for (int k = 0; k < R; ++k) shells[uint64_t(k) * s.N + v] = r[6 + k];
  }
  return BMS_OK;
}

int bms_get_schedule(bms_ctx* c, bms_schedule* out) {
  GUARD(c);
  if (!out) return fail(c, BMS_EINVAL, "out is null");
  *out = c->sched;
  return BMS_OK;
}

int bms_set_schedule(bms_ctx* c, const bms_schedule* s) {
  GUARD(c);
  if (!s) return fail(c, BMS_EINVAL, "schedule is null");
  for (int i = 0; i < 3; ++i)
    if (s->blocks_per_sm[i] == 0 || s->blocks_per_sm[i] > 32 || s->warps_per_block[i] == 0 ||
        s->warps_per_block[i] > 8 || s->split_depth[i] > 1 || s->steps[i] == 0 || s->steps[i] > 4096 ||
        s->refill[i] == 0 || s->refill[i] > 32 ||
        s->split_budget[i] > (1u << 31) || (s->word_bits[i] != 32 && s->word_bits[i] != 64) ||
        (i == 0 && s->word_bits[i] != 32) || s->lanes_per_pair[i] == 0 || s->lanes_per_pair[i] > 32 ||
        (s->lanes_per_pair[i] & (s->lanes_per_pair[i] - 1)) != 0)
      return fail(c, BMS_EINVAL, "schedule entry out of range");
  const bms_schedule fixed = default_schedule();
  c->sched = *s;
  for (int i = 0; i < BMS_SCHED_BUCKETS; ++i)  // the bucket bounds are not settable
    c->sched.max_data_nodes[i] = fixed.max_data_nodes[i];
  for (int i = 3; i < BMS_SCHED_BUCKETS; ++i) {
    c->sched.word_bits[i] = fixed.word_bits[i];
    c->sched.lanes_per_pair[i] = fixed.lanes_per_pair[i];
  }
  return BMS_OK;
}

}  // extern "C"
