// bms.hpp — C++ facade over the C ABI (bms.h) shaped like the reference's
// `sigmo` library API, so a driver written against the reference maps call for
// call.  Errors throw std::runtime_error, as the reference does (graph.hpp:200,
// signature.hpp:82).  Header-only; link libbms.so.
//
//   reference (namespace sigmo)                         here (namespace bms::sigmo)
//   io::loadCSRGraphsFromFile (io.hpp:43)               io::loadCSRGraphsFromFile
//   createDeviceCSRGraph (graph.hpp:251)                createDeviceCSRGraph
//   Signature<>::generate/refine{Data,Query}Signatures  Signature::generate.../refine...
//     (signature.hpp:56-73), PathSignature (:455-470),  PathSignature, CycleSignature
//     CycleSignature (:574-589)
//   Candidates{queue, Qn, Dn} (candidates.hpp:161)      Candidates
//   isomorphism::filter::filterCandidates (isomorphism.hpp:30)   filter::filterCandidates
//   isomorphism::filter::refineCandidates (isomorphism.hpp:106)  filter::refineCandidates
//   isomorphism::mapping::GMCR::generateGMCR (gmcr.hpp:35)       mapping::GMCR::generateGMCR
//   isomorphism::join::joinCandidates (isomorphism.hpp:291)      join::joinCandidates
//   joinPartialCandidates2 + joinWithPartialMatches (:1021, :756) join::joinWithPartialMatches
//
// The reference's stage objects each own device memory; here one Queue owns a
// bms_ctx and the stage objects are views on it.  Signatures are computed for
// both sides at once: generateDataSignatures + generateQuerySignatures of all
// three kinds and refine*Signatures(k) for k = 1..R collapse into one
// bms_signatures(R) call, issued lazily by the first filter.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "bms.h"

namespace bms {
namespace sigmo {

inline void check(int st, const void* ctx = nullptr) {
  if (st != BMS_OK) throw std::runtime_error(std::string(bms_status_name(st)) + ": " + bms_last_error(ctx));
}

// A batch of graphs on the host (the reference's std::vector<CSRGraph>).
class GraphBatch {
 public:
  GraphBatch() = default;
  explicit GraphBatch(bms_graphs* g) : g_(g) {}
  GraphBatch(GraphBatch&& o) noexcept : g_(o.g_) { o.g_ = nullptr; }
  GraphBatch& operator=(GraphBatch&& o) noexcept {
    if (this != &o) {
      bms_graphs_free(g_);
      g_ = o.g_;
      o.g_ = nullptr;
    }
    return *this;
  }
  GraphBatch(const GraphBatch&) = delete;
  GraphBatch& operator=(const GraphBatch&) = delete;
  ~GraphBatch() { bms_graphs_free(g_); }
  const bms_graphs* get() const { return g_; }
  bms_graphs_view view() const {
    bms_graphs_view v{};
    check(bms_graphs_view_of(g_, &v));
    return v;
  }
  size_t size() const { return view().n_graphs; }
  // --query-filter min:max (BMS2.cpp:27-34)
  GraphBatch filterSize(uint32_t min_nodes, uint32_t max_nodes) const {
    bms_graphs* out = nullptr;
    check(bms_graphs_filter_size(g_, min_nodes, max_nodes, &out));
    return GraphBatch(out);
  }

 private:
  bms_graphs* g_ = nullptr;
};

namespace io {
// io::loadCSRGraphsFromFile (io.hpp:43-52)
inline GraphBatch loadCSRGraphsFromFile(const std::string& filename, uint32_t max_graphs = 0) {
  bms_graphs* g = nullptr;
  check(bms_graphs_parse_file(filename.c_str(), max_graphs, 0, &g));
  return GraphBatch(g);
}
}  // namespace io

// The reference's sycl::queue: one device, one stream, one engine context.
class Queue {
 public:
  explicit Queue(int device = 0) { check(bms_create(device, &ctx_)); }
  Queue(const Queue&) = delete;
  Queue& operator=(const Queue&) = delete;
  ~Queue() { bms_destroy(ctx_); }
  bms_ctx* ctx() const { return ctx_; }
  int refine_steps = -1;       // steps requested so far (signatures are computed once for R)
  bool signatures_done = false;

 private:
  bms_ctx* ctx_ = nullptr;
};

struct DeviceBatchedCSRGraph {
  int kind;
  uint32_t num_graphs;
  size_t total_nodes;
};

// createDeviceCSRGraph (graph.hpp:251-310).  The first call uploads the query
// side, the second the data side, matching the reference driver (BMS2.cpp:50-51);
// pass kind explicitly to choose.
inline DeviceBatchedCSRGraph createDeviceCSRGraph(Queue& q, const GraphBatch& g, int kind) {
  check(bms_load_graphs(q.ctx(), kind, g.get()), q.ctx());
  q.signatures_done = false;
  const bms_graphs_view v = g.view();
  return DeviceBatchedCSRGraph{kind, v.n_graphs, size_t(v.n_nodes)};
}

namespace signature {
// Signature<>, PathSignature, CycleSignature: refinement steps are recorded and
// the signatures are produced by one device pass when the filter first needs them.
class Signature {
 public:
  Signature(Queue& q, size_t, size_t) : q_(q) {}
  void generateDataSignatures(const DeviceBatchedCSRGraph&) {}
  void generateQuerySignatures(const DeviceBatchedCSRGraph&) {}
  void refineDataSignatures(const DeviceBatchedCSRGraph&, size_t view_size) { note(view_size); }
  void refineQuerySignatures(const DeviceBatchedCSRGraph&, size_t view_size) { note(view_size); }
  void ensure() {
    if (!q_.signatures_done) {
      check(bms_signatures(q_.ctx(), q_.refine_steps < 0 ? 0 : q_.refine_steps), q_.ctx());
      q_.signatures_done = true;
    }
  }
  Queue& queue() { return q_; }

 private:
  void note(size_t k) {
    if (int(k) > q_.refine_steps) {
      q_.refine_steps = int(k);
      q_.signatures_done = false;
    }
  }
  Queue& q_;
};
class PathSignature {
 public:
  PathSignature(Queue&, size_t, size_t) {}
  void generateDataPathSignatures(const DeviceBatchedCSRGraph&) {}
  void generateQueryPathSignatures(const DeviceBatchedCSRGraph&) {}
};
class CycleSignature {
 public:
  CycleSignature(Queue&, size_t, size_t) {}
  void generateDataCycleSignatures(const DeviceBatchedCSRGraph&) {}
  void generateQueryCycleSignatures(const DeviceBatchedCSRGraph&) {}
};
}  // namespace signature

namespace candidates {
// Candidates (candidates.hpp:10-200): the dense query-major bitset.
class Candidates {
 public:
  Candidates(Queue& q, size_t source_nodes, size_t target_nodes)
      : q_(q), source_(source_nodes), words_((target_nodes + 31) / 32) {}
  // getHostCandidates (candidates.hpp:181-186)
  std::vector<uint32_t> getHostCandidates() const {
    std::vector<uint32_t> w(source_ * words_);
    check(bms_get_candidates(q_.ctx(), w.data(), w.size()), q_.ctx());
    return w;
  }
  // getCandidatesCount(source) (candidates.hpp:73-77)
  static uint32_t count(const std::vector<uint32_t>& host, size_t words, size_t source) {
    uint32_t c = 0;
    for (size_t i = 0; i < words; ++i) c += uint32_t(__builtin_popcount(host[source * words + i]));
    return c;
  }
  size_t wordsPerRow() const { return words_; }
  Queue& queue() const { return q_; }

 private:
  Queue& q_;
  size_t source_, words_;
};
}  // namespace candidates

namespace isomorphism {
namespace filter {
// filterCandidates (isomorphism.hpp:30-104)
inline void filterCandidates(Queue& q, const DeviceBatchedCSRGraph&, const DeviceBatchedCSRGraph&,
                             signature::Signature& sig, signature::PathSignature&, signature::CycleSignature&,
                             candidates::Candidates&) {
  sig.ensure();
  check(bms_filter(q.ctx()), q.ctx());
}
// refineCandidates (isomorphism.hpp:106-203) with the shell of step k.
inline void refineCandidates(Queue& q, const DeviceBatchedCSRGraph&, const DeviceBatchedCSRGraph&,
                             signature::Signature& sig, candidates::Candidates&, int step) {
  sig.ensure();
  check(bms_refine(q.ctx(), step), q.ctx());
}
}  // namespace filter

namespace mapping {
// GMCR (gmcr.hpp:16-145)
class GMCR {
 public:
  explicit GMCR(Queue& q) : q_(q) {}
  size_t generateGMCR(const DeviceBatchedCSRGraph&, const DeviceBatchedCSRGraph&, candidates::Candidates&) {
    uint64_t n = 0;
    check(bms_map(q_.ctx(), &n), q_.ctx());
    total_ = n;
    return size_t(n);
  }
  size_t total_query_indices() const { return total_; }
  void copyToHost(std::vector<uint32_t>& data_graph_offsets, std::vector<uint32_t>& query_graph_indices,
                  uint32_t num_data_graphs) const {
    data_graph_offsets.resize(num_data_graphs + 1);
    query_graph_indices.resize(total_);
    check(bms_get_gmcr(q_.ctx(), data_graph_offsets.data(), query_graph_indices.data(), total_), q_.ctx());
  }

 private:
  Queue& q_;
  size_t total_ = 0;
};
}  // namespace mapping

namespace join {
// joinCandidates (isomorphism.hpp:291-472): *num_matches += sum of per-pair
// counts (find_first: pairs with a match).
inline void joinCandidates(Queue& q, const DeviceBatchedCSRGraph&, const DeviceBatchedCSRGraph&,
                           candidates::Candidates&, mapping::GMCR&, size_t* num_matches, bool find_first = true,
                           int order = BMS_ORDER_GMCR, int semantics = BMS_SEM_EXACT) {
  uint64_t total = 0;
  check(bms_join(q.ctx(), find_first ? BMS_FIND_FIRST : BMS_COUNT_ALL, order, semantics, &total), q.ctx());
  *num_matches += size_t(total);
}

// The --use-cs pair joinPartialCandidates2 (isomorphism.hpp:1021-1178) +
// joinWithPartialMatches (:756-977) as one call: query 0 is the prototype, the
// partial matches stay on the device; *num_partial_matches (nullable) receives
// their number.  The context's plain-join setting is restored afterwards.
inline void joinWithPartialMatches(Queue& q, const DeviceBatchedCSRGraph&, const DeviceBatchedCSRGraph&,
                                   candidates::Candidates&, mapping::GMCR&, size_t* num_matches, bool find_first = true,
                                   int semantics = BMS_SEM_EXACT, size_t* num_partial_matches = nullptr) {
  check(bms_set_option(q.ctx(), BMS_OPT_USE_CS, 1), q.ctx());
  uint64_t total = 0;
  const int st = bms_join(q.ctx(), find_first ? BMS_FIND_FIRST : BMS_COUNT_ALL, BMS_ORDER_GMCR, semantics, &total);
  bms_set_option(q.ctx(), BMS_OPT_USE_CS, 0);
  check(st, q.ctx());
  *num_matches += size_t(total);
  if (num_partial_matches) {
    bms_stats s{};
    check(bms_get_stats(q.ctx(), &s), q.ctx());
    *num_partial_matches = size_t(s.n_partial_matches);
  }
}
}  // namespace join
}  // namespace isomorphism

}  // namespace sigmo
}  // namespace bms
