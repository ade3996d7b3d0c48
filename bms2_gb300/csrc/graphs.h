// Host-side batched CSR graphs and shared helpers of libbms (not part of the C ABI).
#pragma once
#include <cstdint>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/bms.h"

struct bms_graphs {
  std::vector<uint32_t> goff{0};  // [G+1]
  std::vector<uint32_t> rowp{0};  // [N+1] global
  std::vector<uint32_t> col;      // [E2] global ids
  std::vector<uint8_t> lab;       // [N]
  std::vector<uint8_t> elab;      // [E2]
  uint32_t max_nodes = 0;
  // page-locked ranges (bms_graphs_pin) and the function that releases them
  std::vector<void*> pinned;
  void (*release_pins)(bms_graphs*) = nullptr;

  bms_graphs() = default;
  bms_graphs(const bms_graphs&) = delete;
  bms_graphs& operator=(const bms_graphs&) = delete;
  ~bms_graphs() {
    if (release_pins) release_pins(this);
  }
  uint32_t n_graphs() const { return uint32_t(goff.size() - 1); }
  uint64_t n_nodes() const { return lab.size(); }
};

namespace bms {

// thread-local message for calls without a context
void set_thread_error(const std::string& msg);
const char* thread_error();

using Edge = std::tuple<uint32_t, uint32_t, uint8_t>;

// Append one graph given as labels + edge list, building its CSR exactly like
// IntermediateGraph::toCSRGraph (graph.hpp:212-243): row sizes counted per edge
// endpoint, entries filled in edge order, u's row gets v and v's row gets u.
// For a self-loop (a, a) the reference writes the same slot twice and leaves
// the second slot at its zero initial value (local node 0); that is kept.
void append_graph(bms_graphs& g, const std::vector<uint8_t>& labels, const std::vector<Edge>& edges);

// Parse one text line (graph.hpp:150-202).  Returns false with a message on a
// malformed line.
bool parse_line(const char* s, size_t len, std::vector<uint8_t>& labels, std::vector<Edge>& edges, std::string& err);

}  // namespace bms
