// Data-graph shards across GPUs: the reference MPI driver's load balancing
// (BMS2_mpi.cpp:78-157) as a host routine.  Cost of a data graph = nodes^2 +
// edges (edges = CSR entries / 2); graphs are taken by decreasing cost (a
// stable order: equal costs keep their batch order) and each goes to the rank
// with the smallest load so far (the lowest rank among equal loads).
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <queue>
#include <vector>

#include "../../include/bms.h"
#include "graphs.h"

extern "C" int bms_shard_lpt(uint32_t n_graphs, const uint32_t* graph_offsets, const uint32_t* row_offsets,
                             uint32_t world, uint32_t* owners, double* loads) {
  if (world == 0 || (n_graphs && (!graph_offsets || !row_offsets || !owners))) {
    bms::set_thread_error("bms_shard_lpt: world must be >= 1 and the arrays non-null");
    return BMS_EINVAL;
  }
  try {
    std::vector<double> cost(n_graphs);
    for (uint32_t g = 0; g < n_graphs; ++g) {
      const uint32_t a = graph_offsets[g], b = graph_offsets[g + 1];
      if (b < a) {
        bms::set_thread_error("bms_shard_lpt: graph_offsets must be non-decreasing");
        return BMS_EINVAL;
      }
      const double nodes = double(b - a);
      const double edges = double((row_offsets[b] - row_offsets[a]) / 2u);
      cost[g] = std::max(1.0, nodes * nodes + edges);
    }
    std::vector<uint32_t> order(n_graphs);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return cost[x] > cost[y]; });
    // min-heap on (load, rank): the least-loaded rank, the lowest on ties
    using Slot = std::pair<double, uint32_t>;
    std::priority_queue<Slot, std::vector<Slot>, std::greater<Slot>> heap;
    for (uint32_t r = 0; r < world; ++r) heap.push({0.0, r});
    for (uint32_t g : order) {
      Slot s = heap.top();
      heap.pop();
      owners[g] = s.second;
      s.first += cost[g];
      heap.push(s);
    }
    if (loads) {
      std::fill(loads, loads + world, 0.0);
      while (!heap.empty()) {
        loads[heap.top().second] = heap.top().first;
        heap.pop();
      }
    }
  } catch (const std::bad_alloc&) {
    return BMS_ENOMEM;
  }
  return BMS_OK;
}
