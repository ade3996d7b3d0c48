// bms2 — command-line driver of libbms with the reference driver's flags
// (library/src/BMS2.cpp:7-393, flags library/src/utils.hpp:39-87):
//   -Q FILE -D FILE        query and data graphs (reference text format)
//   -i N                   refinement steps (default 0, as the reference)
//   --find-all             count every embedding (default: find-first per pair)
//   --max-data-graphs N    (default 1000000)   --max-query-graphs N (default 1000)
//   --query-filter A[:B]   keep queries with A..B nodes
//   -m/-d/-q K             replicate all / data / query graphs K times
//   --skip-join            stop after the mapping
//   -p                     print candidates per query node (staged pipeline)
//   --skip-candidates-analysis
//   --use-cs               clustered join: query 0 is the prototype (BMS2.cpp:218-296)
// and the engine's own:
//   --staged               run the reference-shaped staged pipeline (dense matrix)
//   --order gmcr|learned   search order (learned needs --model FILE)
//   --semantics exact|reference
//   --device N  --json
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "bms.hpp"

using namespace bms::sigmo;

namespace {

struct Args {
  std::string qfile, dfile, order = "gmcr", semantics = "exact", model;
  int steps = 0, device = 0;
  bool find_all = false, skip_join = false, print_cand = false, skip_cand = false, staged = false, json = false;
  bool use_cs = false;
  size_t max_data = 1000000, max_query = 1000, mul_data = 1, mul_query = 1;
  bool qfilter = false;
  uint32_t qmin = 0, qmax = 0xFFFFFFFFu;
};

[[noreturn]] void usage(const char* msg) {
  std::fprintf(stderr, "bms2: %s\n", msg);
  std::fprintf(stderr,
               "usage: bms2 -Q queries -D data [-i steps] [--find-all] [--max-data-graphs N] [--max-query-graphs N]\n"
               "            [--query-filter A[:B]] [-m K|-d K|-q K] [--skip-join] [-p] [--skip-candidates-analysis]\n"
               "            [--use-cs]\n"
               "            [--staged] [--order gmcr|learned --model FILE] [--semantics exact|reference] [--device N]\n"
               "            [--json]\n");
  std::exit(2);
}

Args parse(int argc, char** argv) {
  Args a;
  auto need = [&](int& i) -> const char* {
    if (i + 1 >= argc) usage("missing value");
    return argv[++i];
  };
  for (int i = 1; i < argc; ++i) {
    std::string s = argv[i];
    if (s == "-Q") a.qfile = need(i);
    else if (s == "-D") a.dfile = need(i);
    else if (s == "-i" || s == "--iterations") a.steps = std::atoi(need(i));
    else if (s == "--find-all") a.find_all = true;
    else if (s == "--skip-join") a.skip_join = true;
    else if (s == "--use-cs") a.use_cs = true;
    else if (s == "-p" || s == "--print-candidates") a.print_cand = true;
    else if (s == "--skip-candidates-analysis") a.skip_cand = true;
    else if (s == "--max-data-graphs") a.max_data = std::strtoull(need(i), nullptr, 10);
    else if (s == "--max-query-graphs") a.max_query = std::strtoull(need(i), nullptr, 10);
    else if (s == "-m" || s == "--multiply") a.mul_data = a.mul_query = std::strtoull(need(i), nullptr, 10);
    else if (s == "-d" || s == "--mul-data") a.mul_data = std::strtoull(need(i), nullptr, 10);
    else if (s == "-q" || s == "--mul-query") a.mul_query = std::strtoull(need(i), nullptr, 10);
    else if (s == "--query-filter") {
      std::string f = need(i);
      a.qfilter = true;
      size_t c = f.find(':');
      a.qmin = uint32_t(std::atoi(f.substr(0, c).c_str()));
      if (c != std::string::npos) a.qmax = uint32_t(std::atoi(f.substr(c + 1).c_str()));
    } else if (s == "--staged") a.staged = true;
    else if (s == "--order") a.order = need(i);
    else if (s == "--model") a.model = need(i);
    else if (s == "--semantics") a.semantics = need(i);
    else if (s == "--device") a.device = std::atoi(need(i));
    else if (s == "--json") a.json = true;
    else if (s == "-c" || s == "--candidates-domain") need(i);  // only the query domain exists
    else usage(("unknown flag " + s).c_str());
  }
  if (a.qfile.empty() || a.dfile.empty()) usage("Both query and data files must be provided");
  if (a.order != "gmcr" && a.order != "learned") usage("--order must be gmcr or learned");
  if (a.semantics != "exact" && a.semantics != "reference") usage("--semantics must be exact or reference");
  if (a.mul_data == 0 || a.mul_query == 0) usage("multiply factors must be positive");
  return a;
}

// Replicate a batch k times and cut it to at most `limit` graphs (BMS2.cpp:40-49).
GraphBatch replicate(const GraphBatch& g, size_t k, size_t limit) {
  const bms_graphs_view v = g.view();
  const size_t G = std::min<size_t>(size_t(v.n_graphs) * k, limit);
  std::vector<uint32_t> goff{0}, rowp{0}, col;
  std::vector<uint8_t> lab, el;
  for (size_t i = 0; i < G; ++i) {
    const size_t src = i % v.n_graphs;
    const uint32_t s = v.graph_offsets[src], e = v.graph_offsets[src + 1];
    const uint32_t nb = uint32_t(lab.size()), eb = uint32_t(col.size());
    for (uint32_t x = s; x < e; ++x) {
      lab.push_back(v.node_labels[x]);
      rowp.push_back(eb + (v.row_offsets[x + 1] - v.row_offsets[s]));
    }
    for (uint32_t j = v.row_offsets[s]; j < v.row_offsets[e]; ++j) {
      col.push_back(v.column_indices[j] - s + nb);
      el.push_back(v.edge_labels[j]);
    }
    goff.push_back(nb + (e - s));
  }
  bms_graphs* out = nullptr;
  check(bms_graphs_from_csr(uint32_t(G), goff.data(), rowp.data(), col.data(), lab.data(), el.data(), &out));
  return GraphBatch(out);
}

}  // namespace

int main(int argc, char** argv) {
  try {
    const Args a = parse(argc, argv);
    auto t0 = std::chrono::steady_clock::now();
    GraphBatch qg = io::loadCSRGraphsFromFile(a.qfile);
    GraphBatch dg = io::loadCSRGraphsFromFile(a.dfile);
    if (a.qfilter) qg = qg.filterSize(a.qmin, a.qmax);
    qg = replicate(qg, a.mul_query, a.max_query);
    dg = replicate(dg, a.mul_data, a.max_data);
    auto t1 = std::chrono::steady_clock::now();
    Queue queue(a.device);
    auto q = createDeviceCSRGraph(queue, qg, BMS_QUERY);
    auto d = createDeviceCSRGraph(queue, dg, BMS_DATA);
    const int mode = a.find_all ? BMS_COUNT_ALL : BMS_FIND_FIRST;
    const int order = a.order == "learned" ? BMS_ORDER_LEARNED : BMS_ORDER_GMCR;
    const int sem = a.semantics == "reference" ? BMS_SEM_REFERENCE_DFS : BMS_SEM_EXACT;
    if (order == BMS_ORDER_LEARNED) {
      if (a.model.empty()) usage("--order learned needs --model FILE");
      check(bms_model_load(queue.ctx(), a.model.c_str()), queue.ctx());
    }
    if (a.use_cs) check(bms_set_option(queue.ctx(), BMS_OPT_USE_CS, 1), queue.ctx());
    size_t matches = 0;
    uint64_t pairs = 0;
    std::vector<uint32_t> cand_counts;
    if (a.staged || a.print_cand || a.skip_join) {
      signature::Signature sig(queue, d.total_nodes, q.total_nodes);
      signature::PathSignature path(queue, d.total_nodes, q.total_nodes);
      signature::CycleSignature cyc(queue, d.total_nodes, q.total_nodes);
      candidates::Candidates cand(queue, q.total_nodes, d.total_nodes);
      for (int k = 1; k <= a.steps; ++k) {
        sig.refineDataSignatures(d, size_t(k));
        sig.refineQuerySignatures(q, size_t(k));
      }
      isomorphism::filter::filterCandidates(queue, q, d, sig, path, cyc, cand);
      for (int k = 1; k <= a.steps; ++k) isomorphism::filter::refineCandidates(queue, q, d, sig, cand, k);
      if (!a.skip_cand) {
        const auto host = cand.getHostCandidates();
        for (size_t u = 0; u < q.total_nodes; ++u)
          cand_counts.push_back(candidates::Candidates::count(host, cand.wordsPerRow(), u));
      }
      if (!a.skip_join) {
        isomorphism::mapping::GMCR gmcr(queue);
        pairs = gmcr.generateGMCR(q, d, cand);
        isomorphism::join::joinCandidates(queue, q, d, cand, gmcr, &matches, !a.find_all, order, sem);
      }
    } else {
      uint64_t total = 0;
      check(bms_run(queue.ctx(), a.steps, mode, order, sem, &total), queue.ctx());
      matches = size_t(total);
    }
    bms_stats st{};
    check(bms_get_stats(queue.ctx(), &st), queue.ctx());
    if (!pairs) pairs = st.n_valid_pairs;
    auto t2 = std::chrono::steady_clock::now();
    const double load_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    const double run_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    if (a.json) {
      std::printf("{\"query_graphs\":%u,\"data_graphs\":%u,\"query_nodes\":%llu,\"data_nodes\":%llu,\"gmcr_pairs\":%llu,"
                  "\"matches\":%zu,\"expansions\":%llu,\"load_ms\":%.3f,\"run_ms\":%.3f,\"device_ms\":%.3f}\n",
                  st.n_query_graphs, st.n_data_graphs, (unsigned long long)st.n_query_nodes,
                  (unsigned long long)st.n_data_nodes, (unsigned long long)pairs, matches,
                  (unsigned long long)st.expansions, load_ms, run_ms, st.ms_total);
      return 0;
    }
    std::printf("------------- Input Data -------------\n");
    std::printf("# Query Nodes %llu\n# Query Graphs %u\n# Data Nodes %llu\n# Data Graphs %u\n",
                (unsigned long long)st.n_query_nodes, st.n_query_graphs, (unsigned long long)st.n_data_nodes,
                st.n_data_graphs);
    std::printf("------------- Configs -------------\nFind all: %s\nRefinement steps: %d\nOrder: %s\nSemantics: %s\n",
                a.find_all ? "Yes" : "No", a.steps, a.order.c_str(), a.semantics.c_str());
    std::printf("------------- Overall Stats -------------\n");
    std::printf("Load time: %.1f ms (not included in total)\nTotal time: %.1f ms\n", load_ms, run_ms);
    std::printf("------------- Results -------------\n");
    if (!cand_counts.empty()) {
      std::vector<uint32_t> s = cand_counts;
      uint64_t tot = 0, zero = 0;
      for (uint32_t c : s) {
        tot += c;
        zero += c == 0;
      }
      std::sort(s.begin(), s.end());
      std::printf("# Total candidates: %llu\n# Average candidates: %llu\n# Median candidates: %u\n"
                  "# Zero candidates: %llu\n",
                  (unsigned long long)tot, (unsigned long long)(tot / s.size()), s[s.size() / 2],
                  (unsigned long long)zero);
      if (a.print_cand)
        for (size_t u = 0; u < cand_counts.size(); ++u) std::fprintf(stderr, "Node %zu: %u\n", u, cand_counts[u]);
    }
    if (!a.skip_join && a.use_cs) std::printf("# Partial matches: %llu\n", (unsigned long long)st.n_partial_matches);
    if (!a.skip_join) std::printf("# GMCR pairs: %llu\n# Matches: %zu\n", (unsigned long long)pairs, matches);
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "bms2: %s\n", e.what());
    return 1;
  }
}
