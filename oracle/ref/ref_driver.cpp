// Runs the reference's own pipeline (its headers, patched only as
// build_ref.py discloses) on the CPU through the host-only SYCL stand-in and
// dumps every intermediate, in the call order of the reference driver
// (BMS2.cpp:23-24 load, graph.hpp:251 device batch, BMS2.cpp:131-165
// signatures, :170 filter, :178-198 refinement steps, :211-212 GMCR, :231-234
// join).
//
// Test infrastructure only: it produces the fixtures the oracle and the GPU
// engine are compared with.
//
//   ref_driver QUERY_FILE DATA_FILE R OUT_DIR [join]
//
// OUT_DIR receives one raw little-endian file per array and manifest.txt
// ("name dtype count" per line).  With "join" it also runs the reference join
// over the whole GMCR (totals) and once per GMCR pair, each time over a GMCR
// that holds that one pair, so every pair's count comes from a fresh launch.
#include <sycl/sycl.hpp>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <limits>
#include <memory>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

// The per-pair runs need a GMCR holding one chosen pair; its storage is a
// private member without a setter, so the reference's headers are read with
// private members opened (every standard header they use is included above,
// so only the reference's own classes are affected).
#define private public
#include "sigmo.hpp"
#undef private

namespace {

std::string g_out;
std::ofstream g_manifest;

template <typename T>
void dump(const std::string& name, const T* p, size_t n, const char* dtype) {
  std::ofstream f(g_out + "/" + name + ".bin", std::ios::binary);
  if (n) f.write(reinterpret_cast<const char*>(p), static_cast<std::streamsize>(n * sizeof(T)));
  g_manifest << name << " " << dtype << " " << n << "\n";
}

void dump_graph(const char* side, const sigmo::DeviceBatchedCSRGraph& g) {
  const std::string s(side);
  dump(s + "_graph_offsets", g.graph_offsets, g.num_graphs + 1, "u32");
  dump(s + "_row_offsets", g.row_offsets, g.total_nodes + 1, "u32");
  dump(s + "_column_indices", g.column_indices, g.total_edges, "u32");
  dump(s + "_node_labels", g.node_labels, g.total_nodes, "u8");
  dump(s + "_edge_labels", g.edge_labels, g.total_edges, "u8");
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s QUERY_FILE DATA_FILE R OUT_DIR [join]\n", argv[0]);
    return 2;
  }
  const int R = std::stoi(argv[3]);
  g_out = argv[4];
  const bool join = argc > 5 && std::string(argv[5]) == "join";
  g_manifest.open(g_out + "/manifest.txt");

  auto query_graphs = sigmo::io::loadCSRGraphsFromFile(argv[1]);
  auto data_graphs = sigmo::io::loadCSRGraphsFromFile(argv[2]);
  sycl::queue queue;
  auto dq = sigmo::createDeviceCSRGraph(queue, query_graphs);
  auto dd = sigmo::createDeviceCSRGraph(queue, data_graphs);
  dump_graph("q", dq);
  dump_graph("d", dd);

  sigmo::candidates::Candidates candidates{queue, dq.total_nodes, dd.total_nodes};
  sigmo::signature::Signature<> signatures{queue, dd.total_nodes, dq.total_nodes};
  sigmo::signature::PathSignature path_signatures{queue, dd.total_nodes, dq.total_nodes};
  sigmo::signature::CycleSignature cycle_signatures{queue, dd.total_nodes, dq.total_nodes};

  signatures.generateDataSignatures(dd);
  path_signatures.generateDataPathSignatures(dd);
  cycle_signatures.generateDataCycleSignatures(dd);
  signatures.generateQuerySignatures(dq);
  path_signatures.generateQueryPathSignatures(dq);
  cycle_signatures.generateQueryCycleSignatures(dq);
  queue.wait_and_throw();

  static_assert(sizeof(*signatures.getDeviceDataSignatures()) == 8, "label signature is one uint64");
  static_assert(sizeof(*path_signatures.getDeviceDataSignatures()) == 32, "path signature is 4 x uint64");
  static_assert(sizeof(*cycle_signatures.getDeviceDataSignatures()) == 8, "cycle signature is 4 x uint16");
  dump("d_label_gen", reinterpret_cast<const uint64_t*>(signatures.getDeviceDataSignatures()), dd.total_nodes, "u64");
  dump("q_label_gen", reinterpret_cast<const uint64_t*>(signatures.getDeviceQuerySignatures()), dq.total_nodes, "u64");
  dump("d_path", reinterpret_cast<const uint64_t*>(path_signatures.getDeviceDataSignatures()), 4 * dd.total_nodes,
       "u64");
  dump("q_path", reinterpret_cast<const uint64_t*>(path_signatures.getDeviceQuerySignatures()), 4 * dq.total_nodes,
       "u64");
  dump("d_cycle", reinterpret_cast<const uint16_t*>(cycle_signatures.getDeviceDataSignatures()), 4 * dd.total_nodes,
       "u16");
  dump("q_cycle", reinterpret_cast<const uint16_t*>(cycle_signatures.getDeviceQuerySignatures()), 4 * dq.total_nodes,
       "u16");

  sigmo::isomorphism::filter::filterCandidates(queue, dq, dd, signatures, path_signatures, cycle_signatures,
                                               candidates);
  queue.wait_and_throw();
  const auto cdev = candidates.getCandidatesDevice();
  const size_t words = cdev.source_nodes * cdev.single_node_size;
  dump("cand_filter", cdev.candidates, words, "u32");

  for (int k = 1; k <= R; ++k) {
    signatures.refineDataSignatures(dd, k);
    signatures.refineQuerySignatures(dq, k);
    sigmo::isomorphism::filter::refineCandidates(queue, dq, dd, signatures, candidates);
    queue.wait_and_throw();
    const std::string ks = std::to_string(k);
    dump("d_shell_" + ks, reinterpret_cast<const uint64_t*>(signatures.getDeviceDataSignatures()), dd.total_nodes,
         "u64");
    dump("q_shell_" + ks, reinterpret_cast<const uint64_t*>(signatures.getDeviceQuerySignatures()), dq.total_nodes,
         "u64");
    dump("cand_step_" + ks, cdev.candidates, words, "u32");
  }

  sigmo::isomorphism::mapping::GMCR gmcr{queue};
  gmcr.generateGMCR(dq, dd, candidates);
  const auto gdev = gmcr.getGMCRDevice();
  dump("gmcr_offsets", gdev.data_graph_offsets, dd.num_graphs + 1, "u32");
  dump("gmcr_query_indices", gdev.query_graph_indices, gdev.total_query_indices, "u32");

  if (join) {
    size_t* matches = sycl::malloc_shared<size_t>(1, queue);
    for (int find_first = 1; find_first >= 0; --find_first) {
      matches[0] = 0;
      sigmo::isomorphism::join::joinCandidates(queue, dq, dd, candidates, gmcr, matches, find_first != 0);
      queue.wait_and_throw();
      const uint64_t m = matches[0];
      dump(find_first ? "join_total_find_first" : "join_total_find_all", &m, 1, "u64");
    }
    // one launch per GMCR pair (data graph d, query q)
    const size_t T = gdev.total_query_indices;
    std::vector<uint64_t> pair_ff(T), pair_fa(T);
    size_t d = 0;
    for (size_t t = 0; t < T; ++t) {
      while (gdev.data_graph_offsets[d + 1] <= t) ++d;
      sigmo::isomorphism::mapping::GMCR one{queue};
      one.gmcr.data_graph_offsets = sycl::malloc_shared<uint32_t>(dd.num_graphs + 1, queue);
      one.gmcr.query_graph_indices = sycl::malloc_shared<uint32_t>(1, queue);
      for (size_t i = 0; i <= dd.num_graphs; ++i) one.gmcr.data_graph_offsets[i] = i > d ? 1u : 0u;
      one.gmcr.query_graph_indices[0] = gdev.query_graph_indices[t];
      one.gmcr.total_query_indices = 1;
      for (int find_first = 1; find_first >= 0; --find_first) {
        matches[0] = 0;
        sigmo::isomorphism::join::joinCandidates(queue, dq, dd, candidates, one, matches, find_first != 0);
        queue.wait_and_throw();
        (find_first ? pair_ff : pair_fa)[t] = matches[0];
      }
    }
    dump("join_pair_find_first", pair_ff.data(), T, "u64");
    dump("join_pair_find_all", pair_fa.data(), T, "u64");
    sycl::free(matches, queue);
  }
  sigmo::destroyDeviceCSRGraph(dq, queue);
  sigmo::destroyDeviceCSRGraph(dd, queue);
  return 0;
}
