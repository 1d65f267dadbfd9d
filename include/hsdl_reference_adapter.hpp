// hsdl_reference_adapter.hpp - drop-in C++ replacements for the reference's
// HSDL entry points, implemented over the C ABI in hsdl.h.
//
// A program written against the reference headers keeps its calls and types:
// include this header after the reference's graph_v_of_v / case_info headers
// and call hsdl_gpu::hop_constrained_two_hop_labels_generation (etc.) instead
// of the CPU versions.  The functions are templates over the caller's graph
// and case-info types, so they bind to the reference's own classes without
// redefining them:
//
//   Graph    - size() and operator[](v) yielding pairs (neighbour, weight),
//              like graph_v_of_v<int> (CPU_HopHL/include/graph_v_of_v/
//              graph_v_of_v.h:46-87); vertex ids must already be ranks.
//   CaseInfo - fields upper_k, use_2023WWW_generation, use_canonical_repair, time_initialization,
//              time_generate_labels, time_sortL, time_canonical_repair,
//              time_total, label_size_before_canonical_repair,
//              label_size_after_canonical_repair,
//              canonical_repair_remove_label_ratio and
//              L (vector<vector<Label>>), like hop_constrained_case_info
//              (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:54-142).
//   Label    - fields hub_vertex, parent_vertex, hop, distance
//              (hop_constrained_two_hop_labels.h:6-21).
//
// Errors: the reference prints and exits; these functions throw
// hsdl_gpu::error carrying hsdl_last_error().
#pragma once

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hsdl.h"

namespace hsdl_gpu {

struct error : std::runtime_error {
  int code;
  error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
  if (rc != HSDL_OK) throw error(rc, hsdl_last_error());
}

// Owns a device graph built from a graph_v_of_v-like adjacency.
class device_graph {
 public:
  template <class Graph>
  explicit device_graph(Graph& g) {
    int32_t n = (int32_t)g.size();
    std::vector<int64_t> rp((size_t)n + 1, 0);
    std::vector<int32_t> col, w;
    for (int32_t v = 0; v < n; v++) {
      for (auto& e : g[v]) {
        col.push_back((int32_t)e.first);
        w.push_back((int32_t)e.second);
      }
      rp[v + 1] = (int64_t)col.size();
    }
    check(hsdl_graph_create(n, rp.data(), col.data(), w.data(), &g_));
  }
  ~device_graph() { hsdl_graph_destroy(g_); }
  device_graph(const device_graph&) = delete;
  device_graph& operator=(const device_graph&) = delete;
  hsdl_graph* get() const { return g_; }

 private:
  hsdl_graph* g_ = nullptr;
};

template <class Label>
void copy_out(hsdl_index* idx, std::vector<std::vector<Label>>& L) {
  hsdl_index_info info;
  check(hsdl_index_get_info(idx, &info));
  std::vector<int64_t> off((size_t)info.n + 1);
  std::vector<hsdl_label> lab((size_t)(info.labels > 0 ? info.labels : 1));
  check(hsdl_export(idx, off.data(), lab.data()));
  L.assign((size_t)info.n, {});
  for (int32_t v = 0; v < info.n; v++) {
    L[v].reserve((size_t)(off[v + 1] - off[v]));
    for (int64_t i = off[v]; i < off[v + 1]; i++) {
      Label x;
      x.hub_vertex = lab[i].hub_vertex;
      x.parent_vertex = lab[i].parent_vertex;
      x.hop = lab[i].hop;
      x.distance = lab[i].distance;
      L[v].push_back(x);
    }
  }
}

template <class Label>
hsdl_index* copy_in(const std::vector<std::vector<Label>>& L, int K) {
  int32_t n = (int32_t)L.size();
  std::vector<int64_t> off((size_t)n + 1, 0);
  std::vector<hsdl_label> lab;
  for (int32_t v = 0; v < n; v++) {
    for (auto& x : L[v]) lab.push_back({x.hub_vertex, x.parent_vertex, x.hop, x.distance});
    off[v + 1] = (int64_t)lab.size();
  }
  hsdl_index* idx = nullptr;
  check(hsdl_import(n, K, off.data(), lab.empty() ? nullptr : lab.data(), &idx));
  return idx;
}

// Replaces hop_constrained_two_hop_labels_generation(graph_v_of_v<int>&,
// hop_constrained_case_info&) (CPU_HopHL/include/HBPLL/
// hop_constrained_two_hop_labels_generation.h:513): fills case_info.L (sorted
// per vertex by (hub, hop, distance)), the timers and the label counts.
template <class Graph, class CaseInfo>
void hop_constrained_two_hop_labels_generation(Graph& input_graph, CaseInfo& case_info) {
  auto t0 = std::chrono::high_resolution_clock::now();
  device_graph g(input_graph);
  auto t1 = std::chrono::high_resolution_clock::now();
  hsdl_build_opts o;
  hsdl_build_opts_default(&o);
  o.clean = 0;
  o.generation = case_info.use_2023WWW_generation ? 1 : 0;  // generation.h:568-574
  hsdl_index* idx = nullptr;
  check(hsdl_build(g.get(), case_info.upper_k, &o, &idx));
  hsdl_index_info before;
  check(hsdl_index_get_info(idx, &before));
  if (case_info.use_canonical_repair) check(hsdl_clean(idx));
  hsdl_index_info info;
  check(hsdl_index_get_info(idx, &info));
  copy_out(idx, case_info.L);
  hsdl_index_destroy(idx);
  case_info.time_initialization = std::chrono::duration<double>(t1 - t0).count();
  case_info.time_generate_labels = info.time_generate_s;
  case_info.time_sortL = info.time_sort_s;
  case_info.time_canonical_repair = case_info.use_canonical_repair ? info.time_clean_s : 0.0;
  case_info.time_total = case_info.time_initialization + case_info.time_generate_labels + case_info.time_sortL +
                         case_info.time_canonical_repair;
  case_info.label_size_before_canonical_repair = (double)before.labels;
  case_info.label_size_after_canonical_repair = (double)info.labels;
  case_info.canonical_repair_remove_label_ratio =
      before.labels ? (double)(before.labels - info.labels) / (double)before.labels : 0.0;
}

// Replaces hop_constrained_clean_L(hop_constrained_case_info&, int thread_num)
// (generation.h:422).  case_info.L must be sorted per vertex, as after sortL.
template <class CaseInfo>
void hop_constrained_clean_L(CaseInfo& case_info, int /*thread_num*/) {
  hsdl_index* idx = copy_in(case_info.L, case_info.upper_k);
  hsdl_index_info before;
  check(hsdl_index_get_info(idx, &before));
  check(hsdl_clean(idx));
  hsdl_index_info info;
  check(hsdl_index_get_info(idx, &info));
  copy_out(idx, case_info.L);
  hsdl_index_destroy(idx);
  case_info.label_size_before_canonical_repair = (double)before.labels;
  case_info.label_size_after_canonical_repair = (double)info.labels;
  case_info.canonical_repair_remove_label_ratio =
      before.labels ? (double)(before.labels - info.labels) / (double)before.labels : 0.0;
}

// A resident index for repeated queries: construct once from case_info.L,
// then extract_distance / query_batch replace hop_constrained_extract_distance
// (hop_constrained_two_hop_labels.h:144) and gpu_query
// (Query_mdnd/src/gpu_query.cu:84).
class resident_labels {
 public:
  template <class Label>
  resident_labels(const std::vector<std::vector<Label>>& L, int K) : idx_(copy_in(L, K)) {}
  ~resident_labels() { hsdl_index_destroy(idx_); }
  resident_labels(const resident_labels&) = delete;
  resident_labels& operator=(const resident_labels&) = delete;

  int extract_distance(int source, int terminal, int hop_cst) {
    int32_t out = 0;
    check(hsdl_query_batch(idx_, 1, &source, &terminal, &hop_cst, &out));
    return out;
  }
  void query_batch(int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k, int32_t* out) {
    check(hsdl_query_batch(idx_, nq, s, t, k, out));
  }
  std::vector<std::pair<int, int>> extract_shortest_path(int s, int t, int k) {
    std::vector<int32_t> e(2 * 64);
    int32_t cnt = 0;
    check(hsdl_extract_path(idx_, s, t, k, e.data(), 64, &cnt));
    std::vector<std::pair<int, int>> p;
    for (int32_t i = 0; i < cnt; i++) p.push_back({e[2 * i], e[2 * i + 1]});
    return p;
  }
  hsdl_index* get() const { return idx_; }

 private:
  hsdl_index* idx_;
};

}  // namespace hsdl_gpu
