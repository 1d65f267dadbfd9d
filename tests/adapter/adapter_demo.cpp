// Drives include/hsdl_reference_adapter.hpp the way a program written against
// the reference's headers would: a graph_v_of_v-shaped adjacency, a
// hop_constrained_case_info-shaped record, generation + canonical repair,
// then single and batched distance queries and one path.  Prints what it got
// so the test can compare it with the C ABI's own answers.
//
// Input (stdin): n m K, then m lines "a b w" (ranked ids), then q, then q
// lines "s t k".  Output: "labels <before> <after>", "row <v> <count>" for
// every vertex, "ans <d>" per query (single-query calls) and "batch <d>" per
// query (one batched call), "path <edges>" for the first query.
#include <cstdio>
#include <cstring>
#include <vector>

#include "hsdl_reference_adapter.hpp"

struct label_like {
  int hub_vertex, parent_vertex, hop, distance;
};

struct graph_like {  // graph_v_of_v<int>: ADJs[v] = sorted (neighbour, weight) pairs
  std::vector<std::vector<std::pair<int, int>>> ADJs;
  size_t size() const { return ADJs.size(); }
  std::vector<std::pair<int, int>>& operator[](int v) { return ADJs[v]; }
};

struct case_like {  // hop_constrained_case_info
  int upper_k = 5;
  bool use_2023WWW_generation = false;
  bool use_canonical_repair = true;
  double time_initialization = 0, time_generate_labels = 0, time_sortL = 0, time_canonical_repair = 0,
         time_total = 0;
  double label_size_before_canonical_repair = 0, label_size_after_canonical_repair = 0,
         canonical_repair_remove_label_ratio = 0;
  std::vector<std::vector<label_like>> L;
};

int main(int argc, char** argv) {
  int n, m, K;
  if (std::scanf("%d %d %d", &n, &m, &K) != 3) return 2;
  graph_like g;
  g.ADJs.resize(n);
  for (int i = 0; i < m; i++) {
    int a, b, w;
    if (std::scanf("%d %d %d", &a, &b, &w) != 3) return 2;
    g.ADJs[a].push_back({b, w});
    g.ADJs[b].push_back({a, w});
  }
  for (auto& row : g.ADJs) std::sort(row.begin(), row.end());
  case_like ci;
  ci.upper_k = K;
  ci.use_2023WWW_generation = argc > 1 && std::strcmp(argv[1], "www") == 0;
  try {
    hsdl_gpu::hop_constrained_two_hop_labels_generation(g, ci);
    std::printf("labels %.0f %.0f\n", ci.label_size_before_canonical_repair, ci.label_size_after_canonical_repair);
    for (int v = 0; v < n; v++) std::printf("row %d %zu\n", v, ci.L[v].size());
    int q;
    if (std::scanf("%d", &q) != 1) return 2;
    std::vector<int32_t> s(q), t(q), k(q), out(q);
    for (int i = 0; i < q; i++)
      if (std::scanf("%d %d %d", &s[i], &t[i], &k[i]) != 3) return 2;
    hsdl_gpu::resident_labels idx(ci.L, K);
    for (int i = 0; i < q; i++) std::printf("ans %d\n", idx.extract_distance(s[i], t[i], k[i]));
    idx.query_batch(q, s.data(), t.data(), k.data(), out.data());
    for (int i = 0; i < q; i++) std::printf("batch %d\n", out[i]);
    if (q > 0) std::printf("path %zu\n", idx.extract_shortest_path(s[0], t[0], k[0]).size());
  } catch (const hsdl_gpu::error& e) {
    std::printf("error %d %s\n", e.code, e.what());
    return 1;
  }
  return 0;
}
