// C-ABI driver around the reference's own CPU implementation (CPU_HopHL).
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled against the reference's
// headers *where they lie* (include path CPU_HopHL/include of the reference
// checkout, plus oracle/shim for the two Boost names) into oracle/_ref/.
// Nothing of the reference is copied here: the driver only builds the
// reference's graph type from a CSR, calls the reference's entry points and
// copies the results out through plain pointers.
//
// Entry points called:
//   hop_constrained_two_hop_labels_generation   (CPU_HopHL/include/HBPLL/
//       hop_constrained_two_hop_labels_generation.h:513)
//   hop_constrained_extract_distance            (CPU_HopHL/include/HBPLL/
//       hop_constrained_two_hop_labels.h:144)
//   hop_constrained_extract_shortest_path       (same file, :224)
//   graph_v_of_v_hop_constrained_shortest_distance (CPU_HopHL/include/
//       graph_v_of_v/graph_v_of_v_hop_constrained_shortest_distance.h:7)
#include <HBPLL/test.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>

namespace {

struct RefResult {
  std::vector<std::vector<hop_constrained_two_hop_label>> L;
  double t_init = 0, t_gen = 0, t_sort = 0, t_clean = 0;
  double before = 0, after = 0;
};

RefResult g_last;
graph_v_of_v<int> g_graph;

void load_graph(int n, const int64_t* row_ptr, const int32_t* col, const int32_t* w) {
  g_graph = graph_v_of_v<int>(n);
  for (int v = 0; v < n; v++) {
    auto& adj = g_graph.ADJs[v];
    adj.reserve(row_ptr[v + 1] - row_ptr[v]);
    // The CSR rows are sorted by neighbour id, which is the order the
    // reference's sorted-vector add_edge keeps.
    for (int64_t e = row_ptr[v]; e < row_ptr[v + 1]; e++) adj.push_back({col[e], w[e]});
  }
}

}  // namespace

extern "C" {

// Runs generation (+ sortL, + canonical repair if `clean`) with the reference's
// thread pool of `threads` workers; `www` selects the reference's 2023WWW
// generation (_2023WWW_thread_function, hop_constrained_two_hop_labels_generation.h:226-370)
// instead of HSDL_thread_function.  Returns the total label count.
int64_t ref_build(int n, const int64_t* row_ptr, const int32_t* col, const int32_t* w, int K,
                  int threads, int clean, int www) {
  load_graph(n, row_ptr, col, w);
  hop_constrained_case_info mm;
  mm.upper_k = K;
  mm.use_rank_prune = 1;
  mm.use_2023WWW_generation = www ? 1 : 0;
  mm.use_canonical_repair = clean ? 1 : 0;
  mm.thread_num = threads;
  hop_constrained_two_hop_labels_generation(g_graph, mm);
  g_last.L.swap(mm.L);
  g_last.t_init = mm.time_initialization;
  g_last.t_gen = mm.time_generate_labels;
  g_last.t_sort = mm.time_sortL;
  g_last.t_clean = mm.time_canonical_repair;
  g_last.before = clean ? mm.label_size_before_canonical_repair : 0;
  g_last.after = clean ? mm.label_size_after_canonical_repair : 0;
  int64_t total = 0;
  for (auto& x : g_last.L) total += (int64_t)x.size();
  return total;
}

// times[0..3] = initialization, generation, sortL, canonical repair (seconds)
void ref_times(double* times) {
  times[0] = g_last.t_init;
  times[1] = g_last.t_gen;
  times[2] = g_last.t_sort;
  times[3] = g_last.t_clean;
}

// offsets: n+1 int64; labels: total*4 int32 as (hub, parent, hop, distance)
void ref_export(int64_t* offsets, int32_t* labels) {
  int64_t pos = 0;
  offsets[0] = 0;
  for (size_t v = 0; v < g_last.L.size(); v++) {
    for (auto& x : g_last.L[v]) {
      labels[4 * pos + 0] = x.hub_vertex;
      labels[4 * pos + 1] = x.parent_vertex;
      labels[4 * pos + 2] = x.hop;
      labels[4 * pos + 3] = x.distance;
      pos++;
    }
    offsets[v + 1] = pos;
  }
}

// Answers queries with the reference merge-join over the last build's labels.
// threads == 1 is the reference's single-thread query loop; more threads split
// the query list into contiguous chunks.
void ref_query(int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k, int32_t* out,
               int threads) {
  auto work = [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; i++) out[i] = hop_constrained_extract_distance(g_last.L, s[i], t[i], k[i]);
  };
  if (threads <= 1) {
    work(0, nq);
    return;
  }
  std::vector<std::thread> pool;
  int64_t chunk = (nq + threads - 1) / threads;
  for (int i = 0; i < threads; i++) {
    int64_t lo = i * chunk, hi = std::min<int64_t>(nq, lo + chunk);
    if (lo < hi) pool.emplace_back(work, lo, hi);
  }
  for (auto& th : pool) th.join();
}

// Hop-bounded Bellman-Ford distances from `src` on the last loaded graph.
void ref_bf(int src, int k, int32_t* dist_out) {
  std::vector<int> d;
  graph_v_of_v_hop_constrained_shortest_distance(g_graph, src, k, d);
  for (size_t i = 0; i < d.size(); i++) dist_out[i] = d[i];
}

// Path extraction over the last build's labels.  Writes up to `cap` edges as
// (a, b) pairs and returns the number of edges (or -1 if cap is too small).
int ref_path(int s, int t, int k, int32_t* edges, int cap) {
  auto p = hop_constrained_extract_shortest_path(g_last.L, s, t, k);
  if ((int)p.size() > cap) return -1;
  for (size_t i = 0; i < p.size(); i++) {
    edges[2 * i] = p[i].first;
    edges[2 * i + 1] = p[i].second;
  }
  return (int)p.size();
}

}  // extern "C"
