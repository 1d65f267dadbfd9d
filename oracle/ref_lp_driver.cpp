// C-ABI driver around the reference's LP group assembly (generate_Group_CDLP,
// Hybrid_Generation_Clean/include/vgroup/CDLP_group.cuh:20-107).
//
// TEST INFRASTRUCTURE ONLY.  The reference header is compiled where it lies
// (include path Hybrid_Generation_Clean/include of the reference checkout).
// Only its deterministic half is exercised: the label propagation it calls
// first (CDLP_GPU, vgroup/CDLP/GPU_Community_Detection.cuh:93) caps group
// sizes with racy atomics, so its output changes from run to run.  This driver
// keeps that header out (its include guard CDLPGPU is defined first) and
// supplies, in its place, a CDLP_GPU that returns the labels the caller gives
// and a CSR type the assembly never reads.  Everything after the propagation -
// bucketing by label, the greedy merge of small groups, the ordering by total
// degree - is the reference's own code.
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <set>
#include <vector>

#include <fcntl.h>
#include <unistd.h>

#include <graph_v_of_v/graph_v_of_v.h>

#define CDLPGPU  // the include guard of vgroup/CDLP/GPU_Community_Detection.cuh

template <typename weight_type>
struct CSR_graph {};

template <typename weight_type>
CSR_graph<weight_type> graph_v_of_v_to_CSR(graph_v_of_v<weight_type>&) {
  return {};
}

namespace {
std::vector<int> g_given_labels;
}

void CDLP_GPU(int, CSR_graph<int>&, std::vector<int>& res, int, int) { res = g_given_labels; }

#include <vgroup/CDLP_group.cuh>

extern "C" {

// Groups of the CSR graph (rows sorted) from propagation labels `labels`
// (each in [0, n)) by the reference's assembly; group_of_vertex[v] = index of
// v's group in the reference's output order.  Returns the number of groups.
int ref_lp_assemble(int n, const int64_t* row_ptr, const int32_t* col, const int32_t* labels, int max_group,
                    int32_t* group_of_vertex) {
  graph_v_of_v<int> g(n);
  for (int v = 0; v < n; v++)
    for (int64_t e = row_ptr[v]; e < row_ptr[v + 1]; e++) g.ADJs[v].push_back({col[e], 1});
  g_given_labels.assign(labels, labels + n);
  std::vector<std::vector<int>> groups;
  // the reference prints every group's size: stdout goes to /dev/null for
  // the call and is restored after it
  std::fflush(stdout);
  std::cout.flush();
  const int saved = dup(1), devnull = open("/dev/null", O_WRONLY);
  if (saved >= 0 && devnull >= 0) dup2(devnull, 1);
  generate_Group_CDLP(g, groups, max_group);
  std::fflush(stdout);
  std::cout.flush();
  if (saved >= 0 && devnull >= 0) dup2(saved, 1);
  if (devnull >= 0) close(devnull);
  if (saved >= 0) close(saved);
  for (size_t i = 0; i < groups.size(); i++)
    for (int v : groups[i]) group_of_vertex[v] = (int32_t)i;
  return (int)groups.size();
}

}  // extern "C"
