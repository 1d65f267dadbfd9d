// Autotuning of the build's launch shapes: threads per expansion block,
// frontier entries a block takes at a time, lanes per pruning candidate and
// hubs per wave.  Results never depend on these (every configuration yields
// the canonical labels); only the time does.
//
// One graph: the tuner times the generation of the graph's first hubs - the
// highest-ranked, whose searches are the widest and which dominate the build
// - under each candidate configuration.  A batch of graphs: it times batched
// builds of an evenly spread sample of the graphs.  The search is coordinate
// descent (hubs per wave, then block threads, then frontier tile, then prune
// lanes), keeping the incumbent unless a candidate is faster by 3%.
// No counterpart in the reference, whose launch shapes are compile-time
// constants.
#include <algorithm>
#include <chrono>
#include <functional>
#include <string>
#include <vector>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

int new_index_handle(hsdl_index** out);  // api.cu
void free_index_handle(hsdl_index* idx);  // api.cu

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Axis {
  int32_t hsdl_build_opts::*field;
  std::vector<int32_t> values;
};

// Coordinate descent over the axes; `trial` returns the seconds of one run
// (negative on error, which aborts the search with that status).
int descend(hsdl_build_opts* best, const std::vector<Axis>& axes, const std::function<double(const hsdl_build_opts&, int*)>& trial,
            double* best_s, int32_t* trials) {
  int rc = HSDL_OK;
  double inc = trial(*best, &rc);  // first run also warms up
  if (rc != HSDL_OK) return rc;
  inc = std::min(inc, trial(*best, &rc));
  if (rc != HSDL_OK) return rc;
  int32_t count = 2;
  for (const Axis& ax : axes) {
    const int32_t start = best->*ax.field;
    for (int32_t v : ax.values) {
      if (v == start) continue;
      hsdl_build_opts c = *best;
      c.*ax.field = v;
      double t = trial(c, &rc);
      count++;
      if (rc != HSDL_OK) return rc;
      if (t < inc * 0.97) {
        inc = t;
        *best = c;
      }
    }
  }
  if (best_s) *best_s = inc;
  if (trials) *trials = count;
  return HSDL_OK;
}

std::vector<Axis> axes_for(bool batched) {
  std::vector<Axis> a;
  if (batched)
    a.push_back({&hsdl_build_opts::max_wave, {65536, 131072, 262144, 524288}});
  else
    a.push_back({&hsdl_build_opts::max_wave, {1024, 2048, 4096, 8192}});
  a.push_back({&hsdl_build_opts::block_threads, {128, 256, 512}});
  a.push_back({&hsdl_build_opts::frontier_tile, {0, 1024, 4096}});
  a.push_back({&hsdl_build_opts::prune_lanes, {0, 8, 16, 32}});
  a.push_back({&hsdl_build_opts::prune_pairs, {1, 2}});
  return a;
}

}  // namespace
}  // namespace hsdl

using namespace hsdl;

extern "C" {

int hsdl_build_autotune(hsdl_graph* g, int32_t K, int32_t sample_hubs, hsdl_build_opts* opts, double* best_seconds,
                        int32_t* trials) {
  if (!g || !opts || K < 1 || K > kMaxK || opts->struct_size != (int32_t)sizeof(hsdl_build_opts)) {
    set_error("hsdl_build_autotune: bad arguments");
    return HSDL_ERR_INVALID;
  }
  if ((int64_t)K * g->max_w > (int64_t)kDistMask) {
    set_error("K * max edge weight must be < 2^28");
    return HSDL_ERR_INVALID;
  }
  // default sample: the whole generation up to 2M vertices (a prefix of hubs
  // misjudges the wave width: at n = 1M the first 16,384 hubs favoured 1024
  // hubs per wave, the whole build 8192), else the first 262,144 hubs
  const int32_t limit =
      sample_hubs > 0 ? std::min(sample_hubs, g->n) : (g->n <= 2000000 ? g->n : std::min<int32_t>(g->n, 262144));
  hsdl_build_opts best = *opts;
  if (best.max_wave == 0) best.max_wave = 4096;
  if (best.block_threads == 0) best.block_threads = 256;
  auto trial = [&](const hsdl_build_opts& c, int* rc) -> double {
    hsdl_index* idx = nullptr;
    *rc = new_index_handle(&idx);
    if (*rc != HSDL_OK) return -1;
    hsdl_build_opts o = c;
    o.clean = 0;
    *rc = build_index(g, K, o, idx, nullptr, limit);
    const double t = idx->t_gen;
    free_index_handle(idx);
    return t;
  };
  int rc = descend(&best, axes_for(false), trial, best_seconds, trials);
  if (rc != HSDL_OK) return rc;
  *opts = best;
  return HSDL_OK;
}

int hsdl_build_batched_autotune(int32_t num_graphs, const int32_t* n, const int64_t* const* row_ptr,
                                const int32_t* const* col, const int32_t* const* w, const int32_t* K,
                                int32_t sample_graphs, hsdl_build_opts* opts, double* best_seconds,
                                int32_t* trials) {
  if (num_graphs < 1 || !n || !row_ptr || !col || !w || !K || !opts ||
      opts->struct_size != (int32_t)sizeof(hsdl_build_opts)) {
    set_error("hsdl_build_batched_autotune: bad arguments");
    return HSDL_ERR_INVALID;
  }
  const int32_t S = sample_graphs > 0 ? std::min(sample_graphs, num_graphs) : std::min(num_graphs, 256);
  std::vector<int32_t> sn(S), sk(S);
  std::vector<const int64_t*> srp(S);
  std::vector<const int32_t*> scol(S), sw(S);
  for (int32_t i = 0; i < S; i++) {
    const int32_t j = (int32_t)((int64_t)i * num_graphs / S);  // spread over the input
    sn[i] = n[j];
    sk[i] = K[j];
    srp[i] = row_ptr[j];
    scol[i] = col[j];
    sw[i] = w[j];
  }
  std::vector<hsdl_index*> out((size_t)S, nullptr);
  hsdl_build_opts best = *opts;
  if (best.max_wave == 0) best.max_wave = 262144;
  if (best.block_threads == 0) best.block_threads = 256;
  auto trial = [&](const hsdl_build_opts& c, int* rc) -> double {
    hsdl_build_opts o = c;
    o.clean = 1;
    const double t0 = now_s();
    *rc = hsdl_build_batched(S, sn.data(), srp.data(), scol.data(), sw.data(), sk.data(), &o, out.data());
    const double t = now_s() - t0;
    for (auto& x : out) {
      if (x) hsdl_index_destroy(x);
      x = nullptr;
    }
    return t;
  };
  int rc = descend(&best, axes_for(true), trial, best_seconds, trials);
  if (rc != HSDL_OK) return rc;
  *opts = best;
  return HSDL_OK;
}

}  // extern "C"
