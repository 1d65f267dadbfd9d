// Batched build: many independent graphs indexed together.
//
// The reference builds one graph per run (hop_constrained_two_hop_labels_
// generation, CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_
// generation.h:513; label_gen, Hybrid_Generation_Clean/src/label_gen.cu:603).
// Here a batch of graphs is laid out as one disjoint union whose vertex order
// interleaves the graphs by rank: all graphs' rank-0 vertices first, then all
// rank-1 vertices, and so on.  Inside every graph the rank order is kept, so
// the hop-bounded searches of the union are exactly the per-graph searches
// (no path leaves a graph) and the cleaned labels of each graph are its own
// canonical labels.  A wave covers a range of rank layers: it holds the hubs
// of the same ranks of many graphs at once - thousands of independent hubs in
// flight - while within one graph only a few consecutive ranks share a wave.
// The wave engine (gen.cu) gives every slot a candidate row as long as its
// own graph and stops each graph's search at its own hop bound.  Graphs are
// grouped into sub-batches whose estimated labels fit the device budget; each
// sub-batch is one union build and clean, then one kernel scatters the
// union's rows into per-graph indexes with ids mapped back to each graph's own.
#include <algorithm>
#include <cmath>
#include <deque>
#include <numeric>
#include <string>
#include <vector>

#include "hsdl_device.cuh"
#include "hsdl_internal.h"
#include "hsdl_runtime.h"

namespace hsdl {

int new_index_handle(hsdl_index** out);  // api.cu
void free_index_handle(hsdl_index* idx);  // api.cu
int upload_graph(int32_t n, const int64_t* rp, const int32_t* col, const int32_t* w, hsdl_graph_impl* g);  // api.cu

namespace {

__global__ void k_split(int64_t nu, const int64_t* __restrict__ uoff, const uint64_t* __restrict__ ukey,
                        const int32_t* __restrict__ upar, const int32_t* __restrict__ comp,
                        const int32_t* __restrict__ lid, const int64_t* __restrict__ dst,
                        uint64_t* const* __restrict__ dkey, int32_t* const* __restrict__ dpar) {
  const int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = warp; u < nu; u += nwarps) {
    const int g = comp[u];
    const int64_t lo = uoff[u], len = uoff[u + 1] - lo, at = dst[u];
    uint64_t* ok = dkey[g];
    int32_t* op = dpar[g];
    for (int64_t j = lane; j < len; j += 32) {
      const uint64_t k = ukey[lo + j];
      ok[at + j] = ((uint64_t)(uint32_t)lid[lkey_hub(k)] << 32) | lkey_hd(k);  // hub id inside its own graph
      op[at + j] = lid[upar[lo + j]];
    }
  }
}

// Labels of one graph, for admission into a sub-batch only: labels per vertex
// ~ 0.53 sqrt(n) (avg_deg / 10) (K / 5), at least 2 avg_deg^(K/2) for graphs
// without hubs, capped by n (K + 1); 16 bytes per label with generation slack.
int64_t batch_estimate_bytes(int32_t n, int64_t m2, int32_t K) {
  double avg = n ? (double)m2 / n : 0.0;
  // twice the power-law rule of thumb: on the 4,096-graph ER/BA batch the
  // rule alone predicted 1.62 G labels for the first 1,024 graphs, which had
  // 3.34 G (a build peak of 31 B per label against the 48 B allowed here)
  double pv = 2.0 * std::max(0.53 * std::sqrt((double)n) * std::max(0.25, avg / 10.0) * (K / 5.0),
                             2.0 * std::pow(std::max(1.0, avg), K / 2.0));
  pv = std::min(pv, (double)n * (K + 1));
  return (int64_t)(48.0 * std::max(1.0, pv) * n) + 64 * (int64_t)n + 16 * m2;
}

struct GraphIn {
  int32_t n;
  const int64_t* rp;
  const int32_t* col;
  const int32_t* w;
  int32_t K;
};

int build_sub_batch(const std::vector<GraphIn>& G, const std::vector<int32_t>& members,
                    const hsdl_build_opts& opts, hsdl_index** out) {
  const int B = (int)members.size();
  // rank-interleaved layout: graphs ordered by size (largest first) so layer r
  // holds a prefix of them
  std::vector<int32_t> order(members);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return G[a].n > G[b].n; });
  int32_t max_n = G[order[0]].n;
  std::vector<int64_t> layer_start((size_t)max_n + 1, 0);
  {
    int p = B;
    for (int32_t r = 0; r < max_n; r++) {
      while (p > 0 && G[order[p - 1]].n <= r) p--;
      layer_start[r + 1] = layer_start[r] + p;
    }
  }
  const int64_t nu = layer_start[max_n];
  if (nu >= (int64_t)kIdMask) {
    set_error("batched build: sub-batch exceeds 2^28 vertices");
    return HSDL_ERR_INVALID;
  }
  // gid(b, r) = layer_start[r] + pos(b)
  auto gid = [&](int pos, int32_t r) -> int32_t { return (int32_t)(layer_start[r] + pos); };
  std::vector<int32_t> comp((size_t)nu), lid((size_t)nu);
  std::vector<uint8_t> vk((size_t)nu);
  BatchPlan plan;
  plan.comp_n.resize((size_t)nu);
  std::vector<int64_t> urp((size_t)nu + 1, 0);
  for (int32_t r = 0; r < max_n; r++) {
    for (int64_t u = layer_start[r]; u < layer_start[r + 1]; u++) {
      const int pos = (int)(u - layer_start[r]);
      const GraphIn& gi = G[order[pos]];
      comp[u] = pos;
      lid[u] = r;
      vk[u] = (uint8_t)gi.K;
      plan.comp_n[u] = gi.n;
      urp[u + 1] = gi.rp[r + 1] - gi.rp[r];
    }
  }
  for (int64_t u = 0; u < nu; u++) urp[u + 1] += urp[u];
  std::vector<int32_t> ucol((size_t)urp[nu]), uw((size_t)urp[nu]);
  for (int64_t u = 0; u < nu; u++) {
    const GraphIn& gi = G[order[comp[u]]];
    const int32_t r = lid[u];
    int64_t at = urp[u];
    for (int64_t e = gi.rp[r]; e < gi.rp[r + 1]; e++, at++) {
      ucol[at] = gid(comp[u], gi.col[e]);  // monotone in the neighbour's rank: rows stay sorted
      uw[at] = gi.w[e];
    }
  }
  int32_t Kmax = 1;
  for (int b = 0; b < B; b++) Kmax = std::max(Kmax, G[order[b]].K);
  // waves over rank layers: 1, 1, 2, 4, ... layers, at most 64 layers and
  // opts.max_wave hubs per wave (262,144 when 0)
  plan.bounds.push_back(0);
  {
    const int64_t hub_cap = opts.max_wave > 0 ? opts.max_wave : 262144;
    int32_t r = 0, width = 1;
    while (r < max_n) {
      int32_t r1 = std::min(max_n, r + width);
      while (r1 > r + 1 && layer_start[r1] - layer_start[r] > hub_cap) r1--;
      plan.bounds.push_back((int32_t)layer_start[r1]);
      r = r1;
      width = std::min(64, width * 2);
    }
  }
  hsdl_graph_impl ug;
  HSDL_TRY(upload_graph((int32_t)nu, urp.data(), ucol.data(), uw.data(), &ug));
  ug.h_rp = urp;
  hsdl_index* uidx = nullptr;
  int rc = new_index_handle(&uidx);
  DevBuf<int32_t> d_lid, d_comp;
  DevBuf<uint8_t> d_vk;
  auto cleanup = [&]() {
    d_lid.release();
    d_comp.release();
    d_vk.release();
    if (uidx) free_index_handle(uidx);
    ug.rp.release();
    ug.adj.release();
  };
  if (rc != HSDL_OK) {
    cleanup();
    return rc;
  }
  cudaStream_t st = uidx->stream;
  if ((rc = d_lid.alloc(nu, st)) != HSDL_OK || (rc = d_comp.alloc(nu, st)) != HSDL_OK ||
      (rc = d_vk.alloc(nu, st)) != HSDL_OK) {
    cleanup();
    return rc;
  }
  cudaMemcpyAsync(d_lid.p, lid.data(), sizeof(int32_t) * nu, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_comp.p, comp.data(), sizeof(int32_t) * nu, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_vk.p, vk.data(), nu, cudaMemcpyHostToDevice, st);
  plan.lid = d_lid.p;
  plan.vk = d_vk.p;
  hsdl_build_opts bo = opts;
  bo.clean = 0;
  rc = build_index(&ug, Kmax, bo, uidx, &plan);
  std::vector<int64_t> off_before;
  if (rc == HSDL_OK) {
    off_before = uidx->h_off;
    rc = clean_index(uidx);
  }
  if (rc != HSDL_OK) {
    cleanup();
    return rc;
  }
  // per-graph destinations of every union row
  const std::vector<int64_t>& uo = uidx->h_off;
  std::vector<int64_t> dst((size_t)nu);
  std::vector<std::vector<int64_t>> goff(B);
  std::vector<int64_t> gbefore(B, 0);
  for (int pos = 0; pos < B; pos++) {
    const int32_t gn = G[order[pos]].n;
    auto& o = goff[pos];
    o.assign((size_t)gn + 1, 0);
    for (int32_t r = 0; r < gn; r++) {
      const int32_t u = gid(pos, r);
      dst[u] = o[r];
      o[r + 1] = o[r] + (uo[u + 1] - uo[u]);
      gbefore[pos] += off_before[u + 1] - off_before[u];
    }
  }
  std::vector<hsdl_index*> outs(B, nullptr);
  std::vector<uint64_t*> pk(B);
  std::vector<int32_t*> pp(B);
  for (int pos = 0; pos < B && rc == HSDL_OK; pos++) {
    rc = new_index_handle(&outs[pos]);
    if (rc != HSDL_OK) break;
    hsdl_index* x = outs[pos];
    const int32_t gn = G[order[pos]].n;
    const int64_t tot = goff[pos][gn];
    if ((rc = x->off.alloc((int64_t)gn + 1, st)) != HSDL_OK || (rc = x->key.alloc(tot + kRowPad, st)) != HSDL_OK ||
        (rc = x->par.alloc(tot + kRowPad, st)) != HSDL_OK)
      break;
    cudaMemcpyAsync(x->off.p, goff[pos].data(), sizeof(int64_t) * (gn + 1), cudaMemcpyHostToDevice, st);
    pk[pos] = x->key.p;
    pp[pos] = x->par.p;
  }
  DevBuf<int64_t> d_dst;
  DevBuf<uint64_t*> d_pk;
  DevBuf<int32_t*> d_pp;
  if (rc == HSDL_OK && (rc = d_dst.alloc(nu, st)) == HSDL_OK && (rc = d_pk.alloc(B, st)) == HSDL_OK &&
      (rc = d_pp.alloc(B, st)) == HSDL_OK) {
    cudaMemcpyAsync(d_dst.p, dst.data(), sizeof(int64_t) * nu, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_pk.p, pk.data(), sizeof(uint64_t*) * B, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_pp.p, pp.data(), sizeof(int32_t*) * B, cudaMemcpyHostToDevice, st);
    const int sms = device_sm_count();
    k_split<<<sms * resident_blocks(k_split, 256), 256, 0, st>>>(nu, uidx->off.p, uidx->key.p, uidx->par.p,
                                                                 d_comp.p, d_lid.p, d_dst.p, d_pk.p, d_pp.p);
    launch_counter().fetch_add(1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_error(std::string("batched split: ") + cudaGetErrorString(e));
      rc = HSDL_ERR_CUDA;
    }
  }
  d_dst.release();
  d_pk.release();
  d_pp.release();
  if (rc == HSDL_OK) {
    for (int pos = 0; pos < B; pos++) {
      hsdl_index* x = outs[pos];
      const GraphIn& gi = G[order[pos]];
      // the buffers were allocated on the union's stream; they now belong to
      // the graph's own stream (the union stream has been synchronised)
      x->off.st = x->key.st = x->par.st = x->stream;
      x->n = gi.n;
      x->K = gi.K;
      x->cleaned = true;
      x->h_off = goff[pos];
      x->total = goff[pos][gi.n];
      x->before = gbefore[pos];
      x->after = x->total;
      x->waves = uidx->waves;
      x->t_gen = uidx->t_gen;
      x->t_sort = uidx->t_sort;
      x->t_clean = uidx->t_clean;
      // the sub-batch's build, shared by its graphs
      x->build_peak = uidx->build_peak;
      x->build_pool = uidx->build_pool;
      x->pool_key_bytes = uidx->pool_key_bytes;
      x->work_relax = uidx->work_relax;
      x->work_join_reads = uidx->work_join_reads;
      x->work_join_visible = uidx->work_join_visible;
      x->work_labels_written = uidx->work_labels_written;
      x->work_candidates = uidx->work_candidates;
      x->work_clean_reads = uidx->work_clean_reads;
      x->build_max_cand = uidx->build_max_cand;
      x->wave_splits = uidx->wave_splits;
      x->pool_chunks = uidx->pool_chunks;
      int64_t mr = 0;
      for (int32_t r = 0; r < gi.n; r++) mr = std::max(mr, goff[pos][r + 1] - goff[pos][r]);
      x->max_row = mr;
      out[order[pos]] = x;
    }
  } else {
    for (auto* x : outs)
      if (x) free_index_handle(x);
  }
  cleanup();
  return rc;
}

}  // namespace

}  // namespace hsdl

using namespace hsdl;

extern "C" int hsdl_build_batched(int32_t num_graphs, const int32_t* n, const int64_t* const* row_ptr,
                                  const int32_t* const* col, const int32_t* const* w, const int32_t* K,
                                  const hsdl_build_opts* opts, hsdl_index** out) {
  if (num_graphs < 1 || !n || !row_ptr || !col || !w || !K || !out) {
    set_error("hsdl_build_batched: bad arguments");
    return HSDL_ERR_INVALID;
  }
  hsdl_build_opts o;
  hsdl_build_opts_default(&o);
  if (opts) {
    if (opts->struct_size != (int32_t)sizeof(hsdl_build_opts)) {
      set_error("hsdl_build_opts.struct_size mismatch");
      return HSDL_ERR_INVALID;
    }
    o = *opts;
  }
  std::vector<GraphIn> G((size_t)num_graphs);
  std::vector<int64_t> est((size_t)num_graphs);
  for (int32_t i = 0; i < num_graphs; i++) {
    out[i] = nullptr;
    int rc = hsdl_validate_csr(n[i], row_ptr[i], col[i], w[i]);
    if (rc != HSDL_OK) {
      set_error("graph " + std::to_string(i) + ": " + hsdl_last_error());
      return rc;
    }
    if (K[i] < 1 || K[i] > kMaxK) {
      set_error("graph " + std::to_string(i) + ": K must be in [1, 14]");
      return HSDL_ERR_INVALID;
    }
    int32_t mw = 0;
    for (int64_t e = 0; e < row_ptr[i][n[i]]; e++) mw = std::max(mw, w[i][e]);
    if ((int64_t)K[i] * mw > (int64_t)kDistMask) {
      set_error("graph " + std::to_string(i) + ": K * max edge weight must be < 2^28");
      return HSDL_ERR_INVALID;
    }
    G[i] = GraphIn{n[i], row_ptr[i], col[i], w[i], K[i]};
    est[i] = batch_estimate_bytes(n[i], row_ptr[i][n[i]], K[i]);
  }
  // Sub-batches are formed as the build goes, in input order: each takes
  // graphs while their estimated bytes fit in the budget - the given one, or
  // 45 % of the HBM free at that moment (the indexes of earlier sub-batches
  // stay resident) - and under 2^27 vertices.  A sub-batch that runs out of
  // memory all the same is built again as two halves.
  auto fail = [&](int rc) {
    for (int32_t i = 0; i < num_graphs; i++)
      if (out[i]) {
        free_index_handle(out[i]);
        out[i] = nullptr;
      }
    return rc;
  };
  std::deque<std::vector<int32_t>> retry;
  int32_t next = 0;
  while (next < num_graphs || !retry.empty()) {
    std::vector<int32_t> b;
    if (!retry.empty()) {
      b = std::move(retry.front());
      retry.pop_front();
    } else {
      int64_t budget = o.device_budget_bytes;
      if (budget <= 0) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
          set_error("cudaMemGetInfo failed");
          return fail(HSDL_ERR_CUDA);
        }
        budget = (int64_t)(free_b * 0.45);
      }
      int64_t acc = 0, accn = 0;
      while (next < num_graphs &&
             (b.empty() || (acc + est[next] <= budget && accn + n[next] <= (int64_t)(kIdMask / 2)))) {
        acc += est[next];
        accn += n[next];
        b.push_back(next++);
      }
    }
    const int rc = build_sub_batch(G, b, o, out);
    if (rc == HSDL_ERR_NOMEM && b.size() > 1) {
      cudaGetLastError();  // the failed allocation is not sticky; clear it
      const size_t h = b.size() / 2;
      retry.emplace_front(b.begin() + (std::ptrdiff_t)h, b.end());
      retry.emplace_front(b.begin(), b.begin() + (std::ptrdiff_t)h);
      continue;
    }
    if (rc != HSDL_OK) return fail(rc);
  }
  return HSDL_OK;
}
