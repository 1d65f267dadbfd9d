// Label-propagation vertex grouping (groups of at most G_max vertices).
//
// Reference: generate_Group_CDLP
// (Hybrid_Generation_Clean/include/vgroup/CDLP_group.cuh:20-107) over CDLP_GPU
// (Hybrid_Generation_Clean/include/vgroup/CDLP/GPU_Community_Detection.cuh:
// 29-213): labels start as vertex ids; each iteration gathers the labels of
// every vertex's neighbours (LabelPropagation, :29-42), sorts them per vertex
// (cub::DeviceSegmentedSort, :142,173) and takes the most frequent label whose
// community is not full (Get_New_Label, :58-91); the host then buckets by
// label, greedily merges small groups up to G_max (CDLP_group.cuh:56-82) and
// orders the groups by total degree (:84-100).
//
// The reference's size cap is enforced with racy atomics, so its groups
// change from run to run.  This restatement is deterministic:
//   1. size[c] = vertices labelled c (exact histogram);
//   2. every vertex gathers its neighbours' labels, sorts them (warp bitonic
//      network, rows up to 32) or counts them in a hash table (a block per
//      longer row), and proposes the most frequent label c with c == own
//      label or size[c] < G_max, ties to the smaller label (no neighbours:
//      keep);
//   3. join[c] = vertices proposing c != own label; a label's joiners move
//      iff size[c] + join[c] <= G_max (all or none), so no group exceeds G_max;
//   4. stop when nothing moves or after max_iterations.
// The host merge and ordering then follow the reference's rules exactly.
#include <algorithm>
#include <chrono>
#include <vector>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int kLpThreads = 256;

__global__ void k_lp_init(int32_t n, int32_t* __restrict__ label) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    label[v] = (int32_t)v;
}

__global__ void k_lp_hist(int32_t n, const int32_t* __restrict__ label, int32_t* __restrict__ size) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&size[label[v]], 1);
}

// prop[e] = label[col[e]]  (LabelPropagation)
__global__ void k_lp_gather(int64_t m2, const int2* __restrict__ adj, const int32_t* __restrict__ label,
                            uint32_t* __restrict__ prop) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m2; e += (int64_t)gridDim.x * blockDim.x)
    prop[e] = (uint32_t)label[adj[e].x];
}

// Sorts every row of prop (rows of up to 32 entries; one warp per row).
__global__ void k_lp_sort_small(int32_t n, const int64_t* __restrict__ rp, uint32_t* __restrict__ prop) {
  const int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    int64_t lo = rp[v], len = rp[v + 1] - lo;
    if (len <= 1 || len > 32) continue;
    uint32_t k = lane < len ? prop[lo + lane] : 0xFFFFFFFFu;
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        uint32_t o = __shfl_xor_sync(0xffffffffu, k, stride);
        bool up = ((lane & size) == 0);
        bool lower = ((lane & stride) == 0);
        if (lower == up ? (o < k) : (o > k)) k = o;
      }
    }
    if (lane < len) prop[lo + lane] = k;
  }
}

__global__ void k_lp_list_rows(int32_t n, const int64_t* __restrict__ rp, int32_t* __restrict__ rows,
                               int32_t* __restrict__ count) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    if (rp[v + 1] - rp[v] > 32) rows[atomicAdd(count, 1)] = (int32_t)v;
}

// Mode of the sorted neighbour labels among eligible labels (Get_New_Label):
// one thread per vertex of degree <= 32 (longer rows: k_lp_mode_large).
__global__ void k_lp_choose(int32_t n, const int64_t* __restrict__ rp, const uint32_t* __restrict__ prop,
                            const int32_t* __restrict__ label, const int32_t* __restrict__ size, int32_t gmax,
                            int32_t* __restrict__ proposed, int32_t* __restrict__ join) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = rp[v], hi = rp[v + 1];
    if (hi - lo > 32) continue;
    const int32_t own = label[v];
    int32_t best = own;
    int64_t best_cnt = 0;
    int64_t i = lo;
    while (i < hi) {
      const uint32_t c = prop[i];
      int64_t j = i + 1;
      while (j < hi && prop[j] == c) j++;
      const int64_t cntc = j - i;
      const bool eligible = (int32_t)c == own || size[c] < gmax;
      // strictly more, or equal count and smaller label (runs come in
      // increasing label order, so a later equal count is never smaller)
      if (eligible && cntc > best_cnt) {
        best_cnt = cntc;
        best = (int32_t)c;
      }
      i = j;
    }
    proposed[v] = best;
    if (best != own) atomicAdd(&join[best], 1);
  }
}

// The same choice for the rows longer than 32 (listed in rows[0..*count)),
// one block per row, without sorting: the block counts the row's labels in a
// hash table (shared memory; a per-block table in global scratch for rows of
// more than kLpModeSlots / 2 entries) and takes the eligible label of largest
// count, the smaller label on ties - the run the serial scan of the sorted
// row keeps.  (Sorting the long rows with a block-wide bitonic network and
// scanning the runs with one warp per row took 93 + 25 ms of the 100 rounds
// at n = 1M, the network's barriers and the warps on the longest rows setting
// the time.)
constexpr int kLpModeSlots = 4096;  // shared-memory table: 32 KB of keys and counts

__global__ void __launch_bounds__(kLpThreads) k_lp_mode_large(
    const int32_t* __restrict__ rows, const int32_t* __restrict__ count, const int64_t* __restrict__ rp,
    const uint32_t* __restrict__ prop, const int32_t* __restrict__ label, const int32_t* __restrict__ size,
    int32_t gmax, int32_t* __restrict__ proposed, int32_t* __restrict__ join, uint32_t* __restrict__ gscratch,
    int64_t gslots) {
  __shared__ uint32_t s_key[kLpModeSlots];
  __shared__ uint32_t s_cnt[kLpModeSlots];
  __shared__ unsigned long long s_best[kLpThreads / 32];
  const int nrows = *count;
  const int lane = lane_id(), wid = threadIdx.x >> 5;
  for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
    const int v = rows[r];
    const int64_t lo = rp[v], len = rp[v + 1] - lo;
    int64_t cap = 64;
    while (cap < 2 * len) cap <<= 1;
    uint32_t* key = s_key;
    uint32_t* cnt = s_cnt;
    if (cap > kLpModeSlots) {
      key = gscratch + (int64_t)blockIdx.x * 2 * gslots;
      cnt = key + gslots;
    }
    const uint32_t mask = (uint32_t)cap - 1;
    for (int64_t i = threadIdx.x; i < cap; i += blockDim.x) {
      key[i] = 0xFFFFFFFFu;  // no label is all-ones (labels are vertex ids)
      cnt[i] = 0;
    }
    __syncthreads();
    for (int64_t e = threadIdx.x; e < len; e += blockDim.x) {
      const uint32_t c = prop[lo + e];
      uint32_t ix = table_hash(c, mask);
      for (uint32_t probe = 0; probe <= mask; probe++) {  // the table is at most half full
        const uint32_t old = atomicCAS(&key[ix], 0xFFFFFFFFu, c);
        if (old == 0xFFFFFFFFu || old == c) {
          atomicAdd(&cnt[ix], 1u);
          break;
        }
        ix = (ix + 1) & mask;
      }
    }
    __syncthreads();
    const int32_t own = label[v];
    unsigned long long best = 0;  // (count << 32) | (0xFFFFFFFF - label); 0 = none
    for (int64_t i = threadIdx.x; i < cap; i += blockDim.x) {
      const uint32_t c = key[i];
      if (c != 0xFFFFFFFFu && ((int32_t)c == own || size[c] < gmax)) {
        const unsigned long long k = ((unsigned long long)cnt[i] << 32) | (0xFFFFFFFFu - c);
        best = k > best ? k : best;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, best, o);
      best = x > best ? x : best;
    }
    if (lane == 0) s_best[wid] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < (int)(blockDim.x >> 5); w++) best = s_best[w] > best ? s_best[w] : best;
      const int32_t b = best ? (int32_t)(0xFFFFFFFFu - (uint32_t)(best & 0xFFFFFFFFull)) : own;
      proposed[v] = b;
      if (b != own) atomicAdd(&join[b], 1);
    }
    __syncthreads();  // the next row reuses the table
  }
}

__global__ void k_lp_apply(int32_t n, const int32_t* __restrict__ label, const int32_t* __restrict__ proposed,
                           const int32_t* __restrict__ size, const int32_t* __restrict__ join, int32_t gmax,
                           int32_t* __restrict__ out, unsigned long long* changed) {
  unsigned long long local = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t own = label[v], c = proposed[v];
    int32_t nl = own;
    if (c != own && size[c] + join[c] <= gmax) nl = c;
    out[v] = nl;
    local += nl != own;
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if (lane_id() == 0 && local) atomicAdd(changed, local);
}

}  // namespace

// Host side of generate_Group_CDLP (CDLP_group.cuh:39-100): bucket by label,
// merge small groups greedily, order by total degree.
// The reference's rules with flat arrays: labels bucketed by a counting sort
// (each bucket's vertices ascending), groups kept in per-size stacks with a
// bitmap of non-empty sizes, merged groups as chains of buckets.  A set of
// node-vector groups did the same in 0.35 s at n = 1M (most of the grouping's
// time); this takes milliseconds.
void assemble_groups(int32_t n, const int32_t* label, const int64_t* rp, int32_t gmax,
                     std::vector<std::vector<int32_t>>& groups) {
  // buckets of vertices by label, in label order
  std::vector<int64_t> start((size_t)n + 1, 0);
  for (int32_t v = 0; v < n; v++) start[(size_t)label[v] + 1]++;
  for (int32_t c = 0; c < n; c++) start[(size_t)c + 1] += start[c];
  std::vector<int32_t> members((size_t)n);
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int32_t v = 0; v < n; v++) members[(size_t)fill[label[v]]++] = v;
  }
  std::vector<int32_t> part_label;  // group g = the g-th non-empty bucket
  for (int32_t c = 0; c < n; c++)
    if (start[(size_t)c + 1] > start[c]) part_label.push_back(c);
  const int64_t G = (int64_t)part_label.size();
  std::vector<int64_t> size((size_t)G), tail((size_t)G), next((size_t)G, -1);
  // groups ordered by (size, id): per-size max-heaps of ids; sizes above gmax
  // (only unmerged buckets can be that large) share the last stack, ordered
  // by (size, id) themselves
  const int64_t S = (int64_t)gmax + 1;
  std::vector<std::vector<int64_t>> by_size((size_t)S + 1);
  std::vector<uint64_t> nonempty((size_t)(S + 64) / 64 + 1, 0);
  std::vector<std::pair<int64_t, int64_t>> big;  // (size, id) of groups larger than gmax, kept sorted
  auto push = [&](int64_t g) {
    if (size[g] > gmax) {
      big.insert(std::upper_bound(big.begin(), big.end(), std::make_pair(size[g], g)), std::make_pair(size[g], g));
      return;
    }
    auto& h = by_size[(size_t)size[g]];
    h.push_back(g);
    std::push_heap(h.begin(), h.end());
    nonempty[(size_t)size[g] / 64] |= 1ull << (size[g] % 64);
  };
  auto pop = [&](int64_t s) {
    auto& h = by_size[(size_t)s];
    std::pop_heap(h.begin(), h.end());
    const int64_t g = h.back();
    h.pop_back();
    if (h.empty()) nonempty[(size_t)s / 64] &= ~(1ull << (s % 64));
    return g;
  };
  // largest non-empty size <= lim (0 if none)
  auto highest = [&](int64_t lim) -> int64_t {
    if (lim <= 0) return 0;
    lim = std::min(lim, (int64_t)gmax);
    for (int64_t w = lim / 64; w >= 0; w--) {
      uint64_t bits = nonempty[(size_t)w];
      if (w == lim / 64) bits &= (lim % 64 == 63) ? ~0ull : ((1ull << (lim % 64 + 1)) - 1);
      if (bits) return w * 64 + (63 - __builtin_clzll(bits));
    }
    return 0;
  };
  for (int64_t g = 0; g < G; g++) {
    size[g] = start[(size_t)part_label[g] + 1] - start[part_label[g]];
    tail[g] = g;
    push(g);
  }
  std::vector<int64_t> after;  // finished groups (their head bucket), in order
  int64_t live = G;
  while (live > 0) {
    // the largest group (size, then id)
    int64_t g1;
    if (!big.empty()) {
      g1 = big.back().second;
      big.pop_back();
    } else {
      g1 = pop(highest(gmax));
    }
    live--;
    // the largest other group that still fits (CDLP_group.cuh:56-82)
    const int64_t s2 = highest(gmax - size[g1]);
    if (s2 > 0) {
      const int64_t g2 = pop(s2);
      next[tail[g1]] = g2;
      tail[g1] = tail[g2];
      size[g1] += size[g2];
      push(g1);
    } else {
      after.push_back(g1);
    }
  }
  // order by total degree, largest first (ties by position)
  std::vector<std::pair<int64_t, int64_t>> order;  // (-total degree, position)
  order.reserve(after.size());
  for (size_t i = 0; i < after.size(); i++) {
    int64_t tot = 0;
    for (int64_t p = after[i]; p >= 0; p = next[p])
      for (int64_t j = start[part_label[p]]; j < start[(size_t)part_label[p] + 1]; j++) {
        const int32_t v = members[(size_t)j];
        tot -= rp[v + 1] - rp[v];
      }
    order.push_back({tot, (int64_t)i});
  }
  std::sort(order.begin(), order.end());
  groups.clear();
  groups.reserve(order.size());
  for (auto& o : order) {
    std::vector<int32_t> nodes;
    for (int64_t p = after[(size_t)o.second]; p >= 0; p = next[p])
      nodes.insert(nodes.end(), members.begin() + start[part_label[p]],
                   members.begin() + start[(size_t)part_label[p] + 1]);
    groups.push_back(std::move(nodes));
  }
}

int group_lp(hsdl_graph_impl* g, int32_t gmax, int32_t max_iter, int32_t* group_of_vertex, int32_t* num_groups,
             int32_t* iterations_run) {
  const int32_t n = g->n;
  const int64_t m2 = g->m2;
  cudaStream_t st = nullptr;
  HSDL_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  } sg{st};
  const int sms = device_sm_count();
  DevBuf<int32_t> label, nlabel, size, join, proposed, rows, count;
  DevBuf<uint32_t> prop, gscratch;
  DevBuf<unsigned long long> changed;
  HSDL_TRY(label.alloc(n, st));
  HSDL_TRY(nlabel.alloc(n, st));
  HSDL_TRY(size.alloc(n, st));
  HSDL_TRY(join.alloc(n, st));
  HSDL_TRY(proposed.alloc(n, st));
  HSDL_TRY(rows.alloc(n, st));
  HSDL_TRY(count.alloc(1, st));
  HSDL_TRY(prop.alloc(std::max<int64_t>(1, m2), st));
  HSDL_TRY(changed.alloc(1, st));
  int64_t maxdeg = 0;
  for (int32_t v = 0; v < n; v++) maxdeg = std::max(maxdeg, g->h_rp[v + 1] - g->h_rp[v]);
  // rows past the shared-memory table count in a per-block global table
  int64_t gslots = 64;
  while (gslots < 2 * maxdeg) gslots <<= 1;
  const int mode_grid = sms * resident_blocks(k_lp_mode_large, kLpThreads);
  if (gslots > kLpModeSlots) HSDL_TRY(gscratch.alloc((int64_t)mode_grid * 2 * gslots, st));
  const int grid = sms * resident_blocks(k_lp_choose, kLpThreads);
  HSDL_CUDA(cudaMemsetAsync(count.p, 0, sizeof(int32_t), st));
  k_lp_list_rows<<<grid, kLpThreads, 0, st>>>(n, g->rp.p, rows.p, count.p);
  HSDL_LAUNCHED();
  k_lp_init<<<grid, kLpThreads, 0, st>>>(n, label.p);
  HSDL_LAUNCHED();
  int32_t it = 0;
  for (; it < max_iter; it++) {
    HSDL_CUDA(cudaMemsetAsync(size.p, 0, sizeof(int32_t) * n, st));
    HSDL_CUDA(cudaMemsetAsync(join.p, 0, sizeof(int32_t) * n, st));
    HSDL_CUDA(cudaMemsetAsync(changed.p, 0, sizeof(unsigned long long), st));
    k_lp_hist<<<grid, kLpThreads, 0, st>>>(n, label.p, size.p);
    HSDL_LAUNCHED();
    if (m2 > 0) {
      k_lp_gather<<<grid, kLpThreads, 0, st>>>(m2, g->adj.p, label.p, prop.p);
      HSDL_LAUNCHED();
      k_lp_sort_small<<<grid, kLpThreads, 0, st>>>(n, g->rp.p, prop.p);
      HSDL_LAUNCHED();
    }
    k_lp_choose<<<grid, kLpThreads, 0, st>>>(n, g->rp.p, prop.p, label.p, size.p, gmax, proposed.p, join.p);
    HSDL_LAUNCHED();
    if (m2 > 0) {
      k_lp_mode_large<<<mode_grid, kLpThreads, 0, st>>>(rows.p, count.p, g->rp.p, prop.p, label.p, size.p, gmax,
                                                        proposed.p, join.p, gscratch.p, gslots);
      HSDL_LAUNCHED();
    }
    k_lp_apply<<<grid, kLpThreads, 0, st>>>(n, label.p, proposed.p, size.p, join.p, gmax, nlabel.p, changed.p);
    HSDL_LAUNCHED();
    std::swap(label.p, nlabel.p);
    unsigned long long h_changed = 0;
    HSDL_CUDA(cudaMemcpyAsync(&h_changed, changed.p, sizeof(h_changed), cudaMemcpyDeviceToHost, st));
    HSDL_CUDA(cudaStreamSynchronize(st));
    if (h_changed == 0) {
      it++;
      break;
    }
  }
  std::vector<int32_t> h_label((size_t)n);
  HSDL_CUDA(cudaMemcpyAsync(h_label.data(), label.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  std::vector<std::vector<int32_t>> groups;
  assemble_groups(n, h_label.data(), g->h_rp.data(), gmax, groups);
  for (size_t gi = 0; gi < groups.size(); gi++)
    for (int32_t v : groups[gi]) group_of_vertex[v] = (int32_t)gi;
  *num_groups = (int32_t)groups.size();
  if (iterations_run) *iterations_run = it;
  label.release(); nlabel.release(); size.release(); join.release(); proposed.release(); rows.release();
  count.release(); prop.release(); gscratch.release(); changed.release();
  return HSDL_OK;
}

}  // namespace hsdl
