// HSDL label generation on one GPU.
//
// Reference algorithm: HSDL_thread_function
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:45-224)
// run for every hub in rank order (:586-595), and its hop-synchronous GPU form
// label_gen / gen_label_hsdl_v4 / query_parallel_v2 / Push_Back_L
// (Hybrid_Generation_Clean/src/label_gen.cu:603-837, 477-593, 87-110, 113-150).
//
// Design (one GPU, HBM-resident):
//  * Hubs run in waves of consecutive ranks.  Every hub of a wave owns a slot:
//    a dense row cand[slot][0..n) of packed candidate keys
//    (distance:32 | hop:4 | parent:28).  A wave runs K hop rounds:
//      expand: every frontier entry (slot, x, d_x) relaxes the neighbours of x
//              ranked below the hub; atomicMin on the candidate key keeps the
//              best (distance, hop, parent); the first improvement of a
//              (slot, v) in this hop appends it to the candidate list.
//              A candidate that does not beat the best distance of any earlier
//              hop never improves the key - that is the reference's own-label
//              dominance (generation.h:127-146).
//      prune:  one warp per candidate joins the committed labels of v with the
//              hub's hop-prefix-min table (a hash table per slot, built from
//              the hub's own labels) and keeps the candidate iff its distance
//              is below the 2-hop query (generation.h:146-161).  Kept
//              candidates become labels and the next frontier.
//  * A wave's labels are committed after its last hop, so hubs of one wave do
//    not see each other: the result is a superset of the canonical labels,
//    which the clean reduces exactly to the canonical set.  Waves start at one
//    hub and double, so the highest-ranked hubs - which produce most labels
//    and prune the most - are seen by nearly everyone.
//  * Committed labels live in a pool of per-vertex rows with slack capacity
//    (bump allocation, rows double when they overflow), so a commit only
//    touches the rows that receive labels.  The final index is compacted to
//    exact CSR and each row sorted by label key.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <functional>
#include <vector>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int kThreads = 256;

struct Counters {
  unsigned long long c_count;     // candidate-list entries this wave (all hops)
  unsigned long long wl_count;    // labels found this wave
  unsigned long long overflow;    // candidate list overflowed
  unsigned long long tab_total;   // hub-table slots this wave
  unsigned long long reloc_need;  // pool entries the commit's row moves need
  unsigned long long touched;     // rows receiving labels this wave
  unsigned long long relax;       // relaxations this wave (work counter)
  unsigned long long reads;       // committed labels read by the pruning join (work counter)
  unsigned long long hop_c[16];   // candidate-list start of each hop
  unsigned long long hop_f[16];   // frontier size of each hop
};

// Where slot rows live.  One graph: slot s owns cand[s*n .. s*n + n) and vertex
// ids are row indices.  A batch of graphs laid out as one disjoint union: slot
// s owns base[s] .. base[s] + (size of its hub's graph), a vertex's index in
// the row is its id inside its own graph (lid), and each vertex carries its
// graph's hop bound (vk).
struct SlotMap {
  int32_t n;
  const int64_t* base;
  const int32_t* lid;
  const uint8_t* vk;
  __device__ int64_t row(int slot) const { return base ? base[slot] : (int64_t)slot * n; }
  __device__ int32_t local(int v) const { return lid ? lid[v] : v; }
  __device__ int hop_bound(int hub, int K) const { return vk ? (int)vk[hub] : K; }
};

// ---------------------------------------------------------------------------
// wave set-up
// ---------------------------------------------------------------------------
__global__ void k_wave_init(int32_t W, int32_t s_hub, SlotMap map, uint64_t* __restrict__ cand, int2* __restrict__ C,
                            int4* __restrict__ F, Counters* ctr) {
  int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot < W) {
    int hub = s_hub + slot;
    cand[map.row(slot) + map.local(hub)] = ckey(0, 0, (uint32_t)hub);
    C[slot] = make_int2(slot, hub);
    F[slot] = make_int4(slot, hub, 0, 0);
  }
  if (slot == 0) {
    ctr->c_count = W;
    ctr->hop_c[0] = 0;
    ctr->hop_c[1] = W;
    ctr->hop_f[0] = W;
  }
}

// Hub-table sizes: a power of two >= 2x the hub's label count (0 if none).
__global__ void k_table_size(int32_t W, int32_t s_hub, const int32_t* __restrict__ row_len,
                             int32_t* __restrict__ tab_cap, int64_t* __restrict__ tab_off, Counters* ctr) {
  __shared__ int64_t sm[32];
  int64_t running = 0;
  for (int base = 0; base < W; base += blockDim.x) {
    int slot = base + threadIdx.x;
    int64_t cap = 0;
    if (slot < W) {
      int len = row_len[s_hub + slot];
      if (len > 0) {
        cap = 8;
        while (cap < 2 * (int64_t)len) cap <<= 1;
      }
      tab_cap[slot] = (int32_t)cap;
    }
    int64_t total;
    int64_t pre = block_exclusive_scan(cap, sm, &total);
    if (slot < W) tab_off[slot] = running + pre;
    running += total;
  }
  if (threadIdx.x == 0) ctr->tab_total = running;
}

// Inserts every label (w, hop, d) of the hub into its table: T[w][hop] = min d.
__global__ void k_table_fill(int32_t W, int32_t s_hub, const int64_t* __restrict__ row_off,
                             const int32_t* __restrict__ row_len, const uint64_t* __restrict__ keys,
                             const int64_t* __restrict__ tab_off, const int32_t* __restrict__ tab_cap,
                             int32_t* __restrict__ tab, int stride) {
  int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t slot = warp; slot < W; slot += nwarps) {
    int cap = tab_cap[slot];
    if (cap == 0) continue;
    int hub = s_hub + (int)slot;
    int32_t* T = tab + tab_off[slot] * stride;
    uint32_t mask = (uint32_t)cap - 1;
    int64_t lo = row_off[hub];
    int len = row_len[hub];
    for (int j = lane; j < len; j += 32) {
      uint64_t k = keys[lo + j];
      int32_t w = (int32_t)lkey_hub(k);
      uint32_t i = table_hash((uint32_t)w, mask);
      bool placed = false;
      for (int probe = 0; probe < cap; probe++) {  // tables are at most half full
        int32_t old = atomicCAS(&T[(int64_t)i * stride], kEmptyKey, w);
        if (old == kEmptyKey || old == w) {
          placed = true;
          break;
        }
        i = (i + 1) & mask;
      }
      if (placed) atomicMin(&T[(int64_t)i * stride + 1 + lkey_hop(k)], (int32_t)lkey_dist(k));
    }
  }
}

// T[w][j] <- min over hops <= j (the hop-prefix-min table).
__global__ void k_table_prefix(const Counters* ctr, int32_t* __restrict__ tab, int stride, int K) {
  int64_t total = (int64_t)ctr->tab_total;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int32_t* row = tab + e * stride;
    if (row[0] == kEmptyKey) continue;
    int32_t m = row[1];
    for (int j = 1; j <= K; j++) {
      m = min(m, row[1 + j]);
      row[1 + j] = m;
    }
  }
}

// ---------------------------------------------------------------------------
// hop round: expansion
// ---------------------------------------------------------------------------
// Each block takes tiles of kThreads frontier entries.  Only neighbours ranked
// below the hub are relaxed (rank prune, generation.h:107-110); rows are
// sorted by neighbour id, so they are the suffix after the hub's id, found by
// binary search.  The tile's relaxations are spread evenly over the block
// through an exclusive scan of the suffix lengths.
__global__ void __launch_bounds__(kThreads) k_expand(SlotMap map, int32_t h, int32_t K, int32_t s_hub,
                                                     const int64_t* __restrict__ rp, const int2* __restrict__ adj,
                                                     const int4* __restrict__ F, uint64_t* __restrict__ cand,
                                                     int2* __restrict__ C, int64_t capC, Counters* ctr) {
  __shared__ int64_t s_start[kThreads];
  __shared__ int64_t s_lo[kThreads];
  __shared__ int4 s_e[kThreads];
  __shared__ int64_t s_scan[32];
  const int64_t nf = (int64_t)ctr->hop_f[h - 1];
  for (int64_t tile = blockIdx.x; tile * kThreads < nf; tile += gridDim.x) {
    int64_t i = tile * kThreads + threadIdx.x;
    int64_t len = 0, lo = 0;
    int4 e = make_int4(0, 0, 0, 0);
    if (i < nf && h <= map.hop_bound(s_hub + F[i].x, K)) {
      e = F[i];
      int hub = s_hub + e.x;
      lo = rp[e.y];
      int64_t hi = rp[e.y + 1];
      int64_t a = lo, b = hi;
      while (a < b) {
        int64_t mid = (a + b) >> 1;
        if (adj[mid].x <= hub) a = mid + 1; else b = mid;
      }
      lo = a;
      len = hi - a;
    }
    int64_t total;
    int64_t pre = block_exclusive_scan(len, s_scan, &total);
    if (threadIdx.x == 0 && total) atomicAdd(&ctr->relax, (unsigned long long)total);
    s_start[threadIdx.x] = pre;
    s_lo[threadIdx.x] = lo;
    s_e[threadIdx.x] = e;
    __syncthreads();
    for (int64_t j = threadIdx.x; j < total; j += kThreads) {
      int a = 0, b = kThreads - 1;
      while (a < b) {
        int mid = (a + b + 1) >> 1;
        if (s_start[mid] <= j) a = mid; else b = mid - 1;
      }
      int4 oe = s_e[a];
      int2 nb = adj[s_lo[a] + (j - s_start[a])];
      uint64_t key = ckey((uint32_t)oe.z + (uint32_t)nb.y, (uint32_t)h, (uint32_t)oe.y);
      uint64_t* p = cand + map.row(oe.x) + map.local(nb.x);
      bool app = false;
      if (key < __ldcg((const unsigned long long*)p)) {
        uint64_t old = atomicMin((unsigned long long*)p, (unsigned long long)key);
        app = key < old && ckey_hop(old) != (uint32_t)h;
      }
      long long pos = warp_append(app, &ctr->c_count);
      if (app) {
        if (pos < capC) C[pos] = make_int2(oe.x, nb.x);
        else ctr->overflow = 1;
      }
    }
    __syncthreads();
  }
}

// Closes hop h's candidate range.  On overflow the range stops at the list's
// end; the wave is then rerun, so the truncated hop is never committed.
__global__ void k_mark(Counters* ctr, int h, int64_t capC) {
  unsigned long long c = ctr->c_count;
  ctr->hop_c[h + 1] = c < (unsigned long long)capC ? c : (unsigned long long)capC;
}

// ---------------------------------------------------------------------------
// hop round: pruning query (one warp per candidate)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_prune(SlotMap map, int32_t h, int32_t K, int32_t s_hub,
                                                    const int2* __restrict__ C, const uint64_t* __restrict__ cand,
                                                    const int64_t* __restrict__ row_off,
                                                    const int32_t* __restrict__ row_len,
                                                    const uint64_t* __restrict__ keys,
                                                    const int64_t* __restrict__ tab_off,
                                                    const int32_t* __restrict__ tab_cap,
                                                    const int32_t* __restrict__ tab, int stride,
                                                    int4* __restrict__ Fout, int32_t* __restrict__ wl_v,
                                                    uint64_t* __restrict__ wl_key, int32_t* __restrict__ wl_par,
                                                    Counters* ctr) {
  const int lane = lane_id();
  const int64_t c0 = (int64_t)ctr->hop_c[h], c1 = (int64_t)ctr->hop_c[h + 1];
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  unsigned long long scanned = 0;
  for (int64_t i = c0 + warp; i < c1; i += nwarps) {
    int2 e = C[i];
    int slot = e.x, v = e.y;
    uint64_t ck = cand[map.row(slot) + map.local(v)];
    long long d = (long long)ckey_dist(ck);
    long long q = LLONG_MAX;
    int cap = tab_cap[slot];
    if (cap > 0) {
      const int32_t* T = tab + tab_off[slot] * stride;
      uint32_t mask = (uint32_t)cap - 1;
      int64_t lo = row_off[v];
      int len = row_len[v];
      for (int j0 = 0; j0 < len; j0 += 32) {
        int j = j0 + lane;
        if (j < len) {
          uint64_t k = keys[lo + j];
          uint32_t h1 = lkey_hop(k);
          if ((int)h1 <= h) {
            int32_t w = (int32_t)lkey_hub(k);
            uint32_t ix = table_hash((uint32_t)w, mask);
            for (int probe = 0; probe < cap; probe++) {
              int32_t kk = T[(int64_t)ix * stride];
              if (kk == w) {
                int32_t t = T[(int64_t)ix * stride + 1 + (h - (int)h1)];
                if (t != kInf32) {
                  long long c = (long long)lkey_dist(k) + t;
                  q = c < q ? c : q;
                }
                break;
              }
              if (kk == kEmptyKey) break;
              ix = (ix + 1) & mask;
            }
          }
        }
        scanned += (unsigned long long)min(32, len - j0);
        if (__any_sync(0xffffffffu, q <= d)) break;  // already dominated
      }
      q = warp_min_ll(q);
    }
    if (d < q && lane == 0) {
      unsigned long long p = atomicAdd(&ctr->wl_count, 1ull);
      wl_v[p] = v;
      wl_key[p] = lkey((uint32_t)(s_hub + slot), (uint32_t)h, (uint32_t)d);
      wl_par[p] = (int32_t)ckey_parent(ck);
      if (h < map.hop_bound(s_hub + slot, K)) {
        unsigned long long f = atomicAdd(&ctr->hop_f[h], 1ull);
        Fout[f] = make_int4(slot, v, (int)d, 0);
      }
    }
  }
  if (lane == 0 && scanned) atomicAdd(&ctr->reads, scanned);
}

// ---------------------------------------------------------------------------
// commit
// ---------------------------------------------------------------------------
__global__ void k_count(const Counters* ctr, const int32_t* __restrict__ wl_v, int32_t* __restrict__ cnt,
                        int32_t* __restrict__ touched, Counters* wctr) {
  int64_t total = (int64_t)ctr->wl_count;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    int v = wl_v[p];
    bool first = atomicAdd(&cnt[v], 1) == 0;
    long long pos = warp_append(first, &wctr->touched);
    if (first) touched[pos] = v;
  }
}

__device__ inline int32_t grown_cap(int64_t need) {
  int64_t c = 8;
  while (c < 2 * need) c <<= 1;
  return (int32_t)c;
}

__global__ void k_reserve_need(const Counters* ctr, const int32_t* __restrict__ touched,
                               const int32_t* __restrict__ row_len, const int32_t* __restrict__ row_cap,
                               const int32_t* __restrict__ cnt, Counters* wctr) {
  int64_t total = (int64_t)ctr->touched;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int v = touched[i];
    int64_t need = (int64_t)row_len[v] + cnt[v];
    if (need > row_cap[v]) atomicAdd(&wctr->reloc_need, (unsigned long long)grown_cap(need));
  }
}

// One warp per touched row: move the row to a bigger region if it overflows.
__global__ void k_relocate(const Counters* ctr, const int32_t* __restrict__ touched, int64_t* __restrict__ row_off,
                           const int32_t* __restrict__ row_len, int32_t* __restrict__ row_cap,
                           const int32_t* __restrict__ cnt, uint64_t* __restrict__ keys, int32_t* __restrict__ par,
                           unsigned long long* pool_tail) {
  int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t total = (int64_t)ctr->touched;
  for (int64_t i = warp; i < total; i += nwarps) {
    int v = touched[i];
    int len = row_len[v];
    int64_t need = (int64_t)len + cnt[v];
    if (need <= row_cap[v]) continue;
    int32_t ncap = grown_cap(need);
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(pool_tail, (unsigned long long)ncap);
    base = __shfl_sync(0xffffffffu, base, 0);
    int64_t old = row_off[v];
    for (int j = lane; j < len; j += 32) {
      keys[base + j] = keys[old + j];
      par[base + j] = par[old + j];
    }
    if (lane == 0) {
      row_off[v] = (int64_t)base;
      row_cap[v] = ncap;
    }
  }
}

__global__ void k_scatter(const Counters* ctr, const int32_t* __restrict__ wl_v, const uint64_t* __restrict__ wl_key,
                          const int32_t* __restrict__ wl_par, const int64_t* __restrict__ row_off,
                          int32_t* __restrict__ row_len, uint64_t* __restrict__ keys, int32_t* __restrict__ par) {
  int64_t total = (int64_t)ctr->wl_count;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    int v = wl_v[p];
    int pos = atomicAdd(&row_len[v], 1);
    int64_t at = row_off[v] + pos;
    keys[at] = wl_key[p];
    par[at] = wl_par[p];
  }
}

__global__ void k_clear_cnt(const Counters* ctr, const int32_t* __restrict__ touched, int32_t* __restrict__ cnt) {
  int64_t total = (int64_t)ctr->touched;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    cnt[touched[i]] = 0;
}

__global__ void k_reset(const Counters* ctr, const int2* __restrict__ C, uint64_t* __restrict__ cand, SlotMap map,
                        int64_t capC) {
  int64_t total = (int64_t)ctr->c_count;
  if (total > capC) total = capC;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int2 e = C[i];
    cand[map.row(e.x) + map.local(e.y)] = kEmptyCand;
  }
}

// ---------------------------------------------------------------------------
// finalize: exact CSR + self labels
// ---------------------------------------------------------------------------
__global__ void k_final_len(int32_t n, const int32_t* __restrict__ row_len, int64_t* __restrict__ flen) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    flen[v] = (int64_t)row_len[v] + 1;
}

__global__ void k_final_copy(int32_t n, const int64_t* __restrict__ row_off, const int32_t* __restrict__ row_len,
                             const uint64_t* __restrict__ keys, const int32_t* __restrict__ par,
                             const int64_t* __restrict__ foff, uint32_t* __restrict__ fhub,
                             uint32_t* __restrict__ fhd, int32_t* __restrict__ fpar) {
  int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    int64_t src = row_off[v], dst = foff[v];
    int len = row_len[v];
    for (int j = lane; j < len; j += 32) {
      uint64_t k = keys[src + j];
      fhub[dst + j] = lkey_hub(k);
      fhd[dst + j] = lkey_hd(k);
      fpar[dst + j] = par[src + j];
    }
    if (lane == 0) {
      // self label (v, v, 0, 0), pushed by the reference when hub v starts
      // (generation.h:74-85)
      fhub[dst + len] = (uint32_t)v;
      fhd[dst + len] = hd_pack(0, 0);
      fpar[dst + len] = (int32_t)v;
    }
  }
}

__global__ void k_row_max(int32_t n, const int64_t* __restrict__ off, unsigned long long* out) {
  unsigned long long m = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long l = (unsigned long long)(off[v + 1] - off[v]);
    m = l > m ? l : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  if (lane_id() == 0) atomicMax(out, m);
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// Wave schedule: widths first, 2*first, 4*first, ... capped at max_wave.
std::vector<int32_t> wave_schedule(int32_t n, int32_t first, int32_t max_wave) {
  std::vector<int32_t> b{0};
  int64_t w = std::max(1, first);
  while (b.back() < n) {
    b.push_back((int32_t)std::min<int64_t>(n, (int64_t)b.back() + w));
    w = std::min<int64_t>(std::max(1, max_wave), w * 2);
  }
  return b;
}

int32_t auto_max_wave(int32_t n, int64_t budget_bytes) {
  // dense candidate rows: max_wave * n * 8 B within a quarter of the budget,
  // at most 2048 hubs per wave
  int64_t avail = budget_bytes > 0 ? budget_bytes / 4 : (int64_t)16 << 30;
  int64_t w = avail / ((int64_t)n * 8);
  w = std::max<int64_t>(1, std::min<int64_t>(2048, w));
  return (int32_t)w;
}

int row_max(int32_t n, const int64_t* d_off, int64_t* out, cudaStream_t st) {
  unsigned long long* d = nullptr;
  HSDL_CUDA(cudaMallocAsync(&d, sizeof(unsigned long long), st));
  HSDL_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), st));
  k_row_max<<<device_sm_count() * 4, 256, 0, st>>>(n, d_off, d);
  HSDL_LAUNCHED();
  unsigned long long h = 0;
  HSDL_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  HSDL_CUDA(cudaFreeAsync(d, st));
  *out = (int64_t)h;
  return HSDL_OK;
}

int build_index(hsdl_graph_impl* g, int32_t K, const hsdl_build_opts& opts, hsdl_index_impl* idx,
                const BatchPlan* plan) {
  const int32_t n = g->n;
  cudaStream_t st = idx->stream;
  const int sms = device_sm_count();
  const int stride = (K + 2 <= 8) ? 8 : 16;  // hub-table slot: key + K+1 distances, 32 or 64 B
  double t0 = now_s();

  size_t free_b = 0, total_b = 0;
  HSDL_CUDA(cudaMemGetInfo(&free_b, &total_b));
  int64_t budget = opts.device_budget_bytes > 0 ? opts.device_budget_bytes : (int64_t)free_b;
  std::vector<int32_t> bounds;
  if (plan) {
    bounds = plan->bounds;
  } else {
    int32_t max_wave = opts.max_wave > 0 ? opts.max_wave : auto_max_wave(n, budget);
    bounds = wave_schedule(n, opts.first_wave > 0 ? opts.first_wave : 1, max_wave);
  }
  int32_t Wmax = 0;
  int64_t cand_entries = 0;  // largest wave's candidate rows
  for (size_t i = 0; i + 1 < bounds.size(); i++) {
    Wmax = std::max(Wmax, bounds[i + 1] - bounds[i]);
    int64_t e = 0;
    if (plan) {
      for (int32_t v = bounds[i]; v < bounds[i + 1]; v++) e += plan->comp_n[v];
    } else {
      e = (int64_t)(bounds[i + 1] - bounds[i]) * n;
    }
    cand_entries = std::max(cand_entries, e);
  }
  std::vector<int64_t> h_base;
  DevBuf<int64_t> d_base;
  if (plan) {
    h_base.resize(Wmax);
    HSDL_TRY(d_base.alloc(Wmax, st));
  }
  SlotMap map{n, plan ? d_base.p : nullptr, plan ? plan->lid : nullptr, plan ? plan->vk : nullptr};

  // --- device state --------------------------------------------------------
  DevBuf<uint64_t> cand;
  DevBuf<int64_t> row_off;
  DevBuf<int32_t> row_len, row_cap, cnt, touched;
  DevBuf<uint64_t> pool_keys;
  DevBuf<int32_t> pool_par;
  DevBuf<int2> Cl;
  DevBuf<int4> Fa, Fb;
  DevBuf<int32_t> wl_v, wl_par;
  DevBuf<uint64_t> wl_key;
  DevBuf<int64_t> tab_off;
  DevBuf<int32_t> tab_cap, tab;
  DevBuf<Counters> ctr;
  DevBuf<unsigned long long> pool_tail;
  auto release_all = [&]() {
    cand.release(); row_off.release(); row_len.release(); row_cap.release(); cnt.release(); touched.release();
    pool_keys.release(); pool_par.release(); Cl.release(); Fa.release(); Fb.release(); wl_v.release();
    wl_par.release(); wl_key.release(); tab_off.release(); tab_cap.release(); tab.release(); ctr.release();
    pool_tail.release(); d_base.release();
  };
  struct Guard {
    std::function<void()> f;
    ~Guard() { f(); }
  } guard{release_all};

  HSDL_TRY(cand.alloc(cand_entries, st));
  HSDL_CUDA(cudaMemsetAsync(cand.p, 0xFF, (size_t)cand.bytes(), st));
  HSDL_TRY(row_off.alloc(n, st));
  HSDL_TRY(row_len.alloc(n, st));
  HSDL_TRY(row_cap.alloc(n, st));
  HSDL_TRY(cnt.alloc(n, st));
  HSDL_TRY(touched.alloc(n, st));
  HSDL_CUDA(cudaMemsetAsync(row_off.p, 0, (size_t)row_off.bytes(), st));
  HSDL_CUDA(cudaMemsetAsync(row_len.p, 0, (size_t)row_len.bytes(), st));
  HSDL_CUDA(cudaMemsetAsync(row_cap.p, 0, (size_t)row_cap.bytes(), st));
  HSDL_CUDA(cudaMemsetAsync(cnt.p, 0, (size_t)cnt.bytes(), st));
  int64_t pool_cap = std::max<int64_t>(1 << 20, (int64_t)n * 16);
  HSDL_TRY(pool_keys.alloc(pool_cap, st));
  HSDL_TRY(pool_par.alloc(pool_cap, st));
  int64_t capC = std::max<int64_t>(1 << 20, (int64_t)n * 4);
  auto alloc_lists = [&](int64_t c) -> int {
    HSDL_TRY(Cl.alloc(c, st));
    HSDL_TRY(Fa.alloc(c, st));
    HSDL_TRY(Fb.alloc(c, st));
    HSDL_TRY(wl_v.alloc(c, st));
    HSDL_TRY(wl_par.alloc(c, st));
    HSDL_TRY(wl_key.alloc(c, st));
    return HSDL_OK;
  };
  HSDL_TRY(alloc_lists(capC));
  HSDL_TRY(tab_off.alloc(Wmax, st));
  HSDL_TRY(tab_cap.alloc(Wmax, st));
  int64_t tab_cap_entries = 1 << 16;
  HSDL_TRY(tab.alloc(tab_cap_entries * stride, st));
  HSDL_TRY(ctr.alloc(1, st));
  HSDL_TRY(pool_tail.alloc(1, st));
  HSDL_CUDA(cudaMemsetAsync(pool_tail.p, 0, sizeof(unsigned long long), st));
  Counters hc;
  unsigned long long h_tail = 0;

  // grids of exactly one resident wave per kernel (grid-stride loops inside)
  const int grid = sms * resident_blocks(k_scatter, 256);
  const int g_expand = sms * resident_blocks(k_expand, kThreads);
  const int g_prune = sms * resident_blocks(k_prune, kThreads);
  for (size_t wv = 0; wv + 1 < bounds.size(); wv++) {
    const int32_t s_hub = bounds[wv], W = bounds[wv + 1] - bounds[wv];
    int64_t wave_entries = (int64_t)W * n;
    if (plan) {
      // each slot's row is as long as its hub's graph
      int64_t acc = 0;
      for (int32_t i = 0; i < W; i++) {
        h_base[i] = acc;
        acc += plan->comp_n[s_hub + i];
      }
      wave_entries = acc;
      HSDL_CUDA(cudaMemcpyAsync(d_base.p, h_base.data(), sizeof(int64_t) * W, cudaMemcpyHostToDevice, st));
    }
    for (int attempt = 0;; attempt++) {
      HSDL_CUDA(cudaMemsetAsync(ctr.p, 0, sizeof(Counters), st));
      k_wave_init<<<(W + 255) / 256, 256, 0, st>>>(W, s_hub, map, cand.p, Cl.p, Fa.p, ctr.p);
      HSDL_LAUNCHED();
      k_table_size<<<1, 1024, 0, st>>>(W, s_hub, row_len.p, tab_cap.p, tab_off.p, ctr.p);
      HSDL_LAUNCHED();
      HSDL_CUDA(cudaMemcpyAsync(&hc, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
      HSDL_CUDA(cudaStreamSynchronize(st));
      int64_t tab_need = (int64_t)hc.tab_total;
      if (tab_need > tab_cap_entries) {
        while (tab_cap_entries < tab_need) tab_cap_entries *= 2;
        HSDL_TRY(tab.alloc(tab_cap_entries * stride, st));
      }
      if (tab_need > 0) {
        HSDL_CUDA(cudaMemsetAsync(tab.p, 0x7F, (size_t)tab_need * stride * sizeof(int32_t), st));
        k_table_fill<<<std::min(grid, (W + 7) / 8), 256, 0, st>>>(W, s_hub, row_off.p, row_len.p, pool_keys.p,
                                                                   tab_off.p, tab_cap.p, tab.p, stride);
        HSDL_LAUNCHED();
        k_table_prefix<<<grid, 256, 0, st>>>(ctr.p, tab.p, stride, K);
        HSDL_LAUNCHED();
      }
      for (int32_t h = 1; h <= K; h++) {
        int4* Fin = (h & 1) ? Fa.p : Fb.p;
        int4* Fout = (h & 1) ? Fb.p : Fa.p;
        k_expand<<<g_expand, kThreads, 0, st>>>(map, h, K, s_hub, g->rp.p, g->adj.p, Fin, cand.p, Cl.p, capC, ctr.p);
        HSDL_LAUNCHED();
        k_mark<<<1, 1, 0, st>>>(ctr.p, h, capC);
        HSDL_LAUNCHED();
        k_prune<<<g_prune, kThreads, 0, st>>>(map, h, K, s_hub, Cl.p, cand.p, row_off.p, row_len.p, pool_keys.p,
                                              tab_off.p, tab_cap.p, tab.p, stride, Fout, wl_v.p, wl_key.p,
                                              wl_par.p, ctr.p);
        HSDL_LAUNCHED();
      }
      HSDL_CUDA(cudaMemcpyAsync(&hc, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
      HSDL_CUDA(cudaStreamSynchronize(st));
      if (!hc.overflow) break;
      // The candidate list overflowed: entries past its end were never
      // recorded, so clear this wave's slots wholesale and rerun the wave with
      // room for twice what was asked.
      HSDL_CUDA(cudaMemsetAsync(cand.p, 0xFF, (size_t)wave_entries * sizeof(uint64_t), st));
      capC = std::max<int64_t>(capC * 2, (int64_t)hc.c_count * 2);
      HSDL_TRY(alloc_lists(capC));
      if (attempt > 40) {
        set_error("candidate list could not be sized");
        return HSDL_ERR_NOMEM;
      }
    }
    idx->work_relax += (int64_t)hc.relax;
    idx->work_join_reads += (int64_t)hc.reads;
    idx->work_labels_written += (int64_t)hc.wl_count;
    // commit the wave's labels
    if (hc.wl_count > 0) {
      k_count<<<grid, 256, 0, st>>>(ctr.p, wl_v.p, cnt.p, touched.p, ctr.p);
      HSDL_LAUNCHED();
      k_reserve_need<<<grid, 256, 0, st>>>(ctr.p, touched.p, row_len.p, row_cap.p, cnt.p, ctr.p);
      HSDL_LAUNCHED();
      HSDL_CUDA(cudaMemcpyAsync(&hc, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
      HSDL_CUDA(cudaMemcpyAsync(&h_tail, pool_tail.p, sizeof(h_tail), cudaMemcpyDeviceToHost, st));
      HSDL_CUDA(cudaStreamSynchronize(st));
      int64_t need = (int64_t)h_tail + (int64_t)hc.reloc_need;
      if (need > pool_cap) {
        int64_t nc = pool_cap;
        while (nc < need) nc *= 2;
        HSDL_TRY(pool_keys.grow(nc, (int64_t)h_tail, st));
        HSDL_TRY(pool_par.grow(nc, (int64_t)h_tail, st));
        pool_cap = nc;
      }
      k_relocate<<<grid, 256, 0, st>>>(ctr.p, touched.p, row_off.p, row_len.p, row_cap.p, cnt.p, pool_keys.p,
                                       pool_par.p, pool_tail.p);
      HSDL_LAUNCHED();
      k_scatter<<<grid, 256, 0, st>>>(ctr.p, wl_v.p, wl_key.p, wl_par.p, row_off.p, row_len.p, pool_keys.p,
                                      pool_par.p);
      HSDL_LAUNCHED();
      k_clear_cnt<<<grid, 256, 0, st>>>(ctr.p, touched.p, cnt.p);
      HSDL_LAUNCHED();
    }
    k_reset<<<grid, 256, 0, st>>>(ctr.p, Cl.p, cand.p, map, capC);
    HSDL_LAUNCHED();
    idx->waves++;
  }
  HSDL_CUDA(cudaStreamSynchronize(st));
  double t1 = now_s();
  cand.release();

  // --- finalize: exact CSR with self labels, rows sorted by key ------------
  DevBuf<int64_t> flen;
  HSDL_TRY(flen.alloc((int64_t)n + 1, st));
  HSDL_TRY(idx->off.alloc((int64_t)n + 1, st));
  k_final_len<<<grid, 256, 0, st>>>(n, row_len.p, flen.p);
  HSDL_LAUNCHED();
  HSDL_TRY(exclusive_scan_i64(flen.p, idx->off.p, n, st));
  int64_t total = 0;
  HSDL_CUDA(cudaMemcpyAsync(&total, idx->off.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  HSDL_TRY(idx->hub.alloc(total + kRowPad, st));
  HSDL_TRY(idx->hd.alloc(total + kRowPad, st));
  HSDL_TRY(idx->par.alloc(total + kRowPad, st));
  k_final_copy<<<grid * 2, 256, 0, st>>>(n, row_off.p, row_len.p, pool_keys.p, pool_par.p, idx->off.p,
                                         idx->hub.p, idx->hd.p, idx->par.p);
  HSDL_LAUNCHED();
  flen.release();
  release_all();
  int64_t mr = 0;
  HSDL_TRY(row_max(n, idx->off.p, &mr, st));
  HSDL_TRY(sort_rows(n, idx->off.p, idx->hub.p, idx->hd.p, idx->par.p, mr, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  double t2 = now_s();
  idx->n = n;
  idx->K = K;
  idx->total = total;
  idx->before = total;
  idx->after = total;
  idx->max_row = mr;
  idx->cleaned = false;
  idx->t_gen = t1 - t0;
  idx->t_sort = t2 - t1;
  idx->h_off.resize((size_t)n + 1);
  HSDL_CUDA(cudaMemcpy(idx->h_off.data(), idx->off.p, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost));
  return HSDL_OK;
}

}  // namespace hsdl
