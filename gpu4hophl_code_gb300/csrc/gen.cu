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
//              ranked below the hub (all of them in the 2023WWW search,
//              generation.h:226-370); atomicMin on the candidate key keeps the
//              best (distance, hop, parent); the first improvement of a
//              (slot, v) in this hop appends it to the candidate list.
//              A candidate that does not beat the best distance of any earlier
//              hop never improves the key - that is the reference's own-label
//              dominance (generation.h:127-146).
//      prune:  a group of lanes per candidate joins the committed labels of v with the
//              hub's hop-prefix-min table (a hash table per slot, built from
//              the hub's own labels) and keeps the candidate iff its distance
//              is below the 2-hop query (generation.h:146-161).  Kept
//              candidates become labels and the next frontier.
//  * A wave's labels are committed after its last hop, so hubs of one wave do
//    not see each other: the result is a superset of the canonical labels,
//    which the clean reduces exactly to the canonical set.  Waves start at one
//    hub and double, so the highest-ranked hubs - which produce most labels
//    and prune the most - are seen by nearly everyone.
//  * Committed labels live in a pool of per-vertex rows made of doubling
//    segments (nothing is moved when a row grows), so a commit only touches
//    the rows that receive labels.  The final index is compacted to exact CSR
//    and each row sorted by label key.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <functional>
#include <vector>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int kThreads = 256;
// Committed label rows are lists of doubling segments: segment i of a row
// holds its labels [8 (2^i - 1), 8 (2^(i+1) - 1)).  A row that fills its
// segments gets the next one; nothing is ever moved or copied, and a row's
// capacity is below twice its length.  Segments are carved from pool chunks
// (separate device allocations added as the pool grows) and named by a
// 64-bit reference chunk:16 | entry:48.
constexpr int kSegs = 25;  // 8 (2^25 - 1) >= 2^28 labels per row
constexpr int kMaxChunks = 1024;
constexpr int64_t kEntryMask = ((int64_t)1 << 48) - 1;

__device__ inline int seg_of(int j) { return 31 - __clz((j >> 3) + 1); }
__device__ inline int seg_first(int i) { return 8 * ((1 << i) - 1); }
__device__ inline int segs_for(int64_t len) { return len <= 0 ? 0 : seg_of((int)(len - 1)) + 1; }

// The pool's label keys are 8-byte keys (Fmt64: hub:32 | hop:4 | distance:28)
// or, when the graph's ranges fit, 4-byte keys (Fmt32: hub:H | hop:P |
// distance:D with H = bits of n - 1, P = bits of K + 1, every distance below
// 2^D since it is at most K x the largest weight): a join's 16-byte load then
// brings four labels instead of two.  In either format the all-ones key has a
// hop field above K (never within a hop bound): it marks "no label".
template <class F>
struct Rows {
  using KT = typename F::key_t;
  const int64_t* seg;        // [n][kSegs] segment references
  void* const* ck;           // chunk -> label keys (KT)
  int32_t* const* cp;        // chunk -> parents
  F f;                       // key format
  // where label j of row v lives: chunk and entry
  __device__ inline int64_t ref(int v, int j) const {
    const int i = seg_of(j);
    return __ldg(seg + (int64_t)v * kSegs + i) + (j - seg_first(i));
  }
  __device__ inline KT* keys_of(int64_t r) const { return (KT*)ck[r >> 48] + (r & kEntryMask); }
  __device__ inline KT key(int v, int j) const {
    const int64_t r = ref(v, j);
    return __ldg((const KT*)ck[r >> 48] + (r & kEntryMask));
  }
};
// Per-slot membership filter of the hub's own label hubs (4,096 bits): most
// labels of a candidate vertex name hubs the wave's hub has no label for, and
// a clear bit settles those with one load instead of a table probe sequence.
constexpr int kSlotFilterBits = 12;  // 1,024 / 4,096 / 16,384 bits: 2.23 / 2.19 / 2.22 s of generation at n = 1M
constexpr int kSlotFilterWords = (1 << kSlotFilterBits) / 32;
// per candidate-list entry: C, both frontier buffers, and the found-label lists
constexpr int64_t kListEntryBytes = 2 * sizeof(int2) + 2 * sizeof(int4) + 2 * sizeof(int32_t) + sizeof(uint64_t);

// An instantiated CUDA graph of one wave's hop kernels, keyed by the buffers
// and sizes its launches name.
struct HopGraph {
  static constexpr int kKey = 12;
  cudaGraphExec_t exec = nullptr;
  uintptr_t key[kKey] = {};
  ~HopGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
  template <class F>
  int ensure(const uintptr_t* k, cudaStream_t st, F&& launches) {
    if (exec && std::memcmp(k, key, sizeof key) == 0) return HSDL_OK;
    if (exec) {
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
    HSDL_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int rc = launches();
    cudaGraph_t gr = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &gr);
    if (rc != HSDL_OK) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    HSDL_CUDA(e);
    const cudaError_t ei = cudaGraphInstantiate(&exec, gr, 0);
    cudaGraphDestroy(gr);
    HSDL_CUDA(ei);
    std::memcpy(key, k, sizeof key);
    return HSDL_OK;
  }
};

struct Counters {
  unsigned long long c_count;     // candidate-list entries this wave (all hops)
  unsigned long long wl_count;    // labels found this wave
  unsigned long long overflow;    // candidate list overflowed
  unsigned long long tab_total;   // hub-table slots this wave
  unsigned long long touched;     // rows receiving labels this wave
  unsigned long long relax;       // relaxations this wave (work counter)
  unsigned long long reads;       // committed labels read by the pruning join (work counter)
  unsigned long long visible;     // committed labels of the joined candidates' rows (work counter)
  unsigned long long hop_c[16];   // candidate-list start of each hop
  unsigned long long hop_f[16];   // frontier size of each hop
  unsigned long long seg_need;     // pool entries of the segments this commit adds
  unsigned long long seg_over;     // a row would need more than kSegs segments
  unsigned long long take_e[16];  // expansion tiles taken (dynamic work distribution)
  unsigned long long take_p[16];  // pruning candidates taken
  unsigned long long heavy_chunks[16];  // chunks of heavy expansion tiles in the chunk map
  unsigned long long take_h[16];        // heavy chunks taken
  unsigned long long take_t[16];        // slot tiles taken by the slot-tiled pruning join
  int s_hub;                      // first hub of the wave (read by the captured hop kernels)
  int pad32;
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
                            int4* __restrict__ F, Counters* ctr, int32_t* __restrict__ wave_end_of) {
  int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot < W) {
    int hub = s_hub + slot;
    wave_end_of[hub] = s_hub + W;
    cand[map.row(slot) + map.local(hub)] = ckey(0, 0, (uint32_t)hub);
    C[slot] = make_int2(slot, hub);
    F[slot] = make_int4(slot, hub, 0, 0);
  }
  if (slot == 0) {
    ctr->s_hub = s_hub;
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
// Also records, per slot, the end of the wave of the hub's highest hub id
// (tab_theta): labels of a vertex at or past it come from later waves, whose
// hubs the wave's hub has no label for, so the pruning join stops there.
template <class F>
__global__ void k_table_fill(int32_t W, int32_t s_hub, Rows<F> rows, const int32_t* __restrict__ row_len,
                             const int64_t* __restrict__ tab_off, const int32_t* __restrict__ tab_cap,
                             int32_t* __restrict__ tab, int stride, uint32_t* __restrict__ filt,
                             const int32_t* __restrict__ wave_end_of, int32_t* __restrict__ tab_theta) {
  int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t slot = warp; slot < W; slot += nwarps) {
    int cap = tab_cap[slot];
    if (cap == 0) continue;
    int hub = s_hub + (int)slot;
    int32_t* T = tab + tab_off[slot] * stride;
    uint32_t mask = (uint32_t)cap - 1;
    int len = row_len[hub];
    int32_t wmax = 0;
    for (int j = lane; j < len; j += 32) {
      const typename F::key_t k = rows.key(hub, j);
      int32_t w = (int32_t)rows.f.hub(k);
      wmax = max(wmax, w);
      const uint32_t fb = filter_bit<kSlotFilterBits>((uint32_t)w);
      atomicOr(&filt[slot * kSlotFilterWords + (fb >> 5)], 1u << (fb & 31));
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
      if (placed) atomicMin(&T[(int64_t)i * stride + 1 + rows.f.hop(k)], (int32_t)rows.f.dist(k));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    if (lane == 0) tab_theta[slot] = wave_end_of[wmax];
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
// Relaxations of one heavy tile per chunk of the expansion's second kernel,
// and the tile size (in relaxations) above which a tile is split that way.
constexpr int64_t kExpandChunk = 8192;
constexpr int64_t kExpandHeavy = 2 * kExpandChunk;
constexpr int64_t kExpandChunkCap = 1 << 20;  // chunk-map entries (8 MB); past it tiles run whole

template <int TPB>
struct ExpandTile {
  int64_t start[TPB];
  int64_t lo[TPB];
  int4 e[TPB];
  int64_t scan[32];
};

// Loads frontier tile `tile` into the block's shared arrays: per entry its
// relaxation count (with rank_prune the suffix of its row after the hub's id,
// found by binary search; otherwise the whole row) and the exclusive scan of
// the counts.  Returns the tile's relaxations (every thread).
template <int TPB>
__device__ inline int64_t expand_tile_setup(ExpandTile<TPB>& t, SlotMap map, int32_t h, int32_t K, int32_t rank_prune,
                                            int64_t tile, int64_t nf, int32_t s_hub, const int64_t* __restrict__ rp,
                                            const int2* __restrict__ adj, const int4* __restrict__ F) {
  const int64_t i = tile * TPB + threadIdx.x;
  int64_t len = 0, lo = 0;
  int4 e = make_int4(0, 0, 0, 0);
  if (i < nf && h <= map.hop_bound(s_hub + F[i].x, K)) {
    e = F[i];
    const int hub = s_hub + e.x;
    lo = rp[e.y];
    const int64_t hi = rp[e.y + 1];
    if (rank_prune) {
      int64_t a = lo, b = hi;
      while (a < b) {
        const int64_t mid = (a + b) >> 1;
        if (adj[mid].x <= hub) a = mid + 1; else b = mid;
      }
      lo = a;
    }
    len = hi - lo;
  }
  int64_t total;
  const int64_t pre = block_exclusive_scan(len, t.scan, &total);
  t.start[threadIdx.x] = pre;
  t.lo[threadIdx.x] = lo;
  t.e[threadIdx.x] = e;
  __syncthreads();
  return total;
}

// Relaxations [j0, j1) of the tile in shared memory, spread over the block:
// atomicMin on the candidate key keeps the best (distance, hop, parent), and
// the first improvement of a (slot, v) in this hop appends it to the
// candidate list.
template <int TPB>
__device__ inline void expand_relax(const ExpandTile<TPB>& t, SlotMap map, int32_t h, int64_t j0, int64_t j1,
                                    const int2* __restrict__ adj, uint64_t* __restrict__ cand,
                                    int2* __restrict__ C, int64_t capC, Counters* ctr, int2* wbuf, int& wn) {
  const int lane = lane_id();
  // warp-uniform trip count: lanes past j1 stage nothing
  for (int64_t jw = j0 + (int64_t)(threadIdx.x - lane); jw < j1; jw += TPB) {
    const int64_t j = jw + lane;
    bool app = false;
    int2 entry = make_int2(0, 0);
    if (j < j1) {
      int a = 0, b = TPB - 1;
      while (a < b) {
        const int mid = (a + b + 1) >> 1;
        if (t.start[mid] <= j) a = mid; else b = mid - 1;
      }
      const int4 oe = t.e[a];
      const int2 nb = adj[t.lo[a] + (j - t.start[a])];
      const uint64_t key = ckey((uint32_t)oe.z + (uint32_t)nb.y, (uint32_t)h, (uint32_t)oe.y);
      uint64_t* p = cand + map.row(oe.x) + map.local(nb.x);
      if (key < __ldcg((const unsigned long long*)p)) {
        const uint64_t old = atomicMin((unsigned long long*)p, (unsigned long long)key);
        app = key < old && ckey_hop(old) != (uint32_t)h;
      }
      entry = make_int2(oe.x, nb.x);
    }
    warp_stage(wbuf, wn, app, entry, &ctr->c_count, C, capC, &ctr->overflow);
  }
}

// Each block takes `tiles` tiles of TPB frontier entries at a time from a
// per-hop counter and relaxes them.  With rank_prune (the HSDL search) only
// neighbours ranked below the hub are relaxed (generation.h:107-110); without
// it (the 2023WWW search, generation.h:338-347) every neighbour is.  A tile
// with more than kExpandHeavy relaxations is not relaxed here: its chunks of
// kExpandChunk relaxations go to the chunk map for k_expand_heavy, which
// spreads them over all blocks, so that no single block carries a tile's
// whole work while the others idle (the first hop's frontier is the wave's
// hubs, 256 consecutive ranks of similar degree per tile: a wave of 4,375
// hubs is only 17 tiles; an ncu capture of one expansion at n = 200k had one
// SM active for 1.49 M cycles against 13 K on average).
template <int TPB>
__global__ void __launch_bounds__(TPB) k_expand(SlotMap map, int32_t h, int32_t K, int32_t rank_prune, int32_t tiles,
                                                const int64_t* __restrict__ rp, const int2* __restrict__ adj,
                                                const int4* __restrict__ F, uint64_t* __restrict__ cand,
                                                int2* __restrict__ C, int64_t capC, Counters* ctr,
                                                int2* __restrict__ chunk_map) {
  __shared__ ExpandTile<TPB> t;
  __shared__ int64_t s_tile, s_defer;
  __shared__ int2 s_stage[TPB / 32][64];  // per-warp staging of candidate-list appends
  int2* wbuf = s_stage[threadIdx.x >> 5];
  int wn = 0;
  const int32_t s_hub = ctr->s_hub;
  const int64_t nf = (int64_t)ctr->hop_f[h - 1];
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int64_t)atomicAdd(&ctr->take_e[h], (unsigned long long)tiles);
    __syncthreads();
    const int64_t first = s_tile;
    if (first * TPB >= nf) break;
    for (int64_t tile = first; tile < first + tiles && tile * TPB < nf; tile++) {
      const int64_t total = expand_tile_setup(t, map, h, K, rank_prune, tile, nf, s_hub, rp, adj, F);
      if (threadIdx.x == 0 && total) atomicAdd(&ctr->relax, (unsigned long long)total);
      if (total > kExpandHeavy) {
        const int64_t nch = (total + kExpandChunk - 1) / kExpandChunk;
        if (threadIdx.x == 0) {
          const int64_t c0 = (int64_t)atomicAdd(&ctr->heavy_chunks[h], (unsigned long long)nch);
          s_defer = c0 + nch <= kExpandChunkCap ? c0 : -1 - c0;
        }
        __syncthreads();
        const int64_t d = s_defer;
        if (d >= 0) {
          for (int64_t q = threadIdx.x; q < nch; q += TPB) chunk_map[d + q] = make_int2((int)tile, (int)q);
          __syncthreads();
          continue;
        }
        // the map is full: mark this tile's entries in it as done and relax it here
        for (int64_t c = -1 - d + threadIdx.x; c < kExpandChunkCap; c += TPB) chunk_map[c] = make_int2(-1, 0);
      }
      expand_relax(t, map, h, 0, total, adj, cand, C, capC, ctr, wbuf, wn);
      __syncthreads();
    }
  }
  warp_stage_flush(wbuf, wn, &ctr->c_count, C, capC, &ctr->overflow);
}

// The chunks of the heavy tiles k_expand deferred: each block takes a chunk,
// rebuilds its tile's scan and relaxes the chunk's kExpandChunk relaxations.
template <int TPB>
__global__ void __launch_bounds__(TPB) k_expand_heavy(SlotMap map, int32_t h, int32_t K, int32_t rank_prune,
                                                      const int64_t* __restrict__ rp, const int2* __restrict__ adj,
                                                      const int4* __restrict__ F, uint64_t* __restrict__ cand,
                                                      int2* __restrict__ C, int64_t capC, Counters* ctr,
                                                      const int2* __restrict__ chunk_map) {
  __shared__ ExpandTile<TPB> t;
  __shared__ int64_t s_chunk;
  __shared__ int2 s_stage[TPB / 32][64];
  int2* wbuf = s_stage[threadIdx.x >> 5];
  int wn = 0;
  const int32_t s_hub = ctr->s_hub;
  const int64_t nf = (int64_t)ctr->hop_f[h - 1];
  const int64_t nch = min((int64_t)ctr->heavy_chunks[h], kExpandChunkCap);
  for (;;) {
    if (threadIdx.x == 0) s_chunk = (int64_t)atomicAdd(&ctr->take_h[h], 1ull);
    __syncthreads();
    const int64_t c = s_chunk;
    __syncthreads();
    if (c >= nch) break;
    const int2 m = chunk_map[c];
    if (m.x < 0) continue;
    const int64_t total = expand_tile_setup(t, map, h, K, rank_prune, (int64_t)m.x, nf, s_hub, rp, adj, F);
    const int64_t j0 = (int64_t)m.y * kExpandChunk;
    expand_relax(t, map, h, j0, min(j0 + kExpandChunk, total), adj, cand, C, capC, ctr, wbuf, wn);
    __syncthreads();
  }
  warp_stage_flush(wbuf, wn, &ctr->c_count, C, capC, &ctr->overflow);
}

// Closes hop h's candidate range.  On overflow the range stops at the list's
// end; the wave is then rerun, so the truncated hop is never committed.
// ---------------------------------------------------------------------------
// hop round: candidates grouped by vertex range before the pruning join
// ---------------------------------------------------------------------------
// The expansion appends (slot, v) in frontier order, so consecutive pruning
// groups read the rows of unrelated vertices, and a vertex that is a candidate
// of many hubs of the wave has its row fetched from DRAM again for each.  One
// radix partition by v >> shift (at most kPartBuckets ranges of consecutive
// ids) puts every hub's candidates of a vertex range next to each other: the
// joins then read a range's rows while L2 holds them.  Order inside a range is
// arbitrary (the join's decisions do not depend on it).
constexpr int kPartBuckets = 2048;  // vertex ranges of the by-range order
constexpr int kPartMaxBuckets = 8192;  // buckets of either order (the by-slot order has one per slot)
constexpr int kPartTile = 8192;  // list entries a block partitions at a time

__device__ inline void part_bounds(const Counters* ctr, int h, int64_t& c0, int64_t& c1) {
  c0 = (int64_t)ctr->hop_c[h];
  c1 = (int64_t)ctr->hop_c[h + 1];
}

// Bucket of a candidate: its slot, or its vertex's id range.
template <bool BY_SLOT>
__device__ inline int part_bucket(int2 x, int shift) {
  return BY_SLOT ? x.x : (x.y >> shift);
}

// Bucket sizes of the hop's list (shared-memory histogram of nb buckets per
// tile, one global atomic per non-empty bucket and tile).
template <bool BY_SLOT>
__global__ void __launch_bounds__(kThreads) k_part_count(const Counters* ctr, int h, const int2* __restrict__ C,
                                                         unsigned int* __restrict__ bcnt, int shift, int nb) {
  extern __shared__ unsigned int hist[];
  int64_t c0, c1;
  part_bounds(ctr, h, c0, c1);
  const int64_t tiles = (c1 - c0 + kPartTile - 1) / kPartTile;
  for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    for (int b = threadIdx.x; b < nb; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    const int64_t a = c0 + tile * kPartTile, e = min(c1, a + kPartTile);
    for (int64_t i = a + threadIdx.x; i < e; i += blockDim.x) atomicAdd(&hist[part_bucket<BY_SLOT>(C[i], shift)], 1u);
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
      if (hist[b]) atomicAdd(&bcnt[b], hist[b]);
    __syncthreads();
  }
}

// Bucket starts (exclusive scan from the hop's list start) into bcur; clears
// the counts for the next hop.  With tile > 0 it also records each bucket's
// start in bstart and its first work tile of `tile` candidates in tstart
// (bstart[nb] = list end, tstart[nb] = tiles in all).  One block of 1,024
// threads, nb <= kPartMaxBuckets.
__global__ void k_part_scan(const Counters* ctr, int h, unsigned int* __restrict__ bcnt,
                            unsigned long long* __restrict__ bcur, int nb, int tile,
                            unsigned long long* __restrict__ bstart, unsigned long long* __restrict__ tstart) {
  __shared__ int64_t warp_tot[32];
  constexpr int kPer = kPartMaxBuckets / 1024;
  const int per = (nb + 1023) / 1024;
  int64_t c0, c1;
  part_bounds(ctr, h, c0, c1);
  unsigned int v[kPer];
  int64_t mine = 0, mtiles = 0;
#pragma unroll
  for (int j = 0; j < kPer; j++) {
    const int b = threadIdx.x * per + j;
    v[j] = (j < per && b < nb) ? bcnt[b] : 0u;
    mine += v[j];
    if (tile > 0) mtiles += (v[j] + tile - 1) / tile;
  }
  int64_t total, ttotal = 0;
  int64_t x = block_exclusive_scan(mine, warp_tot, &total) + c0;
  int64_t tx = tile > 0 ? block_exclusive_scan(mtiles, warp_tot, &ttotal) : 0;
#pragma unroll
  for (int j = 0; j < kPer; j++) {
    const int b = threadIdx.x * per + j;
    if (j < per && b < nb) {
      bcur[b] = (unsigned long long)x;
      if (tile > 0) {
        bstart[b] = (unsigned long long)x;
        tstart[b] = (unsigned long long)tx;
        tx += (v[j] + tile - 1) / tile;
      }
      x += v[j];
      bcnt[b] = 0;
    }
  }
  if (tile > 0 && threadIdx.x == 0) {
    bstart[nb] = (unsigned long long)c1;
    tstart[nb] = (unsigned long long)ttotal;
  }
}

// Scatters the hop's list into Cs by bucket, at the same list positions.
template <bool BY_SLOT>
__global__ void __launch_bounds__(kThreads) k_part_scatter(const Counters* ctr, int h, const int2* __restrict__ C,
                                                           int2* __restrict__ Cs,
                                                           unsigned long long* __restrict__ bcur, int shift, int nb) {
  extern __shared__ unsigned long long base[];  // nb bucket bases, then nb counters
  unsigned int* hist = (unsigned int*)(base + nb);
  int64_t c0, c1;
  part_bounds(ctr, h, c0, c1);
  const int64_t tiles = (c1 - c0 + kPartTile - 1) / kPartTile;
  for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    for (int b = threadIdx.x; b < nb; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    const int64_t a = c0 + tile * kPartTile, e = min(c1, a + kPartTile);
    for (int64_t i = a + threadIdx.x; i < e; i += blockDim.x) atomicAdd(&hist[part_bucket<BY_SLOT>(C[i], shift)], 1u);
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      if (hist[b]) base[b] = atomicAdd(&bcur[b], (unsigned long long)hist[b]);
      hist[b] = 0;
    }
    __syncthreads();
    for (int64_t i = a + threadIdx.x; i < e; i += blockDim.x) {
      const int2 x = C[i];
      const int b = part_bucket<BY_SLOT>(x, shift);
      Cs[base[b] + atomicAdd(&hist[b], 1u)] = x;
    }
    __syncthreads();
  }
}

__global__ void k_mark(Counters* ctr, int h, int64_t capC) {
  unsigned long long c = ctr->c_count;
  ctr->hop_c[h + 1] = c < (unsigned long long)capC ? c : (unsigned long long)capC;
}

// Moves a warp's staged kept candidates (slot, v, d, parent) to the wave's
// found-label lists, and those below their hub's hop bound to the next
// frontier: one atomic per list per 32 entries.  Every lane calls it.
__device__ inline void prune_flush(int4* kbuf, int& kn, SlotMap map, int32_t h, int32_t K, int32_t s_hub,
                                   int4* __restrict__ Fout, int32_t* __restrict__ wl_v,
                                   uint64_t* __restrict__ wl_key, int32_t* __restrict__ wl_par, Counters* ctr) {
  __syncwarp();
  const int lane = lane_id();
  unsigned long long base = 0;
  if (lane == 0 && kn > 0) base = atomicAdd(&ctr->wl_count, (unsigned long long)kn);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int jb = 0; jb < kn; jb += 32) {
    const int j = jb + lane;
    const bool valid = j < kn;
    const int4 x = valid ? kbuf[j] : make_int4(0, 0, 0, 0);
    if (valid) {
      const unsigned long long p = base + (unsigned long long)j;
      wl_v[p] = x.y;
      wl_key[p] = lkey((uint32_t)(s_hub + x.x), (uint32_t)h, (uint32_t)x.z);
      wl_par[p] = x.w;
    }
    const bool fr = valid && h < map.hop_bound(s_hub + x.x, K);
    const unsigned fm = __ballot_sync(0xffffffffu, fr);
    unsigned long long fb = 0;
    if (lane == 0 && fm) fb = atomicAdd(&ctr->hop_f[h], (unsigned long long)__popc(fm));
    fb = __shfl_sync(0xffffffffu, fb, 0);
    if (fr) Fout[fb + __popc(fm & ((1u << lane) - 1u))] = make_int4(x.x, x.y, x.z, 0);
  }
  __syncwarp();
  kn = 0;
}

// ---------------------------------------------------------------------------
// hop round: pruning query (a group of G lanes per candidate)
// ---------------------------------------------------------------------------
// A candidate (slot, v) at distance d is kept iff no committed label (w, h1, d1)
// of v with h1 <= h meets the wave hub's table entry T[w][h - h1] (the least
// distance from the hub to w within h - h1 hops) at d1 + T <= d: the
// reference's pruning query (generation.h:146-161).  The G lanes of a group
// read G labels of v at a time and stop as soon as one dominates.  Groups take
// kPruneTake candidates at a time from a per-hop counter, so candidates with
// long label lists do not hold back a statically assigned share.
// Candidates a lane group takes at a time from the hop's counter: 2 / 4 / 8 /
// 32 gave generation 1.95 / 1.92 / 1.93 / 2.05 s at n = 1M (larger takes
// leave a longer tail, smaller ones contend on the counter).
constexpr int kPruneTake = 4;
// The pruning query of one candidate e = (slot, v) by a group of G lanes (gl =
// lane in the group, gmask = the group's lanes): the slot's hub table T (cap
// slots of `stride` ints: hub id, then hop-prefix-min distances), its
// membership filter Fl and stop threshold theta may live in global or shared
// memory: with FLT_ANY the filter is read with plain (generic) loads, which
// may name either space; without it, through the read-only global path
// (ld.global.nc), which must not be given a shared-memory address.  Returns
// true on lane 0 of the group when the candidate is kept; `kept` receives
// (slot, v, d, parent).
template <bool FLT_ANY>
__device__ inline uint32_t filter_word(const uint32_t* Fl, uint32_t i) {
  if constexpr (FLT_ANY) return Fl[i];
  else return __ldg(Fl + i);
}

template <int G, int P, bool SELF, class F, bool FLT_ANY = false>
__device__ inline bool prune_candidate(int2 e, int32_t h, int32_t s_hub, SlotMap map,
                                       const uint64_t* __restrict__ cand, const Rows<F>& rows,
                                       const int32_t* __restrict__ row_len, const int32_t* T, int cap, int stride,
                                       const uint32_t* Fl, uint32_t theta, int gl, unsigned gmask,
                                       unsigned long long& scanned, unsigned long long& visible, int4& kept) {
  const int slot = e.x, v = e.y;
  const uint64_t ck = cand[map.row(slot) + map.local(v)];
  const long long d = (long long)ckey_dist(ck);
  long long q = LLONG_MAX;
  if (cap > 0) {
        const uint32_t mask = (uint32_t)cap - 1;
        int len = row_len[v];
        visible += (unsigned long long)len;
        // lane gl of the group holds the address of the row's segment gl, so
        // a label's address takes a shuffle instead of two dependent loads
        using KT = typename F::key_t;
        // labels per lane per load: 2 (one 16-byte load of 8-byte keys, one
        // 8-byte load of 4-byte keys).  Four 4-byte keys per 16-byte load
        // doubled the step (more labels read past the dominating one) and
        // took 48 registers against 32: generation 2.28 s against 1.78 s.
        constexpr int V = 2;
        constexpr KT kNone = (KT)~(KT)0;          // hop field above K: never within the bound
        const KT* my_seg = nullptr;
        if (gl < segs_for(len)) {
          const int64_t r = __ldg(rows.seg + (int64_t)v * kSegs + gl);
          my_seg = (const KT*)rows.ck[r >> 48] + (r & kEntryMask);
        }
        // Each lane takes V adjacent labels (one load; segment sizes and
        // starts are multiples of 8, so a load never straddles one) and loads
        // the next ones before it probes the current ones.
        auto load_vec = [&](int jp, KT (&k)[V]) {
          const int si = seg_of(min(jp, len - 1));
          const KT* sp = (const KT*)__shfl_sync(gmask, (unsigned long long)my_seg, si < G ? si : 0, G);
#pragma unroll
          for (int x = 0; x < V; x++) k[x] = kNone;
          if (jp < len) {
            if (si < G) {
              if constexpr (sizeof(KT) == 8) {
                const uint4 q4 = __ldg((const uint4*)(sp + (jp - seg_first(si))));
                k[0] = (KT)(((uint64_t)q4.y << 32) | q4.x);
                k[1] = (KT)(((uint64_t)q4.w << 32) | q4.z);
              } else {
                const uint2 q2 = __ldg((const uint2*)(sp + (jp - seg_first(si))));
                k[0] = (KT)q2.x;
                k[1] = (KT)q2.y;
              }
            } else {
#pragma unroll
              for (int x = 0; x < V; x++)
                if (jp + x < len) k[x] = rows.key(v, jp + x);
            }
#pragma unroll
            for (int x = 1; x < V; x++)
              if (jp + x >= len) k[x] = kNone;
          }
        };
        // the table probe of a label whose hub passed the slot's filter
        auto probe = [&](uint32_t w, int h1, long long d1) {
          uint32_t ix = table_hash(w, mask);
          for (int pr = 0; pr < cap; pr++) {
            const int32_t kk = T[(int64_t)ix * stride];
            if (kk == (int32_t)w) {
              const int32_t t = T[(int64_t)ix * stride + 1 + (h - h1)];
              if (t != kInf32) {
                const long long c = d1 + t;
                q = c < q ? c : q;
              }
              return;
            }
            if (kk == kEmptyKey) return;
            ix = (ix + 1) & mask;
          }
        };
        // A candidate from an earlier wave (only the 2023WWW search, which
        // has no rank prune, reaches one) also has its self label (v, 0, 0):
        // the reference pushes it when v's own search starts, and here it is
        // added to the rows only when the index is finalised.
        if (SELF && v < s_hub && gl == 0) {
          const uint32_t fb = filter_bit<kSlotFilterBits>((uint32_t)v);
          if ((filter_word<FLT_ANY>(Fl, fb >> 5) >> (fb & 31)) & 1u) probe((uint32_t)v, 0, 0);
        }
        // a step covers V P G labels: lane gl takes the vectors at V gl + V G p
        KT a[P][V];
#pragma unroll
        for (int p = 0; p < P; p++) load_vec(V * gl + V * G * p, a[p]);
        for (int j0 = 0; j0 < len; j0 += V * G * P) {
          KT b[P][V];
#pragma unroll
          for (int p = 0; p < P; p++) load_vec(j0 + V * G * P + V * gl + V * G * p, b[p]);
          // the filter bit of each label's hub (0 for labels past the hop bound)
          uint32_t f[P][V];
#pragma unroll
          for (int p = 0; p < P; p++)
#pragma unroll
            for (int x = 0; x < V; x++) {
              const uint32_t fb = filter_bit<kSlotFilterBits>(rows.f.hub(a[p][x]));
              f[p][x] = (int)rows.f.hop(a[p][x]) <= h ? (filter_word<FLT_ANY>(Fl, fb >> 5) >> (fb & 31)) & 1u : 0u;
            }
          bool past = false;  // a label from a wave after the hub's last hub: the rest of the row is too
#pragma unroll
          for (int p = 0; p < P; p++)
#pragma unroll
            for (int x = 0; x < V; x++) {
              if (f[p][x]) probe(rows.f.hub(a[p][x]), (int)rows.f.hop(a[p][x]), (long long)rows.f.dist(a[p][x]));
              past |= a[p][x] != kNone && rows.f.hub(a[p][x]) >= theta;
            }
          scanned += (unsigned long long)min(V * G * P, len - j0);
          if (__any_sync(gmask, q <= d || past)) break;  // dominated, or nothing further can match
#pragma unroll
          for (int p = 0; p < P; p++)
#pragma unroll
            for (int x = 0; x < V; x++) a[p][x] = b[p][x];
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
          long long x = __shfl_xor_sync(gmask, q, o);
          q = x < q ? x : q;
        }
      }
  kept = make_int4(slot, v, (int)d, (int32_t)ckey_parent(ck));
  return d < q && gl == 0;
}

template <int G, int P, bool SELF, class F>
__global__ void __launch_bounds__(kThreads) k_prune(SlotMap map, int32_t h, int32_t K,
                                                    const int2* __restrict__ C, const uint64_t* __restrict__ cand,
                                                    Rows<F> rows, const int32_t* __restrict__ row_len,
                                                    const int64_t* __restrict__ tab_off,
                                                    const int32_t* __restrict__ tab_cap,
                                                    const int32_t* __restrict__ tab, int stride,
                                                    const uint32_t* __restrict__ filt,
                                                    const int32_t* __restrict__ tab_theta,
                                                    int4* __restrict__ Fout, int32_t* __restrict__ wl_v,
                                                    uint64_t* __restrict__ wl_key, int32_t* __restrict__ wl_par,
                                                    Counters* ctr) {
  constexpr int NG = 32 / G;
  const int lane = lane_id();
  const int gi = lane / G, gl = lane % G;
  const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (gi * G));
  const int32_t s_hub = ctr->s_hub;
  const int64_t c0 = (int64_t)ctr->hop_c[h], c1 = (int64_t)ctr->hop_c[h + 1];
  unsigned long long scanned = 0, visible = 0;
  __shared__ int4 s_kept[kThreads / 32][64];  // per-warp staging of kept candidates: slot, v, d, parent
  int4* kbuf = s_kept[threadIdx.x >> 5];
  int kn = 0;
  for (;;) {
    unsigned long long took = 0;
    if (lane == 0) took = atomicAdd(&ctr->take_p[h], (unsigned long long)(kPruneTake * NG));
    took = __shfl_sync(0xffffffffu, took, 0);
    const int64_t i0 = c0 + (int64_t)took;
    if (i0 >= c1) break;
    const int64_t i1 = min(c1, i0 + kPruneTake * NG);
    // (Loading the set-up of a group's 8 candidates up front, one lane each,
    // doubled the registers of the 32-lane kernel and halved its occupancy:
    // generation went from 2.28 s to 2.83 s at n = 1M.)
    // warp-uniform trip count: a group past i1 decides nothing but stages with the warp
    for (int64_t ib = i0; ib < i1; ib += NG) {
      const int64_t i = ib + gi;
      bool keep = false;
      int4 kept = make_int4(0, 0, 0, 0);
      if (i < i1) {
      const int2 e = C[i];
      const int cap = tab_cap[e.x];
      keep = prune_candidate<G, P, SELF, F>(e, h, s_hub, map, cand, rows, row_len, tab + tab_off[e.x] * stride, cap,
                                            stride, filt + (int64_t)e.x * kSlotFilterWords,
                                            (uint32_t)tab_theta[e.x], gl, gmask, scanned, visible, kept);
      }
      // kept candidates become labels (and the next frontier) through the
      // warp's staging buffer: one atomic per 32 or more labels
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) kbuf[kn + __popc(m & ((1u << lane) - 1u))] = kept;
      kn += __popc(m);
      if (kn >= 32) prune_flush(kbuf, kn, map, h, K, s_hub, Fout, wl_v, wl_key, wl_par, ctr);
    }
  }
  prune_flush(kbuf, kn, map, h, K, s_hub, Fout, wl_v, wl_key, wl_par, ctr);
  if (gl == 0 && scanned) atomicAdd(&ctr->reads, scanned);
  if (gl == 0 && visible) atomicAdd(&ctr->visible, visible);
}

// The pruning join with the hub's table in shared memory.  The hop's list is
// grouped by slot and cut into tiles of up to kSlotTile candidates of one
// slot; a block of kSlotThreads takes a tile, copies the slot's hub table and
// membership filter into shared memory (when the table fits kSlotTableBytes),
// and its warps join the tile's candidates, so a label's filter test and
// table probe are shared-memory reads and only the label itself comes from
// global memory.
constexpr int kSlotThreads = 1024;
constexpr int kSlotTile = 2048;
constexpr int kSlotTableBytes = 64 * 1024;
constexpr size_t kSlotSmem = kSlotTableBytes + sizeof(uint32_t) * kSlotFilterWords +
                             sizeof(int4) * (kSlotThreads / 32) * 64;

template <class F>
__global__ void __launch_bounds__(kSlotThreads, 2)
    k_prune_slot(SlotMap map, int32_t h, int32_t K, const int2* __restrict__ C, const uint64_t* __restrict__ cand,
                 Rows<F> rows, const int32_t* __restrict__ row_len, const int64_t* __restrict__ tab_off,
                 const int32_t* __restrict__ tab_cap, const int32_t* __restrict__ tab, int stride,
                 const uint32_t* __restrict__ filt, const int32_t* __restrict__ tab_theta,
                 const unsigned long long* __restrict__ bstart, const unsigned long long* __restrict__ tstart, int nb,
                 int4* __restrict__ Fout, int32_t* __restrict__ wl_v, uint64_t* __restrict__ wl_key,
                 int32_t* __restrict__ wl_par, Counters* ctr) {
  extern __shared__ __align__(16) unsigned char smem[];
  int32_t* s_tab = (int32_t*)smem;
  uint32_t* s_filt = (uint32_t*)(smem + kSlotTableBytes);
  int4* kbuf = (int4*)(smem + kSlotTableBytes + sizeof(uint32_t) * kSlotFilterWords) + (threadIdx.x >> 5) * 64;
  __shared__ int64_t s_lo, s_hi;
  __shared__ int s_slot, s_staged;
  __shared__ unsigned long long s_take;
  const int lane = lane_id();
  const int32_t s_hub = ctr->s_hub;
  const unsigned long long tiles = tstart[nb];
  unsigned long long scanned = 0, visible = 0;
  int kn = 0;
  if (threadIdx.x == 0) s_staged = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long t = atomicAdd(&ctr->take_t[h], 1ull);
      int slot = -1;
      if (t < tiles) {
        int lo = 0, hi = nb;  // the last slot whose first tile is <= t
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (tstart[mid] <= t) lo = mid; else hi = mid;
        }
        slot = lo;
        const int64_t b0 = (int64_t)bstart[slot], b1 = (int64_t)bstart[slot + 1];
        s_lo = b0 + (int64_t)(t - tstart[slot]) * kSlotTile;
        s_hi = min(b1, s_lo + kSlotTile);
      }
      s_slot = slot;
      s_take = 0;
    }
    __syncthreads();
    const int slot = s_slot;
    if (slot < 0) break;
    const int cap = tab_cap[slot];
    const bool in_smem = cap > 0 && (int64_t)cap * stride * (int64_t)sizeof(int32_t) <= kSlotTableBytes;
    if (in_smem && s_staged != slot) {
      const int4* src = (const int4*)(tab + tab_off[slot] * stride);
      int4* dst = (int4*)s_tab;
      const int n16 = cap * stride / 4;  // stride is 8 or 16 ints
      for (int j = threadIdx.x; j < n16; j += blockDim.x) dst[j] = __ldg(src + j);
      const uint32_t* fsrc = filt + (int64_t)slot * kSlotFilterWords;
      for (int j = threadIdx.x; j < kSlotFilterWords; j += blockDim.x) s_filt[j] = __ldg(fsrc + j);
      __syncthreads();
      if (threadIdx.x == 0) s_staged = slot;
    }
    const int32_t* T = in_smem ? s_tab : tab + tab_off[slot] * stride;
    const uint32_t* Fl = in_smem ? s_filt : filt + (int64_t)slot * kSlotFilterWords;
    const uint32_t theta = (uint32_t)tab_theta[slot];
    const int64_t lo = s_lo, hi = s_hi;
    for (;;) {
      unsigned long long took = 0;
      if (lane == 0) took = atomicAdd(&s_take, (unsigned long long)kPruneTake);
      took = __shfl_sync(0xffffffffu, took, 0);
      const int64_t i0 = lo + (int64_t)took;
      if (i0 >= hi) break;
      const int64_t i1 = min(hi, i0 + kPruneTake);
      for (int64_t i = i0; i < i1; i++) {
        int4 kept = make_int4(0, 0, 0, 0);
        const bool keep = prune_candidate<32, 1, false, F, true>(C[i], h, s_hub, map, cand, rows, row_len, T, cap, stride,
                                                           Fl, theta, lane, 0xffffffffu, scanned, visible, kept);
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) kbuf[kn + __popc(m & ((1u << lane) - 1u))] = kept;
        kn += __popc(m);
        if (kn >= 32) prune_flush(kbuf, kn, map, h, K, s_hub, Fout, wl_v, wl_key, wl_par, ctr);
      }
    }
    __syncthreads();  // the tile's joins are done before the table is replaced
  }
  prune_flush(kbuf, kn, map, h, K, s_hub, Fout, wl_v, wl_key, wl_par, ctr);
  if (lane == 0 && scanned) atomicAdd(&ctr->reads, scanned);
  if (lane == 0 && visible) atomicAdd(&ctr->visible, visible);
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

// Pool entries of the segments each touched row needs for this commit's
// arrivals.
__global__ void k_seg_need(const Counters* ctr, const int32_t* __restrict__ touched,
                           const int32_t* __restrict__ row_len, const int32_t* __restrict__ cnt, Counters* wctr) {
  int64_t total = (int64_t)ctr->touched;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int v = touched[i];
    const int64_t len = row_len[v], need = len + cnt[v];
    const int s0 = segs_for(len), s1 = segs_for(need);
    if (s1 > kSegs) {
      wctr->seg_over = 1;
      continue;
    }
    if (s1 > s0) atomicAdd(&wctr->seg_need, (unsigned long long)(seg_first(s1) - seg_first(s0)));
  }
}

// Carves the new segments of every touched row from the current chunk.
__global__ void k_seg_alloc(const Counters* ctr, const int32_t* __restrict__ touched,
                            const int32_t* __restrict__ row_len, const int32_t* __restrict__ cnt,
                            int64_t* __restrict__ seg, int64_t chunk, unsigned long long* chunk_tail) {
  int64_t total = (int64_t)ctr->touched;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int v = touched[i];
    const int64_t len = row_len[v], need = len + cnt[v];
    const int s0 = segs_for(len), s1 = min(segs_for(need), kSegs);
    if (s1 <= s0) continue;
    const unsigned long long base =
        atomicAdd(chunk_tail, (unsigned long long)(seg_first(s1) - seg_first(s0)));
    for (int j = s0; j < s1; j++)
      seg[(int64_t)v * kSegs + j] = (chunk << 48) | (int64_t)(base + (unsigned long long)(seg_first(j) - seg_first(s0)));
  }
}

template <class F>
__global__ void k_scatter(const Counters* ctr, const int32_t* __restrict__ wl_v, const uint64_t* __restrict__ wl_key,
                          const int32_t* __restrict__ wl_par, int32_t* __restrict__ row_len, Rows<F> rows) {
  int64_t total = (int64_t)ctr->wl_count;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int v = wl_v[p];
    const int pos = atomicAdd(&row_len[v], 1);
    const int i = seg_of(pos);
    const int64_t r = rows.seg[(int64_t)v * kSegs + i] + (pos - seg_first(i));
    const uint64_t x = wl_key[p];
    *rows.keys_of(r) = rows.f.pack(lkey_hub(x), lkey_hop(x), lkey_dist(x));
    rows.cp[r >> 48][r & kEntryMask] = wl_par[p];
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

template <class F>
__global__ void k_final_copy(int32_t n, Rows<F> rows, const int32_t* __restrict__ row_len,
                             const int64_t* __restrict__ foff, uint64_t* __restrict__ fkey,
                             int32_t* __restrict__ fpar) {
  int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    int64_t dst = foff[v];
    int len = row_len[v];
    for (int j = lane; j < len; j += 32) {
      const int64_t r = rows.ref((int)v, j);
      const typename F::key_t x = *rows.keys_of(r);
      fkey[dst + j] = lkey(rows.f.hub(x), rows.f.hop(x), rows.f.dist(x));
      fpar[dst + j] = rows.cp[r >> 48][r & kEntryMask];
    }
    if (lane == 0) {
      // self label (v, v, 0, 0), pushed by the reference when hub v starts
      // (generation.h:74-85)
      fkey[dst + len] = lkey((uint32_t)v, 0, 0);
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
  // dense candidate rows: max_wave * n * 8 B within an eighth of the budget,
  // at most 8192 hubs per wave (at n = 1M: 2048 hubs 2.26 s, 4096 2.21 s,
  // 8192 2.16 s of generation)
  int64_t avail = budget_bytes > 0 ? budget_bytes / 8 : (int64_t)16 << 30;
  int64_t w = avail / ((int64_t)n * 8);
  w = std::max<int64_t>(1, std::min<int64_t>(8192, w));
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
                const BatchPlan* plan, int32_t hub_limit) {
  const int32_t n = g->n;
  cudaStream_t st = idx->stream;
  const int sms = device_sm_count();
  const int stride = (K + 2 <= 8) ? 8 : 16;  // hub-table slot: key + K+1 distances, 32 or 64 B
  const int32_t rank_prune = opts.generation == 0 ? 1 : 0;  // the HSDL search; 0 = the 2023WWW search
  double t0 = now_s();

  size_t free_b = 0, total_b = 0;
  HSDL_CUDA(cudaMemGetInfo(&free_b, &total_b));
  int64_t budget = opts.device_budget_bytes > 0 ? opts.device_budget_bytes : (int64_t)free_b;
  std::vector<int32_t> bounds;
  if (plan) {
    // the plan's layer waves, split where a wave's dense candidate rows would
    // pass an eighth of the budget
    const int64_t cand_cap = std::max<int64_t>((int64_t)1 << 20, budget / 8 / (int64_t)sizeof(uint64_t));
    bounds.push_back(0);
    for (size_t i = 0; i + 1 < plan->bounds.size(); i++) {
      int64_t acc = 0;
      for (int32_t v = plan->bounds[i]; v < plan->bounds[i + 1]; v++) {
        if (acc > 0 && acc + plan->comp_n[v] > cand_cap) {
          bounds.push_back(v);
          acc = 0;
        }
        acc += plan->comp_n[v];
      }
      bounds.push_back(plan->bounds[i + 1]);
    }
  } else {
    int32_t max_wave = opts.max_wave > 0 ? opts.max_wave : auto_max_wave(n, budget);
    bounds = wave_schedule(n, opts.first_wave > 0 ? opts.first_wave : 1, max_wave);
    if (hub_limit > 0 && hub_limit < n) {  // only the first hub_limit hubs search
      while (bounds.size() > 1 && bounds.back() > hub_limit) bounds.pop_back();
      if (bounds.back() < hub_limit) bounds.push_back(hub_limit);
    }
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
  DevBuf<int32_t> row_len, cnt, touched;
  DevBuf<int64_t> seg;  // [n][kSegs] segment references of the committed rows
  // the label pool: chunks of keys and parents, and their device tables
  std::vector<DevBuf<uint64_t>> chunk_keys;  // KT keys, stored in 8-byte words
  std::vector<DevBuf<int32_t>> chunk_par;
  DevBuf<void*> d_ck;
  DevBuf<int32_t*> d_cp;
  DevBuf<unsigned long long> chunk_tail;
  DevBuf<int2> Cl, Cs;  // the candidate list, and its copy grouped by vertex range
  DevBuf<unsigned int> bcnt;
  DevBuf<unsigned long long> bcur, bstart, tstart;
  DevBuf<int4> Fa, Fb;
  DevBuf<int32_t> wl_v, wl_par;
  DevBuf<uint64_t> wl_key;
  DevBuf<int64_t> tab_off;
  DevBuf<int32_t> tab_cap, tab;
  DevBuf<uint32_t> filt;
  DevBuf<int32_t> wave_end_of, tab_theta;  // end of each started hub's wave; per-slot stop threshold
  DevBuf<Counters> ctr;
  auto release_pool = [&]() {
    for (auto& c : chunk_keys) c.release();
    for (auto& c : chunk_par) c.release();
    chunk_keys.clear();
    chunk_par.clear();
    d_ck.release(); d_cp.release(); chunk_tail.release(); seg.release();
  };
  auto release_all = [&]() {
    cand.release(); row_len.release(); cnt.release(); touched.release();
    Cl.release(); Cs.release(); bcnt.release(); bcur.release(); bstart.release(); tstart.release(); Fa.release(); Fb.release(); wl_v.release();
    wl_par.release(); wl_key.release(); tab_off.release(); tab_cap.release(); tab.release(); ctr.release();
    d_base.release(); filt.release(); wave_end_of.release(); tab_theta.release();
    release_pool();
  };
  struct Guard {
    std::function<void()> f;
    ~Guard() { f(); }
  } guard{release_all};

  HSDL_TRY(cand.alloc(cand_entries, st));
  HSDL_CUDA(cudaMemsetAsync(cand.p, 0xFF, (size_t)cand.bytes(), st));
  HSDL_TRY(row_len.alloc(n, st));
  HSDL_TRY(cnt.alloc(n, st));
  HSDL_TRY(touched.alloc(n, st));
  HSDL_TRY(seg.alloc((int64_t)n * kSegs, st));
  HSDL_CUDA(cudaMemsetAsync(row_len.p, 0, (size_t)row_len.bytes(), st));
  HSDL_CUDA(cudaMemsetAsync(cnt.p, 0, (size_t)cnt.bytes(), st));
  HSDL_TRY(d_ck.alloc(kMaxChunks, st));
  HSDL_TRY(d_cp.alloc(kMaxChunks, st));
  HSDL_TRY(chunk_tail.alloc(1, st));
  std::vector<void*> h_ck;
  // pool key format: 4-byte keys (Fmt32) when every hub id, hop (<= K, with
  // room for the all-ones "no label" hop above it) and distance (<= K x the
  // largest weight) fit, unless the options ask for 8-byte keys
  int fH = 1, fP = 1;
  while (fH < 32 && ((uint32_t)std::max(0, n - 1) >> fH) != 0) fH++;
  while (fP < 32 && ((uint32_t)(K + 1) >> fP) != 0) fP++;
  const int fD = 32 - fH - fP;
  const bool pool32 = opts.pool_key_bytes != 8 && fD >= 1 && fD < 31 &&
                      (int64_t)K * std::max(1, g->max_w) < ((int64_t)1 << fD);
  const Fmt32 f32{(uint32_t)(fP + fD), (uint32_t)std::max(fD, 1)};
  const int64_t pool_entry_bytes = (pool32 ? 4 : 8) + (int64_t)sizeof(int32_t);  // label key + parent
  idx->pool_key_bytes = pool32 ? 4 : 8;
  std::vector<int32_t*> h_cp;
  // Memory plan: the candidate lists of a wave take at most a quarter of the
  // budget (a wave needing more is split); the label pool takes what is left.
  const int64_t c_limit = std::max<int64_t>(1 << 16, budget / 4 / kListEntryBytes);
  // First pool chunk: 1.4x the expected label count (about 0.53 sqrt(n)
  // (deg / 10) (K / 5) labels per vertex on power-law graphs; segments hold
  // rows at 1.4x their length on average), within a third of the budget.
  // Later chunks add a quarter of the pool (at least what the commit needs).
  int64_t first_chunk = std::max<int64_t>(1 << 20, (int64_t)n * 16);
  if (!plan) {
    const double deg = (double)g->m2 / std::max(1, n);
    const double per_v = 0.53 * std::sqrt((double)n) * std::max(1.0, deg / 10.0) * K / 5.0;
    first_chunk = std::max<int64_t>(first_chunk, (int64_t)(1.4 * per_v * n));
  }
  first_chunk = std::max<int64_t>(1 << 16, std::min<int64_t>(first_chunk, budget / 3 / pool_entry_bytes));
  int64_t pool_total = 0, chunk_cap = 0, chunk_used = 0;
  auto add_chunk = [&](int64_t entries) -> int {
    if ((int)chunk_keys.size() >= kMaxChunks) {
      set_error("label pool: too many chunks");
      return HSDL_ERR_NOMEM;
    }
    chunk_keys.emplace_back();
    chunk_par.emplace_back();
    HSDL_TRY(chunk_keys.back().alloc(pool32 ? (entries + 1) / 2 : entries, st));
    HSDL_TRY(chunk_par.back().alloc(entries, st));
    h_ck.push_back(chunk_keys.back().p);
    h_cp.push_back(chunk_par.back().p);
    HSDL_CUDA(cudaMemcpyAsync(d_ck.p, h_ck.data(), sizeof(void*) * h_ck.size(), cudaMemcpyHostToDevice, st));
    HSDL_CUDA(cudaMemcpyAsync(d_cp.p, h_cp.data(), sizeof(int32_t*) * h_cp.size(), cudaMemcpyHostToDevice, st));
    HSDL_CUDA(cudaMemsetAsync(chunk_tail.p, 0, sizeof(unsigned long long), st));
    pool_total += entries;
    chunk_cap = entries;
    chunk_used = 0;
    return HSDL_OK;
  };
  HSDL_TRY(add_chunk(first_chunk));
  const Rows<Fmt64> rows64{seg.p, d_ck.p, d_cp.p, Fmt64{}};
  const Rows<Fmt32> rows32{seg.p, d_ck.p, d_cp.p, f32};
  int64_t capC = std::min<int64_t>(std::max<int64_t>(1 << 20, (int64_t)n * 4), c_limit);
  // candidate order of the pruning join: 0 = grouped by vertex range, 2 =
  // grouped by slot and joined with the hub table in shared memory (the
  // HSDL search, waves of at most kPartMaxBuckets hubs, 32 lanes per
  // candidate; other waves are grouped by vertex range), 1 = expansion order
  const bool part = opts.prune_order != 1;
  const bool by_slot_opt = opts.prune_order == 2 && rank_prune && Wmax <= kPartMaxBuckets;
  auto alloc_lists = [&](int64_t c) -> int {
    HSDL_TRY(Cl.alloc(c, st));
    if (part) HSDL_TRY(Cs.alloc(c, st));
    HSDL_TRY(Fa.alloc(c, st));
    HSDL_TRY(Fb.alloc(c, st));
    HSDL_TRY(wl_v.alloc(c, st));
    HSDL_TRY(wl_par.alloc(c, st));
    HSDL_TRY(wl_key.alloc(c, st));
    return HSDL_OK;
  };
  HSDL_TRY(alloc_lists(capC));
  // vertex ranges of the candidate partition: ids >> part_shift < kPartBuckets
  int part_shift = 0;
  while (((int64_t)(n - 1) >> part_shift) >= kPartBuckets) part_shift++;
  if (part) {
    HSDL_TRY(bcnt.alloc(kPartMaxBuckets, st));
    HSDL_TRY(bcur.alloc(kPartMaxBuckets, st));
    HSDL_CUDA(cudaMemsetAsync(bcnt.p, 0, (size_t)bcnt.bytes(), st));
  }
  if (by_slot_opt) {
    HSDL_TRY(bstart.alloc((int64_t)Wmax + 1, st));
    HSDL_TRY(tstart.alloc((int64_t)Wmax + 1, st));
  }
  const int nb_slot = std::max(1, Wmax);
  const size_t smem_rc = sizeof(unsigned int) * kPartBuckets, smem_rs = 12 * (size_t)kPartBuckets;
  const size_t smem_sc = sizeof(unsigned int) * nb_slot, smem_ss = 12 * (size_t)nb_slot;
  HSDL_CUDA(cudaFuncSetAttribute(k_part_scatter<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(12 * kPartMaxBuckets)));
  HSDL_CUDA(cudaFuncSetAttribute(k_part_count<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(4 * kPartMaxBuckets)));
  HSDL_CUDA(cudaFuncSetAttribute(k_prune_slot<Fmt32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotSmem));
  HSDL_CUDA(cudaFuncSetAttribute(k_prune_slot<Fmt64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotSmem));
  const int g_part = sms * resident_blocks(k_part_scatter<false>, kThreads, smem_rs);
  const int g_part_slot = sms * resident_blocks(k_part_scatter<true>, kThreads, smem_ss);
  const int g_slot = sms * (pool32 ? resident_blocks(k_prune_slot<Fmt32>, kSlotThreads, kSlotSmem)
                                   : resident_blocks(k_prune_slot<Fmt64>, kSlotThreads, kSlotSmem));
  HSDL_TRY(tab_off.alloc(Wmax, st));
  HSDL_TRY(tab_cap.alloc(Wmax, st));
  HSDL_TRY(filt.alloc((int64_t)Wmax * kSlotFilterWords, st));
  HSDL_TRY(wave_end_of.alloc(n, st));
  HSDL_TRY(tab_theta.alloc(Wmax, st));
  int64_t tab_cap_entries = 1 << 16;
  HSDL_TRY(tab.alloc(tab_cap_entries * stride, st));
  HSDL_TRY(ctr.alloc(1, st));
  // grids of exactly one resident wave per kernel (grid-stride loops inside)
  const int grid = sms * resident_blocks(k_scatter<Fmt64>, 256);
  // tunables: threads per expansion block, frontier entries a block takes at
  // a time, lanes per pruning candidate (0 = chosen per wave from the mean
  // committed row length)
  const int tpb = (opts.block_threads == 128 || opts.block_threads == 512) ? opts.block_threads : 256;
  const int32_t tiles = std::max(1, opts.frontier_tile / tpb);
  const int fixed_lanes = (opts.prune_lanes == 8 || opts.prune_lanes == 16 || opts.prune_lanes == 32)
                              ? opts.prune_lanes : 0;
  const int g_expand = sms * (tpb == 128   ? resident_blocks(k_expand<128>, 128)
                              : tpb == 512 ? resident_blocks(k_expand<512>, 512)
                                           : resident_blocks(k_expand<256>, 256));
  const int g_heavy = sms * (tpb == 128   ? resident_blocks(k_expand_heavy<128>, 128)
                             : tpb == 512 ? resident_blocks(k_expand_heavy<512>, 512)
                                          : resident_blocks(k_expand_heavy<256>, 256));
  DevBuf<int2> chunk_map;  // heavy expansion tiles, split into chunks
  HSDL_TRY(chunk_map.alloc(kExpandChunkCap, st));
  const int pairs = opts.prune_pairs == 2 ? 2 : 1;
  auto prune_blocks = [&](auto fmt, auto g) -> int {
    using Fm = decltype(fmt);
    constexpr int G = decltype(g)::value;
    return sms * (!rank_prune ? resident_blocks(k_prune<G, 1, true, Fm>, kThreads)
                  : pairs == 2 ? resident_blocks(k_prune<G, 2, false, Fm>, kThreads)
                               : resident_blocks(k_prune<G, 1, false, Fm>, kThreads));
  };
  using G8 = std::integral_constant<int, 8>;
  using G16 = std::integral_constant<int, 16>;
  using G32 = std::integral_constant<int, 32>;
  const int g_prune8 = pool32 ? prune_blocks(Fmt32{}, G8{}) : prune_blocks(Fmt64{}, G8{});
  const int g_prune16 = pool32 ? prune_blocks(Fmt32{}, G16{}) : prune_blocks(Fmt64{}, G16{});
  const int g_prune32 = pool32 ? prune_blocks(Fmt32{}, G32{}) : prune_blocks(Fmt64{}, G32{});
  int lanes = 32;

  Counters hc;
  int64_t committed = 0;  // labels in the pool

  auto held = [&]() -> int64_t {
    return cand.bytes() + row_len.bytes() + cnt.bytes() + touched.bytes() + seg.bytes() +
           pool_total * pool_entry_bytes + Cl.bytes() + Cs.bytes() + Fa.bytes() + Fb.bytes() + wl_v.bytes() +
           wl_par.bytes() + wl_key.bytes() + tab_off.bytes() + tab_cap.bytes() + tab.bytes() + d_base.bytes() +
           filt.bytes() + chunk_map.bytes() + idx->off.bytes() + idx->key.bytes() + idx->par.bytes();
  };
  auto note_peak = [&]() { idx->build_peak = std::max(idx->build_peak, held()); };
  note_peak();
  // The K hops of a wave (expand, mark, prune per hop) run as one CUDA graph.
  // The kernels read the wave's first hub and their list bounds from the
  // counters in device memory, so one graph serves every wave until a buffer
  // it names is reallocated (then it is captured again).
  HopGraph hops;
  auto launch_hops = [&]() -> int {
    for (int32_t h = 1; h <= K; h++) {
      int4* Fin = (h & 1) ? Fa.p : Fb.p;
      int4* Fout = (h & 1) ? Fb.p : Fa.p;
#define HSDL_EXPAND(TPB)                                                                                  \
  k_expand<TPB><<<g_expand, TPB, 0, st>>>(map, h, K, rank_prune, tiles, g->rp.p, g->adj.p, Fin, cand.p, Cl.p, \
                                          capC, ctr.p, chunk_map.p);                                         \
  HSDL_CUDA(cudaGetLastError());                                                                            \
  k_expand_heavy<TPB><<<g_heavy, TPB, 0, st>>>(map, h, K, rank_prune, g->rp.p, g->adj.p, Fin, cand.p, Cl.p,  \
                                               capC, ctr.p, chunk_map.p)
      if (tpb == 128) {
        HSDL_EXPAND(128);
      } else if (tpb == 512) {
        HSDL_EXPAND(512);
      } else {
        HSDL_EXPAND(256);
      }
#undef HSDL_EXPAND
      HSDL_CUDA(cudaGetLastError());
      k_mark<<<1, 1, 0, st>>>(ctr.p, h, capC);
      HSDL_CUDA(cudaGetLastError());
      const bool slot_mode = by_slot_opt && lanes == 32;
      if (slot_mode) {
        k_part_count<true><<<g_part_slot, kThreads, smem_sc, st>>>(ctr.p, h, Cl.p, bcnt.p, 0, nb_slot);
        HSDL_CUDA(cudaGetLastError());
        k_part_scan<<<1, 1024, 0, st>>>(ctr.p, h, bcnt.p, bcur.p, nb_slot, kSlotTile, bstart.p, tstart.p);
        HSDL_CUDA(cudaGetLastError());
        k_part_scatter<true><<<g_part_slot, kThreads, smem_ss, st>>>(ctr.p, h, Cl.p, Cs.p, bcur.p, 0, nb_slot);
        HSDL_CUDA(cudaGetLastError());
        if (pool32)
          k_prune_slot<Fmt32><<<g_slot, kSlotThreads, kSlotSmem, st>>>(
              map, h, K, Cs.p, cand.p, rows32, row_len.p, tab_off.p, tab_cap.p, tab.p, stride, filt.p, tab_theta.p,
              bstart.p, tstart.p, nb_slot, Fout, wl_v.p, wl_key.p, wl_par.p, ctr.p);
        else
          k_prune_slot<Fmt64><<<g_slot, kSlotThreads, kSlotSmem, st>>>(
              map, h, K, Cs.p, cand.p, rows64, row_len.p, tab_off.p, tab_cap.p, tab.p, stride, filt.p, tab_theta.p,
              bstart.p, tstart.p, nb_slot, Fout, wl_v.p, wl_key.p, wl_par.p, ctr.p);
        HSDL_CUDA(cudaGetLastError());
        continue;
      }
      if (part) {
        k_part_count<false><<<g_part, kThreads, smem_rc, st>>>(ctr.p, h, Cl.p, bcnt.p, part_shift, kPartBuckets);
        HSDL_CUDA(cudaGetLastError());
        k_part_scan<<<1, 1024, 0, st>>>(ctr.p, h, bcnt.p, bcur.p, kPartBuckets, 0, nullptr, nullptr);
        HSDL_CUDA(cudaGetLastError());
        k_part_scatter<false><<<g_part, kThreads, smem_rs, st>>>(ctr.p, h, Cl.p, Cs.p, bcur.p, part_shift,
                                                                 kPartBuckets);
        HSDL_CUDA(cudaGetLastError());
      }
      const int2* Cp = part ? Cs.p : Cl.p;
#define HSDL_PRUNE(G, P, SELF, GRID)                                                                          \
  do {                                                                                                        \
    if (pool32)                                                                                               \
      k_prune<G, P, SELF, Fmt32><<<GRID, kThreads, 0, st>>>(map, h, K, Cp, cand.p, rows32, row_len.p,       \
                                                            tab_off.p, tab_cap.p, tab.p, stride, filt.p,     \
                                                            tab_theta.p, Fout, wl_v.p, wl_key.p, wl_par.p,   \
                                                            ctr.p);                                          \
    else                                                                                                      \
      k_prune<G, P, SELF, Fmt64><<<GRID, kThreads, 0, st>>>(map, h, K, Cp, cand.p, rows64, row_len.p,       \
                                                            tab_off.p, tab_cap.p, tab.p, stride, filt.p,     \
                                                            tab_theta.p, Fout, wl_v.p, wl_key.p, wl_par.p,   \
                                                            ctr.p);                                          \
  } while (0)
      if (!rank_prune) {  // the 2023WWW search: candidates from earlier waves probe their self label
        if (lanes == 8) HSDL_PRUNE(8, 1, true, g_prune8);
        else if (lanes == 16) HSDL_PRUNE(16, 1, true, g_prune16);
        else HSDL_PRUNE(32, 1, true, g_prune32);
      } else if (pairs == 2) {
        if (lanes == 8) HSDL_PRUNE(8, 2, false, g_prune8);
        else if (lanes == 16) HSDL_PRUNE(16, 2, false, g_prune16);
        else HSDL_PRUNE(32, 2, false, g_prune32);
      } else {
        if (lanes == 8) HSDL_PRUNE(8, 1, false, g_prune8);
        else if (lanes == 16) HSDL_PRUNE(16, 1, false, g_prune16);
        else HSDL_PRUNE(32, 1, false, g_prune32);
      }
#undef HSDL_PRUNE
      HSDL_CUDA(cudaGetLastError());
    }
    return HSDL_OK;
  };
  auto run_hops = [&]() -> int {
    const uintptr_t key[HopGraph::kKey] = {(uintptr_t)Cl.p, (uintptr_t)Fa.p, (uintptr_t)Fb.p,
                                           (uintptr_t)cand.p, (uintptr_t)tab.p, (uintptr_t)seg.p,
                                           (uintptr_t)wl_v.p, (uintptr_t)wl_key.p, (uintptr_t)wl_par.p,
                                           (uintptr_t)capC, (uintptr_t)lanes, (uintptr_t)Cs.p};
    HSDL_TRY(hops.ensure(key, st, launch_hops));
    HSDL_CUDA(cudaGraphLaunch(hops.exec, st));
    launch_counter().fetch_add((part ? 6 : 3) * K, std::memory_order_relaxed);
    return HSDL_OK;
  };
  for (size_t wv = 0; wv + 1 < bounds.size();) {
    const int32_t s_hub = bounds[wv], W = bounds[wv + 1] - bounds[wv];
    bool split = false;
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
      k_wave_init<<<(W + 255) / 256, 256, 0, st>>>(W, s_hub, map, cand.p, Cl.p, Fa.p, ctr.p, wave_end_of.p);
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
        HSDL_CUDA(cudaMemsetAsync(filt.p, 0, (size_t)W * kSlotFilterWords * sizeof(uint32_t), st));
        if (pool32)
          k_table_fill<Fmt32><<<std::min(grid, (W + 7) / 8), 256, 0, st>>>(
              W, s_hub, rows32, row_len.p, tab_off.p, tab_cap.p, tab.p, stride, filt.p, wave_end_of.p, tab_theta.p);
        else
          k_table_fill<Fmt64><<<std::min(grid, (W + 7) / 8), 256, 0, st>>>(
              W, s_hub, rows64, row_len.p, tab_off.p, tab_cap.p, tab.p, stride, filt.p, wave_end_of.p, tab_theta.p);
        HSDL_LAUNCHED();
        k_table_prefix<<<grid, 256, 0, st>>>(ctr.p, tab.p, stride, K);
        HSDL_LAUNCHED();
      }
      if (fixed_lanes) {
        lanes = fixed_lanes;
      } else {
        const int64_t mean_row = committed / std::max<int32_t>(n, 1);
        lanes = mean_row < 24 ? 8 : mean_row < 96 ? 16 : 32;
      }
      HSDL_TRY(run_hops());
      HSDL_CUDA(cudaMemcpyAsync(&hc, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
      HSDL_CUDA(cudaStreamSynchronize(st));
      idx->build_max_cand = std::max<int64_t>(idx->build_max_cand, (int64_t)hc.c_count);
      if (!hc.overflow) break;
      // The candidate list overflowed: entries past its end were never
      // recorded, so clear this wave's slots wholesale and rerun the wave with
      // room for twice what was asked, or, when that would pass the lists'
      // share of memory, as two half waves (any split of a wave in rank
      // order generates a superset of the canonical labels).
      HSDL_CUDA(cudaMemsetAsync(cand.p, 0xFF, (size_t)wave_entries * sizeof(uint64_t), st));
      const int64_t want = std::max<int64_t>(capC * 2, (int64_t)hc.c_count * 2);
      size_t fb_now = 0, tb_now = 0;
      HSDL_CUDA(cudaMemGetInfo(&fb_now, &tb_now));
      // the lists are replaced, not grown: the old ones are freed first
      const int64_t list_room = ((int64_t)fb_now + capC * kListEntryBytes) / 2;
      if ((want > c_limit || want * kListEntryBytes > list_room) && W > 1) {
        bounds.insert(bounds.begin() + (std::ptrdiff_t)wv + 1, s_hub + W / 2);
        idx->wave_splits++;
        split = true;
        break;
      }
      capC = want;
      HSDL_TRY(alloc_lists(capC));
      note_peak();
      if (attempt > 40) {
        set_error("candidate list could not be sized");
        return HSDL_ERR_NOMEM;
      }
    }
    if (split) continue;
    idx->work_relax += (int64_t)hc.relax;
    idx->work_candidates += (int64_t)std::min<unsigned long long>(hc.c_count, (unsigned long long)capC);
    idx->work_join_reads += (int64_t)hc.reads;
    idx->work_join_visible += (int64_t)hc.visible;
    idx->work_labels_written += (int64_t)hc.wl_count;
    // commit the wave's labels
    if (hc.wl_count > 0) {
      k_count<<<grid, 256, 0, st>>>(ctr.p, wl_v.p, cnt.p, touched.p, ctr.p);
      HSDL_LAUNCHED();
      k_seg_need<<<grid, 256, 0, st>>>(ctr.p, touched.p, row_len.p, cnt.p, ctr.p);
      HSDL_LAUNCHED();
      HSDL_CUDA(cudaMemcpyAsync(&hc, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
      HSDL_CUDA(cudaStreamSynchronize(st));
      if (hc.seg_over) {
        set_error("a label row outgrew 2^28 labels");
        return HSDL_ERR_INVALID;
      }
      const int64_t need = (int64_t)hc.seg_need;
      if (chunk_used + need > chunk_cap) {
        // a new chunk: a quarter of the pool so far, at least this commit's need
        HSDL_TRY(add_chunk(std::max<int64_t>(need, std::max<int64_t>(1 << 20, pool_total / 4))));
        note_peak();
      }
      k_seg_alloc<<<grid, 256, 0, st>>>(ctr.p, touched.p, row_len.p, cnt.p, seg.p, (int64_t)chunk_keys.size() - 1,
                                        chunk_tail.p);
      HSDL_LAUNCHED();
      chunk_used += need;
      idx->build_pool += need;
      if (pool32)
        k_scatter<Fmt32><<<grid, 256, 0, st>>>(ctr.p, wl_v.p, wl_key.p, wl_par.p, row_len.p, rows32);
      else
        k_scatter<Fmt64><<<grid, 256, 0, st>>>(ctr.p, wl_v.p, wl_key.p, wl_par.p, row_len.p, rows64);
      HSDL_LAUNCHED();
      k_clear_cnt<<<grid, 256, 0, st>>>(ctr.p, touched.p, cnt.p);
      HSDL_LAUNCHED();
      committed += (int64_t)hc.wl_count;
    }
    k_reset<<<grid, 256, 0, st>>>(ctr.p, Cl.p, cand.p, map, capC);
    HSDL_LAUNCHED();
    idx->waves++;
    wv++;
  }
  HSDL_CUDA(cudaStreamSynchronize(st));
  double t1 = now_s();
  idx->pool_chunks = (int32_t)chunk_keys.size();
  {
    // each hub's wave, for the clean's wave window
    std::vector<int32_t> h_lo((size_t)n, 0);
    for (size_t i = 0; i + 1 < bounds.size(); i++)
      for (int32_t u = bounds[i]; u < bounds[i + 1] && u < n; u++) h_lo[u] = bounds[i];
    HSDL_TRY(idx->wave_lo.alloc(n, st));
    HSDL_CUDA(cudaMemcpyAsync(idx->wave_lo.p, h_lo.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    HSDL_CUDA(cudaStreamSynchronize(st));
  }
  // only the rows and the pool are needed from here on
  cand.release(); cnt.release(); touched.release(); Cl.release(); Fa.release(); Fb.release(); wl_v.release();
  wl_par.release(); wl_key.release(); tab_off.release(); tab_cap.release(); tab.release(); filt.release(); wave_end_of.release(); tab_theta.release();

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
  HSDL_TRY(idx->key.alloc(total + kRowPad, st));
  HSDL_TRY(idx->par.alloc(total + kRowPad, st));
  note_peak();
  if (pool32)
    k_final_copy<Fmt32><<<grid * 2, 256, 0, st>>>(n, rows32, row_len.p, idx->off.p, idx->key.p, idx->par.p);
  else
    k_final_copy<Fmt64><<<grid * 2, 256, 0, st>>>(n, rows64, row_len.p, idx->off.p, idx->key.p, idx->par.p);
  HSDL_LAUNCHED();
  flen.release();
  release_all();
  int64_t mr = 0;
  HSDL_TRY(row_max(n, idx->off.p, &mr, st));
  HSDL_TRY(sort_rows(n, idx->off.p, idx->key.p, idx->par.p, mr, st));
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
