// Canonical repair (clean) of a generated label set.
//
// Reference rule: hop_constrained_clean_L
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:422-511).
// For every vertex v, label (u, h, d) in L[v] is dropped iff some label
// (w, h1, d1) of L[u] and some label (w, h2, d2) of v already accepted satisfy
// h1 + h2 <= h and d1 + d2 <= d (:451-482).
//
// Parallel form.  The reference walks L[v] in order and checks against the
// labels of v accepted so far.  For a label set that is a superset of the
// canonical labels and whose every label is a real walk (what generation
// produces), checking against *all* labels of v gives the same verdict: a
// covering pair through a non-accepted label is itself a walk from u to v
// through a hub ranked at or above u within h hops and distance d, so the
// label is not canonical either way.  The one pair to exclude is the label
// against itself: the only label of L[u] with hub u is u's self label
// (u, 0, 0), so for hub w = u the check uses v's labels of hub u with fewer
// than h hops.  Every label is therefore decided independently.
//
// Only hubs ranked above u are witnesses: in the reference's walk over the
// sorted L[v], the accepted labels of v when (u, h, d) comes up have hubs
// ranked at or above u.  For labels of the HSDL search every hub of L[u] is
// ranked at or above u anyway; labels of the 2023WWW search (no rank prune)
// also put hubs ranked below u into L[u], and those are skipped.  below[u]
// counts the labels of the sorted L[u] with hubs ranked above u (its prefix).
//
// Wave window.  For labels generated by the wave engine, the pruning query of
// u's search already saw every pair through a hub w of an earlier wave: both
// w's label of u and w's label of v were committed before u's wave, and the
// pruning rule is this rule.  What it could not see are hubs of u's own wave
// (ranked above u), whose labels were committed with u's.  So when the index
// records each hub's wave (wave_lo[u] = the wave's first hub), a label (u, h, d)
// of v is checked against the hubs w of L[u] with wave_lo[u] <= w < u - the
// tail of the prefix below[u] - plus u's own fewer-hop labels of v.  Without
// the record (an imported label set) the whole prefix is scanned.
//
// Kernel: one block per vertex v (persistent blocks take vertices from a work
// counter).  The block builds v's hop-prefix-min table T_v (hash on hub id, in
// shared memory, or in a per-block global scratch area for very long rows),
// then each warp takes labels (u, h, d) of v and scans L[u] with its lanes,
// probing T_v and reducing with a warp-wide min.
#include <algorithm>
#include <chrono>
#include <climits>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int kCleanThreads = 512;  // 256 / 512 / 1024 threads: clean 0.275 / 0.207 / 0.220 s at n = 1M
// Membership filter of v's hubs: one bit per hash value of a hub id, 65,536
// bits in shared memory.  Most hubs of L[u] are not hubs of v; a clear bit
// answers those with one shared-memory load instead of a probe sequence
// (whose longest chain in a warp sets the warp's time).
constexpr int kFilterBits = 16;
constexpr int kFilterWords = (1 << kFilterBits) / 32;

// v's hub table: keys Tk[cap] (one word per slot, so the 32 lanes of a probe
// spread over the shared-memory banks) and rows Td[cap][K+1] of
// hop-prefix-min distances.  Returns the slot of hub w, or -1.
__device__ inline int tab_find(const int32_t* Tk, uint32_t mask, int32_t w) {
  uint32_t ix = table_hash((uint32_t)w, mask);
  for (uint32_t probe = 0; probe <= mask; probe++) {
    const int32_t kk = Tk[ix];
    if (kk == w) return (int)ix;
    if (kk == kEmptyKey) return -1;
    ix = (ix + 1) & mask;
  }
  return -1;
}

__global__ void __launch_bounds__(kCleanThreads) k_clean(int32_t n, int32_t K, const int64_t* __restrict__ off,
                                                         const uint64_t* __restrict__ key,
                                                         uint8_t* __restrict__ keep, int64_t* __restrict__ kept,
                                                         const int32_t* __restrict__ wave_lo,
                                                         const int32_t* __restrict__ below,
                                                         int smem_slots, int32_t* __restrict__ gscratch,
                                                         int64_t gscratch_slots, int* __restrict__ next_v,
                                                         unsigned long long* __restrict__ reads) {
  extern __shared__ int32_t smem_tab[];
  __shared__ uint32_t s_filter[kFilterWords];
  __shared__ int s_v;
  __shared__ int s_kept[kCleanThreads / 32];
  const int lane = lane_id(), wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int R = K + 1;  // distances per slot
  unsigned long long scanned = 0;
  for (;;) {
    if (threadIdx.x == 0) s_v = atomicAdd(next_v, 1);
    __syncthreads();
    const int v = s_v;
    if (v >= n) {
      if (lane == 0 && scanned) atomicAdd(reads, scanned);
      break;
    }
    const int64_t lo = off[v];
    const int len = (int)(off[v + 1] - lo);
    int64_t cap = 8;
    while (cap < (int64_t)len + len / 2) cap <<= 1;  // load factor <= 2/3
    int32_t* Tk = (cap <= smem_slots) ? smem_tab : gscratch + (int64_t)blockIdx.x * gscratch_slots * (1 + R);
    int32_t* Td = Tk + cap;
    const uint32_t mask = (uint32_t)cap - 1;
    for (int64_t i = threadIdx.x; i < cap * (1 + R); i += blockDim.x) Tk[i] = kInf32;
    for (int i = threadIdx.x; i < kFilterWords; i += blockDim.x) s_filter[i] = 0u;
    __syncthreads();
    for (int j = threadIdx.x; j < len; j += blockDim.x) {
      const uint64_t kv = key[lo + j];
      int32_t w = (int32_t)lkey_hub(kv);
      uint32_t x = lkey_hd(kv);
      const uint32_t fb = filter_bit<kFilterBits>((uint32_t)w);
      atomicOr(&s_filter[fb >> 5], 1u << (fb & 31));
      uint32_t ix = table_hash((uint32_t)w, mask);
      bool placed = false;
      for (uint32_t probe = 0; probe <= mask; probe++) {  // the table is at most 2/3 full
        int32_t old = atomicCAS(&Tk[ix], kEmptyKey, w);
        if (old == kEmptyKey || old == w) {
          placed = true;
          break;
        }
        ix = (ix + 1) & mask;
      }
      if (placed) atomicMin(&Td[(int64_t)ix * R + hd_hop(x)], (int32_t)hd_dist(x));
    }
    __syncthreads();
    for (int64_t e = threadIdx.x; e < cap; e += blockDim.x) {
      if (Tk[e] == kEmptyKey) continue;
      int32_t* row = Td + e * R;
      int32_t m = row[0];
      for (int j = 1; j <= K; j++) {
        m = min(m, row[j]);
        row[j] = m;
      }
    }
    __syncthreads();
    int my_kept = 0;
    for (int i = wid; i < len; i += nw) {
      const uint64_t kv = key[lo + i];
      int u = (int)lkey_hub(kv);
      uint32_t x = lkey_hd(kv);
      int h = (int)hd_hop(x);
      long long d = (long long)hd_dist(x);
      bool keepit;
      if (u == v) {
        keepit = true;  // the self label (v, 0, 0) is never covered
      } else if (i > 0 && (key[lo + i - 1] >> 28) == (kv >> 28)) {
        // the row's previous label has the same hub and hop and a distance
        // <= d: once accepted it covers this one through u's self label, as
        // in the reference; if it was covered, so is this one.  (Only
        // imported label sets repeat a (hub, hop); a generated row has one
        // label per hub and hop.)
        keepit = false;
      } else {
        long long q = LLONG_MAX;
        // hub u itself: labels of v with hub u and fewer hops
        const int su = tab_find(Tk, mask, u);
        if (su >= 0 && Td[(int64_t)su * R + h - 1] != kInf32) q = Td[(int64_t)su * R + h - 1];
        if (!(q <= d)) {
          // L[u] is sorted by hub, so the hubs ranked above u are its prefix
          // [0, below[u]) and the hubs of u's own wave the prefix's tail:
          // scan 32 labels at a time from the prefix's end while the chunk's
          // first hub is still in the window.
          const int64_t ulo = off[u];
          const int ws = wave_lo ? wave_lo[u] : 0;
          for (int j1 = below[u]; j1 > 0; j1 -= 32) {
            const int j = j1 - 32 + lane;
            bool in_window = false;
            if (j >= 0) {
              const uint64_t k1 = key[ulo + j];
              const int w = (int)lkey_hub(k1);
              const uint32_t x1 = lkey_hd(k1);
              const uint32_t fb = filter_bit<kFilterBits>((uint32_t)w);
              const int h1 = (int)hd_hop(x1);
              in_window = w >= ws;
              if (in_window && w != u && h1 <= h && ((s_filter[fb >> 5] >> (fb & 31)) & 1u)) {
                const int sw = tab_find(Tk, mask, w);
                if (sw >= 0) {
                  const int32_t t = Td[(int64_t)sw * R + h - h1];
                  if (t != kInf32) {
                    long long c = (long long)hd_dist(x1) + t;
                    q = c < q ? c : q;
                  }
                }
              }
            }
            scanned += (unsigned long long)min(32, j1);
            if (__any_sync(0xffffffffu, q <= d)) break;
            if (!__shfl_sync(0xffffffffu, in_window, 0)) break;  // lane 0 holds the chunk's first label
          }
          q = warp_min_ll(q);
        }
        keepit = !(q <= d);
      }
      if (lane == 0) keep[lo + i] = keepit ? 1 : 0;
      my_kept += keepit ? 1 : 0;
    }
    if (lane == 0) s_kept[wid] = my_kept;
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t s = 0;
      for (int i = 0; i < nw; i++) s += s_kept[i];
      kept[v] = s;
    }
    __syncthreads();
  }
}

// below[u] = labels of the sorted row L[u] whose hub is ranked above u (the
// first index with hub >= u, by binary search over the keys).
__global__ void k_below(int32_t n, const int64_t* __restrict__ off, const uint64_t* __restrict__ key,
                        int32_t* __restrict__ below) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    const uint64_t first = (uint64_t)(uint32_t)u << 32;
    int64_t a = off[u], b = off[u + 1];
    const int64_t lo = a;
    while (a < b) {
      const int64_t mid = (a + b) >> 1;
      if (key[mid] < first) a = mid + 1; else b = mid;
    }
    below[u] = (int32_t)(a - lo);
  }
}

__global__ void k_compact(int32_t n, const int64_t* __restrict__ off, const uint64_t* __restrict__ key,
                          const int32_t* __restrict__ par,
                          const uint8_t* __restrict__ keep, const int64_t* __restrict__ noff,
                          uint64_t* __restrict__ nkey, int32_t* __restrict__ npar) {
  const int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    int64_t lo = off[v], len = off[v + 1] - lo, dst = noff[v];
    for (int64_t j0 = 0; j0 < len; j0 += 32) {
      int64_t j = j0 + lane;
      bool k = j < len && keep[lo + j];
      unsigned b = __ballot_sync(0xffffffffu, k);
      if (k) {
        int64_t at = dst + __popc(b & ((1u << lane) - 1));
        nkey[at] = key[lo + j];
        npar[at] = par[lo + j];
      }
      dst += __popc(b);
    }
  }
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int clean_index(hsdl_index_impl* idx) {
  cudaStream_t st = idx->stream;
  const int32_t n = idx->n, K = idx->K;
  const int sms = device_sm_count();
  const int words = K + 2;  // per slot: key + K+1 distances
  double t0 = now_s();
  // shared-memory table within 64 KB per block, plus the 8 KB filter (three
  // blocks per SM); a power-of-two slot count
  int smem_slots = 8;
  while ((int64_t)smem_slots * 2 * words * 4 <= 64 * 1024) smem_slots *= 2;
  const size_t smem = (size_t)smem_slots * words * 4;
  HSDL_CUDA(cudaFuncSetAttribute(k_clean, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t need_slots = 8;
  while (need_slots < idx->max_row + idx->max_row / 2) need_slots <<= 1;
  const int grid = sms * resident_blocks(k_clean, kCleanThreads, smem);
  int64_t gslots = need_slots > smem_slots ? need_slots : 0;
  DevBuf<int32_t> gscratch;
  if (gslots > 0) HSDL_TRY(gscratch.alloc((int64_t)grid * gslots * words, st));
  DevBuf<uint8_t> keep;
  DevBuf<int64_t> kept, noff;
  DevBuf<int> next;
  DevBuf<unsigned long long> reads;
  HSDL_TRY(reads.alloc(1, st));
  HSDL_CUDA(cudaMemsetAsync(reads.p, 0, sizeof(unsigned long long), st));
  HSDL_TRY(keep.alloc(std::max<int64_t>(1, idx->total), st));
  HSDL_TRY(kept.alloc((int64_t)n + 1, st));
  HSDL_TRY(noff.alloc((int64_t)n + 1, st));
  HSDL_TRY(next.alloc(1, st));
  HSDL_CUDA(cudaMemsetAsync(next.p, 0, sizeof(int), st));
  DevBuf<int32_t> below;
  HSDL_TRY(below.alloc(std::max<int32_t>(1, n), st));
  k_below<<<sms * 8, 256, 0, st>>>(n, idx->off.p, idx->key.p, below.p);
  HSDL_LAUNCHED();
  k_clean<<<grid, kCleanThreads, smem, st>>>(n, K, idx->off.p, idx->key.p, keep.p, kept.p, idx->wave_lo.p,
                                             below.p, smem_slots, gscratch.p, gslots, next.p, reads.p);
  HSDL_LAUNCHED();
  HSDL_TRY(exclusive_scan_i64(kept.p, noff.p, n, st));
  int64_t total = 0;
  unsigned long long h_reads = 0;
  HSDL_CUDA(cudaMemcpyAsync(&total, noff.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaMemcpyAsync(&h_reads, reads.p, sizeof(h_reads), cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  DevBuf<uint64_t> nkey;
  DevBuf<int32_t> npar;
  HSDL_TRY(nkey.alloc(total + kRowPad, st));
  HSDL_TRY(npar.alloc(total + kRowPad, st));
  k_compact<<<sms * 8, 256, 0, st>>>(n, idx->off.p, idx->key.p, idx->par.p, keep.p, noff.p, nkey.p, npar.p);
  HSDL_LAUNCHED();
  HSDL_CUDA(cudaStreamSynchronize(st));
  std::swap(idx->off.p, noff.p);
  std::swap(idx->off.cap, noff.cap);
  std::swap(idx->key.p, nkey.p);
  std::swap(idx->key.cap, nkey.cap);
  std::swap(idx->par.p, npar.p);
  std::swap(idx->par.cap, npar.cap);
  noff.release();
  nkey.release();
  npar.release();
  keep.release();
  kept.release();
  gscratch.release();
  next.release();
  reads.release();
  below.release();
  idx->wave_lo.release();  // the clean is done; a repeat would need the full scan
  idx->work_clean_reads += (int64_t)h_reads;
  idx->before = idx->total;
  idx->total = total;
  idx->after = total;
  idx->cleaned = true;
  idx->h_off.resize((size_t)n + 1);
  HSDL_CUDA(cudaMemcpy(idx->h_off.data(), idx->off.p, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost));
  int64_t mr = 0;
  for (int32_t v = 0; v < n; v++) mr = std::max(mr, idx->h_off[v + 1] - idx->h_off[v]);
  idx->max_row = mr;
  idx->t_clean = now_s() - t0;
  return HSDL_OK;
}

}  // namespace hsdl
