// Device-side helpers shared by the HSDL kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hsdl {

// ---------------------------------------------------------------------------
// Packed encodings.
//
// Label key (8 B):
//     hub:32 | hop:4 | distance:28          (bits 63..32 | 31..28 | 27..0)
// Unsigned order of the key is exactly the reference's label order
// (hub asc, hop asc, distance asc; compare_hop_constrained_two_hop_label,
// CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:373-387),
// so sorting keys sorts labels.  A resident index stores one key per label
// (a join gets hop and distance with the hub id, no dependent load), with
// parent_vertex in a parallel int32 array; hd = hop:4|distance:28 is the
// key's low word.  Limits: vertex ids < 2^28
// (the reference itself stops at 10^7, generation.h:528-532), hop <= 14,
// distance < 2^28 (K * max edge weight < 2^28).
//
// Candidate key (per-slot search state, 8 B):
//     distance:32 | hop:4 | parent:28
// atomicMin on it keeps the smallest distance, then the smallest hop, then the
// smallest predecessor id.  The all-ones value marks an untouched state (its
// hop field, 15, is never a real hop).
// ---------------------------------------------------------------------------
constexpr uint64_t kEmptyCand = ~0ull;
constexpr uint32_t kIdMask = (1u << 28) - 1;
constexpr int32_t kMaxK = 14;
constexpr int32_t kInf32 = 0x7F7F7F7F;  // "no value" in hub tables (memset 0x7F)
constexpr int32_t kEmptyKey = 0x7F7F7F7F;

constexpr uint32_t kDistMask = (1u << 28) - 1;

__host__ __device__ inline uint32_t hd_pack(uint32_t hop, uint32_t dist) { return (hop << 28) | dist; }
__host__ __device__ inline uint32_t hd_hop(uint32_t x) { return x >> 28; }
__host__ __device__ inline uint32_t hd_dist(uint32_t x) { return x & kDistMask; }

__host__ __device__ inline uint64_t lkey(uint32_t hub, uint32_t hop, uint32_t dist) {
  return ((uint64_t)hub << 32) | (uint64_t)hd_pack(hop, dist);
}
__host__ __device__ inline uint32_t lkey_hub(uint64_t k) { return (uint32_t)(k >> 32); }
__host__ __device__ inline uint32_t lkey_hd(uint64_t k) { return (uint32_t)k; }
__host__ __device__ inline uint32_t lkey_hop(uint64_t k) { return hd_hop((uint32_t)k); }
__host__ __device__ inline uint32_t lkey_dist(uint64_t k) { return hd_dist((uint32_t)k); }

// Compact query key (4 B), used by the query joins when the index's ranges
// fit: hub:H | hop:P | distance:D with H = bits of n (the all-ones key is
// then a hub above every real one), P = bits of K and
// D = 32 - H - P >= the bits of the largest distance in the index (n = 1M,
// K = 5, weights <= 100: 20 | 3 | 9).  Unsigned order is again the label
// order, so the rows keep their sort; a join streams half the bytes of the
// 8-byte keys.  Indexes whose ranges do not fit keep only the 8-byte keys.
struct Fmt64 {
  using key_t = uint64_t;
  __host__ __device__ uint32_t hub(uint64_t k) const { return (uint32_t)(k >> 32); }
  __host__ __device__ uint32_t hop(uint64_t k) const { return hd_hop((uint32_t)k); }
  __host__ __device__ uint32_t dist(uint64_t k) const { return hd_dist((uint32_t)k); }
  __host__ __device__ uint64_t pack(uint32_t hub, uint32_t hop, uint32_t dist) const {
    return ((uint64_t)hub << 32) | (uint64_t)hd_pack(hop, dist);
  }
};
struct Fmt32 {
  using key_t = uint32_t;
  uint32_t hub_shift;  // P + D
  uint32_t dist_bits;  // D
  __host__ __device__ uint32_t hub(uint32_t k) const { return k >> hub_shift; }
  __host__ __device__ uint32_t hop(uint32_t k) const {
    return (k >> dist_bits) & ((1u << (hub_shift - dist_bits)) - 1u);
  }
  __host__ __device__ uint32_t dist(uint32_t k) const { return k & ((1u << dist_bits) - 1u); }
  __host__ __device__ uint32_t pack(uint32_t hub, uint32_t hop, uint32_t dist) const {
    return (hub << hub_shift) | (hop << dist_bits) | dist;
  }
};

__host__ __device__ inline uint64_t ckey(uint32_t dist, uint32_t hop, uint32_t parent) {
  return ((uint64_t)dist << 32) | ((uint64_t)hop << 28) | (uint64_t)parent;
}
__host__ __device__ inline uint32_t ckey_dist(uint64_t k) { return (uint32_t)(k >> 32); }
__host__ __device__ inline uint32_t ckey_hop(uint64_t k) { return (uint32_t)(k >> 28) & 15u; }
__host__ __device__ inline uint32_t ckey_parent(uint64_t k) { return (uint32_t)k & kIdMask; }

// Hub-table slot index for hub id w in a table of `mask+1` (power of two) slots.
__device__ inline uint32_t table_hash(uint32_t w, uint32_t mask) {
  uint32_t h = w * 2654435761u;
  return (h ^ (h >> 15)) & mask;
}

// Bit of hub w in a membership filter of 2^bits bits (a second, independent
// multiplicative hash; the top bits are taken).
template <int bits>
__device__ inline uint32_t filter_bit(uint32_t w) {
  return (w * 0x85EBCA6Bu) >> (32 - bits);
}

// ---------------------------------------------------------------------------
// Warp helpers.
// ---------------------------------------------------------------------------
__device__ inline int lane_id() { return threadIdx.x & 31; }

__device__ inline long long warp_min_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
  return v;
}

__device__ inline int64_t warp_sum_i64(int64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp-aggregated append: every lane of the currently active mask with `pred`
// gets a distinct slot from *counter; one atomic per warp.  Returns the slot
// or -1 when pred is false.
__device__ inline long long warp_append(bool pred, unsigned long long* counter) {
  unsigned mask = __activemask();
  unsigned ballot = __ballot_sync(mask, pred);
  if (ballot == 0) return -1;
  int leader = __ffs(ballot) - 1;
  int lane = lane_id();
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(ballot));
  base = __shfl_sync(mask, base, leader);
  if (!pred) return -1;
  return (long long)(base + __popc(ballot & ((1u << lane) - 1)));
}

// Per-warp staging of list appends.  Lanes with an entry put it in the
// warp's shared-memory buffer (64 entries); once the buffer holds 32 or more,
// the warp moves it to the global list with a single atomic on the list's
// counter.  Many warps appending one entry each to the same counter
// serialise on the one L2 slice that holds it; staging cuts those atomics by
// the buffer's fill.  Every lane of the warp must call these (convergent);
// `n` is warp-uniform.
template <class T>
__device__ inline void warp_stage_flush(T* buf, int& n, unsigned long long* counter, T* out, int64_t cap,
                                        unsigned long long* overflow) {
  __syncwarp();
  const int lane = lane_id();
  unsigned long long base = 0;
  if (lane == 0 && n > 0) base = atomicAdd(counter, (unsigned long long)n);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int j = lane; j < n; j += 32) {
    const unsigned long long p = base + (unsigned long long)j;
    if ((int64_t)p < cap) out[p] = buf[j];
    else *overflow = 1;
  }
  __syncwarp();
  n = 0;
}

template <class T>
__device__ inline void warp_stage(T* buf, int& n, bool pred, const T& val, unsigned long long* counter, T* out,
                                  int64_t cap, unsigned long long* overflow) {
  const unsigned m = __ballot_sync(0xffffffffu, pred);
  if (pred) buf[n + __popc(m & ((1u << lane_id()) - 1u))] = val;
  n += __popc(m);
  if (n >= 32) warp_stage_flush(buf, n, counter, out, cap, overflow);
}

// Block-wide exclusive scan of one int64 per thread (blockDim.x <= 1024,
// multiple of 32).  `smem` must hold 32 int64.  Returns the exclusive prefix;
// *total receives the block sum.
__device__ inline int64_t block_exclusive_scan(int64_t v, int64_t* smem, int64_t* total) {
  int lane = lane_id(), wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t s = lane < nw ? smem[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) smem[lane] = s;
  }
  __syncthreads();
  int64_t warp_prefix = wid > 0 ? smem[wid - 1] : 0;
  int64_t t = smem[nw - 1];
  __syncthreads();
  if (total) *total = t;
  return warp_prefix + x - v;
}

}  // namespace hsdl
