// The (s, t, k) distance join on a resident label index, one warp per query.
//
// Reference: hop_constrained_extract_distance
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144-222): the
// minimum d1 + d2 over label pairs of a common hub with h1 + h2 <= k;
// INT_MAX for k < 0, then 0 for s == t, then INT_MAX for k == 0, and INT_MAX
// when no pair qualifies.
//
// The merged hub order of the two rows is cut into 32 equal pieces (merge
// path: each lane finds its split with one binary search along its diagonal,
// A's labels ordered before B's on equal hubs), and every lane merges its
// piece with two pointers, streaming 4-byte hub ids and reading hop and
// distance only on a hub match.  When the lane takes a label of A with hub w,
// B's run of hub w starts at the lane's B pointer; it is scanned with the
// reference's hop-sum break (possibly past the lane's piece).  A warp min
// combines the lanes.
#pragma once
#include <climits>

#include "hsdl_device.cuh"

namespace hsdl {

// One lane's share of the merge-path join of hub rows A (la labels) and B (lb
// labels) under hop bound k >= 1, the merge split over a group of G lanes
// (G = 8, 16 or 32; gl = lane index in the group); returns the lane's minimum
// (INT_MAX if none).  A and B may point to shared or global memory; Ahd/Bhd
// are the matching hop|distance words (read only on hub matches).
template <int G>
__device__ inline long long lane_merge(const uint32_t* A, int la, const uint32_t* B, int lb,
                                       const uint32_t* __restrict__ Ahd, const uint32_t* __restrict__ Bhd, int k,
                                       int gl) {
  long long best = INT_MAX;
  const int tot = la + lb;
  const int d0 = (int)(((int64_t)tot * gl) / G), d1 = (int)(((int64_t)tot * (gl + 1)) / G);
  // merge-path split of diagonal d0: ia labels of A precede it.  The search
  // runs a fixed number of halvings (enough for the longest range) so the
  // lanes of a group stay converged.
  int lo = max(0, d0 - lb), hi = min(d0, la);
  for (int span = la; span > 0; span >>= 1) {
    if (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (A[mid] <= B[d0 - 1 - mid]) lo = mid + 1; else hi = mid;
    }
  }
  int ia = lo, ib = d0 - lo;
  uint32_t wa = ia < la ? A[ia] : 0xFFFFFFFFu;
  uint32_t wb = ib < lb ? B[ib] : 0xFFFFFFFFu;
  // Each step takes the smaller head (A's on ties) and loads its successor
  // through one selected pointer, with no branch on which side moved.
  for (int step = d0; step < d1; step++) {
    const bool take_a = ia < la && (ib >= lb || wa <= wb);
    if (take_a && wa == wb) {  // a common hub: B's run of it starts at ib
      const uint32_t xa = __ldg(Ahd + ia);
      const int h1 = (int)hd_hop(xa);
      if (h1 <= k) {
        const long long da = hd_dist(xa);
        for (int p = ib; p < lb && B[p] == wa; p++) {
          const uint32_t xb = __ldg(Bhd + p);
          if (h1 + (int)hd_hop(xb) > k) break;  // rows are hop-sorted within a hub
          const long long c = da + hd_dist(xb);
          best = c < best ? c : best;
        }
      }
    }
    ia += take_a ? 1 : 0;
    ib += take_a ? 0 : 1;
    const int at = take_a ? ia : ib;
    const int lim = take_a ? la : lb;
    const uint32_t nxt = at < lim ? (take_a ? A : B)[at] : 0xFFFFFFFFu;
    wa = take_a ? nxt : wa;
    wb = take_a ? wb : nxt;
  }
  return best;
}

// Min over the G lanes of each group (every lane of the warp must call it).
template <int G>
__device__ inline long long group_min(long long v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
  return v;
}

// TMA bulk prefetch of [p, p + bytes) into L2 (16-byte aligned, multiple of 16).
__device__ inline void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Prefetches the 16-byte aligned spans holding rows s and t of the hub array
// into L2 (one lane issues).  The hub array carries padding so the spans stay
// inside the allocation.
__device__ inline void prefetch_rows(const int64_t* __restrict__ off, const uint32_t* __restrict__ hub, int32_t n,
                                     int s, int t) {
  if (s < 0 || s >= n || t < 0 || t >= n || s == t) return;
  const int64_t r[2] = {s, t};
#pragma unroll
  for (int i = 0; i < 2; i++) {
    int64_t a = off[r[i]] & ~(int64_t)3, b = (off[r[i] + 1] + 3) & ~(int64_t)3;
    if (b > a) prefetch_l2(hub + a, (uint32_t)(b - a) * 4u);
  }
}

// Checks that decide an answer without a join; returns true and sets *ans.
__device__ inline bool trivial_answer(int32_t n, int s, int t, int k, int32_t* ans) {
  if (s < 0 || s >= n || t < 0 || t >= n) {
    *ans = INT_MAX;  // ids outside the index answer "unreachable"
    return true;
  }
  if (k < 0) {
    *ans = INT_MAX;
    return true;
  }
  if (s == t) {
    *ans = 0;
    return true;
  }
  if (k == 0) {
    *ans = INT_MAX;
    return true;
  }
  return false;
}

__device__ inline int32_t clamp_answer(long long best) { return best >= INT_MAX ? INT_MAX : (int32_t)best; }

// Each group of G lanes answers its own (s, t, k), rows read from global
// memory; every lane of the warp must call it (inactive groups pass
// active = false).  Every lane of a group returns the group's answer.
template <int G>
__device__ inline int32_t group_query(bool active, int32_t n, const int64_t* __restrict__ off,
                                      const uint32_t* __restrict__ hub, const uint32_t* __restrict__ hd, int s,
                                      int t, int k) {
  int32_t ans = INT_MAX;
  long long best = INT_MAX;
  const bool trivial = !active || trivial_answer(n, s, t, k, &ans);
  if (!trivial) {
    int64_t a0 = off[s], a1 = off[s + 1], b0 = off[t], b1 = off[t + 1];
    if (a1 - a0 > b1 - b0) {  // A = the shorter row
      int64_t x = a0; a0 = b0; b0 = x;
      x = a1; a1 = b1; b1 = x;
    }
    best = lane_merge<G>(hub + a0, (int)(a1 - a0), hub + b0, (int)(b1 - b0), hd + a0, hd + b0, k,
                         lane_id() & (G - 1));
  }
  best = group_min<G>(best);
  return trivial ? ans : clamp_answer(best);
}

// The whole answer of one (s, t, k) by a full warp (every lane must call it).
__device__ inline int32_t warp_query(int32_t n, const int64_t* __restrict__ off, const uint32_t* __restrict__ hub,
                                     const uint32_t* __restrict__ hd, const int s, const int t, const int k) {
  return group_query<32>(true, n, off, hub, hd, s, t, k);
}

}  // namespace hsdl
